// Internal declarations of the learned-initializer kernels (nn_conv.cu,
// nn_unet.cu, nn_data.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace pty {

cudaError_t ensure_smem_limit(const void* fn, int bytes);

namespace nn {

using bf16 = __nv_bfloat16;

// C (M, N) f32 = A (M, K) B (N, K)^T, bf16 row-major operands, K % 8 == 0.
cudaError_t gemm_bf16(const bf16* a, const bf16* b, float* c, int M, int N, int K, int* err,
                      cudaStream_t s);

// 3 x 3 convolution, stride 1, zero padding 1, NHWC bf16; channel counts are
// multiples of 8 (outputs of the forward pass: multiples of 16) and the width a
// multiple of 8. w: (cout, 9, cin) bf16; wt: (cin, 9, cout) bf16 (w with the
// channel axes exchanged).
cudaError_t conv3x3_forward(const bf16* x, int nb, int H, int W, int cin, const bf16* w,
                            const float* bias, int cout, int relu, bf16* y, int* err,
                            cudaStream_t s);
cudaError_t conv3x3_backward_data(const bf16* dy, int nb, int H, int W, int cout, const bf16* wt,
                                  int cin, float* dx, int* err, cudaStream_t s);
int wgrad_splits(int npix);
size_t conv3x3_wgrad_workspace(int nb, int H, int W, int cin, int cout);
cudaError_t conv3x3_backward_weight(const bf16* x, const bf16* dy, int nb, int H, int W, int cin,
                                    int cout, float* dw, float* db, float* part, int* err,
                                    cudaStream_t s);

}  // namespace nn
}  // namespace pty
