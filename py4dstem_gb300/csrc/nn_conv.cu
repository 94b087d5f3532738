// Convolution and elementwise kernels of the learned initializer (a BF16 U-Net
// that maps virtual bright-field and centre-of-mass images of a scan to an
// initial object phase). There is no counterpart in the reference.
//
// Activations are NHWC bfloat16 with a channel count that is a multiple of 8.
// The 3 x 3 convolutions (stride 1, zero padding 1) are implicit GEMMs on the
// tensor cores through tc_gemm_kernel (tc_gemm.cuh):
//   forward         y[p, co]   = sum_{tap, ci} x[p + off(tap), ci] w[co, tap, ci]
//                   rows = pixels p, columns = co, K = 9 Cin
//   input gradient  dx[p, ci]  = sum_{tap, co} dy[p - off(tap), co] wt[ci, tap, co]
//                   rows = pixels, columns = ci, K = 9 Cout (wt: w transposed)
//   weight gradient dw[co, tap, ci] = sum_p dy[p, co] x[p + off(tap), ci]
//                   rows = (tap, ci), columns = co, K = pixels, split over K
//                   into fixed chunks whose partial sums are added in order
// with off(tap) = (tap / 3 - 1, tap % 3 - 1) in (y, x). Every reduction here is
// deterministic (no float atomics).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "nn_internal.h"
#include "tc_gemm.cuh"

namespace pty {
namespace nn {
namespace {

constexpr int kEw = 256;  // threads of the elementwise kernels

__device__ __forceinline__ uint4 zero16() { return make_uint4(0u, 0u, 0u, 0u); }

// ------------------------------------------------------------ GEMM operands
struct RowMajorBf16 {  // rows x K, row-major
  const bf16* p;
  int rows, K;
  __device__ uint4 operator()(int r, int kc) const {
    if (r >= rows) return zero16();
    return *reinterpret_cast<const uint4*>(p + (size_t)r * K + 8 * kc);
  }
};

struct StoreF32 {  // C (M, N) row-major float
  float* c;
  int M, N;
  __device__ void operator()(int r, int c0, const float (&v)[16], int) const {
#pragma unroll
    for (int i = 0; i < 16; ++i)
      if (c0 + i < N) c[(size_t)r * N + c0 + i] = v[i];
  }
};

struct Im2colFwd {  // rows = pixels, K = 9 Cin: 8 channels of one tap per chunk
  const bf16* x;
  int nb, H, W, C;
  __device__ uint4 operator()(int r, int kc) const {
    if (r >= nb * H * W) return zero16();
    const int k = 8 * kc;
    const int tap = k / C;
    const int ci = k - tap * C;
    const int xx = r % W;
    const int t = r / W;
    const int yy = t % H;
    const int n = t / H;
    const int sy = yy + tap / 3 - 1;
    const int sx = xx + tap % 3 - 1;
    if (sy < 0 || sy >= H || sx < 0 || sx >= W) return zero16();
    return *reinterpret_cast<const uint4*>(x + (((size_t)n * H + sy) * W + sx) * C + ci);
  }
};

struct Im2colBwdData {  // rows = pixels, K = 9 Cout: dy at p - off(tap)
  const bf16* dy;
  int nb, H, W, C;
  __device__ uint4 operator()(int r, int kc) const {
    if (r >= nb * H * W) return zero16();
    const int k = 8 * kc;
    const int tap = k / C;
    const int co = k - tap * C;
    const int xx = r % W;
    const int t = r / W;
    const int yy = t % H;
    const int n = t / H;
    const int sy = yy - (tap / 3 - 1);
    const int sx = xx - (tap % 3 - 1);
    if (sy < 0 || sy >= H || sx < 0 || sx >= W) return zero16();
    return *reinterpret_cast<const uint4*>(dy + (((size_t)n * H + sy) * W + sx) * C + co);
  }
};

// rows = (tap, ci) (9 Cin), K = pixels (8 consecutive pixels of one image row:
// the width is a multiple of 8)
struct Im2colWgradA {
  const bf16* x;
  int nb, H, W, C;
  __device__ uint4 operator()(int r, int kc) const {
    if (r >= 9 * C) return zero16();
    const int tap = r / C;
    const int ci = r - tap * C;
    const int p0 = 8 * kc;
    if (p0 >= nb * H * W) return zero16();
    const int x0 = p0 % W;
    const int t = p0 / W;
    const int yy = t % H;
    const int n = t / H;
    const int sy = yy + tap / 3 - 1;
    if (sy < 0 || sy >= H) return zero16();
    const int dx = tap % 3 - 1;
    const bf16* row = x + (((size_t)n * H + sy) * W) * C + ci;
    __align__(16) bf16 v[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int sx = x0 + j + dx;
      v[j] = (sx >= 0 && sx < W) ? row[(size_t)sx * C] : __float2bfloat16(0.0f);
    }
    return *reinterpret_cast<const uint4*>(v);
  }
};

struct WgradB {  // rows = co, K = pixels: dy[p, co] for 8 consecutive pixels
  const bf16* dy;
  int npix, C;
  __device__ uint4 operator()(int r, int kc) const {
    if (r >= C) return zero16();
    const int p0 = 8 * kc;
    if (p0 >= npix) return zero16();
    __align__(16) bf16 v[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = dy[(size_t)(p0 + j) * C + r];
    return *reinterpret_cast<const uint4*>(v);
  }
};

struct StoreActivation {  // y[p, co] = bf16(act(v + bias[co])), Cout a multiple of 16
  bf16* y;
  const float* bias;
  int Cout, relu;
  __device__ void operator()(int r, int c0, const float (&v)[16], int) const {
    __align__(16) bf16 o[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      float t = v[i] + (bias ? bias[c0 + i] : 0.0f);
      if (relu) t = fmaxf(t, 0.0f);
      o[i] = __float2bfloat16(t);
    }
    uint4* dst = reinterpret_cast<uint4*>(y + (size_t)r * Cout + c0);
    dst[0] = reinterpret_cast<const uint4*>(o)[0];
    dst[1] = reinterpret_cast<const uint4*>(o)[1];
  }
};

struct StoreGradInput {  // dx[p, ci] (float), columns beyond Cin dropped
  float* dx;
  int Cin;
  __device__ void operator()(int r, int c0, const float (&v)[16], int) const {
#pragma unroll
    for (int i = 0; i < 16; ++i)
      if (c0 + i < Cin) dx[(size_t)r * Cin + c0 + i] = v[i];
  }
};

struct StoreWgradPartial {  // part[z][co][r] with r = (tap, ci)
  float* part;
  int rows, Cout;
  __device__ void operator()(int r, int c0, const float (&v)[16], int z) const {
    float* base = part + (size_t)z * Cout * rows;
#pragma unroll
    for (int i = 0; i < 16; ++i)
      if (c0 + i < Cout) base[(size_t)(c0 + i) * rows + r] = v[i];
  }
};

template <int BN, class LA, class LB, class EP>
cudaError_t launch_gemm(int M, int N, int K, int splits, int k_per_split, LA la, LB lb, EP ep,
                        int* err, cudaStream_t s) {
  auto kern = tc_gemm_kernel<BN, LA, LB, EP>;
  const int smem = GemmSmem<BN>::kBytes;
  cudaError_t e = ensure_smem_limit(reinterpret_cast<const void*>(kern), smem);
  if (e != cudaSuccess) return e;
  dim3 grid((M + kBM - 1) / kBM, (N + BN - 1) / BN, splits);
  kern<<<grid, kGemmThreads, smem, s>>>(M, N, K, k_per_split, la, lb, ep, err);
  return cudaGetLastError();
}

// Largest of 256/128/64/32 that divides n (n a multiple of 8 and >= 32), else 32.
int pick_bn(int n) {
  for (int bn : {256, 128, 64, 32})
    if (n % bn == 0) return bn;
  return 32;
}

template <class LA, class LB, class EP>
cudaError_t launch_gemm_bn(int bn, int M, int N, int K, int splits, int kps, LA la, LB lb, EP ep,
                           int* err, cudaStream_t s) {
  switch (bn) {
    case 256: return launch_gemm<256>(M, N, K, splits, kps, la, lb, ep, err, s);
    case 128: return launch_gemm<128>(M, N, K, splits, kps, la, lb, ep, err, s);
    case 64: return launch_gemm<64>(M, N, K, splits, kps, la, lb, ep, err, s);
    default: return launch_gemm<32>(M, N, K, splits, kps, la, lb, ep, err, s);
  }
}

// ------------------------------------------------------------ elementwise
__global__ void wgrad_reduce_kernel(const float* part, int splits, size_t n, float* dw) {
  const size_t i = (size_t)blockIdx.x * kEw + threadIdx.x;
  if (i >= n) return;
  float s = 0.0f;
  for (int z = 0; z < splits; ++z) s += part[(size_t)z * n + i];
  dw[i] = s;
}

// bias gradient: sum over pixels of dy[:, c]; one block per channel, fixed order
__global__ void bias_grad_kernel(const bf16* dy, int npix, int C, float* db) {
  __shared__ float red[kEw / 32];
  const int c = blockIdx.x;
  float s = 0.0f;
  for (int p = threadIdx.x; p < npix; p += kEw) s += __bfloat162float(dy[(size_t)p * C + c]);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.0f;
    for (int w = 0; w < kEw / 32; ++w) t += red[w];
    db[c] = t;
  }
}

}  // namespace

cudaError_t gemm_bf16(const bf16* a, const bf16* b, float* c, int M, int N, int K, int* err,
                      cudaStream_t s) {
  return launch_gemm_bn(pick_bn(N), M, N, K, 1, K, RowMajorBf16{a, M, K}, RowMajorBf16{b, N, K},
                        StoreF32{c, M, N}, err, s);
}

cudaError_t conv3x3_forward(const bf16* x, int nb, int H, int W, int cin, const bf16* w,
                            const float* bias, int cout, int relu, bf16* y, int* err,
                            cudaStream_t s) {
  const int M = nb * H * W;
  return launch_gemm_bn(pick_bn(cout), M, cout, 9 * cin, 1, 9 * cin,
                        Im2colFwd{x, nb, H, W, cin}, RowMajorBf16{w, cout, 9 * cin},
                        StoreActivation{y, bias, cout, relu}, err, s);
}

cudaError_t conv3x3_backward_data(const bf16* dy, int nb, int H, int W, int cout, const bf16* wt,
                                  int cin, float* dx, int* err, cudaStream_t s) {
  const int M = nb * H * W;
  return launch_gemm_bn(pick_bn(cin), M, cin, 9 * cout, 1, 9 * cout,
                        Im2colBwdData{dy, nb, H, W, cout}, RowMajorBf16{wt, cin, 9 * cout},
                        StoreGradInput{dx, cin}, err, s);
}

size_t conv3x3_wgrad_workspace(int nb, int H, int W, int cin, int cout) {
  const int splits = wgrad_splits(nb * H * W);
  return sizeof(float) * (size_t)splits * 9 * cin * cout;
}

int wgrad_splits(int npix) {
  // K chunks of at least 2048 pixels (a multiple of the 64-element K stage), at
  // most 64 of them
  int splits = (npix + 2047) / 2048;
  return splits > 64 ? 64 : (splits < 1 ? 1 : splits);
}

cudaError_t conv3x3_backward_weight(const bf16* x, const bf16* dy, int nb, int H, int W, int cin,
                                    int cout, float* dw, float* db, float* part, int* err,
                                    cudaStream_t s) {
  const int npix = nb * H * W;
  const int splits = wgrad_splits(npix);
  int kps = (npix + splits - 1) / splits;
  kps = (kps + kBK - 1) / kBK * kBK;
  const int M = 9 * cin;
  cudaError_t e = launch_gemm_bn(pick_bn(cout), M, cout, npix, splits, kps,
                                 Im2colWgradA{x, nb, H, W, cin}, WgradB{dy, npix, cout},
                                 StoreWgradPartial{part, M, cout}, err, s);
  if (e != cudaSuccess) return e;
  const size_t n = (size_t)M * cout;
  wgrad_reduce_kernel<<<(unsigned)((n + kEw - 1) / kEw), kEw, 0, s>>>(part, splits, n, dw);
  if (db) bias_grad_kernel<<<cout, kEw, 0, s>>>(dy, npix, cout, db);
  return cudaGetLastError();
}

}  // namespace nn
}  // namespace pty

// ------------------------------------------------------------------ C ABI
// (declared in include/ptycho_gb300.h; bf16 arrays are passed as raw 16-bit
// words)
#include "../../include/ptycho_gb300.h"

namespace {
int conv_shape_ok(int nb, int H, int W, int cin, int cout) {
  return nb >= 1 && H >= 1 && W >= 8 && W % 8 == 0 && cin >= 8 && cin % 8 == 0 && cout >= 16 &&
         cout % 16 == 0;
}
}  // namespace

extern "C" {

int ptycho_nn_gemm_bf16(const void* a, const void* b, float* c, int32_t m, int32_t n, int32_t k,
                        int32_t* err_flag, void* stream) {
  if (!a || !b || !c || !err_flag || m < 1 || n < 16 || n % 16 || k < 8 || k % 8)
    return PTYCHO_ERR_INVALID_ARGUMENT;
  using pty::nn::bf16;
  cudaError_t e = pty::nn::gemm_bf16(static_cast<const bf16*>(a), static_cast<const bf16*>(b), c,
                                     m, n, k, err_flag, static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? PTYCHO_OK : PTYCHO_ERR_CUDA;
}

int ptycho_nn_conv3x3_forward(const void* x, int32_t batch, int32_t height, int32_t width,
                              int32_t cin, const void* weight, const float* bias, int32_t cout,
                              int32_t relu, void* y, int32_t* err_flag, void* stream) {
  if (!x || !weight || !y || !err_flag || !conv_shape_ok(batch, height, width, cin, cout))
    return PTYCHO_ERR_INVALID_ARGUMENT;
  using pty::nn::bf16;
  cudaError_t e = pty::nn::conv3x3_forward(
      static_cast<const bf16*>(x), batch, height, width, cin, static_cast<const bf16*>(weight),
      bias, cout, relu ? 1 : 0, static_cast<bf16*>(y), err_flag, static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? PTYCHO_OK : PTYCHO_ERR_CUDA;
}

int ptycho_nn_conv3x3_backward_data(const void* dy, int32_t batch, int32_t height,
                                    int32_t width, int32_t cout, const void* weight_t,
                                    int32_t cin, float* dx, int32_t* err_flag, void* stream) {
  if (!dy || !weight_t || !dx || !err_flag || !conv_shape_ok(batch, height, width, cin, cout))
    return PTYCHO_ERR_INVALID_ARGUMENT;
  using pty::nn::bf16;
  cudaError_t e = pty::nn::conv3x3_backward_data(
      static_cast<const bf16*>(dy), batch, height, width, cout,
      static_cast<const bf16*>(weight_t), cin, dx, err_flag, static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? PTYCHO_OK : PTYCHO_ERR_CUDA;
}

size_t ptycho_nn_conv3x3_wgrad_workspace_bytes(int32_t batch, int32_t height, int32_t width,
                                               int32_t cin, int32_t cout) {
  if (!conv_shape_ok(batch, height, width, cin, cout)) return 0;
  return pty::nn::conv3x3_wgrad_workspace(batch, height, width, cin, cout);
}

int ptycho_nn_conv3x3_backward_weight(const void* x, const void* dy, int32_t batch,
                                      int32_t height, int32_t width, int32_t cin, int32_t cout,
                                      float* dweight, float* dbias, void* workspace,
                                      size_t workspace_bytes, int32_t* err_flag, void* stream) {
  if (!x || !dy || !dweight || !workspace || !err_flag ||
      !conv_shape_ok(batch, height, width, cin, cout))
    return PTYCHO_ERR_INVALID_ARGUMENT;
  if (workspace_bytes < pty::nn::conv3x3_wgrad_workspace(batch, height, width, cin, cout))
    return PTYCHO_ERR_WORKSPACE;
  using pty::nn::bf16;
  cudaError_t e = pty::nn::conv3x3_backward_weight(
      static_cast<const bf16*>(x), static_cast<const bf16*>(dy), batch, height, width, cin, cout,
      dweight, dbias, static_cast<float*>(workspace), err_flag, static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? PTYCHO_OK : PTYCHO_ERR_CUDA;
}

}  // extern "C"
