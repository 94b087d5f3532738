// The learned initializer's network: a 4-level U-Net with 32 base channels,
// BF16 weights and activations, FP32 accumulation (the convolutions run on the
// tensor cores, nn_conv.cu), trained with Adam on FP32 master weights. There is
// no counterpart in the reference.
//
// Architecture (H, W multiples of 64; channels per level 32 / 64 / 128 / 256):
//   encoder  L0 conv 8->32, L1 32->32 | pool | L2 32->64, L3 64->64 | pool |
//            L4 64->128, L5 128->128 | pool | L6 128->256, L7 256->256
//   decoder  up + concat L5: L8 384->128, L9 128->128 | up + concat L3:
//            L10 192->64, L11 64->64 | up + concat L1: L12 96->32, L13 32->32
//   head     1 x 1 convolution 32 -> 1 (the phase), no activation
// Every 3 x 3 convolution is followed by ReLU; pooling is 2 x 2 max, upsampling
// nearest-neighbour. Input: (batch, H, W, 2) float32 (the scan's virtual
// bright-field and centre-of-mass magnitude images, normalised by the caller),
// zero-padded to 8 channels. Output: (batch, H, W) float32.
//
// The caller owns every buffer: the parameters (ptycho_nn_unet_param_bytes) and
// a workspace for the activations and gradients of one batch
// (ptycho_nn_unet_workspace_bytes). Reductions run in a fixed order, so a
// training step is deterministic for given inputs.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>

#include "../../include/ptycho_gb300.h"
#include "nn_internal.h"

namespace pty {
namespace nn {
namespace {

constexpr int kT = 256;
constexpr int kLayers = 14;
constexpr int kCin[kLayers] = {8, 32, 32, 64, 64, 128, 128, 256, 384, 128, 192, 64, 96, 32};
constexpr int kCout[kLayers] = {32, 32, 64, 64, 128, 128, 256, 256, 128, 128, 64, 64, 32, 32};
constexpr int kLevel[kLayers] = {0, 0, 1, 1, 2, 2, 3, 3, 2, 2, 1, 1, 0, 0};
constexpr int kHeadC = 32;

size_t a256(size_t v) { return (v + 255) & ~size_t(255); }

// ------------------------------------------------------------ parameter layout
struct ParamLayout {
  size_t w16[kLayers], wt16[kLayers], w32[kLayers], b32[kLayers];
  size_t gw[kLayers], gb[kLayers], mw[kLayers], vw[kLayers], mb[kLayers], vb[kLayers];
  size_t hw, hb, ghw, ghb, mhw, vhw, mhb, vhb;
  size_t total;
};

ParamLayout param_layout() {
  ParamLayout L{};
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off = a256(off + bytes);
    return o;
  };
  for (int l = 0; l < kLayers; ++l) {
    const size_t n = (size_t)kCout[l] * 9 * kCin[l];
    L.w16[l] = take(2 * n);
    L.wt16[l] = take(2 * n);
    L.w32[l] = take(4 * n);
    L.b32[l] = take(4 * kCout[l]);
    L.gw[l] = take(4 * n);
    L.gb[l] = take(4 * kCout[l]);
    L.mw[l] = take(4 * n);
    L.vw[l] = take(4 * n);
    L.mb[l] = take(4 * kCout[l]);
    L.vb[l] = take(4 * kCout[l]);
  }
  L.hw = take(4 * kHeadC);
  L.hb = take(4);
  L.ghw = take(4 * kHeadC);
  L.ghb = take(4);
  L.mhw = take(4 * kHeadC);
  L.vhw = take(4 * kHeadC);
  L.mhb = take(4);
  L.vhb = take(4);
  L.total = off;
  return L;
}

// ------------------------------------------------------------ activation layout
struct ActLayout {
  size_t in8;
  size_t y[kLayers];        // conv outputs (post-ReLU), bf16
  size_t pool[3], idx[3];   // pooled encoder outputs (bf16) and argmax (uint8)
  size_t cat[3];            // decoder inputs (concat), bf16; cat[2] feeds L8
  size_t out;               // (n) f32
  size_t dout;              // (n) f32
  size_t dcat[3];           // f32 gradients wrt the concat inputs (kept for the skips)
  size_t dx;                // f32 scratch: gradient wrt a layer input
  size_t g[2];              // bf16 ping-pong gradients wrt pre-activations
  size_t wpart;             // weight-gradient partial sums
  size_t red;               // reduction scratch (f32)
  size_t err;               // int error flag of the tensor-core kernels
  size_t total;
};

int level_px(int nb, int H, int W, int lev) { return nb * (H >> lev) * (W >> lev); }

ActLayout act_layout(int nb, int H, int W) {
  ActLayout A{};
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off = a256(off + bytes);
    return o;
  };
  const int n0 = level_px(nb, H, W, 0);
  A.in8 = take(2 * (size_t)n0 * 8);
  size_t max_in = 0, max_out = 0, max_part = 0;
  for (int l = 0; l < kLayers; ++l) {
    const size_t np = level_px(nb, H, W, kLevel[l]);
    A.y[l] = take(2 * np * kCout[l]);
    max_in = max_in > np * kCin[l] ? max_in : np * kCin[l];
    max_out = max_out > np * kCout[l] ? max_out : np * kCout[l];
    const size_t part = conv3x3_wgrad_workspace(nb, H >> kLevel[l], W >> kLevel[l], kCin[l],
                                                kCout[l]);
    max_part = max_part > part ? max_part : part;
  }
  const int pc[3] = {32, 64, 128};
  for (int k = 0; k < 3; ++k) {
    const size_t np = level_px(nb, H, W, k + 1);
    A.pool[k] = take(2 * np * pc[k]);
    A.idx[k] = take(np * pc[k]);
  }
  // cat[0]: level 0, 96 channels (L12); cat[1]: level 1, 192 (L10); cat[2]: level 2, 384 (L8)
  A.cat[0] = take(2 * (size_t)level_px(nb, H, W, 0) * 96);
  A.cat[1] = take(2 * (size_t)level_px(nb, H, W, 1) * 192);
  A.cat[2] = take(2 * (size_t)level_px(nb, H, W, 2) * 384);
  A.out = take(4 * (size_t)n0);
  A.dout = take(4 * (size_t)n0);
  A.dcat[0] = take(4 * (size_t)level_px(nb, H, W, 0) * 96);
  A.dcat[1] = take(4 * (size_t)level_px(nb, H, W, 1) * 192);
  A.dcat[2] = take(4 * (size_t)level_px(nb, H, W, 2) * 384);
  A.dx = take(4 * max_in);
  A.g[0] = take(2 * max_out);
  A.g[1] = take(2 * max_out);
  A.wpart = take(max_part);
  // per-block partials of the loss (one float per block) and of the head's
  // gradient (kHeadC + 1 floats per block), blocks of kT pixels
  A.red = take(4 * (size_t)((n0 + kT - 1) / kT) * (kHeadC + 1));
  A.err = take(sizeof(int));
  A.total = off;
  return A;
}

// ------------------------------------------------------------ small kernels
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  // SplitMix64 finaliser
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ float uniform01(uint64_t key) {
  return ((mix64(key) >> 40) + 0.5f) * (1.0f / 16777216.0f);
}

// Gaussian by Box-Muller from two counter-based uniforms.
__device__ __forceinline__ float normal01(uint64_t key) {
  const float u1 = uniform01(2 * key);
  const float u2 = uniform01(2 * key + 1);
  return sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
}

__global__ void init_conv_kernel(float* w32, bf16* w16, bf16* wt16, float* b32, int cout,
                                 int cin, float stddev, uint64_t seed) {
  const size_t n = (size_t)cout * 9 * cin;
  const size_t i = (size_t)blockIdx.x * kT + threadIdx.x;
  if (i < n) {
    const float v = stddev * normal01(seed * 0x100000000ull + i);
    w32[i] = v;
    w16[i] = __float2bfloat16(v);
    const int co = (int)(i / (9 * cin));
    const int r = (int)(i % (9 * cin));
    const int tap = r / cin, ci = r % cin;
    wt16[((size_t)ci * 9 + tap) * cout + co] = __float2bfloat16(v);
  }
  if (i < (size_t)cout) b32[i] = 0.0f;
}

// head weights ~ N(0, 1/32), bias 0 (the parameter block starts zeroed)
__global__ void init_head_kernel(float* hw, uint64_t seed) {
  const int c = threadIdx.x;
  if (c < kHeadC) hw[c] = sqrtf(1.0f / kHeadC) * normal01(seed * 0x100000000ull + c);
}

__global__ void pack_input_kernel(const float* in, int n, bf16* x8) {
  const int p = blockIdx.x * kT + threadIdx.x;
  if (p >= n) return;
  __align__(16) bf16 v[8];
  v[0] = __float2bfloat16(in[2 * (size_t)p]);
  v[1] = __float2bfloat16(in[2 * (size_t)p + 1]);
#pragma unroll
  for (int c = 2; c < 8; ++c) v[c] = __float2bfloat16(0.0f);
  *reinterpret_cast<uint4*>(x8 + (size_t)p * 8) = *reinterpret_cast<const uint4*>(v);
}

// 2 x 2 max pooling; idx = argmax within the window (row-major, first maximum)
__global__ void maxpool_kernel(const bf16* x, int nb, int H, int W, int C, bf16* y,
                               uint8_t* idx) {
  const int h = H / 2, w = W / 2;
  const size_t total = (size_t)nb * h * w * C;
  const size_t i = (size_t)blockIdx.x * kT + threadIdx.x;
  if (i >= total) return;
  const int c = (int)(i % C);
  size_t t = i / C;
  const int xo = (int)(t % w);
  t /= w;
  const int yo = (int)(t % h);
  const int n = (int)(t / h);
  float best = -INFINITY;
  int bi = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int yy = 2 * yo + (k >> 1), xx = 2 * xo + (k & 1);
    const float v = __bfloat162float(x[(((size_t)n * H + yy) * W + xx) * C + c]);
    if (v > best) {
      best = v;
      bi = k;
    }
  }
  y[i] = __float2bfloat16(best);
  idx[i] = (uint8_t)bi;
}

// out[:, :, :, 0:C1] = nearest-upsampled low; out[:, :, :, C1:C1+C2] = skip
__global__ void up_concat_kernel(const bf16* low, int C1, const bf16* skip, int C2, int nb,
                                 int H, int W, bf16* out) {
  const int Ct = C1 + C2;
  const size_t total = (size_t)nb * H * W * Ct;
  const size_t i = (size_t)blockIdx.x * kT + threadIdx.x;
  if (i >= total) return;
  const int c = (int)(i % Ct);
  const size_t p = i / Ct;
  const int xx = (int)(p % W);
  const size_t t = p / W;
  const int yy = (int)(t % H);
  const int n = (int)(t / H);
  if (c < C1) {
    out[i] = low[(((size_t)n * (H / 2) + yy / 2) * (W / 2) + xx / 2) * C1 + c];
  } else {
    out[i] = skip[p * C2 + (c - C1)];
  }
}

// g = dx * (y > 0) in bf16 (gradient wrt the pre-activation of the layer that
// produced y = relu(pre))
__global__ void relu_grad_kernel(const float* dx, const bf16* y, size_t n, bf16* g) {
  const size_t i = (size_t)blockIdx.x * kT + threadIdx.x;
  if (i >= n) return;
  g[i] = __float2bfloat16(__bfloat162float(y[i]) > 0.0f ? dx[i] : 0.0f);
}

// Gradient of the upsampled part of a concat input: channels [0, C1) of dcat
// (nb, H, W, Ct) summed over each 2 x 2 block, times the ReLU mask of low.
__global__ void up_grad_kernel(const float* dcat, int Ct, int C1, const bf16* low, int nb, int h,
                               int w, bf16* g) {
  const size_t total = (size_t)nb * h * w * C1;
  const size_t i = (size_t)blockIdx.x * kT + threadIdx.x;
  if (i >= total) return;
  const int c = (int)(i % C1);
  size_t t = i / C1;
  const int xo = (int)(t % w);
  t /= w;
  const int yo = (int)(t % h);
  const int n = (int)(t / h);
  const int H = 2 * h, W = 2 * w;
  float s = 0.0f;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int yy = 2 * yo + (k >> 1), xx = 2 * xo + (k & 1);
    s += dcat[(((size_t)n * H + yy) * W + xx) * Ct + c];
  }
  g[i] = __float2bfloat16(__bfloat162float(low[i]) > 0.0f ? s : 0.0f);
}

// Gradient of an encoder output y (nb, H, W, C) that feeds both a max pool and
// a decoder concat: the pooled gradient dp routed to the argmax, plus channels
// [C1, C1 + C) of dcat (nb, H, W, Ct), times the ReLU mask of y.
__global__ void pool_skip_grad_kernel(const float* dp, const uint8_t* idx, const float* dcat,
                                      int Ct, int C1, const bf16* y, int nb, int H, int W, int C,
                                      bf16* g) {
  const size_t total = (size_t)nb * H * W * C;
  const size_t i = (size_t)blockIdx.x * kT + threadIdx.x;
  if (i >= total) return;
  const int c = (int)(i % C);
  const size_t p = i / C;
  const int xx = (int)(p % W);
  const size_t t = p / W;
  const int yy = (int)(t % H);
  const int n = (int)(t / H);
  const size_t q = (((size_t)n * (H / 2) + yy / 2) * (W / 2) + xx / 2) * C + c;
  const int k = ((yy & 1) << 1) | (xx & 1);
  float s = idx[q] == k ? dp[q] : 0.0f;
  s += dcat[p * Ct + C1 + c];
  g[i] = __float2bfloat16(__bfloat162float(y[i]) > 0.0f ? s : 0.0f);
}

__global__ void head_forward_kernel(const bf16* x, int n, const float* hw, const float* hb,
                                    float* out) {
  const int p = blockIdx.x * kT + threadIdx.x;
  if (p >= n) return;
  const uint4* row = reinterpret_cast<const uint4*>(x + (size_t)p * kHeadC);
  float s = hb[0];
#pragma unroll
  for (int q = 0; q < kHeadC / 8; ++q) {
    uint4 v = row[q];
    const bf16* e = reinterpret_cast<const bf16*>(&v);
#pragma unroll
    for (int j = 0; j < 8; ++j) s += __bfloat162float(e[j]) * hw[8 * q + j];
  }
  out[p] = s;
}

// dout = 2 (out - target) mask / sum(mask) and per-block partial sums of the
// masked squared error (loss = their fixed-order sum / sum(mask))
__global__ void loss_kernel(const float* out, const float* target, const float* mask, int n,
                            float inv_count, float* dout, float* part) {
  __shared__ float red[kT / 32];
  const int p = blockIdx.x * kT + threadIdx.x;
  float e = 0.0f;
  if (p < n) {
    const float m = mask ? mask[p] : 1.0f;
    const float d = out[p] - target[p];
    dout[p] = 2.0f * d * m * inv_count;
    e = d * d * m;
  }
  for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = e;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.0f;
    for (int w = 0; w < kT / 32; ++w) t += red[w];
    part[blockIdx.x] = t;
  }
}

// Fixed-order sum of `n` partials times `scale` into *dst (one block).
__global__ void sum_partials_kernel(const float* part, int n, float scale, float* dst) {
  __shared__ float red[kT / 32];
  float s = 0.0f;
  const int per = (n + kT - 1) / kT;
  for (int i = threadIdx.x * per; i < min(n, (threadIdx.x + 1) * per); ++i) s += part[i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.0f;
    for (int w = 0; w < kT / 32; ++w) t += red[w];
    *dst = t * scale;
  }
}

// Head backward: g = dout * hw (masked by x > 0) in bf16, and per-block partials
// of dL/dhw (kHeadC values) and dL/dhb.
__global__ void head_backward_kernel(const float* dout, const bf16* x, int n, const float* hw,
                                     bf16* g, float* part) {
  __shared__ float red[kHeadC + 1][kT / 32];
  const int p = blockIdx.x * kT + threadIdx.x;
  float acc[kHeadC + 1];
#pragma unroll
  for (int c = 0; c <= kHeadC; ++c) acc[c] = 0.0f;
  if (p < n) {
    const float d = dout[p];
#pragma unroll
    for (int c = 0; c < kHeadC; ++c) {
      const float xv = __bfloat162float(x[(size_t)p * kHeadC + c]);
      acc[c] = d * xv;
      g[(size_t)p * kHeadC + c] = __float2bfloat16(xv > 0.0f ? d * hw[c] : 0.0f);
    }
    acc[kHeadC] = d;
  }
#pragma unroll
  for (int c = 0; c <= kHeadC; ++c) {
    float v = acc[c];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[c][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x <= kHeadC) {
    float t = 0.0f;
    for (int w = 0; w < kT / 32; ++w) t += red[threadIdx.x][w];
    part[(size_t)blockIdx.x * (kHeadC + 1) + threadIdx.x] = t;
  }
}

// dst[c] = sum over blocks of part[b * stride + c] (fixed order), c < count
__global__ void column_sum_kernel(const float* part, int blocks, int stride, int count,
                                  float* dst) {
  const int c = threadIdx.x;
  if (c >= count) return;
  float s = 0.0f;
  for (int b = 0; b < blocks; ++b) s += part[(size_t)b * stride + c];
  dst[c] = s;
}

// Adam on FP32 master weights; refreshes the bf16 copy and its transpose.
__global__ void adam_kernel(float* w, const float* gw, float* m, float* v, size_t n, float lr,
                            float b1, float b2, float eps, float c1, float c2, bf16* w16,
                            bf16* wt16, int cout, int cin) {
  const size_t i = (size_t)blockIdx.x * kT + threadIdx.x;
  if (i >= n) return;
  const float g = gw[i];
  const float mi = b1 * m[i] + (1.0f - b1) * g;
  const float vi = b2 * v[i] + (1.0f - b2) * g * g;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  w[i] = wi;
  if (w16) {
    w16[i] = __float2bfloat16(wi);
    const int co = (int)(i / (9 * cin));
    const int r = (int)(i % (9 * cin));
    const int tap = r / cin, ci = r % cin;
    wt16[((size_t)ci * 9 + tap) * cout + co] = __float2bfloat16(wi);
  }
}

unsigned blocks(size_t n) { return (unsigned)((n + kT - 1) / kT); }

struct Net {
  char* P;
  char* A;
  ParamLayout pl;
  ActLayout al;
  int nb, H, W;
  int* err;
  cudaStream_t s;

  template <class T>
  T* p(size_t off) const { return reinterpret_cast<T*>(P + off); }
  template <class T>
  T* a(size_t off) const { return reinterpret_cast<T*>(A + off); }
  int hl(int l) const { return H >> kLevel[l]; }
  int wl(int l) const { return W >> kLevel[l]; }
  size_t npx(int lev) const { return (size_t)level_px(nb, H, W, lev); }

  cudaError_t conv(int l, const bf16* x) {
    return conv3x3_forward(x, nb, hl(l), wl(l), kCin[l], p<bf16>(pl.w16[l]), p<float>(pl.b32[l]),
                           kCout[l], 1, a<bf16>(al.y[l]), err, s);
  }

  cudaError_t forward(const float* input, float* output) {
    cudaError_t e;
    const size_t n0 = npx(0);
    pack_input_kernel<<<blocks(n0), kT, 0, s>>>(input, (int)n0, a<bf16>(al.in8));
    if ((e = conv(0, a<bf16>(al.in8))) != cudaSuccess) return e;
    if ((e = conv(1, a<bf16>(al.y[0]))) != cudaSuccess) return e;
    const int enc_out[3] = {1, 3, 5};
    const int enc_next[3] = {2, 4, 6};
    for (int k = 0; k < 3; ++k) {
      const int l = enc_out[k];
      const size_t np = npx(k + 1) * kCout[l];
      maxpool_kernel<<<blocks(np), kT, 0, s>>>(a<bf16>(al.y[l]), nb, hl(l), wl(l), kCout[l],
                                               a<bf16>(al.pool[k]), a<uint8_t>(al.idx[k]));
      if ((e = conv(enc_next[k], a<bf16>(al.pool[k]))) != cudaSuccess) return e;
      if ((e = conv(enc_next[k] + 1, a<bf16>(al.y[enc_next[k]]))) != cudaSuccess) return e;
    }
    // decoder: (low layer, skip layer, concat buffer, first decoder layer)
    const int low[3] = {7, 9, 11}, skip[3] = {5, 3, 1}, cat[3] = {2, 1, 0}, dec[3] = {8, 10, 12};
    for (int k = 0; k < 3; ++k) {
      const int d = dec[k];
      const size_t nt = npx(kLevel[d]) * kCin[d];
      up_concat_kernel<<<blocks(nt), kT, 0, s>>>(a<bf16>(al.y[low[k]]), kCout[low[k]],
                                                 a<bf16>(al.y[skip[k]]), kCout[skip[k]], nb,
                                                 hl(d), wl(d), a<bf16>(al.cat[cat[k]]));
      if ((e = conv(d, a<bf16>(al.cat[cat[k]]))) != cudaSuccess) return e;
      if ((e = conv(d + 1, a<bf16>(al.y[d]))) != cudaSuccess) return e;
    }
    head_forward_kernel<<<blocks(n0), kT, 0, s>>>(a<bf16>(al.y[13]), (int)n0, p<float>(pl.hw),
                                                  p<float>(pl.hb), output);
    return cudaGetLastError();
  }

  // Weight and bias gradients of layer l from its input x and the gradient g
  // wrt its pre-activation; then, if dx is given, the gradient wrt x (f32).
  cudaError_t conv_back(int l, const bf16* x, const bf16* g, float* dx) {
    cudaError_t e = conv3x3_backward_weight(x, g, nb, hl(l), wl(l), kCin[l], kCout[l],
                                            p<float>(pl.gw[l]), p<float>(pl.gb[l]),
                                            a<float>(al.wpart), err, s);
    if (e != cudaSuccess || !dx) return e;
    return conv3x3_backward_data(g, nb, hl(l), wl(l), kCout[l], p<bf16>(pl.wt16[l]), kCin[l],
                                 dx, err, s);
  }

  // g_out = dx * (y_l > 0): gradient wrt the pre-activation of layer l
  void relu_grad(int l, const float* dx, bf16* g_out) {
    const size_t n = npx(kLevel[l]) * kCout[l];
    relu_grad_kernel<<<blocks(n), kT, 0, s>>>(dx, a<bf16>(al.y[l]), n, g_out);
  }

  // Loss, then gradients of every parameter (into the gw / gb / ghw / ghb slots).
  cudaError_t backward(const float* target, const float* mask, float mask_count, float* loss) {
    cudaError_t e;
    const size_t n0 = npx(0);
    const unsigned nbk = blocks(n0);
    float* red = a<float>(al.red);
    float* dx = a<float>(al.dx);
    bf16* g[2] = {a<bf16>(al.g[0]), a<bf16>(al.g[1])};
    loss_kernel<<<nbk, kT, 0, s>>>(a<float>(al.out), target, mask, (int)n0, 1.0f / mask_count,
                                   a<float>(al.dout), red);
    sum_partials_kernel<<<1, kT, 0, s>>>(red, (int)nbk, 1.0f / mask_count, loss);
    // head (1 x 1): gradient wrt the pre-activation of L13, and the head's own
    head_backward_kernel<<<nbk, kT, 0, s>>>(a<float>(al.dout), a<bf16>(al.y[13]), (int)n0,
                                            p<float>(pl.hw), g[0], red);
    column_sum_kernel<<<1, 64, 0, s>>>(red, (int)nbk, kHeadC + 1, kHeadC, p<float>(pl.ghw));
    column_sum_kernel<<<1, 64, 0, s>>>(red + kHeadC, (int)nbk, kHeadC + 1, 1, p<float>(pl.ghb));
    int c = 0;  // g[c]: gradient wrt the pre-activation of the current layer
    // decoder levels from the top: second conv d + 1, first conv d (input: concat)
    const int dec[3] = {12, 10, 8}, low[3] = {11, 9, 7}, cat[3] = {0, 1, 2};
    for (int k = 0; k < 3; ++k) {
      const int d = dec[k];
      if ((e = conv_back(d + 1, a<bf16>(al.y[d]), g[c], dx)) != cudaSuccess) return e;
      relu_grad(d, dx, g[c ^ 1]);
      c ^= 1;
      float* dcat = a<float>(al.dcat[cat[k]]);
      if ((e = conv_back(d, a<bf16>(al.cat[cat[k]]), g[c], dcat)) != cudaSuccess) return e;
      const int lo = low[k];
      const size_t n = npx(kLevel[lo]) * kCout[lo];
      up_grad_kernel<<<blocks(n), kT, 0, s>>>(dcat, kCin[d], kCout[lo], a<bf16>(al.y[lo]), nb,
                                              hl(lo), wl(lo), g[c ^ 1]);
      c ^= 1;
    }
    // g[c]: gradient wrt the pre-activation of L7. Encoder levels from the
    // bottom: second conv l + 1 (input y_l), first conv l (input: pooled level
    // above); the pooled gradient plus the skip part of the concat gradient form
    // the gradient of the level above's output.
    const int enc[4] = {6, 4, 2, 0};
    const int skip_cat[3] = {2, 1, 0};  // dcat buffer holding the skip of level 2, 1, 0
    for (int k = 0; k < 4; ++k) {
      const int l = enc[k];
      if ((e = conv_back(l + 1, a<bf16>(al.y[l]), g[c], dx)) != cudaSuccess) return e;
      relu_grad(l, dx, g[c ^ 1]);
      c ^= 1;
      if (l == 0) {
        if ((e = conv_back(0, a<bf16>(al.in8), g[c], nullptr)) != cudaSuccess) return e;
        break;
      }
      const int pool = 2 - k;  // pool[2] feeds L6, pool[1] L4, pool[0] L2
      if ((e = conv_back(l, a<bf16>(al.pool[pool]), g[c], dx)) != cudaSuccess) return e;
      const int up = l - 1;  // the encoder output that was pooled (y5, y3, y1)
      const int dcat_i = skip_cat[k];
      const int dlayer = dec[2 - k];  // the decoder conv whose concat holds this skip
      const int Ct = kCin[dlayer];
      const int C1 = Ct - kCout[up];
      const size_t n = npx(kLevel[up]) * kCout[up];
      pool_skip_grad_kernel<<<blocks(n), kT, 0, s>>>(
          dx, a<uint8_t>(al.idx[pool]), a<float>(al.dcat[dcat_i]), Ct, C1, a<bf16>(al.y[up]),
          nb, hl(up), wl(up), kCout[up], g[c ^ 1]);
      c ^= 1;
    }
    return cudaGetLastError();
  }

  cudaError_t adam(float lr, int step) {
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
    for (int l = 0; l < kLayers; ++l) {
      const size_t n = (size_t)kCout[l] * 9 * kCin[l];
      adam_kernel<<<blocks(n), kT, 0, s>>>(p<float>(pl.w32[l]), p<float>(pl.gw[l]),
                                           p<float>(pl.mw[l]), p<float>(pl.vw[l]), n, lr, b1,
                                           b2, eps, c1, c2, p<bf16>(pl.w16[l]),
                                           p<bf16>(pl.wt16[l]), kCout[l], kCin[l]);
      adam_kernel<<<blocks(kCout[l]), kT, 0, s>>>(p<float>(pl.b32[l]), p<float>(pl.gb[l]),
                                                  p<float>(pl.mb[l]), p<float>(pl.vb[l]),
                                                  kCout[l], lr, b1, b2, eps, c1, c2, nullptr,
                                                  nullptr, 0, 1);
    }
    adam_kernel<<<1, kT, 0, s>>>(p<float>(pl.hw), p<float>(pl.ghw), p<float>(pl.mhw),
                                 p<float>(pl.vhw), kHeadC, lr, b1, b2, eps, c1, c2, nullptr,
                                 nullptr, 0, 1);
    adam_kernel<<<1, kT, 0, s>>>(p<float>(pl.hb), p<float>(pl.ghb), p<float>(pl.mhb),
                                 p<float>(pl.vhb), 1, lr, b1, b2, eps, c1, c2, nullptr, nullptr,
                                 0, 1);
    return cudaGetLastError();
  }
};

// ------------------------------------------------------------------ C ABI helpers
thread_local char g_nn_error[256] = "";

int nn_fail(int code, const char* msg) {
  snprintf(g_nn_error, sizeof(g_nn_error), "%s", msg);
  return code;
}

bool shape_ok(int nb, int H, int W) {
  return nb >= 1 && H >= 64 && W >= 64 && H % 64 == 0 && W % 64 == 0;
}

}  // namespace
}  // namespace nn
}  // namespace pty

using namespace pty::nn;

extern "C" {

const char* ptycho_nn_last_error(void) { return g_nn_error; }

size_t ptycho_nn_unet_param_bytes(void) { return param_layout().total; }

int64_t ptycho_nn_unet_param_offset(int32_t layer, int32_t field) {
  const ParamLayout pl = param_layout();
  if (layer >= 0 && layer < kLayers) {
    switch (field) {
      case 0: return (int64_t)pl.w16[layer];
      case 1: return (int64_t)pl.wt16[layer];
      case 2: return (int64_t)pl.w32[layer];
      case 3: return (int64_t)pl.b32[layer];
      case 4: return (int64_t)pl.gw[layer];
      case 5: return (int64_t)pl.gb[layer];
      default: return -1;
    }
  }
  if (layer == kLayers) {
    switch (field) {
      case 2: return (int64_t)pl.hw;
      case 3: return (int64_t)pl.hb;
      case 4: return (int64_t)pl.ghw;
      case 5: return (int64_t)pl.ghb;
      default: return -1;
    }
  }
  return -1;
}

size_t ptycho_nn_unet_workspace_bytes(int32_t batch, int32_t height, int32_t width) {
  if (!shape_ok(batch, height, width)) return 0;
  return act_layout(batch, height, width).total;
}

int ptycho_nn_unet_init(void* params, uint64_t seed, void* stream) {
  if (!params) return nn_fail(PTYCHO_ERR_INVALID_ARGUMENT, "params is null");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const ParamLayout pl = param_layout();
  char* P = static_cast<char*>(params);
  cudaError_t e = cudaMemsetAsync(P, 0, pl.total, s);
  if (e != cudaSuccess) return nn_fail(PTYCHO_ERR_CUDA, cudaGetErrorString(e));
  for (int l = 0; l < kLayers; ++l) {
    const size_t n = (size_t)kCout[l] * 9 * kCin[l];
    // He initialisation for ReLU: std = sqrt(2 / fan_in); the first layer's fan
    // in counts its 2 real input channels
    const int fan_in = 9 * (l == 0 ? 2 : kCin[l]);
    init_conv_kernel<<<blocks(n), kT, 0, s>>>(
        reinterpret_cast<float*>(P + pl.w32[l]), reinterpret_cast<bf16*>(P + pl.w16[l]),
        reinterpret_cast<bf16*>(P + pl.wt16[l]), reinterpret_cast<float*>(P + pl.b32[l]),
        kCout[l], kCin[l], sqrtf(2.0f / fan_in), seed * 64 + l);
  }
  init_head_kernel<<<1, 64, 0, s>>>(reinterpret_cast<float*>(P + pl.hw), seed * 64 + kLayers);
  e = cudaGetLastError();
  if (e != cudaSuccess) return nn_fail(PTYCHO_ERR_CUDA, cudaGetErrorString(e));
  return PTYCHO_OK;
}

int ptycho_nn_unet_forward(const void* params, const float* input, int32_t batch, int32_t height,
                           int32_t width, float* output, void* workspace, size_t workspace_bytes,
                           void* stream) {
  if (!params || !input || !output || !workspace)
    return nn_fail(PTYCHO_ERR_INVALID_ARGUMENT, "params, input, output and workspace must be "
                                                "non-null");
  if (!shape_ok(batch, height, width))
    return nn_fail(PTYCHO_ERR_UNSUPPORTED, "height and width must be multiples of 64");
  const ActLayout al = act_layout(batch, height, width);
  if (workspace_bytes < al.total || reinterpret_cast<uintptr_t>(workspace) % 256)
    return nn_fail(PTYCHO_ERR_WORKSPACE, "workspace too small or not 256-byte aligned");
  Net net{static_cast<char*>(const_cast<void*>(params)), static_cast<char*>(workspace),
          param_layout(), al, batch, height, width,
          reinterpret_cast<int*>(static_cast<char*>(workspace) + al.err),
          static_cast<cudaStream_t>(stream)};
  cudaError_t e = net.forward(input, output);
  if (e != cudaSuccess) return nn_fail(PTYCHO_ERR_CUDA, cudaGetErrorString(e));
  return PTYCHO_OK;
}

int ptycho_nn_unet_train_step(void* params, const float* input, const float* target,
                              const float* mask, float mask_count, int32_t batch, int32_t height,
                              int32_t width, float learning_rate, int32_t step, float* loss,
                              void* workspace, size_t workspace_bytes, void* stream) {
  if (!params || !input || !target || !loss || !workspace)
    return nn_fail(PTYCHO_ERR_INVALID_ARGUMENT, "params, input, target, loss and workspace "
                                                "must be non-null");
  if (!shape_ok(batch, height, width))
    return nn_fail(PTYCHO_ERR_UNSUPPORTED, "height and width must be multiples of 64");
  if (step < 1 || !(mask_count > 0.0f))
    return nn_fail(PTYCHO_ERR_INVALID_ARGUMENT, "step must be >= 1 and mask_count > 0");
  const ActLayout al = act_layout(batch, height, width);
  if (workspace_bytes < al.total || reinterpret_cast<uintptr_t>(workspace) % 256)
    return nn_fail(PTYCHO_ERR_WORKSPACE, "workspace too small or not 256-byte aligned");
  Net net{static_cast<char*>(params), static_cast<char*>(workspace), param_layout(), al, batch,
          height, width, reinterpret_cast<int*>(static_cast<char*>(workspace) + al.err),
          static_cast<cudaStream_t>(stream)};
  cudaError_t e = net.forward(input, reinterpret_cast<float*>(net.A + al.out));
  if (e == cudaSuccess) e = net.backward(target, mask, mask_count, loss);
  if (e == cudaSuccess) e = net.adam(learning_rate, step);
  if (e != cudaSuccess) return nn_fail(PTYCHO_ERR_CUDA, cudaGetErrorString(e));
  return PTYCHO_OK;
}

int ptycho_nn_check(void* workspace, int32_t batch, int32_t height, int32_t width, void* stream) {
  if (!workspace || !shape_ok(batch, height, width))
    return nn_fail(PTYCHO_ERR_INVALID_ARGUMENT, "bad workspace or shape");
  const ActLayout al = act_layout(batch, height, width);
  int flag = 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int* dflag = reinterpret_cast<int*>(static_cast<char*>(workspace) + al.err);
  cudaError_t e = cudaMemcpyAsync(&flag, dflag, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return nn_fail(PTYCHO_ERR_CUDA, cudaGetErrorString(e));
  if (flag) {
    e = cudaMemsetAsync(dflag, 0, sizeof(int), s);
    return nn_fail(PTYCHO_ERR_CUDA, "a tensor-core wait timed out");
  }
  return PTYCHO_OK;
}

}  // extern "C"
