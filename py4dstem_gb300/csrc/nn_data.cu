// Training data and inputs of the learned initializer (no counterpart in the
// reference):
//   lattice objects  the synthetic object model of the benchmark workloads on
//                    the device: phase = sum of Gaussian atoms (peak, sigma) on a
//                    rotated square lattice, object = exp(-0.1 phase) exp(i phase)
//   scan images      for every scan position: the ptychographic forward model
//                    (sub-pixel shifted probe times the object patch, FFT2), the
//                    far-field intensities scaled to a dose and drawn with Poisson
//                    noise, then the virtual bright-field signal (counts inside
//                    the bright-field disc) and the centre of mass of the counts;
//                    plus the object phase at the position (the training target)
//   virtual images   the same bright-field sum and centre of mass from measured
//                    (preprocessed) amplitudes, the network's input at inference
// The forward model uses the shared-memory FFT of the reconstruction kernels
// (fft_smem.cuh) with the same conventions (corner-centred detector, patch
// rows (round(x) + fftfreq) mod P).
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/ptycho_gb300.h"
#include "fft_smem.cuh"
#include "ptycho_internal.h"

namespace pty {
namespace nn_data {
namespace {

constexpr int S = 128;  // detector / ROI edge of the scan-image kernel
constexpr int N = S * S;
constexpr int NT = 1024;
constexpr int LD = S + 1;

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ float uniform01(uint64_t key) {
  return ((mix64(key) >> 40) + 0.5f) * (1.0f / 16777216.0f);
}

// Poisson(lambda): multiplication method below 12, rounded normal approximation
// N(lambda, lambda) above (training data only; documented approximation).
__device__ __forceinline__ float poisson(float lam, uint64_t key) {
  if (!(lam > 0.0f)) return 0.0f;
  if (lam < 12.0f) {
    const float L = __expf(-lam);
    float p = 1.0f;
    int k = -1;
    uint64_t j = 0;
    do {
      ++k;
      p *= uniform01(key * 64 + j++);
    } while (p > L && k < 64);
    return (float)k;
  }
  const float u1 = uniform01(key * 64 + 62), u2 = uniform01(key * 64 + 63);
  const float z = sqrtf(-2.0f * __logf(u1)) * __cosf(6.2831853f * u2);
  return fmaxf(0.0f, rintf(lam + sqrtf(lam) * z));
}

__global__ void lattice_objects_kernel(int count, int P, float sampling, const float* params,
                                       float sigma, float peak, float* phase, float2* object) {
  const size_t total = (size_t)count * P * P;
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= total) return;
  const int s = (int)(idx / ((size_t)P * P));
  const int r = (int)(idx % ((size_t)P * P));
  const int i = r / P, j = r % P;
  const float a = params[5 * s + 0];
  const float th = params[5 * s + 1];
  const float ox = params[5 * s + 2], oy = params[5 * s + 3];
  const float c = cosf(th), sn = sinf(th);
  const float cx = 0.5f * P * sampling, cy = cx;
  const float px = i * sampling - cx, py = j * sampling - cy;
  // lattice coordinates of the pixel: q = R(-theta) p - offset
  const float qu = c * px + sn * py - ox;
  const float qv = -sn * px + c * py - oy;
  const int mu = (int)floorf(qu / a), mv = (int)floorf(qv / a);
  const float inv2s2 = 1.0f / (2.0f * sigma * sigma);
  float ph = 0.0f;
  for (int du = -1; du <= 2; ++du)
    for (int dv = -1; dv <= 2; ++dv) {
      const float eu = qu - (mu + du) * a, ev = qv - (mv + dv) * a;
      const float d2 = eu * eu + ev * ev;
      if (d2 < 25.0f * sigma * sigma) ph += peak * __expf(-d2 * inv2s2);
    }
  phase[idx] = ph;
  const float amp = __expf(-0.1f * ph);
  float sv, cv;
  sincosf(ph, &sv, &cv);
  object[idx] = make_float2(amp * cv, amp * sv);
}

// Block-wide sums of 5 floats in a fixed order; result valid in thread 0.
__device__ __forceinline__ void block_sum5(float (&v)[5], float (*red)[NT / 32]) {
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    float x = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) red[k][threadIdx.x >> 5] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      float t = 0.0f;
      for (int w = 0; w < NT / 32; ++w) t += red[k][w];
      v[k] = t;
    }
  }
  __syncthreads();
}

__device__ __forceinline__ int fint(int i) { return i < S / 2 ? i : i - S; }

// One block per (position, scan). spectra: (scans, N) FFT2 of each scan's probe;
// objects (scans, P, P); phase (scans, P, P); positions (scans, J, 2) pixels.
// Outputs (scans, J): bf, com_x, com_y, target.
__global__ void __launch_bounds__(NT, 1)
    scan_images_kernel(int J, int P, const float2* spectra, const float2* objects,
                       const float* phase, const float* positions, float dose, float bf_r2,
                       uint64_t seed, float* bf, float* com_x, float* com_y, float* target) {
  extern __shared__ float4 smem4[];
  float2* buf = reinterpret_cast<float2*>(smem4);
  float2* twx = buf + S * LD;
  float2* twy = twx + S;
  float2* rpx = twy + S;
  float2* rpy = rpx + S;
  __shared__ float red[5][NT / 32];
  __shared__ float total_s;
  const int j = blockIdx.x;
  const int sc = blockIdx.y;
  const int tid = threadIdx.x;
  const float* pos = positions + ((size_t)sc * J + j) * 2;
  const float posx = pos[0], posy = pos[1];
  const float rx = rintf(posx), ry = rintf(posy);
  const float dx = posx - rx, dy = posy - ry;
  fill_twiddles<S, NT>(twx);
  fill_twiddles<S, NT>(twy);
  for (int i = tid; i < S; i += NT) {
    const float k = (float)fint(i) / (float)S;
    rpx[i] = cis_rounded(__fmul_rn(__fmul_rn(-6.2831855f, k), dx));
    rpy[i] = cis_rounded(__fmul_rn(__fmul_rn(-6.2831855f, k), dy));
  }
  __syncthreads();
  const float2* spec = spectra + (size_t)sc * N;
  for (int e = tid; e < N; e += NT) {
    const int x = e / S, y = e % S;
    buf[x * LD + y] = c_mul(spec[e], c_mul(rpx[x], rpy[y]));
  }
  __syncthreads();
  fft2d<S, S, NT, +1>(buf, twx, twy);
  const float2* obj = objects + (size_t)sc * P * P;
  const int bx = ((int)rx - S / 2) % P, by = ((int)ry - S / 2) % P;
  const float invN = 1.0f / (float)N;
  for (int e = tid; e < N; e += NT) {
    const int x = e / S, y = e % S;
    int ox = bx + (x + S / 2) % S;
    int oy = by + (y + S / 2) % S;
    ox = ((ox % P) + P) % P;
    oy = ((oy % P) + P) % P;
    buf[x * LD + y] = c_mul(c_scale(buf[x * LD + y], invN), obj[(size_t)ox * P + oy]);
  }
  __syncthreads();
  fft2d<S, S, NT, -1>(buf, twx, twy);
  float v[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  for (int e = tid; e < N; e += NT) v[0] += c_abs2(buf[(e / S) * LD + e % S]);
  block_sum5(v, red);
  if (tid == 0) total_s = v[0];
  __syncthreads();
  const float scale = dose / total_s;
  const uint64_t key0 = mix64(seed ^ mix64(((uint64_t)sc << 32) | (uint32_t)j));
  float w[5] = {0.f, 0.f, 0.f, 0.f, 0.f};  // bf, sum, sum kx, sum ky
  for (int e = tid; e < N; e += NT) {
    const int x = e / S, y = e % S;
    const float n = poisson(c_abs2(buf[x * LD + y]) * scale, key0 + (uint64_t)e);
    const float kx = (float)fint(x), ky = (float)fint(y);
    if (kx * kx + ky * ky < bf_r2) w[0] += n;
    w[1] += n;
    w[2] += n * kx;
    w[3] += n * ky;
  }
  block_sum5(w, red);
  if (tid == 0) {
    const size_t o = (size_t)sc * J + j;
    bf[o] = w[0];
    com_x[o] = w[1] > 0.f ? w[2] / w[1] : 0.f;
    com_y[o] = w[1] > 0.f ? w[3] / w[1] : 0.f;
    // bilinear phase at the (continuous) position, periodic
    const float* ph = phase + (size_t)sc * P * P;
    const float fx = floorf(posx), fy = floorf(posy);
    const float tx = posx - fx, ty = posy - fy;
    const int x0 = (((int)fx % P) + P) % P, y0 = (((int)fy % P) + P) % P;
    const int x1 = (x0 + 1) % P, y1 = (y0 + 1) % P;
    target[o] = (1.f - tx) * ((1.f - ty) * ph[(size_t)x0 * P + y0] + ty * ph[(size_t)x0 * P + y1]) +
                tx * ((1.f - ty) * ph[(size_t)x1 * P + y0] + ty * ph[(size_t)x1 * P + y1]);
  }
}

// One block (256 threads) per pattern of corner-centred amplitudes (sx, sy):
// intensities A^2, their sum inside the bright-field disc and centre of mass.
__global__ void virtual_images_kernel(const float* amps, int sx, int sy, float bf_r2, float* bf,
                                      float* com_x, float* com_y) {
  __shared__ float red[4][8];
  const float* a = amps + (size_t)blockIdx.x * sx * sy;
  float v[4] = {0.f, 0.f, 0.f, 0.f};
  for (int e = threadIdx.x; e < sx * sy; e += 256) {
    const int x = e / sy, y = e % sy;
    const float kx = (float)(x < (sx + 1) / 2 ? x : x - sx);
    const float ky = (float)(y < (sy + 1) / 2 ? y : y - sy);
    const float I = a[e] * a[e];
    if (kx * kx + ky * ky < bf_r2) v[0] += I;
    v[1] += I;
    v[2] += I * kx;
    v[3] += I * ky;
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    float x = v[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) red[k][threadIdx.x >> 5] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float t[4];
    for (int k = 0; k < 4; ++k) {
      t[k] = 0.f;
      for (int w = 0; w < 8; ++w) t[k] += red[k][w];
    }
    bf[blockIdx.x] = t[0];
    com_x[blockIdx.x] = t[1] > 0.f ? t[2] / t[1] : 0.f;
    com_y[blockIdx.x] = t[1] > 0.f ? t[3] / t[1] : 0.f;
  }
}

}  // namespace
}  // namespace nn_data
}  // namespace pty

using namespace pty::nn_data;

extern "C" {

int ptycho_nn_lattice_objects(int32_t count, int32_t object_px, float sampling,
                              const float* params, float sigma, float peak, float* phase,
                              void* object, void* stream) {
  if (count < 1 || object_px < 8 || !params || !phase || !object || !(sampling > 0.f) ||
      !(sigma > 0.f))
    return PTYCHO_ERR_INVALID_ARGUMENT;
  const size_t total = (size_t)count * object_px * object_px;
  lattice_objects_kernel<<<(unsigned)((total + 255) / 256), 256, 0,
                           static_cast<cudaStream_t>(stream)>>>(
      count, object_px, sampling, params, sigma, peak, phase, static_cast<float2*>(object));
  return cudaGetLastError() == cudaSuccess ? PTYCHO_OK : PTYCHO_ERR_CUDA;
}

int ptycho_nn_scan_images(int32_t scans, int32_t positions, int32_t object_px,
                          const void* spectra, const void* objects, const float* phase,
                          const float* positions_px, float dose, float bf_radius_px,
                          uint64_t seed, float* bf, float* com_x, float* com_y, float* target,
                          void* stream) {
  if (scans < 1 || positions < 1 || object_px < S || !spectra || !objects || !phase ||
      !positions_px || !bf || !com_x || !com_y || !target || !(dose > 0.f))
    return PTYCHO_ERR_INVALID_ARGUMENT;
  const int smem = (int)(sizeof(float2) * (size_t)(S * LD + 4 * S));
  cudaError_t e = pty::ensure_smem_limit(reinterpret_cast<const void*>(scan_images_kernel), smem);
  if (e != cudaSuccess) return PTYCHO_ERR_CUDA;
  scan_images_kernel<<<dim3(positions, scans), NT, smem, static_cast<cudaStream_t>(stream)>>>(
      positions, object_px, static_cast<const float2*>(spectra),
      static_cast<const float2*>(objects), phase, positions_px, dose,
      bf_radius_px * bf_radius_px, seed, bf, com_x, com_y, target);
  return cudaGetLastError() == cudaSuccess ? PTYCHO_OK : PTYCHO_ERR_CUDA;
}

int ptycho_nn_virtual_images(const float* amplitudes, int32_t count, int32_t sx, int32_t sy,
                             float bf_radius_px, float* bf, float* com_x, float* com_y,
                             void* stream) {
  if (!amplitudes || count < 1 || sx < 1 || sy < 1 || !bf || !com_x || !com_y)
    return PTYCHO_ERR_INVALID_ARGUMENT;
  virtual_images_kernel<<<count, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      amplitudes, sx, sy, bf_radius_px * bf_radius_px, bf, com_x, com_y);
  return cudaGetLastError() == cudaSuccess ? PTYCHO_OK : PTYCHO_ERR_CUDA;
}

}  // extern "C"
