// Training data and inputs of the learned initializer (no counterpart in the
// reference):
//   lattice objects  the synthetic object model of the benchmark workloads on
//                    the device: phase = sum of Gaussian atoms (peak, sigma) on a
//                    rotated square lattice, object = exp(-0.1 phase) exp(i phase)
//   scan images      for every scan position: the ptychographic forward model
//                    (sub-pixel shifted probe times the object patch, FFT2), the
//                    far-field intensities scaled to a dose, then the virtual
//                    bright-field signal (counts inside the bright-field disc)
//                    and the centre of mass of the counts, with the Poisson noise
//                    of those sums (see scan_images_kernel); plus the blurred
//                    object phase at the position (the training target)
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

// Standard normal from two counter-based uniforms (Box-Muller).
__device__ __forceinline__ float normal01(uint64_t key) {
  const float u1 = uniform01(2 * key), u2 = uniform01(2 * key + 1);
  return sqrtf(-2.0f * __logf(u1)) * __cosf(6.2831853f * u2);
}

__global__ void lattice_objects_kernel(int count, int P, float sampling, const float* params,
                                       float sigma, float peak, float sigma_blur, float* phase,
                                       float* phase_blur, float2* object) {
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
  // the atoms, and the same atoms blurred by a Gaussian of sigma_blur (a
  // Gaussian of variance sigma^2 + sigma_blur^2 with the same integral)
  const float s2 = sigma * sigma, t2 = s2 + sigma_blur * sigma_blur;
  const float inv2s2 = 1.0f / (2.0f * s2), inv2t2 = 1.0f / (2.0f * t2);
  const float peak_t = peak * s2 / t2;
  float ph = 0.0f, pb = 0.0f;
  for (int du = -2; du <= 3; ++du)
    for (int dv = -2; dv <= 3; ++dv) {
      const float eu = qu - (mu + du) * a, ev = qv - (mv + dv) * a;
      const float d2 = eu * eu + ev * ev;
      if (d2 < 25.0f * s2) ph += peak * __expf(-d2 * inv2s2);
      if (d2 < 25.0f * t2) pb += peak_t * __expf(-d2 * inv2t2);
    }
  phase[idx] = ph;
  phase_blur[idx] = pb;
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
  // moments of the intensities: the bright-field sum, the total, the first and
  // second moments along kx and ky
  float w[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  float w2[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  for (int e = tid; e < N; e += NT) {
    const int x = e / S, y = e % S;
    const float I = c_abs2(buf[x * LD + y]);
    const float kx = (float)fint(x), ky = (float)fint(y);
    if (kx * kx + ky * ky < bf_r2) w[0] += I;
    w[1] += I;
    w[2] += I * kx;
    w[3] += I * ky;
    w2[0] += I * kx * kx;
    w2[1] += I * ky * ky;
  }
  block_sum5(w, red);
  block_sum5(w2, red);
  if (tid == 0) {
    // Counts: the intensities scaled to `dose`. Sums of independent Poisson
    // counts are Poisson with the summed means; at these doses (1e4 - 1e5 per
    // pattern) they are drawn from their normal approximations: bright field
    // N(m, m), total N(dose, dose), first moments with variances
    // sum(k^2 lambda). The centre of mass is their ratio.
    const float scale = dose / w[1];
    const uint64_t key = mix64(seed ^ mix64(((uint64_t)sc << 32) | (uint32_t)j)) * 8;
    const float mbf = w[0] * scale, mx = w[2] * scale, my = w[3] * scale;
    const float vx = w2[0] * scale, vy = w2[1] * scale;
    const float nbf = fmaxf(0.f, mbf + sqrtf(mbf) * normal01(key));
    const float ntot = fmaxf(1.f, dose + sqrtf(dose) * normal01(key + 1));
    const float nx = mx + sqrtf(vx) * normal01(key + 2);
    const float ny = my + sqrtf(vy) * normal01(key + 3);
    const size_t o = (size_t)sc * J + j;
    bf[o] = nbf;
    com_x[o] = nx / ntot;
    com_y[o] = ny / ntot;
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
                              const float* params, float sigma, float peak, float sigma_blur,
                              float* phase, float* phase_blur, void* object, void* stream) {
  if (count < 1 || object_px < 8 || !params || !phase || !phase_blur || !object ||
      !(sampling > 0.f) || !(sigma > 0.f) || !(sigma_blur >= 0.f))
    return PTYCHO_ERR_INVALID_ARGUMENT;
  const size_t total = (size_t)count * object_px * object_px;
  lattice_objects_kernel<<<(unsigned)((total + 255) / 256), 256, 0,
                           static_cast<cudaStream_t>(stream)>>>(
      count, object_px, sampling, params, sigma, peak, sigma_blur, phase, phase_blur,
      static_cast<float2*>(object));
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
