// The 256 x 256 region of interest: the per-position model as a sequence of
// batch-wide kernels over waves in global memory.
//
// A 256^2 complex64 wave is 512 KiB, more than the 227 KiB of shared memory one
// block can hold, so the fused one-block-per-position kernel of
// ptycho_position.cuh does not apply. Here the B waves of a batch live in the
// workspace's far-field buffer (scratch_f, B x 256^2 complex64: 128 MiB for 256
// positions) and each step of the model is one kernel over the whole batch:
//
//   ramps        per position: the sub-pixel shift ramps exp(-2 pi i k d) along x
//                and y (phase formed in float32, cos/sin rounded once, as in the
//                fused kernel) and the rounded origin
//   shift        W = FFT2(P) . ramp_x ramp_y
//   lines        a 2D transform is two passes of 1D transforms of length 256:
//                16 lines of one position per block staged in shared memory and
//                transformed by the radix-16 x 16 Stockham passes of
//                fft_smem.cuh. Rows first (along y, as the fused kernel), then
//                columns; a column block moves 16 adjacent columns, so every
//                row segment it reads or writes is 128 bytes.
//   overlap      P_s = W / N (stashed in st_probe), W = P_s O_patch
//   projection   F = W: chunk partials of sum (A - |F|)^2, W = A F/|F| - F
//                (detector mask applied to F and to the result)
//   adjoint      chi = W / N: conj(P_s) chi (Re(-i conj(O) conj(P) chi) for a
//                potential) and |P_s|^2 for the object, conj(O) chi for the
//                probe; |O|^2 is gathered by the probe reduction from the object
//
// then the deterministic reductions and updates of ptycho_reduce.cu, as for the
// fused path. The operators are those of ptycho_position.cuh (reference:
// py4DSTEM 0.14.18 ptychographic_methods.py:1482-1527 overlap, :1576-1640
// Fourier projection, :1818-1908 adjoint). Gradient descent of the
// single-slice, single-probe model, the forward-only pass (self-consistency
// errors), the object gradient, the probe-overlap map and the probe
// centre-of-mass and aperture constraints run at 256^2; the C ABI refuses the
// other models at this size.
//
// Scratch inside the workspace: the ramps (B x 512 float2) sit in st_nobj and
// the error partials (B x 32 floats) in st_nprobe, both free until the adjoint
// writes st_nobj (the ramps are dead by then) and never read as |O|^2 (the
// probe reduction of this model gathers |O|^2 from the object).
#include <cuda_runtime.h>

#include "ptycho_position.cuh"

namespace pty {
namespace {

constexpr int S = 256;
constexpr int N = S * S;
constexpr int kLines = 16;        // lines per block of a transform pass
constexpr int kLineThreads = 256;
constexpr int kLD = S + 1;        // shared-memory pitch of a staged line
constexpr int kEwThreads = 256;   // elementwise kernels: 8 samples per thread
constexpr int kPer = 8;
constexpr int kChunk = kEwThreads * kPer;
constexpr int kChunks = N / kChunk;  // elementwise blocks per position (32)
static_assert(N % kChunk == 0, "chunking");

// Object index of patch pixel (x, y) for a position with rounded origin r:
// ((r - S/2) mod P + (x + S/2) mod S) mod P, as obj_x / obj_y of the fused kernel.
__device__ __forceinline__ size_t patch_index(const BatchArgs& a, int2 r, int x, int y) {
  int ox = pmod(r.x - S / 2, a.Px) + (x + S / 2) % S;
  int oy = pmod(r.y - S / 2, a.Py) + (y + S / 2) % S;
  if (ox >= a.Px) ox -= a.Px;
  if (oy >= a.Py) oy -= a.Py;
  return (size_t)ox * a.Py + oy;
}

__device__ __forceinline__ float2 patch_value(const BatchArgs& a, int2 r, int x, int y) {
  const size_t idx = patch_index(a, r, x, y);
  if (a.potential) {
    float sv, cv;
    sincosf(reinterpret_cast<const float*>(a.object)[idx], &sv, &cv);
    return make_float2(cv, sv);
  }
  return reinterpret_cast<const float2*>(a.object)[idx];
}

// One block per position: ramps[b] = (ramp_x[256], ramp_y[256]) and the rounded
// origin. `direct` positions are indexed by b (probe overlap), else by pos_rows.
__global__ void __launch_bounds__(S) staged_ramps_kernel(BatchArgs a, float2* ramps, int direct) {
  const int b = blockIdx.x;
  const int prow = (!direct && a.pos_rows) ? a.pos_rows[b] : b;
  const float posx = finite_or_zero(a.positions[2 * prow]);
  const float posy = finite_or_zero(a.positions[2 * prow + 1]);
  const float rx = rintf(posx);  // numpy.round: half to even
  const float ry = rintf(posy);
  const float dx = posx - rx, dy = posy - ry;
  const int i = threadIdx.x;
  const float k = (float)fint(i, S) / (float)S;
  ramps[(size_t)b * 2 * S + i] = cis_rounded(__fmul_rn(__fmul_rn(-6.2831855f, k), dx));
  ramps[(size_t)b * 2 * S + S + i] = cis_rounded(__fmul_rn(__fmul_rn(-6.2831855f, k), dy));
  if (i == 0) a.pos_round[b] = make_int2((int)rx, (int)ry);
}

// W[b] = spec . ramp_x ramp_y (grid: B x kChunks)
__global__ void __launch_bounds__(kEwThreads) staged_shift_kernel(const float2* __restrict__ spec,
                                                                  const float2* __restrict__ ramps,
                                                                  float2* W) {
  const int b = blockIdx.x;
  const float2* r = ramps + (size_t)b * 2 * S;
  const int e0 = blockIdx.y * kChunk + threadIdx.x;
#pragma unroll
  for (int i = 0; i < kPer; ++i) {
    const int e = e0 + i * kEwThreads;
    W[(size_t)b * N + e] = c_mul(__ldg(spec + e), c_mul(r[e / S], r[S + e % S]));
  }
}

// One pass of 1D transforms of length 256 over 16 lines of wave blockIdx.x, rows
// (along y) or columns (along x); the results are multiplied by `scale`.
template <int DIR, bool ROWS>
__global__ void __launch_bounds__(kLineThreads) staged_lines_kernel(float2* W, float scale) {
  __shared__ float2 buf[kLines * kLD];
  __shared__ float2 tw[S];
  float2* w = W + (size_t)blockIdx.x * N;
  const int l0 = blockIdx.y * kLines;
  fill_twiddles<S, kLineThreads>(tw);
  if (ROWS) {
    for (int e = threadIdx.x; e < kLines * S; e += kLineThreads) {
      const int l = e / S, j = e % S;
      buf[l * kLD + j] = w[(size_t)(l0 + l) * S + j];
    }
  } else {
    // column l0 + l, element j is w[j * S + l0 + l]: 16 adjacent columns per row
    for (int e = threadIdx.x; e < kLines * S; e += kLineThreads) {
      const int j = e / kLines, l = e % kLines;
      buf[l * kLD + j] = w[(size_t)j * S + l0 + l];
    }
  }
  __syncthreads();
  Schedule<S>::template run<kLines, kLineThreads, DIR>(buf, kLD, 1, tw);
  if (ROWS) {
    for (int e = threadIdx.x; e < kLines * S; e += kLineThreads) {
      const int l = e / S, j = e % S;
      w[(size_t)(l0 + l) * S + j] = c_scale(buf[l * kLD + j], scale);
    }
  } else {
    for (int e = threadIdx.x; e < kLines * S; e += kLineThreads) {
      const int j = e / kLines, l = e % kLines;
      w[(size_t)j * S + l0 + l] = c_scale(buf[l * kLD + j], scale);
    }
  }
}

// FFT2 (DIR -1) or unnormalised inverse (DIR +1) of `count` waves in place,
// times `scale`.
template <int DIR>
cudaError_t fft2_waves(float2* W, int count, float scale, cudaStream_t s) {
  const dim3 grid(count, S / kLines);
  staged_lines_kernel<DIR, true><<<grid, kLineThreads, 0, s>>>(W, 1.0f);
  staged_lines_kernel<DIR, false><<<grid, kLineThreads, 0, s>>>(W, scale);
  return cudaGetLastError();
}

// P_s = W / N (stashed), W = P_s O_patch
__global__ void __launch_bounds__(kEwThreads) staged_overlap_kernel(BatchArgs a, float2* W) {
  const int b = blockIdx.x;
  const int2 r = a.pos_round[b];
  const float invN = 1.0f / (float)N;
  const int e0 = blockIdx.y * kChunk + threadIdx.x;
  float2 ov[kPer];
#pragma unroll
  for (int i = 0; i < kPer; ++i) {
    const int e = e0 + i * kEwThreads;
    ov[i] = patch_value(a, r, e / S, e % S);
  }
#pragma unroll
  for (int i = 0; i < kPer; ++i) {
    const size_t k = (size_t)b * N + e0 + i * kEwThreads;
    const float2 p = c_scale(W[k], invN);
    a.st_probe[k] = p;
    W[k] = c_mul(p, ov[i]);
  }
}

// Chunk partials of sum (A - |F|)^2; W = A F/|F| - F (masked) unless forward only.
__global__ void __launch_bounds__(kEwThreads) staged_projection_kernel(BatchArgs a, float2* W,
                                                                       float* err_part) {
  __shared__ float red[kEwThreads / 32];
  const int b = blockIdx.x;
  const int arow = a.amp_rows ? a.amp_rows[b] : b;
  const float* amp = a.amplitudes + (size_t)arow * N;
  const int e0 = blockIdx.y * kChunk + threadIdx.x;
  float av[kPer];
#pragma unroll
  for (int i = 0; i < kPer; ++i) av[i] = __ldg(amp + e0 + i * kEwThreads);
  float err = 0.0f;
#pragma unroll
  for (int i = 0; i < kPer; ++i) {
    const int e = e0 + i * kEwThreads;
    const size_t k = (size_t)b * N + e;
    float2 f = W[k];
    const float mk = a.det_mask ? a.det_mask[e] : 1.0f;
    if (a.det_mask) f = c_scale(f, mk);
    const float af = c_abs(f);
    const float A = av[i];
    const float d = A - af;
    err += d * d;
    if (!a.forward_only) {
      const float q = af > 0.0f ? A / af : 0.0f;
      float2 rr = af > 0.0f ? make_float2(fmaf(f.x, q, -f.x), fmaf(f.y, q, -f.y))
                            : c_sub(make_float2(A, 0.0f), f);
      if (a.det_mask) rr = c_scale(rr, mk);
      W[k] = rr;
    }
  }
  const float t = block_sum<kEwThreads>(err, red);
  if (threadIdx.x == 0) err_part[(size_t)b * kChunks + blockIdx.y] = t;
}

// err[b] = the position's chunk partials summed in order; NaN for a non-finite
// position (reported as PTYCHO_ERR_NONFINITE).
__global__ void staged_error_kernel(BatchArgs a, const float* err_part) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.B) return;
  float t = 0.0f;
  for (int c = 0; c < kChunks; ++c) t += err_part[(size_t)b * kChunks + c];
  const int prow = a.pos_rows ? a.pos_rows[b] : b;
  const bool ok = isfinite(a.positions[2 * prow]) && isfinite(a.positions[2 * prow + 1]);
  a.err[b] = ok ? t : __int_as_float(0x7fc00000);
}

// chi = W / N: object terms and |P_s|^2, probe term conj(O) chi
__global__ void __launch_bounds__(kEwThreads) staged_adjoint_kernel(BatchArgs a,
                                                                    const float2* W) {
  const int b = blockIdx.x;
  const int2 r = a.pos_round[b];
  const float invN = 1.0f / (float)N;
  const int e0 = blockIdx.y * kChunk + threadIdx.x;
  float2 ov[kPer];
#pragma unroll
  for (int i = 0; i < kPer; ++i) {
    const int e = e0 + i * kEwThreads;
    ov[i] = patch_value(a, r, e / S, e % S);
  }
#pragma unroll
  for (int i = 0; i < kPer; ++i) {
    const size_t k = (size_t)b * N + e0 + i * kEwThreads;
    const float2 chi = c_scale(W[k], invN);
    const float2 p = a.st_probe[k];
    a.st_obj[k] = object_term(a.potential, ov[i], p, chi);
    a.st_nobj[k] = c_abs2(p);
    a.st_probe[k] = c_conj_mul(ov[i], chi);
  }
}

// |P_b|^2 = |W / N|^2, abs() then square as numpy forms it
__global__ void __launch_bounds__(kEwThreads) staged_intensity_kernel(BatchArgs a,
                                                                      const float2* W) {
  const int b = blockIdx.x;
  const float invN = 1.0f / (float)N;
  const int e0 = blockIdx.y * kChunk + threadIdx.x;
#pragma unroll
  for (int i = 0; i < kPer; ++i) {
    const size_t k = (size_t)b * N + e0 + i * kEwThreads;
    const float2 p = c_scale(W[k], invN);
    const float av = hypotf(p.x, p.y);
    a.st_nobj[k] = av * av;
  }
}

__global__ void copy_waves_kernel(const float2* __restrict__ src, float2* dst, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[i];
}

// W[m] *= ramp(-CoM) for the probe centre-of-mass constraint, the CoM from
// probe_com_kernel cast to float32 as the reference's shift does.
__global__ void __launch_bounds__(kEwThreads) staged_com_ramp_kernel(BatchArgs a, float2* W) {
  __shared__ float2 rx[S], ry[S];
  const float dx = (float)(-a.com[0]);
  const float dy = (float)(-a.com[1]);
  for (int i = threadIdx.x; i < S; i += kEwThreads) {
    const float k = (float)fint(i, S) / (float)S;
    rx[i] = cis_rounded(__fmul_rn(__fmul_rn(-6.2831855f, k), dx));
    ry[i] = cis_rounded(__fmul_rn(__fmul_rn(-6.2831855f, k), dy));
  }
  __syncthreads();
  const int e0 = blockIdx.y * kChunk + threadIdx.x;
#pragma unroll
  for (int i = 0; i < kPer; ++i) {
    const int e = e0 + i * kEwThreads;
    const size_t k = (size_t)blockIdx.x * N + e;
    W[k] = c_mul(W[k], c_mul(rx[e / S], ry[e % S]));
  }
}

// out[0] = sum |p|^2 over one wave (abs() then square), one 1024-thread block:
// thread partials, then a fixed shuffle tree and warp order.
__global__ void __launch_bounds__(1024) staged_power_kernel(const float2* p, float* out) {
  __shared__ float red[32];
  float part = 0.0f;
  for (int e = threadIdx.x; e < N; e += 1024) {
    const float2 v = p[e];
    const float av = hypotf(v.x, v.y);
    part += av * av;
  }
  const float t = block_sum<1024>(part, red);
  if (threadIdx.x == 0) *out = t;
}

// F <- aperture . exp(i angle F)
__global__ void __launch_bounds__(kEwThreads) staged_aperture_kernel(float2* F,
                                                                     const float* aperture) {
  const int e0 = blockIdx.y * kChunk + threadIdx.x;
#pragma unroll
  for (int i = 0; i < kPer; ++i) {
    const int e = e0 + i * kEwThreads;
    const float2 f = F[e];
    float sn, cs;
    sincosf(atan2f(f.y, f.x), &sn, &cs);
    const float ap = aperture[e];
    F[e] = make_float2(cs * ap, sn * ap);
  }
}

// p *= sqrt(pw[0] / pw[1])
__global__ void __launch_bounds__(kEwThreads) staged_rescale_kernel(float2* p, const float* pw) {
  const float k = sqrtf(pw[0] / pw[1]);
  const int e0 = blockIdx.y * kChunk + threadIdx.x;
#pragma unroll
  for (int i = 0; i < kPer; ++i) p[e0 + i * kEwThreads] = c_scale(p[e0 + i * kEwThreads], k);
}

}  // namespace

bool staged_roi(int Sx, int Sy) { return Sx == S && Sy == S; }

bool staged_batch_supported(const BatchArgs& a) {
  return a.T == 1 && a.M == 1 && !a.projection && !a.mixed_formula && !a.keep_farfield &&
         !a.exact_probe_grad && !a.staging_t;
}

cudaError_t launch_staged_spectrum(const BatchArgs& a, cudaStream_t s) {
  const size_t n = (size_t)a.M * N;
  copy_waves_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a.probe, a.probe_spec, n);
  return fft2_waves<-1>(a.probe_spec, a.M, 1.0f, s);
}

cudaError_t launch_staged_positions(const BatchArgs& a, cudaStream_t s) {
  if (!staged_batch_supported(a)) return cudaErrorNotSupported;
  float2* ramps = reinterpret_cast<float2*>(a.st_nobj);
  float* err_part = a.st_nprobe;
  float2* W = a.scratch_f;
  const dim3 ew(a.B, kChunks);
  staged_ramps_kernel<<<a.B, S, 0, s>>>(a, ramps, 0);
  staged_shift_kernel<<<ew, kEwThreads, 0, s>>>(a.probe_spec, ramps, W);
  cudaError_t e = fft2_waves<+1>(W, a.B, 1.0f, s);
  if (e != cudaSuccess) return e;
  staged_overlap_kernel<<<ew, kEwThreads, 0, s>>>(a, W);
  if ((e = fft2_waves<-1>(W, a.B, 1.0f, s)) != cudaSuccess) return e;
  staged_projection_kernel<<<ew, kEwThreads, 0, s>>>(a, W, err_part);
  staged_error_kernel<<<(a.B + 255) / 256, 256, 0, s>>>(a, err_part);
  if (a.forward_only) return cudaGetLastError();
  if ((e = fft2_waves<+1>(W, a.B, 1.0f, s)) != cudaSuccess) return e;
  staged_adjoint_kernel<<<ew, kEwThreads, 0, s>>>(a, W);
  return cudaGetLastError();
}

cudaError_t launch_staged_intensity(const BatchArgs& a, cudaStream_t s) {
  // ramps in st_obj, waves in scratch_f, |P_b|^2 into st_nobj
  float2* ramps = a.st_obj;
  float2* W = a.scratch_f;
  const dim3 ew(a.B, kChunks);
  staged_ramps_kernel<<<a.B, S, 0, s>>>(a, ramps, 1);
  staged_shift_kernel<<<ew, kEwThreads, 0, s>>>(a.probe_spec, ramps, W);
  cudaError_t e = fft2_waves<+1>(W, a.B, 1.0f, s);
  if (e != cudaSuccess) return e;
  staged_intensity_kernel<<<ew, kEwThreads, 0, s>>>(a, W);
  return cudaGetLastError();
}

cudaError_t launch_staged_probe_shift(const BatchArgs& a, cudaStream_t s) {
  // every mode through the probe spectrum buffer (free between batches)
  cudaError_t e = launch_staged_spectrum(a, s);
  if (e != cudaSuccess) return e;
  staged_com_ramp_kernel<<<dim3(a.M, kChunks), kEwThreads, 0, s>>>(a, a.probe_spec);
  if ((e = fft2_waves<+1>(a.probe_spec, a.M, 1.0f / (float)N, s)) != cudaSuccess) return e;
  const size_t n = (size_t)a.M * N;
  copy_waves_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a.probe_spec, a.probe, n);
  return cudaGetLastError();
}

cudaError_t launch_staged_aperture(const BatchArgs& a, cudaStream_t s) {
  // mode 0 in place; its power before and after in two stream-ordered floats
  float* pw = nullptr;
  cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&pw), 2 * sizeof(float), s);
  if (e != cudaSuccess) return e;
  float2* p = a.probe;
  staged_power_kernel<<<1, 1024, 0, s>>>(p, pw);
  if ((e = fft2_waves<-1>(p, 1, 1.0f, s)) == cudaSuccess) {
    staged_aperture_kernel<<<dim3(1, kChunks), kEwThreads, 0, s>>>(p, a.aperture);
    if ((e = fft2_waves<+1>(p, 1, 1.0f / (float)N, s)) == cudaSuccess) {
      staged_power_kernel<<<1, 1024, 0, s>>>(p, pw + 1);
      staged_rescale_kernel<<<dim3(1, kChunks), kEwThreads, 0, s>>>(p, pw);
      e = cudaGetLastError();
    }
  }
  const cudaError_t f = cudaFreeAsync(pw, s);
  return e != cudaSuccess ? e : f;
}

}  // namespace pty
