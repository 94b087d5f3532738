// The per-position model as a sequence of batch-wide kernels over waves in
// global memory (the "staged" path), for what the fused one-block-per-position
// kernel of ptycho_position.cuh cannot hold or does not do:
//
//  * the 256 x 256 region of interest: a 256^2 complex64 wave is 512 KiB, more
//    than the 227 KiB of shared memory one block can hold;
//  * a far field resampled to a detector of another shape (the reference's
//    region_of_interest_shape, ptychographic_methods.py:1601-1631): the Fourier
//    projection then runs on the detector grid, between two resampling steps.
//
// The waves of a batch (B x M, one per position and probe mode) live in the
// workspace's far-field buffer and every step of the model is one kernel over
// the whole batch:
//
//   ramps        per position: the sub-pixel shift ramps exp(-2 pi i k d) along x
//                and y (phase formed in float32, cos/sin rounded once, as in the
//                fused kernel) and the rounded origin
//   shift        W_m = FFT2(P_m) . ramp_x ramp_y
//   lines        a 2D transform is two passes of 1D transforms: 16 lines of one
//                wave per block staged in shared memory and transformed by the
//                Stockham passes of fft_smem.cuh, rows (along y) first, then
//                columns (a column block moves 16 adjacent columns, so each row
//                segment it reads or writes is contiguous)
//   overlap      P_{s,m} = W_m / N (stashed), W_m = P_{s,m} O_s patch; between
//                slices W_m <- IFFT2(FFT2(W_m) H_s)
//   projection   single probe: err = sum (A - |F|)^2, G = A F/|F| - F; mixed
//                state: |F|_tot = sqrt(sum_m |F_m|^2), G_m = (A/|F|_tot) F_m - F_m;
//                the detector mask multiplies F and G. With resampling, F_m is
//                first interpolated onto the detector grid and G_m back onto the
//                region of interest (bilinear_resample below)
//   adjoint      chi_m = IFFT2(G_m), walking back through the slices: object term
//                sum_m conj(P_{s,m}) chi_{s,m} (Re(-i conj(O) conj(P) chi) for a
//                potential) and sum_m |P_{s,m}|^2, then chi_m conj(O_s) propagated
//                back by conj(H); at slice 0 the probe term conj(O_0) chi_m
//
// then the deterministic reductions and updates of ptycho_reduce.cu, as for the
// fused path. The operators are those of ptycho_position.cuh (reference:
// py4DSTEM 0.14.18 ptychographic_methods.py:1482-1527 and 2300-2351 overlap,
// :1576-1635 and 2742-2804 Fourier projection, :1818-1908, 2353-2458 and
// 2906-3000 adjoint). Gradient descent of every model (single slice,
// multislice, mixed state, both), the forward-only pass (self-consistency
// errors) and the object gradient run here; projection sets, position
// correction and the exact probe gradient are refused by the C ABI for the
// batches this path runs.
//
// bilinear_resample (utils.py:2347-2428) calls scipy.ndimage.zoom(order=1,
// mode="grid-wrap", grid_mode=True) on the complex far field. SciPy zooms a
// complex array as its real and imaginary parts without passing grid_mode on,
// so the interpolation it performs maps output index k to input coordinate
// k (n_in - 1) / (n_out - 1) (end points aligned), linear between the two
// neighbouring samples; the result is divided by the ratio of the two grids'
// pixel counts (conserve_array_sums). The same mapping is used here, with the
// weights formed in float64 and the sums in float32.
//
// Workspace use: the ramps sit in st_nobj (dead before the adjoint writes it),
// the error partials in err_part, the detector-grid far fields (resampling
// only) in det_f. The stash P_{s,m} is st_probe (single slice), st_obj
// (multislice, one probe; overwritten by the object term of the same element)
// or st_pm (mixed-state multislice), as in the fused kernel.
#include <cuda_runtime.h>

#include "ptycho_position.cuh"

namespace pty {
namespace {

constexpr int kLines = 16;        // lines per block of a transform pass
constexpr int kLineThreads = 256;
constexpr int kEwThreads = 256;   // elementwise kernels: up to 8 samples per thread
constexpr int kPer = 8;
constexpr int kChunk = kEwThreads * kPer;

int chunks_of(int n) { return (n + kChunk - 1) / kChunk; }

__device__ __forceinline__ size_t patch_index(const BatchArgs& a, int s, int2 r, int x, int y) {
  int ox = pmod(r.x - a.Sx / 2, a.Px) + (x + a.Sx / 2) % a.Sx;
  int oy = pmod(r.y - a.Sy / 2, a.Py) + (y + a.Sy / 2) % a.Sy;
  if (ox >= a.Px) ox -= a.Px;
  if (oy >= a.Py) oy -= a.Py;
  return ((size_t)s * a.Px + ox) * a.Py + oy;
}

__device__ __forceinline__ float2 patch_value(const BatchArgs& a, int s, int2 r, int x, int y) {
  const size_t idx = patch_index(a, s, r, x, y);
  if (a.potential) {
    float sv, cv;
    sincosf(reinterpret_cast<const float*>(a.object)[idx], &sv, &cv);
    return make_float2(cv, sv);
  }
  return reinterpret_cast<const float2*>(a.object)[idx];
}

// P_{s,m} of position b, element e
__device__ __forceinline__ float2* stash(const BatchArgs& a, int s, int b, int m) {
  const size_t N = (size_t)a.Sx * a.Sy;
  if (a.T == 1) return a.st_probe + ((size_t)b * a.M + m) * N;
  if (a.M == 1) return a.st_obj + ((size_t)s * a.B + b) * N;
  return a.st_pm + (((size_t)s * a.B + b) * a.M + m) * N;
}

// One block per position: ramps[b] = (ramp_x[Sx], ramp_y[Sy]) and the rounded
// origin. `direct` positions are indexed by b (probe overlap), else by pos_rows.
__global__ void __launch_bounds__(256) staged_ramps_kernel(BatchArgs a, float2* ramps, int direct) {
  const int b = blockIdx.x;
  const int prow = (!direct && a.pos_rows) ? a.pos_rows[b] : b;
  const float posx = finite_or_zero(a.positions[2 * prow]);
  const float posy = finite_or_zero(a.positions[2 * prow + 1]);
  const float rx = rintf(posx);  // numpy.round: half to even
  const float ry = rintf(posy);
  const float dx = posx - rx, dy = posy - ry;
  float2* r = ramps + (size_t)b * (a.Sx + a.Sy);
  for (int i = threadIdx.x; i < a.Sx + a.Sy; i += 256) {
    const bool along_x = i < a.Sx;
    const int j = along_x ? i : i - a.Sx;
    const int n = along_x ? a.Sx : a.Sy;
    const float k = (float)fint(j, n) / (float)n;
    r[i] = cis_rounded(__fmul_rn(__fmul_rn(-6.2831855f, k), along_x ? dx : dy));
  }
  if (threadIdx.x == 0) a.pos_round[b] = make_int2((int)rx, (int)ry);
}

// W[b, m] = spec[m] . ramp_x ramp_y (grid: B M x chunks)
__global__ void __launch_bounds__(kEwThreads) staged_shift_kernel(BatchArgs a,
                                                                  const float2* __restrict__ ramps,
                                                                  float2* W) {
  const int N = a.Sx * a.Sy;
  const int b = blockIdx.x / a.M, m = blockIdx.x % a.M;
  const float2* rx = ramps + (size_t)b * (a.Sx + a.Sy);
  const float2* ry = rx + a.Sx;
  const float2* spec = a.probe_spec + (size_t)m * N;
  const int e0 = blockIdx.y * kChunk + threadIdx.x;
#pragma unroll
  for (int i = 0; i < kPer; ++i) {
    const int e = e0 + i * kEwThreads;
    if (e < N)
      W[(size_t)blockIdx.x * N + e] = c_mul(__ldg(spec + e), c_mul(rx[e / a.Sy], ry[e % a.Sy]));
  }
}

// One pass of 1D transforms of length L over 16 lines of wave blockIdx.x: rows
// (ROWS, line l is elements l Sy .. l Sy + Sy - 1, L = Sy) or columns (line l is
// elements l, l + Sy, ..., L = Sx), read from `src` and written, times `scale`,
// to W (src may be W). Block (0, 0) also publishes its twiddle table to
// tw_out when that is not null.
template <int DIR, int L, bool ROWS>
__global__ void __launch_bounds__(kLineThreads) staged_lines_kernel(const float2* src, float2* W,
                                                                    int N, int Sy, float scale,
                                                                    float2* tw_out) {
  constexpr int LD = L + 1;
  __shared__ float2 buf[kLines * LD];
  __shared__ float2 tw[L];
  const float2* r = src + (size_t)blockIdx.x * N;
  float2* w = W + (size_t)blockIdx.x * N;
  const int l0 = blockIdx.y * kLines;
  fill_twiddles<L, kLineThreads>(tw);
  if (tw_out && blockIdx.x == 0 && blockIdx.y == 0)
    for (int i = threadIdx.x; i < L; i += kLineThreads) tw_out[i] = tw[i];
  if (ROWS) {
    for (int e = threadIdx.x; e < kLines * L; e += kLineThreads) {
      const int l = e / L, j = e % L;
      buf[l * LD + j] = r[(size_t)(l0 + l) * Sy + j];
    }
  } else {
    for (int e = threadIdx.x; e < kLines * L; e += kLineThreads) {
      const int j = e / kLines, l = e % kLines;
      buf[l * LD + j] = r[(size_t)j * Sy + l0 + l];
    }
  }
  __syncthreads();
  Schedule<L>::template run<kLines, kLineThreads, DIR>(buf, LD, 1, tw, threadIdx.x);
  if (ROWS) {
    for (int e = threadIdx.x; e < kLines * L; e += kLineThreads) {
      const int l = e / L, j = e % L;
      w[(size_t)(l0 + l) * Sy + j] = c_scale(buf[l * LD + j], scale);
    }
  } else {
    for (int e = threadIdx.x; e < kLines * L; e += kLineThreads) {
      const int j = e / kLines, l = e % kLines;
      w[(size_t)j * Sy + l0 + l] = c_scale(buf[l * LD + j], scale);
    }
  }
}

template <int DIR, int L, bool ROWS>
void lines_t(const float2* src, float2* W, int count, int Sx, int Sy, float scale,
             float2* tw_out, cudaStream_t s) {
  const int nlines = ROWS ? Sx : Sy;
  staged_lines_kernel<DIR, L, ROWS><<<dim3(count, nlines / kLines), kLineThreads, 0, s>>>(
      src, W, Sx * Sy, Sy, scale, tw_out);
}

template <int DIR, bool ROWS>
cudaError_t lines(const float2* src, float2* W, int count, int L, int Sx, int Sy, float scale,
                  float2* tw_out, cudaStream_t s) {
  switch (L) {
    case 32: lines_t<DIR, 32, ROWS>(src, W, count, Sx, Sy, scale, tw_out, s); break;
    case 48: lines_t<DIR, 48, ROWS>(src, W, count, Sx, Sy, scale, tw_out, s); break;
    case 64: lines_t<DIR, 64, ROWS>(src, W, count, Sx, Sy, scale, tw_out, s); break;
    case 96: lines_t<DIR, 96, ROWS>(src, W, count, Sx, Sy, scale, tw_out, s); break;
    case 128: lines_t<DIR, 128, ROWS>(src, W, count, Sx, Sy, scale, tw_out, s); break;
    case 256: lines_t<DIR, 256, ROWS>(src, W, count, Sx, Sy, scale, tw_out, s); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// FFT2 (DIR -1) or unnormalised inverse (DIR +1) of `count` Sx x Sy waves, from
// src (rows first, along y) into W, times `scale`; tw_out (or null) receives the
// x table then the y table.
template <int DIR>
cudaError_t fft2_waves(const float2* src, float2* W, int count, int Sx, int Sy, float scale,
                       float2* tw_out, cudaStream_t s) {
  cudaError_t e = lines<DIR, true>(src, W, count, Sy, Sx, Sy, 1.0f,
                                   tw_out ? tw_out + Sx : nullptr, s);
  if (e != cudaSuccess) return e;
  return lines<DIR, false>(W, W, count, Sx, Sx, Sy, scale, tw_out, s);
}

template <int DIR>
cudaError_t fft2_waves(float2* W, int count, int Sx, int Sy, float scale, cudaStream_t s) {
  return fft2_waves<DIR>(W, W, count, Sx, Sy, scale, nullptr, s);
}

// Slice s of the forward model: P_{s,m} = W_m / N (stashed), W_m = P_{s,m} O_s
__global__ void __launch_bounds__(kEwThreads) staged_overlap_kernel(BatchArgs a, float2* W,
                                                                    int s) {
  const int N = a.Sx * a.Sy;
  const int b = blockIdx.x;
  const int2 r = a.pos_round[b];
  const float invN = 1.0f / (float)N;
  const int e0 = blockIdx.y * kChunk + threadIdx.x;
#pragma unroll
  for (int i = 0; i < kPer; ++i) {
    const int e = e0 + i * kEwThreads;
    if (e >= N) break;
    const float2 o = patch_value(a, s, r, e / a.Sy, e % a.Sy);
    for (int m = 0; m < a.M; ++m) {
      const size_t k = ((size_t)b * a.M + m) * N + e;
      const float2 p = c_scale(W[k], invN);
      stash(a, s, b, m)[e] = p;
      W[k] = c_mul(p, o);
    }
  }
}

// W *= H_s (or conj(H_s)) for every wave of the batch (grid: B M x chunks)
__global__ void __launch_bounds__(kEwThreads) staged_propagate_kernel(BatchArgs a, float2* W,
                                                                      int s, int conjugate) {
  const int N = a.Sx * a.Sy;
  const float2* h = a.props + (size_t)s * N;
  const int e0 = blockIdx.y * kChunk + threadIdx.x;
#pragma unroll
  for (int i = 0; i < kPer; ++i) {
    const int e = e0 + i * kEwThreads;
    if (e >= N) break;
    float2 hv = h[e];
    if (conjugate) hv.y = -hv.y;
    const size_t k = (size_t)blockIdx.x * N + e;
    W[k] = c_mul(W[k], hv);
  }
}

// Fourier projection at one detector pixel of position b: `f[m]` are the far
// fields of the modes there (modified in place into G_m), A the amplitude,
// mk the mask value; returns (A - |F|)^2.
template <bool kSingle>
__device__ __forceinline__ float project_pixel(const BatchArgs& a, float2* f, float A, float mk,
                                               bool masked) {
  const bool mixed = !kSingle && (a.M > 1 || a.mixed_formula);
  if (kSingle || !mixed) {
    float2 v = f[0];
    if (masked) v = c_scale(v, mk);
    const float af = c_abs(v);
    const float d = A - af;
    const float q = af > 0.0f ? A / af : 0.0f;
    float2 r = af > 0.0f ? make_float2(fmaf(v.x, q, -v.x), fmaf(v.y, q, -v.y))
                         : c_sub(make_float2(A, 0.0f), v);
    if (masked) r = c_scale(r, mk);
    f[0] = r;
    return d * d;
  }
  if constexpr (kSingle) return 0.0f;
  float itot = 0.0f;
  for (int m = 0; m < a.M; ++m) {
    if (masked) f[m] = c_scale(f[m], mk);
    const float av = hypotf(f[m].x, f[m].y);  // |F_m|^2 as numpy forms it
    itot += av * av;
  }
  const float tot = sqrtf(itot);
  const float d = A - tot;
  const float ratio = tot == 0.0f ? 0.0f : A / tot;
  for (int m = 0; m < a.M; ++m) {
    float2 r = c_sub(c_scale(f[m], ratio), f[m]);
    if (masked) r = c_scale(r, mk);
    f[m] = r;
  }
  return d * d;
}

// Block partial of the error into err_part[b * chunks + blockIdx.y]
__device__ __forceinline__ void store_partial(const BatchArgs& a, float err, int chunks) {
  __shared__ float red[kEwThreads / 32];
  const float t = block_sum<kEwThreads>(err, red);
  if (threadIdx.x == 0) a.err_part[(size_t)blockIdx.x * chunks + blockIdx.y] = t;
}

// Projection on the region-of-interest grid (no resampling), W in place;
// kSingle: one probe without the mixed-state formula (M = 1)
template <bool kSingle>
__global__ void __launch_bounds__(kEwThreads) staged_projection_kernel(BatchArgs a, float2* W) {
  const int N = a.Sx * a.Sy;
  const int M = kSingle ? 1 : a.M;
  const int b = blockIdx.x;
  const int arow = a.amp_rows ? a.amp_rows[b] : b;
  const float* amp = a.amplitudes + (size_t)arow * N;
  const int e0 = blockIdx.y * kChunk + threadIdx.x;
  float err = 0.0f;
  float2 f[kSingle ? 1 : 16];
#pragma unroll
  for (int i = 0; i < kPer; ++i) {
    const int e = e0 + i * kEwThreads;
    if (e >= N) break;
    for (int m = 0; m < M; ++m) f[m] = W[((size_t)b * M + m) * N + e];
    const float mk = a.det_mask ? a.det_mask[e] : 1.0f;
    err += project_pixel<kSingle>(a, f, __ldg(amp + e), mk, a.det_mask != nullptr);
    if (!a.forward_only)
      for (int m = 0; m < M; ++m) W[((size_t)b * M + m) * N + e] = f[m];
  }
  store_partial(a, err, gridDim.y);
}

// Interpolation of output index k onto an input axis of n samples from an
// output axis of n_out samples (end points aligned): lower index and weight of
// the upper neighbour, formed in float64.
struct Tap {
  int i0, i1;
  float t;
};
__device__ __forceinline__ Tap tap(int k, int n, int n_out) {
  const double z = n_out > 1 ? (double)(n - 1) / (double)(n_out - 1) : 1.0;
  const double cc = (double)k * z;
  const double f = floor(cc);
  int i0 = (int)f;
  int i1 = i0 + 1;
  if (i0 >= n) i0 -= n;  // grid-wrap (only the upper neighbour of the last sample)
  if (i1 >= n) i1 -= n;
  return Tap{i0, i1, (float)(cc - f)};
}

__device__ __forceinline__ float2 bilerp(const float2* g, int ny, Tap tx, Tap ty) {
  const float ux = 1.0f - tx.t, uy = 1.0f - ty.t;
  float2 v = c_scale(g[(size_t)tx.i0 * ny + ty.i0], ux * uy);
  v = c_add(v, c_scale(g[(size_t)tx.i0 * ny + ty.i1], ux * ty.t));
  v = c_add(v, c_scale(g[(size_t)tx.i1 * ny + ty.i0], tx.t * uy));
  return c_add(v, c_scale(g[(size_t)tx.i1 * ny + ty.i1], tx.t * ty.t));
}

// Resampled projection: per detector pixel, F_m interpolated from the ROI grid
// (divided by the pixel-count ratio), projected; G_m into det_f
__global__ void __launch_bounds__(kEwThreads) staged_projection_resampled_kernel(
    BatchArgs a, const float2* __restrict__ W) {
  const int N = a.Sx * a.Sy;
  const int Nd = a.Ax * a.Ay;
  const int b = blockIdx.x;
  const int arow = a.amp_rows ? a.amp_rows[b] : b;
  const float* amp = a.amplitudes + (size_t)arow * Nd;
  // far field sums are kept: divide by (Ax / Sx)(Ay / Sy)
  const float ratio = (float)(((double)a.Ax / a.Sx) * ((double)a.Ay / a.Sy));
  const int e0 = blockIdx.y * kChunk + threadIdx.x;
  float err = 0.0f;
  float2 f[16];
#pragma unroll 1
  for (int i = 0; i < kPer; ++i) {
    const int e = e0 + i * kEwThreads;
    if (e >= Nd) break;
    const Tap tx = tap(e / a.Ay, a.Sx, a.Ax);
    const Tap ty = tap(e % a.Ay, a.Sy, a.Ay);
    for (int m = 0; m < a.M; ++m) {
      const float2 v = bilerp(W + ((size_t)b * a.M + m) * N, a.Sy, tx, ty);
      f[m] = make_float2(__fdiv_rn(v.x, ratio), __fdiv_rn(v.y, ratio));
    }
    const float mk = a.det_mask ? a.det_mask[e] : 1.0f;
    err += project_pixel<false>(a, f, __ldg(amp + e), mk, a.det_mask != nullptr);
    if (!a.forward_only)
      for (int m = 0; m < a.M; ++m) a.det_f[((size_t)b * a.M + m) * Nd + e] = f[m];
  }
  store_partial(a, err, gridDim.y);
}

// G_m from the detector grid back onto the ROI grid (grid: B M x chunks)
__global__ void __launch_bounds__(kEwThreads) staged_resample_back_kernel(BatchArgs a,
                                                                          float2* W) {
  const int N = a.Sx * a.Sy;
  const int Nd = a.Ax * a.Ay;
  const float ratio = (float)(((double)a.Sx / a.Ax) * ((double)a.Sy / a.Ay));
  const float2* g = a.det_f + (size_t)blockIdx.x * Nd;
  const int e0 = blockIdx.y * kChunk + threadIdx.x;
#pragma unroll 1
  for (int i = 0; i < kPer; ++i) {
    const int e = e0 + i * kEwThreads;
    if (e >= N) break;
    const float2 v = bilerp(g, a.Ay, tap(e / a.Sy, a.Ax, a.Sx), tap(e % a.Sy, a.Ay, a.Sy));
    W[(size_t)blockIdx.x * N + e] = make_float2(__fdiv_rn(v.x, ratio), __fdiv_rn(v.y, ratio));
  }
}

// err[b] = the position's chunk partials summed in order; NaN for a non-finite
// position (reported as PTYCHO_ERR_NONFINITE).
__global__ void staged_error_kernel(BatchArgs a, int chunks) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.B) return;
  float t = 0.0f;
  for (int c = 0; c < chunks; ++c) t += a.err_part[(size_t)b * chunks + c];
  const int prow = a.pos_rows ? a.pos_rows[b] : b;
  const bool ok = isfinite(a.positions[2 * prow]) && isfinite(a.positions[2 * prow + 1]);
  a.err[b] = ok ? t : __int_as_float(0x7fc00000);
}

// Adjoint at slice s: chi_m = W_m / N; object terms summed over the modes in
// order; chi_m conj(O_s) back into W_m (s > 0) or into the probe term (s = 0)
__global__ void __launch_bounds__(kEwThreads) staged_adjoint_kernel(BatchArgs a, float2* W,
                                                                    int s) {
  const int N = a.Sx * a.Sy;
  const int b = blockIdx.x;
  const int2 r = a.pos_round[b];
  const float invN = 1.0f / (float)N;
  const int e0 = blockIdx.y * kChunk + threadIdx.x;
#pragma unroll 1
  for (int i = 0; i < kPer; ++i) {
    const int e = e0 + i * kEwThreads;
    if (e >= N) break;
    const float2 o = patch_value(a, s, r, e / a.Sy, e % a.Sy);
    float2 g = make_float2(0.0f, 0.0f);
    float pn = 0.0f;
    for (int m = 0; m < a.M; ++m) {
      const size_t k = ((size_t)b * a.M + m) * N + e;
      const float2 chi = c_scale(W[k], invN);
      const float2 p = stash(a, s, b, m)[e];
      const float2 gm = object_term(a.potential, o, p, chi);
      g = m == 0 ? gm : c_add(g, gm);
      pn = m == 0 ? c_abs2(p) : pn + c_abs2(p);
      const float2 bt = c_conj_mul(o, chi);
      if (s > 0) {
        W[k] = bt;
      } else {
        a.st_probe[k] = bt;
      }
    }
    a.st_obj[((size_t)s * a.B + b) * N + e] = g;
    a.st_nobj[((size_t)s * a.B + b) * N + e] = pn;
    if (s == 0 && !a.nprobe_from_object) a.st_nprobe[(size_t)b * N + e] = c_abs2(o);
  }
}

// |P_b|^2 = |W / N|^2, abs() then square as numpy forms it
__global__ void __launch_bounds__(kEwThreads) staged_intensity_kernel(BatchArgs a,
                                                                      const float2* W) {
  const int N = a.Sx * a.Sy;
  const int b = blockIdx.x;
  const float invN = 1.0f / (float)N;
  const int e0 = blockIdx.y * kChunk + threadIdx.x;
#pragma unroll
  for (int i = 0; i < kPer; ++i) {
    const int e = e0 + i * kEwThreads;
    if (e >= N) break;
    const size_t k = (size_t)b * N + e;
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
  __shared__ float2 rx[256], ry[256];
  const int N = a.Sx * a.Sy;
  const float dx = (float)(-a.com[0]);
  const float dy = (float)(-a.com[1]);
  for (int i = threadIdx.x; i < a.Sx; i += kEwThreads) {
    const float k = (float)fint(i, a.Sx) / (float)a.Sx;
    rx[i] = cis_rounded(__fmul_rn(__fmul_rn(-6.2831855f, k), dx));
  }
  for (int i = threadIdx.x; i < a.Sy; i += kEwThreads) {
    const float k = (float)fint(i, a.Sy) / (float)a.Sy;
    ry[i] = cis_rounded(__fmul_rn(__fmul_rn(-6.2831855f, k), dy));
  }
  __syncthreads();
  const int e0 = blockIdx.y * kChunk + threadIdx.x;
#pragma unroll
  for (int i = 0; i < kPer; ++i) {
    const int e = e0 + i * kEwThreads;
    if (e >= N) break;
    const size_t k = (size_t)blockIdx.x * N + e;
    W[k] = c_mul(W[k], c_mul(rx[e / a.Sy], ry[e % a.Sy]));
  }
}

// The probe aperture constraint of mode 0 at 256 x 256 in one 512-thread block
// (ptychographic_constraints.py:1004-1040): P <- IFFT2(A exp(i angle FFT2(P))),
// rescaled to the power sum |P|^2 it had before. The transforms walk the wave in
// global memory 16 lines at a time; the two power sums stay in the block, so
// the call allocates nothing and concurrent calls do not share state.
constexpr int kBlockThreads = 512;

template <int DIR, bool ROWS>
__device__ void block_lines_256(float2* w, float scale, float2* buf, const float2* tw) {
  constexpr int L = 256, LD = L + 1;
  for (int l0 = 0; l0 < L; l0 += kLines) {
    for (int e = threadIdx.x; e < kLines * L; e += kBlockThreads) {
      if (ROWS) {
        const int l = e / L, j = e % L;
        buf[l * LD + j] = w[(size_t)(l0 + l) * L + j];
      } else {
        const int j = e / kLines, l = e % kLines;
        buf[l * LD + j] = w[(size_t)j * L + l0 + l];
      }
    }
    __syncthreads();
    Schedule<L>::template run<kLines, kBlockThreads, DIR>(buf, LD, 1, tw, threadIdx.x);
    for (int e = threadIdx.x; e < kLines * L; e += kBlockThreads) {
      if (ROWS) {
        const int l = e / L, j = e % L;
        w[(size_t)(l0 + l) * L + j] = c_scale(buf[l * LD + j], scale);
      } else {
        const int j = e / kLines, l = e % kLines;
        w[(size_t)j * L + l0 + l] = c_scale(buf[l * LD + j], scale);
      }
    }
    __syncthreads();
  }
}

// sum |p|^2 (abs() then square): thread partials, a fixed shuffle tree, warp order
__device__ float block_power_256(const float2* p, float* red) {
  float part = 0.0f;
  for (int e = threadIdx.x; e < 256 * 256; e += kBlockThreads) {
    const float2 v = p[e];
    const float av = hypotf(v.x, v.y);
    part += av * av;
  }
  const float t = block_sum<kBlockThreads>(part, red);
  __syncthreads();
  if (threadIdx.x == 0) red[0] = t;
  __syncthreads();
  const float r = red[0];
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(kBlockThreads) staged_aperture_block_kernel(
    float2* p, const float* __restrict__ aperture) {
  constexpr int N = 256 * 256;
  __shared__ float2 buf[kLines * 257];
  __shared__ float2 tw[256];
  __shared__ float red[kBlockThreads / 32];
  fill_twiddles<256, kBlockThreads>(tw);
  const float s0 = block_power_256(p, red);  // (its barriers also cover the tables)
  block_lines_256<-1, true>(p, 1.0f, buf, tw);
  block_lines_256<-1, false>(p, 1.0f, buf, tw);
  for (int e = threadIdx.x; e < N; e += kBlockThreads) {
    const float2 f = p[e];
    float sn, cs;
    sincosf(atan2f(f.y, f.x), &sn, &cs);
    const float ap = aperture[e];
    p[e] = make_float2(cs * ap, sn * ap);
  }
  __syncthreads();
  block_lines_256<+1, true>(p, 1.0f, buf, tw);
  block_lines_256<+1, false>(p, 1.0f / (float)N, buf, tw);
  const float s1 = block_power_256(p, red);
  const float k = sqrtf(s0 / s1);
  for (int e = threadIdx.x; e < N; e += kBlockThreads) p[e] = c_scale(p[e], k);
}

}  // namespace

bool staged_roi(int Sx, int Sy) { return Sx == 256 && Sy == 256; }

bool staged_batch(const BatchArgs& a) { return staged_roi(a.Sx, a.Sy) || a.resample; }

bool staged_batch_supported(const BatchArgs& a) {
  return a.M <= 16 && !a.projection && !a.keep_farfield && !a.exact_probe_grad && !a.staging_t;
}

cudaError_t launch_staged_spectrum(const BatchArgs& a, cudaStream_t s) {
  // FFT2 of every probe mode into the spectrum buffer, the x and y twiddle
  // tables published for the fused position kernels
  return fft2_waves<-1>(a.probe, a.probe_spec, a.M, a.Sx, a.Sy, 1.0f, a.tw, s);
}

cudaError_t launch_staged_positions(const BatchArgs& a, cudaStream_t s) {
  if (!staged_batch_supported(a)) return cudaErrorNotSupported;
  const int N = a.Sx * a.Sy;
  const int BM = a.B * a.M;
  float2* ramps = reinterpret_cast<float2*>(a.st_nobj);
  float2* W = a.scratch_f;
  const dim3 per_pos(a.B, chunks_of(N));
  const dim3 per_wave(BM, chunks_of(N));
  staged_ramps_kernel<<<a.B, 256, 0, s>>>(a, ramps, 0);
  staged_shift_kernel<<<per_wave, kEwThreads, 0, s>>>(a, ramps, W);
  cudaError_t e = fft2_waves<+1>(W, BM, a.Sx, a.Sy, 1.0f, s);
  for (int sl = 0; sl < a.T && e == cudaSuccess; ++sl) {
    staged_overlap_kernel<<<per_pos, kEwThreads, 0, s>>>(a, W, sl);
    if (sl + 1 < a.T) {
      if ((e = fft2_waves<-1>(W, BM, a.Sx, a.Sy, 1.0f, s)) != cudaSuccess) break;
      staged_propagate_kernel<<<per_wave, kEwThreads, 0, s>>>(a, W, sl, 0);
      e = fft2_waves<+1>(W, BM, a.Sx, a.Sy, 1.0f, s);
    }
  }
  if (e != cudaSuccess) return e;
  if ((e = fft2_waves<-1>(W, BM, a.Sx, a.Sy, 1.0f, s)) != cudaSuccess) return e;
  int chunks;
  if (a.resample) {
    chunks = chunks_of(a.Ax * a.Ay);
    staged_projection_resampled_kernel<<<dim3(a.B, chunks), kEwThreads, 0, s>>>(a, W);
    if (!a.forward_only)
      staged_resample_back_kernel<<<per_wave, kEwThreads, 0, s>>>(a, W);
  } else {
    chunks = chunks_of(N);
    if (a.M == 1 && !a.mixed_formula)
      staged_projection_kernel<true><<<per_pos, kEwThreads, 0, s>>>(a, W);
    else
      staged_projection_kernel<false><<<per_pos, kEwThreads, 0, s>>>(a, W);
  }
  staged_error_kernel<<<(a.B + 255) / 256, 256, 0, s>>>(a, chunks);
  if (a.forward_only) return cudaGetLastError();
  if ((e = fft2_waves<+1>(W, BM, a.Sx, a.Sy, 1.0f, s)) != cudaSuccess) return e;
  for (int sl = a.T - 1; sl >= 0; --sl) {
    staged_adjoint_kernel<<<per_pos, kEwThreads, 0, s>>>(a, W, sl);
    if (sl > 0) {
      if ((e = fft2_waves<-1>(W, BM, a.Sx, a.Sy, 1.0f, s)) != cudaSuccess) return e;
      staged_propagate_kernel<<<per_wave, kEwThreads, 0, s>>>(a, W, sl - 1, 1);
      if ((e = fft2_waves<+1>(W, BM, a.Sx, a.Sy, 1.0f, s)) != cudaSuccess) return e;
    }
  }
  return cudaGetLastError();
}

cudaError_t launch_staged_intensity(const BatchArgs& a, cudaStream_t s) {
  // mode 0 only (a.M = 1); ramps in st_obj, waves in scratch_f, |P_b|^2 into st_nobj
  const int N = a.Sx * a.Sy;
  float2* ramps = a.st_obj;
  float2* W = a.scratch_f;
  const dim3 ew(a.B, chunks_of(N));
  staged_ramps_kernel<<<a.B, 256, 0, s>>>(a, ramps, 1);
  staged_shift_kernel<<<ew, kEwThreads, 0, s>>>(a, ramps, W);
  cudaError_t e = fft2_waves<+1>(W, a.B, a.Sx, a.Sy, 1.0f, s);
  if (e != cudaSuccess) return e;
  staged_intensity_kernel<<<ew, kEwThreads, 0, s>>>(a, W);
  return cudaGetLastError();
}

cudaError_t launch_staged_probe_shift(const BatchArgs& a, cudaStream_t s) {
  // every mode through the probe spectrum buffer (free between batches)
  const int N = a.Sx * a.Sy;
  cudaError_t e = launch_staged_spectrum(a, s);
  if (e != cudaSuccess) return e;
  staged_com_ramp_kernel<<<dim3(a.M, chunks_of(N)), kEwThreads, 0, s>>>(a, a.probe_spec);
  if ((e = fft2_waves<+1>(a.probe_spec, a.M, a.Sx, a.Sy, 1.0f / (float)N, s)) != cudaSuccess)
    return e;
  const size_t n = (size_t)a.M * N;
  copy_waves_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a.probe_spec, a.probe, n);
  return cudaGetLastError();
}

cudaError_t launch_staged_aperture(const BatchArgs& a, cudaStream_t s) {
  if (a.Sx != 256 || a.Sy != 256) return cudaErrorInvalidValue;
  staged_aperture_block_kernel<<<1, kBlockThreads, 0, s>>>(a.probe, a.aperture);
  return cudaGetLastError();
}

}  // namespace pty
