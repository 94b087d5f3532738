// Register-resident fused position kernel for a 128 x 128 ROI, single slice,
// single probe, gradient descent (complex or potential object, optional detector
// mask). One 1024-thread block per scan position.
//
// Each 2D FFT is a four-step transform per axis (128 = 16 x 8): a radix-16 stage,
// an inter-stage twiddle and a radix-8 stage, first along y (each warp owns 4
// full rows), then along x (each warp owns 4 full columns). Every thread keeps 16
// samples in registers; between stages the samples move through one swizzled
// 128 KB shared-memory wave. Exchanges inside an axis stay within the warp
// (__syncwarp); the switch between axes is the only block barrier. The three
// transforms of a position alternate decompositions (inverse, transposed
// forward, inverse) so that the last stage of one and the first stage of the
// next use the same thread-to-sample map: the elementwise steps between them
// (object multiply, Fourier projection) run on registers with no exchange.
// A position costs 9 shared-memory round trips and 3 block barriers.
//
// Swizzle: sample (x, y) lives at x * 128 + (y ^ ((y >> 4) & 7) ^ t(x)) with
// t(x) = (x & 15) ^ ((x >> 4) & 7); every access pattern of the schedule hits 16
// distinct bank pairs per half-warp.
//
// Staging outputs are written in y-major order (e' = y * 128 + x), the order in
// which a warp's lanes hold them (BatchArgs::staging_t = 1).
#include <cuda_runtime.h>

#include "fft_smem.cuh"
#include "ptycho_internal.h"

namespace pty {
namespace {

constexpr int S = 128;
constexpr int N = S * S;
constexpr int NT = 1024;
constexpr int GA = 1;  // A groups (16 samples) per thread
constexpr int GB = 2;  // B groups (8 samples) per thread

__device__ __forceinline__ int pmod(int v, int m) {
  int r = v % m;
  return r < 0 ? r + m : r;
}

__device__ __forceinline__ int fint(int i) { return i < S / 2 ? i : i - S; }

// Object coordinate of patch index i: (c0 + fint(i)) mod P, computed from
// base = (c0 - S/2) mod P as base + ((i + S/2) mod S) with one conditional wrap
// (valid because P >= S).
__device__ __forceinline__ int wrap_obj(int base, int i, int P) {
  const int t = base + (i ^ (S / 2));
  return t >= P ? t - P : t;
}

__device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }

template <int R, int DIR>
__device__ __forceinline__ void dft_at(float2* v) {
  float2 (&g)[R] = *reinterpret_cast<float2 (*)[R]>(v);
  dft<R, DIR>(g);
}

__device__ __forceinline__ float2 load_obj(const BatchArgs& a, int ox, int oy) {
  const size_t idx = (size_t)ox * a.Py + oy;
  if (a.potential) {
    float sv, cv;
    sincosf(reinterpret_cast<const float*>(a.object)[idx], &sv, &cv);
    return make_float2(cv, sv);
  }
  return reinterpret_cast<const float2*>(a.object)[idx];
}

// Thread-to-sample maps. A: groups of 16 samples at stride 8 along the line;
// B: groups of 8 samples at stride 16 (GA = 1, GB = 2 with 1024 threads: each
// warp owns 4 lines). `base` is the warp's first line.
struct Maps {
  int base, lane, c, n2, aa, k1;
  __device__ Maps() {
    const int w = threadIdx.x >> 5;
    lane = threadIdx.x & 31;
    base = 16 * (w >> 2) + 2 * (w & 3);
    c = lane >> 4;
    n2 = lane & 7;
    aa = (lane >> 3) & 1;
    k1 = lane & 15;
  }
  __device__ int lineA(int g) const { return base + 8 * aa + c + 16 * g; }
  __device__ int lineB(int g) const { return base + c + 8 * g; }
};

// Closed forms of swz() for the access patterns of the schedule: a compile-time
// part (loop indices j, k, n) XOR a per-thread part, so every shared-memory
// access costs one XOR and one add.
__device__ __forceinline__ int u_of(int y) { return (y >> 4) & 7; }
__device__ __forceinline__ int t_of(int x) { return (x & 15) ^ ((x >> 4) & 7); }
__host__ __device__ constexpr int KA(int j) { return (8 * j) ^ (j >> 1); }
__host__ __device__ constexpr int KB(int k) { return (16 * k) ^ (k & 7); }
__host__ __device__ constexpr int CA(int j) { return (8 * (j & 1)) ^ (j >> 1); }

// A registers <-> positions 8 j + n2 of line lineA(g)
template <bool ROWS>
__device__ __forceinline__ void store_A(const float2* v, float2* buf, const Maps& m) {
#pragma unroll
  for (int g = 0; g < GA; ++g) {
    const int line = m.lineA(g);
    if (ROWS) {
      float2* row = buf + line * S;
      const int r = m.n2 ^ t_of(line);
#pragma unroll
      for (int j = 0; j < 16; ++j) row[KA(j) ^ r] = v[16 * g + j];
    } else {
      float2* col = buf + m.n2 * S;
      const int r = line ^ u_of(line) ^ m.n2;
#pragma unroll
      for (int j = 0; j < 16; ++j) col[8 * j * S + (r ^ CA(j))] = v[16 * g + j];
    }
  }
}

template <bool ROWS>
__device__ __forceinline__ void load_A(float2* v, const float2* buf, const Maps& m) {
#pragma unroll
  for (int g = 0; g < GA; ++g) {
    const int line = m.lineA(g);
    if (ROWS) {
      const float2* row = buf + line * S;
      const int r = m.n2 ^ t_of(line);
#pragma unroll
      for (int j = 0; j < 16; ++j) v[16 * g + j] = row[KA(j) ^ r];
    } else {
      const float2* col = buf + m.n2 * S;
      const int r = line ^ u_of(line) ^ m.n2;
#pragma unroll
      for (int j = 0; j < 16; ++j) v[16 * g + j] = col[8 * j * S + (r ^ CA(j))];
    }
  }
}

// A registers <- positions j + 16 n2 of line lineA(g) (second forward stage)
template <bool ROWS>
__device__ __forceinline__ void load_A16(float2* v, const float2* buf, const Maps& m) {
#pragma unroll
  for (int g = 0; g < GA; ++g) {
    const int line = m.lineA(g);
    if (ROWS) {
      const float2* row = buf + line * S;
      const int r = (16 * m.n2) ^ m.n2 ^ t_of(line);
#pragma unroll
      for (int j = 0; j < 16; ++j) v[16 * g + j] = row[j ^ r];
    } else {
      const float2* col = buf + 16 * m.n2 * S;
      const int r = line ^ u_of(line) ^ m.n2;
#pragma unroll
      for (int j = 0; j < 16; ++j) v[16 * g + j] = col[j * S + (r ^ j)];
    }
  }
}

// B registers <-> positions k1 + 16 k of line lineB(g)
template <bool ROWS>
__device__ __forceinline__ void store_B(const float2* v, float2* buf, const Maps& m) {
#pragma unroll
  for (int g = 0; g < GB; ++g) {
    const int line = m.lineB(g);
    if (ROWS) {
      float2* row = buf + line * S;
      const int r = m.k1 ^ t_of(line);
#pragma unroll
      for (int k = 0; k < 8; ++k) row[KB(k) ^ r] = v[8 * g + k];
    } else {
      float2* col = buf + m.k1 * S;
      const int r = line ^ u_of(line) ^ m.k1;
#pragma unroll
      for (int k = 0; k < 8; ++k) col[16 * k * S + (r ^ (k & 7))] = v[8 * g + k];
    }
  }
}

template <bool ROWS>
__device__ __forceinline__ void load_B(float2* v, const float2* buf, const Maps& m) {
#pragma unroll
  for (int g = 0; g < GB; ++g) {
    const int line = m.lineB(g);
    if (ROWS) {
      const float2* row = buf + line * S;
      const int r = m.k1 ^ t_of(line);
#pragma unroll
      for (int k = 0; k < 8; ++k) v[8 * g + k] = row[KB(k) ^ r];
    } else {
      const float2* col = buf + m.k1 * S;
      const int r = line ^ u_of(line) ^ m.k1;
#pragma unroll
      for (int k = 0; k < 8; ++k) v[8 * g + k] = col[16 * k * S + (r ^ (k & 7))];
    }
  }
}

// B registers <- positions 8 k1 + n of line lineB(g), times the inverse
// inter-stage twiddle conj(W^(n k1)) (second inverse stage)
template <bool ROWS>
__device__ __forceinline__ void load_B8(float2* v, const float2* buf, const float2* tw,
                                        const Maps& m) {
  float2 t[8];
#pragma unroll
  for (int n = 0; n < 8; ++n) t[n] = conjf2(tw[n * m.k1]);
#pragma unroll
  for (int g = 0; g < GB; ++g) {
    const int line = m.lineB(g);
    if (ROWS) {
      const float2* row = buf + line * S;
      const int r = (8 * m.k1) ^ (m.k1 >> 1) ^ t_of(line);
#pragma unroll
      for (int n = 0; n < 8; ++n) v[8 * g + n] = c_mul(row[n ^ r], t[n]);
    } else {
      const float2* col = buf + 8 * m.k1 * S;
      const int r = line ^ u_of(line) ^ (8 * (m.k1 & 1)) ^ (m.k1 >> 1);
#pragma unroll
      for (int n = 0; n < 8; ++n) v[8 * g + n] = c_mul(col[n * S + (r ^ n)], t[n]);
    }
  }
}

// Inverse stage pair along one axis: A registers x[8 n1 + n2] -> B registers
// X[k1 + 16 k2]. rows: lines are x (y varies), else lines are y. The mode is a
// runtime value so that one copy of the radix code serves all six passes.
__device__ __forceinline__ void inverse_axis(float2* v, float2* buf, const float2* tw,
                                             const Maps& m, bool rows) {
#pragma unroll
  for (int g = 0; g < GA; ++g) dft_at<16, +1>(v + 16 * g);
  __syncwarp();
  if (rows) store_A<true>(v, buf, m); else store_A<false>(v, buf, m);  // Y[k1,n2] at 8 k1 + n2
  __syncwarp();
  if (rows) load_B8<true>(v, buf, tw, m); else load_B8<false>(v, buf, tw, m);
#pragma unroll
  for (int g = 0; g < GB; ++g) dft_at<8, +1>(v + 8 * g);
}

// Forward transposed stage pair: B registers psi[m1 + 16 m2] (group m1 = k1) ->
// A registers F[8 q1 + q2] (group q2 = n2).
__device__ __forceinline__ void forward_axis(float2* v, float2* buf, const float2* tw,
                                             const Maps& m, bool rows) {
  float2 t[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) t[q] = tw[m.k1 * q];
#pragma unroll
  for (int g = 0; g < GB; ++g) {
    dft_at<8, -1>(v + 8 * g);
#pragma unroll
    for (int q = 1; q < 8; ++q) v[8 * g + q] = c_mul(v[8 * g + q], t[q]);
  }
  __syncwarp();
  if (rows) store_B<true>(v, buf, m); else store_B<false>(v, buf, m);  // Z[m1,q2] at m1 + 16 q2
  __syncwarp();
  if (rows) load_A16<true>(v, buf, m); else load_A16<false>(v, buf, m);
#pragma unroll
  for (int g = 0; g < GA; ++g) dft_at<16, -1>(v + 16 * g);
}

__global__ void __launch_bounds__(NT, 1) gd128_kernel(BatchArgs a) {
  extern __shared__ float4 smem4[];
  float2* buf = reinterpret_cast<float2*>(smem4);
  __shared__ float2 tw[S];
  __shared__ float2 rpx[S];
  __shared__ float2 rpy[S];
  __shared__ float red[NT / 32];

  const int b = blockIdx.x;
  const int tid = threadIdx.x;
  const int prow = a.pos_rows ? a.pos_rows[b] : b;
  const int arow = a.amp_rows ? a.amp_rows[b] : b;
  const bool pos_ok = isfinite(a.positions[2 * prow]) && isfinite(a.positions[2 * prow + 1]);
  const float posx = finite_or_zero(a.positions[2 * prow]);
  const float posy = finite_or_zero(a.positions[2 * prow + 1]);
  const float rx = rintf(posx);
  const float ry = rintf(posy);
  const float dx = posx - rx;
  const float dy = posy - ry;
  const int x0 = (int)rx;
  const int y0 = (int)ry;
  const float invN = 1.0f / (float)N;

  if (tid < S) {
    tw[tid] = a.tw[tid];
    const float k = (float)fint(tid) / (float)S;
    rpx[tid] = cis_rounded(__fmul_rn(__fmul_rn(-6.2831855f, k), dx));
  } else if (tid < 2 * S) {
    const int i = tid - S;
    const float k = (float)fint(i) / (float)S;
    rpy[i] = cis_rounded(__fmul_rn(__fmul_rn(-6.2831855f, k), dy));
  }
  if (tid == 0) a.pos_round[b] = make_int2(x0, y0);
  const int bx = pmod(x0 - S / 2, a.Px);
  const int by = pmod(y0 - S / 2, a.Py);
  __syncthreads();

  const Maps m;
  float2 v[16 * GA];

  // ---- IFFT_1 input: FFT2(P) . ramp, straight from L2 into A registers (rows)
#pragma unroll
  for (int g = 0; g < GA; ++g) {
    const int x = m.lineA(g);
    const float2 rxv = rpx[x];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const int y = 8 * j + m.n2;
      v[16 * g + j] = c_mul(a.probe_spec[x * S + y], c_mul(rxv, rpy[y]));
    }
  }

  float2* pst = a.st_probe + (size_t)b * N;
  float err = 0.0f;
  // Six axis passes: IFFT_1 (y, x), FFT_2 (x, y), IFFT_3 (y, x).
#pragma unroll 1
  for (int pass = 0; pass < 6; ++pass) {
    const bool inv = pass != 2 && pass != 3;
    const bool rows = pass == 0 || pass == 3 || pass == 4;
    if (inv) inverse_axis(v, buf, tw, m, rows); else forward_axis(v, buf, tw, m, rows);

    if (pass == 0 || pass == 4) {
      // y done -> x: natural B data to rows, block barrier, A loads along columns
      __syncwarp();
      store_B<true>(v, buf, m);
      __syncthreads();
      load_A<false>(v, buf, m);
    } else if (pass == 2) {
      // x done -> y
      __syncwarp();
      store_A<false>(v, buf, m);
      __syncthreads();
      load_B<true>(v, buf, m);
    } else if (pass == 1) {
      // shifted probe P at (x = k1 + 16 k, y = lineB): stash P, psi = P O
#pragma unroll
      for (int g = 0; g < GB; ++g) {
        const int y = m.lineB(g);
        const int oy = wrap_obj(by, y, a.Py);
        float2 o[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) o[k] = load_obj(a, wrap_obj(bx, m.k1 + 16 * k, a.Px), oy);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          const float2 p = c_scale(v[8 * g + k], invN);
          pst[y * S + m.k1 + 16 * k] = p;
          v[8 * g + k] = c_mul(p, o[k]);
        }
      }
    } else if (pass == 3) {
      // Fourier projection on A registers: F at (x = lineA, y = 8 q1 + q2)
      const float* amp = a.amplitudes + (size_t)arow * N;
#pragma unroll
      for (int g = 0; g < GA; ++g) {
        const int x = m.lineA(g);
        float A[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) A[j] = amp[x * S + 8 * j + m.n2];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          float2 f = v[16 * g + j];
          float mk = 1.0f;
          if (a.det_mask) {
            mk = a.det_mask[x * S + 8 * j + m.n2];
            f = c_scale(f, mk);
          }
          const float af = c_abs(f);
          const float d = A[j] - af;
          err += d * d;
          // A exp(i angle F) - F = F (A/|F| - 1); A - F where F = 0 (angle 0)
          float2 r;
          if (af > 0.0f) {
            const float q = A[j] / af;
            r = make_float2(fmaf(f.x, q, -f.x), fmaf(f.y, q, -f.y));
          } else {
            r = make_float2(A[j] - f.x, -f.y);
          }
          if (a.det_mask) r = c_scale(r, mk);
          v[16 * g + j] = r;
        }
      }
    } else {
      // adjoint terms at (x = k1 + 16 k, y = lineB), y-major staging
      float2* gobj = a.st_obj + (size_t)b * N;
      float* nobj = a.st_nobj + (size_t)b * N;
      float* nprb = a.st_nprobe + (size_t)b * N;
#pragma unroll
      for (int g = 0; g < GB; ++g) {
        const int y = m.lineB(g);
        const int oy = wrap_obj(by, y, a.Py);
#pragma unroll
        for (int h = 0; h < 8; h += 4) {
          float2 ob[4], pb[4];
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            ob[k] = load_obj(a, wrap_obj(bx, m.k1 + 16 * (h + k), a.Px), oy);
            pb[k] = pst[y * S + m.k1 + 16 * (h + k)];
          }
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const int e = y * S + m.k1 + 16 * (h + k);
            const float2 chi = c_scale(v[8 * g + h + k], invN);
            const float2 p = pb[k];
            const float2 o = ob[k];
            if (a.potential) {
              const float2 t = make_float2(-o.y, -o.x);
              const float2 u = c_mul(t, conjf2(p));
              gobj[e] = make_float2(c_mul(u, chi).x, 0.0f);
            } else {
              gobj[e] = c_conj_mul(p, chi);
            }
            nobj[e] = c_abs2(p);
            pst[e] = c_conj_mul(o, chi);
            nprb[e] = c_abs2(o);
          }
        }
      }
    }
  }

  // ---- batch error of this position (fixed-order block sum)
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) err += __shfl_xor_sync(0xffffffffu, err, o);
  if ((tid & 31) == 0) red[tid >> 5] = err;
  __syncthreads();
  if (tid == 0) {
    float t = 0.0f;
#pragma unroll
    for (int w = 0; w < NT / 32; ++w) t += red[w];
    a.err[b] = pos_ok ? t : __int_as_float(0x7fc00000);
  }
}

}  // namespace

namespace {
// 0: default (the shared-memory passes, measured faster on GB300), 1: shared-memory
// passes, 2: register-resident
int g_schedule_128 = 0;
}

int set_schedule(int roi, int schedule) {
  if (roi != S) return 0;
  const int prev = g_schedule_128;
  g_schedule_128 = schedule;
  return prev;
}

int get_schedule(int roi) { return roi == S ? g_schedule_128 : 0; }

bool position_v2_eligible(const BatchArgs& a) {
  if (g_schedule_128 != 2) return false;
  return a.Sx == S && a.Sy == S && a.T == 1 && a.M == 1 && !a.projection && !a.mixed_formula &&
         !a.forward_only && !a.keep_farfield;
}

cudaError_t launch_position_v2(const BatchArgs& a, cudaStream_t s) {
  const size_t smem = sizeof(float2) * N;
  {
    const cudaError_t e0 =
        ensure_smem_limit(reinterpret_cast<const void*>(gd128_kernel),
                          (int)smem);
    if (e0 != cudaSuccess) return e0;
  }
  timing_before(s);
  gd128_kernel<<<a.B, NT, smem, s>>>(a);
  cudaError_t e = cudaGetLastError();
  timing_after(s);
  return e;
}

}  // namespace pty
