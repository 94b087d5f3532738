// In-shared-memory 2D FFT building blocks for one thread block.
//
// A wave of SX x SY complex64 samples lives in shared memory, row-major, with a
// row pitch of SY + 1 float2 so that both row and column passes are free of bank
// conflicts (see line_pass below). The 1D transforms are Stockham auto-sort
// passes: each pass reads R samples of a line with stride L/R, applies the
// inter-pass twiddles, runs a radix-R DFT in registers and writes the results
// back in natural order. The pass is in place: every thread keeps its samples in
// registers across a block barrier between the read and the write phase.
//
// Radix-R DFTs (R in {2,4,8,16}) are radix-2 decimation-in-frequency networks
// fully unrolled in registers; R = 3 uses the standard 3-point butterfly. Their
// internal twiddles are exact 16th roots of unity. Inter-pass twiddles come from
// a table exp(-2 pi i m / L), m < L, computed at compile time and rounded once.
//
// Conventions match numpy.fft: forward = exp(-2 pi i n k / L) unnormalised,
// inverse = exp(+2 pi i n k / L); the caller applies the 1/(SX*SY) factor.
#pragma once

#include <cuda_runtime.h>

namespace pty {

// ---------------------------------------------------------------- complex ops
// (Packed f32x2 forms of these were measured slower here: the register pairing
// they need adds moves and spills in the radix passes.)
__device__ __forceinline__ float2 c_add(float2 a, float2 b) {
  return make_float2(a.x + b.x, a.y + b.y);
}
__device__ __forceinline__ float2 c_sub(float2 a, float2 b) {
  return make_float2(a.x - b.x, a.y - b.y);
}
__device__ __forceinline__ float2 c_mul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// conj(a) * b
__device__ __forceinline__ float2 c_conj_mul(float2 a, float2 b) {
  return make_float2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float2 c_scale(float2 a, float s) {
  return make_float2(a.x * s, a.y * s);
}
__device__ __forceinline__ float c_abs2(float2 a) { return a.x * a.x + a.y * a.y; }
// |a| as one IEEE square root of a fused x^2 + y^2 (within 1 ulp of hypotf for
// the finite, non-extreme magnitudes of a far field; a third of its instructions).
__device__ __forceinline__ float c_abs(float2 a) { return __fsqrt_rn(fmaf(a.x, a.x, a.y * a.y)); }

// cos(2 pi m / 16) and sin(2 pi m / 16) for compile-time m after unrolling.
__device__ __forceinline__ float cos16(int m) {
  switch (m & 15) {
    case 0: return 1.0f;
    case 1: return 0.92387953251128674f;
    case 2: return 0.70710678118654752f;
    case 3: return 0.38268343236508977f;
    case 4: return 0.0f;
    case 5: return -0.38268343236508977f;
    case 6: return -0.70710678118654752f;
    case 7: return -0.92387953251128674f;
    case 8: return -1.0f;
    case 9: return -0.92387953251128674f;
    case 10: return -0.70710678118654752f;
    case 11: return -0.38268343236508977f;
    case 12: return 0.0f;
    case 13: return 0.38268343236508977f;
    case 14: return 0.70710678118654752f;
    default: return 0.92387953251128674f;
  }
}
__device__ __forceinline__ float sin16(int m) { return cos16(m - 4); }

// d * exp(DIR * 2 pi i m / 16), specialised for the trivial roots.
template <int DIR>
__device__ __forceinline__ float2 rot16(float2 d, int m) {
  m &= 15;
  if (m == 0) return d;
  if (m == 4) return DIR < 0 ? make_float2(d.y, -d.x) : make_float2(-d.y, d.x);
  if (m == 8) return make_float2(-d.x, -d.y);
  if (m == 12) return DIR < 0 ? make_float2(-d.y, d.x) : make_float2(d.y, -d.x);
  const float c = cos16(m);
  const float s = DIR < 0 ? -sin16(m) : sin16(m);
  return make_float2(d.x * c - d.y * s, d.x * s + d.y * c);
}

template <int R>
__device__ __forceinline__ constexpr int bitrev(int k) {
  int r = 0;
  for (int b = 1; b < R; b <<= 1) {
    r = (r << 1) | (k & 1);
    k >>= 1;
  }
  return r;
}

// In-register DFT of length R (power of two, R <= 16), natural order in/out.
template <int R, int DIR>
__device__ __forceinline__ void dft_pow2(float2 (&a)[R]) {
#pragma unroll
  for (int half = R / 2; half >= 1; half >>= 1) {
#pragma unroll
    for (int base = 0; base < R; base += 2 * half) {
#pragma unroll
      for (int i = 0; i < half; ++i) {
        const float2 u = a[base + i];
        const float2 v = a[base + i + half];
        a[base + i] = c_add(u, v);
        a[base + i + half] = rot16<DIR>(c_sub(u, v), i * (16 / (2 * half)));
      }
    }
  }
  float2 t[R];
#pragma unroll
  for (int k = 0; k < R; ++k) t[k] = a[bitrev<R>(k)];
#pragma unroll
  for (int k = 0; k < R; ++k) a[k] = t[k];
}

template <int DIR>
__device__ __forceinline__ void dft3(float2 (&a)[3]) {
  const float h = 0.86602540378443865f;  // sqrt(3)/2
  const float2 t = c_add(a[1], a[2]);
  const float2 m = make_float2(a[0].x - 0.5f * t.x, a[0].y - 0.5f * t.y);
  const float2 d = c_sub(a[1], a[2]);
  // s = d * (DIR * i * sqrt(3)/2)
  const float2 s = DIR < 0 ? make_float2(h * d.y, -h * d.x) : make_float2(-h * d.y, h * d.x);
  a[0] = c_add(a[0], t);
  a[1] = c_add(m, s);
  a[2] = c_sub(m, s);
}

template <int R, int DIR>
__device__ __forceinline__ void dft(float2 (&a)[R]) {
  if constexpr (R == 3) {
    dft3<DIR>(a);
  } else {
    static_assert((R & (R - 1)) == 0 && R <= 16, "radix must be 3 or a power of two <= 16");
    dft_pow2<R, DIR>(a);
  }
}

// Twiddle tables exp(-2 pi i m / L), m < L, evaluated at compile time: the
// angle is reduced to a quarter turn by integer arithmetic (exact), cos and sin
// of x = (pi/2) r/L in [0, pi/2) are summed as Taylor series in double (16 terms:
// truncation below 1e-20), and each entry is rounded once to float. Every entry
// equals the float nearest to the exact root of unity (checked against 40-digit
// values for L = 32, 48, 64, 96, 128).
namespace twiddle_detail {
constexpr double kHalfPi = 1.57079632679489661923;
constexpr double sin_series(double x) {
  double term = x, sum = x;
  for (int k = 1; k < 16; ++k) {
    term *= -x * x / ((2.0 * k) * (2.0 * k + 1.0));
    sum += term;
  }
  return sum;
}
constexpr double cos_series(double x) {
  double term = 1.0, sum = 1.0;
  for (int k = 1; k < 16; ++k) {
    term *= -x * x / ((2.0 * k - 1.0) * (2.0 * k));
    sum += term;
  }
  return sum;
}
template <int L>
struct Table {
  float2 v[L];
};
template <int L>
constexpr Table<L> make_table() {
  Table<L> t{};
  for (int m = 0; m < L; ++m) {
    const int q = (4 * m) / L;  // quarter turns
    const int r = 4 * m - q * L;
    const double x = kHalfPi * (double)r / (double)L;
    const double c0 = cos_series(x), s0 = sin_series(x);
    double c = c0, s = s0;
    if (q == 1) { c = -s0; s = c0; }
    if (q == 2) { c = -c0; s = -s0; }
    if (q == 3) { c = s0; s = -c0; }
    t.v[m].x = (float)c;
    t.v[m].y = (float)-s;
  }
  return t;
}
template <int L>
__device__ const Table<L> kTable = make_table<L>();
}  // namespace twiddle_detail

// Fill tw[m] = exp(-2 pi i m / L) for m < L from the table (block-cooperative,
// no barrier).
template <int L, int NT>
__device__ __forceinline__ void fill_twiddles(float2* tw) {
  for (int m = threadIdx.x; m < L; m += NT) tw[m] = twiddle_detail::kTable<L>.v[m];
}

// exp(i phi) for a float32 phase |phi| <= 1.6 (the sub-pixel shift ramps:
// |2 pi k d| <= pi / 2), cos and sin each rounded once to float.
//
// GB300 runs float64 at a small fraction of its float32 rate, so the values
// are summed in double-float arithmetic (an unevaluated float pair hi + lo,
// about 44 significant bits) from their Taylor series: sin phi = phi S(phi^2),
// cos phi = C(phi^2), with S and C evaluated by Horner's rule over 12 terms
// (truncation below 2e-18 for |phi| <= 1.6). The pair's leading float is the
// float nearest to the sum. The coefficients (-1)^n / (2n+1)! and
// (-1)^n / (2n)! are split into float pairs at compile time. Larger arguments
// fall back to float64.
namespace cis_detail {
struct DF {
  float hi, lo;
};
__device__ __forceinline__ DF two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ DF quick_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ DF df_mul(DF a, DF b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return quick_two_sum(p, e);
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
  DF s = two_sum(a.hi, b.hi);
  s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return quick_two_sum(s.hi, s.lo);
}
constexpr double factorial(int n) { return n <= 1 ? 1.0 : n * factorial(n - 1); }
constexpr double coef(int n, bool sine) {
  return (n % 2 ? -1.0 : 1.0) / factorial(sine ? 2 * n + 1 : 2 * n);
}
struct Coefs {
  float shi[12], slo[12], chi[12], clo[12];
};
constexpr Coefs make_coefs() {
  Coefs c{};
  for (int n = 0; n < 12; ++n) {
    const double s = coef(n, true), k = coef(n, false);
    c.shi[n] = (float)s;
    c.slo[n] = (float)(s - (double)(float)s);
    c.chi[n] = (float)k;
    c.clo[n] = (float)(k - (double)(float)k);
  }
  return c;
}
__device__ constexpr Coefs kCoefs = make_coefs();
}  // namespace cis_detail

__device__ __forceinline__ float2 cis_rounded(float phi) {
  using namespace cis_detail;
  if (!(fabsf(phi) <= 1.6f)) {
    double s, c;
    sincos((double)phi, &s, &c);
    return make_float2((float)c, (float)s);
  }
  const DF x{phi, 0.0f};
  const DF x2 = df_mul(x, x);
  DF s{kCoefs.shi[11], kCoefs.slo[11]};
  DF c{kCoefs.chi[11], kCoefs.clo[11]};
#pragma unroll
  for (int n = 10; n >= 0; --n) {
    s = df_add(df_mul(s, x2), DF{kCoefs.shi[n], kCoefs.slo[n]});
    c = df_add(df_mul(c, x2), DF{kCoefs.chi[n], kCoefs.clo[n]});
  }
  s = df_mul(s, x);
  return make_float2(__fadd_rn(c.hi, c.lo), __fadd_rn(s.hi, s.lo));
}

// Barriers a pass synchronises its threads with: the whole block, or a named
// barrier of one group of warps that owns its lines alone (bar.sync id, n;
// ids 1..15, id 0 being the block barrier).
struct BlockSync {
  __device__ __forceinline__ void operator()() const { __syncthreads(); }
};
struct GroupSync {
  int id, threads;
  __device__ __forceinline__ void operator()() const {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(threads) : "memory");
  }
};

// One Stockham pass over NLINES lines of length L with radix R; NS is the length
// of the sub-transforms already completed. Lanes of a warp take consecutive
// lines, so with a pitch of SY+1 rows (row pass) or unit-stride columns (column
// pass) the 32 lanes touch 32 distinct banks pairs. The NT threads that own the
// lines (thread index tid < NT among them) synchronise through `sync`.
template <int L, int R, int NS, int NLINES, int NT, int DIR, typename Sync>
__device__ __forceinline__ void line_pass(float2* buf, int line_stride, int elem_stride,
                                          const float2* __restrict__ tw, int tid, Sync sync) {
  constexpr int BF = L / R;            // butterflies per line
  constexpr int WORK = NLINES * BF;    // butterflies per pass
  constexpr int ITEMS = (WORK + NT - 1) / NT;
  static_assert(L % (NS * R) == 0, "invalid Stockham schedule");
  float2 v[ITEMS][R];
#pragma unroll
  for (int it = 0; it < ITEMS; ++it) {
    const int w = tid + it * NT;
    if (WORK % NT == 0 || w < WORK) {
      const int line = w % NLINES;
      const int j = w / NLINES;
      const float2* p = buf + line * line_stride;
#pragma unroll
      for (int k = 0; k < R; ++k) v[it][k] = p[(j + k * BF) * elem_stride];
      if constexpr (NS > 1) {
        const int jm = j % NS;
#pragma unroll
        for (int k = 1; k < R; ++k) {
          float2 t = tw[(jm * k * (L / (NS * R))) % L];
          if (DIR > 0) t.y = -t.y;
          v[it][k] = c_mul(v[it][k], t);
        }
      }
      float2 (&row)[R] = v[it];
      dft<R, DIR>(row);
    }
  }
  sync();
#pragma unroll
  for (int it = 0; it < ITEMS; ++it) {
    const int w = tid + it * NT;
    if (WORK % NT == 0 || w < WORK) {
      const int line = w % NLINES;
      const int j = w / NLINES;
      const int jm = j % NS;
      const int base = (j / NS) * NS * R + jm;
      float2* p = buf + line * line_stride;
#pragma unroll
      for (int k = 0; k < R; ++k) p[(base + k * NS) * elem_stride] = v[it][k];
    }
  }
  sync();
}

// Radix schedule per transform length: a compile-time list of passes.
#define PTY_PASS(L, R, NS) line_pass<L, R, NS, NLINES, NT, DIR>(b, ls, es, tw, tid, sync)
#define PTY_SCHEDULE_RUN                                                                  \
  template <int NLINES, int NT, int DIR, typename Sync = BlockSync>                       \
  __device__ static void run(float2* b, int ls, int es, const float2* tw, int tid,        \
                             Sync sync = Sync())
template <int L>
struct Schedule;
template <>
struct Schedule<16> {
  PTY_SCHEDULE_RUN { PTY_PASS(16, 16, 1); }
};
template <>
struct Schedule<32> {
  PTY_SCHEDULE_RUN {
    PTY_PASS(32, 8, 1);
    PTY_PASS(32, 4, 8);
  }
};
template <>
struct Schedule<48> {
  PTY_SCHEDULE_RUN {
    PTY_PASS(48, 16, 1);
    PTY_PASS(48, 3, 16);
  }
};
template <>
struct Schedule<64> {
  PTY_SCHEDULE_RUN {
    PTY_PASS(64, 8, 1);
    PTY_PASS(64, 8, 8);
  }
};
template <>
struct Schedule<96> {
  PTY_SCHEDULE_RUN {
    PTY_PASS(96, 8, 1);
    PTY_PASS(96, 4, 8);
    PTY_PASS(96, 3, 32);
  }
};
template <>
struct Schedule<128> {
  PTY_SCHEDULE_RUN {
    PTY_PASS(128, 16, 1);
    PTY_PASS(128, 8, 16);
  }
};
template <>
struct Schedule<256> {
  PTY_SCHEDULE_RUN {
    PTY_PASS(256, 16, 1);
    PTY_PASS(256, 16, 16);
  }
};
#undef PTY_SCHEDULE_RUN
#undef PTY_PASS

// Full 2D transform of the SX x SY block in shared memory (pitch SY + 1).
// twx: table for length SX, twy: table for length SY.
template <int SX, int SY, int NT, int DIR>
__device__ __forceinline__ void fft2d(float2* buf, const float2* twx, const float2* twy) {
  constexpr int LD = SY + 1;
  // rows: SX lines of length SY, contiguous
  Schedule<SY>::template run<SX, NT, DIR>(buf, LD, 1, twy, threadIdx.x);
  // columns: SY lines of length SX, stride LD
  Schedule<SX>::template run<SY, NT, DIR>(buf, 1, LD, twx, threadIdx.x);
}

}  // namespace pty
