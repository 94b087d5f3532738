// Fused per-position kernel: one thread block owns one scan position of the
// batch and runs the whole forward model, Fourier projection and the per-position
// half of the adjoint with the wave resident in shared memory.
//
// Per position b (reference operators in parentheses, py4DSTEM 0.14.18):
//   shifted probe   P_m = IFFT2( FFT2(P_m) . exp(-2 pi i (kx dx + ky dy)) )
//                                  (utils.py:468-533 fft_shift, ptychographic_methods.py:1482)
//   object patch    O_s = object_s[(x0 + fx) mod Px, (y0 + fy) mod Py], exp(iV) for
//                   potentials   (phase_base_class.py:1970-2003, ptychographic_methods.py:1489-1527)
//   multislice      P_{s+1} = IFFT2( FFT2(P_s O_s) H_s )     (ptychographic_methods.py:2300-2351, 383-401)
//   projection      F = FFT2(psi); err = sum (A - |F|)^2;
//                   GD: chi = IFFT2(A F/|F| - F); mixed: chi_m = IFFT2((A/|F|tot) F_m - F_m)
//                   projection sets: exit-wave update with (a,b,c)
//                                  (ptychographic_methods.py:1576-1734, 2742-2904)
//   adjoint terms   conj(P_s) chi_s, |P_s|^2 (object), conj(O) chi, |O|^2 (probe);
//                   multislice back-transmits and back-propagates chi
//                                  (ptychographic_methods.py:1818-1908, 2353-2565, 2906-3093)
// The adjoint terms go to position-major staging buffers; ptycho_reduce.cu sums
// them over positions in a fixed order. position_one runs every phase with the
// whole block; position_grouped_128 (the default at 128 x 128) runs the same
// model with 8 groups of warps that synchronise among themselves between the
// turns of its transforms.
//
// This header holds the kernel templates; ptycho_position_<S>.cu instantiates
// them for one region-of-interest edge S each (the translation units compile in
// parallel) and ptycho_position.cu dispatches on the edge.
#pragma once

#include <cuda_runtime.h>

#include "fft_smem.cuh"
#include "ptycho_internal.h"

namespace pty {
namespace {

__device__ __forceinline__ int pmod(int v, int m) {
  int r = v % m;
  return r < 0 ? r + m : r;
}

// numpy.fft.fftfreq(n, 1/n) as an integer: i for i < (n+1)/2, else i - n.
__device__ __forceinline__ int fint(int i, int n) { return i < (n + 1) / 2 ? i : i - n; }

template <int SX, int SY>
struct Layout {
  static constexpr int N = SX * SY;
  static constexpr int LD = SY + 1;
  static constexpr size_t smem_bytes(bool mixed) {
    return sizeof(float2) * (size_t)(SX * LD + 2 * SX + 2 * SY) + (mixed ? sizeof(float) * N : 0);
  }
};

__device__ __forceinline__ float2 load_object(const BatchArgs& a, int s, int ox, int oy) {
  const size_t idx = ((size_t)s * a.Px + ox) * a.Py + oy;
  if (a.potential) {
    float sv, cv;
    sincosf(reinterpret_cast<const float*>(a.object)[idx], &sv, &cv);
    return make_float2(cv, sv);
  }
  return reinterpret_cast<const float2*>(a.object)[idx];
}

// Object-gradient term for one pixel: conj(P) chi for complex objects and
// Re(-i conj(O) conj(P) chi) for potentials (stored in .x).
__device__ __forceinline__ float2 object_term(int potential, float2 o, float2 p, float2 chi) {
  if (potential) {
    const float2 t = make_float2(-o.y, -o.x);          // -i * conj(O)
    const float2 u = c_mul(t, make_float2(p.x, -p.y));  // * conj(P)
    const float2 v = c_mul(u, chi);                     // * chi
    return make_float2(v.x, 0.0f);
  }
  return c_conj_mul(p, chi);
}

// Block-wide deterministic sum (fixed shuffle tree, then warp order).
template <int NT>
__device__ __forceinline__ float block_sum(float v, float* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  float t = 0.0f;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int w = 0; w < NT / 32; ++w) t += red[w];
  }
  return t;  // valid in thread 0
}


// Everything of one scan position b (see the file header); the block's shared
// memory holds the wave, the tables and the ramps. `red` is the block-sum scratch.
// kMode fixes at compile time what the batch is (fewer live registers, fewer
// spills): 0 any single slice or single-probe multislice, 1 single slice /
// single probe, 2 single-slice mixed state, 3 multislice / single probe, 4
// mixed-state multislice; modes 1-3 are gradient descent with no projection
// sets, forward-only pass, kept far fields or exact probe gradient; mode 4 runs
// every variant of the mixed-state multislice model (its far fields always stay
// in scratch_f).
template <int SX, int SY, int NT, int kMode>
__device__ __forceinline__ void position_one(const BatchArgs& a, const int b, float* red) {
  constexpr bool kPlain = kMode >= 1 && kMode <= 3;
  constexpr bool kT1 = kMode == 1 || kMode == 2;
  constexpr bool kM1 = kMode == 1 || kMode == 3;
  using L = Layout<SX, SY>;
  constexpr int N = L::N;
  constexpr int LD = L::LD;
  extern __shared__ float4 smem4[];
  float2* buf = reinterpret_cast<float2*>(smem4);
  float2* twx = buf + SX * LD;
  float2* twy = twx + SX;
  float2* rpx = twy + SY;
  float2* rpy = rpx + SX;
  float* itot = reinterpret_cast<float*>(rpy + SY);  // N floats, mixed only

  const int tid = threadIdx.x;
  const int T = kT1 ? 1 : a.T;
  const int M = kM1 ? 1 : a.M;
  const int prow = a.pos_rows ? a.pos_rows[b] : b;
  const int arow = a.amp_rows ? a.amp_rows[b] : b;
  const bool pos_ok = isfinite(a.positions[2 * prow]) && isfinite(a.positions[2 * prow + 1]);
  const float posx = finite_or_zero(a.positions[2 * prow]);
  const float posy = finite_or_zero(a.positions[2 * prow + 1]);
  const float rx = rintf(posx);  // numpy.round: half to even
  const float ry = rintf(posy);
  const float dx = posx - rx;
  const float dy = posy - ry;
  const int x0 = (int)rx;
  const int y0 = (int)ry;
  const float invN = 1.0f / (float)N;
  const bool ps = !kPlain && a.projection != 0;
  const bool fwd = !kPlain && a.forward_only != 0;  // per-position error only (block-uniform)
  const float* amp = a.amplitudes + (size_t)arow * N;

  for (int i = tid; i < SX; i += NT) twx[i] = a.tw[i];  // tables from the spectrum kernel
  for (int i = tid; i < SY; i += NT) twy[i] = a.tw[SX + i];
  // separable sub-pixel shift ramps exp(-2 pi i k d): the phase is formed in
  // float32 like the reference's complex64 expression, its cos/sin rounded once
  for (int i = tid; i < SX; i += NT) {
    const float k = (float)fint(i, SX) / (float)SX;
    rpx[i] = cis_rounded(__fmul_rn(__fmul_rn(-6.2831855f, k), dx));
  }
  for (int i = tid; i < SY; i += NT) {
    const float k = (float)fint(i, SY) / (float)SY;
    rpy[i] = cis_rounded(__fmul_rn(__fmul_rn(-6.2831855f, k), dy));
  }
  if (tid == 0) a.pos_round[b] = make_int2(x0, y0);
  __syncthreads();

  // (c0 + fint(i)) mod P as base + ((i + S/2) mod S) with one wrap (P >= S)
  const int bx = pmod(x0 - SX / 2, a.Px);
  const int by = pmod(y0 - SY / 2, a.Py);
  auto obj_x = [&](int x) {
    const int t = bx + (x + SX / 2) % SX;
    return t >= a.Px ? t - a.Px : t;
  };
  auto obj_y = [&](int y) {
    const int t = by + (y + SY / 2) % SY;
    return t >= a.Py ? t - a.Py : t;
  };

  // Elementwise phases walk e = tid + i * NT (PER samples per thread) in chunks of
  // CH: all global loads of a chunk are issued before any of them is used, so a
  // thread keeps CH L2 requests in flight instead of one.
  constexpr int PER = N / NT;
  constexpr int CH = PER % 8 == 0 ? 8 : (PER % 6 == 0 ? 6 : (PER % 4 == 0 ? 4 : 1));
  static_assert(N % NT == 0 && PER % CH == 0, "samples per thread");

  // buf <- IFFT2(FFT2(P_m) . ramp) * 1/N  (sub-pixel shifted probe, mode m)
  auto shifted_probe = [&](int m) {
    const float2* __restrict__ spec = a.probe_spec + (size_t)m * N;
#pragma unroll
    for (int c0 = 0; c0 < PER; c0 += CH) {
      float2 sv[CH];
#pragma unroll
      for (int i = 0; i < CH; ++i) sv[i] = __ldg(spec + tid + (c0 + i) * NT);
#pragma unroll
      for (int i = 0; i < CH; ++i) {
        const int e = tid + (c0 + i) * NT;
        const int x = e / SY, y = e % SY;
        buf[x * LD + y] = c_mul(sv[i], c_mul(rpx[x], rpy[y]));
      }
    }
    __syncthreads();
    fft2d<SX, SY, NT, +1>(buf, twx, twy);
  };

  // Exact probe gradient (autograd backward): the probe reaches position b
  // through the sub-pixel shift S_b = IFFT2 diag(ramp) FFT2, so its term is
  // S_b^H (conj(O) chi) = IFFT2(conj(ramp) FFT2(conj(O) chi)). The reference's
  // update omits S_b^H; here the FFT2 and the conj(ramp) are applied per position
  // and the IFFT2 once to the batch sum. buf holds conj(O) chi on entry.
  const bool exact = !kPlain && a.exact_probe_grad != 0;
  auto unshift_probe_term = [&](float2* dst) {
    fft2d<SX, SY, NT, -1>(buf, twx, twy);
    for (int e = tid; e < N; e += NT) {
      const int x = e / SY, y = e % SY;
      const float2 r = c_mul(rpx[x], rpy[y]);
      dst[e] = c_mul(buf[x * LD + y], make_float2(r.x, -r.y));
    }
    __syncthreads();
  };

  float err = 0.0f;
  const float px_ = 1.0f - a.pa - a.pb;  // projection x
  const float py_ = 1.0f - a.pc;          // projection y

  if constexpr (kMode == 4) {
    // ------------------------------- mixed-state multislice (GD or projection sets)
    // (ptychographic_methods.py:3102-3160 forward, 2742-2904 projections,
    // 3162-3400 adjoints). Every mode runs through the slices on its own:
    // P_{s+1,m} = IFFT2(FFT2(O_s P_{s,m}) H_s), with each P_{s,m} stashed; the far
    // fields F_m share the ratio A / sqrt(sum_m |F_m|^2); the adjoint of each mode
    // walks back through the slices, adding conj(P_{s,m}) chi_{s,m} and |P_{s,m}|^2
    // into slice s's staged terms.
    for (int m = 0; m < M; ++m) {
      shifted_probe(m);
      for (int s = 0; s < T; ++s) {
        float2* pst = a.st_pm + (((size_t)s * a.B + b) * M + m) * N;
        for (int e = tid; e < N; e += NT) {
          const int x = e / SY, y = e % SY;
          const float2 p = c_scale(buf[x * LD + y], invN);
          pst[e] = p;
          buf[x * LD + y] = c_mul(load_object(a, s, obj_x(x), obj_y(y)), p);
        }
        __syncthreads();
        if (s + 1 < T) {
          fft2d<SX, SY, NT, -1>(buf, twx, twy);
          const float2* h = a.props + (size_t)s * N;
          for (int e = tid; e < N; e += NT) {
            const int idx = (e / SY) * LD + e % SY;
            buf[idx] = c_mul(buf[idx], h[e]);
          }
          __syncthreads();
          fft2d<SX, SY, NT, +1>(buf, twx, twy);
        }
      }
      if (ps) {
        // projection sets: the factor c psi + (1 - c) exit wave is projected
        const float2* ew = a.exit_waves + ((size_t)prow * M + m) * N;
        for (int e = tid; e < N; e += NT) {
          const int idx = (e / SY) * LD + e % SY;
          const float2 psi = buf[idx];
          const float2 w = a.ew_valid ? ew[e] : psi;
          buf[idx] = c_add(c_scale(psi, a.pc), c_scale(w, py_));
        }
        __syncthreads();
      }
      fft2d<SX, SY, NT, -1>(buf, twx, twy);
      float2* f = a.scratch_f + ((size_t)b * M + m) * N;
      for (int e = tid; e < N; e += NT) {
        const float2 v = buf[(e / SY) * LD + e % SY];
        f[e] = v;
        const float av = hypotf(v.x, v.y);  // |F_m|^2 as numpy forms it
        itot[e] = (m == 0 ? 0.0f : itot[e]) + av * av;
      }
      __syncthreads();
    }
    for (int e = tid; e < N; e += NT) {
      const float mk = a.det_mask ? a.det_mask[e] : 1.0f;
      float tot = sqrtf(itot[e]);
      if (a.det_mask) tot = sqrtf(itot[e] * mk * mk);
      const float A = amp[e];
      const float d = A - tot;
      err += d * d;
      itot[e] = tot == 0.0f ? 0.0f : A / tot;
    }
    __syncthreads();
    if (fwd) goto done;
    for (int m = 0; m < M; ++m) {
      const float2* f = a.scratch_f + ((size_t)b * M + m) * N;
      for (int e = tid; e < N; e += NT) {
        const float mk = a.det_mask ? a.det_mask[e] : 1.0f;
        float2 fv = f[e];
        if (a.det_mask) fv = c_scale(fv, mk);
        float2 r = c_scale(fv, itot[e]);
        if (!ps) {
          r = c_sub(r, fv);
          if (a.det_mask) r = c_scale(r, mk);
        }
        buf[(e / SY) * LD + e % SY] = r;
      }
      __syncthreads();
      fft2d<SX, SY, NT, +1>(buf, twx, twy);
      if (ps) {
        // new exit wave x w + a psi + b projected; psi recomputed from the stash
        float2* ew = a.exit_waves + ((size_t)prow * M + m) * N;
        const float2* plast = a.st_pm + (((size_t)(T - 1) * a.B + b) * M + m) * N;
        for (int e = tid; e < N; e += NT) {
          const int x = e / SY, y = e % SY;
          const float2 proj = c_scale(buf[x * LD + y], invN);
          const float2 psi = c_mul(load_object(a, T - 1, obj_x(x), obj_y(y)), plast[e]);
          const float2 w = a.ew_valid ? ew[e] : psi;
          const float2 nw = c_add(c_add(c_scale(w, px_), c_scale(psi, a.pa)), c_scale(proj, a.pb));
          ew[e] = nw;
          buf[x * LD + y] = c_scale(nw, (float)N);  // keep buf in unscaled units
        }
        __syncthreads();
      }
      for (int s = T - 1; s >= 0; --s) {
        const float2* pst = a.st_pm + (((size_t)s * a.B + b) * M + m) * N;
        float2* gobj = a.st_obj + ((size_t)s * a.B + b) * N;
        float* nobj = a.st_nobj + ((size_t)s * a.B + b) * N;
        for (int e = tid; e < N; e += NT) {
          const int x = e / SY, y = e % SY;
          const int idx = x * LD + y;
          const float2 chi = c_scale(buf[idx], invN);
          const float2 p = pst[e];
          const float2 o = load_object(a, s, obj_x(x), obj_y(y));
          const float2 g = object_term(a.potential, o, p, chi);
          const float pn = c_abs2(p);
          if (m == 0) {
            gobj[e] = g;
            nobj[e] = pn;
          } else {
            gobj[e] = c_add(gobj[e], g);
            nobj[e] = nobj[e] + pn;
          }
          const float2 bt = c_mul(chi, make_float2(o.x, -o.y));  // chi * conj(O_s)
          if (s > 0 || exact) {
            buf[idx] = bt;
          } else {
            a.st_probe[((size_t)b * M + m) * N + e] = bt;
          }
          if (s == 0 && m == 0) a.st_nprobe[(size_t)b * N + e] = c_abs2(o);
        }
        __syncthreads();
        if (s == 0 && exact) unshift_probe_term(a.st_probe + ((size_t)b * M + m) * N);
        if (s > 0) {
          fft2d<SX, SY, NT, -1>(buf, twx, twy);
          const float2* h = a.props + (size_t)(s - 1) * N;
          for (int e = tid; e < N; e += NT) {
            const int idx = (e / SY) * LD + e % SY;
            const float2 hv = h[e];
            buf[idx] = c_mul(buf[idx], make_float2(hv.x, -hv.y));
          }
          __syncthreads();
          fft2d<SX, SY, NT, +1>(buf, twx, twy);
        }
      }
    }
    if (ps && a.keep_farfield) {
      // projection sets with position correction: the far field of each mode's
      // psi at the last slice, O_{T-1} P_{T-1,m} from the stash
      for (int m = 0; m < M; ++m) {
        const float2* plast = a.st_pm + (((size_t)(T - 1) * a.B + b) * M + m) * N;
        __syncthreads();
        for (int e = tid; e < N; e += NT) {
          const int x = e / SY, y = e % SY;
          buf[x * LD + y] = c_mul(load_object(a, T - 1, obj_x(x), obj_y(y)), plast[e]);
        }
        __syncthreads();
        fft2d<SX, SY, NT, -1>(buf, twx, twy);
        float2* f = a.scratch_f + ((size_t)b * M + m) * N;
        for (int e = tid; e < N; e += NT) f[e] = buf[(e / SY) * LD + e % SY];
      }
    }
  } else {
  if (T == 1) {
    // ------------------------------------------------------------ single slice
    const bool mixed = kMode == 2 || (kMode == 0 && (M > 1 || a.mixed_formula));
    for (int m = 0; m < M; ++m) {
      shifted_probe(m);
      float2* pst = a.st_probe + ((size_t)b * M + m) * N;  // stash P_m
      const float2* ew = a.exit_waves ? a.exit_waves + ((size_t)prow * M + m) * N : nullptr;
#pragma unroll
      for (int c0 = 0; c0 < PER; c0 += CH) {
        float2 ov[CH];
#pragma unroll
        for (int i = 0; i < CH; ++i) {
          const int e = tid + (c0 + i) * NT;
          ov[i] = load_object(a, 0, obj_x(e / SY), obj_y(e % SY));
        }
#pragma unroll
        for (int i = 0; i < CH; ++i) {
          const int e = tid + (c0 + i) * NT;
          const int x = e / SY, y = e % SY;
          const float2 p = c_scale(buf[x * LD + y], invN);
          pst[e] = p;
          const float2 psi = c_mul(p, ov[i]);
          float2 v = psi;
          if (ps) {
            const float2 w = a.ew_valid ? ew[e] : psi;
            v = c_add(c_scale(psi, a.pc), c_scale(w, py_));
            // position correction works on FFT2(psi), not on the projected factor;
            // a single probe's psi waits here and is transformed at the end
            if (a.keep_farfield && !mixed) a.scratch_f[(size_t)b * N + e] = psi;
          }
          buf[x * LD + y] = v;
        }
      }
      __syncthreads();
      fft2d<SX, SY, NT, -1>(buf, twx, twy);
      if (mixed) {
        float2* f = a.scratch_f + ((size_t)b * M + m) * N;
        for (int e = tid; e < N; e += NT) {
          const float2 v = buf[(e / SY) * LD + e % SY];
          f[e] = v;
          // |F_m|^2 as numpy forms it: abs() then square
          const float av = hypotf(v.x, v.y);
          itot[e] = (m == 0 ? 0.0f : itot[e]) + av * av;
        }
        __syncthreads();
      }
    }

    if (!mixed) {
      // single probe: A exp(i angle F) - F (GD) or A exp(i angle F) (projection)
#pragma unroll
      for (int c0 = 0; c0 < PER; c0 += CH) {
      float av[CH];
#pragma unroll
      for (int i = 0; i < CH; ++i) av[i] = __ldg(amp + tid + (c0 + i) * NT);
#pragma unroll
      for (int i = 0; i < CH; ++i) {
        const int e = tid + (c0 + i) * NT;
        const int idx = (e / SY) * LD + e % SY;
        float2 f = buf[idx];
        if (!kPlain && a.keep_farfield && !ps) a.scratch_f[(size_t)b * N + e] = f;  // unmasked, A16
        const float mk = a.det_mask ? a.det_mask[e] : 1.0f;
        if (a.det_mask) f = c_scale(f, mk);
        const float af = c_abs(f);
        const float A = av[i];
        const float d = A - af;
        err += d * d;
        // A exp(i angle F) (- F for gradient descent), one division per pixel
        const float q = af > 0.0f ? A / af : 0.0f;
        float2 r = af > 0.0f ? c_scale(f, q) : make_float2(A, 0.0f);
        if (!ps) {
          r = af > 0.0f ? make_float2(fmaf(f.x, q, -f.x), fmaf(f.y, q, -f.y)) : c_sub(r, f);
          if (a.det_mask) r = c_scale(r, mk);
        }
        buf[idx] = r;
      }
      }
      if (!fwd) {
        __syncthreads();
        fft2d<SX, SY, NT, +1>(buf, twx, twy);
      }
    } else {
      // mixed state: shared ratio A / sqrt(sum_m |F_m|^2), 0 where the model is 0
      for (int e = tid; e < N; e += NT) {
        const float mk = a.det_mask ? a.det_mask[e] : 1.0f;
        float tot = sqrtf(itot[e]);
        if (a.det_mask) tot = sqrtf(itot[e] * mk * mk);
        const float A = amp[e];
        const float d = A - tot;
        err += d * d;
        itot[e] = tot == 0.0f ? 0.0f : A / tot;
      }
      __syncthreads();
    }

    // adjoint terms, mode by mode
    for (int m = 0; m < (fwd ? 0 : M); ++m) {
      if (mixed) {
        const float2* f = a.scratch_f + ((size_t)b * M + m) * N;
        for (int e = tid; e < N; e += NT) {
          const float mk = a.det_mask ? a.det_mask[e] : 1.0f;
          float2 fv = f[e];
          if (a.det_mask) fv = c_scale(fv, mk);
          float2 r = c_scale(fv, itot[e]);
          if (!ps) {
            r = c_sub(r, fv);
            if (a.det_mask) r = c_scale(r, mk);
          }
          buf[(e / SY) * LD + e % SY] = r;
        }
        __syncthreads();
        fft2d<SX, SY, NT, +1>(buf, twx, twy);
      }
      float2* pst = a.st_probe + ((size_t)b * M + m) * N;
      float2* ew = a.exit_waves ? a.exit_waves + ((size_t)prow * M + m) * N : nullptr;
      float2* gobj = a.st_obj + (size_t)b * N;
      float* nobj = a.st_nobj + (size_t)b * N;
#pragma unroll
      for (int c0 = 0; c0 < PER; c0 += CH) {
      float2 ov[CH], pv[CH];
#pragma unroll
      for (int i = 0; i < CH; ++i) {
        const int e = tid + (c0 + i) * NT;
        ov[i] = load_object(a, 0, obj_x(e / SY), obj_y(e % SY));
        pv[i] = pst[e];
      }
#pragma unroll
      for (int i = 0; i < CH; ++i) {
        const int e = tid + (c0 + i) * NT;
        const int x = e / SY, y = e % SY;
        float2 chi = c_scale(buf[x * LD + y], invN);
        const float2 p = pv[i];
        const float2 o = ov[i];
        if (ps) {
          const float2 psi = c_mul(p, o);
          const float2 w = a.ew_valid ? ew[e] : psi;
          chi = c_add(c_add(c_scale(w, px_), c_scale(psi, a.pa)), c_scale(chi, a.pb));
          ew[e] = chi;
        }
        const float2 g = object_term(a.potential, o, p, chi);
        const float pn = c_abs2(p);
        if (m == 0) {
          gobj[e] = g;
          nobj[e] = pn;
        } else {
          gobj[e] = c_add(gobj[e], g);
          nobj[e] = nobj[e] + pn;
        }
        const float2 yv = c_conj_mul(o, chi);
        if (exact) buf[x * LD + y] = yv; else pst[e] = yv;
        // (the plain GD instantiation stages no |O|^2: the probe-side
        // reduction gathers it from the object, nprobe_from_object)
        if (kMode != 1 && m == 0) a.st_nprobe[(size_t)b * N + e] = c_abs2(o);
      }
      }
      __syncthreads();
      if (exact) unshift_probe_term(pst);
    }
  } else {
    // ------------------------------------------------------------- multislice
    shifted_probe(0);
    for (int s = 0; s < T; ++s) {
      float2* pst = a.st_obj + ((size_t)s * a.B + b) * N;  // stash P_s
      for (int e = tid; e < N; e += NT) {
        const int x = e / SY, y = e % SY;
        float2 p = buf[x * LD + y];
        p = c_scale(p, invN);
        const float2 o = load_object(a, s, obj_x(x), obj_y(y));
        pst[e] = p;
        buf[x * LD + y] = c_mul(o, p);
      }
      __syncthreads();
      if (s + 1 < T) {
        fft2d<SX, SY, NT, -1>(buf, twx, twy);
        const float2* h = a.props + (size_t)s * N;
        for (int e = tid; e < N; e += NT) {
          const int idx = (e / SY) * LD + e % SY;
          buf[idx] = c_mul(buf[idx], h[e]);
        }
        __syncthreads();
        fft2d<SX, SY, NT, +1>(buf, twx, twy);
      }
    }
    // buf = psi_{T-1} (unscaled exit wave of the last slice)
    const float2* ew_in = a.exit_waves ? a.exit_waves + (size_t)prow * N : nullptr;
    if (ps) {
      for (int e = tid; e < N; e += NT) {
        const int idx = (e / SY) * LD + e % SY;
        const float2 psi = buf[idx];
        const float2 w = a.ew_valid ? ew_in[e] : psi;
        buf[idx] = c_add(c_scale(psi, a.pc), c_scale(w, py_));
        if (a.keep_farfield) a.scratch_f[(size_t)b * N + e] = psi;  // see the single slice
      }
      __syncthreads();
    }
    fft2d<SX, SY, NT, -1>(buf, twx, twy);
    for (int e = tid; e < N; e += NT) {
      const int idx = (e / SY) * LD + e % SY;
      float2 f = buf[idx];
      if (a.keep_farfield && !ps) a.scratch_f[(size_t)b * N + e] = f;  // unmasked, for A16
      const float mk = a.det_mask ? a.det_mask[e] : 1.0f;
      if (a.det_mask) f = c_scale(f, mk);
      const float af = c_abs(f);
      const float A = amp[e];
      const float d = A - af;
      err += d * d;
      // A exp(i angle F) (- F for gradient descent), one division per pixel
      const float q = af > 0.0f ? A / af : 0.0f;
      float2 r = af > 0.0f ? c_scale(f, q) : make_float2(A, 0.0f);
      if (!ps) {
        r = af > 0.0f ? make_float2(fmaf(f.x, q, -f.x), fmaf(f.y, q, -f.y)) : c_sub(r, f);
        if (a.det_mask) r = c_scale(r, mk);
      }
      buf[idx] = r;
    }
    if (fwd) goto done;
    __syncthreads();
    fft2d<SX, SY, NT, +1>(buf, twx, twy);
    if (ps) {
      // new exit wave of the last slice; psi recomputed from the stash
      float2* ew = a.exit_waves + (size_t)prow * N;
      const float2* pst = a.st_obj + ((size_t)(T - 1) * a.B + b) * N;
      for (int e = tid; e < N; e += NT) {
        const int x = e / SY, y = e % SY;
        const float2 proj = c_scale(buf[x * LD + y], invN);
        const float2 psi = c_mul(load_object(a, T - 1, obj_x(x), obj_y(y)), pst[e]);
        const float2 w = a.ew_valid ? ew[e] : psi;
        const float2 nw = c_add(c_add(c_scale(w, px_), c_scale(psi, a.pa)), c_scale(proj, a.pb));
        ew[e] = nw;
        buf[x * LD + y] = c_scale(nw, (float)N);  // keep buf in unscaled units
      }
      __syncthreads();
    }
    for (int s = T - 1; s >= 0; --s) {
      float2* pst = a.st_obj + ((size_t)s * a.B + b) * N;
      float* nst = a.st_nobj + ((size_t)s * a.B + b) * N;
      for (int e = tid; e < N; e += NT) {
        const int x = e / SY, y = e % SY;
        const int idx = x * LD + y;
        const float2 chi = c_scale(buf[idx], invN);
        const float2 p = pst[e];
        const float2 o = load_object(a, s, obj_x(x), obj_y(y));
        pst[e] = object_term(a.potential, o, p, chi);
        nst[e] = c_abs2(p);
        const float2 bt = c_mul(chi, make_float2(o.x, -o.y));  // chi * conj(O_s)
        if (s > 0 || exact) buf[idx] = bt;
        if (s == 0) {
          if (!exact) a.st_probe[(size_t)b * N + e] = bt;
          a.st_nprobe[(size_t)b * N + e] = c_abs2(o);
        }
      }
      __syncthreads();
      if (s == 0 && exact) unshift_probe_term(a.st_probe + (size_t)b * N);
      if (s > 0) {
        fft2d<SX, SY, NT, -1>(buf, twx, twy);
        const float2* h = a.props + (size_t)(s - 1) * N;
        for (int e = tid; e < N; e += NT) {
          const int idx = (e / SY) * LD + e % SY;
          const float2 hv = h[e];
          buf[idx] = c_mul(buf[idx], make_float2(hv.x, -hv.y));
        }
        __syncthreads();
        fft2d<SX, SY, NT, +1>(buf, twx, twy);
      }
    }
  }

    if (ps && a.keep_farfield) {
      // projection sets with position correction: the far field of psi
      if (T > 1 || !(M > 1 || a.mixed_formula)) {
        float2* f = a.scratch_f + (size_t)b * N;
        __syncthreads();
        for (int e = tid; e < N; e += NT) buf[(e / SY) * LD + e % SY] = f[e];
        __syncthreads();
        fft2d<SX, SY, NT, -1>(buf, twx, twy);
        for (int e = tid; e < N; e += NT) f[e] = buf[(e / SY) * LD + e % SY];
      } else {
        // mixed state: psi_m = P_m O again (the probe stash now holds the
        // probe terms), then its far field, mode by mode
        for (int m = 0; m < M; ++m) {
          __syncthreads();
          shifted_probe(m);
          for (int e = tid; e < N; e += NT) {
            const int x = e / SY, y = e % SY;
            const float2 p = c_scale(buf[x * LD + y], invN);
            buf[x * LD + y] = c_mul(p, load_object(a, 0, obj_x(x), obj_y(y)));
          }
          __syncthreads();
          fft2d<SX, SY, NT, -1>(buf, twx, twy);
          float2* f = a.scratch_f + ((size_t)b * M + m) * N;
          for (int e = tid; e < N; e += NT) f[e] = buf[(e / SY) * LD + e % SY];
        }
      }
    }
  }  // kMode != 4

done:
  const float tot = block_sum<NT>(err, red);
  if (tid == 0) a.err[b] = pos_ok ? tot : __int_as_float(0x7fc00000);
}

// One block per position. (A persistent form, one block per SM walking the
// batch, measured 2% slower at 128 x 128 and was dropped.)
template <int SX, int SY, int NT, int kMode>
__global__ void __launch_bounds__(NT, 1) position_kernel(BatchArgs a) {
  __shared__ float red[NT / 32];
  position_one<SX, SY, NT, kMode>(a, blockIdx.x, red);
}

// The per-position model at 128 x 128 (kKind, see position_grouped_kernel) with
// the block split into 8 groups of 4 warps. A group owns 16 rows in the
// real-space phases and 16 columns in the Fourier-space phases; its elementwise
// work and its share of each 2D transform (the same Stockham passes and
// twiddles as fft2d, on its own lines) synchronise through a named barrier of
// its 128 threads. A block-wide barrier is needed only where a transform turns
// from one axis to the other (one per transform: 4 per position of single-slice
// gradient descent instead of the 24 of the block-wide schedule), and between
// them the groups drift apart in phase (one
// loading from memory while another runs its passes). To need no extra turn,
// the inverse transforms run columns then rows and the forward ones rows then
// columns (fft2d: rows then columns both ways), so results agree with the
// block-wide schedule to rounding, not bit for bit.
//   real space (row group g):      x = 16 g + i,          y = t        (i < 16)
//   Fourier space (column group g): x = t / 16 + 8 i,     y = 16 g + t % 16
// for thread t < 128 of the group; both walks are bank-conflict free on the
// pitch-129 wave and coalesced in global memory.
template <int NT, int kKind>
__device__ __forceinline__ void position_grouped_128(const BatchArgs& a, const int b,
                                                     float* red) {
  constexpr int S = 128;
  using L = Layout<S, S>;
  constexpr int N = L::N;
  constexpr int LD = L::LD;
  constexpr int GT = 128;                // threads per group
  constexpr int G = NT / GT;             // groups
  constexpr int LINES = S / G;           // rows (columns) a group owns
  constexpr int PER = LINES * S / GT;    // samples per thread
  constexpr int CH = 8;                  // global loads in flight per thread
  static_assert(NT == 1024 && LINES == 16 && PER == 16, "grouped 128 x 128 layout");
  extern __shared__ float4 smem4[];
  float2* buf = reinterpret_cast<float2*>(smem4);
  float2* twx = buf + S * LD;
  float2* twy = twx + S;
  float2* rpx = twy + S;
  float2* rpy = rpx + S;

  const int tid = threadIdx.x;
  const int g = tid / GT;
  const int tg = tid % GT;
  const GroupSync gsync{1 + g, GT};
  const int prow = a.pos_rows ? a.pos_rows[b] : b;
  const int arow = a.amp_rows ? a.amp_rows[b] : b;
  const bool pos_ok = isfinite(a.positions[2 * prow]) && isfinite(a.positions[2 * prow + 1]);
  const float posx = finite_or_zero(a.positions[2 * prow]);
  const float posy = finite_or_zero(a.positions[2 * prow + 1]);
  const float rx = rintf(posx);  // numpy.round: half to even
  const float ry = rintf(posy);
  const float dx = posx - rx;
  const float dy = posy - ry;
  const int x0 = (int)rx;
  const int y0 = (int)ry;
  const float invN = 1.0f / (float)N;
  const float* amp = a.amplitudes + (size_t)arow * N;

  for (int i = tid; i < S; i += NT) {
    twx[i] = a.tw[i];
    twy[i] = a.tw[S + i];
    const float k = (float)fint(i, S) / (float)S;
    rpx[i] = cis_rounded(__fmul_rn(__fmul_rn(-6.2831855f, k), dx));
  }
  for (int i = tid - S; i >= 0 && i < S; i += NT) {
    const float k = (float)fint(i, S) / (float)S;
    rpy[i] = cis_rounded(__fmul_rn(__fmul_rn(-6.2831855f, k), dy));
  }
  if (tid == 0) a.pos_round[b] = make_int2(x0, y0);
  __syncthreads();

  const int bx = pmod(x0 - S / 2, a.Px);
  const int by = pmod(y0 - S / 2, a.Py);
  auto obj_x = [&](int x) {
    const int t = bx + (x + S / 2) % S;
    return t >= a.Px ? t - a.Px : t;
  };
  auto obj_y = [&](int y) {
    const int t = by + (y + S / 2) % S;
    return t >= a.Py ? t - a.Py : t;
  };
  // sample i of this thread in either walk
  const int ry0 = LINES * g;                // real space: rows ry0 + i, column tg
  const int fx0 = tg / LINES;               // Fourier space: rows fx0 + 8 i,
  const int fy = LINES * g + tg % LINES;    //   column fy
  constexpr int FXS = GT / LINES;
  float2* const rows_g = buf + ry0 * LD;    // the group's rows
  float2* const cols_g = buf + LINES * g;   // the group's columns

  // the transforms of the group's lines: forward = rows then columns (real
  // space in, Fourier space out), inverse = columns then rows
  auto forward = [&]() {
    Schedule<S>::template run<LINES, GT, -1>(rows_g, LD, 1, twy, tg, gsync);
    __syncthreads();
    Schedule<S>::template run<LINES, GT, -1>(cols_g, 1, LD, twx, tg, gsync);
  };
  auto inverse = [&]() {
    Schedule<S>::template run<LINES, GT, +1>(cols_g, 1, LD, twx, tg, gsync);
    __syncthreads();
    Schedule<S>::template run<LINES, GT, +1>(rows_g, LD, 1, twy, tg, gsync);
  };
  // shifted probe of mode m: spectrum x ramps, inverse transform (columns,
  // then rows)
  auto shifted_probe = [&](int m) {
    const float2* __restrict__ spec = a.probe_spec + (size_t)m * N;
#pragma unroll 1  // (unrolled, the chunks' live values spill)
    for (int c0 = 0; c0 < PER; c0 += CH) {
      float2 sv[CH];
#pragma unroll
      for (int i = 0; i < CH; ++i) sv[i] = __ldg(spec + (fx0 + FXS * (c0 + i)) * S + fy);
#pragma unroll
      for (int i = 0; i < CH; ++i) {
        const int x = fx0 + FXS * (c0 + i);
        buf[x * LD + fy] = c_mul(sv[i], c_mul(rpx[x], rpy[fy]));
      }
    }
    gsync();
    inverse();
  };
  shifted_probe(0);

  // A exp(i angle F) - F on the group's columns, one division per pixel;
  // returns this thread's share of sum (A - |F|)^2. keep (or null) receives F
  // unmasked, for the position correction after the batch update.
  auto project = [&](float2* keep) {
    float err = 0.0f;
#pragma unroll 1  // (unrolled, the chunks' live values spill)
    for (int c0 = 0; c0 < PER; c0 += CH) {
      float av[CH];
#pragma unroll
      for (int i = 0; i < CH; ++i) av[i] = __ldg(amp + (fx0 + FXS * (c0 + i)) * S + fy);
#pragma unroll
      for (int i = 0; i < CH; ++i) {
        const int x = fx0 + FXS * (c0 + i);
        const int e = x * S + fy;
        const int idx = x * LD + fy;
        float2 f = buf[idx];
        if (keep) keep[e] = f;
        const float mk = a.det_mask ? a.det_mask[e] : 1.0f;
        if (a.det_mask) f = c_scale(f, mk);
        const float af = c_abs(f);
        const float A = av[i];
        const float d = A - af;
        err += d * d;
        const float q = af > 0.0f ? A / af : 0.0f;
        float2 r = af > 0.0f ? make_float2(fmaf(f.x, q, -f.x), fmaf(f.y, q, -f.y))
                             : c_sub(make_float2(A, 0.0f), f);
        if (a.det_mask) r = c_scale(r, mk);
        buf[idx] = r;
      }
    }
    return err;
  };
  float err = 0.0f;

  if constexpr (kKind == 0 || kKind == 5) {
    // psi = P O; P stashed for the adjoint
    float2* pst = a.st_probe + (size_t)b * N;
#pragma unroll 1  // (unrolled, the chunks' live values spill)
    for (int c0 = 0; c0 < PER; c0 += CH) {
      float2 ov[CH];
#pragma unroll
      for (int i = 0; i < CH; ++i) ov[i] = load_object(a, 0, obj_x(ry0 + c0 + i), obj_y(tg));
#pragma unroll
      for (int i = 0; i < CH; ++i) {
        const int x = ry0 + c0 + i;
        const float2 p = c_scale(buf[x * LD + tg], invN);
        pst[x * S + tg] = p;
        buf[x * LD + tg] = c_mul(p, ov[i]);
      }
    }
    gsync();
    forward();
    err = project(kKind == 5 ? a.scratch_f + (size_t)b * N : nullptr);
    gsync();
    inverse();

    // adjoint terms: conj(P) chi (or the potential's), |P|^2, conj(O) chi
    float2* gobj = a.st_obj + (size_t)b * N;
    float* nobj = a.st_nobj + (size_t)b * N;
#pragma unroll 1  // (unrolled, the chunks' live values spill)
    for (int c0 = 0; c0 < PER; c0 += CH) {
      float2 ov[CH], pv[CH];
#pragma unroll
      for (int i = 0; i < CH; ++i) {
        const int x = ry0 + c0 + i;
        ov[i] = load_object(a, 0, obj_x(x), obj_y(tg));
        pv[i] = pst[x * S + tg];
      }
#pragma unroll
      for (int i = 0; i < CH; ++i) {
        const int x = ry0 + c0 + i;
        const int e = x * S + tg;
        const float2 chi = c_scale(buf[x * LD + tg], invN);
        gobj[e] = object_term(a.potential, ov[i], pv[i], chi);
        nobj[e] = c_abs2(pv[i]);
        pst[e] = c_conj_mul(ov[i], chi);
        // (plain gradient descent leaves |O|^2 to the probe side's gather from
        // the object; with kept far fields the probe side reads it staged)
        if constexpr (kKind == 5) a.st_nprobe[(size_t)b * N + e] = c_abs2(ov[i]);
      }
    }
  } else if constexpr (kKind == 1) {
    // multislice: P_{s+1} = IFFT2(FFT2(O_s P_s) H_s), each P_s stashed in its
    // slice's object-term row (the adjoint overwrites it with the term)
    const int T = a.T;
    // buf (Fourier space, the group's columns) times H or conj(H)
    auto propagate = [&](const float2* __restrict__ h, bool conjugate) {
#pragma unroll 1
      for (int c0 = 0; c0 < PER; c0 += CH) {
        float2 hv[CH];
#pragma unroll
        for (int i = 0; i < CH; ++i) hv[i] = __ldg(h + (fx0 + FXS * (c0 + i)) * S + fy);
#pragma unroll
        for (int i = 0; i < CH; ++i) {
          const int idx = (fx0 + FXS * (c0 + i)) * LD + fy;
          buf[idx] = c_mul(buf[idx], conjugate ? make_float2(hv[i].x, -hv[i].y) : hv[i]);
        }
      }
    };
    for (int s = 0; s < T; ++s) {
      float2* pst = a.st_obj + ((size_t)s * a.B + b) * N;
#pragma unroll 1  // (unrolled, the chunks' live values spill)
      for (int c0 = 0; c0 < PER; c0 += CH) {
        float2 ov[CH];
#pragma unroll
        for (int i = 0; i < CH; ++i) ov[i] = load_object(a, s, obj_x(ry0 + c0 + i), obj_y(tg));
#pragma unroll
        for (int i = 0; i < CH; ++i) {
          const int x = ry0 + c0 + i;
          const float2 p = c_scale(buf[x * LD + tg], invN);
          pst[x * S + tg] = p;
          buf[x * LD + tg] = c_mul(ov[i], p);
        }
      }
      gsync();
      if (s + 1 < T) {
        forward();
        propagate(a.props + (size_t)s * N, false);
        gsync();
        inverse();
      }
    }
    forward();  // far field of the last slice's exit wave
    err = project(nullptr);
    gsync();
    inverse();
    // adjoint, slice by slice backwards; chi conj(O_s) goes back through the
    // propagator into the slice before, at slice 0 it is the probe term
    for (int s = T - 1; s >= 0; --s) {
      float2* pst = a.st_obj + ((size_t)s * a.B + b) * N;
      float* nst = a.st_nobj + ((size_t)s * a.B + b) * N;
#pragma unroll 1  // (unrolled, the chunks' live values spill)
      for (int c0 = 0; c0 < PER; c0 += CH) {
        float2 ov[CH], pv[CH];
#pragma unroll
        for (int i = 0; i < CH; ++i) {
          const int x = ry0 + c0 + i;
          ov[i] = load_object(a, s, obj_x(x), obj_y(tg));
          pv[i] = pst[x * S + tg];
        }
#pragma unroll
        for (int i = 0; i < CH; ++i) {
          const int x = ry0 + c0 + i;
          const int e = x * S + tg;
          const int idx = x * LD + tg;
          const float2 chi = c_scale(buf[idx], invN);
          pst[e] = object_term(a.potential, ov[i], pv[i], chi);
          nst[e] = c_abs2(pv[i]);
          const float2 bt = c_mul(chi, make_float2(ov[i].x, -ov[i].y));  // chi conj(O_s)
          if (s > 0) {
            buf[idx] = bt;
          } else {
            a.st_probe[(size_t)b * N + e] = bt;
            a.st_nprobe[(size_t)b * N + e] = c_abs2(ov[i]);
          }
        }
      }
      if (s > 0) {
        gsync();
        forward();
        propagate(a.props + (size_t)(s - 1) * N, true);
        gsync();
        inverse();
      }
    }
  } else if constexpr (kKind == 4) {
    // mixed-state multislice gradient descent: every mode through every slice,
    // P_{s+1,m} = IFFT2(FFT2(O_s P_{s,m}) H_s) with each P_{s,m} stashed; the far
    // fields F_m share the ratio A / sqrt(sum_m |F_m|^2); each mode's adjoint
    // walks back through the slices, summing its terms into slice s's rows
    const int T = a.T, M = a.M;
    float* itot = reinterpret_cast<float*>(rpy + S);  // N, indexed by Fourier pixel
    auto propagate = [&](const float2* __restrict__ h, bool conjugate) {
#pragma unroll 1
      for (int c0 = 0; c0 < PER; c0 += CH) {
        float2 hv[CH];
#pragma unroll
        for (int i = 0; i < CH; ++i) hv[i] = __ldg(h + (fx0 + FXS * (c0 + i)) * S + fy);
#pragma unroll
        for (int i = 0; i < CH; ++i) {
          const int idx = (fx0 + FXS * (c0 + i)) * LD + fy;
          buf[idx] = c_mul(buf[idx], conjugate ? make_float2(hv[i].x, -hv[i].y) : hv[i]);
        }
      }
    };
    for (int m = 0; m < M; ++m) {
      if (m > 0) shifted_probe(m);
      for (int s = 0; s < T; ++s) {
        float2* pst = a.st_pm + (((size_t)s * a.B + b) * M + m) * N;
#pragma unroll 1  // (unrolled, the chunks' live values spill)
        for (int c0 = 0; c0 < PER; c0 += CH) {
          float2 ov[CH];
#pragma unroll
          for (int i = 0; i < CH; ++i)
            ov[i] = load_object(a, s, obj_x(ry0 + c0 + i), obj_y(tg));
#pragma unroll
          for (int i = 0; i < CH; ++i) {
            const int x = ry0 + c0 + i;
            const float2 p = c_scale(buf[x * LD + tg], invN);
            pst[x * S + tg] = p;
            buf[x * LD + tg] = c_mul(ov[i], p);
          }
        }
        gsync();
        if (s + 1 < T) {
          forward();
          propagate(a.props + (size_t)s * N, false);
          gsync();
          inverse();
        }
      }
      forward();
      float2* f = a.scratch_f + ((size_t)b * M + m) * N;
      for (int i = 0; i < PER; ++i) {
        const int x = fx0 + FXS * i;
        const int e = x * S + fy;
        const float2 v = buf[x * LD + fy];
        f[e] = v;
        const float av = hypotf(v.x, v.y);  // |F_m|^2 as numpy forms it
        itot[e] = (m == 0 ? 0.0f : itot[e]) + av * av;
      }
    }
    for (int i = 0; i < PER; ++i) {
      const int e = (fx0 + FXS * i) * S + fy;
      const float mk = a.det_mask ? a.det_mask[e] : 1.0f;
      float tot = sqrtf(itot[e]);
      if (a.det_mask) tot = sqrtf(itot[e] * mk * mk);
      const float A = __ldg(amp + e);
      const float d = A - tot;
      err += d * d;
      itot[e] = tot == 0.0f ? 0.0f : A / tot;
    }
    for (int m = 0; m < M; ++m) {
      // (the previous mode's adjoint read the wave by rows)
      if (m > 0) __syncthreads();
      const float2* f = a.scratch_f + ((size_t)b * M + m) * N;
      for (int i = 0; i < PER; ++i) {
        const int x = fx0 + FXS * i;
        const int e = x * S + fy;
        const float mk = a.det_mask ? a.det_mask[e] : 1.0f;
        float2 fv = f[e];
        if (a.det_mask) fv = c_scale(fv, mk);
        float2 r = c_sub(c_scale(fv, itot[e]), fv);
        if (a.det_mask) r = c_scale(r, mk);
        buf[x * LD + fy] = r;
      }
      gsync();
      inverse();
      for (int s = T - 1; s >= 0; --s) {
        const float2* pst = a.st_pm + (((size_t)s * a.B + b) * M + m) * N;
        float2* gobj = a.st_obj + ((size_t)s * a.B + b) * N;
        float* nobj = a.st_nobj + ((size_t)s * a.B + b) * N;
#pragma unroll 1  // (unrolled, the chunks' live values spill)
        for (int c0 = 0; c0 < PER; c0 += CH) {
          float2 ov[CH], pv[CH];
#pragma unroll
          for (int i = 0; i < CH; ++i) {
            const int x = ry0 + c0 + i;
            ov[i] = load_object(a, s, obj_x(x), obj_y(tg));
            pv[i] = pst[x * S + tg];
          }
#pragma unroll
          for (int i = 0; i < CH; ++i) {
            const int x = ry0 + c0 + i;
            const int e = x * S + tg;
            const int idx = x * LD + tg;
            const float2 chi = c_scale(buf[idx], invN);
            const float2 g = object_term(a.potential, ov[i], pv[i], chi);
            const float pn = c_abs2(pv[i]);
            if (m == 0) {
              gobj[e] = g;
              nobj[e] = pn;
            } else {
              gobj[e] = c_add(gobj[e], g);
              nobj[e] = nobj[e] + pn;
            }
            const float2 bt = c_mul(chi, make_float2(ov[i].x, -ov[i].y));  // chi conj(O_s)
            if (s > 0) {
              buf[idx] = bt;
            } else {
              a.st_probe[((size_t)b * M + m) * N + e] = bt;
              if (m == 0) a.st_nprobe[(size_t)b * N + e] = c_abs2(ov[i]);
            }
          }
        }
        if (s > 0) {
          gsync();
          forward();
          propagate(a.props + (size_t)(s - 1) * N, true);
          gsync();
          inverse();
        }
      }
    }
  } else if constexpr (kKind == 3) {
    // projection sets, single slice and probe: the factor c psi + (1 - c) w of
    // the exit wave w is projected, A exp(i angle F); the new exit wave
    // x w + a psi + b projected is kept and is chi of the adjoint
    const float px_ = 1.0f - a.pa - a.pb;
    const float py_ = 1.0f - a.pc;
    float2* pst = a.st_probe + (size_t)b * N;
    float2* ew = a.exit_waves + (size_t)prow * N;
#pragma unroll 1  // (unrolled, the chunks' live values spill)
    for (int c0 = 0; c0 < PER; c0 += CH) {
      float2 ov[CH];
#pragma unroll
      for (int i = 0; i < CH; ++i) ov[i] = load_object(a, 0, obj_x(ry0 + c0 + i), obj_y(tg));
#pragma unroll
      for (int i = 0; i < CH; ++i) {
        const int x = ry0 + c0 + i;
        const int e = x * S + tg;
        const float2 p = c_scale(buf[x * LD + tg], invN);
        pst[e] = p;
        const float2 psi = c_mul(p, ov[i]);
        const float2 w = a.ew_valid ? ew[e] : psi;
        buf[x * LD + tg] = c_add(c_scale(psi, a.pc), c_scale(w, py_));
      }
    }
    gsync();
    forward();
#pragma unroll 1  // (unrolled, the chunks' live values spill)
    for (int c0 = 0; c0 < PER; c0 += CH) {
      float av[CH];
#pragma unroll
      for (int i = 0; i < CH; ++i) av[i] = __ldg(amp + (fx0 + FXS * (c0 + i)) * S + fy);
#pragma unroll
      for (int i = 0; i < CH; ++i) {
        const int x = fx0 + FXS * (c0 + i);
        const int e = x * S + fy;
        const int idx = x * LD + fy;
        float2 f = buf[idx];
        if (a.det_mask) f = c_scale(f, a.det_mask[e]);
        const float af = c_abs(f);
        const float A = av[i];
        const float d = A - af;
        err += d * d;
        const float q = af > 0.0f ? A / af : 0.0f;
        buf[idx] = af > 0.0f ? c_scale(f, q) : make_float2(A, 0.0f);
      }
    }
    gsync();
    inverse();
    float2* gobj = a.st_obj + (size_t)b * N;
    float* nobj = a.st_nobj + (size_t)b * N;
#pragma unroll 1  // (unrolled, the chunks' live values spill)
    for (int c0 = 0; c0 < PER; c0 += CH) {
      float2 ov[CH], pv[CH];
#pragma unroll
      for (int i = 0; i < CH; ++i) {
        const int x = ry0 + c0 + i;
        ov[i] = load_object(a, 0, obj_x(x), obj_y(tg));
        pv[i] = pst[x * S + tg];
      }
#pragma unroll
      for (int i = 0; i < CH; ++i) {
        const int x = ry0 + c0 + i;
        const int e = x * S + tg;
        const float2 proj = c_scale(buf[x * LD + tg], invN);
        const float2 psi = c_mul(pv[i], ov[i]);
        const float2 w = a.ew_valid ? ew[e] : psi;
        const float2 chi =
            c_add(c_add(c_scale(w, px_), c_scale(psi, a.pa)), c_scale(proj, a.pb));
        ew[e] = chi;
        gobj[e] = object_term(a.potential, ov[i], pv[i], chi);
        nobj[e] = c_abs2(pv[i]);
        pst[e] = c_conj_mul(ov[i], chi);
        a.st_nprobe[(size_t)b * N + e] = c_abs2(ov[i]);
      }
    }
  } else {
    // mixed state: the far fields F_m of every mode share the ratio
    // A / sqrt(sum_m |F_m|^2) (0 where the model is 0); F_m wait in scratch_f
    const int M = a.M;
    float* itot = reinterpret_cast<float*>(rpy + S);  // N, indexed by Fourier pixel
    for (int m = 0; m < M; ++m) {
      if (m > 0) shifted_probe(m);
      float2* pst = a.st_probe + ((size_t)b * M + m) * N;
#pragma unroll 1  // (unrolled, the chunks' live values spill)
      for (int c0 = 0; c0 < PER; c0 += CH) {
        float2 ov[CH];
#pragma unroll
        for (int i = 0; i < CH; ++i) ov[i] = load_object(a, 0, obj_x(ry0 + c0 + i), obj_y(tg));
#pragma unroll
        for (int i = 0; i < CH; ++i) {
          const int x = ry0 + c0 + i;
          const float2 p = c_scale(buf[x * LD + tg], invN);
          pst[x * S + tg] = p;
          buf[x * LD + tg] = c_mul(p, ov[i]);
        }
      }
      gsync();
      forward();
      float2* f = a.scratch_f + ((size_t)b * M + m) * N;
      for (int i = 0; i < PER; ++i) {
        const int x = fx0 + FXS * i;
        const int e = x * S + fy;
        const float2 v = buf[x * LD + fy];
        f[e] = v;
        const float av = hypotf(v.x, v.y);  // |F_m|^2 as numpy forms it
        itot[e] = (m == 0 ? 0.0f : itot[e]) + av * av;
      }
    }
#pragma unroll 1  // (unrolled, the chunks' live values spill)
    for (int c0 = 0; c0 < PER; c0 += CH) {
      float av[CH];
#pragma unroll
      for (int i = 0; i < CH; ++i) av[i] = __ldg(amp + (fx0 + FXS * (c0 + i)) * S + fy);
#pragma unroll
      for (int i = 0; i < CH; ++i) {
        const int e = (fx0 + FXS * (c0 + i)) * S + fy;
        const float mk = a.det_mask ? a.det_mask[e] : 1.0f;
        float tot = sqrtf(itot[e]);
        if (a.det_mask) tot = sqrtf(itot[e] * mk * mk);
        const float A = av[i];
        const float d = A - tot;
        err += d * d;
        itot[e] = tot == 0.0f ? 0.0f : A / tot;
      }
    }
    float2* gobj = a.st_obj + (size_t)b * N;
    float* nobj = a.st_nobj + (size_t)b * N;
    for (int m = 0; m < M; ++m) {
      // (the previous mode's adjoint read the wave by rows)
      if (m > 0) __syncthreads();
      const float2* f = a.scratch_f + ((size_t)b * M + m) * N;
      for (int i = 0; i < PER; ++i) {
        const int x = fx0 + FXS * i;
        const int e = x * S + fy;
        const float mk = a.det_mask ? a.det_mask[e] : 1.0f;
        float2 fv = f[e];
        if (a.det_mask) fv = c_scale(fv, mk);
        float2 r = c_sub(c_scale(fv, itot[e]), fv);
        if (a.det_mask) r = c_scale(r, mk);
        buf[x * LD + fy] = r;
      }
      gsync();
      inverse();
      float2* pst = a.st_probe + ((size_t)b * M + m) * N;
#pragma unroll 1  // (unrolled, the chunks' live values spill)
      for (int c0 = 0; c0 < PER; c0 += CH) {
        float2 ov[CH], pv[CH];
#pragma unroll
        for (int i = 0; i < CH; ++i) {
          const int x = ry0 + c0 + i;
          ov[i] = load_object(a, 0, obj_x(x), obj_y(tg));
          pv[i] = pst[x * S + tg];
        }
#pragma unroll
        for (int i = 0; i < CH; ++i) {
          const int x = ry0 + c0 + i;
          const int e = x * S + tg;
          const float2 chi = c_scale(buf[x * LD + tg], invN);
          const float2 g = object_term(a.potential, ov[i], pv[i], chi);
          const float pn = c_abs2(pv[i]);
          if (m == 0) {
            gobj[e] = g;
            nobj[e] = pn;
            a.st_nprobe[(size_t)b * N + e] = c_abs2(ov[i]);
          } else {
            gobj[e] = c_add(gobj[e], g);
            nobj[e] = nobj[e] + pn;
          }
          pst[e] = c_conj_mul(ov[i], chi);
        }
      }
    }
  }
  const float tot = block_sum<NT>(err, red);
  if (tid == 0) a.err[b] = pos_ok ? tot : __int_as_float(0x7fc00000);
}

// kKind: gradient descent 0 single slice, 1 multislice, 2 mixed state (single
// slice), 4 mixed-state multislice, 5 single slice keeping the far fields for
// the position correction; 3 projection sets (single slice and probe)
template <int NT, int kKind>
__global__ void __launch_bounds__(NT, 1) position_grouped_kernel(BatchArgs a) {
  __shared__ float red[NT / 32];
  position_grouped_128<NT, kKind>(a, blockIdx.x, red);
}


// Position correction of one batch (ptychographic_methods.py:2071-2225), run
// after the batch's object update. One block per position:
//   F0_m = FFT2(P_m O_old)        kept by the forward pass in scratch_f
//   Fx_m = FFT2(P_m O_new[x+1,y]),  Fy_m = FFT2(P_m O_new[x,y+1])
//   gx = sum_m 2 Re((F0_m - Fx_m) conj(F0_m)),  gy likewise
//   d  = A^2 - |F0|^2             (|F0|^2 = sum_m |F0_m|^2 for mixed state)
//   (ux, uy) = step * inv([gx gy]^T [gx gy]) [gx gy]^T d
// then the per-update and total-distance limits, and positions -= u.
// P_m is recomputed from the batch's probe spectrum exactly as the forward pass
// formed it. gx and gy go to the |P|^2 / |O|^2 staging rows, which the batch's
// reductions have consumed by now. The 2x2 normal equations are summed in
// double (per-thread float partials, then a fixed-order block sum).
template <int NT>
__device__ __forceinline__ void block_sum5(double (&v)[5], double (*red)[NT / 32]) {
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    double x = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) red[k][threadIdx.x >> 5] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      double t = 0.0;
      for (int w = 0; w < NT / 32; ++w) t += red[k][w];
      v[k] = t;
    }
  }
}

// The position update from the summed normal equations s5 = (xx, xy, yy, xd,
// yd): the 2 x 2 solve, both distance limits, positions -= u (thread 0).
__device__ __forceinline__ void correction_update(const BatchArgs& a, int prow, float posx,
                                                  float posy, bool pos_ok, const double* s5) {
  const double det = s5[0] * s5[2] - s5[1] * s5[1];
  float ux = 0.0f, uy = 0.0f;
  if (det != 0.0 && isfinite(det)) {  // the reference's inverse fails on a singular system
    ux = __fmul_rn((float)((s5[2] * s5[3] - s5[1] * s5[4]) / det), a.pc_step);
    uy = __fmul_rn((float)((s5[0] * s5[4] - s5[1] * s5[3]) / det), a.pc_step);
  }
  if (a.pc_max_update >= 0.0) {
    const float n = sqrtf(__fadd_rn(__fmul_rn(ux, ux), __fmul_rn(uy, uy)));
    if ((double)n > a.pc_max_update) {
      const double r = (double)n / a.pc_max_update;
      ux = (float)((double)ux / r);
      uy = (float)((double)uy / r);
    }
  }
  if (a.pc_max_total >= 0.0) {
    const float ddx = __fsub_rn(__fsub_rn(posx, a.positions_initial[2 * prow]), ux);
    const float ddy = __fsub_rn(__fsub_rn(posy, a.positions_initial[2 * prow + 1]), uy);
    const float dist = sqrtf(__fadd_rn(__fmul_rn(ddx, ddx), __fmul_rn(ddy, ddy)));
    if ((double)dist > a.pc_max_total) ux = uy = 0.0f;
  }
  if (pos_ok) {  // a non-finite position stays as it is (its error is already NaN)
    a.positions_rw[2 * prow] = __fsub_rn(posx, ux);
    a.positions_rw[2 * prow + 1] = __fsub_rn(posy, uy);
  }
}

template <int SX, int SY, int NT>
__global__ void __launch_bounds__(NT, 1) position_correction_kernel(BatchArgs a) {
  using L = Layout<SX, SY>;
  constexpr int N = L::N;
  constexpr int LD = L::LD;
  extern __shared__ float4 smem4[];
  float2* buf = reinterpret_cast<float2*>(smem4);
  float2* twx = buf + SX * LD;
  float2* twy = twx + SX;
  float2* rpx = twy + SY;
  float2* rpy = rpx + SX;
  __shared__ double red[5][NT / 32];

  const int b = blockIdx.x;
  const int tid = threadIdx.x;
  const int M = a.M;
  const int prow = a.pos_rows ? a.pos_rows[b] : b;
  const int arow = a.amp_rows ? a.amp_rows[b] : b;
  const bool pos_ok = isfinite(a.positions_rw[2 * prow]) && isfinite(a.positions_rw[2 * prow + 1]);
  const float posx = finite_or_zero(a.positions_rw[2 * prow]);
  const float posy = finite_or_zero(a.positions_rw[2 * prow + 1]);
  const float rx = rintf(posx);
  const float ry = rintf(posy);
  const float dx = posx - rx;
  const float dy = posy - ry;
  const int x0 = (int)rx;
  const int y0 = (int)ry;
  const float invN = 1.0f / (float)N;

  for (int i = tid; i < SX; i += NT) twx[i] = a.tw[i];
  for (int i = tid; i < SY; i += NT) twy[i] = a.tw[SX + i];
  for (int i = tid; i < SX; i += NT) {
    const float k = (float)fint(i, SX) / (float)SX;
    rpx[i] = cis_rounded(__fmul_rn(__fmul_rn(-6.2831855f, k), dx));
  }
  for (int i = tid; i < SY; i += NT) {
    const float k = (float)fint(i, SY) / (float)SY;
    rpy[i] = cis_rounded(__fmul_rn(__fmul_rn(-6.2831855f, k), dy));
  }
  __syncthreads();

  const int bx = pmod(x0 - SX / 2, a.Px);
  const int by = pmod(y0 - SY / 2, a.Py);
  auto obj_x = [&](int x) {
    const int t = bx + (x + SX / 2) % SX;
    return t >= a.Px ? t - a.Px : t;
  };
  auto obj_y = [&](int y) {
    const int t = by + (y + SY / 2) % SY;
    return t >= a.Py ? t - a.Py : t;
  };

  float* gx = a.st_nobj + (size_t)b * N;
  float* gy = a.st_nprobe + (size_t)b * N;
  const float2* f0 = a.scratch_f + (size_t)b * M * N;
  const int T = a.T;
  // object pixel of ROI sample (x, y) with the patch moved one pixel along dir
  auto moved = [&](int dir, int x, int y, int& ox, int& oy) {
    ox = obj_x(x);
    oy = obj_y(y);
    if (dir == 0) ox = ox + 1 == a.Px ? 0 : ox + 1;
    else oy = oy + 1 == a.Py ? 0 : oy + 1;
  };
  for (int m = 0; m < M; ++m) {
    const float2* __restrict__ spec = a.probe_spec + (size_t)m * N;
    for (int dir = 0; dir < 2; ++dir) {
      if (T == 1) {
        // P_m shifted as in the forward pass, times the moved object patch
        for (int e = tid; e < N; e += NT) {
          const int x = e / SY, y = e % SY;
          buf[x * LD + y] = c_mul(spec[e], c_mul(rpx[x], rpy[y]));
        }
        __syncthreads();
        fft2d<SX, SY, NT, +1>(buf, twx, twy);
        for (int e = tid; e < N; e += NT) {
          const int x = e / SY, y = e % SY;
          int ox, oy;
          moved(dir, x, y, ox, oy);
          const float2 p = c_scale(buf[x * LD + y], invN);
          buf[x * LD + y] = c_mul(p, load_object(a, 0, ox, oy));
        }
        __syncthreads();
      } else {
        // multislice: the updated, unshifted probe through all moved slices
        for (int s = 0; s < T; ++s) {
          for (int e = tid; e < N; e += NT) {
            const int x = e / SY, y = e % SY;
            int ox, oy;
            moved(dir, x, y, ox, oy);
            const float2 p = s == 0 ? a.probe[(size_t)m * N + e] : c_scale(buf[x * LD + y], invN);
            buf[x * LD + y] = c_mul(load_object(a, s, ox, oy), p);
          }
          __syncthreads();
          if (s + 1 < T) {
            fft2d<SX, SY, NT, -1>(buf, twx, twy);
            const float2* h = a.props + (size_t)s * N;
            for (int e = tid; e < N; e += NT) {
              const int idx = (e / SY) * LD + e % SY;
              buf[idx] = c_mul(buf[idx], h[e]);
            }
            __syncthreads();
            fft2d<SX, SY, NT, +1>(buf, twx, twy);
          }
        }
      }
      fft2d<SX, SY, NT, -1>(buf, twx, twy);
      float* g = dir == 0 ? gx : gy;
      for (int e = tid; e < N; e += NT) {
        const float2 f = buf[(e / SY) * LD + e % SY];
        const float2 r = f0[(size_t)m * N + e];
        const float2 d = c_sub(r, f);
        const float v = 2.0f * __fadd_rn(__fmul_rn(d.x, r.x), __fmul_rn(d.y, r.y));
        g[e] = m == 0 ? v : g[e] + v;
      }
      __syncthreads();  // buf is rewritten by the next pass
    }
  }

  const float* amp = a.amplitudes + (size_t)arow * N;
  const bool mixed = M > 1 || a.mixed_formula;
  float sxx = 0.f, sxy = 0.f, syy = 0.f, sxd = 0.f, syd = 0.f;
  for (int e = tid; e < N; e += NT) {
    float est;
    if (mixed) {
      float t = 0.0f;
      for (int m = 0; m < M; ++m) {
        const float2 r = f0[(size_t)m * N + e];
        const float av = hypotf(r.x, r.y);
        t += av * av;
      }
      const float amp_tot = sqrtf(t);
      est = amp_tot * amp_tot;
    } else {
      const float2 r = f0[e];
      const float af = hypotf(r.x, r.y);
      est = af * af;
    }
    const float A = amp[e];
    const float d = __fsub_rn(__fmul_rn(A, A), est);
    const float px = gx[e], py = gy[e];
    sxx = fmaf(px, px, sxx);
    sxy = fmaf(px, py, sxy);
    syy = fmaf(py, py, syy);
    sxd = fmaf(px, d, sxd);
    syd = fmaf(py, d, syd);
  }
  double s5[5] = {sxx, sxy, syy, sxd, syd};
  block_sum5<NT>(s5, red);
  if (tid == 0) correction_update(a, prow, posx, posy, pos_ok, s5);
}

// Position correction of a single-slice batch at 128 x 128 with the passes and
// walks of position_grouped_kernel: per mode and direction the shifted probe
// (Fourier space by columns, inverse transform), times the moved object patch
// (real space by rows), forward transform, and the gradient term against the
// kept far field (Fourier space by columns); the normal-equation sums walk the
// same columns. Same expressions as position_correction_kernel.
template <int NT>
__global__ void __launch_bounds__(NT, 1) position_correction_grouped_kernel(BatchArgs a) {
  constexpr int S = 128;
  using L = Layout<S, S>;
  constexpr int N = L::N;
  constexpr int LD = L::LD;
  constexpr int GT = 128;
  constexpr int G = NT / GT;
  constexpr int LINES = S / G;
  constexpr int PER = LINES * S / GT;
  constexpr int CH = 8;
  constexpr int FXS = GT / LINES;
  static_assert(NT == 1024 && LINES == 16 && PER == 16, "grouped 128 x 128 layout");
  extern __shared__ float4 smem4[];
  float2* buf = reinterpret_cast<float2*>(smem4);
  float2* twx = buf + S * LD;
  float2* twy = twx + S;
  float2* rpx = twy + S;
  float2* rpy = rpx + S;
  __shared__ double red[5][NT / 32];

  const int b = blockIdx.x;
  const int tid = threadIdx.x;
  const int g = tid / GT;
  const int tg = tid % GT;
  const GroupSync gsync{1 + g, GT};
  const int M = a.M;
  const int prow = a.pos_rows ? a.pos_rows[b] : b;
  const int arow = a.amp_rows ? a.amp_rows[b] : b;
  const bool pos_ok = isfinite(a.positions_rw[2 * prow]) && isfinite(a.positions_rw[2 * prow + 1]);
  const float posx = finite_or_zero(a.positions_rw[2 * prow]);
  const float posy = finite_or_zero(a.positions_rw[2 * prow + 1]);
  const float rx = rintf(posx);
  const float ry = rintf(posy);
  const float dx = posx - rx;
  const float dy = posy - ry;
  const int x0 = (int)rx;
  const int y0 = (int)ry;
  const float invN = 1.0f / (float)N;

  for (int i = tid; i < S; i += NT) {
    twx[i] = a.tw[i];
    twy[i] = a.tw[S + i];
    const float k = (float)fint(i, S) / (float)S;
    rpx[i] = cis_rounded(__fmul_rn(__fmul_rn(-6.2831855f, k), dx));
  }
  for (int i = tid - S; i >= 0 && i < S; i += NT) {
    const float k = (float)fint(i, S) / (float)S;
    rpy[i] = cis_rounded(__fmul_rn(__fmul_rn(-6.2831855f, k), dy));
  }
  __syncthreads();

  const int bx = pmod(x0 - S / 2, a.Px);
  const int by = pmod(y0 - S / 2, a.Py);
  const int ry0 = LINES * g;
  const int fx0 = tg / LINES;
  const int fy = LINES * g + tg % LINES;
  float2* const rows_g = buf + ry0 * LD;
  float2* const cols_g = buf + LINES * g;
  auto forward = [&]() {
    Schedule<S>::template run<LINES, GT, -1>(rows_g, LD, 1, twy, tg, gsync);
    __syncthreads();
    Schedule<S>::template run<LINES, GT, -1>(cols_g, 1, LD, twx, tg, gsync);
  };
  auto inverse = [&]() {
    Schedule<S>::template run<LINES, GT, +1>(cols_g, 1, LD, twx, tg, gsync);
    __syncthreads();
    Schedule<S>::template run<LINES, GT, +1>(rows_g, LD, 1, twy, tg, gsync);
  };
  // object column of this thread's real-space samples, and the object row of
  // sample i, with the patch moved one pixel along x (dir 0) or y (dir 1)
  auto obj_col = [&](int dir) {
    int t2 = by + (tg + S / 2) % S;
    if (t2 >= a.Py) t2 -= a.Py;
    if (dir == 1) t2 = t2 + 1 == a.Py ? 0 : t2 + 1;
    return t2;
  };
  auto obj_row = [&](int dir, int x) {
    int t2 = bx + (x + S / 2) % S;
    if (t2 >= a.Px) t2 -= a.Px;
    if (dir == 0) t2 = t2 + 1 == a.Px ? 0 : t2 + 1;
    return t2;
  };

  float* gx = a.st_nobj + (size_t)b * N;
  float* gy = a.st_nprobe + (size_t)b * N;
  const float2* f0 = a.scratch_f + (size_t)b * M * N;
  for (int m = 0; m < M; ++m) {
    const float2* __restrict__ spec = a.probe_spec + (size_t)m * N;
    for (int dir = 0; dir < 2; ++dir) {
      // P_m shifted as in the forward pass
#pragma unroll 1
      for (int c0 = 0; c0 < PER; c0 += CH) {
        float2 sv[CH];
#pragma unroll
        for (int i = 0; i < CH; ++i) sv[i] = __ldg(spec + (fx0 + FXS * (c0 + i)) * S + fy);
#pragma unroll
        for (int i = 0; i < CH; ++i) {
          const int x = fx0 + FXS * (c0 + i);
          buf[x * LD + fy] = c_mul(sv[i], c_mul(rpx[x], rpy[fy]));
        }
      }
      gsync();
      inverse();
      // times the moved object patch
      const int oy = obj_col(dir);
#pragma unroll 1
      for (int c0 = 0; c0 < PER; c0 += CH) {
        float2 ov[CH];
#pragma unroll
        for (int i = 0; i < CH; ++i) ov[i] = load_object(a, 0, obj_row(dir, ry0 + c0 + i), oy);
#pragma unroll
        for (int i = 0; i < CH; ++i) {
          const int idx = (ry0 + c0 + i) * LD + tg;
          const float2 p = c_scale(buf[idx], invN);
          buf[idx] = c_mul(p, ov[i]);
        }
      }
      gsync();
      forward();
      float* gd = dir == 0 ? gx : gy;
      for (int i = 0; i < PER; ++i) {
        const int x = fx0 + FXS * i;
        const int e = x * S + fy;
        const float2 f = buf[x * LD + fy];
        const float2 r = f0[(size_t)m * N + e];
        const float2 d = c_sub(r, f);
        const float v = 2.0f * __fadd_rn(__fmul_rn(d.x, r.x), __fmul_rn(d.y, r.y));
        gd[e] = m == 0 ? v : gd[e] + v;
      }
    }
  }

  const float* amp = a.amplitudes + (size_t)arow * N;
  const bool mixed = M > 1 || a.mixed_formula;
  float sxx = 0.f, sxy = 0.f, syy = 0.f, sxd = 0.f, syd = 0.f;
  for (int i = 0; i < PER; ++i) {
    const int e = (fx0 + FXS * i) * S + fy;
    float est;
    if (mixed) {
      float tt = 0.0f;
      for (int m = 0; m < M; ++m) {
        const float2 r = f0[(size_t)m * N + e];
        const float av = hypotf(r.x, r.y);
        tt += av * av;
      }
      const float amp_tot = sqrtf(tt);
      est = amp_tot * amp_tot;
    } else {
      const float2 r = f0[e];
      const float af = hypotf(r.x, r.y);
      est = af * af;
    }
    const float A = amp[e];
    const float d = __fsub_rn(__fmul_rn(A, A), est);
    const float px = gx[e], py = gy[e];
    sxx = fmaf(px, px, sxx);
    sxy = fmaf(px, py, sxy);
    syy = fmaf(py, py, syy);
    sxd = fmaf(px, d, sxd);
    syd = fmaf(py, d, syd);
  }
  double s5[5] = {sxx, sxy, syy, sxd, syd};
  block_sum5<NT>(s5, red);
  if (tid == 0) correction_update(a, prow, posx, posy, pos_ok, s5);
}

template <int SX, int SY, int NT>
cudaError_t launch_correction_t(const BatchArgs& a, cudaStream_t s) {
  const size_t smem = Layout<SX, SY>::smem_bytes(false);
  if constexpr (SX == 128 && SY == 128 && NT == 1024) {
    const int schedule = get_schedule(128);
    if (a.T == 1 && (schedule == 0 || schedule == 3)) {
      const void* fn = reinterpret_cast<const void*>(position_correction_grouped_kernel<NT>);
      const cudaError_t e0 = ensure_smem_limit(fn, (int)smem);
      if (e0 != cudaSuccess) return e0;
      position_correction_grouped_kernel<NT><<<a.B, NT, smem, s>>>(a);
      return cudaGetLastError();
    }
  }
  {
    const cudaError_t e0 =
        ensure_smem_limit(reinterpret_cast<const void*>(position_correction_kernel<SX, SY, NT>),
                          (int)smem);
    if (e0 != cudaSuccess) return e0;
  }
  position_correction_kernel<SX, SY, NT><<<a.B, NT, smem, s>>>(a);
  return cudaGetLastError();
}

// probe_grad[m] <- IFFT2(probe_grad[m]) for every mode (one block per mode):
// the last step of the exact probe gradient, applied to the batch sum.
template <int SX, int SY, int NT>
__global__ void __launch_bounds__(NT, 1) probe_inverse_kernel(BatchArgs a) {
  using L = Layout<SX, SY>;
  extern __shared__ float4 smem4[];
  float2* buf = reinterpret_cast<float2*>(smem4);
  float2* twx = buf + SX * L::LD;
  float2* twy = twx + SX;
  fill_twiddles<SX, NT>(twx);
  fill_twiddles<SY, NT>(twy);
  float2* g = a.probe_grad + (size_t)blockIdx.x * L::N;
  for (int e = threadIdx.x; e < L::N; e += NT) buf[(e / SY) * L::LD + e % SY] = g[e];
  __syncthreads();
  fft2d<SX, SY, NT, +1>(buf, twx, twy);
  const float invN = 1.0f / (float)L::N;
  for (int e = threadIdx.x; e < L::N; e += NT) g[e] = c_scale(buf[(e / SY) * L::LD + e % SY], invN);
}

// |P_b|^2 of the sub-pixel shifted probe (mode 0) of batch position b, staged like
// the position kernel's |P|^2 term; summed over positions it is the probe-overlap
// map the preprocessing thresholds into the field-of-view mask
// (singleslice_ptychography.py:504-526: ifft2(fft2(P) ramp), abs() squared).
template <int SX, int SY, int NT>
__global__ void __launch_bounds__(NT, 1) probe_intensity_kernel(BatchArgs a) {
  using L = Layout<SX, SY>;
  constexpr int N = L::N;
  constexpr int LD = L::LD;
  extern __shared__ float4 smem4[];
  float2* buf = reinterpret_cast<float2*>(smem4);
  float2* twx = buf + SX * LD;
  float2* twy = twx + SX;
  float2* rpx = twy + SY;
  float2* rpy = rpx + SX;
  const int tid = threadIdx.x;
  const int b = blockIdx.x;
  const float posx = finite_or_zero(a.positions[2 * b]);
  const float posy = finite_or_zero(a.positions[2 * b + 1]);
  const float rx = rintf(posx);
  const float ry = rintf(posy);
  const float dx = posx - rx;
  const float dy = posy - ry;
  for (int i = tid; i < SX; i += NT) twx[i] = a.tw[i];
  for (int i = tid; i < SY; i += NT) twy[i] = a.tw[SX + i];
  for (int i = tid; i < SX; i += NT) {
    const float k = (float)fint(i, SX) / (float)SX;
    rpx[i] = cis_rounded(__fmul_rn(__fmul_rn(-6.2831855f, k), dx));
  }
  for (int i = tid; i < SY; i += NT) {
    const float k = (float)fint(i, SY) / (float)SY;
    rpy[i] = cis_rounded(__fmul_rn(__fmul_rn(-6.2831855f, k), dy));
  }
  if (tid == 0) a.pos_round[b] = make_int2((int)rx, (int)ry);
  __syncthreads();
  for (int e = tid; e < N; e += NT) {
    const int x = e / SY, y = e % SY;
    buf[x * LD + y] = c_mul(__ldg(a.probe_spec + e), c_mul(rpx[x], rpy[y]));
  }
  __syncthreads();
  fft2d<SX, SY, NT, +1>(buf, twx, twy);
  const float invN = 1.0f / (float)N;
  float* dst = a.st_nobj + (size_t)b * N;
  for (int e = tid; e < N; e += NT) {
    const float2 p = c_scale(buf[(e / SY) * LD + e % SY], invN);
    const float av = hypotf(p.x, p.y);
    dst[e] = av * av;
  }
}

template <int SX, int SY, int NT>
cudaError_t launch_probe_intensity_t(const BatchArgs& a, cudaStream_t s) {
  const size_t smem = Layout<SX, SY>::smem_bytes(false);
  {
    const cudaError_t e0 =
        ensure_smem_limit(reinterpret_cast<const void*>(probe_intensity_kernel<SX, SY, NT>),
                          (int)smem);
    if (e0 != cudaSuccess) return e0;
  }
  probe_intensity_kernel<SX, SY, NT><<<a.B, NT, smem, s>>>(a);
  return cudaGetLastError();
}

// Power of a block's values: sum over the block in a fixed order (thread
// partials, then warp order), broadcast to every thread.
template <int NT>
__device__ __forceinline__ float block_sum_all_f(float v, float* red) {
  const float t = block_sum<NT>(v, red);
  __syncthreads();
  if (threadIdx.x == 0) red[0] = t;
  __syncthreads();
  const float r = red[0];
  __syncthreads();
  return r;
}

// Probe aperture constraint on probe mode 0 (ptychographic_constraints.py:1004-1040,
// mode 0 only for mixed states :1243-1247): P <- IFFT2(exp(i angle FFT2(P)) A),
// rescaled to the power sum |P|^2 it had before.
template <int SX, int SY, int NT>
__global__ void __launch_bounds__(NT, 1) probe_aperture_kernel(BatchArgs a) {
  using L = Layout<SX, SY>;
  constexpr int N = L::N;
  constexpr int LD = L::LD;
  extern __shared__ float4 smem4[];
  float2* buf = reinterpret_cast<float2*>(smem4);
  float2* twx = buf + SX * LD;
  float2* twy = twx + SX;
  __shared__ float red[NT / 32];
  fill_twiddles<SX, NT>(twx);
  fill_twiddles<SY, NT>(twy);
  float part = 0.0f;
  for (int e = threadIdx.x; e < N; e += NT) {
    const float2 p = a.probe[e];
    const float av = hypotf(p.x, p.y);
    part += av * av;
    buf[(e / SY) * LD + e % SY] = p;
  }
  const float s0 = block_sum_all_f<NT>(part, red);
  fft2d<SX, SY, NT, -1>(buf, twx, twy);
  for (int e = threadIdx.x; e < N; e += NT) {
    const int idx = (e / SY) * LD + e % SY;
    const float2 f = buf[idx];
    float sn, cs;
    sincosf(atan2f(f.y, f.x), &sn, &cs);
    const float ap = a.aperture[e];
    buf[idx] = make_float2(cs * ap, sn * ap);
  }
  __syncthreads();
  fft2d<SX, SY, NT, +1>(buf, twx, twy);
  const float invN = 1.0f / (float)N;
  part = 0.0f;
  for (int e = threadIdx.x; e < N; e += NT) {
    const float2 u = c_scale(buf[(e / SY) * LD + e % SY], invN);
    const float av = hypotf(u.x, u.y);
    part += av * av;
  }
  const float s1 = block_sum_all_f<NT>(part, red);
  const float k = sqrtf(s0 / s1);
  for (int e = threadIdx.x; e < N; e += NT)
    a.probe[e] = c_scale(c_scale(buf[(e / SY) * LD + e % SY], invN), k);
}

template <int SX, int SY, int NT>
cudaError_t launch_probe_aperture_t(const BatchArgs& a, cudaStream_t s) {
  const size_t smem = Layout<SX, SY>::smem_bytes(false);
  {
    const cudaError_t e0 =
        ensure_smem_limit(reinterpret_cast<const void*>(probe_aperture_kernel<SX, SY, NT>),
                          (int)smem);
    if (e0 != cudaSuccess) return e0;
  }
  probe_aperture_kernel<SX, SY, NT><<<1, NT, smem, s>>>(a);
  return cudaGetLastError();
}

template <int SX, int SY, int NT>
cudaError_t launch_probe_inverse_t(const BatchArgs& a, cudaStream_t s) {
  const size_t smem = Layout<SX, SY>::smem_bytes(false);
  {
    const cudaError_t e0 =
        ensure_smem_limit(reinterpret_cast<const void*>(probe_inverse_kernel<SX, SY, NT>),
                          (int)smem);
    if (e0 != cudaSuccess) return e0;
  }
  probe_inverse_kernel<SX, SY, NT><<<a.M, NT, smem, s>>>(a);
  return cudaGetLastError();
}


template <int SX, int SY, int NT>
cudaError_t launch_position_t(const BatchArgs& a, cudaStream_t s) {
  const bool mixed_ms = a.T > 1 && a.M > 1;
  const bool mixed = (a.T == 1 && (a.M > 1 || a.mixed_formula)) || mixed_ms;
  const size_t smem = Layout<SX, SY>::smem_bytes(mixed);
  {
    const int bytes = (int)Layout<SX, SY>::smem_bytes(true);
    const void* modes[5] = {reinterpret_cast<const void*>(position_kernel<SX, SY, NT, 0>),
                            reinterpret_cast<const void*>(position_kernel<SX, SY, NT, 1>),
                            reinterpret_cast<const void*>(position_kernel<SX, SY, NT, 2>),
                            reinterpret_cast<const void*>(position_kernel<SX, SY, NT, 3>),
                            reinterpret_cast<const void*>(position_kernel<SX, SY, NT, 4>)};
    for (const void* fn : modes) {
      const cudaError_t e0 = ensure_smem_limit(fn, bytes);
      if (e0 != cudaSuccess) return e0;
    }
  }
  // plain gradient-descent batches run an instantiation with the other modes
  // compiled out (see position_one); mixed-state multislice has its own
  const bool plain = !a.projection && !a.forward_only && !a.keep_farfield && !a.exact_probe_grad;
  const int mode = mixed_ms ? 4
                   : !plain ? 0
                   : a.T == 1 ? (a.M == 1 && !a.mixed_formula ? 1 : 2)
                   : 3;
  if constexpr (SX == 128 && SY == 128 && NT == 1024) {
    // the default (0) and schedule 3: passes by groups of warps
    const int schedule = get_schedule(128);
    // projection sets of one slice and probe without kept far fields
    const bool ps1 = mode == 0 && a.projection && a.T == 1 && a.M == 1 && !a.mixed_formula &&
                     !a.forward_only && !a.keep_farfield && !a.exact_probe_grad;
    // mixed-state multislice gradient descent (its far fields are kept anyway)
    const bool mms_gd = mode == 4 && !a.projection && !a.forward_only && !a.exact_probe_grad;
    // single-slice single-probe gradient descent keeping its far fields
    const bool keep1 = mode == 0 && !a.projection && a.keep_farfield && a.T == 1 && a.M == 1 &&
                       !a.mixed_formula && !a.forward_only && !a.exact_probe_grad;
    if ((mode == 1 || mode == 2 || mode == 3 || ps1 || mms_gd || keep1) &&
        (schedule == 0 || schedule == 3)) {
      const void* fn =
          mode == 1   ? reinterpret_cast<const void*>(position_grouped_kernel<NT, 0>)
          : mode == 3 ? reinterpret_cast<const void*>(position_grouped_kernel<NT, 1>)
          : mode == 2 ? reinterpret_cast<const void*>(position_grouped_kernel<NT, 2>)
          : mms_gd    ? reinterpret_cast<const void*>(position_grouped_kernel<NT, 4>)
          : keep1     ? reinterpret_cast<const void*>(position_grouped_kernel<NT, 5>)
                      : reinterpret_cast<const void*>(position_grouped_kernel<NT, 3>);
      const cudaError_t e0 = ensure_smem_limit(fn, (int)smem);
      if (e0 != cudaSuccess) return e0;
      timing_before(s);
      if (mode == 1)
        position_grouped_kernel<NT, 0><<<a.B, NT, smem, s>>>(a);
      else if (mode == 3)
        position_grouped_kernel<NT, 1><<<a.B, NT, smem, s>>>(a);
      else if (mode == 2)
        position_grouped_kernel<NT, 2><<<a.B, NT, smem, s>>>(a);
      else if (mms_gd)
        position_grouped_kernel<NT, 4><<<a.B, NT, smem, s>>>(a);
      else if (keep1)
        position_grouped_kernel<NT, 5><<<a.B, NT, smem, s>>>(a);
      else
        position_grouped_kernel<NT, 3><<<a.B, NT, smem, s>>>(a);
      const cudaError_t e1 = cudaGetLastError();
      timing_after(s);
      return e1;
    }
  }
  timing_before(s);
  switch (mode) {
    case 1: position_kernel<SX, SY, NT, 1><<<a.B, NT, smem, s>>>(a); break;
    case 2: position_kernel<SX, SY, NT, 2><<<a.B, NT, smem, s>>>(a); break;
    case 3: position_kernel<SX, SY, NT, 3><<<a.B, NT, smem, s>>>(a); break;
    case 4: position_kernel<SX, SY, NT, 4><<<a.B, NT, smem, s>>>(a); break;
    default: position_kernel<SX, SY, NT, 0><<<a.B, NT, smem, s>>>(a); break;
  }
  cudaError_t e = cudaGetLastError();
  timing_after(s);
  return e;
}

}  // namespace
}  // namespace pty

// Externally visible launchers of the kernels for one region of interest
// SX x SY with NT threads per block, named launch_<kernel>_<NAME> (one
// translation unit per size).
#define PTY_POSITION_INSTANCES_XY(SX, SY, NAME, NT)                                      \
  namespace pty {                                                                        \
  cudaError_t launch_position_kernel_##NAME(const BatchArgs& a, cudaStream_t s) {        \
    return launch_position_t<SX, SY, NT>(a, s);                                          \
  }                                                                                      \
  cudaError_t launch_position_correction_##NAME(const BatchArgs& a, cudaStream_t s) {    \
    return launch_correction_t<SX, SY, NT>(a, s);                                        \
  }                                                                                      \
  cudaError_t launch_probe_inverse_##NAME(const BatchArgs& a, cudaStream_t s) {          \
    return launch_probe_inverse_t<SX, SY, NT>(a, s);                                     \
  }                                                                                      \
  cudaError_t launch_probe_intensity_##NAME(const BatchArgs& a, cudaStream_t s) {        \
    return launch_probe_intensity_t<SX, SY, NT>(a, s);                                   \
  }                                                                                      \
  cudaError_t launch_probe_aperture_##NAME(const BatchArgs& a, cudaStream_t s) {         \
    return launch_probe_aperture_t<SX, SY, NT>(a, s);                                    \
  }                                                                                      \
  }

// Square regions of interest S x S.
#define PTY_POSITION_INSTANCES(S, NT) PTY_POSITION_INSTANCES_XY(S, S, S, NT)
