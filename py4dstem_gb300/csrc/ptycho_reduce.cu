// Deterministic reductions of the per-position adjoint terms and the object /
// probe updates, plus the per-iteration constraints.
//
// Object side (replaces _sum_overlapping_patches_bincounts, phase_base_class.py:1905-1968,
// and the update lines of _gradient_descent_adjoint / _projection_sets_adjoint):
//   object_reduce_kernel   one block per 16x16 object tile and slice. It lists, in
//                          batch order, the positions whose patch touches the
//                          tile; each warp sums every eighth list entry (a warp
//                          load reads two whole staged tile rows), and the warp
//                          partials are added in warp order (fixed, so the result
//                          is deterministic); then the tile maximum of the
//                          normaliser sums. Every staged value is read once.
//   object_update_kernel   N_O = 1/sqrt(1e-16 + ((1-m) S)^2 + (m max S)^2);
//                          O += step G N_O (GD) or O = G N_O (projection sets).
// Probe side: a chunked fixed-order sum over the batch, then the same
// normaliser with max over the probe pixels.
// The two sides read disjoint staging buffers and write disjoint state, so the
// probe side runs on a helper stream concurrently with the object side (fork and
// join through events on the caller's stream).
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <utility>

#include "fft_smem.cuh"
#include "ptycho_internal.h"

namespace pty {
namespace {

constexpr int NT = kReduceThreads;

__device__ __forceinline__ int pmod(int v, int m) {
  int r = v % m;
  return r < 0 ? r + m : r;
}

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Block max; result valid in every thread.
__device__ __forceinline__ float block_max(float v, float* red) {
  v = warp_max(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    float t = threadIdx.x < NT / 32 ? red[threadIdx.x] : -INFINITY;
    t = warp_max(t);
    if (threadIdx.x == 0) red[0] = t;
  }
  __syncthreads();
  const float r = red[0];
  __syncthreads();
  return r;
}

// Block sum in a fixed order; result valid in every thread.
template <typename F>
__device__ __forceinline__ F block_sum_all(F v, F* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    F t = 0;
    for (int w = 0; w < NT / 32; ++w) t += red[w];
    red[0] = t;
  }
  __syncthreads();
  const F r = red[0];
  __syncthreads();
  return r;
}

__device__ __forceinline__ float normaliser(float s, float smax, float m) {
  const float a = __fmul_rn(1.0f - m, s);
  const float c = __fmul_rn(m, smax);
  return 1.0f / sqrtf(__fadd_rn(__fadd_rn(1e-16f, __fmul_rn(a, a)), __fmul_rn(c, c)));
}

// A NaN or infinite object or probe value after an update makes the batch's
// error sum NaN, so the per-iteration error read-back (ptycho_read_error)
// reports PTYCHO_ERR_NONFINITE. Finite values leave the sum untouched.
__device__ __forceinline__ void mark_nonfinite(const BatchArgs& a, float2 v) {
  if (!(isfinite(v.x) && isfinite(v.y))) atomicAdd(a.error_accum, __int_as_float(0x7fc00000));
}

// ------------------------------------------------------------------ object side
constexpr int kListChunk = 2048;
constexpr int kRowsPerLane = 8;  // tile rows one lane visits per list entry (every other row)

// One block (8 warps) per 16x16 object tile and slice. The block lists, in batch
// order, the positions whose patch touches the tile (with the tile origin in
// patch coordinates); warp w sums list entries w, w + 8, w + 16, ... For an
// entry, lane l covers tile column l % 16 of rows l / 16, l / 16 + 2, ..., so
// each warp load reads two whole 16-sample staged rows (two 128-byte lines of
// the object term, two 64-byte ones of |P|^2) and the column arithmetic is paid
// once per entry. The eight warp partials are then added in warp order for
// each pixel (a fixed order: the result is deterministic), written as the
// object gradient and normaliser sums, and the tile maximum of the normaliser
// is taken. Every staged value is read once.
__global__ void __launch_bounds__(NT, 4) object_reduce_kernel(BatchArgs a) {
  __shared__ int list[kListChunk];
  __shared__ int list_d[kListChunk];  // (dx << 16) | dy: tile origin in patch coordinates
  __shared__ int warp_count[NT / 32];
  __shared__ int warp_base[NT / 32 + 1];
  __shared__ float part[NT / 32][3][NT];  // per-warp partials (g.x, g.y, n) per tile pixel
  __shared__ float red[NT / 32];
  static_assert(kTile * kTile == NT && kTile == 2 * kRowsPerLane, "tile layout");
  const int s = blockIdx.y;
  const int ntx = (a.Px + kTile - 1) / kTile;
  const int nty = (a.Py + kTile - 1) / kTile;
  // tile rows from the middle outwards (16, 15, 17, 14, ...): the scan sits in
  // the middle of the object, so the tiles with the longest lists start first
  // and the short ones at the edges fill the end of the launch
  const int k = blockIdx.x / nty;
  const int mid = ntx / 2;
  const int trow = (k & 1) ? mid - ((k + 1) >> 1) : mid + (k >> 1);
  const int tile = trow * nty + blockIdx.x % nty;
  const int tx0 = trow * kTile;
  const int ty0 = (tile % nty) * kTile;
  const int tw = min(kTile, a.Px - tx0);
  const int th = min(kTile, a.Py - ty0);
  const int N = a.Sx * a.Sy;
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;

  // staging axes: u is the slow one (rows), v the contiguous one
  const bool tr = a.staging_t != 0;
  const int Pu = tr ? a.Py : a.Px, Pv = tr ? a.Px : a.Py;
  const int Su = tr ? a.Sy : a.Sx, Sv = tr ? a.Sx : a.Sy;
  const int tu = tr ? th : tw, tv = tr ? tw : th;
  const int hu = Su / 2, hv = Sv / 2;  // fftfreq origin: patch sample k sits at (k + S/2) mod S
  const int iv = lane & (kTile - 1);   // this lane's tile column (v)
  const int iu0 = lane >> 4;           // and first row (u); rows iu0, iu0 + 2, ...

  float gx[kRowsPerLane], gy[kRowsPerLane], gn[kRowsPerLane];
#pragma unroll
  for (int k = 0; k < kRowsPerLane; ++k) gx[k] = gy[k] = gn[k] = 0.f;
  const float2* __restrict__ st = a.st_obj + (size_t)s * a.B * N;
  const float* __restrict__ sn = a.st_nobj + (size_t)s * a.B * N;
  const int fminx = -(a.Sx / 2), fminy = -(a.Sy / 2);

  for (int c0 = 0; c0 < a.B; c0 += kListChunk) {
    const int cn = min(kListChunk, a.B - c0);
    int count = 0;
    // ordered compaction of the positions whose patch touches this tile
    for (int base = 0; base < cn; base += NT) {
      const int i = base + tid;
      bool hit = false;
      int dx = 0, dy = 0;
      if (i < cn) {
        const int2 r = a.pos_round[c0 + i];
        dx = pmod(tx0 - (r.x + fminx), a.Px);
        dy = pmod(ty0 - (r.y + fminy), a.Py);
        hit = (dx < a.Sx || dx + tw - 1 >= a.Px) && (dy < a.Sy || dy + th - 1 >= a.Py);
      }
      const unsigned bal = __ballot_sync(0xffffffffu, hit);
      if (lane == 0) warp_count[warp] = __popc(bal);
      __syncthreads();
      if (tid == 0) {
        warp_base[0] = count;
        for (int w = 0; w < NT / 32; ++w) warp_base[w + 1] = warp_base[w] + warp_count[w];
      }
      __syncthreads();
      if (hit) {
        const int slot = warp_base[warp] + __popc(bal & ((1u << lane) - 1u));
        list[slot] = c0 + i;
        list_d[slot] = (dx << 16) | dy;
      }
      count = warp_base[NT / 32];
      __syncthreads();
    }
    for (int l = warp; l < count; l += NT / 32) {
      const int b = list[l];
      const int d = list_d[l];
      const int du = tr ? (d & 0xffff) : (d >> 16);
      const int dv = tr ? (d >> 16) : (d & 0xffff);
      // this lane's column: patch coordinate sv (one object wrap at most)
      int sv = dv + iv;
      if (sv >= Pv) sv -= Pv;
      const bool vok = iv < tv && sv < Sv;
      const int lv = sv >= hv ? sv - hv : sv + hv;
      const size_t col = (size_t)b * N + lv;
      float2 v[kRowsPerLane];
      float w[kRowsPerLane];
#pragma unroll
      for (int k = 0; k < kRowsPerLane; ++k) {
        const int iu = iu0 + 2 * k;
        int su = du + iu;
        if (su >= Pu) su -= Pu;
        v[k] = make_float2(0.f, 0.f);
        w[k] = 0.f;
        if (vok && iu < tu && su < Su) {
          const int lu = su >= hu ? su - hu : su + hu;
          const size_t e = col + (size_t)lu * Sv;
          if (!a.nobj_only) v[k] = st[e];
          w[k] = sn[e];
        }
      }
#pragma unroll
      for (int k = 0; k < kRowsPerLane; ++k) {
        gx[k] += v[k].x;
        gy[k] += v[k].y;
        gn[k] += w[k];
      }
    }
    __syncthreads();  // the list is rewritten by the next chunk
  }

  // warp partials in warp order, per tile pixel (u-major index iu * 16 + iv)
#pragma unroll
  for (int k = 0; k < kRowsPerLane; ++k) {
    const int t = (iu0 + 2 * k) * kTile + iv;
    part[warp][0][t] = gx[k];
    part[warp][1][t] = gy[k];
    part[warp][2][t] = gn[k];
  }
  __syncthreads();
  float2 g = make_float2(part[0][0][tid], part[0][1][tid]);
  float n = part[0][2][tid];
#pragma unroll
  for (int w = 1; w < NT / 32; ++w) {
    g.x += part[w][0][tid];
    g.y += part[w][1][tid];
    n += part[w][2][tid];
  }
  const int pu = tid / kTile, pv = tid % kTile;
  const int px = tx0 + (tr ? pv : pu);
  const int py = ty0 + (tr ? pu : pv);
  float m = 0.0f;
  if (px < a.Px && py < a.Py) {
    const size_t o = ((size_t)s * a.Px + px) * a.Py + py;
    if (!a.nobj_only) a.obj_grad[o] = g;
    a.obj_nrm[o] = n;
    m = n;
  }
  m = block_max(m, red);
  if (tid == 0) a.tile_max[s * gridDim.x + tile] = m;
}

__global__ void __launch_bounds__(NT) object_update_kernel(BatchArgs a, int ntiles) {
  __shared__ float red[NT / 32];
  const int s = blockIdx.y;
  float m = 0.0f;
  for (int i = threadIdx.x; i < ntiles; i += NT) m = fmaxf(m, a.tile_max[s * ntiles + i]);
  const float smax = block_max(m, red);

  // batch error, summed in batch order by one block
  if (blockIdx.x == 0 && s == 0) {
    float e = 0.0f;
    const int per = (a.B + NT - 1) / NT;
    const int lo = threadIdx.x * per;
    const int hi = min(a.B, lo + per);
    for (int i = lo; i < hi; ++i) e += a.err[i];
    const float tot = block_sum_all(e, red);
    // atomic only so that a concurrent non-finite mark (below, or from the
    // probe side) cannot be overwritten; one add per batch keeps the order
    if (threadIdx.x == 0) atomicAdd(a.error_accum, tot);
  }

  const size_t P = (size_t)a.Px * a.Py;
  const size_t i = (size_t)blockIdx.x * NT + threadIdx.x;
  if (i >= P) return;
  const size_t o = (size_t)s * P + i;
  const float nrm = normaliser(a.obj_nrm[o], smax, a.norm_min);
  const float2 g = a.obj_grad[o];
  const bool mixed_order = a.M > 1 || a.mixed_formula;
  float2 r;
  if (a.potential) {
    float* obj = reinterpret_cast<float*>(a.object);
    if (a.projection) {
      r.x = __fmul_rn(g.x, nrm);
    } else if (mixed_order) {
      r.x = __fadd_rn(obj[o], __fmul_rn(__fmul_rn(a.step, g.x), nrm));
    } else {
      r.x = __fadd_rn(obj[o], __fmul_rn(a.step, __fmul_rn(g.x, nrm)));
    }
    r.y = 0.0f;
    obj[o] = r.x;
  } else {
    float2* obj = reinterpret_cast<float2*>(a.object);
    float2 u;
    if (a.projection) {
      u = make_float2(__fmul_rn(g.x, nrm), __fmul_rn(g.y, nrm));
      r = u;
    } else {
      if (mixed_order) {
        u = make_float2(__fmul_rn(__fmul_rn(a.step, g.x), nrm), __fmul_rn(__fmul_rn(a.step, g.y), nrm));
      } else {
        u = make_float2(__fmul_rn(a.step, __fmul_rn(g.x, nrm)), __fmul_rn(a.step, __fmul_rn(g.y, nrm)));
      }
      const float2 v = obj[o];
      r = make_float2(__fadd_rn(v.x, u.x), __fadd_rn(v.y, u.y));
    }
    obj[o] = r;
  }
  mark_nonfinite(a, r);
}

// overlap += the batch's |P|^2 sums (the object reduction's normaliser sums): the
// probe-overlap map of the preprocessing, one batch at a time
// (singleslice_ptychography.py:504-526).
__global__ void __launch_bounds__(NT) overlap_accumulate_kernel(BatchArgs a, float* overlap) {
  const size_t P = (size_t)a.Px * a.Py;
  const size_t i = (size_t)blockIdx.x * NT + threadIdx.x;
  if (i >= P) return;
  overlap[i] = overlap[i] + a.obj_nrm[i];
}

// ------------------------------------------------------------------- probe side
constexpr int kProbeChunkMax = 1024;  // positions per chunk whose patch origins are staged

__global__ void __launch_bounds__(NT) probe_reduce_kernel(BatchArgs a) {
  __shared__ int2 origin[kProbeChunkMax];  // patch origins (pmod'ed) of this chunk's positions
  const int N = a.Sx * a.Sy;
  const int e = blockIdx.x * NT + threadIdx.x;
  const int c = blockIdx.y;
  const int per = (a.B + kProbeChunks - 1) / kProbeChunks;
  const int lo = c * per;
  const int hi = min(a.B, lo + per);
  const bool staged_origins = a.nprobe_from_object && hi - lo <= kProbeChunkMax;
  if (staged_origins) {
    // the integer modulo of each position's patch origin once per block, not
    // once per pixel and position
    for (int i = threadIdx.x; i < hi - lo; i += NT) {
      const int2 r = a.pos_round[lo + i];
      origin[i] = make_int2(pmod(r.x - a.Sx / 2, a.Px), pmod(r.y - a.Sy / 2, a.Py));
    }
    __syncthreads();
  }
  if (e >= N) return;
  const float2* __restrict__ sp = a.st_probe;
  const float* __restrict__ snp = a.st_nprobe;
  for (int m = 0; m < a.M; ++m) {
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll 8
    for (int b = lo; b < hi; ++b) {
      const float2 v = sp[((size_t)b * a.M + m) * N + e];
      acc.x += v.x;
      acc.y += v.y;
    }
    a.probe_part[((size_t)c * a.M + m) * N + e] = acc;
  }
  float n = 0.f;
  if (a.nprobe_from_object) {
    // |O|^2 of each position's patch at this probe pixel, gathered from the
    // object (the plain GD position kernel stages none)
    const int x = e / a.Sy, y = e % a.Sy;
    const int xo = (x + a.Sx / 2) % a.Sx, yo = (y + a.Sy / 2) % a.Sy;
#pragma unroll 4
    for (int b = lo; b < hi; ++b) {
      int2 base;
      if (staged_origins) {
        base = origin[b - lo];
      } else {
        const int2 r = a.pos_round[b];
        base = make_int2(pmod(r.x - a.Sx / 2, a.Px), pmod(r.y - a.Sy / 2, a.Py));
      }
      int ox = base.x + xo;
      int oy = base.y + yo;
      if (ox >= a.Px) ox -= a.Px;
      if (oy >= a.Py) oy -= a.Py;
      const size_t idx = (size_t)ox * a.Py + oy;
      float2 o;
      if (a.potential) {
        float sv, cv;
        sincosf(reinterpret_cast<const float*>(a.object)[idx], &sv, &cv);
        o = make_float2(cv, sv);
      } else {
        o = reinterpret_cast<const float2*>(a.object)[idx];
      }
      n += o.x * o.x + o.y * o.y;
    }
  } else {
#pragma unroll 8
    for (int b = lo; b < hi; ++b) n += snp[(size_t)b * N + e];
  }
  a.probe_npart[(size_t)c * N + e] = n;
}

__global__ void __launch_bounds__(NT) probe_finalize_kernel(BatchArgs a) {
  __shared__ float red[NT / 32];
  const int N = a.Sx * a.Sy;
  const int e = blockIdx.x * NT + threadIdx.x;
  float mx = 0.f;
  if (e < N) {
    for (int m = 0; m < a.M; ++m) {
      float2 acc = make_float2(0.f, 0.f);
      for (int c = 0; c < kProbeChunks; ++c) {
        const float2 v = a.probe_part[((size_t)c * a.M + m) * N + e];
        acc.x += v.x;
        acc.y += v.y;
      }
      a.probe_grad[(size_t)m * N + e] = acc;
    }
    float n = 0.f;
    for (int c = 0; c < kProbeChunks; ++c) n += a.probe_npart[(size_t)c * N + e];
    a.probe_nrm[e] = n;
    mx = n;
  }
  mx = block_max(mx, red);
  if (threadIdx.x == 0) a.probe_bmax[blockIdx.x] = mx;
}

__global__ void __launch_bounds__(NT) probe_update_kernel(BatchArgs a, int nblocks) {
  __shared__ float red[NT / 32];
  const int N = a.Sx * a.Sy;
  float m = 0.f;
  for (int i = threadIdx.x; i < nblocks; i += NT) m = fmaxf(m, a.probe_bmax[i]);
  const float smax = block_max(m, red);
  const int e = blockIdx.x * NT + threadIdx.x;
  if (e >= N) return;
  // sums are in staging order; the probe is natural (x-major)
  const int es = a.staging_t ? (e % a.Sy) * a.Sx + e / a.Sy : e;
  const float nrm = normaliser(a.probe_nrm[es], smax, a.norm_min);
  const bool ms_order = a.T > 1;
  for (int mm = 0; mm < a.M; ++mm) {
    const size_t o = (size_t)mm * N + e;
    const float2 g = a.probe_grad[(size_t)mm * N + es];
    if (a.projection) {
      a.probe[o] = make_float2(__fmul_rn(g.x, nrm), __fmul_rn(g.y, nrm));
    } else {
      float2 u;
      if (ms_order) {
        u = make_float2(__fmul_rn(__fmul_rn(a.step, g.x), nrm), __fmul_rn(__fmul_rn(a.step, g.y), nrm));
      } else {
        u = make_float2(__fmul_rn(a.step, __fmul_rn(g.x, nrm)), __fmul_rn(a.step, __fmul_rn(g.y, nrm)));
      }
      const float2 v = a.probe[o];
      a.probe[o] = make_float2(__fadd_rn(v.x, u.x), __fadd_rn(v.y, u.y));
    }
    mark_nonfinite(a, a.probe[o]);
  }
}

// ------------------------------------------------------------- gradient export
// Loss and gradients of one batch without an update (the autograd backward):
// loss = sum_b err_b in batch order; object and probe gradients are the summed
// adjoint terms times `scale` (-2N: the adjoint terms are -1/(2N) times the
// gradient of the loss with respect to the real and imaginary parts).
__global__ void __launch_bounds__(NT) gradient_export_kernel(BatchArgs a, void* object_grad,
                                                            float2* probe_grad, float* loss,
                                                            float scale) {
  __shared__ float red[NT / 32];
  if (blockIdx.x == 0) {
    float e = 0.0f;
    const int per = (a.B + NT - 1) / NT;
    const int lo = threadIdx.x * per;
    const int hi = min(a.B, lo + per);
    for (int i = lo; i < hi; ++i) e += a.err[i];
    const float tot = block_sum_all(e, red);
    if (threadIdx.x == 0) loss[0] = tot;
  }
  const size_t TP = (size_t)a.T * a.Px * a.Py;
  const size_t MN = (size_t)a.M * a.Sx * a.Sy;
  const size_t stride = (size_t)gridDim.x * NT;
  for (size_t i = (size_t)blockIdx.x * NT + threadIdx.x; i < TP; i += stride) {
    const float2 g = a.obj_grad[i];
    if (a.potential) {
      reinterpret_cast<float*>(object_grad)[i] = scale * g.x;
    } else {
      reinterpret_cast<float2*>(object_grad)[i] = make_float2(scale * g.x, scale * g.y);
    }
  }
  if (probe_grad) {
    for (size_t i = (size_t)blockIdx.x * NT + threadIdx.x; i < MN; i += stride) {
      const float2 g = a.probe_grad[i];
      probe_grad[i] = make_float2(scale * g.x, scale * g.y);
    }
  }
}

// --------------------------------------------------------------- constraints
constexpr int kConstraintBlocks = 256;

__global__ void __launch_bounds__(NT) masked_mean_partial_kernel(BatchArgs a, const uint8_t* mask) {
  __shared__ double redd[NT / 32];
  const size_t P = (size_t)a.Px * a.Py;
  double sum = 0.0;
  double cnt = 0.0;
  for (size_t i = (size_t)blockIdx.x * NT + threadIdx.x; i < P; i += (size_t)gridDim.x * NT) {
    if (!mask[i]) continue;
    for (int s = 0; s < a.T; ++s) {
      const size_t o = (size_t)s * P + i;
      float v;
      if (a.potential) {
        v = reinterpret_cast<const float*>(a.object)[o];
      } else {
        const float2 z = reinterpret_cast<const float2*>(a.object)[o];
        v = atan2f(z.y, z.x);
      }
      sum += (double)v;
      cnt += 1.0;
    }
  }
  const double ts = block_sum_all(sum, redd);
  const double tc = block_sum_all(cnt, redd);
  if (threadIdx.x == 0) {
    reinterpret_cast<double*>(a.red)[2 * blockIdx.x] = ts;
    reinterpret_cast<double*>(a.red)[2 * blockIdx.x + 1] = tc;
  }
}

// The masked mean's block partials added once, by one block in a fixed order
// (thread b holds partial b; then the block's shuffle tree and warp order), into
// red[2 kConstraintBlocks] and [2 kConstraintBlocks + 1].
__global__ void __launch_bounds__(NT) masked_mean_final_kernel(BatchArgs a) {
  static_assert(kConstraintBlocks == NT, "one partial per thread");
  __shared__ double redd[NT / 32];
  const double* part = reinterpret_cast<const double*>(a.red);
  const double s = block_sum_all(part[2 * threadIdx.x], redd);
  const double c = block_sum_all(part[2 * threadIdx.x + 1], redd);
  if (threadIdx.x == 0) {
    reinterpret_cast<double*>(a.red)[2 * kConstraintBlocks] = s;
    reinterpret_cast<double*>(a.red)[2 * kConstraintBlocks + 1] = c;
  }
}

__global__ void __launch_bounds__(NT) object_constraint_kernel(BatchArgs a, int use_mask,
                                                                 float shrinkage,
                                                                 int apply_shrinkage,
                                                                 int pure_phase,
                                                                 int positivity) {
  float shrink = shrinkage;
  if (use_mask) {
    const double* ms = reinterpret_cast<const double*>(a.red) + 2 * kConstraintBlocks;
    shrink = shrink + (float)(ms[0] / ms[1]);
  }
  const size_t P = (size_t)a.Px * a.Py * a.T;
  const size_t i = (size_t)blockIdx.x * NT + threadIdx.x;
  if (i >= P) return;
  if (a.potential) {
    float* obj = reinterpret_cast<float*>(a.object);
    float v = obj[i];
    if (apply_shrinkage) v = v - shrink;
    if (positivity) v = fmaxf(v, 0.0f);
    obj[i] = v;
  } else {
    float2* obj = reinterpret_cast<float2*>(a.object);
    float2 z = obj[i];
    if (apply_shrinkage) {
      const float amp = hypotf(z.x, z.y);
      const float ph = atan2f(z.y, z.x) - shrink;
      float sv, cv;
      sincosf(ph, &sv, &cv);
      z = make_float2(amp * cv, amp * sv);
    }
    const float ph = atan2f(z.y, z.x);
    const float amp = pure_phase ? 1.0f : fminf(hypotf(z.x, z.y), 1.0f);
    float sv, cv;
    sincosf(ph, &sv, &cv);
    obj[i] = make_float2(amp * cv, amp * sv);
  }
}

// Probe CoM of |P_0|^2 with corner-centred (fftfreq) coordinates, in float64:
// kComBlocks blocks each sum a contiguous slice of the pixels (partials in
// a.red), then one thread adds the partials in block order.
constexpr int kComBlocks = 16;

__global__ void __launch_bounds__(NT) probe_com_partial_kernel(BatchArgs a) {
  __shared__ double redd[NT / 32];
  const int N = a.Sx * a.Sy;
  const int per = (N + kComBlocks - 1) / kComBlocks;
  const int lo = blockIdx.x * per, hi = min(N, lo + per);
  double t = 0.0, sx = 0.0, sy = 0.0;
  for (int e = lo + threadIdx.x; e < hi; e += NT) {
    const float2 p = a.probe[e];
    const float h = hypotf(p.x, p.y);
    const float v = h * h;
    const int x = e / a.Sy, y = e % a.Sy;
    const int fx = x < (a.Sx + 1) / 2 ? x : x - a.Sx;
    const int fy = y < (a.Sy + 1) / 2 ? y : y - a.Sy;
    t += (double)v;
    sx += (double)fx * (double)v;
    sy += (double)fy * (double)v;
  }
  const double tt = block_sum_all(t, redd);
  const double tx = block_sum_all(sx, redd);
  const double ty = block_sum_all(sy, redd);
  if (threadIdx.x == 0) {
    double* part = reinterpret_cast<double*>(a.red) + 3 * blockIdx.x;
    part[0] = tt;
    part[1] = tx;
    part[2] = ty;
  }
}

__global__ void probe_com_final_kernel(BatchArgs a) {
  const double* part = reinterpret_cast<const double*>(a.red);
  double tt = 0.0, tx = 0.0, ty = 0.0;
  for (int b = 0; b < kComBlocks; ++b) {
    tt += part[3 * b];
    tx += part[3 * b + 1];
    ty += part[3 * b + 2];
  }
  const double tf = (double)(float)tt;  // total intensity is a float32 sum
  a.com[0] = tx / tf;
  a.com[1] = ty / tf;
}

template <int SX, int SY, int NTF>
__global__ void __launch_bounds__(NTF, 1) probe_shift_kernel(BatchArgs a) {
  constexpr int LD = SY + 1;
  constexpr int N = SX * SY;
  extern __shared__ float4 smem4[];
  float2* buf = reinterpret_cast<float2*>(smem4);
  float2* twx = buf + SX * LD;
  float2* twy = twx + SX;
  float2* rpx = twy + SY;
  float2* rpy = rpx + SX;
  fill_twiddles<SX, NTF>(twx);
  fill_twiddles<SY, NTF>(twy);
  // shift by -CoM: positions cast to float32 as the reference does
  const float dx = (float)(-a.com[0]);
  const float dy = (float)(-a.com[1]);
  for (int i = threadIdx.x; i < SX; i += NTF) {
    const int f = i < (SX + 1) / 2 ? i : i - SX;
    const float k = (float)f / (float)SX;
    rpx[i] = cis_rounded(__fmul_rn(__fmul_rn(-6.2831855f, k), dx));
  }
  for (int i = threadIdx.x; i < SY; i += NTF) {
    const int f = i < (SY + 1) / 2 ? i : i - SY;
    const float k = (float)f / (float)SY;
    rpy[i] = cis_rounded(__fmul_rn(__fmul_rn(-6.2831855f, k), dy));
  }
  float2* p = a.probe + (size_t)blockIdx.x * N;
  for (int e = threadIdx.x; e < N; e += NTF) buf[(e / SY) * LD + e % SY] = p[e];
  __syncthreads();
  fft2d<SX, SY, NTF, -1>(buf, twx, twy);
  for (int e = threadIdx.x; e < N; e += NTF) {
    const int x = e / SY, y = e % SY;
    buf[x * LD + y] = c_mul(buf[x * LD + y], c_mul(rpx[x], rpy[y]));
  }
  __syncthreads();
  fft2d<SX, SY, NTF, +1>(buf, twx, twy);
  const float invN = 1.0f / (float)N;
  for (int e = threadIdx.x; e < N; e += NTF) p[e] = c_scale(buf[(e / SY) * LD + e % SY], invN);
}

template <int SX, int SY, int NTF>
cudaError_t launch_shift_t(const BatchArgs& a, cudaStream_t s) {
  const size_t smem = sizeof(float2) * (size_t)(SX * (SY + 1) + 2 * SX + 2 * SY);
  {
    const cudaError_t e0 =
        ensure_smem_limit(reinterpret_cast<const void*>(probe_shift_kernel<SX, SY, NTF>),
                          (int)smem);
    if (e0 != cudaSuccess) return e0;
  }
  probe_shift_kernel<SX, SY, NTF><<<a.M, NTF, smem, s>>>(a);
  return cudaGetLastError();
}

__global__ void __launch_bounds__(NT) probe_gram_kernel(int M, int N, const float2* probe,
                                                        float2* gram) {
  __shared__ float red[NT / 32];
  const int i = blockIdx.x / M;
  const int j = blockIdx.x % M;
  float re = 0.f, im = 0.f;
  for (int e = threadIdx.x; e < N; e += NT) {
    const float2 v = c_conj_mul(probe[(size_t)i * N + e], probe[(size_t)j * N + e]);
    re += v.x;
    im += v.y;
  }
  re = block_sum_all(re, red);
  im = block_sum_all(im, red);
  if (threadIdx.x == 0) gram[i * M + j] = make_float2(re, im);
}

__global__ void __launch_bounds__(NT) probe_mix_kernel(int M, int N, const float2* in,
                                                       const float2* coeffs, float2* out) {
  const int i = blockIdx.y;
  const int e = blockIdx.x * NT + threadIdx.x;
  if (e >= N) return;
  float2 acc = make_float2(0.f, 0.f);
  for (int j = 0; j < M; ++j) {
    const float2 c = coeffs[i * M + j];
    const float2 v = in[(size_t)j * N + e];
    acc = c_add(acc, c_mul(c, v));
  }
  out[(size_t)i * N + e] = acc;
}

// Eigen-decomposition of the M x M Hermitian Gram matrix on the device (cyclic
// Jacobi in double, one thread; M <= 16), then the mixing coefficients of the
// orthogonalised modes: mode i = sum_j coeffs[i*M+j] P_j with the eigenvectors
// ordered by decreasing eigenvalue (= decreasing mode intensity), each
// eigenvector's phase fixed so that its largest component is real and positive.
// Rotation of pair (p, q): remove the phase of g_pq, then the real Jacobi
// rotation t = sgn(tau)/(|tau| + sqrt(1 + tau^2)), tau = (g_qq - g_pp)/(2|g_pq|).
// At most 32 sweeps; each sweep visits every pair once.
__global__ void probe_eigh_kernel(int M, const float2* gram, float2* coeffs) {
  __shared__ double2 A[16][16];
  __shared__ double2 V[16][16];
  __shared__ double w[16];
  __shared__ int order[16];
  if (threadIdx.x != 0) return;
  for (int i = 0; i < M; ++i)
    for (int j = 0; j < M; ++j) {
      // upper triangle is the reference's input (eigh with UPLO='U')
      const float2 g = i <= j ? gram[i * M + j] : gram[j * M + i];
      A[i][j] = i <= j ? make_double2(g.x, g.y) : make_double2(g.x, -g.y);
      if (i == j) A[i][j].y = 0.0;
      V[i][j] = make_double2(i == j ? 1.0 : 0.0, 0.0);
    }
  for (int sweep = 0; sweep < 32; ++sweep) {
    double off = 0.0, diag = 0.0;
    for (int i = 0; i < M; ++i) {
      diag += A[i][i].x * A[i][i].x;
      for (int j = i + 1; j < M; ++j) off += A[i][j].x * A[i][j].x + A[i][j].y * A[i][j].y;
    }
    if (off <= 1e-30 * diag || off == 0.0) break;
    for (int p = 0; p < M - 1; ++p) {
      for (int q = p + 1; q < M; ++q) {
        const double re = A[p][q].x, im = A[p][q].y;
        const double mag = sqrt(re * re + im * im);
        if (mag == 0.0) continue;
        const double ephr = re / mag, ephi = im / mag;  // e^{i phi}
        const double tau = (A[q][q].x - A[p][p].x) / (2.0 * mag);
        const double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
        const double c = 1.0 / sqrt(1.0 + t * t);
        const double sn = t * c;
        // J = [[c, s], [-s e^{-i phi}, c e^{-i phi}]] on columns (p, q): A <- J^H A J
        for (int k = 0; k < M; ++k) {  // columns
          const double2 akp = A[k][p], akq = A[k][q];
          const double2 aq = make_double2(akq.x * ephr + akq.y * ephi, akq.y * ephr - akq.x * ephi);
          A[k][p] = make_double2(c * akp.x - sn * aq.x, c * akp.y - sn * aq.y);
          A[k][q] = make_double2(sn * akp.x + c * aq.x, sn * akp.y + c * aq.y);
          const double2 vkp = V[k][p], vkq = V[k][q];
          const double2 vq = make_double2(vkq.x * ephr + vkq.y * ephi, vkq.y * ephr - vkq.x * ephi);
          V[k][p] = make_double2(c * vkp.x - sn * vq.x, c * vkp.y - sn * vq.y);
          V[k][q] = make_double2(sn * vkp.x + c * vq.x, sn * vkp.y + c * vq.y);
        }
        for (int k = 0; k < M; ++k) {  // rows: conjugate of the column transform
          const double2 apk = A[p][k], aqk = A[q][k];
          const double2 aq = make_double2(aqk.x * ephr - aqk.y * ephi, aqk.y * ephr + aqk.x * ephi);
          A[p][k] = make_double2(c * apk.x - sn * aq.x, c * apk.y - sn * aq.y);
          A[q][k] = make_double2(sn * apk.x + c * aq.x, sn * apk.y + c * aq.y);
        }
        A[p][q] = make_double2(0.0, 0.0);
        A[q][p] = make_double2(0.0, 0.0);
        A[p][p].y = 0.0;
        A[q][q].y = 0.0;
      }
    }
  }
  for (int i = 0; i < M; ++i) {
    w[i] = A[i][i].x;
    order[i] = i;
  }
  for (int i = 1; i < M; ++i) {  // stable insertion sort, decreasing eigenvalue
    const int o = order[i];
    int k = i - 1;
    while (k >= 0 && w[order[k]] < w[o]) {
      order[k + 1] = order[k];
      --k;
    }
    order[k + 1] = o;
  }
  for (int i = 0; i < M; ++i) {
    const int col = order[i];
    int big = 0;
    double bmag = -1.0;
    for (int j = 0; j < M; ++j) {
      const double mg = V[j][col].x * V[j][col].x + V[j][col].y * V[j][col].y;
      if (mg > bmag) {
        bmag = mg;
        big = j;
      }
    }
    const double bm = sqrt(bmag);
    const double pr = V[big][col].x / bm, pi = -V[big][col].y / bm;  // e^{-i arg}
    for (int j = 0; j < M; ++j) {
      const double2 v = V[j][col];
      coeffs[i * M + j] = make_float2((float)(v.x * pr - v.y * pi), (float)(v.x * pi + v.y * pr));
    }
  }
}

__global__ void __launch_bounds__(256) fma_probe_kernel(int iters, float* sink) {
  float a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = (float)(threadIdx.x + k) * 1e-3f;
  const float m = 0.9999f, c = 1e-4f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fmaf(a[k], m, c);
  }
  float t = 0.f;
#pragma unroll
  for (int k = 0; k < 8; ++k) t += a[k];
  sink[blockIdx.x * 256 + threadIdx.x] = t;
}

}  // namespace

cudaError_t launch_fma_probe(int blocks, int iters, float* sink, cudaStream_t s) {
  fma_probe_kernel<<<blocks, 256, 0, s>>>(iters, sink);
  return cudaGetLastError();
}

namespace {

// Helper stream and fork/join events per (device, caller stream), created on
// the first batch issued on that stream and kept for the life of the process.
struct ForkJoin {
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr;
  cudaEvent_t join = nullptr;
  cudaEvent_t gathered = nullptr;  // the probe side has read the object
};
std::mutex g_fork_mu;
std::map<std::pair<int, cudaStream_t>, ForkJoin> g_fork;

cudaError_t fork_join_for(cudaStream_t s, ForkJoin& out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(g_fork_mu);
  ForkJoin& fj = g_fork[std::make_pair(dev, s)];
  if (!fj.side) {
    int prio = 0;
    if (s != nullptr && (e = cudaStreamGetPriority(s, &prio)) != cudaSuccess) return e;
    ForkJoin n;
    if ((e = cudaStreamCreateWithPriority(&n.side, cudaStreamNonBlocking, prio)) != cudaSuccess)
      return e;
    if ((e = cudaEventCreateWithFlags(&n.fork, cudaEventDisableTiming)) != cudaSuccess) return e;
    if ((e = cudaEventCreateWithFlags(&n.join, cudaEventDisableTiming)) != cudaSuccess) return e;
    if ((e = cudaEventCreateWithFlags(&n.gathered, cudaEventDisableTiming)) != cudaSuccess)
      return e;
    fj = n;
  }
  out = fj;
  return cudaSuccess;
}

}  // namespace

cudaError_t prepare_stream(cudaStream_t s) {
  ForkJoin fj;
  return fork_join_for(s, fj);
}

cudaError_t launch_reduce_and_update(const BatchArgs& a, cudaStream_t s) {
  const int ntx = (a.Px + kTile - 1) / kTile;
  const int nty = (a.Py + kTile - 1) / kTile;
  const int ntiles = ntx * nty;
  ForkJoin fj;
  cudaError_t e;
  if (!a.fix_probe) {
    // probe side on the helper stream, after everything issued so far on s
    if ((e = fork_join_for(s, fj)) != cudaSuccess) return e;
    if ((e = cudaEventRecord(fj.fork, s)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(fj.side, fj.fork, 0)) != cudaSuccess) return e;
    const int N = a.Sx * a.Sy;
    const int nb = (N + NT - 1) / NT;
    probe_reduce_kernel<<<dim3(nb, kProbeChunks), NT, 0, fj.side>>>(a);
    // gathering |O|^2 the probe reduction reads the object, which the object
    // update below rewrites: the update waits for it
    if (a.nprobe_from_object && (e = cudaEventRecord(fj.gathered, fj.side)) != cudaSuccess)
      return e;
    probe_finalize_kernel<<<nb, NT, 0, fj.side>>>(a);
    probe_update_kernel<<<nb, NT, 0, fj.side>>>(a, nb);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // the next batch's spectrum of the updated probe, off the critical path
    if (a.prepare_spectrum && (e = launch_probe_spectrum(a, fj.side)) != cudaSuccess) return e;
    if ((e = cudaEventRecord(fj.join, fj.side)) != cudaSuccess) return e;
  }
  object_reduce_kernel<<<dim3(ntiles, a.T), NT, 0, s>>>(a);
  if (!a.fix_probe && a.nprobe_from_object &&
      (e = cudaStreamWaitEvent(s, fj.gathered, 0)) != cudaSuccess)
    return e;
  const size_t P = (size_t)a.Px * a.Py;
  object_update_kernel<<<dim3((unsigned)((P + NT - 1) / NT), a.T), NT, 0, s>>>(a, ntiles);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (!a.fix_probe && (e = cudaStreamWaitEvent(s, fj.join, 0)) != cudaSuccess) return e;
  return cudaSuccess;
}

// Probe amplitude constraint (ptychographic_constraints.py:920-957, every mode of a
// mixed state :1256-1262): P_m <- P_m mask, rescaled to the power it had before.
// One block per mode; the power sums in float64.
__global__ void __launch_bounds__(NT) probe_amplitude_kernel(BatchArgs a, const float* mask) {
  __shared__ double red[NT / 32];
  const int N = a.Sx * a.Sy;
  float2* p = a.probe + (size_t)blockIdx.x * N;
  double s0 = 0.0, s1 = 0.0;
  for (int e = threadIdx.x; e < N; e += NT) {
    const float2 v = p[e];
    const double m = mask[e];
    s0 += (double)v.x * v.x + (double)v.y * v.y;
    s1 += ((double)v.x * v.x + (double)v.y * v.y) * m * m;
  }
  const double t0 = block_sum_all(s0, red);
  const double t1 = block_sum_all(s1, red);
  const double k = sqrt(t0 / t1);
  for (int e = threadIdx.x; e < N; e += NT) {
    const float2 v = p[e];
    const double f = (double)mask[e] * k;
    p[e] = make_float2((float)(v.x * f), (float)(v.y * f));
  }
}

// Identical-slices constraint (ptychographic_constraints.py:630-647): every slice
// takes the mean over slices (sum in slice order, then / T).
__global__ void __launch_bounds__(NT) identical_slices_kernel(BatchArgs a) {
  const size_t P = (size_t)a.Px * a.Py;
  const size_t i = (size_t)blockIdx.x * NT + threadIdx.x;
  if (i >= P) return;
  const float tf = (float)a.T;
  if (a.potential) {
    float* o = reinterpret_cast<float*>(a.object);
    float m = o[i];
    for (int s = 1; s < a.T; ++s) m = __fadd_rn(m, o[(size_t)s * P + i]);
    m = __fdiv_rn(m, tf);
    for (int s = 0; s < a.T; ++s) o[(size_t)s * P + i] = m;
  } else {
    float2* o = reinterpret_cast<float2*>(a.object);
    float2 m = o[i];
    for (int s = 1; s < a.T; ++s) {
      const float2 v = o[(size_t)s * P + i];
      m = make_float2(__fadd_rn(m.x, v.x), __fadd_rn(m.y, v.y));
    }
    m = make_float2(__fdiv_rn(m.x, tf), __fdiv_rn(m.y, tf));
    for (int s = 0; s < a.T; ++s) o[(size_t)s * P + i] = m;
  }
}

// One axis of the object Gaussian constraint (ptychographic_constraints.py:119-151,
// scipy.ndimage.gaussian_filter with mode "reflect"): out = sum_j w_j in[i + j]
// over j in [-R, R] along `axis` of a (C, n0, n1, n2) float32 array (C = 2 for the
// real and imaginary parts), in float64 as the centre term plus the symmetric
// pairs from the outermost in, rounded once to float32 per pass.
__global__ void __launch_bounds__(NT) gaussian_pass_kernel(const float* in, float* out, int n0,
                                                           int n1, int n2, int axis,
                                                           const double* w, int R, size_t total) {
  const size_t i = (size_t)blockIdx.x * NT + threadIdx.x;
  if (i >= total) return;
  const size_t vol = (size_t)n0 * n1 * n2;
  const size_t c = i / vol;
  size_t r = i - c * vol;
  const int i0 = (int)(r / ((size_t)n1 * n2));
  r -= (size_t)i0 * n1 * n2;
  const int i1 = (int)(r / n2);
  const int i2 = (int)(r - (size_t)i1 * n2);
  const int n = axis == 0 ? n0 : axis == 1 ? n1 : n2;
  const int k = axis == 0 ? i0 : axis == 1 ? i1 : i2;
  const size_t stride = axis == 0 ? (size_t)n1 * n2 : axis == 1 ? (size_t)n2 : 1;
  const size_t base = i - (size_t)k * stride;
  auto at = [&](int j) {  // reflect: d c b a | a b c d | d c b a
    const int period = 2 * n;
    int m = j % period;
    if (m < 0) m += period;
    if (m >= n) m = period - 1 - m;
    return (double)in[base + (size_t)m * stride];
  };
  double acc = __dmul_rn(at(k), w[R]);
  for (int j = R; j >= 1; --j) acc = __dadd_rn(acc, __dmul_rn(__dadd_rn(at(k - j), at(k + j)), w[R - j]));
  out[i] = __double2float_rn(acc);
}

// Phase of a complex object into a float array, and back as exp(i phase).
__global__ void __launch_bounds__(NT) object_phase_kernel(const float2* o, float* ph, size_t n) {
  const size_t i = (size_t)blockIdx.x * NT + threadIdx.x;
  if (i < n) ph[i] = atan2f(o[i].y, o[i].x);
}
__global__ void __launch_bounds__(NT) object_from_phase_kernel(const float* ph, float2* o, size_t n) {
  const size_t i = (size_t)blockIdx.x * NT + threadIdx.x;
  if (i < n) {
    float sn, cs;
    sincosf(ph[i], &sn, &cs);
    o[i] = make_float2(cs, sn);
  }
}
// Interleaved complex <-> planar (real plane, imaginary plane).
__global__ void __launch_bounds__(NT) deinterleave_kernel(const float2* o, float* p, size_t n) {
  const size_t i = (size_t)blockIdx.x * NT + threadIdx.x;
  if (i < n) {
    p[i] = o[i].x;
    p[n + i] = o[i].y;
  }
}
__global__ void __launch_bounds__(NT) interleave_kernel(const float* p, float2* o, size_t n) {
  const size_t i = (size_t)blockIdx.x * NT + threadIdx.x;
  if (i < n) o[i] = make_float2(p[i], p[n + i]);
}

cudaError_t launch_object_gaussian(const BatchArgs& a, const double* w, int R, int pure_phase,
                                   float* scratch, cudaStream_t s) {
  const size_t n = (size_t)a.T * a.Px * a.Py;
  const unsigned gb = (unsigned)((n + NT - 1) / NT);
  // planes: scratch[0 .. 2n) data, scratch[2n .. 4n) ping-pong
  float* x = scratch;
  float* y = scratch + 2 * n;
  int C;
  if (a.potential) {
    cudaError_t e = cudaMemcpyAsync(x, a.object, sizeof(float) * n, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
    C = 1;
  } else if (pure_phase) {
    object_phase_kernel<<<gb, NT, 0, s>>>(static_cast<const float2*>(a.object), x, n);
    C = 1;
  } else {
    deinterleave_kernel<<<gb, NT, 0, s>>>(static_cast<const float2*>(a.object), x, n);
    C = 2;
  }
  // axes of the (T, Px, Py) array in order; a single slice is a 2D array
  const int dims[3] = {a.T, a.Px, a.Py};
  const size_t total = (size_t)C * n;
  const unsigned gt = (unsigned)((total + NT - 1) / NT);
  for (int ax = a.T > 1 ? 0 : 1; ax < 3; ++ax) {
    gaussian_pass_kernel<<<gt, NT, 0, s>>>(x, y, dims[0], dims[1], dims[2], ax, w, R, total);
    float* t = x;
    x = y;
    y = t;
  }
  if (a.potential) {
    cudaError_t e = cudaMemcpyAsync(a.object, x, sizeof(float) * n, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
  } else if (pure_phase) {
    object_from_phase_kernel<<<gb, NT, 0, s>>>(x, static_cast<float2*>(a.object), n);
  } else {
    interleave_kernel<<<gb, NT, 0, s>>>(x, static_cast<float2*>(a.object), n);
  }
  return cudaGetLastError();
}

cudaError_t launch_probe_amplitude(const BatchArgs& a, const float* mask, cudaStream_t s) {
  probe_amplitude_kernel<<<a.M, NT, 0, s>>>(a, mask);
  return cudaGetLastError();
}

cudaError_t launch_identical_slices(const BatchArgs& a, cudaStream_t s) {
  const size_t P = (size_t)a.Px * a.Py;
  identical_slices_kernel<<<(unsigned)((P + NT - 1) / NT), NT, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_overlap_accumulate(const BatchArgs& a, float* overlap, cudaStream_t s) {
  const int ntx = (a.Px + kTile - 1) / kTile;
  const int nty = (a.Py + kTile - 1) / kTile;
  object_reduce_kernel<<<dim3(ntx * nty, 1), NT, 0, s>>>(a);
  const size_t P = (size_t)a.Px * a.Py;
  overlap_accumulate_kernel<<<(unsigned)((P + NT - 1) / NT), NT, 0, s>>>(a, overlap);
  return cudaGetLastError();
}

cudaError_t launch_gradient(const BatchArgs& a, void* object_grad, float2* probe_grad,
                            float* loss, cudaStream_t s) {
  const int ntx = (a.Px + kTile - 1) / kTile;
  const int nty = (a.Py + kTile - 1) / kTile;
  const int ntiles = ntx * nty;
  object_reduce_kernel<<<dim3(ntiles, a.T), NT, 0, s>>>(a);
  if (probe_grad) {
    const int N = a.Sx * a.Sy;
    const int nb = (N + NT - 1) / NT;
    probe_reduce_kernel<<<dim3(nb, kProbeChunks), NT, 0, s>>>(a);
    probe_finalize_kernel<<<nb, NT, 0, s>>>(a);
    if (a.exact_probe_grad) {
      cudaError_t e = launch_probe_inverse(a, s);
      if (e != cudaSuccess) return e;
    }
  }
  const float scale = -2.0f * (float)(a.Sx * a.Sy);
  gradient_export_kernel<<<1024, NT, 0, s>>>(a, object_grad, probe_grad, loss, scale);
  return cudaGetLastError();
}

cudaError_t launch_object_constraints(const BatchArgs& a, const uint8_t* mask, float shrinkage,
                                      int apply_shrinkage, int pure_phase, int positivity,
                                      cudaStream_t s) {
  const int use_mask = (apply_shrinkage && mask != nullptr) ? 1 : 0;
  if (use_mask) {
    masked_mean_partial_kernel<<<kConstraintBlocks, NT, 0, s>>>(a, mask);
    masked_mean_final_kernel<<<1, NT, 0, s>>>(a);
  }
  const size_t P = (size_t)a.Px * a.Py * a.T;
  object_constraint_kernel<<<(unsigned)((P + NT - 1) / NT), NT, 0, s>>>(
      a, use_mask, shrinkage, apply_shrinkage, pure_phase, positivity);
  return cudaGetLastError();
}

cudaError_t launch_probe_com(const BatchArgs& a, cudaStream_t s) {
  probe_com_partial_kernel<<<kComBlocks, NT, 0, s>>>(a);
  probe_com_final_kernel<<<1, 1, 0, s>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  switch (a.Sx * 4096 + a.Sy) {
    case 32 * 4096 + 32: return launch_shift_t<32, 32, 128>(a, s);
    case 48 * 4096 + 48: return launch_shift_t<48, 48, 192>(a, s);
    case 64 * 4096 + 64: return launch_shift_t<64, 64, 256>(a, s);
    case 96 * 4096 + 96: return launch_shift_t<96, 96, 384>(a, s);
    case 128 * 4096 + 128: return launch_shift_t<128, 128, 512>(a, s);
    case 96 * 4096 + 128: return launch_shift_t<96, 128, 512>(a, s);
    case 128 * 4096 + 96: return launch_shift_t<128, 96, 512>(a, s);
    case 256 * 4096 + 256: return launch_staged_probe_shift(a, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_probe_gram(const BatchArgs& a, const float2* probe, float2* gram,
                              cudaStream_t s) {
  probe_gram_kernel<<<a.M * a.M, NT, 0, s>>>(a.M, a.Sx * a.Sy, probe, gram);
  return cudaGetLastError();
}

cudaError_t launch_probe_orthogonalize(const BatchArgs& a, float2* scratch_probe, float2* gram,
                                       float2* coeffs, cudaStream_t s) {
  const int N = a.Sx * a.Sy;
  probe_gram_kernel<<<a.M * a.M, NT, 0, s>>>(a.M, N, a.probe, gram);
  probe_eigh_kernel<<<1, 32, 0, s>>>(a.M, gram, coeffs);
  probe_mix_kernel<<<dim3((N + NT - 1) / NT, a.M), NT, 0, s>>>(a.M, N, a.probe, coeffs,
                                                               scratch_probe);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return cudaMemcpyAsync(a.probe, scratch_probe, sizeof(float2) * a.M * N,
                         cudaMemcpyDeviceToDevice, s);
}

cudaError_t launch_probe_mix(const BatchArgs& a, const float2* in, const float2* coeffs,
                             float2* out, cudaStream_t s) {
  const int N = a.Sx * a.Sy;
  probe_mix_kernel<<<dim3((N + NT - 1) / NT, a.M), NT, 0, s>>>(a.M, N, in, coeffs, out);
  return cudaGetLastError();
}

}  // namespace pty
