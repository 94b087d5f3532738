// One-time preprocessing of the diffraction data on the device: the per-pattern
// centre of mass, the real/reciprocal rotation search and the corner-centring /
// square-root normalisation that py4DSTEM 0.14.18 runs before the reconstruction
// loop (phase_base_class.py:613-767, 1086-1182, 1347-1460).
//
// The reference evaluates these in float32 NumPy. Every sum here reproduces the
// order NumPy's float32 add.reduce uses for a contiguous run of n values
// (numpy/_core/src/umath/loops_utils.h.src, pairwise_sum; the reduction's
// identity 0 is added in front): runs of at most 128 values are summed with 8
// interleaved accumulators, longer runs split in two halves at a multiple of 8.
// Products, quotients and the bilinear weights are formed with the same single
// roundings (no contraction into FMAs), so the results are the reference's bits.
//
// Kernels (one block per pattern, or per angle and transpose):
//   pattern_com_kernel        sum I, sum I kx, sum I ky of the (masked) pattern
//   rotation_search_kernel    mean |curl| (or |div|) of the rotated CoM field
//   pattern_normalize_kernel  periodic bilinear shift by -CoM, pattern sum,
//                             sqrt(max(., 0)) with the optional corner crop
// When every split of the summation tree halves a multiple of 16 (all square
// detectors of 32..128 pixels), the tree is perfect: 2^d leaves of equal length
// l. The fast kernels then give each of a leaf's 8 accumulator chains its own
// lane (8 lanes per leaf, chains combined by shuffles in NumPy's order) and add
// the leaves level by level in parallel. Other sizes take the *_general
// kernels, in which one thread walks the tree.
#include <cuda_runtime.h>

#include <type_traits>

#include "ptycho_internal.h"

namespace pty {
namespace {

constexpr int kPwBlock = 128;  // PW_BLOCKSIZE of NumPy's pairwise sum
constexpr int kPreThreads = 256;

__host__ __device__ __forceinline__ int pw_half(int n) {
  int h = n / 2;
  return h - h % 8;
}

// Single-rounding add / multiply / divide in the accumulation type (float32
// for float32 NumPy arrays, float64 where NumPy promotes to float64).
__device__ __forceinline__ float acc_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double acc_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float acc_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double acc_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float acc_div(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double acc_div(double a, double b) { return __ddiv_rn(a, b); }

// Leaves of the pairwise tree over n values, left to right (one thread).
__device__ int pairwise_leaves(int n, int* lo, int* len) {
  int slo[40], sn[40];
  int sp = 0, k = 0;
  slo[sp] = 0;
  sn[sp] = n;
  ++sp;
  while (sp > 0) {
    --sp;
    const int l = slo[sp], m = sn[sp];
    if (m <= kPwBlock) {
      lo[k] = l;
      len[k] = m;
      ++k;
      continue;
    }
    const int h = pw_half(m);
    slo[sp] = l + h;  // right half, taken after the left one
    sn[sp] = m - h;
    ++sp;
    slo[sp] = l;
    sn[sp] = h;
    ++sp;
  }
  return k;
}

// Sum of one leaf [l, l + m) of values f(i).
template <typename Acc, typename F>
__device__ __forceinline__ Acc leaf_sum(const F& f, int l, int m) {
  if (m < 8) {
    Acc r = 0;
    for (int i = 0; i < m; ++i) r = acc_add(r, (Acc)f(l + i));
    return r;
  }
  Acc r[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) r[j] = f(l + j);
  int i = 8;
  for (; i < m - (m % 8); i += 8) {
#pragma unroll
    for (int j = 0; j < 8; ++j) r[j] = acc_add(r[j], (Acc)f(l + i + j));
  }
  Acc res = acc_add(acc_add(acc_add(r[0], r[1]), acc_add(r[2], r[3])),
                    acc_add(acc_add(r[4], r[5]), acc_add(r[6], r[7])));
  for (; i < m; ++i) res = acc_add(res, (Acc)f(l + i));
  return res;
}

// Combines the leaf sums of the tree over n values in tree order (one thread).
// Post-order walk with an explicit stack: each frame is a node still waiting for
// its right half.
template <typename Acc>
__device__ Acc pairwise_combine(int n, const Acc* leaf) {
  int fn[40];      // size of the node's right half
  Acc fv[40];      // value of its left half
  int sp = 0, k = 0;
  int m = n;
  for (;;) {
    // descend along left halves to a leaf
    while (m > kPwBlock) {
      const int h = pw_half(m);
      fn[sp] = m - h;
      fv[sp] = 0;
      ++sp;
      m = h;
    }
    Acc v = leaf[k++];
    // climb: a finished left half starts its right sibling; a finished right
    // half completes its parent
    for (;;) {
      if (sp == 0) return v;
      if (fn[sp - 1] > 0) {  // v is a left half
        fv[sp - 1] = v;
        m = fn[sp - 1];
        fn[sp - 1] = -1;
        break;
      }
      --sp;  // v is a right half
      v = acc_add(fv[sp], v);
    }
  }
}

__device__ __forceinline__ int pmod(int v, int m) {
  int r = v % m;
  return r < 0 ? r + m : r;
}

// ------------------------------------------------------------ centre of mass
// cx[p] = sum(I kx) / sum(I), cy[p] = sum(I ky) / sum(I) with I = pattern * mask
// (phase_base_class.py:646-688): kx, ky are the pixel indices along x and y.
// Mask modes follow NumPy's promotion of pattern (float32) * mask:
//   0  no mask;
//   1  boolean or float32 mask: float32 products and sums;
//   2  float64 mask, vectorised form: the float64 array, float64 sums;
//   3  float64 mask, per-pattern loop (mi *= mask in place): the float64 product
//      rounded to float32, float32 sums.
template <int kMask>
struct MaskedPixel {
  using Acc = typename std::conditional<kMask == 2, double, float>::type;
  const float* src;
  const void* mask;
  __device__ __forceinline__ Acc operator()(int e) const {
    const float v = __ldg(src + e);
    if constexpr (kMask == 0) {
      return v;
    } else if constexpr (kMask == 1) {
      return __fmul_rn(v, __ldg(static_cast<const float*>(mask) + e));
    } else if constexpr (kMask == 2) {
      return __dmul_rn((double)v, __ldg(static_cast<const double*>(mask) + e));
    } else {
      return __double2float_rn(__dmul_rn((double)v, __ldg(static_cast<const double*>(mask) + e)));
    }
  }
};

template <int kMask>
__global__ void __launch_bounds__(kPreThreads) pattern_com_general_kernel(
    const float* __restrict__ in, int Qx, int Qy, const void* __restrict__ mask,
    int max_leaves, void* cx_out, void* cy_out) {
  using Px = MaskedPixel<kMask>;
  using Acc = typename Px::Acc;
  extern __shared__ float4 smem4[];
  const int N = Qx * Qy;
  Acc* leaf = reinterpret_cast<Acc*>(smem4);                       // 3 * max_leaves
  int* llo = reinterpret_cast<int*>(leaf + 3 * max_leaves);        // max_leaves
  int* llen = llo + max_leaves;                                    // max_leaves
  __shared__ int nleaves;
  const Px px{in + (size_t)blockIdx.x * N, mask};
  if (threadIdx.x == 0) nleaves = pairwise_leaves(N, llo, llen);
  __syncthreads();
  const int L = nleaves;
  for (int t = threadIdx.x; t < 3 * L; t += kPreThreads) {
    const int q = t / L, j = t - q * L;
    Acc s;
    if (q == 0) {
      s = leaf_sum<Acc>(px, llo[j], llen[j]);
    } else if (q == 1) {
      s = leaf_sum<Acc>([&](int e) { return acc_mul(px(e), (Acc)(e / Qy)); }, llo[j], llen[j]);
    } else {
      s = leaf_sum<Acc>([&](int e) { return acc_mul(px(e), (Acc)(e % Qy)); }, llo[j], llen[j]);
    }
    leaf[q * max_leaves + j] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const Acc s0 = acc_add((Acc)0, pairwise_combine<Acc>(N, leaf));
    const Acc s1 = acc_add((Acc)0, pairwise_combine<Acc>(N, leaf + max_leaves));
    const Acc s2 = acc_add((Acc)0, pairwise_combine<Acc>(N, leaf + 2 * max_leaves));
    static_cast<Acc*>(cx_out)[blockIdx.x] = acc_div(s1, s0);
    static_cast<Acc*>(cy_out)[blockIdx.x] = acc_div(s2, s0);
  }
}

// ----------------------------------------------------------- rotation search
// vals[t * A + a] = mean over the interior of |d cy/dx - d cx/dy| (curl) or
// |d cx/dx + d cy/dy| (divergence, `div` != 0) of the CoM field rotated by angle
// a (cos_a, sin_a) and, for t = 1, with x and y exchanged
// (phase_base_class.py:1086-1182; central differences over two pixels).
// T is the type of the CoM field (float64 when the centre of mass was formed in
// float64); the float32 cos / sin of the angles are promoted to it, as NumPy does.
template <typename T>
__global__ void __launch_bounds__(kPreThreads) rotation_search_kernel(
    const T* __restrict__ nx, const T* __restrict__ ny, int R0, int R1,
    const float* __restrict__ cos_a, const float* __restrict__ sin_a, int A, int div,
    int max_leaves, T* __restrict__ vals) {
  extern __shared__ float4 smem4[];
  T* leaf = reinterpret_cast<T*>(smem4);
  int* llo = reinterpret_cast<int*>(leaf + max_leaves);
  int* llen = llo + max_leaves;
  __shared__ int nleaves;
  const int a = blockIdx.x % A;
  const int t = blockIdx.x / A;
  const T c = cos_a[a], s = sin_a[a];
  const int W = R1 - 2;
  const int n = (R0 - 2) * W;
  auto rx = [&](int i, int j) {
    const T X = nx[i * R1 + j], Y = ny[i * R1 + j];
    return t ? acc_add(acc_mul(c, Y), -acc_mul(s, X)) : acc_add(acc_mul(c, X), -acc_mul(s, Y));
  };
  auto ry = [&](int i, int j) {
    const T X = nx[i * R1 + j], Y = ny[i * R1 + j];
    return t ? acc_add(acc_mul(s, Y), acc_mul(c, X)) : acc_add(acc_mul(s, X), acc_mul(c, Y));
  };
  auto value = [&](int e) {
    const int i = e / W, j = e - (e / W) * W;
    if (div) {
      const T gxx = acc_add(rx(i + 2, j + 1), -rx(i, j + 1));
      const T gyy = acc_add(ry(i + 1, j + 2), -ry(i + 1, j));
      return abs(acc_add(gxx, gyy));
    }
    const T gxy = acc_add(rx(i + 1, j + 2), -rx(i + 1, j));
    const T gyx = acc_add(ry(i + 2, j + 1), -ry(i, j + 1));
    return abs(acc_add(gyx, -gxy));
  };
  if (threadIdx.x == 0) nleaves = pairwise_leaves(n, llo, llen);
  __syncthreads();
  for (int j = threadIdx.x; j < nleaves; j += kPreThreads) leaf[j] = leaf_sum<T>(value, llo[j], llen[j]);
  __syncthreads();
  if (threadIdx.x == 0) {
    const T sum = acc_add((T)0, pairwise_combine<T>(n, leaf));
    vals[blockIdx.x] = acc_div(sum, (T)n);
  }
}

// ------------------------------------------------------------- normalisation
// Output pattern o takes source pattern rows[o] (all patterns in order when
// rows is null), shifts it periodically and bilinearly by (-cfx, -cfy)
// (preprocess/utils.py:59-120 bilinear branch: four rolled copies weighted
// (1-wx)(1-wy), wx(1-wy), (1-wx)wy, wx wy, added in that order), stores its sum
// in sums[o] and sqrt(max(shifted, 0)) in amps, cropped to the four crop_w x
// crop_w corners when crop_w > 0 (phase_base_class.py:1385-1445).
__global__ void __launch_bounds__(kPreThreads) pattern_normalize_general_kernel(
    const float* __restrict__ in, int Qx, int Qy, const int32_t* __restrict__ rows,
    const float* __restrict__ cfx, const float* __restrict__ cfy, int crop_w, int max_leaves,
    float* __restrict__ amps, float* __restrict__ sums) {
  extern __shared__ float4 smem4[];
  const int N = Qx * Qy;
  float* pat = reinterpret_cast<float*>(smem4);
  float* sh = pat + N;
  float* leaf = sh + N;
  int* llo = reinterpret_cast<int*>(leaf + max_leaves);
  int* llen = llo + max_leaves;
  __shared__ int nleaves;
  const int o = blockIdx.x;
  const int r = rows ? rows[o] : o;
  const float* src = in + (size_t)r * N;
  for (int e = threadIdx.x; e < N; e += kPreThreads) pat[e] = src[e];
  if (threadIdx.x == 0) nleaves = pairwise_leaves(N, llo, llen);

  const float xs = -cfx[r], ys = -cfy[r];
  const float xf = floorf(xs), yf = floorf(ys);
  const float wx = __fsub_rn(xs, xf), wy = __fsub_rn(ys, yf);
  const float ux = __fsub_rn(1.0f, wx), uy = __fsub_rn(1.0f, wy);
  const float w00 = __fmul_rn(ux, uy), w10 = __fmul_rn(wx, uy);
  const float w01 = __fmul_rn(ux, wy), w11 = __fmul_rn(wx, wy);
  const int ix = (int)xf, iy = (int)yf;
  __syncthreads();
  for (int e = threadIdx.x; e < N; e += kPreThreads) {
    const int i = e / Qy, j = e - (e / Qy) * Qy;
    const int i0 = pmod(i - ix, Qx), i1 = pmod(i - ix - 1, Qx);
    const int j0 = pmod(j - iy, Qy), j1 = pmod(j - iy - 1, Qy);
    float v = __fmul_rn(pat[i0 * Qy + j0], w00);
    v = __fadd_rn(v, __fmul_rn(pat[i1 * Qy + j0], w10));
    v = __fadd_rn(v, __fmul_rn(pat[i0 * Qy + j1], w01));
    v = __fadd_rn(v, __fmul_rn(pat[i1 * Qy + j1], w11));
    sh[e] = v;
  }
  __syncthreads();
  for (int j = threadIdx.x; j < nleaves; j += kPreThreads)
    leaf[j] = leaf_sum<float>([&](int e) { return sh[e]; }, llo[j], llen[j]);
  // amplitudes (numpy.maximum keeps its first argument unless it is below the second)
  const int Cx = crop_w > 0 ? 2 * crop_w : Qx;
  const int Cy = crop_w > 0 ? 2 * crop_w : Qy;
  float* dst = amps + (size_t)o * Cx * Cy;
  for (int e = threadIdx.x; e < Cx * Cy; e += kPreThreads) {
    const int u = e / Cy, w = e - (e / Cy) * Cy;
    const int x = crop_w > 0 && u >= crop_w ? Qx - Cx + u : u;
    const int y = crop_w > 0 && w >= crop_w ? Qy - Cy + w : w;
    float v = sh[x * Qy + y];
    if (!(v >= 0.0f) && !isnan(v)) v = 0.0f;
    dst[e] = __fsqrt_rn(v);
  }
  __syncthreads();
  if (threadIdx.x == 0) sums[o] = __fadd_rn(0.0f, pairwise_combine<float>(N, leaf));
}


// Normalisation of patterns too large to stage in shared memory (256 x 256):
// the same values as pattern_normalize_general_kernel, each shifted value
// formed from the pattern in global memory where it is used (leaf sums, one
// thread per leaf; then the amplitudes of the kept pixels).
__global__ void __launch_bounds__(kPreThreads) pattern_normalize_global_kernel(
    const float* __restrict__ in, int Qx, int Qy, const int32_t* __restrict__ rows,
    const float* __restrict__ cfx, const float* __restrict__ cfy, int crop_w, int max_leaves,
    float* __restrict__ amps, float* __restrict__ sums) {
  extern __shared__ float4 smem4[];
  const int N = Qx * Qy;
  float* leaf = reinterpret_cast<float*>(smem4);
  int* llo = reinterpret_cast<int*>(leaf + max_leaves);
  int* llen = llo + max_leaves;
  __shared__ int nleaves;
  const int o = blockIdx.x;
  const int r = rows ? rows[o] : o;
  const float* src = in + (size_t)r * N;
  if (threadIdx.x == 0) nleaves = pairwise_leaves(N, llo, llen);
  const float xs = -cfx[r], ys = -cfy[r];
  const float xf = floorf(xs), yf = floorf(ys);
  const float wx = __fsub_rn(xs, xf), wy = __fsub_rn(ys, yf);
  const float ux = __fsub_rn(1.0f, wx), uy = __fsub_rn(1.0f, wy);
  const float w00 = __fmul_rn(ux, uy), w10 = __fmul_rn(wx, uy);
  const float w01 = __fmul_rn(ux, wy), w11 = __fmul_rn(wx, wy);
  const int ix = (int)xf, iy = (int)yf;
  auto shifted = [&](int e) {
    const int i = e / Qy, j = e - (e / Qy) * Qy;
    const int i0 = pmod(i - ix, Qx), i1 = pmod(i - ix - 1, Qx);
    const int j0 = pmod(j - iy, Qy), j1 = pmod(j - iy - 1, Qy);
    float v = __fmul_rn(__ldg(src + i0 * Qy + j0), w00);
    v = __fadd_rn(v, __fmul_rn(__ldg(src + i1 * Qy + j0), w10));
    v = __fadd_rn(v, __fmul_rn(__ldg(src + i0 * Qy + j1), w01));
    v = __fadd_rn(v, __fmul_rn(__ldg(src + i1 * Qy + j1), w11));
    return v;
  };
  __syncthreads();
  for (int j = threadIdx.x; j < nleaves; j += kPreThreads)
    leaf[j] = leaf_sum<float>(shifted, llo[j], llen[j]);
  const int Cx = crop_w > 0 ? 2 * crop_w : Qx;
  const int Cy = crop_w > 0 ? 2 * crop_w : Qy;
  float* dst = amps + (size_t)o * Cx * Cy;
  for (int e = threadIdx.x; e < Cx * Cy; e += kPreThreads) {
    const int u = e / Cy, w = e - (e / Cy) * Cy;
    const int x = crop_w > 0 && u >= crop_w ? Qx - Cx + u : u;
    const int y = crop_w > 0 && w >= crop_w ? Qy - Cy + w : w;
    float v = shifted(x * Qy + y);
    if (!(v >= 0.0f) && !isnan(v)) v = 0.0f;
    dst[e] = __fsqrt_rn(v);
  }
  __syncthreads();
  if (threadIdx.x == 0) sums[o] = __fadd_rn(0.0f, pairwise_combine<float>(N, leaf));
}

// ------------------------------------------------------- perfect-tree kernels
// Chain j (0..7) of a leaf of length l starting at element `lo`: r = a[lo + j],
// then r += a[lo + j + 8 k] for k = 1 .. l/8 - 1 (values from `val`). Lane j of
// an 8-lane group holds chain j; the group's lane 0 gets the leaf sum
// ((r0 + r1) + (r2 + r3)) + ((r4 + r5) + (r6 + r7)) plus the l % 8 tail in order.
template <typename Acc, typename V>
__device__ __forceinline__ Acc leaf_chain_sum(const V& val, int lo, int l) {
  const int j = threadIdx.x & 7;
  const int groups = l >> 3;
  Acc r = val(lo + j);
  for (int k = 1; k < groups; ++k) r = acc_add(r, (Acc)val(lo + j + 8 * k));
  Acc o = __shfl_down_sync(0xffffffffu, r, 1, 8);
  if ((j & 1) == 0) r = acc_add(r, o);
  o = __shfl_down_sync(0xffffffffu, r, 2, 8);
  if ((j & 3) == 0) r = acc_add(r, o);
  o = __shfl_down_sync(0xffffffffu, r, 4, 8);
  if (j == 0) {
    r = acc_add(r, o);
    for (int i = groups * 8; i < l; ++i) r = acc_add(r, (Acc)val(lo + i));
  }
  return r;
}

// In-place pairwise sum of q arrays of L = 2^levels leaf sums each (arrays at
// vals + q * L): level by level, vals[j] += vals[j + s]; the totals land in
// vals[q * L]. Called by all threads of the block.
template <typename Acc>
__device__ __forceinline__ void tree_add(Acc* vals, int q, int L) {
  for (int s = 1; s < L; s <<= 1) {
    const int pairs = L / (2 * s);
    for (int t = threadIdx.x; t < q * pairs; t += blockDim.x) {
      const int a = t / pairs, k = t - (t / pairs) * pairs;
      Acc* v = vals + a * L + 2 * s * k;
      v[0] = acc_add(v[0], v[s]);
    }
    __syncthreads();
  }
}

// Centre of mass, perfect tree: block = 8 L threads (at least one warp), one
// pattern per block, lane group g sums leaf g of the three quantities straight
// from global memory (each warp load covers four 32-byte runs).
template <int kMask>
__global__ void __launch_bounds__(1024) pattern_com_kernel(
    const float* __restrict__ in, int Qx, int Qy, const void* __restrict__ mask, int leaf,
    int L, void* cx_out, void* cy_out) {
  using Px = MaskedPixel<kMask>;
  using Acc = typename Px::Acc;
  __shared__ Acc vals[3 * 128];
  const int N = Qx * Qy;
  const int g = threadIdx.x >> 3;
  const Px px{in + (size_t)blockIdx.x * N, mask};
  // lanes past the last leaf (blocks of one warp) sum elements 0..7 and drop
  // the result: every lane of a warp takes part in the shuffles
  const int lo = g < L ? g * leaf : 0;
  const int len = g < L ? leaf : 8;
  const Acc s0 = leaf_chain_sum<Acc>(px, lo, len);
  const Acc s1 = leaf_chain_sum<Acc>(
      [&](int e) { return acc_mul(px(e), (Acc)(e / Qy)); }, lo, len);
  const Acc s2 = leaf_chain_sum<Acc>(
      [&](int e) { return acc_mul(px(e), (Acc)(e - (e / Qy) * Qy)); }, lo, len);
  if (g < L && (threadIdx.x & 7) == 0) {
    vals[g] = s0;
    vals[L + g] = s1;
    vals[2 * L + g] = s2;
  }
  __syncthreads();
  tree_add<Acc>(vals, 3, L);
  if (threadIdx.x == 0) {
    const Acc t0 = acc_add((Acc)0, vals[0]);
    static_cast<Acc*>(cx_out)[blockIdx.x] = acc_div(acc_add((Acc)0, vals[L]), t0);
    static_cast<Acc*>(cy_out)[blockIdx.x] = acc_div(acc_add((Acc)0, vals[2 * L]), t0);
  }
}

// Normalisation, perfect tree: block = 8 L threads, one pattern per block. The
// pattern is staged in shared memory, each thread forms its l/8 shifted values
// (elements tid + k blockDim) in registers, writes them back in place, then the
// lane groups sum the leaves and every thread writes its amplitudes.
constexpr int kMaxPerThread = 16;  // l / 8 <= 128 / 8

__global__ void __launch_bounds__(1024) pattern_normalize_kernel(
    const float* __restrict__ in, int Qx, int Qy, const int32_t* __restrict__ rows,
    const float* __restrict__ cfx, const float* __restrict__ cfy, int crop_w, int leaf, int L,
    float* __restrict__ amps, float* __restrict__ sums) {
  extern __shared__ float4 smem4[];
  __shared__ float vals[128];
  float* pat = reinterpret_cast<float*>(smem4);
  const int N = Qx * Qy;
  const int NT = blockDim.x;
  const int tid = threadIdx.x;
  const int o = blockIdx.x;
  const int r = rows ? rows[o] : o;
  const float* src = in + (size_t)r * N;
  if ((N & 3) == 0 && (reinterpret_cast<uintptr_t>(src) & 15) == 0) {
    const float4* s4 = reinterpret_cast<const float4*>(src);
    for (int e = tid; e < N / 4; e += NT) smem4[e] = __ldg(s4 + e);
  } else {
    for (int e = tid; e < N; e += NT) pat[e] = __ldg(src + e);
  }

  const float xs = -cfx[r], ys = -cfy[r];
  const float xf = floorf(xs), yf = floorf(ys);
  const float wx = __fsub_rn(xs, xf), wy = __fsub_rn(ys, yf);
  const float ux = __fsub_rn(1.0f, wx), uy = __fsub_rn(1.0f, wy);
  const float w00 = __fmul_rn(ux, uy), w10 = __fmul_rn(wx, uy);
  const float w01 = __fmul_rn(ux, wy), w11 = __fmul_rn(wx, wy);
  const int ixm = pmod((int)xf, Qx), iym = pmod((int)yf, Qy);
  __syncthreads();

  // shifted values of elements e = tid + k NT, (i, j) advanced incrementally
  const int per = (N + NT - 1) / NT;
  const int di = NT / Qy, dj = NT - (NT / Qy) * Qy;
  float v[kMaxPerThread];
  {
    int i = tid / Qy, j = tid - (tid / Qy) * Qy;
#pragma unroll
    for (int k = 0; k < kMaxPerThread; ++k) {
      if (k < per && tid + k * NT < N) {
        int i0 = i - ixm;
        if (i0 < 0) i0 += Qx;
        int i1 = i0 - 1;
        if (i1 < 0) i1 += Qx;
        int j0 = j - iym;
        if (j0 < 0) j0 += Qy;
        int j1 = j0 - 1;
        if (j1 < 0) j1 += Qy;
        float t = __fmul_rn(pat[i0 * Qy + j0], w00);
        t = __fadd_rn(t, __fmul_rn(pat[i1 * Qy + j0], w10));
        t = __fadd_rn(t, __fmul_rn(pat[i0 * Qy + j1], w01));
        t = __fadd_rn(t, __fmul_rn(pat[i1 * Qy + j1], w11));
        v[k] = t;
      }
      i += di;
      j += dj;
      if (j >= Qy) {
        j -= Qy;
        ++i;
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kMaxPerThread; ++k)
    if (k < per && tid + k * NT < N) pat[tid + k * NT] = v[k];
  __syncthreads();

  const int g = tid >> 3;
  const float ls = leaf_chain_sum<float>([&](int e) { return pat[e]; }, g < L ? g * leaf : 0,
                                  g < L ? leaf : 8);
  if (g < L && (tid & 7) == 0) vals[g] = ls;

  // amplitudes (numpy.maximum keeps its first argument unless it is below the second)
  const int Cx = crop_w > 0 ? 2 * crop_w : Qx;
  const int Cy = crop_w > 0 ? 2 * crop_w : Qy;
  float* dst = amps + (size_t)o * Cx * Cy;
  for (int e = tid; e < Cx * Cy; e += NT) {
    int x = e / Cy, y = e - (e / Cy) * Cy;
    if (crop_w > 0) {
      if (x >= crop_w) x += Qx - Cx;
      if (y >= crop_w) y += Qy - Cy;
    }
    float a = pat[x * Qy + y];
    if (!(a >= 0.0f) && !isnan(a)) a = 0.0f;
    dst[e] = __fsqrt_rn(a);
  }
  __syncthreads();
  tree_add<float>(vals, 1, L);
  if (tid == 0) sums[o] = __fadd_rn(0.0f, vals[0]);
}

// Number of leaves of the pairwise tree over n values (host side, for sizing).
int pairwise_leaf_count(int n) {
  if (n <= kPwBlock) return 1;
  const int h = pw_half(n);
  return pairwise_leaf_count(h) + pairwise_leaf_count(n - h);
}

// Perfect tree over n values: every split halves a multiple of 16, down to
// 2^levels leaves of length leaf (8 <= leaf <= 128); at most 128 leaves (the
// fast kernels run 8 lanes per leaf in one block of at most 1024 threads).
bool pairwise_perfect(int n, int& leaf, int& levels) {
  levels = 0;
  while (n > kPwBlock) {
    if (n % 16 != 0) return false;
    n /= 2;
    ++levels;
  }
  if (n < 8 || levels > 7) return false;
  leaf = n;
  return true;
}

cudaError_t set_smem(const void* fn, size_t bytes) {
  return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

}  // namespace

size_t preprocess_smem_limit() { return 227 * 1024; }

template <int kMask>
cudaError_t launch_pattern_com_t(const float* in, int num, int Qx, int Qy, const void* mask,
                                 void* cx, void* cy, cudaStream_t s) {
  using Acc = typename MaskedPixel<kMask>::Acc;
  const int N = Qx * Qy;
  int leaf = 0, levels = 0;
  if (pairwise_perfect(N, leaf, levels)) {
    const int L = 1 << levels;
    const int threads = 8 * L < 32 ? 32 : 8 * L;
    pattern_com_kernel<kMask><<<num, threads, 0, s>>>(in, Qx, Qy, mask, leaf, L, cx, cy);
    return cudaGetLastError();
  }
  const int L = pairwise_leaf_count(N);
  const size_t smem = sizeof(Acc) * 3 * (size_t)L + sizeof(int) * 2 * L;
  if (smem > preprocess_smem_limit()) return cudaErrorInvalidValue;
  cudaError_t e = set_smem((const void*)pattern_com_general_kernel<kMask>, smem);
  if (e != cudaSuccess) return e;
  pattern_com_general_kernel<kMask><<<num, kPreThreads, smem, s>>>(in, Qx, Qy, mask, L, cx, cy);
  return cudaGetLastError();
}

cudaError_t launch_pattern_com(const float* in, int num, int Qx, int Qy, const void* mask,
                               int mask_mode, void* cx, void* cy, cudaStream_t s) {
  switch (mask_mode) {
    case 0: return launch_pattern_com_t<0>(in, num, Qx, Qy, nullptr, cx, cy, s);
    case 1: return launch_pattern_com_t<1>(in, num, Qx, Qy, mask, cx, cy, s);
    case 2: return launch_pattern_com_t<2>(in, num, Qx, Qy, mask, cx, cy, s);
    case 3: return launch_pattern_com_t<3>(in, num, Qx, Qy, mask, cx, cy, s);
    default: return cudaErrorInvalidValue;
  }
}

template <typename T>
cudaError_t launch_rotation_search_t(const void* nx, const void* ny, int R0, int R1,
                                     const float* cos_a, const float* sin_a, int A, int div,
                                     void* vals, cudaStream_t s) {
  const int n = (R0 - 2) * (R1 - 2);
  const int L = pairwise_leaf_count(n);
  const size_t smem = sizeof(T) * L + sizeof(int) * 2 * (size_t)L;
  if (smem > preprocess_smem_limit()) return cudaErrorInvalidValue;
  cudaError_t e = set_smem((const void*)rotation_search_kernel<T>, smem);
  if (e != cudaSuccess) return e;
  rotation_search_kernel<T><<<2 * A, kPreThreads, smem, s>>>(
      static_cast<const T*>(nx), static_cast<const T*>(ny), R0, R1, cos_a, sin_a, A, div, L,
      static_cast<T*>(vals));
  return cudaGetLastError();
}

cudaError_t launch_rotation_search(const void* nx, const void* ny, int R0, int R1,
                                   const float* cos_a, const float* sin_a, int A, int div,
                                   int is_double, void* vals, cudaStream_t s) {
  return is_double ? launch_rotation_search_t<double>(nx, ny, R0, R1, cos_a, sin_a, A, div, vals, s)
                   : launch_rotation_search_t<float>(nx, ny, R0, R1, cos_a, sin_a, A, div, vals, s);
}

cudaError_t launch_pattern_normalize(const float* in, int Qx, int Qy, const int32_t* rows,
                                     int num_out, const float* cfx, const float* cfy,
                                     int crop_w, float* amps, float* sums, cudaStream_t s) {
  const int N = Qx * Qy;
  int leaf = 0, levels = 0;
  if (pairwise_perfect(N, leaf, levels)) {
    const int L = 1 << levels;
    const int threads = 8 * L < 32 ? 32 : 8 * L;
    const size_t smem = sizeof(float) * (size_t)N;
    cudaError_t e = set_smem((const void*)pattern_normalize_kernel, smem);
    if (e != cudaSuccess) return e;
    pattern_normalize_kernel<<<num_out, threads, smem, s>>>(in, Qx, Qy, rows, cfx, cfy, crop_w,
                                                            leaf, L, amps, sums);
    return cudaGetLastError();
  }
  const int L = pairwise_leaf_count(N);
  const size_t smem = sizeof(float) * (2 * (size_t)N + L) + sizeof(int) * 2 * L;
  if (smem > preprocess_smem_limit()) {
    // too large to stage: values formed from global memory
    const size_t gsmem = (sizeof(float) + 2 * sizeof(int)) * (size_t)L;
    if (gsmem > preprocess_smem_limit()) return cudaErrorInvalidValue;
    cudaError_t e = set_smem((const void*)pattern_normalize_global_kernel, gsmem);
    if (e != cudaSuccess) return e;
    pattern_normalize_global_kernel<<<num_out, kPreThreads, gsmem, s>>>(
        in, Qx, Qy, rows, cfx, cfy, crop_w, L, amps, sums);
    return cudaGetLastError();
  }
  cudaError_t e = set_smem((const void*)pattern_normalize_general_kernel, smem);
  if (e != cudaSuccess) return e;
  pattern_normalize_general_kernel<<<num_out, kPreThreads, smem, s>>>(in, Qx, Qy, rows, cfx, cfy,
                                                              crop_w, L, amps, sums);
  return cudaGetLastError();
}

// ---- batch pattern gather
//
// out[i, :] = patterns[rows[i], :] for i < n (rows = null: row i). Serves the
// host-resident amplitudes of a reconstruction: the source is page-locked host
// memory mapped into the device address space, read at the CPU-GPU link's rate,
// and the gather of batch k + 1 runs on a second stream while batch k computes.
// A few blocks with 8 loads of 16 bytes in flight per thread keep the link busy;
// they are launched at the device's greatest stream priority, so that they take
// the SM slots that blocks of the running batch free instead of waiting behind
// all of them. A row index outside [0, num_patterns) yields a row of NaN (the
// batch error then reads non-finite) instead of an access outside the source.
namespace {
constexpr int kGatherThreads = 1024;
constexpr int kGatherBlocks = 4;
constexpr int kGatherRows = 2;  // rows per block step
constexpr int kGatherCols = 4;  // vectors per row and thread in one step

template <typename V>
__device__ __forceinline__ V nan_value();
template <>
__device__ __forceinline__ float nan_value<float>() { return __int_as_float(0x7fc00000); }
template <>
__device__ __forceinline__ float4 nan_value<float4>() {
  const float q = __int_as_float(0x7fc00000);
  return make_float4(q, q, q, q);
}

template <typename V>
__global__ void __launch_bounds__(kGatherThreads)
    gather_rows_kernel(const V* __restrict__ src, const int32_t* __restrict__ rows, int n,
                       int num_patterns, int row_len, V* __restrict__ dst) {
  for (int r0 = blockIdx.x * kGatherRows; r0 < n; r0 += gridDim.x * kGatherRows) {
    const V* sp[kGatherRows];
#pragma unroll
    for (int q = 0; q < kGatherRows; ++q) {
      const int r = r0 + q;
      const int sr = r < n ? (rows ? rows[r] : r) : -1;
      sp[q] = (sr >= 0 && sr < num_patterns) ? src + (size_t)sr * row_len : nullptr;
    }
    for (int c0 = threadIdx.x; c0 < row_len; c0 += kGatherThreads * kGatherCols) {
      V v[kGatherRows][kGatherCols];
#pragma unroll
      for (int q = 0; q < kGatherRows; ++q) {
#pragma unroll
        for (int k = 0; k < kGatherCols; ++k) {
          const int c = c0 + k * kGatherThreads;
          v[q][k] = (sp[q] && c < row_len) ? __ldg(sp[q] + c) : nan_value<V>();
        }
      }
#pragma unroll
      for (int q = 0; q < kGatherRows; ++q) {
        const int r = r0 + q;
        if (r >= n) continue;
        V* d = dst + (size_t)r * row_len;
#pragma unroll
        for (int k = 0; k < kGatherCols; ++k) {
          const int c = c0 + k * kGatherThreads;
          if (c < row_len) d[c] = v[q][k];
        }
      }
    }
  }
}

template <typename V>
cudaError_t launch_gather(const V* src, const int32_t* rows, int n, int num_patterns, int row_len,
                          V* dst, cudaStream_t s) {
  int least = 0, greatest = 0;
  cudaError_t e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  const int blocks = (n + kGatherRows - 1) / kGatherRows;
  cfg.gridDim = dim3(blocks < kGatherBlocks ? blocks : kGatherBlocks);
  cfg.blockDim = dim3(kGatherThreads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributePriority;
  attr[0].val.priority = greatest;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, gather_rows_kernel<V>, src, rows, n, num_patterns, row_len, dst);
}
}  // namespace

cudaError_t launch_gather_patterns(const float* src, const int32_t* rows, int n, int num_patterns,
                                   int pattern_size, float* dst, cudaStream_t s) {
  const bool vec = pattern_size % 4 == 0 && reinterpret_cast<uintptr_t>(src) % 16 == 0 &&
                   reinterpret_cast<uintptr_t>(dst) % 16 == 0;
  if (vec)
    return launch_gather(reinterpret_cast<const float4*>(src), rows, n, num_patterns,
                         pattern_size / 4, reinterpret_cast<float4*>(dst), s);
  return launch_gather(src, rows, n, num_patterns, pattern_size, dst, s);
}

}  // namespace pty
