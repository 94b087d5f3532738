// Volume operations of ptychographic tomography: rotating the (Z, Px, Py)
// potential volume into each tilt's frame, projecting it onto the multislice
// slices, expanding a slice update back onto the voxels, and the per-iteration
// volume constraints.
//
// Reference (py4DSTEM 0.14.18):
//   _rotate_zxy_volume      ptychographic_methods.py:849-868
//     scipy.ndimage.affine_transform(volume, tf, offset, order=3), mode
//     "constant" (cval 0), prefilter on, output in the input's type
//   _project_sliced_object  ptychographic_methods.py:783-812
//   _expand_sliced_object   ptychographic_methods.py:814-847
//   collective update, object constraints
//                           ptychographic_tomography.py:991-1240,
//                           ptychographic_constraints.py:60-118, 836-887
//
// Rotation. The volume is first turned into cubic B-spline coefficients, one
// separable recursive filter per axis (Unser, Aldroubi & Eden, "B-spline signal
// processing", IEEE Trans. Signal Process. 41 (1993); the single pole of the cubic
// spline z = sqrt(3) - 2 and gain (1 - z)(1 - 1/z)), with the exact initial values
// of a mirror-symmetric (whole-sample) extension. Each output voxel o then reads
// the input at c = offset + M o; a coordinate outside [0, n - 1] on any axis gives
// 0, otherwise the 4 x 4 x 4 cubic B-spline weights of c around floor(c) - 1
// combine the coefficients (indices mirrored at the edges). All of it runs in
// float64, like SciPy's, with the coordinate formed as offset + m0 o0 + m1 o1 +
// m2 o2 in that order and without fused multiply-adds, so that the in/out
// decision at the volume's faces falls the same way as SciPy's.

#include <cuda_runtime.h>

#include <cstdint>

#include "ptycho_internal.h"

namespace pty {
namespace {

constexpr int kThreads = 256;

struct Affine {
  double m[9];
  double off[3];
};

__global__ void volume_load_kernel(const void* in, int in_is_double, double* c, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    c[i] = in_is_double ? static_cast<const double*>(in)[i]
                        : (double)static_cast<const float*>(in)[i];
  }
}

// First sample and sample stride of line `line` along `axis` of (n0, n1, n2).
__device__ __forceinline__ void line_geometry(size_t line, int n1, int n2, int axis,
                                              size_t& base, size_t& stride) {
  if (axis == 0) {
    base = line;
    stride = (size_t)n1 * n2;
  } else if (axis == 1) {
    const size_t i0 = line / n2, i2 = line % n2;
    base = i0 * (size_t)n1 * n2 + i2;
    stride = n2;
  } else {
    base = line * (size_t)n2;
    stride = 1;
  }
}

// Cubic B-spline coefficients of one line of L >= 2 samples x[0], x[stride], ...
// in place: gain, causal recursion from the exact initial value of the
// mirror-symmetric extension (period 2L - 2: the sum over one period of z^k x_k
// divided by 1 - z^(2L-2)), anti-causal recursion from its initial value.
__device__ __forceinline__ void spline_line(double* x, size_t stride, int L) {
  const double z = __dadd_rn(sqrt(3.0), -2.0);
  const double gain = __dmul_rn(__dadd_rn(1.0, -z), __dadd_rn(1.0, -__ddiv_rn(1.0, z)));
  for (int i = 0; i < L; ++i) x[i * stride] = __dmul_rn(x[i * stride], gain);
  double zl = 1.0;
  for (int i = 0; i < L - 1; ++i) zl = __dmul_rn(zl, z);  // z^(L-1)
  double s = __dadd_rn(x[0], __dmul_rn(zl, x[(size_t)(L - 1) * stride]));
  double zi = z;
  for (int i = 1; i < L - 1; ++i) {
    const double pair = __dadd_rn(x[i * stride], __dmul_rn(zl, x[(size_t)(L - 1 - i) * stride]));
    s = __dadd_rn(s, __dmul_rn(zi, pair));
    zi = __dmul_rn(zi, z);
  }
  x[0] = __ddiv_rn(s, __dadd_rn(1.0, -__dmul_rn(zl, zl)));
  for (int i = 1; i < L; ++i)
    x[i * stride] = __dadd_rn(x[i * stride], __dmul_rn(z, x[(size_t)(i - 1) * stride]));
  const size_t last = (size_t)(L - 1) * stride;
  x[last] = __ddiv_rn(
      __dmul_rn(__dadd_rn(__dmul_rn(z, x[last - stride]), x[last]), z),
      __dadd_rn(__dmul_rn(z, z), -1.0));
  for (int i = L - 2; i >= 0; --i)
    x[i * stride] = __dmul_rn(z, __dadd_rn(x[(size_t)(i + 1) * stride], -x[i * stride]));
}

// One thread per line along `axis`, in global memory (lines too long to stage).
__global__ void spline_prefilter_kernel(double* c, int n0, int n1, int n2, int axis) {
  const int L = axis == 0 ? n0 : axis == 1 ? n1 : n2;
  const size_t lines = (size_t)n0 * n1 * n2 / (size_t)L;
  const size_t line = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (line >= lines || L < 2) return;
  size_t base, stride;
  line_geometry(line, n1, n2, axis, base, stride);
  spline_line(c + base, stride, L);
}

// Lines staged in shared memory: each warp of the block owns 32 consecutive
// lines, loaded and stored with coalesced accesses (row by row for the
// contiguous axis), and runs the recursions there. Sample i of the warp's line l
// sits at s[i * kLineLD + l]; the odd pitch spreads a row's samples over banks.
constexpr int kLineLD = 33;

__global__ void spline_prefilter_staged_kernel(double* c, int n0, int n1, int n2, int axis) {
  extern __shared__ double staged[];
  const int L = axis == 0 ? n0 : axis == 1 ? n1 : n2;
  const size_t lines = (size_t)n0 * n1 * n2 / (size_t)L;
  const int warps = blockDim.x / 32;
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const size_t first = ((size_t)blockIdx.x * warps + warp) * 32;
  if (first >= lines || L < 2) return;  // the same for every lane of the warp
  double* s = staged + (size_t)warp * kLineLD * L;
  const size_t line = first + lane;
  const bool active = line < lines;
  const int nl = (int)(lines - first < 32 ? lines - first : 32);
  size_t base = 0, stride = 1;
  if (active) line_geometry(line, n1, n2, axis, base, stride);
  if (axis == 2) {
    for (int l = 0; l < nl; ++l) {
      const double* row = c + (first + l) * (size_t)n2;
      for (int i = lane; i < L; i += 32) s[i * kLineLD + l] = row[i];
    }
  } else if (active) {
    for (int i = 0; i < L; ++i) s[i * kLineLD + lane] = c[base + (size_t)i * stride];
  }
  __syncwarp();
  if (active) spline_line(s + lane, kLineLD, L);
  __syncwarp();
  if (axis == 2) {
    for (int l = 0; l < nl; ++l) {
      double* row = c + (first + l) * (size_t)n2;
      for (int i = lane; i < L; i += 32) row[i] = s[i * kLineLD + l];
    }
  } else if (active) {
    for (int i = 0; i < L; ++i) c[base + (size_t)i * stride] = s[i * kLineLD + lane];
  }
}

__device__ __forceinline__ int mirror_index(int i, int n) {
  if (n == 1) return 0;
  const int period = 2 * n - 2;
  i = i < 0 ? -i : i;
  i %= period;
  return i >= n ? period - i : i;
}

// Cubic B-spline weights of the four samples floor(x) - 1 .. floor(x) + 2.
__device__ __forceinline__ void cubic_weights(double t, double w[4]) {
  const double u = __dadd_rn(1.0, -t);
  const double t2 = __dmul_rn(t, t), u2 = __dmul_rn(u, u);
  const double sixth = __ddiv_rn(1.0, 6.0), two3 = __ddiv_rn(2.0, 3.0);
  w[0] = __dmul_rn(__dmul_rn(u2, u), sixth);
  w[1] = __dadd_rn(__dadd_rn(two3, -t2), __dmul_rn(__dmul_rn(t2, t), 0.5));
  w[2] = __dadd_rn(__dadd_rn(two3, -u2), __dmul_rn(__dmul_rn(u2, u), 0.5));
  w[3] = __dmul_rn(__dmul_rn(t2, t), sixth);
}

// out_mode 0: float32 out; 1: float64 out; 2: float32 out += value (the sum
// formed in float64 and rounded once).
__global__ void volume_affine_kernel(const double* __restrict__ c, void* out, int out_mode,
                                     int n0, int n1, int n2, Affine tf) {
  const size_t total = (size_t)n0 * n1 * n2;
  const int n[3] = {n0, n1, n2};
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const double o[3] = {(double)(i / ((size_t)n1 * n2)), (double)((i / n2) % n1),
                         (double)(i % n2)};
    double x[3];
    bool inside = true;
#pragma unroll
    for (int h = 0; h < 3; ++h) {
      double v = tf.off[h];
#pragma unroll
      for (int l = 0; l < 3; ++l) v = __dadd_rn(v, __dmul_rn(tf.m[h * 3 + l], o[l]));
      x[h] = v;
      inside = inside && !(v < 0.0) && !(v > (double)(n[h] - 1));
    }
    double value = 0.0;
    if (inside) {
      int idx[3][4];
      double w[3][4];
#pragma unroll
      for (int h = 0; h < 3; ++h) {
        const double f = floor(x[h]);
        const int start = (int)f - 1;
        cubic_weights(__dadd_rn(x[h], -f), w[h]);
#pragma unroll
        for (int k = 0; k < 4; ++k) idx[h][k] = mirror_index(start + k, n[h]);
      }
      for (int a = 0; a < 4; ++a) {
        const size_t ra = (size_t)idx[0][a] * n1;
        for (int b = 0; b < 4; ++b) {
          const double wab = __dmul_rn(w[0][a], w[1][b]);
          const double* row = c + (ra + idx[1][b]) * n2;
#pragma unroll
          for (int k = 0; k < 4; ++k)
            value = __dadd_rn(value, __dmul_rn(__dmul_rn(wab, w[2][k]), row[idx[2][k]]));
        }
      }
    }
    if (out_mode == 0) {
      static_cast<float*>(out)[i] = (float)value;
    } else if (out_mode == 1) {
      static_cast<double*>(out)[i] = value;
    } else {
      float* dst = static_cast<float*>(out) + i;
      *dst = (float)__dadd_rn((double)*dst, value);
    }
  }
}

// sliced[t] = volume[t*vps] + volume[t*vps + 1] + ... (float32, in voxel order;
// voxels past the end count as the zero padding of the reference).
__global__ void volume_project_kernel(const float* __restrict__ vol, int n0, int T, size_t P,
                                      int vps, float* __restrict__ sliced) {
  const size_t total = (size_t)T * P;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int t = (int)(i / P);
    const size_t p = i % P;
    float s = 0.0f;
    for (int k = 0; k < vps; ++k) {
      const int zz = t * vps + k;
      const float v = zz < n0 ? vol[(size_t)zz * P + p] : 0.0f;
      s = k == 0 ? v : __fadd_rn(s, v);
    }
    sliced[i] = s;
  }
}

// Voxel z of slice t = z / vps receives (sliced - sliced_old)[t] / count_t in
// float64 (count_t = vps, or the remainder for the last slice). out_mode 1:
// float64 out; 2: float32 out += value.
__global__ void volume_expand_kernel(const float* __restrict__ sliced,
                                     const float* __restrict__ old, int n0, size_t P, int vps,
                                     int T, int last_count, void* out, int out_mode) {
  const size_t total = (size_t)n0 * P;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int zz = (int)(i / P);
    const size_t p = i % P;
    const int t = zz / vps;
    const float u = __fsub_rn(sliced[(size_t)t * P + p], old[(size_t)t * P + p]);
    const double v = __ddiv_rn((double)u, (double)(t == T - 1 ? last_count : vps));
    if (out_mode == 1) {
      static_cast<double*>(out)[i] = v;
    } else {
      float* dst = static_cast<float*>(out) + i;
      *dst = (float)__dadd_rn((double)*dst, v);
    }
  }
}

__global__ void volume_add_scaled_kernel(float* vol, const float* addend, size_t n, float div) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    vol[i] = __fadd_rn(vol[i], __fdiv_rn(addend[i], div));
}

__global__ void volume_constraints_kernel(float* vol, size_t n, float shrinkage,
                                          int apply_shrinkage, int positivity) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    float v = vol[i];
    if (apply_shrinkage) v = __fsub_rn(v, shrinkage);
    if (positivity && v < 0.0f) v = 0.0f;
    vol[i] = v;
  }
}

unsigned grid_for(size_t n) {
  const size_t blocks = (n + kThreads - 1) / kThreads;
  return (unsigned)(blocks < 152 * 16 ? (blocks ? blocks : 1) : 152 * 16);
}

}  // namespace

cudaError_t launch_volume_rotate(const void* in, int in_is_double, void* out, int out_mode,
                                 int n0, int n1, int n2, const double* matrix,
                                 const double* offset, double* scratch, cudaStream_t s) {
  const size_t total = (size_t)n0 * n1 * n2;
  Affine tf;
  for (int k = 0; k < 9; ++k) tf.m[k] = matrix[k];
  for (int k = 0; k < 3; ++k) tf.off[k] = offset[k];
  volume_load_kernel<<<grid_for(total), kThreads, 0, s>>>(in, in_is_double, scratch, total);
  int smem_optin = 0;
  {
    // the staged prefilter may use up to the device's opt-in limit of dynamic
    // shared memory; the attribute is set per device
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess)
      e = cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess)
      e = ensure_smem_limit(reinterpret_cast<const void*>(spline_prefilter_staged_kernel),
                            smem_optin);
    if (e != cudaSuccess) return e;
  }
  const int n[3] = {n0, n1, n2};
  for (int axis = 0; axis < 3; ++axis) {
    if (n[axis] < 2) continue;
    const size_t lines = total / (size_t)n[axis];
    const size_t per_warp = sizeof(double) * kLineLD * (size_t)n[axis];
    if (per_warp <= (size_t)smem_optin) {
      int warps = 4;
      while (warps > 1 && (size_t)warps * per_warp > (size_t)smem_optin) warps /= 2;
      const size_t per_block = (size_t)warps * 32;
      spline_prefilter_staged_kernel<<<(unsigned)((lines + per_block - 1) / per_block),
                                       warps * 32, warps * per_warp, s>>>(scratch, n0, n1, n2,
                                                                          axis);
    } else {
      spline_prefilter_kernel<<<(unsigned)((lines + 127) / 128), 128, 0, s>>>(scratch, n0, n1,
                                                                             n2, axis);
    }
  }
  volume_affine_kernel<<<grid_for(total), kThreads, 0, s>>>(scratch, out, out_mode, n0, n1, n2,
                                                            tf);
  return cudaGetLastError();
}

cudaError_t launch_volume_project(const float* vol, int n0, size_t P, int T, float* sliced,
                                  cudaStream_t s) {
  const int vps = (n0 + T - 1) / T;
  volume_project_kernel<<<grid_for((size_t)T * P), kThreads, 0, s>>>(vol, n0, T, P, vps,
                                                                     sliced);
  return cudaGetLastError();
}

cudaError_t launch_volume_expand(const float* sliced, const float* old, int T, int n0, size_t P,
                                 void* out, int out_mode, cudaStream_t s) {
  const int vps = (n0 + T - 1) / T;
  const int rem = vps - (vps * T - n0);
  const int last_count = rem > 0 ? rem : vps;
  volume_expand_kernel<<<grid_for((size_t)n0 * P), kThreads, 0, s>>>(sliced, old, n0, P, vps, T,
                                                                     last_count, out, out_mode);
  return cudaGetLastError();
}

cudaError_t launch_volume_add_scaled(float* vol, const float* addend, size_t n, int divisor,
                                     cudaStream_t s) {
  volume_add_scaled_kernel<<<grid_for(n), kThreads, 0, s>>>(vol, addend, n, (float)divisor);
  return cudaGetLastError();
}

cudaError_t launch_volume_constraints(float* vol, size_t n, float shrinkage, int apply_shrinkage,
                                      int positivity, cudaStream_t s) {
  volume_constraints_kernel<<<grid_for(n), kThreads, 0, s>>>(vol, n, shrinkage, apply_shrinkage,
                                                             positivity);
  return cudaGetLastError();
}

}  // namespace pty
