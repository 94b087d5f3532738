// Row gather for amplitudes kept in host memory (storage="cpu").
//
// The reference keeps the amplitudes on the host with storage="cpu" and copies
// each batch's patterns to the device before its forward pass
// (copy_to_device(self._amplitudes[batch_indices]), singleslice_ptychography.py:
// 873-875). Here a page-locked, mapped host array is gathered by a kernel: the
// batch's rows, in the order the batch visits them, are read over the CPU-GPU
// link with 16-byte loads and written contiguously into a device buffer. Issued
// on a second stream one batch ahead, the transfer of batch k + 1 overlaps the
// computation of batch k (a CUDA graph captures both streams).
#include <cuda_runtime.h>

#include <cstdint>

#include "ptycho_internal.h"

namespace pty {
namespace {

constexpr int kGatherThreads = 256;
constexpr int kUnroll = 4;

// dst[k] = src[rows[k]] for k < num_rows, rows of row_bytes bytes (a multiple of
// 16, both bases 16-byte aligned); blocks stride over the rows.
__global__ void __launch_bounds__(kGatherThreads) gather_rows_kernel(
    const uint4* __restrict__ src, const int32_t* __restrict__ rows, int num_rows,
    size_t row_vecs, uint4* __restrict__ dst) {
  for (int k = blockIdx.x; k < num_rows; k += gridDim.x) {
    const uint4* s = src + (size_t)rows[k] * row_vecs;
    uint4* d = dst + (size_t)k * row_vecs;
    for (size_t i = threadIdx.x; i < row_vecs; i += (size_t)kGatherThreads * kUnroll) {
      uint4 v[kUnroll];
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) {
        const size_t j = i + (size_t)u * kGatherThreads;
        if (j < row_vecs) v[u] = s[j];
      }
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) {
        const size_t j = i + (size_t)u * kGatherThreads;
        if (j < row_vecs) d[j] = v[u];
      }
    }
  }
}

}  // namespace

cudaError_t launch_gather_rows(const void* src, const int32_t* rows, int num_rows,
                               size_t row_bytes, void* dst, cudaStream_t s) {
  if (num_rows <= 0) return cudaSuccess;
  // enough blocks to keep the link busy, few enough to share the SMs with the
  // batch that is computing meanwhile
  const int blocks = num_rows < 128 ? num_rows : 128;
  gather_rows_kernel<<<blocks, kGatherThreads, 0, s>>>(
      static_cast<const uint4*>(src), rows, num_rows, row_bytes / 16, static_cast<uint4*>(dst));
  return cudaGetLastError();
}

}  // namespace pty
