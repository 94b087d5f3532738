// BF16 x BF16 -> FP32 tile GEMM on the fifth-generation tensor cores (sm_103a):
// tcgen05.mma issued by one thread per CTA, operands staged in shared memory in
// the canonical K-major layout without swizzle, the 128 x BN accumulator in
// tensor memory (TMEM), read back with tcgen05.ld for the epilogue.
//
// The operand tiles are gathered by the CTA's threads through loader functors,
// so one kernel serves plain GEMMs and the implicit-GEMM convolutions of the
// learned initializer (im2col addressing inside the loader, zero padding at the
// borders). A loader returns the 16 bytes (8 bf16) of one row at K offset 8*kc.
//
// Shared-memory layout of one operand tile of R rows x 64 K (bf16): core
// matrices of 8 rows x 16 bytes (128 contiguous bytes, row-major), core matrix
// (row group g, K chunk c) at byte (g * 8 + c) * 128. In the matrix descriptor
// the leading-dimension byte offset (between core matrices adjacent in K) is
// 128 and the stride-dimension byte offset (between 8-row groups) is 1024; one
// MMA consumes K = 16 (two core matrices along K), so the k-th MMA of a tile
// starts 256 k bytes further.
//
// Pipeline: two shared-memory stages. The threads fill stage s while the tensor
// core works on stage s^1; tcgen05.commit signals an mbarrier per stage when
// the MMAs reading it are done. Every wait is bounded (about one second of
// %globaltimer): on time-out the kernel records where in *err (non-zero), stops
// issuing, waits (bounded) for the MMAs in flight and frees its TMEM before it
// returns.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace pty {
namespace nn {

constexpr int kBM = 128;  // rows of the accumulator tile (TMEM lanes)
constexpr int kBK = 64;   // K per pipeline stage (bf16 elements)
constexpr int kGemmThreads = 128;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for the phase with the given parity to complete, at most ~1 s.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (global_ns() - t0 > 1000000000ull) return false;
  }
  return true;
}

__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// One warp: allocate `ncols` TMEM columns (power of two, 32..512); the address
// goes to *dst (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(dst)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

// Shared-memory matrix descriptor: start address, leading / stride byte offsets,
// the descriptor version of tcgen05 (bit 46), no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4);
  d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
  d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
  d |= static_cast<uint64_t>(1) << 46;
  return d;
}

// Instruction descriptor of kind::f16: D f32, A and B bf16, both K-major,
// shape M x N.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(N >> 3) << 17) |
         (static_cast<uint32_t>(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

// 16 consecutive fp32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_load16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Byte offset of (row, K chunk) inside an operand tile.
__device__ __forceinline__ uint32_t tile_offset(int row, int kc) {
  return static_cast<uint32_t>(((row >> 3) * 8 + kc) * 128 + (row & 7) * 16);
}

template <int BN>
struct GemmSmem {
  static constexpr int kA = kBM * kBK * 2;  // bytes per A stage
  static constexpr int kB = BN * kBK * 2;   // bytes per B stage
  static constexpr int kBytes = 2 * (kA + kB) + 1024;  // + barriers, TMEM slot, alignment
};

// C tile (blockIdx.x: 128 rows, blockIdx.y: BN columns) = sum over K of A B^T for
// the K range of blockIdx.z (split K: [z * k_per_split, (z + 1) * k_per_split)).
// LoadA(row, kc) / LoadB(col, kc): 16 bytes of row `row` at K = 8 kc (the
// loaders return zeros outside the matrix). Epi(row, col0, v[16], z): columns
// col0..col0+15 of row `row`.
template <int BN, class LoadA, class LoadB, class Epi>
__global__ void __launch_bounds__(kGemmThreads) tc_gemm_kernel(int M, int N, int K,
                                                               int k_per_split, LoadA la,
                                                               LoadB lb, Epi epi, int* err) {
  static_assert(BN == 32 || BN == 64 || BN == 128 || BN == 256, "BN");
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1024-byte aligned base for the operand stages
  unsigned char* base = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* stA[2] = {base, base + GemmSmem<BN>::kA};
  unsigned char* stB[2] = {base + 2 * GemmSmem<BN>::kA,
                           base + 2 * GemmSmem<BN>::kA + GemmSmem<BN>::kB};
  __shared__ uint64_t bar[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;

  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int row0 = blockIdx.x * kBM;
  const int col0 = blockIdx.y * BN;
  const int kbeg = blockIdx.z * k_per_split;
  const int kend = min(K, kbeg + k_per_split);
  const int nk = kend > kbeg ? (kend - kbeg + kBK - 1) / kBK : 0;

  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tmem_alloc(&tmem_slot, BN);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  constexpr uint32_t idesc = idesc_bf16_f32(kBM, BN);

  int issued = -1;  // last iteration whose MMAs were issued (the same in every thread)
  for (int it = 0; it < nk; ++it) {
    const int s = it & 1;
    if (it >= 2) {
      // the MMAs of iteration it - 2 read this stage
      if (!mbar_wait_bounded(&bar[s], ((it >> 1) - 1) & 1)) atomicExch(&abort_flag, 2 + it);
    }
    __syncthreads();
    if (abort_flag) break;
    const int kc0 = (kbeg >> 3) + it * (kBK / 8);  // first K chunk of this stage
    const int kc_end = (kend + 7) >> 3;
    // A: 128 rows x 8 chunks
#pragma unroll 4
    for (int i = tid; i < kBM * (kBK / 8); i += kGemmThreads) {
      const int r = i >> 3, c = i & 7;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (kc0 + c < kc_end) v = la(row0 + r, kc0 + c);
      *reinterpret_cast<uint4*>(stA[s] + tile_offset(r, c)) = v;
    }
#pragma unroll 4
    for (int i = tid; i < BN * (kBK / 8); i += kGemmThreads) {
      const int r = i >> 3, c = i & 7;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (kc0 + c < kc_end) v = lb(col0 + r, kc0 + c);
      *reinterpret_cast<uint4*>(stB[s] + tile_offset(r, c)) = v;
    }
    fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      const uint32_t a0 = smem_u32(stA[s]);
      const uint32_t b0 = smem_u32(stB[s]);
#pragma unroll
      for (int k = 0; k < kBK / 16; ++k) {
        const uint64_t ad = smem_desc(a0 + 256 * k, 128, 1024);
        const uint64_t bd = smem_desc(b0 + 256 * k, 128, 1024);
        mma_bf16(tmem, ad, bd, idesc, (it > 0 || k > 0) ? 1u : 0u);
      }
      mma_commit(&bar[s]);
    }
    issued = it;
  }
  // The last commit covers every MMA issued before it. After an abort this
  // still waits (bounded) for the MMAs in flight before the TMEM is freed.
  if (issued >= 0 && !mbar_wait_bounded(&bar[issued & 1], (issued >> 1) & 1))
    atomicExch(&abort_flag, 1);
  __syncthreads();
  tc_fence_after();
  const bool ok = !abort_flag;
  // *err: 1 = the final wait timed out, 2 + it = the wait before refilling a
  // stage at iteration it (the largest code of any CTA is kept)
  if (!ok && tid == 0) atomicMax(err, abort_flag);
  // epilogue: warp w reads TMEM lanes 32w..32w+31 (rows), 16 columns at a time
  const int row = row0 + warp * 32 + (tid & 31);
  if (ok) {
#pragma unroll 1
    for (int c = 0; c < BN; c += 16) {
      float v[16];
      if (nk > 0) {
        tmem_load16(tmem + (static_cast<uint32_t>(warp * 32) << 16) + c, v);
      } else {
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] = 0.0f;
      }
      if (row < M && col0 + c < N) epi(row, col0 + c, v, static_cast<int>(blockIdx.z));
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, BN);
}

}  // namespace nn
}  // namespace pty
