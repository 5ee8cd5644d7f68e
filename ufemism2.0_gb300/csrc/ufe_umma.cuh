// Blackwell tensor-core building blocks (sm_103a): tcgen05 MMA with operands in shared memory and
// the accumulator in tensor memory (TMEM), mbarrier completion, TMEM -> register loads.
//
// Operand layout: K-major, 128-byte swizzle.  A tile of R rows x 64 BF16 (one 128-byte row per
// matrix row) is stored in 1024-byte atoms of 8 rows; the 16-byte chunk c of row r sits at chunk
// position c ^ (r % 8) of its 128-byte row.  A tile base must be 1024-byte aligned.  For the MMA,
// D[M x N] (+)= A[M x K] * B[N x K]^T: A is M rows x K, B is N rows x K (a Linear layer's weight
// [out x in] as it is stored), both K-major.
//
// Every wait on an mbarrier is bounded: after kSpinLimit polls the waiter gives up and reports
// failure, so a kernel never hangs on a completion that does not come.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace umma {

constexpr int kSpinLimit = 1 << 22;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (r, k) (k < 64) inside a 128B-swizzled K-major tile
__device__ __forceinline__ uint32_t sw128_offset(int r, int k) {
  const int chunk = k >> 3;
  return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((chunk ^ (r & 7)) << 4) + ((k & 7) << 1));
}
// byte offset of 16-byte chunk c (0..7) of row r
__device__ __forceinline__ uint32_t sw128_chunk(int r, int c) {
  return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((c ^ (r & 7)) << 4));
}

// Shared-memory matrix descriptor: start address >> 4 in bits 0-13, leading byte offset >> 4 in
// 16-29 (not used by swizzled K-major operands), stride byte offset >> 4 in 32-45 (1024 B between
// 8-row groups), descriptor version 1 in bits 46-47, swizzle mode in 61-63 (2: 128-byte).
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)(16 >> 4) << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// Instruction descriptor for kind::f16: FP32 accumulator (bits 4-5 = 1), BF16 A and B (bits 7-9,
// 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(idesc), "r"(acc)
      : "memory");
}

// arrive on the mbarrier when all tcgen05 operations issued so far by this thread complete
__device__ __forceinline__ void commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
               : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// make generic-proxy shared-memory writes visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_smem_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}

// bounded wait for the phase with the given parity to complete; false if it did not
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
  for (int i = 0; i < kSpinLimit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// TMEM allocation by one full warp; the base address is written to *slot (shared memory)
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane (warp w reads lanes 32(w%4) .. +31)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Issue D (+)= A * B^T for one 128-row tile: A is `kblocks` 64-wide K blocks of 128 rows
// (16 KB each), B `kblocks` K blocks of N rows (N x 128 B each).  One thread calls this.
template <int N>
__device__ __forceinline__ void mma_tile(uint32_t tmem_d, uint32_t a_smem, uint32_t b_smem, int kblocks,
                                         bool accumulate) {
  constexpr uint32_t idesc = idesc_bf16_f32(128, N);
  for (int kb = 0; kb < kblocks; ++kb) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {   // UMMA_K = 16 BF16 = 32 bytes inside the 128-byte swizzled row
      const uint64_t da = desc_sw128(a_smem + kb * 128 * 128 + j * 32);
      const uint64_t db = desc_sw128(b_smem + kb * N * 128 + j * 32);
      mma_bf16(tmem_d, da, db, idesc, (accumulate || kb > 0 || j > 0) ? 1u : 0u);
    }
  }
}

}  // namespace umma
