// tc.cuh -- 5th-generation tensor-core (tcgen05) helpers for sm_100-family GPUs, as inline PTX:
// tensor-memory (TMEM) allocation, BF16 UMMA with FP32 accumulation in TMEM, completion through an
// mbarrier, and TMEM -> register loads.
//
// Operands come from shared memory through 64-bit matrix descriptors.  This file uses the
// K-major layout without swizzling: the matrix is cut into "core matrices" of 8 rows x 16 bytes
// (8 BF16 values of K), each stored as 128 contiguous bytes (row r of the core matrix at r * 16).
// Core matrices adjacent along K are `lbo` bytes apart (leading byte offset), core matrices
// adjacent along M (or N) are `sbo` bytes apart (stride byte offset).  With lbo = 128 and
// sbo = (K / 8) * 128 a [rows][K] tile occupies rows * K * 2 contiguous bytes and element (m, k)
// sits at (m / 8) * sbo + (k / 8) * 128 + (m % 8) * 16 + (k % 8) * 2.  One MMA consumes K = 16
// (two core matrices along K), so the descriptor start advances by 2 * lbo per K step.
#pragma once
#include <cstdint>

#include "ptx.cuh"

namespace bude {

// Byte offset of element (m, k) of a K-major, unswizzled [rows][kdim] BF16 tile.
__host__ __device__ __forceinline__ uint32_t kmajor_offset(int m, int k, int kdim) {
  return (uint32_t)((m >> 3) * (kdim / 8) * 128 + (k >> 3) * 128 + (m & 7) * 16 + (k & 7) * 2);
}

// Row-tiled global layout of a [rows][kdim] BF16 array (the training pass's features,
// pre-activations and their gradients): 128-row tiles of 128 * kdim * 2 contiguous bytes, each in
// the K-major layout above, so a tile is byte for byte the shared-memory operand tile and the 16
// bytes that 8 consecutive rows keep at the same k form one 128-byte line.  Byte offset of (row, k).
__host__ __device__ __forceinline__ long long tiled_offset(long long row, int k, int kdim) {
  return (row >> 7) * (128LL * kdim * 2) + kmajor_offset((int)(row & 127), k, kdim);
}
__host__ __device__ __forceinline__ long long tiled_rows(long long rows) { return (rows + 127) / 128 * 128; }

// Shared-memory matrix descriptor (sm_100 format): start address, leading and stride byte
// offsets (all >> 4), descriptor version 1 at bits 46-47, base offset 0, no swizzle (bits 61-63).
__device__ __forceinline__ uint64_t umma_desc(uint32_t smem_addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((smem_addr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B BF16 (bits 7-9, 10-12 = 1),
// both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// The same with A and B FP16 (bits 7-12 = 0).
__host__ __device__ constexpr uint32_t umma_idesc_f16(int m, int n) {
  return (1u << 4) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// Allocate `ncols` TMEM columns (power of two >= 32) for this CTA; executed by one whole warp.
// The TMEM address is written to the shared-memory word `slot`.
template <int NCOLS> __device__ __forceinline__ void tmem_alloc(uint32_t *slot) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
               "n"(NCOLS)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

template <int NCOLS> __device__ __forceinline__ void tmem_dealloc(uint32_t taddr) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "n"(NCOLS) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Generic-proxy shared-memory writes become visible to the tensor core (async proxy).
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// D[tmem] (+)= A * B^T for one K = 16 step; issued by a single thread.
__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// D[tmem] (+)= A[tmem] * B^T for one K = 16 step, A read from tensor memory (the thread's lane
// r holds row r of A, two BF16 values of K per 32-bit column, 8 columns per K = 16 step).
__device__ __forceinline__ void umma_bf16_ts(uint32_t tmem_d, uint32_t tmem_a, uint64_t bdesc, uint32_t idesc,
                                             uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(tmem_d),
      "r"(tmem_a), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrive once on `bar` when every MMA this thread issued so far has completed.
__device__ __forceinline__ void umma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// 32 consecutive FP32 columns of this thread's TMEM lane (warp w reads lanes 32w..32w+31).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
      "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
        "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
        "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr)
      : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
        "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr)
      : "memory");
}

// Store 8 / 16 / 32 consecutive 32-bit columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_st8(uint32_t taddr, const uint32_t (&v)[8]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr), "r"(v[0]),
               "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7])
               : "memory");
}
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t (&v)[16]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
               "%16};" ::"r"(taddr),
               "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]),
               "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15])
               : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// body(c, v) over the 8 chunks of 16 columns starting at taddr (c = 0..7, v = the chunk's 16 FP32
// values), with the load of chunk c + 1 in flight while chunk c is processed: one TMEM load
// latency per 128 columns instead of one per chunk.
template <class F> __device__ __forceinline__ void tmem_rows128(uint32_t taddr, F &&body) {
  uint32_t a[16], b[16];
  tmem_ld16(taddr, a);
  tmem_wait_ld();
#pragma unroll
  for (int c = 0; c < 8; c += 2) {
    tmem_ld16(taddr + (uint32_t)((c + 1) * 16), b);
    body(c, a);
    tmem_wait_ld();
    if (c + 2 < 8) tmem_ld16(taddr + (uint32_t)((c + 2) * 16), a);
    body(c + 1, b);
    if (c + 2 < 8) tmem_wait_ld();
  }
}

// Named barrier over `nthreads` threads (a multiple of 32); id 0 is __syncthreads' barrier.
__device__ __forceinline__ void named_sync(uint32_t id, uint32_t nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// Named barrier that also returns whether `v` was true in any of the participating threads.
__device__ __forceinline__ bool named_sync_or(uint32_t id, uint32_t nthreads, bool v) {
  uint32_t r;
  asm volatile("{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.or.pred q, %2, %3, p;\n\t"
               "selp.u32 %0, 1, 0, q;\n\t}"
               : "=r"(r)
               : "r"((uint32_t)v), "r"(id), "r"(nthreads)
               : "memory");
  return r != 0;
}


} // namespace bude
