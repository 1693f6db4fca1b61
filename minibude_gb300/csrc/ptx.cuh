// ptx.cuh -- inline-PTX helpers for sm_103a: mbarriers, 1-D TMA bulk copies and the two
// arithmetic instructions the exact kernel is built on.
#pragma once
#include <cstdint>

namespace bude {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// fma with saturation to [0, 1] (PTX `fma.rn.sat.f32`; a NaN result becomes +0).
__device__ __forceinline__ float fma_sat(float a, float b, float c) {
  float d;
  asm("fma.rn.sat.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}

// Hardware square-root approximation (PTX `sqrt.approx.ftz.f32`); sqrt(+0) = +0.
__device__ __forceinline__ float sqrt_approx(float x) {
  float y;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Packed FP32 pair arithmetic (PTX `*.f32x2`, sm_100+): one instruction for two lanes of work,
// each lane rounded exactly as the scalar instruction would be.
__device__ __forceinline__ unsigned long long f2_bits(float2 v) {
  return (unsigned long long)__float_as_uint(v.x) | ((unsigned long long)__float_as_uint(v.y) << 32);
}
__device__ __forceinline__ float2 f2_from(unsigned long long b) {
  return make_float2(__uint_as_float((unsigned)(b & 0xffffffffull)), __uint_as_float((unsigned)(b >> 32)));
}
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
  unsigned long long d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_bits(a)), "l"(f2_bits(b)));
  return f2_from(d);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) {
  unsigned long long d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_bits(a)), "l"(f2_bits(b)));
  return f2_from(d);
}
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(f2_bits(a)), "l"(f2_bits(b)), "l"(f2_bits(c)));
  return f2_from(d);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Make barrier initialisation visible to the async (TMA) proxy and the rest of the cluster.
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// One arrival on a barrier (its pending count drops by one).
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Retire a barrier before its shared memory is left (used where a wait gave up on it).
__device__ __forceinline__ void mbar_inval(uint64_t *bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// One bounded probe of the barrier's phase; true once the phase with `parity` has completed.
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Limit for every device-side wait: far above any legitimate wait (a bulk copy of a few KB from
// L2 takes microseconds), short enough that a wait that can never finish gives up within a second
// and the kernel returns an error status instead of hanging the GPU.
constexpr uint64_t kWaitLimitNs = 1000ull * 1000ull * 1000ull;
constexpr uint32_t kWaitMaxProbes = 1u << 26;

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint64_t limit_ns = kWaitLimitNs) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer_ns();
  for (uint32_t it = 1; it < kWaitMaxProbes; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 255u) == 0 && globaltimer_ns() - t0 > limit_ns) return false;
  }
  return false;
}

// The same bounded wait with a suspend-time hint: a waiting thread may sleep in the barrier until
// the phase completes (or 1 ms passes) instead of probing it again and again, which leaves the
// shared-memory pipe to the threads doing work.  Used where 128 threads wait on one tensor-core
// commit at a time.
__device__ __forceinline__ bool mbar_try_wait_sleep(uint64_t *bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity), "r"(1000000u)
      : "memory");
  return done != 0;
}
__device__ __forceinline__ bool mbar_wait_sleep_bounded(uint64_t *bar, uint32_t parity) {
  if (mbar_try_wait_sleep(bar, parity)) return true;
  const uint64_t t0 = globaltimer_ns();
  for (uint32_t it = 1; it < kWaitMaxProbes; ++it) {
    if (mbar_try_wait_sleep(bar, parity)) return true;
    if (globaltimer_ns() - t0 > kWaitLimitNs) return false;
  }
  return false;
}

// 16-byte read-only global load that the compiler may not hoist out of a loop.
__device__ __forceinline__ float4 ldg_stream(const float4 *p) {
  float4 v;
  asm volatile("ld.global.nc.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p));
  return v;
}

// 1-D TMA bulk copy global -> this CTA's shared memory, completing on `bar` by transaction bytes.
// dst and src must be 16-byte aligned and bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// Programmatic dependent launch (sm_90+).  A kernel launched with programmatic stream
// serialisation may be scheduled while the kernel before it in the stream is still finishing (its
// blocks as the earlier kernel's blocks exit): grid_dep_wait() blocks until that kernel has
// completed and its memory is visible, and returns at once for a kernel launched without the
// attribute.  Every kernel of such a chain waits before it touches memory that an earlier kernel
// writes or reads, so that completion is transitive along the chain.  (No kernel here releases its
// dependents early with griddepcontrol.launch_dependents: dependents resident beside a running
// kernel made the training step slower, 6.77 s against 6.03 s for 80 epochs.)
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

} // namespace bude
