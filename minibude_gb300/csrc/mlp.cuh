// mlp.cuh -- device helpers of the surrogate MLP: BF16 packing, warp-level BF16 tensor-core MMA
// (mma.sync m16n8k16, FP32 accumulate), ldmatrix fragment loads and the activation (hard-swish).
//
// Fragment layouts of mma.m16n8k16 (lane l, g = l / 4, t = l % 4):
//   A 16x16 (row-major):  a0 = (g, 2t..2t+1)  a1 = (g+8, 2t..)  a2 = (g, 2t+8..)  a3 = (g+8, 2t+8..)
//   B 16x8  (k x n):      b0 = (k 2t..2t+1, n g)   b1 = (k 2t+8..2t+9, n g)
//   C 16x8  (fp32):       c0,c1 = (g, 2t..2t+1)   c2,c3 = (g+8, 2t..2t+1)
// Two adjacent C tiles (n 0..7 and 8..15) hold exactly the A fragment of one 16-wide k step of the
// next layer, so a layer's output feeds the next layer from registers.
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

#include "ptx.cuh"

namespace bude {

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi); // .x = lo (low half), .y = hi
  return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ float2 unpack_bf16(uint32_t v) {
  __nv_bfloat162 h = *reinterpret_cast<__nv_bfloat162 *>(&v);
  return __bfloat1622float2(h);
}

// D = A * B + D, BF16 inputs, FP32 accumulate.
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const void *smem_row) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(static_cast<uint32_t>(__cvta_generic_to_shared(smem_row))));
}

__device__ __forceinline__ void ldsm_x4_trans(uint32_t (&r)[4], const void *smem_row) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(static_cast<uint32_t>(__cvta_generic_to_shared(smem_row))));
}

// The activation of the surrogate: hard-swish, h(z) = z * sat(z / 6 + 1/2), evaluated in FP32 on
// the FMA pipe (one FMA with saturation and one multiply per value; no MUFU operation) and rounded
// to BF16 as the next layer's operand.  Training and inference both use act_pair, so the trained
// weights see exactly the activation that scores poses.
constexpr float kActSlope = 1.f / 6.f;

__device__ __forceinline__ float act(float z) {
  float s;
  asm("fma.rn.sat.f32 %0, %1, %2, 0f3F000000;" : "=f"(s) : "f"(z), "f"(kActSlope));
  return z * s;
}

// Two pre-activations -> packed BF16 activations (lo = z0, hi = z1): act() on both, the two
// multiplies as one packed f32x2 instruction (rounded per lane exactly as the scalar form).
__device__ __forceinline__ uint32_t act_pair(float z0, float z1) {
  float s0, s1;
  asm("fma.rn.sat.f32 %0, %1, %2, 0f3F000000;" : "=f"(s0) : "f"(z0), "f"(kActSlope));
  asm("fma.rn.sat.f32 %0, %1, %2, 0f3F000000;" : "=f"(s1) : "f"(z1), "f"(kActSlope));
  const float2 h = mul2(make_float2(z0, z1), make_float2(s0, s1));
  return pack_bf16(h.x, h.y);
}

// The same activation of two values kept in FP32 (the output layer's input: y = w4 . h3 is
// computed on the FMA pipe, so h3 is not rounded to BF16).
__device__ __forceinline__ float2 act_f2(float z0, float z1) {
  float s0, s1;
  asm("fma.rn.sat.f32 %0, %1, %2, 0f3F000000;" : "=f"(s0) : "f"(z0), "f"(kActSlope));
  asm("fma.rn.sat.f32 %0, %1, %2, 0f3F000000;" : "=f"(s1) : "f"(z1), "f"(kActSlope));
  return mul2(make_float2(z0, z1), make_float2(s0, s1));
}

// FP16 pair (lo in the low half), rounded to nearest and saturated to the largest finite value.
__device__ __forceinline__ uint32_t pack_f16(float lo, float hi) {
  uint32_t d;
  asm("cvt.rn.satfinite.f16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
  return d;
}

// The activation for the FP16 scorer: z rounded to FP16, then s = sat(z / 6 + 1/2) and z * s as
// packed FP16 instructions (three instructions per pair; FP16 keeps 11 significant bits, so the
// result is closer to the FP32 activation than the BF16-rounded one the training pass uses).
__device__ __forceinline__ uint32_t act_pair_f16(float z0, float z1) {
  const uint32_t zh = pack_f16(z0, z1);
  uint32_t s, h;
  asm("fma.rn.sat.f16x2 %0, %1, %2, %3;" : "=r"(s) : "r"(zh), "r"(0x31553155u), "r"(0x38003800u)); // 1/6, 1/2
  asm("mul.rn.f16x2 %0, %1, %2;" : "=r"(h) : "r"(zh), "r"(s));
  return h;
}

// Packed BF16 helpers for the backward pass's element-wise work (one instruction per pair).
__device__ __forceinline__ uint32_t mul_bf16x2(uint32_t a, uint32_t b) {
  uint32_t d;
  asm("mul.rn.bf16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
  return d;
}

// The activation of a BF16 pair in packed BF16 arithmetic, three instructions: s = min(relu(z * c
// + 1/2), 1) with c = 1/6 rounded to BF16 (0.16699), h = z * s.  The weight-gradient kernel
// rebuilds the forward pass's activations from the stored pre-activations this way.
__device__ __forceinline__ uint32_t act_bf16x2(uint32_t z) {
  uint32_t t, h;
  asm("fma.rn.relu.bf16x2 %0, %1, %2, %3;" : "=r"(t) : "r"(z), "r"(0x3E2B3E2Bu), "r"(0x3F003F00u));
  asm("min.bf16x2 %0, %1, %2;" : "=r"(t) : "r"(t), "r"(0x3F803F80u));
  asm("mul.rn.bf16x2 %0, %1, %2;" : "=r"(h) : "r"(z), "r"(t));
  return h;
}

// dh/dz of a BF16 pair as a BF16 pair, five packed instructions: t = z * c + 1/2 with c = 1/3
// rounded to BF16 (0.33398, 0.2% steep), kept where -3 < z < 3; 1 where z >= 3; 0 where z <= -3
// (set.* gives 1.0 or 0.0 per half: act' = t * (gt(-3) - ge(3)) + ge(3)).
__device__ __forceinline__ uint32_t act_grad_bf16x2(uint32_t z) {
  uint32_t t, hi, lo, in, r;
  asm("fma.rn.bf16x2 %0, %1, %2, %3;" : "=r"(t) : "r"(z), "r"(0x3EAB3EABu), "r"(0x3F003F00u));
  asm("set.ge.bf16x2.bf16x2 %0, %1, %2;" : "=r"(hi) : "r"(z), "r"(0x40404040u));
  asm("set.gt.bf16x2.bf16x2 %0, %1, %2;" : "=r"(lo) : "r"(z), "r"(0xC040C040u));
  asm("sub.rn.bf16x2 %0, %1, %2;" : "=r"(in) : "r"(lo), "r"(hi));
  asm("fma.rn.bf16x2 %0, %1, %2, %3;" : "=r"(r) : "r"(t), "r"(in), "r"(hi));
  return r;
}

// dh/dz: 0 below -3, 1 above 3, z / 3 + 1/2 between.
__device__ __forceinline__ float act_grad(float z) {
  return z <= -3.f ? 0.f : (z >= 3.f ? 1.f : fmaf(z, 2.f * kActSlope, 0.5f));
}

} // namespace bude
