// mlp.cuh -- device helpers of the surrogate MLP: BF16 packing, warp-level BF16 tensor-core MMA
// (mma.sync m16n8k16, FP32 accumulate), ldmatrix fragment loads and the SiLU activation.
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

// tanh on the MUFU unit (PTX tanh.approx.f32, sm_75+).
__device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// SiLU(z) = z * sigmoid(z), with sigmoid(z) = 0.5 + 0.5 * tanh(z / 2): one MUFU operation.
__device__ __forceinline__ float silu(float z) {
  const float s = fmaf(0.5f, tanh_approx(0.5f * z), 0.5f);
  return z * s;
}

// The activation of the surrogate on a pair of pre-activations, as packed BF16:
//   SiLU(z) = z * sigmoid(z) = hz + hz * tanh(hz),  hz = z / 2,
// evaluated in BF16x2: hz rounded to BF16, one MUFU tanh for both values (tanh.approx.bf16x2,
// sm_90+), one BF16x2 FMA.  Training and inference both use this function, so the trained weights
// see exactly the activation that scores poses.  hz = bf16(z / 2) = bf16(z) / 2 exactly, so a
// pre-activation saved as BF16 reproduces the same activation.
// silu2_half takes the halved pre-activations z / 2 (hz before rounding) directly.
__device__ __forceinline__ uint32_t silu2_half(float hz0, float hz1) {
  const uint32_t hz = pack_bf16(hz0, hz1);
  uint32_t t, h;
  asm("tanh.approx.bf16x2 %0, %1;" : "=r"(t) : "r"(hz));
  asm("fma.rn.bf16x2 %0, %1, %2, %1;" : "=r"(h) : "r"(hz), "r"(t));
  return h;
}

__device__ __forceinline__ uint32_t silu2(float z0, float z1) { return silu2_half(0.5f * z0, 0.5f * z1); }

// d SiLU / dz = s * (1 + z * (1 - s)), s = sigmoid(z).
__device__ __forceinline__ float silu_grad(float z) {
  const float s = fmaf(0.5f, tanh_approx(0.5f * z), 0.5f);
  return s * fmaf(z, 1.f - s, 1.f);
}

} // namespace bude
