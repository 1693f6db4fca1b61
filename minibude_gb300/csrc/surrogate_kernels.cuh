// surrogate_kernels.cuh -- the learned pre-screen: a per-ligand-atom MLP whose outputs are summed
// per pose to approximate the exact pose energy.
//
// Model (all sizes fixed):
//   features  x (32) = [type embedding (16) | transformed atom position * xyz_scale (3) |
//                       13 protein-field channels sampled at the position]
//   layers    z1 = W1 x + b1 (128), h1 = act(z1); z2 = W2 h1 + b2, h2 = act(z2);
//             z3 = W3 h2 + b3, h3 = act(z3); y = w4 . h3 + b4,   act = hard-swish (mlp.cuh)
//   pose      E_pose = sum over the ligand's atoms of y
// FP32 masters and FP32 Adam state; 16-bit copies for the tensor cores: BF16 (plain and
// transposed) for training and for the warp-level mma.sync scorer in this file, FP16 for the
// tcgen05 scorer (score_tc.cuh).  Activations between hidden layers are rounded to the 16-bit type;
// every product accumulates in FP32.  Weights are stored [out][in] (in contiguous), so a layer's
// mma.sync B fragments are plain ldmatrix loads and a tcgen05 operand tile is a K-major copy.
// This file holds the field grid, the features, the mma.sync scorer (`score_kernel`, selectable
// through bude_surrogate_set_scorer) and the training pass's small kernels; the training GEMMs are
// in score_tc.cuh (forward, backward) and wgrad_tc.cuh (weight gradients).
//
// The protein-field channels come from a grid precomputed once per protein (grid_kernel): for a
// point x and protein atoms p (radius R_p, hphb h_p, elsc q_p, hbtype), distance r = |x - p|:
//   c0..c3   sum_p relu(1 - r / (R + R_p))             probe radius R = 1.0, 1.5, 2.0, 2.5
//   c4, c5   sum_p q_p   * sat(1 - (r - (1.75+R_p))/d)  d = 2, 4
//   c6, c7   sum_p |q_p| * sat(1 - (r - (1.75+R_p))/d)  d = 2, 4
//   c8       sum_{p: 'F'} q_p * sat(1 - (r - (1.75+R_p))/4)
//   c9       sum_{p: h_p<0} h_p * sat(1 - (r - (1.75+R_p))/5.5)
//   c10      sum_{p: h_p>0} h_p * sat(1 - (r - (1.75+R_p))/1)
//   c11      sum_{p: h_p<0} h_p * sat(1 - (r - (1.75+R_p))/1)
//   c12      min_p (r - R_p), clamped to [-3, 8]
// i.e. the distance-dependent shapes of the steric, charge and desolvation terms of the exact
// kernel for a few probe atoms, each scaled to unit standard deviation over the grid.  The scaled
// grid is stored as four FP16 3-D textures (c0..c3, c4..c7, c8..c11, c12) and sampled with the
// texture unit's trilinear filter, clamped at the grid's faces.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cstdint>

#include "../../include/minibude_gb300.h"
#include "mlp.cuh"
#include "ptx.cuh"
#include "tc.cuh"

namespace bude {

constexpr int kFeat = 32;
constexpr int kHid = 128;
constexpr int kEmb = 16;
constexpr int kGridCh = 13;
constexpr int kMaxTypes = 64;
constexpr int kRowsPerCta = 128; // 8 warps x 16 rows
constexpr int kMlpThreads = 256;
constexpr int kLdX = kFeat + 8;  // padded smem row strides (bf16 elements): conflict-free ldmatrix
constexpr int kLdH = kHid + 8;

// Parameters the forward kernels read (device pointers).
struct MlpWeights {
  const __nv_bfloat16 *emb; // [kMaxTypes][16]
  const __nv_bfloat16 *w1;  // [128][32]
  const __nv_bfloat16 *w2;  // [128][128]
  const __nv_bfloat16 *w3;  // [128][128]
  const float *b1, *b2, *b3, *w4, *b4; // [128] x 4, [1]
};

struct FieldGrid {
  cudaTextureObject_t tex[4]; // FP16 3-D textures: c0..c3, c4..c7, c8..c11 (4 channels), c12 (1)
  float ox, oy, oz, inv_h;    // grid origin and 1 / spacing
  float xyz_scale;
};

// ---------------------------------------------------------------------------------------------
// Field grid

struct GridBuild {
  const float4 *protein; // {x, y, z, type bits}
  const bude_ffparams *ff;
  int natpro;
  float ox, oy, oz, h;
  int nx, ny, nz;
  float *out; // [voxels][16]
};

__global__ void __launch_bounds__(128) grid_kernel(GridBuild g) {
  const long long nvox = (long long)g.nx * g.ny * g.nz;
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nvox) return;
  const int ix = (int)(v % g.nx);
  const int iy = (int)((v / g.nx) % g.ny);
  const int iz = (int)(v / ((long long)g.nx * g.ny));
  const float x = g.ox + ix * g.h, y = g.oy + iy * g.h, z = g.oz + iz * g.h;
  float c[kGridCh];
#pragma unroll
  for (int k = 0; k < kGridCh; ++k) c[k] = 0.f;
  c[12] = 8.f;
  for (int j = 0; j < g.natpro; ++j) {
    const float4 p = __ldg(&g.protein[j]);
    const bude_ffparams f = g.ff[__float_as_int(p.w)];
    const float dx = x - p.x, dy = y - p.y, dz = z - p.z;
    const float r = sqrtf(dx * dx + dy * dy + dz * dz);
    c[0] += fmaxf(0.f, 1.f - r / (1.0f + f.radius));
    c[1] += fmaxf(0.f, 1.f - r / (1.5f + f.radius));
    c[2] += fmaxf(0.f, 1.f - r / (2.0f + f.radius));
    c[3] += fmaxf(0.f, 1.f - r / (2.5f + f.radius));
    const float bb = r - (1.75f + f.radius);
    const float s2 = __saturatef(1.f - bb * 0.5f), s4 = __saturatef(1.f - bb * 0.25f);
    const float s55 = __saturatef(1.f - bb * (1.f / 5.5f)), s1 = __saturatef(1.f - bb);
    c[4] += f.elsc * s2;
    c[5] += f.elsc * s4;
    c[6] += fabsf(f.elsc) * s2;
    c[7] += fabsf(f.elsc) * s4;
    if (f.hbtype == 70) c[8] += f.elsc * s4;
    if (f.hphb < 0.f) {
      c[9] += f.hphb * s55;
      c[11] += f.hphb * s1;
    } else if (f.hphb > 0.f) {
      c[10] += f.hphb * s1;
    }
    c[12] = fminf(c[12], r - f.radius);
  }
  c[12] = fmaxf(c[12], -3.f);
  float *o = g.out + v * 16;
#pragma unroll
  for (int k = 0; k < kGridCh; ++k) o[k] = c[k];
  o[13] = o[14] = o[15] = 0.f;
}

// Divide every channel by its scale (channels 13..15 stay zero).
__global__ void grid_scale_kernel(float *grid, long long nvox, const float *inv_scale) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nvox * 16) return;
  grid[i] *= inv_scale[i % 16];
}

// Split the scaled [voxels][16] FP32 grid into the texture layouts (FP16).
__global__ void grid_pack_kernel(const float *grid, long long nvox, __half *t0, __half *t1, __half *t2, __half *t3) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nvox) return;
  const float *c = grid + v * 16;
  __half *dst[3] = {t0, t1, t2};
#pragma unroll
  for (int q = 0; q < 3; ++q)
#pragma unroll
    for (int k = 0; k < 4; ++k) dst[q][v * 4 + k] = __float2half_rn(c[q * 4 + k]);
  t3[v] = __float2half_rn(c[12]);
}

// Trilinear sample of the 13 channels at a position.  Texel centres sit at integer + 0.5 in
// unnormalised texture coordinates, so grid point i of axis u is at u = i + 0.5.
__device__ __forceinline__ void sample_field(const FieldGrid &g, float x, float y, float z, float (&c)[kGridCh]) {
  const float u = fmaf(x - g.ox, g.inv_h, 0.5f), v = fmaf(y - g.oy, g.inv_h, 0.5f), w = fmaf(z - g.oz, g.inv_h, 0.5f);
  const float4 a = tex3D<float4>(g.tex[0], u, v, w);
  const float4 b = tex3D<float4>(g.tex[1], u, v, w);
  const float4 d = tex3D<float4>(g.tex[2], u, v, w);
  c[0] = a.x; c[1] = a.y; c[2] = a.z; c[3] = a.w;
  c[4] = b.x; c[5] = b.y; c[6] = b.z; c[7] = b.w;
  c[8] = d.x; c[9] = d.y; c[10] = d.z; c[11] = d.w;
  c[12] = tex3D<float>(g.tex[3], u, v, w);
}

// Features 16..31 of one (pose, ligand atom) -- the transformed position x 0.1 and the 13 field
// channels -- as 8 packed BF16 pairs (FP16 pairs when F16), from the atom {x, y, z, type bits} and
// the pose's transform rows r0..r2 ({R row, t}).
template <bool F16 = false>
__device__ __forceinline__ void field_features(const FieldGrid &g, float4 la, float4 r0, float4 r1, float4 r2,
                                               uint32_t (&p)[8]) {
  const float x = r0.w + la.x * r0.x + la.y * r0.y + la.z * r0.z;
  const float y = r1.w + la.x * r1.x + la.y * r1.y + la.z * r1.z;
  const float z = r2.w + la.x * r2.x + la.y * r2.y + la.z * r2.z;
  float c[kGridCh];
  sample_field(g, x, y, z, c);
  auto pk = [](float lo, float hi) { return F16 ? pack_f16(lo, hi) : pack_bf16(lo, hi); };
  p[0] = pk(x * g.xyz_scale, y * g.xyz_scale);
  p[1] = pk(z * g.xyz_scale, c[0]);
  p[2] = pk(c[1], c[2]);
  p[3] = pk(c[3], c[4]);
  p[4] = pk(c[5], c[6]);
  p[5] = pk(c[7], c[8]);
  p[6] = pk(c[9], c[10]);
  p[7] = pk(c[11], c[12]);
}

// Features of one (pose, ligand atom) as 16 packed BF16 pairs: the type's embedding e0, e1
// (features 0..15, 16 BF16) and field_features.
__device__ __forceinline__ void features_of(const FieldGrid &g, float4 la, float4 r0, float4 r1, float4 r2, uint4 e0,
                                            uint4 e1, uint32_t (&f)[kFeat / 2]) {
  f[0] = e0.x; f[1] = e0.y; f[2] = e0.z; f[3] = e0.w;
  f[4] = e1.x; f[5] = e1.y; f[6] = e1.z; f[7] = e1.w;
  uint32_t p[8];
  field_features(g, la, r0, r1, r2, p);
#pragma unroll
  for (int i = 0; i < 8; ++i) f[8 + i] = p[i];
}

__device__ __forceinline__ void atom_features(const MlpWeights &W, const FieldGrid &g, float4 la, const float4 *xf,
                                              uint32_t (&f)[kFeat / 2]) {
  const uint4 *e = reinterpret_cast<const uint4 *>(W.emb + __float_as_int(la.w) * kEmb);
  features_of(g, la, __ldg(xf), __ldg(xf + 1), __ldg(xf + 2), __ldg(e), __ldg(e + 1), f);
}

// ---------------------------------------------------------------------------------------------
// Shared-memory copy of the BF16 weights (padded rows) and the FP32 vectors.

struct MlpSmem {
  __nv_bfloat16 w1[kHid * kLdX];
  __nv_bfloat16 w2[kHid * kLdH];
  __nv_bfloat16 w3[kHid * kLdH];
  __nv_bfloat16 x[kRowsPerCta * kLdX];
  float b1[kHid], b2[kHid], b3[kHid], w4[kHid];
};

__device__ __forceinline__ void load_weights(MlpSmem &s, const MlpWeights &W) {
  for (int i = threadIdx.x; i < kHid * kFeat / 8; i += blockDim.x) {
    const int o = i / (kFeat / 8), k8 = i % (kFeat / 8);
    *reinterpret_cast<uint4 *>(&s.w1[o * kLdX + k8 * 8]) = __ldg(reinterpret_cast<const uint4 *>(W.w1) + i);
  }
  for (int i = threadIdx.x; i < kHid * kHid / 8; i += blockDim.x) {
    const int o = i / (kHid / 8), k8 = i % (kHid / 8);
    *reinterpret_cast<uint4 *>(&s.w2[o * kLdH + k8 * 8]) = __ldg(reinterpret_cast<const uint4 *>(W.w2) + i);
    *reinterpret_cast<uint4 *>(&s.w3[o * kLdH + k8 * 8]) = __ldg(reinterpret_cast<const uint4 *>(W.w3) + i);
  }
  for (int i = threadIdx.x; i < kHid; i += blockDim.x) {
    s.b1[i] = W.b1[i];
    s.b2[i] = W.b2[i];
    s.b3[i] = W.b3[i];
    s.w4[i] = W.w4[i];
  }
}

// One 16-row x 128-column layer: acc = A * W^T, A given as 16x16 fragments for NK k-steps.
template <int NK, int LDW>
__device__ __forceinline__ void layer_mma(float (&acc)[16][4], const uint32_t (&a)[NK][4],
                                          const __nv_bfloat16 *w) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int j = 0; j < 16; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
#pragma unroll
  for (int kk = 0; kk < NK; ++kk) {
#pragma unroll
    for (int jp = 0; jp < 8; ++jp) { // n-tiles 2jp, 2jp+1
      uint32_t b[4];
      const int row = jp * 16 + (lane & 7) + ((lane >> 4) << 3);
      const int col = kk * 16 + ((lane >> 3) & 1) * 8;
      ldsm_x4(b, w + row * LDW + col);
      mma_bf16(acc[2 * jp], a[kk], b[0], b[1]);
      mma_bf16(acc[2 * jp + 1], a[kk], b[2], b[3]);
    }
  }
}

// bias + activation on a layer's accumulators and repack them as the next layer's A fragments;
// z (optional) receives the pre-activations as BF16 pairs in accumulator layout.
__device__ __forceinline__ void act_to_frags(float (&acc)[16][4], const float *bias, uint32_t (&a)[8][4],
                                             uint32_t (*z)[2]) {
  const int t = threadIdx.x & 3;
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    const float bl = bias[j * 8 + 2 * t], bh = bias[j * 8 + 2 * t + 1];
    const float z0 = acc[j][0] + bl, z1 = acc[j][1] + bh, z2 = acc[j][2] + bl, z3 = acc[j][3] + bh;
    if (z) {
      z[j][0] = pack_bf16(z0, z1);
      z[j][1] = pack_bf16(z2, z3);
    }
    const uint32_t lo = act_pair(z0, z1); // row g
    const uint32_t hi = act_pair(z2, z3); // row g + 8
    const int kk = j >> 1;
    if ((j & 1) == 0) {
      a[kk][0] = lo;
      a[kk][1] = hi;
    } else {
      a[kk][2] = lo;
      a[kk][3] = hi;
    }
  }
}

// Final layer on A-fragment-packed h3: y for rows g and g+8 (full dot after the quad reduce).
__device__ __forceinline__ float2 last_layer(const uint32_t (&h3)[8][4], const float *w4) {
  const int t = threadIdx.x & 3;
  float y0 = 0.f, y1 = 0.f;
#pragma unroll
  for (int kk = 0; kk < 8; ++kk) {
    const int c0 = kk * 16 + 2 * t, c1 = c0 + 8;
    float2 v;
    v = unpack_bf16(h3[kk][0]);
    y0 = fmaf(v.x, w4[c0], fmaf(v.y, w4[c0 + 1], y0));
    v = unpack_bf16(h3[kk][2]);
    y0 = fmaf(v.x, w4[c1], fmaf(v.y, w4[c1 + 1], y0));
    v = unpack_bf16(h3[kk][1]);
    y1 = fmaf(v.x, w4[c0], fmaf(v.y, w4[c0 + 1], y1));
    v = unpack_bf16(h3[kk][3]);
    y1 = fmaf(v.x, w4[c1], fmaf(v.y, w4[c1 + 1], y1));
  }
  y0 += __shfl_xor_sync(0xffffffffu, y0, 1);
  y0 += __shfl_xor_sync(0xffffffffu, y0, 2);
  y1 += __shfl_xor_sync(0xffffffffu, y1, 1);
  y1 += __shfl_xor_sync(0xffffffffu, y1, 2);
  return make_float2(y0, y1);
}

// Load a warp's 16 rows of the smem feature tile as layer-1 A fragments.
__device__ __forceinline__ void x_frags(const __nv_bfloat16 *xs, int row0, uint32_t (&a)[2][4]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int kk = 0; kk < 2; ++kk) {
    const int row = row0 + (lane & 7) + ((lane >> 3) & 1) * 8;
    const int col = kk * 16 + (lane >> 4) * 8;
    ldsm_x4(a[kk], xs + row * kLdX + col);
  }
}

// ---------------------------------------------------------------------------------------------
// Inference: one block per item (ligand, block of up to 128 poses); features are built per ligand
// atom into shared memory and run through the MLP by 8 warps of 16 poses each.

struct ScoreArgs {
  MlpWeights W;
  FieldGrid g;
  const float4 *ligands; // concatenated ligand atoms
  const float4 *xform;   // [poses][3]
  const int4 *items;     // {first ligand atom, natlig, first pose, pose count}
  float *scores;         // per pose
  int n_items;
};

__global__ void __launch_bounds__(kMlpThreads) score_kernel(const ScoreArgs a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  MlpSmem &s = *reinterpret_cast<MlpSmem *>(smem_raw);
  load_weights(s, a.W);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2;
  for (int item = blockIdx.x; item < a.n_items; item += gridDim.x) {
    const int4 it = __ldg(&a.items[item]);
    float e0 = 0.f, e1 = 0.f; // rows warp*16 + g and + 8
    for (int il = 0; il < it.y; ++il) {
      __syncthreads(); // previous tile consumed (and weights loaded)
      const float4 la = __ldg(&a.ligands[it.x + il]);
      if (threadIdx.x < kRowsPerCta) {
        const int r = threadIdx.x;
        const int pose = it.z + min(r, it.w - 1);
        uint32_t f[kFeat / 2];
        atom_features(a.W, a.g, la, a.xform + (long long)pose * 3, f);
        uint4 *dst = reinterpret_cast<uint4 *>(&s.x[r * kLdX]);
        dst[0] = make_uint4(f[0], f[1], f[2], f[3]);
        dst[1] = make_uint4(f[4], f[5], f[6], f[7]);
        dst[2] = make_uint4(f[8], f[9], f[10], f[11]);
        dst[3] = make_uint4(f[12], f[13], f[14], f[15]);
      }
      __syncthreads();
      uint32_t ax[2][4], h[8][4];
      float acc[16][4];
      x_frags(s.x, warp * 16, ax);
      layer_mma<2, kLdX>(acc, ax, s.w1);
      act_to_frags(acc, s.b1, h, nullptr);
      layer_mma<8, kLdH>(acc, h, s.w2);
      act_to_frags(acc, s.b2, h, nullptr);
      layer_mma<8, kLdH>(acc, h, s.w3);
      act_to_frags(acc, s.b3, h, nullptr);
      const float2 y = last_layer(h, s.w4);
      e0 += y.x;
      e1 += y.y;
    }
    if ((lane & 3) == 0) {
      const float nb4 = it.y * __ldg(a.W.b4);
      const int r0 = warp * 16 + g, r1 = r0 + 8;
      if (r0 < it.w) a.scores[it.z + r0] = e0 + nb4;
      if (r1 < it.w) a.scores[it.z + r1] = e1 + nb4;
    }
  }
}

// ---------------------------------------------------------------------------------------------
// Training.  A batch is a list of poses; its rows (pose, ligand atom) are laid out pose by pose.

struct RowMap {
  const int *pose;    // global pose index per batch pose
  const int *row_off; // batch poses + 1 row offsets
  const int *lig_first, *lig_n; // per global pose: first atom and atom count of its ligand
  int nposes;
};

// One warp per batch pose writes the features (and types) of its rows; X is row-tiled (tc.cuh:
// tiled_offset).  The first kernel of a training step: it also zeroes the step's two work counters
// (`counters`, when given: the forward and backward passes' tile counters).
__global__ void __launch_bounds__(256) train_features_kernel(MlpWeights W, FieldGrid g, const float4 *ligands,
                                                             const float4 *xform, RowMap m, __nv_bfloat16 *X,
                                                             int *row_type, unsigned int *counters) {
  grid_dep_wait();
  if (counters && blockIdx.x == 0 && threadIdx.x < 2) counters[threadIdx.x] = 0u;
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= m.nposes) return;
  const int p = m.pose[i];
  const int first = m.lig_first[p], n = m.lig_n[p], row0 = m.row_off[i];
  for (int a = lane; a < n; a += 32) {
    const float4 la = __ldg(&ligands[first + a]);
    uint32_t f[kFeat / 2];
    atom_features(W, g, la, xform + (long long)p * 3, f);
    unsigned char *xb = reinterpret_cast<unsigned char *>(X);
#pragma unroll
    for (int q = 0; q < 4; ++q)
      *reinterpret_cast<uint4 *>(xb + tiled_offset(row0 + a, q * 8, kFeat)) =
          make_uint4(f[4 * q], f[4 * q + 1], f[4 * q + 2], f[4 * q + 3]);
    row_type[row0 + a] = __float_as_int(la.w);
  }
}

// Per batch pose: prediction = sum of its rows' y + natlig * b4; loss on the compressed scale
// c(E) = S * asinh(E / S); dy (per row) = dLoss/dprediction.  loss_out[i] = the pose's squared
// error (summed on the host, deterministic); dsum[block] = the sum of dy over the block's rows.
// One warp per pose (lanes take rows a, a + 32, ...; a butterfly sum gives every lane the total),
// so a warp's row loads and dy stores are consecutive floats; kLossPoses warps per block keep the
// number of dsum parts that the gradient reduction folds small.
constexpr float kLossScale = 20.f;
constexpr int kLossPoses = 32; // warps (poses) per block

__global__ void __launch_bounds__(32 * kLossPoses) train_loss_kernel(RowMap m, const float *y, const float *b4,
                                                                     const float *labels, float *pred,
                                                                     float *loss_out, float *dy, float *dsum,
                                                                     float inv_batch) {
  grid_dep_wait();
  __shared__ float share[kLossPoses];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int i = blockIdx.x * kLossPoses + warp;
  float mine = 0.f;
  if (i < m.nposes) {
    const int row0 = m.row_off[i], n = m.row_off[i + 1] - row0;
    float s = 0.f;
    for (int a = lane; a < n; a += 32) s += y[row0 + a];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    s += n * b4[0];
    const float cs = kLossScale * asinhf(s / kLossScale), ce = kLossScale * asinhf(labels[m.pose[i]] / kLossScale);
    const float d = cs - ce;
    const float grad = 2.f * d * rsqrtf(1.f + (s / kLossScale) * (s / kLossScale)) * inv_batch;
    for (int a = lane; a < n; a += 32) dy[row0 + a] = grad;
    if (lane == 0) {
      pred[i] = s;
      loss_out[i] = d * d;
    }
    mine = (float)n * grad; // the pose's share of the b4 gradient (sum of dy over its rows)
  }
  if (lane == 0) share[warp] = mine;
  __syncthreads();
  // dsum[block] = the block's poses' shares in a fixed butterfly order
  if (warp == 0) {
    float t = share[lane];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) dsum[blockIdx.x] = t;
  }
}

// The per-step gradient reductions in one launch: segment k sums parts [0, nparts) of
// part[p * stride + i] into dst[i] for i < n.  A block of 8 warps takes 32 consecutive elements
// (lane = element, so every load of a warp reads 32 consecutive floats); warp j adds parts
// j, j + 8, j + 16, ... in order (24 loads in flight), and warp 0 adds the eight warps' sums in
// warp order, so the result is the same bits on every run.
constexpr int kMaxReduceSegs = 10;
constexpr int kReduceWarps = 8;

struct ReduceSegs {
  const float *part[kMaxReduceSegs];
  float *dst[kMaxReduceSegs];
  long long stride[kMaxReduceSegs];
  int n[kMaxReduceSegs];
  int nparts[kMaxReduceSegs];
  int first[kMaxReduceSegs + 1]; // prefix sums of n: element e belongs to segment k with first[k] <= e
  int tr_rows[kMaxReduceSegs];   // > 0: the parts hold a tr_rows x tr_cols matrix column by column
  int tr_cols[kMaxReduceSegs];   // (element i at (i % tr_rows) * tr_cols + i / tr_rows of dst)
  int nseg;
};

// Destination of element i of a segment whose parts hold an R x C matrix column by column (element
// [row][col] at col * R + row) in the row-major result; R = 0: the identity.
__host__ __device__ __forceinline__ int reduce_dst_index(int i, int R, int C) {
  return R > 0 ? (i % R) * C + i / R : i;
}

__global__ void __launch_bounds__(32 * kReduceWarps) reduce_segments_kernel(const ReduceSegs r) {
  grid_dep_wait();
  __shared__ float sums[kReduceWarps][32];
  const int lane = threadIdx.x & 31, j = threadIdx.x >> 5;
  const int e = blockIdx.x * 32 + lane;
  const bool live = e < r.first[r.nseg];
  int k = 0;
  while (live && k + 1 < r.nseg && r.first[k + 1] <= e) ++k;
  float v = 0.f;
  if (live) {
    const float *part = r.part[k] + (e - r.first[k]);
    const long long stride = r.stride[k];
    const int np = r.nparts[k];
    // 24 parts per round, all loads in flight at once (a part past the end adds +0).
    for (int p = j; p < np; p += 24 * kReduceWarps) {
      float x[24];
#pragma unroll
      for (int q = 0; q < 24; ++q) x[q] = p + q * kReduceWarps < np ? part[(long long)(p + q * kReduceWarps) * stride] : 0.f;
#pragma unroll
      for (int q = 0; q < 24; ++q) v += x[q];
    }
  }
  sums[j][lane] = v;
  __syncthreads();
  if (j == 0 && live) {
    float t = sums[0][lane];
    for (int w = 1; w < kReduceWarps; ++w) t += sums[w][lane];
    r.dst[k][reduce_dst_index(e - r.first[k], r.tr_rows[k], r.tr_cols[k])] = t;
  }
}

// 16-bit copies of FP32 master matrices inside the parameter vector: matrix k is the [rows][cols]
// block at off[k], copied to BF16 plainly and/or transposed, and to FP16 plainly (null pointers
// skip a copy).
struct BfCopies {
  long long off[4];
  int rows[4], cols[4];
  __nv_bfloat16 *plain[4], *trans[4];
  __half *half[4];
  int n;
};

__device__ __forceinline__ void bf_copy(const BfCopies &c, long long i, float w) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const long long j = i - c.off[k];
    if (k < c.n && j >= 0 && j < (long long)c.rows[k] * c.cols[k]) {
      const int r = (int)(j / c.cols[k]), col = (int)(j % c.cols[k]);
      const __nv_bfloat16 b = __float2bfloat16_rn(w);
      if (c.plain[k]) c.plain[k][j] = b;
      if (c.trans[k]) c.trans[k][(long long)col * c.rows[k] + r] = b;
      if (c.half[k]) c.half[k][j] = __float2half_rn(w);
    }
  }
}

// Adam on the FP32 masters (Kingma & Ba, with the bias corrections applied as torch.optim.Adam
// applies them): m = b1 m + (1-b1) g, v = b2 v + (1-b2) g^2,
// w -= (lr / bc1) * m / (sqrt(v) / sqrt(bc2) + eps), with bc1 = 1 - b1^t and bc2 = 1 - b2^t
// precomputed on the host as step = lr / bc1 and bc2_sqrt = sqrt(bc2).  The updated weights'
// BF16 copies are written in the same pass.
__global__ void adam_kernel(float *w, float *m, float *v, const float *grad, long long n, float step, float bc2_sqrt,
                            float b1, float b2, float eps, const BfCopies copies) {
  grid_dep_wait();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gr = grad[i];
  const float mi = b1 * m[i] + (1.f - b1) * gr;
  const float vi = b2 * v[i] + (1.f - b2) * gr * gr;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - step * (mi / (sqrtf(vi) / bc2_sqrt + eps));
  w[i] = wi;
  bf_copy(copies, i, wi);
}

// The BF16 copies of the whole parameter vector's matrices, without an update.
__global__ void publish_kernel(const float *w, long long n, const BfCopies copies) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) bf_copy(copies, i, w[i]);
}

} // namespace bude
