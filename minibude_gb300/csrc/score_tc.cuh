// score_tc.cuh -- surrogate inference on the 5th-generation tensor cores (tcgen05 + TMEM).
//
// The scorer computes in FP16 (weights, features and activations; FP32 accumulators and output
// layer): FP16's packed FMA has the saturation the activation needs (mlp.cuh act_pair_f16), one
// instruction per pair fewer than BF16 on the epilogue's critical path, and its 11 significant bits
// put the scores closer to the FP32 network than the BF16 training pass.  The training forward
// pass below runs the same chain in BF16.
//
// A block runs G independent tile groups of 128 threads (G = 4 for scoring alone; G = 3 leaves
// shared memory and registers on each SM for exact-kernel blocks, which the screening pipeline
// runs beside it).  A group scores one item at a
// time: up to 128 poses of one ligand, pose r = thread r = TMEM lane r of the group's 128 TMEM
// columns.  For every ligand atom the group
//   1. builds each pose's 32 features (the type embedding, and surrogate_kernels.cuh:
//      field_features, whose field channels come from the texture unit) into its `act` tile, in
//      the K-major core-matrix layout (tc.cuh); the field features of the next atom are fetched
//      while this atom's layer-3 UMMA runs;
//   2. runs layers 1..3 as UMMAs issued by the group's first thread: D[128 x 128] = 1 * B_l^T
//      (the bias) + act * W_l^T over K = 32, 128, 128, FP32 accumulators in TMEM, completion
//      signalled through the group's mbarrier;
//   3. after each layer loads its row of D (= z) from TMEM (tc.cuh tmem_rows128: 16 columns at a
//      time, the next chunk's load in flight), applies the activation (mlp.cuh: act_pair_f16)
//      and writes the FP16 row back into `act` as the next layer's input;
//   4. computes the output layer on the FMA pipe from the layer-3 accumulators: h3 (in FP32:
//      mlp.cuh act_f2) . w4, added to the pose's energy.  (An N = 16 UMMA for it spent a fifth of
//      the tensor time on 1% of the FLOPs and a fourth UMMA round trip per atom; measured 251 M
//      poses/s with it, 257 M without.)
// The bias enters as a K = 16 UMMA of a tile of ones against b_l split into three 16-bit parts
// (k = 0, 1, 2), so no FP32 add is left in the epilogue.  The groups of a block share the weights in
// shared memory and interleave, so one group's epilogue overlaps another's MMAs.  Every mbarrier
// wait is bounded; a wait that runs out sets bit 0 of the error word, the group leaves at its next
// vote, and the block releases its TMEM.
#pragma once
#include <cstddef>

#include "surrogate_kernels.cuh"
#include "tc.cuh"

namespace bude {

constexpr int kTcGroups = 4;         // tile groups per block when the scorer runs alone
constexpr int kTcGroupThreads = 128; // warp w of a group reads TMEM lanes 32w .. 32w + 31
constexpr int kTcCols = 128;         // TMEM columns per group
constexpr int kTcBiasK = 16;         // K of the bias UMMA (3 of 16 used)

template <int G> struct TcSmem {
  alignas(128) unsigned char w1[kHid * kFeat * 2];          // W1: [128 out][32 in], K-major
  alignas(128) unsigned char w2[kHid * kHid * 2];           // W2
  alignas(128) unsigned char w3[kHid * kHid * 2];           // W3
  alignas(128) unsigned char bias[3][kHid * kTcBiasK * 2];  // b_l in three 16-bit parts at k = 0..2
  alignas(128) unsigned char ones[kHid * kTcBiasK * 2];     // 1 at k = 0..2
  alignas(128) unsigned char act[G][kHid * kHid * 2];         // per group: the layer input tile
  alignas(16) float w4f[kHid];                               // output weights, FP32
  uint4 emb[kMaxTypes * 2];                                  // type embeddings (16 x 16 bits each)
  alignas(8) uint64_t bar[G];
  int item[G]; // per group: the tile it took from a work counter (training forward pass)
  uint32_t tmem;
};

static_assert(offsetof(TcSmem<4>, ones) + sizeof(TcSmem<4>::ones) - offsetof(TcSmem<4>, bias) ==
                  sizeof(TcSmem<4>::bias) + sizeof(TcSmem<4>::ones),
              "bias and ones tiles are contiguous (zeroed as one range)");
static_assert(sizeof(TcSmem<4>) <= 227 * 1024, "one block per SM fits the 227 KB shared-memory limit");
// Every variant keeps a second scorer block (and its TMEM allocation) off an SM.
static_assert(sizeof(TcSmem<3>) > 114 * 1024, "shared memory keeps a second scorer block off the SM");

// TMEM columns a block allocates: a power of two covering G groups of 128.
template <int G> __host__ __device__ constexpr int tc_alloc_cols() { return G * kTcCols <= 256 ? 256 : 512; }

// The weights a tcgen05 kernel stages: 16-bit matrices ([out][in]; BF16, or FP16 for the scorer)
// and the FP32 vectors.
struct TcWeights {
  const void *emb, *w1, *w2, *w3;
  const float *b1, *b2, *b3, *w4, *b4;
};
__host__ __device__ inline TcWeights tc_weights(const MlpWeights &W) {
  return TcWeights{W.emb, W.w1, W.w2, W.w3, W.b1, W.b2, W.b3, W.w4, W.b4};
}

struct ScoreTcArgs {
  ScoreArgs s;   // s.W unused: the scorer reads the FP16 copies in w
  TcWeights w;   // FP16 matrices and embeddings
  unsigned int *err;
  float w4[kHid]; // output weights as launch parameters: operands of the output layer's FMAs
                  // straight from the constant bank, no shared-memory loads
};

template <bool F16> __device__ __forceinline__ void st_16(unsigned char *tile, uint32_t off, float v) {
  if (F16) *reinterpret_cast<__half *>(tile + off) = __float2half_rn(v);
  else *reinterpret_cast<__nv_bfloat16 *>(tile + off) = __float2bfloat16_rn(v);
}
template <bool F16> __device__ __forceinline__ float round_16(float v) {
  return F16 ? __half2float(__float2half_rn(v)) : __bfloat162float(__float2bfloat16_rn(v));
}

// Copy a global [N][K] row-major 16-bit matrix into the K-major core-matrix layout.
__device__ __forceinline__ void to_kmajor(unsigned char *dst, const void *src, int n, int k) {
  const uint4 *s16 = reinterpret_cast<const uint4 *>(src);
  for (int i = threadIdx.x; i < n * k / 8; i += blockDim.x) {
    const int row = i / (k / 8), k8 = i % (k / 8);
    *reinterpret_cast<uint4 *>(dst + kmajor_offset(row, k8 * 8, k)) = __ldg(s16 + (long long)row * (k / 8) + k8);
  }
}

// The block's constant tiles: weights, bias tiles, the ones tile, output weights, embeddings, in
// BF16 or (F16) FP16.
template <bool F16, class Smem> __device__ __forceinline__ void tc_setup(Smem &s, const TcWeights &W) {
  const int tid = threadIdx.x;
  {
    uint4 *z = reinterpret_cast<uint4 *>(s.bias);
    const int n16 = (int)((sizeof s.bias + sizeof s.ones) / 16);
    for (int i = tid; i < n16; i += blockDim.x) z[i] = make_uint4(0, 0, 0, 0);
  }
  to_kmajor(s.w1, W.w1, kHid, kFeat);
  to_kmajor(s.w2, W.w2, kHid, kHid);
  to_kmajor(s.w3, W.w3, kHid, kHid);
  for (int i = tid; i < kMaxTypes * 2; i += blockDim.x) s.emb[i] = __ldg(reinterpret_cast<const uint4 *>(W.emb) + i);
  for (int i = tid; i < kHid; i += blockDim.x) s.w4f[i] = __ldg(&W.w4[i]);
  __syncthreads(); // zeroed tiles before their non-zero entries
  for (int i = tid; i < 3 * kHid; i += blockDim.x) {
    const int l = i / kHid, n = i % kHid;
    const float *b = l == 0 ? W.b1 : (l == 1 ? W.b2 : W.b3);
    const float v = __ldg(&b[n]);
    const float hi = round_16<F16>(v);
    const float mid = round_16<F16>(v - hi);
    st_16<F16>(s.bias[l], kmajor_offset(n, 0, kTcBiasK), hi);
    st_16<F16>(s.bias[l], kmajor_offset(n, 1, kTcBiasK), mid);
    st_16<F16>(s.bias[l], kmajor_offset(n, 2, kTcBiasK), v - hi - mid);
  }
  for (int m = tid; m < kHid; m += blockDim.x)
    for (int k = 0; k < 3; ++k) st_16<F16>(s.ones, kmajor_offset(m, k, kTcBiasK), 1.f);
}

template <int G>
__global__ void __launch_bounds__(G * kTcGroupThreads, 1) score_tc_kernel(const ScoreTcArgs A) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  TcSmem<G> &s = *reinterpret_cast<TcSmem<G> *>(smem_raw);
  const ScoreArgs &a = A.s;
  const int tid = threadIdx.x, g = tid / kTcGroupThreads, lt = tid % kTcGroupThreads;
  const uint32_t bar_id = 1 + g; // named barrier of the group

  tc_setup<true>(s, A.w);
  if (tid == 0) {
    for (int q = 0; q < G; ++q) mbar_init(&s.bar[q], 1);
    mbar_fence_init();
  }
  if (tid < 32) tmem_alloc<tc_alloc_cols<G>()>(&s.tmem);
  fence_proxy_async();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();

  const uint32_t tmem = s.tmem + (uint32_t)(g * kTcCols);
  const uint32_t lane_addr = tmem + ((uint32_t)((lt / 32) * 32) << 16);
  unsigned char *act = s.act[g];
  const uint32_t act_a = smem_u32(act), ones_a = smem_u32(s.ones);
  const uint32_t idesc = umma_idesc_f16(kHid, kHid);
  const float b4 = __ldg(A.w.b4);
  uint64_t *bar = &s.bar[g];
  uint32_t phase = 0;
  bool failed = false;

  // Hidden layer: D = ones * bias^T + act * W^T over kdim, issued by the group's first thread;
  // layer_wait waits for it.
  auto layer_issue = [&](uint32_t w, uint32_t bias, int kdim) {
    if (lt == 0) {
      tc_fence_after();
      const uint32_t sbo = (uint32_t)(kdim / 8) * 128u, bsbo = (kTcBiasK / 8) * 128u;
      umma_bf16(tmem, umma_desc(ones_a, 128u, bsbo), umma_desc(bias, 128u, bsbo), idesc, 0u);
      for (int kk = 0; kk < kdim / 16; ++kk)
        umma_bf16(tmem, umma_desc(act_a + kk * 256u, 128u, sbo), umma_desc(w + kk * 256u, 128u, sbo), idesc, 1u);
      umma_commit(bar);
    }
  };
  auto layer_wait = [&]() {
    if (!mbar_wait_sleep_bounded(bar, phase)) failed = true;
    phase ^= 1u;
    tc_fence_after();
  };
  auto hidden = [&](uint32_t w, uint32_t bias, int kdim) {
    layer_issue(w, bias, kdim);
    layer_wait();
  };
  // Activation of the group's D rows into act (K = 128 layout), then the group barrier.
  auto epilogue = [&]() {
    tmem_rows128(lane_addr, [&](int c, const uint32_t (&v)[16]) {
      uint32_t h[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) h[i] = act_pair_f16(__uint_as_float(v[2 * i]), __uint_as_float(v[2 * i + 1]));
#pragma unroll
      for (int q = 0; q < 2; ++q)
        *reinterpret_cast<uint4 *>(act + kmajor_offset(lt, c * 16 + q * 8, kHid)) =
            make_uint4(h[4 * q], h[4 * q + 1], h[4 * q + 2], h[4 * q + 3]);
    });
    fence_proxy_async();
    tc_fence_before();
    named_sync(bar_id, kTcGroupThreads);
  };

  for (int item = blockIdx.x * G + g; item < a.n_items; item += gridDim.x * G) {
    const int4 it = __ldg(&a.items[item]);
    const float4 *xf = a.xform + (long long)(it.z + min(lt, it.w - 1)) * 3;
    const float4 r0 = __ldg(xf), r1 = __ldg(xf + 1), r2 = __ldg(xf + 2);
    float e = 0.f;
    // Type and field features of the atom the next tile scores.  For every atom after the first
    // they are fetched while the previous atom's layer-3 UMMA runs, so the texture latency is off
    // the chain's critical path.
    int tn = 0;
    uint32_t fp[8];
    auto fetch = [&](int il) {
      const float4 la = __ldg(&a.ligands[it.x + il]);
      tn = __float_as_int(la.w);
      field_features<true>(a.g, la, r0, r1, r2, fp);
    };
    if (it.y > 0) fetch(0);
    for (int il = 0; il < it.y; ++il) {
      *reinterpret_cast<uint4 *>(act + kmajor_offset(lt, 0, kFeat)) = s.emb[2 * tn];
      *reinterpret_cast<uint4 *>(act + kmajor_offset(lt, 8, kFeat)) = s.emb[2 * tn + 1];
      *reinterpret_cast<uint4 *>(act + kmajor_offset(lt, 16, kFeat)) = make_uint4(fp[0], fp[1], fp[2], fp[3]);
      *reinterpret_cast<uint4 *>(act + kmajor_offset(lt, 24, kFeat)) = make_uint4(fp[4], fp[5], fp[6], fp[7]);
      fence_proxy_async();
      tc_fence_before();
      if (named_sync_or(bar_id, kTcGroupThreads, failed)) {
        failed = true;
        break;
      }
      hidden(smem_u32(s.w1), smem_u32(s.bias[0]), kFeat);
      epilogue();
      hidden(smem_u32(s.w2), smem_u32(s.bias[1]), kHid);
      epilogue();
      layer_issue(smem_u32(s.w3), smem_u32(s.bias[2]), kHid);
      if (il + 1 < it.y) {
        fetch(il + 1);
        // The fetched values are complete before the wait below (no reordering past it).
        asm volatile("" ::"r"(fp[0]), "r"(fp[1]), "r"(fp[2]), "r"(fp[3]), "r"(fp[4]), "r"(fp[5]), "r"(fp[6]),
                     "r"(fp[7]), "r"(tn));
      }
      layer_wait();
      // Output layer on the FMA pipe: h3 (FP32) . w4 straight from the layer-3 accumulators (two
      // FP32 partial sums, even and odd features).
      float2 acc = make_float2(0.f, 0.f);
      tmem_rows128(lane_addr, [&](int c, const uint32_t (&v)[16]) {
#pragma unroll
        for (int i = 0; i < 8; ++i)
          acc = fma2(act_f2(__uint_as_float(v[2 * i]), __uint_as_float(v[2 * i + 1])),
                     make_float2(A.w4[c * 16 + 2 * i], A.w4[c * 16 + 2 * i + 1]), acc);
      });
      e += acc.x + acc.y;
      tc_fence_before(); // the next atom's barrier orders these TMEM reads before the next UMMA
    }
    // Group-uniform exit: every thread of the group leaves together.
    if (named_sync_or(bar_id, kTcGroupThreads, failed)) {
      failed = true;
      break;
    }
    if (lt < it.w) a.scores[it.z + lt] = e + (float)it.y * b4;
  }
  if (failed) {
    atomicOr(A.err, 1u);
    if (lt == 0) (void)mbar_wait_bounded(bar, phase ^ 1u); // an outstanding UMMA completes before TMEM goes
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (tid < 32) tmem_dealloc<tc_alloc_cols<G>()>(s.tmem);
}

// ---------------------------------------------------------------------------------------------
// Training forward pass on the same machinery: 128-row tiles of the step's (pose, ligand atom)
// feature rows X instead of poses.  Per tile a group runs layers 1..3 as above and, after each,
// stores the row's pre-activations z_l as BF16 (row-tiled, tc.cuh: tiled_offset; the backward
// pass and the gradient kernel read them) before the activation goes back into `act`; the output layer gives y per row
// (w4 . h3, without b4: the loss kernel adds natlig * b4 per pose).  Tiles come from a work
// counter; a row's arithmetic does not depend on which group runs it.
struct TrainFwdTcArgs {
  MlpWeights W;
  const __nv_bfloat16 *X; // [rows][32], row-tiled
  int rows;
  __nv_bfloat16 *Z1, *Z2, *Z3; // [tiled_rows(rows)][128], row-tiled
  float *y;
  unsigned int *err;
  unsigned int *next; // work counter, zero at launch
};

__global__ void __launch_bounds__(kTcGroups * kTcGroupThreads, 1) train_forward_tc_kernel(const TrainFwdTcArgs A) {
  constexpr int G = kTcGroups;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  TcSmem<G> &s = *reinterpret_cast<TcSmem<G> *>(smem_raw);
  const int tid = threadIdx.x, g = tid / kTcGroupThreads, lt = tid % kTcGroupThreads;
  const uint32_t bar_id = 1 + g;

  if (tid == 0) {
    for (int q = 0; q < G; ++q) mbar_init(&s.bar[q], 1);
    mbar_fence_init();
  }
  if (tid < 32) tmem_alloc<tc_alloc_cols<G>()>(&s.tmem);
  grid_dep_wait(); // the setup above may overlap the features kernel; the weights and X come after
  tc_setup<false>(s, tc_weights(A.W));
  fence_proxy_async();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();

  const uint32_t tmem = s.tmem + (uint32_t)(g * kTcCols);
  const uint32_t lane_addr = tmem + ((uint32_t)((lt / 32) * 32) << 16);
  unsigned char *act = s.act[g];
  const uint32_t act_a = smem_u32(act), ones_a = smem_u32(s.ones);
  const uint32_t idesc = umma_idesc_bf16(kHid, kHid);
  uint64_t *bar = &s.bar[g];
  uint32_t phase = 0;
  bool failed = false;
  const int tiles = (A.rows + kTcGroupThreads - 1) / kTcGroupThreads;

  auto hidden = [&](uint32_t w, uint32_t bias, int kdim) {
    if (lt == 0) {
      tc_fence_after();
      const uint32_t sbo = (uint32_t)(kdim / 8) * 128u, bsbo = (kTcBiasK / 8) * 128u;
      umma_bf16(tmem, umma_desc(ones_a, 128u, bsbo), umma_desc(bias, 128u, bsbo), idesc, 0u);
      for (int kk = 0; kk < kdim / 16; ++kk)
        umma_bf16(tmem, umma_desc(act_a + kk * 256u, 128u, sbo), umma_desc(w + kk * 256u, 128u, sbo), idesc, 1u);
      umma_commit(bar);
    }
    if (!mbar_wait_sleep_bounded(bar, phase)) failed = true;
    phase ^= 1u;
    tc_fence_after();
  };
  // z (the accumulators) -> BF16 row of Z in global memory; act(z) -> the next layer's `act` tile,
  // or, after layer 3, w4 . act(z) -> y.
  auto epilogue = [&](__nv_bfloat16 *Z, long long row, bool valid, bool to_act, float *yout) {
    float2 acc = make_float2(0.f, 0.f);
    // Every row of the tile is stored (rows past the end hold the bias pre-activations: finite,
    // and their gradients are zero), so each warp store fills whole 128-byte lines.
    unsigned char *zt = reinterpret_cast<unsigned char *>(Z) + tiled_offset(row, 0, kHid);
    tmem_rows128(lane_addr, [&](int c, const uint32_t (&v)[16]) {
      uint32_t zb[8], hb[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const float z0 = __uint_as_float(v[2 * i]), z1 = __uint_as_float(v[2 * i + 1]);
        zb[i] = pack_bf16(z0, z1);
        if (to_act) hb[i] = act_pair(z0, z1);
      }
#pragma unroll
      for (int q = 0; q < 2; ++q)
        *reinterpret_cast<uint4 *>(zt + kmajor_offset(0, c * 16 + q * 8, kHid)) =
            make_uint4(zb[4 * q], zb[4 * q + 1], zb[4 * q + 2], zb[4 * q + 3]);
      if (to_act) {
#pragma unroll
        for (int q = 0; q < 2; ++q)
          *reinterpret_cast<uint4 *>(act + kmajor_offset(lt, c * 16 + q * 8, kHid)) =
              make_uint4(hb[4 * q], hb[4 * q + 1], hb[4 * q + 2], hb[4 * q + 3]);
      } else {
#pragma unroll
        for (int i = 0; i < 8; i += 2) {
          const float4 w = *reinterpret_cast<const float4 *>(&s.w4f[c * 16 + 2 * i]);
          acc = fma2(act_f2(__uint_as_float(v[2 * i]), __uint_as_float(v[2 * i + 1])), make_float2(w.x, w.y), acc);
          acc = fma2(act_f2(__uint_as_float(v[2 * i + 2]), __uint_as_float(v[2 * i + 3])), make_float2(w.z, w.w),
                     acc);
        }
      }
    });
    if (yout && valid) *yout = acc.x + acc.y;
    if (to_act) fence_proxy_async();
    tc_fence_before();
    named_sync(bar_id, kTcGroupThreads);
  };

  constexpr uint32_t kXTile = kTcGroupThreads * kFeat * 2;
  for (;;) {
    if (lt == 0) s.item[g] = (int)atomicAdd(A.next, 1u);
    named_sync(bar_id, kTcGroupThreads);
    const int tile = s.item[g]; // rewritten only after the group's end-of-tile barrier below
    if (tile >= tiles) break;
    const long long row = (long long)tile * kTcGroupThreads + lt;
    const bool valid = row < A.rows;
    // The feature tile is the layer-1 operand tile byte for byte; rows past the end are zero.
    const unsigned char *x = reinterpret_cast<const unsigned char *>(A.X) + (long long)tile * kXTile;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint32_t o = kmajor_offset(lt, q * 8, kFeat);
      *reinterpret_cast<uint4 *>(act + o) = valid ? __ldg(reinterpret_cast<const uint4 *>(x + o)) : make_uint4(0, 0, 0, 0);
    }
    fence_proxy_async();
    tc_fence_before();
    if (named_sync_or(bar_id, kTcGroupThreads, failed)) {
      failed = true;
      break;
    }
    hidden(smem_u32(s.w1), smem_u32(s.bias[0]), kFeat);
    epilogue(A.Z1, row, valid, true, nullptr);
    hidden(smem_u32(s.w2), smem_u32(s.bias[1]), kHid);
    epilogue(A.Z2, row, valid, true, nullptr);
    hidden(smem_u32(s.w3), smem_u32(s.bias[2]), kHid);
    epilogue(A.Z3, row, valid, false, A.y + row);
    if (named_sync_or(bar_id, kTcGroupThreads, failed)) {
      failed = true;
      break;
    }
  }
  if (failed) {
    atomicOr(A.err, 1u);
    if (lt == 0) (void)mbar_wait_bounded(bar, phase ^ 1u); // an outstanding UMMA completes before TMEM goes
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (tid < 32) tmem_dealloc<tc_alloc_cols<G>()>(s.tmem);
}

// ---------------------------------------------------------------------------------------------
// Training backward pass through the hidden layers on the same machinery, per 128-row tile:
//   dz3 = dy * w4 * act'(z3)                       (FMA pipe, from the stored z3 and dy)
//   dz2 = (dz3 W3) * act'(z2),  dz1 = (dz2 W2) * act'(z1)   (UMMAs against the transposed weight
//                                                   copies W3^T, W2^T, FP32 accumulators in TMEM)
// Each dz is rounded to BF16, stored (row-tiled, the gradient kernel of wgrad_tc.cuh reads them)
// and written into `act` as the next UMMA's A operand.  Rows past the end have dy = 0, so their
// dz are exactly zero.  The element-wise work runs on BF16 pairs (mlp.cuh act_grad_bf16x2,
// mul_bf16x2: the stored z are BF16 already), about half the instructions of the FP32 form on
// the groups' critical path.  The pass streams the pre-activations once, so a thread keeps its row's
// whole z_l (256 bytes) in registers: the 16 loads of a layer are in flight together, and those of
// z2 and z1 are issued while the UMMA before them runs.  Three groups per block leave each thread
// the registers for that (a fourth would cap it at 128).
constexpr int kBwdGroups = 3;

template <int G> struct TcBwdSmem {
  alignas(128) unsigned char w3t[kHid * kHid * 2]; // W3^T: [in 128][out 128], K-major (K = out)
  alignas(128) unsigned char w2t[kHid * kHid * 2]; // W2^T
  alignas(128) unsigned char act[G][kHid * kHid * 2];
  alignas(16) uint32_t w4h[kHid / 2]; // output weights as BF16 pairs
  alignas(8) uint64_t bar[G];
  int item[G];
  uint32_t tmem;
};
static_assert(sizeof(TcBwdSmem<kBwdGroups>) <= 227 * 1024, "one block per SM fits the 227 KB shared-memory limit");

struct TrainBwdTcArgs {
  const __nv_bfloat16 *w3t, *w2t; // [in][out] BF16 (the published transposed copies)
  const float *w4;
  const __nv_bfloat16 *Z1, *Z2, *Z3; // row-tiled, as the forward pass stored them
  const float *dy;                   // [rows]
  int rows;
  __nv_bfloat16 *dZ1, *dZ2, *dZ3;    // [tiled_rows(rows)][128], row-tiled
  unsigned int *err;
  unsigned int *next; // work counter, zero at launch
};

// Row `row`'s 128 BF16 values of a row-tiled [rows][128] array, as 16 chunks of 8 (all loads issued
// before any is used).
__device__ __forceinline__ void load_row128(const __nv_bfloat16 *src, long long row, uint4 (&v)[16]) {
  const unsigned char *t = reinterpret_cast<const unsigned char *>(src) + tiled_offset(row, 0, kHid);
#pragma unroll
  for (int q = 0; q < 16; ++q) v[q] = __ldg(reinterpret_cast<const uint4 *>(t + kmajor_offset(0, q * 8, kHid)));
}

__global__ void __launch_bounds__(kBwdGroups * kTcGroupThreads, 1) train_backward_tc_kernel(const TrainBwdTcArgs A) {
  constexpr int G = kBwdGroups;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  TcBwdSmem<G> &s = *reinterpret_cast<TcBwdSmem<G> *>(smem_raw);
  const int tid = threadIdx.x, g = tid / kTcGroupThreads, lt = tid % kTcGroupThreads;
  const uint32_t bar_id = 1 + g;

  if (tid == 0) {
    for (int q = 0; q < G; ++q) mbar_init(&s.bar[q], 1);
    mbar_fence_init();
  }
  if (tid < 32) tmem_alloc<tc_alloc_cols<G>()>(&s.tmem);
  grid_dep_wait(); // the setup above may overlap the loss kernel; everything below reads its inputs
  to_kmajor(s.w3t, A.w3t, kHid, kHid);
  to_kmajor(s.w2t, A.w2t, kHid, kHid);
  for (int i = tid; i < kHid / 2; i += blockDim.x) s.w4h[i] = pack_bf16(__ldg(&A.w4[2 * i]), __ldg(&A.w4[2 * i + 1]));
  fence_proxy_async();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();

  const uint32_t tmem = s.tmem + (uint32_t)(g * kTcCols);
  const uint32_t lane_addr = tmem + ((uint32_t)((lt / 32) * 32) << 16);
  unsigned char *act = s.act[g];
  const uint32_t act_a = smem_u32(act);
  const uint32_t idesc = umma_idesc_bf16(kHid, kHid);
  uint64_t *bar = &s.bar[g];
  uint32_t phase = 0;
  bool failed = false;
  const int tiles = (A.rows + kTcGroupThreads - 1) / kTcGroupThreads;

  // D = act * Wt^T over K = 128 (no bias), issued by the group's first thread once every thread's
  // part of `act` is written; product_wait waits for it.
  auto product_issue = [&](uint32_t wt) {
    fence_proxy_async();
    tc_fence_before();
    named_sync(bar_id, kTcGroupThreads);
    if (lt == 0) {
      tc_fence_after();
      constexpr uint32_t sbo = (kHid / 8) * 128u;
      for (int kk = 0; kk < kHid / 16; ++kk)
        umma_bf16(tmem, umma_desc(act_a + kk * 256u, 128u, sbo), umma_desc(wt + kk * 256u, 128u, sbo), idesc,
                  kk ? 1u : 0u);
      umma_commit(bar);
    }
  };
  auto product_wait = [&]() {
    if (!mbar_wait_sleep_bounded(bar, phase)) failed = true;
    phase ^= 1u;
    tc_fence_after();
  };
  // 16 dz values (BF16 pairs) of columns [c0, c0 + 32) -> the row of dZ in global memory and,
  // when to_act, the `act` tile.
  auto put = [&](__nv_bfloat16 *dZ, long long row, int c0, const uint32_t (&d)[16], bool to_act) {
    unsigned char *dt = reinterpret_cast<unsigned char *>(dZ) + tiled_offset(row, 0, kHid);
#pragma unroll
    for (int q = 0; q < 4; ++q)
      *reinterpret_cast<uint4 *>(dt + kmajor_offset(0, c0 + q * 8, kHid)) =
          make_uint4(d[4 * q], d[4 * q + 1], d[4 * q + 2], d[4 * q + 3]);
    if (to_act) {
#pragma unroll
      for (int q = 0; q < 4; ++q)
        *reinterpret_cast<uint4 *>(act + kmajor_offset(lt, c0 + q * 8, kHid)) =
            make_uint4(d[4 * q], d[4 * q + 1], d[4 * q + 2], d[4 * q + 3]);
    }
  };
  auto put16 = [&](__nv_bfloat16 *dZ, long long row, int c0, const uint32_t (&d)[8], bool to_act) {
    unsigned char *dt = reinterpret_cast<unsigned char *>(dZ) + tiled_offset(row, 0, kHid);
#pragma unroll
    for (int q = 0; q < 2; ++q)
      *reinterpret_cast<uint4 *>(dt + kmajor_offset(0, c0 + q * 8, kHid)) =
          make_uint4(d[4 * q], d[4 * q + 1], d[4 * q + 2], d[4 * q + 3]);
    if (to_act) {
#pragma unroll
      for (int q = 0; q < 2; ++q)
        *reinterpret_cast<uint4 *>(act + kmajor_offset(lt, c0 + q * 8, kHid)) =
            make_uint4(d[4 * q], d[4 * q + 1], d[4 * q + 2], d[4 * q + 3]);
    }
  };
  // dz = D (from TMEM) * act'(z) for the row's pre-activations z (in registers).
  auto through = [&](const uint4 (&z)[16], __nv_bfloat16 *dZ, long long row, bool to_act) {
    tmem_rows128(lane_addr, [&](int c, const uint32_t (&v)[16]) {
      const uint32_t *zw = reinterpret_cast<const uint32_t *>(&z[2 * c]);
      uint32_t d[8];
#pragma unroll
      for (int i = 0; i < 8; ++i)
        d[i] = mul_bf16x2(pack_bf16(__uint_as_float(v[2 * i]), __uint_as_float(v[2 * i + 1])),
                          act_grad_bf16x2(zw[i]));
      put16(dZ, row, c * 16, d, to_act);
    });
  };

  for (;;) {
    if (lt == 0) s.item[g] = (int)atomicAdd(A.next, 1u);
    named_sync(bar_id, kTcGroupThreads);
    const int tile = s.item[g]; // rewritten only after the group's end-of-tile barrier below
    if (tile >= tiles) break;
    const long long row = (long long)tile * kTcGroupThreads + lt;
    const bool valid = row < A.rows;
    uint4 z[16];
    const float dy = valid ? A.dy[row] : 0.f;
    const uint32_t dy2 = pack_bf16(dy, dy);
    load_row128(A.Z3, row, z);
    // dz3 = dy * w4 * act'(z3), in packed BF16 (w4 as BF16 pairs)
#pragma unroll
    for (int c = 0; c < kHid / 32; ++c) {
      const uint32_t *zw = reinterpret_cast<const uint32_t *>(&z[4 * c]);
      uint32_t d[16];
#pragma unroll
      for (int i = 0; i < 16; ++i) d[i] = mul_bf16x2(mul_bf16x2(dy2, s.w4h[c * 16 + i]), act_grad_bf16x2(zw[i]));
      put(A.dZ3, row, c * 32, d, true);
    }
    product_issue(smem_u32(s.w3t));
    load_row128(A.Z2, row, z); // in flight while the UMMA runs
    product_wait();
    through(z, A.dZ2, row, true);
    product_issue(smem_u32(s.w2t));
    load_row128(A.Z1, row, z);
    product_wait();
    through(z, A.dZ1, row, false);
    tc_fence_before();
    if (named_sync_or(bar_id, kTcGroupThreads, failed)) {
      failed = true;
      break;
    }
  }
  if (failed) {
    atomicOr(A.err, 1u);
    if (lt == 0) (void)mbar_wait_bounded(bar, phase ^ 1u); // an outstanding UMMA completes before TMEM goes
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (tid < 32) tmem_dealloc<tc_alloc_cols<G>()>(s.tmem);
}

} // namespace bude
