// wgrad_tc.cuh -- the surrogate's weight, bias and embedding gradients of one training step on the
// 5th-generation tensor cores.
//
// Every gradient of a weight or bias reduces over the step's rows (the (pose, ligand atom) rows of
// the batch):
//   dW3 = dZ3^T H2,  db3 = dZ3^T 1,   dW2 = dZ2^T H1,  db2 = dZ2^T 1,
//   dW1 = dZ1^T X,   db1 = dZ1^T 1,   S = dZ1^T T  (T = one-hot of each row's atom type),
//   dw4 = H3^T dy,
// with H_l = act(Z_l) rebuilt from the stored BF16 pre-activations (mlp.cuh act_bf16x2).  Each is one UMMA chain with the
// rows as K: D[M = 128][N] += A[M][K = 16 rows] * B[N][K = 16 rows]^T, the operands staged in
// shared memory in the MN-major core-matrix layout (M or N contiguous: a row's features go in as
// 16-byte stores), the accumulators held in TMEM for the whole launch:
//   columns   0..143  dW3 | db3 (N = 128 + a ones column + 15 zero columns)
//           144..287  dW2 | db2
//           288..399  dW1 | S | db1 (N = 32 + 64 + 16)
//           400..415  dw4 (N = 16: dy as two BF16 parts, hi + lo, and 14 zero columns)
// The embedding gradient follows as dEmb[t][j] = sum_f W1[f][j] S[f][t] (emb_grad_kernel).
//
// A block owns a contiguous range of 128-row tiles (the same on every run), so the partial sums
// and their fixed-order reduction over blocks (reduce_segments_kernel) are deterministic.  Per
// tile, phase A stages and issues layers 3 and 2, phase B layer 1 and the output weights, both in
// one 136 KB region; a phase's UMMAs complete (bounded mbarrier wait) before the region is reused,
// and the next phase's global loads are in flight while they run.
#pragma once
#include <cstdint>

#include "surrogate_kernels.cuh"
#include "tc.cuh"

namespace bude {

constexpr int kWgTile = 128;     // rows per tile: K of 8 UMMAs
constexpr int kWgThreads = 256;  // two threads per row when staging
constexpr int kWgN3 = kHid + 16; // N of the layer-3 and layer-2 chains (features | ones | zeros)
constexpr int kWgN1 = kFeat + kMaxTypes + 16; // N of the layer-1 chain (X | one-hot | ones | zeros)
constexpr int kWgN4 = 16;        // N of the output-weight chain (dy hi | dy lo | zeros)
constexpr int kWgCol3 = 0, kWgCol2 = kWgN3, kWgCol1 = 2 * kWgN3, kWgCol4 = 2 * kWgN3 + kWgN1;
constexpr int kWgCols = kWgCol4 + kWgN4; // 416 TMEM columns used of the 512 allocated
// Partial sums per block, floats: [dW3 128x128 | db3 128 | dW2 | db2 | dW1 128x32 | S 128x64 | db1 | dw4]
constexpr int kWgOffW3 = 0, kWgOffB3 = kWgOffW3 + kHid * kHid, kWgOffW2 = kWgOffB3 + kHid,
              kWgOffB2 = kWgOffW2 + kHid * kHid, kWgOffW1 = kWgOffB2 + kHid, kWgOffS = kWgOffW1 + kHid * kFeat,
              kWgOffB1 = kWgOffS + kHid * kMaxTypes, kWgOffW4 = kWgOffB1 + kHid, kWgPart = kWgOffW4 + kHid;

// MN-major, unswizzled tile of [mn][K = 128 rows]: core matrices of 8 rows (K) x 16 bytes (8 MN
// values) stored as 128 contiguous bytes, MN-adjacent core matrices 128 bytes apart (the
// descriptor's stride byte offset), the 8-row groups (MN / 8) * 128 bytes apart (its leading byte
// offset).  Element (mn, k) of a tile of `nmn` values along MN.
__host__ __device__ __forceinline__ uint32_t mnmajor_offset(int mn, int k, int nmn) {
  return (uint32_t)((mn >> 3) * 128 + (k >> 3) * (nmn / 8) * 128 + (k & 7) * 16 + (mn & 7) * 2);
}
constexpr uint32_t wg_tile_bytes(int nmn) { return (uint32_t)nmn * kWgTile * 2; }

// Phase A: A3 = dZ3 [128], B3 = H2|1 [144], A2 = dZ2 [128], B2 = H1|1 [144].
// Phase B: A1 = dZ1 [128], B1 = X|T|1 [112], A4 = H3 [128], B4 = dy [16].
constexpr uint32_t kWgA3 = 0, kWgB3 = kWgA3 + wg_tile_bytes(kHid), kWgA2 = kWgB3 + wg_tile_bytes(kWgN3),
                   kWgB2 = kWgA2 + wg_tile_bytes(kHid), kWgPhaseA = kWgB2 + wg_tile_bytes(kWgN3);
constexpr uint32_t kWgA1 = 0, kWgB1 = kWgA1 + wg_tile_bytes(kHid), kWgA4 = kWgB1 + wg_tile_bytes(kWgN1),
                   kWgB4 = kWgA4 + wg_tile_bytes(kHid), kWgPhaseB = kWgB4 + wg_tile_bytes(kWgN4);
constexpr uint32_t kWgRegion = kWgPhaseA > kWgPhaseB ? kWgPhaseA : kWgPhaseB;

struct WgTcSmem {
  alignas(128) unsigned char region[kWgRegion];
  alignas(8) uint64_t bar;
  uint32_t tmem;
};
static_assert(sizeof(WgTcSmem) <= 227 * 1024, "the staging region fits one block per SM");

struct WgTcArgs {
  const __nv_bfloat16 *X;                // [rows][32], row-tiled (tc.cuh: tiled_offset)
  const int *row_type;                   // [rows]
  const __nv_bfloat16 *Z1, *Z2, *Z3;     // [tiled_rows(rows)][128] pre-activations, row-tiled
  const __nv_bfloat16 *dZ1, *dZ2, *dZ3;  // [tiled_rows(rows)][128], row-tiled; zero past the end
  const float *dy;                       // [rows] (dy and row_type allocated for tiled_rows(rows))
  int rows;
  float *part;                           // [gridDim.x][kWgPart]
  unsigned int *err;                     // bit 0: a bounded wait ran out
};

// 8 BF16 values as a 16-byte chunk of one row into an MN-major tile (features f0..f0+7 of row k).
__device__ __forceinline__ void wg_put(unsigned char *tile, int nmn, int f0, int k, uint4 v) {
  *reinterpret_cast<uint4 *>(tile + mnmajor_offset(f0, k, nmn)) = v;
}

// The 64 features [h*64, h*64+64) of row r of a row-tiled [rows][128] BF16 array (every row of a
// tile is written: rows past the end have zero gradients and finite pre-activations).
__device__ __forceinline__ void wg_load_half(const __nv_bfloat16 *src, long long r, int h, uint4 (&v)[8]) {
  const unsigned char *t = reinterpret_cast<const unsigned char *>(src) + tiled_offset(r, 0, kHid);
#pragma unroll
  for (int q = 0; q < 8; ++q) v[q] = __ldg(reinterpret_cast<const uint4 *>(t + kmajor_offset(0, h * 64 + q * 8, kHid)));
}

// Store them as row k of an MN-major tile, optionally through the activation (BF16 in, BF16 out).
__device__ __forceinline__ void wg_store_half(unsigned char *tile, int nmn, int h, int k, uint4 (&v)[8],
                                              bool apply_act) {
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    if (apply_act) {
      uint32_t *w = reinterpret_cast<uint32_t *>(&v[q]);
#pragma unroll
      for (int e = 0; e < 4; ++e) w[e] = act_bf16x2(w[e]); // act(0) = 0: rows past the end stay zero
    }
    *reinterpret_cast<uint4 *>(tile + mnmajor_offset(h * 64 + q * 8, k, nmn)) = v[q];
  }
}

// Instruction descriptor: M = 128, N = n, A and B MN-major (bits 15 and 16).
__device__ __forceinline__ uint32_t wg_idesc(int n) {
  return umma_idesc_bf16(kHid, n) | (1u << 15) | (1u << 16);
}

__global__ void __launch_bounds__(kWgThreads, 1) wgrad_tc_kernel(const WgTcArgs a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  WgTcSmem &s = *reinterpret_cast<WgTcSmem *>(smem_raw);
  const int tid = threadIdx.x, r = tid % kWgTile, h = tid / kWgTile; // row of the tile, half
  const int tiles = (a.rows + kWgTile - 1) / kWgTile;
  const int t0 = (int)((long long)tiles * blockIdx.x / gridDim.x);
  const int t1 = (int)((long long)tiles * (blockIdx.x + 1) / gridDim.x);

  if (tid == 0) {
    mbar_init(&s.bar, 1);
    mbar_fence_init();
  }
  if (tid < 32) tmem_alloc<512>(&s.tmem);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  grid_dep_wait(); // the setup above may overlap the backward pass; its outputs are read below
  const uint32_t tmem = s.tmem;
  unsigned char *R = s.region;
  const uint32_t base = smem_u32(R);
  uint32_t phase = 0;
  bool failed = false;
  const uint4 one_first = make_uint4(0x3F80u, 0u, 0u, 0u); // BF16 1.0 in the chunk's first value

  // One UMMA chain over the tile's 128 rows: D[col] += A^T-tile x B^T-tile, 8 K = 16 steps.
  auto chain = [&](uint32_t a_off, uint32_t b_off, int nb, uint32_t col, bool first) {
    const uint32_t a_lbo = (kHid / 8) * 128u, b_lbo = (uint32_t)(nb / 8) * 128u;
    for (int kk = 0; kk < kWgTile / 16; ++kk)
      umma_bf16(tmem + col, umma_desc(base + a_off + kk * 2 * a_lbo, a_lbo, 128u),
                umma_desc(base + b_off + kk * 2 * b_lbo, b_lbo, 128u), wg_idesc(nb), (first && kk == 0) ? 0u : 1u);
  };
  // A phase's tiles are complete in shared memory: one thread issues its UMMAs and commits them.
  auto issue = [&](bool phase_a, bool first) {
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      if (phase_a) {
        chain(kWgA3, kWgB3, kWgN3, kWgCol3, first);
        chain(kWgA2, kWgB2, kWgN3, kWgCol2, first);
      } else {
        chain(kWgA1, kWgB1, kWgN1, kWgCol1, first);
        chain(kWgA4, kWgB4, kWgN4, kWgCol4, first);
      }
      umma_commit(&s.bar);
    }
  };
  // The phase's UMMAs have read the region (bounded wait), so it may be rewritten.
  auto wait = [&]() {
    if (!mbar_wait_bounded(&s.bar, phase)) failed = true;
    phase ^= 1u;
    tc_fence_after();
  };

  // Phase A's loads for a tile (all 32 16-byte loads in flight at once), then per tile: store A,
  // issue A's UMMAs, load phase B while they run, store B once they are done, issue B's UMMAs,
  // load the next tile's phase A while those run.
  uint4 ad3[8], az2[8], ad2[8], az1[8];
  auto load_a = [&](int tile) {
    const long long row = (long long)tile * kWgTile + r;
    wg_load_half(a.dZ3, row, h, ad3);
    wg_load_half(a.Z2, row, h, az2);
    wg_load_half(a.dZ2, row, h, ad2);
    wg_load_half(a.Z1, row, h, az1);
  };
  // The next tile's rows are prefetched into L2 while this one is staged and multiplied.
  auto prefetch = [&](int tile) {
    constexpr uint32_t kZ = kWgTile * kHid * 2, kX = kWgTile * kFeat * 2;
    for (const __nv_bfloat16 *z : {a.dZ3, a.Z2, a.dZ2, a.Z1, a.dZ1, a.Z3})
      prefetch_l2(reinterpret_cast<const unsigned char *>(z) + (long long)tile * kZ, kZ);
    prefetch_l2(reinterpret_cast<const unsigned char *>(a.X) + (long long)tile * kX, kX);
    prefetch_l2(a.dy + (long long)tile * kWgTile, kWgTile * 4);
    prefetch_l2(a.row_type + (long long)tile * kWgTile, kWgTile * 4);
  };
  if (t0 < t1) load_a(t0);
  for (int tile = t0; tile < t1; ++tile) {
    const long long row = (long long)tile * kWgTile + r;
    const bool valid = row < a.rows;
    const bool first = tile == t0;
    if (tid == 0 && tile + 1 < t1) prefetch(tile + 1);
    // Phase A: layers 3 and 2.
    wg_store_half(R + kWgA3, kHid, h, r, ad3, false);
    wg_store_half(R + kWgB3, kWgN3, h, r, az2, true);
    wg_store_half(R + kWgA2, kHid, h, r, ad2, false);
    wg_store_half(R + kWgB2, kWgN3, h, r, az1, true);
    {
      // The bias column (a one per valid row) and 15 zero columns of both B tiles.
      const uint4 ones = (h == 0 && valid) ? one_first : make_uint4(0, 0, 0, 0);
      wg_put(R + kWgB3, kWgN3, kHid + h * 8, r, ones);
      wg_put(R + kWgB2, kWgN3, kHid + h * 8, r, ones);
    }
    issue(true, first);
    // Phase B's loads while phase A's UMMAs run.
    uint4 bd1[8], bz3[8], bx[4] = {};
    int type = -1;
    float d = 0.f;
    wg_load_half(a.dZ1, row, h, bd1);
    wg_load_half(a.Z3, row, h, bz3);
    if (valid) {
      if (h == 0) {
        const unsigned char *xt = reinterpret_cast<const unsigned char *>(a.X) + tiled_offset(row, 0, kFeat);
#pragma unroll
        for (int q = 0; q < 4; ++q) bx[q] = __ldg(reinterpret_cast<const uint4 *>(xt + kmajor_offset(0, q * 8, kFeat)));
        d = a.dy[row];
      } else {
        type = a.row_type[row];
      }
    }
    wait();
    if (__syncthreads_or(failed)) break;
    // Phase B: layer 1 (with the one-hot types and the bias column) and the output weights.
    wg_store_half(R + kWgA1, kHid, h, r, bd1, false);
    wg_store_half(R + kWgA4, kHid, h, r, bz3, true);
    if (h == 0) {
      // X (32 features), the bias column chunk, and dy as two BF16 parts
#pragma unroll
      for (int q = 0; q < 4; ++q) wg_put(R + kWgB1, kWgN1, q * 8, r, bx[q]);
      wg_put(R + kWgB1, kWgN1, kFeat + kMaxTypes, r, valid ? one_first : make_uint4(0, 0, 0, 0));
      const __nv_bfloat16 hi = __float2bfloat16_rn(d);
      const __nv_bfloat16 lo = __float2bfloat16_rn(d - __bfloat162float(hi));
      const uint32_t db = (uint32_t)__bfloat16_as_ushort(hi) | ((uint32_t)__bfloat16_as_ushort(lo) << 16);
      wg_put(R + kWgB4, kWgN4, 0, r, make_uint4(db, 0u, 0u, 0u));
    } else {
      // one-hot of the row's type (8 chunks) and the zero chunks
#pragma unroll
      for (int q = 0; q < kMaxTypes / 8; ++q) {
        uint4 c = make_uint4(0, 0, 0, 0);
        if (type >= q * 8 && type < q * 8 + 8) {
          uint32_t *w = reinterpret_cast<uint32_t *>(&c);
          w[(type - q * 8) >> 1] = ((type - q * 8) & 1) ? 0x3F800000u : 0x3F80u;
        }
        wg_put(R + kWgB1, kWgN1, kFeat + q * 8, r, c);
      }
      wg_put(R + kWgB1, kWgN1, kFeat + kMaxTypes + 8, r, make_uint4(0, 0, 0, 0));
      wg_put(R + kWgB4, kWgN4, 8, r, make_uint4(0, 0, 0, 0));
    }
    issue(false, first);
    if (tile + 1 < t1) load_a(tile + 1);
    wait();
    if (__syncthreads_or(failed)) break;
  }

  if (failed) {
    if (tid == 0) atomicOr(a.err, 1u);
  } else if (t0 < t1) {
    // Accumulators -> this block's partial sums.  Warp w reads TMEM lanes 32 (w % 4) .. + 31 (the
    // M rows: out-features, or H3 features for dw4), warps 0-3 the first half of the columns.
    const int w = tid / 32, lane = tid % 32, m = (w % 4) * 32 + lane;
    const uint32_t lane_addr = tmem + ((uint32_t)((w % 4) * 32) << 16);
    float *p = a.part + (long long)blockIdx.x * kWgPart;
    const int c0 = (w / 4) * (kWgCols / 2), c1 = c0 + kWgCols / 2; // 208 columns per half
    for (int c = c0; c < c1; c += 16) {
      uint32_t v[16];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(lane_addr + (uint32_t)c)
          : "memory");
      tmem_wait_ld();
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int col = c + j;
        const float x = __uint_as_float(v[j]);
        if (col < kWgCol2) { // dW3 | db3
          if (col < kHid) p[kWgOffW3 + m * kHid + col] = x;
          else if (col == kHid) p[kWgOffB3 + m] = x;
        } else if (col < kWgCol1) { // dW2 | db2
          const int cc = col - kWgCol2;
          if (cc < kHid) p[kWgOffW2 + m * kHid + cc] = x;
          else if (cc == kHid) p[kWgOffB2 + m] = x;
        } else if (col < kWgCol4) { // dW1 | S | db1
          const int cc = col - kWgCol1;
          if (cc < kFeat) p[kWgOffW1 + m * kFeat + cc] = x;
          else if (cc < kFeat + kMaxTypes) p[kWgOffS + m * kMaxTypes + (cc - kFeat)] = x;
          else if (cc == kFeat + kMaxTypes) p[kWgOffB1 + m] = x;
        } else if (col == kWgCol4) { // dw4: the hi part's column, then the lo part's
          p[kWgOffW4 + m] = x;
        } else if (col == kWgCol4 + 1) {
          p[kWgOffW4 + m] += x;
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (tid < 32) tmem_dealloc<512>(tmem);
}

// dEmb[t][j] = sum_f W1[f][j] S[f][t] (W1 as the forward pass used it: BF16), for the 64 x 16
// embedding entries; S summed over blocks already.  One warp per entry: lane l takes f = l, l + 32,
// ..., and the lanes' sums are folded by a fixed butterfly, so the result is the same on every run.
__global__ void emb_grad_kernel(const float *S, const __nv_bfloat16 *w1, float *demb) {
  grid_dep_wait();
  const int i = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = (int)(threadIdx.x & 31);
  if (i >= kMaxTypes * kEmb) return;
  const int t = i / kEmb, j = i % kEmb;
  float acc = 0.f;
#pragma unroll
  for (int f = lane; f < kHid; f += 32) acc = fmaf(__bfloat162float(w1[f * kFeat + j]), S[f * kMaxTypes + t], acc);
#pragma unroll
  for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xFFFFFFFFu, acc, o);
  if (lane == 0) demb[i] = acc;
}

} // namespace bude
