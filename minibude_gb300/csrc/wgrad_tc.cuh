// wgrad_tc.cuh -- the surrogate's weight, bias and embedding gradients of one training step on the
// 5th-generation tensor cores.
//
// Every gradient of a weight or bias reduces over the step's rows (the (pose, ligand atom) rows of
// the batch):
//   dW3 = dZ3^T H2,  db3 = dZ3^T 1,   dW2 = dZ2^T H1,  db2 = dZ2^T 1,
//   dW1 = dZ1^T X,   db1 = dZ1^T 1,   S = dZ1^T T  (T = one-hot of each row's atom type),
//   dw4 = H3^T dy,
// with H_l = act(Z_l) rebuilt from the stored BF16 pre-activations (mlp.cuh act_bf16x2).  Each is
// one UMMA chain with the rows as K: D[M = 128][N] += A[M][K = 16 rows] * B[N][K = 16 rows]^T, the
// operands in shared memory in the MN-major core-matrix layout, the accumulators held in TMEM for
// the whole launch:
//   columns   0..127  dW3          128..255  dW2          256..351  dW1 | S (N = 32 + 64)
//           352..367  dw4 (N = 16: dy as two BF16 parts, hi + lo, and 14 zero columns)
//           368..383  db3, 384..399 db2, 400..415 db1 (dZ_l^T against a tile of ones, N = 16)
// The embedding gradient follows as dEmb[t][j] = sum_f W1[f][j] S[f][t] (emb_grad_kernel).
//
// A 128-row tile of a row-tiled [rows][128] array (tc.cuh: tiled_offset) is byte for byte the
// MN-major operand tile of these UMMAs, so the dZ and Z tiles reach shared memory as single 32 KB
// TMA bulk copies, without registers.  Shared memory holds one slot per chain (224 KB in all):
//   slot 3: dZ3 | Z2 -> H2     slot 2: dZ2 | Z1 -> H1     slot 1: dZ1 | X, T (built by threads)
//   slot 4: Z3 -> H3 | dy (built by threads)               and the constant tile of ones.
// The block is warp-specialised, three roles meeting on three barriers per slot:
//   * eight worker warps take the chains of each tile in the order 3, 2, 1, 4: wait for the
//     slot's copies ("full"), rebuild H in place (act) or write the thread-built operand, and
//     arrive on the slot's "ready" barrier;
//   * the issuer (thread 0 of warp 8) waits for "ready", issues the chain's UMMAs and commits them
//     to the slot's "empty" barrier;
//   * the loader (thread 0 of warp 9) waits for "empty" and refills the slot with its next tile.
// Every wait is bounded; one that runs out raises a shared abort flag and every role leaves.
//
// A block owns a contiguous range of 128-row tiles (the same on every run), so the partial sums
// and their fixed-order reduction over blocks (reduce_segments_kernel) are deterministic.  The
// partial sums are stored column by column (coalesced), and the reduction writes each matrix back
// row-major.
#pragma once
#include <cstdint>

#include "surrogate_kernels.cuh"
#include "tc.cuh"

namespace bude {

constexpr int kWgTile = 128;    // rows per tile: K of 8 UMMAs
constexpr int kWgThreads = 256; // worker threads: two per row for the thread-built operands
constexpr int kWgN1 = kFeat + kMaxTypes; // N of the layer-1 chain (X | one-hot)
constexpr int kWgNb = 16;                // N of the output-weight and bias chains
constexpr int kWgCol3 = 0, kWgCol2 = kHid, kWgCol1 = 2 * kHid, kWgCol4 = kWgCol1 + kWgN1,
              kWgColB3 = kWgCol4 + kWgNb, kWgColB2 = kWgColB3 + kWgNb, kWgColB1 = kWgColB2 + kWgNb;
constexpr int kWgCols = kWgColB1 + kWgNb; // 416 TMEM columns used of the 512 allocated
// Partial sums per block, floats: [dW3 | db3 128 | dW2 | db2 | dW1 | S | db1 | dw4], the matrices
// column by column (element [out][in] at in * 128 + out: a warp's 32 lanes, 32 consecutive out
// rows of one TMEM column, store 128 contiguous bytes); the reduction writes them back row-major.
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
static_assert(wg_tile_bytes(kHid) == 128 * kHid * 2, "a [rows][128] tile is one operand tile");

constexpr int kWgChains = 4; // in processing order: layer 3, layer 2, layer 1, output weights
constexpr int kWgCopies = 1; // bulk copies per 32 KB array tile
constexpr uint32_t kWgZ = wg_tile_bytes(kHid); // 32 KB
constexpr uint32_t kWgSlot3 = 0, kWgSlot2 = kWgSlot3 + 2 * kWgZ, kWgSlot1 = kWgSlot2 + 2 * kWgZ,
                   kWgSlot4 = kWgSlot1 + kWgZ + wg_tile_bytes(kWgN1), kWgOnes = kWgSlot4 + kWgZ + wg_tile_bytes(kWgNb),
                   kWgRegion = kWgOnes + wg_tile_bytes(kWgNb);

struct WgTcSmem {
  alignas(128) unsigned char region[kWgRegion];
  alignas(8) uint64_t full[kWgChains];  // a slot's copies have landed (transaction bytes)
  alignas(8) uint64_t ready[kWgChains]; // the workers have built the slot's operands (256 arrivals)
  alignas(8) uint64_t empty[kWgChains]; // a slot's UMMAs have completed (tcgen05.commit)
  uint32_t tmem;
  int abort;                            // set when a wait ran out: everyone leaves
};
static_assert(sizeof(WgTcSmem) <= 227 * 1024, "the slots fit one block per SM");

struct WgTcArgs {
  const __nv_bfloat16 *X;                // [rows][32], row-tiled (tc.cuh: tiled_offset)
  const int *row_type;                   // [rows]
  const __nv_bfloat16 *Z1, *Z2, *Z3;     // [tiled_rows(rows)][128] pre-activations, row-tiled; every
                                         // row of a tile finite (rows past the end: the biases)
  const __nv_bfloat16 *dZ1, *dZ2, *dZ3;  // [tiled_rows(rows)][128], row-tiled; zero past the end
  const float *dy;                       // [rows] (dy and row_type allocated for tiled_rows(rows))
  int rows;
  float *part;                           // [gridDim.x][kWgPart]
  unsigned int *err;                     // bit 0: a bounded wait ran out
};

// 16-byte shared-memory load and store by shared-window address (ld/st.shared: the accesses
// stay on the shared-memory path instead of the generic load/store queue).
__device__ __forceinline__ uint4 lds128(uint32_t addr) {
  uint4 v;
  asm volatile("ld.shared.v4.u32 {%0, %1, %2, %3}, [%4];" : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "r"(addr));
  return v;
}
__device__ __forceinline__ void sts128(uint32_t addr, uint4 v) {
  asm volatile("st.shared.v4.u32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w)
               : "memory");
}

// 8 BF16 values as a 16-byte chunk of one row into an MN-major tile (features f0..f0+7 of row k);
// `tile` is a shared-window address.
__device__ __forceinline__ void wg_put(uint32_t tile, int nmn, int f0, int k, uint4 v) {
  sts128(tile + mnmajor_offset(f0, k, nmn), v);
}

// H = act(Z) in place over one 32 KB tile at shared-window address `tile`: 2,048 16-byte chunks,
// 8 per worker thread, all 8 loads in flight before the first store.
__device__ __forceinline__ void wg_act_tile(uint32_t tile) {
  uint4 v[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = lds128(tile + (uint32_t)(threadIdx.x + i * kWgThreads) * 16u);
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    v[i].x = act_bf16x2(v[i].x);
    v[i].y = act_bf16x2(v[i].y);
    v[i].z = act_bf16x2(v[i].z);
    v[i].w = act_bf16x2(v[i].w);
    sts128(tile + (uint32_t)(threadIdx.x + i * kWgThreads) * 16u, v[i]);
  }
}

// Instruction descriptor: M = 128, N = n, A and B MN-major (bits 15 and 16).
__device__ __forceinline__ uint32_t wg_idesc(int n) {
  return umma_idesc_bf16(kHid, n) | (1u << 15) | (1u << 16);
}

__global__ void __launch_bounds__(kWgThreads + 64, 1) wgrad_tc_kernel(const WgTcArgs a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  WgTcSmem &s = *reinterpret_cast<WgTcSmem *>(smem_raw);
  const int tid = threadIdx.x, r = tid % kWgTile, h = (tid / kWgTile) & 1; // worker: row of the tile, half
  // Warps 0-7: the workers (operand building); thread 0 of warp 8 issues the UMMAs, thread 0 of
  // warp 9 issues the slot copies.
  const bool worker = tid < kWgThreads, issuer = tid == kWgThreads, loader = tid == kWgThreads + 32;
  const int tiles = (a.rows + kWgTile - 1) / kWgTile;
  const int t0 = (int)((long long)tiles * blockIdx.x / gridDim.x);
  const int t1 = (int)((long long)tiles * (blockIdx.x + 1) / gridDim.x);
  unsigned char *R = s.region;

  if (tid == 0) {
    for (int j = 0; j < kWgChains; ++j) {
      mbar_init(&s.full[j], 1);
      mbar_init(&s.ready[j], kWgThreads);
      mbar_init(&s.empty[j], 1);
    }
    s.abort = 0;
    mbar_fence_init();
  }
  if (tid < 32) tmem_alloc<512>(&s.tmem);
  if (worker) {
    // The tile of ones for the bias chains: B[n][k] = 1 for n = 0, 0 for n = 1..15.
    const uint4 one_first = make_uint4(0x3F80u, 0u, 0u, 0u), zero = make_uint4(0u, 0u, 0u, 0u);
    wg_put(smem_u32(R) + kWgOnes, kWgNb, h * 8, r, h == 0 ? one_first : zero);
  }
  fence_proxy_async();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  grid_dep_wait(); // the setup above may overlap the backward pass; its outputs are read below
  const uint32_t tmem = s.tmem;
  const uint32_t base = smem_u32(R);
  bool failed = false;
  volatile int *abort_flag = &s.abort;

  // Thread 0 of warp 9 (the loader): one slot's copies of a tile, each 32 KB array tile as
  // kWgCopies bulk copies.
  auto load = [&](int j, int tile) {
    const long long off = (long long)tile * kWgZ;
    uint64_t *bar = &s.full[j];
    auto copy = [&](uint32_t dst, const __nv_bfloat16 *p) {
      const unsigned char *src = reinterpret_cast<const unsigned char *>(p) + off;
#pragma unroll
      for (int q = 0; q < kWgCopies; ++q)
        bulk_g2s(R + dst + q * (kWgZ / kWgCopies), src + q * (kWgZ / kWgCopies), kWgZ / kWgCopies, bar);
    };
    if (j == 0) {
      mbar_arrive_expect_tx(bar, 2 * kWgZ);
      copy(kWgSlot3, a.dZ3);
      copy(kWgSlot3 + kWgZ, a.Z2);
    } else if (j == 1) {
      mbar_arrive_expect_tx(bar, 2 * kWgZ);
      copy(kWgSlot2, a.dZ2);
      copy(kWgSlot2 + kWgZ, a.Z1);
    } else if (j == 2) {
      mbar_arrive_expect_tx(bar, kWgZ);
      copy(kWgSlot1, a.dZ1);
    } else {
      mbar_arrive_expect_tx(bar, kWgZ);
      copy(kWgSlot4, a.Z3);
    }
  };

  if (loader) {
    // Refill each slot with its next tile as soon as the slot's UMMAs have completed.
    uint32_t eph = 0, issued = 0; // bit j: parity of slot j's next "empty" phase; loads per slot (mod 2)
    for (int j = 0; j < kWgChains && t0 < t1; ++j) {
      load(j, t0);
      issued ^= 1u << j;
    }
    for (int tile = t0; tile < t1 && !failed; ++tile) {
      for (int j = 0; j < kWgChains; ++j) {
        if (!mbar_wait_bounded(&s.empty[j], (eph >> j) & 1u) || *abort_flag) {
          failed = true;
          break;
        }
        eph ^= 1u << j;
        if (tile + 1 < t1) {
          load(j, tile + 1);
          issued ^= 1u << j;
        }
      }
    }
    if (failed) *abort_flag = 1;
    // After a failure: the copies still in flight land before the block leaves its shared memory
    // (the phase of each slot's last copy: bounded waits).
    for (int j = 0; j < kWgChains && failed; ++j)
      (void)mbar_wait_bounded(&s.full[j], ((issued >> j) & 1u) ^ 1u);
  } else if (issuer) {
    // Thread 0 of warp 8: each slot's UMMAs once the workers have built its operands.
    auto chain = [&](uint32_t a_off, int na, uint32_t b_off, int nb, uint32_t col, bool first) {
      const uint32_t a_lbo = (uint32_t)(na / 8) * 128u, b_lbo = (uint32_t)(nb / 8) * 128u;
      for (int kk = 0; kk < kWgTile / 16; ++kk)
        umma_bf16(tmem + col, umma_desc(base + a_off + kk * 2 * a_lbo, a_lbo, 128u),
                  umma_desc(base + b_off + kk * 2 * b_lbo, b_lbo, 128u), wg_idesc(nb), (first && kk == 0) ? 0u : 1u);
    };
    // Bit j: parity of slot j's next "ready" phase; commits to slot j (mod 2); slot j committed to.
    uint32_t rph = 0, cph = 0, cmask = 0;
    for (int tile = t0; tile < t1 && !failed; ++tile) {
      const bool first = tile == t0;
      for (int j = 0; j < kWgChains; ++j) {
        if (!mbar_wait_bounded(&s.ready[j], (rph >> j) & 1u) || *abort_flag) {
          failed = true;
          *abort_flag = 1;
          break;
        }
        rph ^= 1u << j;
        tc_fence_after();
        if (j == 0) {
          chain(kWgSlot3, kHid, kWgSlot3 + kWgZ, kHid, kWgCol3, first);
          chain(kWgSlot3, kHid, kWgOnes, kWgNb, kWgColB3, first);
        } else if (j == 1) {
          chain(kWgSlot2, kHid, kWgSlot2 + kWgZ, kHid, kWgCol2, first);
          chain(kWgSlot2, kHid, kWgOnes, kWgNb, kWgColB2, first);
        } else if (j == 2) {
          chain(kWgSlot1, kHid, kWgSlot1 + kWgZ, kWgN1, kWgCol1, first);
          chain(kWgSlot1, kHid, kWgOnes, kWgNb, kWgColB1, first);
        } else {
          chain(kWgSlot4, kHid, kWgSlot4 + kWgZ, kWgNb, kWgCol4, first);
        }
        umma_commit(&s.empty[j]);
        cph ^= 1u << j;
        cmask |= 1u << j;
      }
    }
    // After a failure the loader may have stopped waiting for "empty": the last UMMAs of every
    // slot complete before the block releases its TMEM (bounded waits on each slot's last phase).
    for (int j = 0; j < kWgChains && failed; ++j)
      if ((cmask >> j) & 1u) (void)mbar_wait_bounded(&s.empty[j], ((cph >> j) & 1u) ^ 1u);
  } else if (worker) {
    uint32_t fph = 0; // bit j: parity of slot j's next "full" phase
    for (int tile = t0; tile < t1 && !failed; ++tile) {
      const long long row = (long long)tile * kWgTile + r;
      const bool valid = row < a.rows;
      // The thread-built operands' inputs, in flight while chains 3 and 2 run.
      uint4 bx[4] = {};
      int type = -1;
      float d = 0.f;
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
      for (int j = 0; j < kWgChains; ++j) {
        if (!mbar_wait_sleep_bounded(&s.full[j], (fph >> j) & 1u) || *abort_flag) {
          failed = true;
          *abort_flag = 1;
          break;
        }
        fph ^= 1u << j;
        if (j == 0) {
          wg_act_tile(base + kWgSlot3 + kWgZ); // H2
        } else if (j == 1) {
          wg_act_tile(base + kWgSlot2 + kWgZ); // H1
        } else if (j == 2) {
          // B1 = X | one-hot of the type (rows past the end: zero)
          const uint32_t b1 = base + kWgSlot1 + kWgZ;
          if (h == 0) {
#pragma unroll
            for (int q = 0; q < 4; ++q) wg_put(b1, kWgN1, q * 8, r, bx[q]);
          } else {
            const int rel = type & 7, word = rel >> 1;
            const uint32_t one = (rel & 1) ? 0x3F800000u : 0x3F80u;
#pragma unroll
            for (int q = 0; q < kMaxTypes / 8; ++q) {
              const bool here = (type >> 3) == q && type >= 0;
              wg_put(b1, kWgN1, kFeat + q * 8, r,
                     make_uint4(here && word == 0 ? one : 0u, here && word == 1 ? one : 0u,
                                here && word == 2 ? one : 0u, here && word == 3 ? one : 0u));
            }
          }
        } else {
          wg_act_tile(base + kWgSlot4); // H3
          // B4 = dy as two BF16 parts (rows past the end: zero)
          const uint32_t b4 = base + kWgSlot4 + kWgZ;
          if (h == 0) {
            const __nv_bfloat16 hi = __float2bfloat16_rn(d);
            const __nv_bfloat16 lo = __float2bfloat16_rn(d - __bfloat162float(hi));
            const uint32_t db = (uint32_t)__bfloat16_as_ushort(hi) | ((uint32_t)__bfloat16_as_ushort(lo) << 16);
            wg_put(b4, kWgNb, 0, r, make_uint4(db, 0u, 0u, 0u));
          } else {
            wg_put(b4, kWgNb, 8, r, make_uint4(0u, 0u, 0u, 0u));
          }
        }
        fence_proxy_async(); // these generic-proxy writes before the UMMAs' reads
        mbar_arrive(&s.ready[j]);
      }
    }
  }
  tc_fence_before();
  failed = __syncthreads_or(failed);
  tc_fence_after();

  if (failed) {
    if (tid == 0) atomicOr(a.err, 1u);
  } else if (worker && t0 < t1) {
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
        if (col < kWgCol2) {
          p[kWgOffW3 + col * kHid + m] = x;
        } else if (col < kWgCol1) {
          p[kWgOffW2 + (col - kWgCol2) * kHid + m] = x;
        } else if (col < kWgCol4) { // dW1 | S
          const int cc = col - kWgCol1;
          if (cc < kFeat) p[kWgOffW1 + cc * kHid + m] = x;
          else p[kWgOffS + (cc - kFeat) * kHid + m] = x;
        } else if (col == kWgCol4) { // dw4: the hi part's column, then the lo part's
          p[kWgOffW4 + m] = x;
        } else if (col == kWgCol4 + 1) {
          p[kWgOffW4 + m] += x;
        } else if (col == kWgColB3) {
          p[kWgOffB3 + m] = x;
        } else if (col == kWgColB2) {
          p[kWgOffB2 + m] = x;
        } else if (col == kWgColB1) {
          p[kWgOffB1 + m] = x;
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
