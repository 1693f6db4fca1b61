// screen.cu -- surrogate-screened virtual screening of a batch (no counterpart in the reference).
//
// For every ligand of the uploaded batch:
//   1. the surrogate scores all poses (surrogate.cu);
//   2. select_kernel picks the top `top_frac` of poses by surrogate energy (lowest first; an exact
//      radix select with ties taken in pose order, so the pick is deterministic) and an audit
//      sample of exactly ceil(audit_frac * n) of the other poses, uniformly at random (the lowest
//      seeded hashes of the pose indices);
//   3. the picked poses are compacted and rescored by the exact kernel (batch_kernel over the
//      compact transforms);
//   4. audit_kernel measures the surrogate's ordering error on the audit sample,
//      1 - Spearman(surrogate, exact); a ligand whose error exceeds `audit_tol` is rescored
//      exhaustively with the exact kernel;
//   5. final energies: exact where rescored, the surrogate's elsewhere.
// The exact kernel is the arbiter throughout: everything the screen reports as an energy of a
// selected pose is an exact energy.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "batch_kernel.cuh"
#include "internal.h"

namespace bude {

__device__ __forceinline__ uint32_t order_key(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u); // ascending float order as unsigned order
}

__device__ __forceinline__ uint32_t mix_hash(uint32_t seed, uint32_t i) {
  uint32_t h = seed ^ (i * 0x9E3779B9u);
  h ^= h >> 16;
  h *= 0x7FEB352Du;
  h ^= h >> 15;
  h *= 0x846CA68Bu;
  h ^= h >> 16;
  return h;
}

constexpr int kSelThreads = 1024;

// Block-wide exclusive scan of 0/1 flags (one per thread), returns the prefix; *total = block sum.
__device__ __forceinline__ int block_scan(int v, int *warp_sums, int *total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int w = lane < (blockDim.x >> 5) ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    warp_sums[lane] = w; // inclusive
  }
  __syncthreads();
  const int before = (warp > 0 ? warp_sums[warp - 1] : 0) + x - v;
  *total = warp_sums[(blockDim.x >> 5) - 1];
  __syncthreads();
  return before;
}

// The counts select_kernel picks for a ligand of n poses; the host computes the same numbers (the
// same float expressions) to lay out the rescoring before any kernel runs.
__host__ __device__ inline int screen_top_count(float top_frac, int n) {
  const int k = (int)ceilf(top_frac * (float)n);
  return k < 0 ? 0 : (k > n ? n : k);
}
__host__ __device__ inline int screen_audit_count(float audit_frac, int n, int k) {
  const int a = (int)ceilf(audit_frac * (float)n);
  return a < 0 ? 0 : (a > n - k ? n - k : a);
}

// Radix select over the 32-bit keys key(i) of the eligible poses i < n (3 passes of 11/11/10 bits):
// *thr = the need-th smallest key, *ties = how many of the keys equal to it are inside the pick,
// *eq = how many eligible keys equal it (so eq == ties: every key equal to *thr is picked).  The
// bin holding the need-th key is found by a block-wide scan of the histogram.
template <class Key>
__device__ void radix_select(int n, int need, Key key, int *hist, int *warp_sums, uint32_t *s_prefix, uint32_t *s_mask,
                             int *s_need, int *s_eq, uint32_t *thr, int *ties, int *eq) {
  if (threadIdx.x == 0) {
    *s_prefix = 0;
    *s_mask = 0;
    *s_need = need;
    *s_eq = 0;
  }
  __syncthreads();
  const int shifts[3] = {21, 10, 0};
  const int widths[3] = {11, 11, 10};
  for (int pass = 0; pass < 3 && need > 0; ++pass) {
    const int sh = shifts[pass];
    const int nb = 1 << widths[pass];
    const uint32_t bm = (uint32_t)nb - 1u;
    for (int i = threadIdx.x; i < 2048; i += blockDim.x) hist[i] = 0;
    __syncthreads();
    const uint32_t prefix = *s_prefix, mask = *s_mask;
    const int left = *s_need; // read before block_scan's barriers; rewritten after them
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      uint32_t k;
      if (key(i, &k) && (k & mask) == prefix) atomicAdd(&hist[(k >> sh) & bm], 1);
    }
    __syncthreads();
    // Thread t owns bins [t * per, t * per + per); the one whose bins hold the left-th key writes
    // the next prefix.
    const int per = (nb + (int)blockDim.x - 1) / (int)blockDim.x;
    const int b0 = (int)threadIdx.x * per;
    int mine = 0;
    for (int j = 0; j < per; ++j)
      if (b0 + j < nb) mine += hist[b0 + j];
    int tot = 0;
    const int before = block_scan(mine, warp_sums, &tot);
    if (before < left && before + mine >= left) {
      int cum = before, b = b0;
      while (cum + hist[b] < left) cum += hist[b++];
      *s_need = left - cum;
      *s_prefix = prefix | ((uint32_t)b << sh);
      *s_mask = mask | (bm << sh);
      *s_eq = hist[b];
    }
    __syncthreads();
  }
  *thr = *s_prefix;
  *ties = *s_need;
  *eq = *s_eq;
  __syncthreads();
}

// Flags per pose: 1 = top pick, 2 = audit, 0 = neither.  Ligand l = lig0 + blockIdx.x.  The picks
// are the screen_top_count lowest surrogate energies (ties in pose order); the audit sample is the
// screen_audit_count other poses with the lowest seeded hash of their pose index (ties in pose
// order), a uniform random sample of exactly that size.  counts[2l] = picks, counts[2l+1] = audit.
__global__ void __launch_bounds__(kSelThreads) select_kernel(const float *scores, const long long *pose_off, int lig0,
                                                             float top_frac, float audit_frac, uint32_t seed,
                                                             unsigned char *flag, int *counts) {
  __shared__ int hist[2048];
  __shared__ int warp_sums[32];
  __shared__ uint32_t s_prefix, s_mask;
  __shared__ int s_need, s_eq;
  const int l = lig0 + blockIdx.x;
  const long long off = pose_off[l];
  const int n = (int)(pose_off[l + 1] - off);
  const int k = screen_top_count(top_frac, n);
  const int ka = screen_audit_count(audit_frac, n, k);
  uint32_t T = 0, Ta = 0;
  int ties = 0, ties_a = 0, eq = 0, eq_a = 0;
  // 1. the picks: keys below T, then the first `ties` keys equal to T in pose order (a scan only
  //    when some key equal to T stays out)
  radix_select(
      n, k,
      [&](int i, uint32_t *key) {
        *key = order_key(scores[off + i]);
        return true;
      },
      hist, warp_sums, &s_prefix, &s_mask, &s_need, &s_eq, &T, &ties, &eq);
  if (k == 0 || eq == ties) {
    for (int i = threadIdx.x; i < n; i += blockDim.x)
      flag[off + i] = (k > 0 && order_key(scores[off + i]) <= T) ? 1 : 0;
  } else {
    int tie_base = 0;
    for (int c0 = 0; c0 < n; c0 += blockDim.x) {
      const int i = c0 + threadIdx.x;
      const uint32_t key = i < n ? order_key(scores[off + i]) : 0xffffffffu;
      const int is_tie = (i < n && key == T) ? 1 : 0;
      int tot = 0;
      const int rank = block_scan(is_tie, warp_sums, &tot);
      if (i < n) flag[off + i] = (key < T || (is_tie && tie_base + rank < ties)) ? 1 : 0;
      tie_base += tot;
    }
  }
  __threadfence_block();
  __syncthreads();
  // 2. the audit sample among the other poses
  radix_select(
      n, ka,
      [&](int i, uint32_t *key) {
        *key = mix_hash(seed, (uint32_t)(off + i));
        return flag[off + i] == 0;
      },
      hist, warp_sums, &s_prefix, &s_mask, &s_need, &s_eq, &Ta, &ties_a, &eq_a);
  if (ka == 0 || eq_a == ties_a) {
    for (int i = threadIdx.x; i < n; i += blockDim.x)
      if (ka > 0 && flag[off + i] == 0 && mix_hash(seed, (uint32_t)(off + i)) <= Ta) flag[off + i] = 2;
  } else {
    int tie_base = 0;
    for (int c0 = 0; c0 < n; c0 += blockDim.x) {
      const int i = c0 + threadIdx.x;
      const bool free_pose = i < n && flag[off + i] == 0;
      const uint32_t h = free_pose ? mix_hash(seed, (uint32_t)(off + i)) : 0xffffffffu;
      const int is_tie = (free_pose && h == Ta) ? 1 : 0;
      int tot = 0;
      const int rank = block_scan(is_tie, warp_sums, &tot);
      if (free_pose && (h < Ta || (is_tie && tie_base + rank < ties_a))) flag[off + i] = 2;
      tie_base += tot;
    }
  }
  if (threadIdx.x == 0) {
    counts[2 * l] = k;
    counts[2 * l + 1] = ka;
  }
}

// Write the picked poses of ligand l (picks first, then audit, each in pose order) from
// comp_off[l] on, and gather their transforms.
__global__ void __launch_bounds__(kSelThreads) compact_kernel(const long long *pose_off, int lig0,
                                                              const unsigned char *flag,
                                                              const long long *comp_off, const int *counts,
                                                              const float4 *xform, int *comp_pose,
                                                              float4 *comp_xform) {
  __shared__ int warp_sums[32];
  const int l = lig0 + blockIdx.x;
  const long long off = pose_off[l];
  const int n = (int)(pose_off[l + 1] - off);
  const long long base = comp_off[l];
  const int nsel = counts[2 * l];
  for (int which = 1; which <= 2; ++which) {
    int run = 0;
    for (int c0 = 0; c0 < n; c0 += blockDim.x) {
      const int i = c0 + threadIdx.x;
      const int hit = (i < n && flag[off + i] == which) ? 1 : 0;
      int tot = 0;
      const int pos = block_scan(hit, warp_sums, &tot);
      if (hit) {
        const long long dst = base + (which == 2 ? nsel : 0) + run + pos;
        const long long p = off + i;
        comp_pose[dst] = (int)p;
        comp_xform[dst * 3 + 0] = xform[p * 3 + 0];
        comp_xform[dst * 3 + 1] = xform[p * 3 + 1];
        comp_xform[dst * 3 + 2] = xform[p * 3 + 2];
      }
      run += tot;
    }
  }
}

// Per ligand: audit error = 1 - Spearman rank correlation between the surrogate and the exact
// energies of its audit poses (at most kAuditMax of them, in pose order; average ranks for ties).
// A pre-screen only has to order poses, so the audit measures the ordering.
constexpr int kAuditMax = 2048;

__global__ void __launch_bounds__(256) audit_kernel(const long long *comp_off, const int *counts,
                                                    const int *comp_pose, const float *comp_exact,
                                                    const float *scores, float *err) {
  __shared__ float sv[kAuditMax], ev[kAuditMax];
  __shared__ double red[5][256];
  const int l = blockIdx.x;
  const long long a0 = comp_off[l] + counts[2 * l];
  const int na = min(counts[2 * l + 1], kAuditMax);
  for (int i = threadIdx.x; i < na; i += blockDim.x) {
    ev[i] = comp_exact[a0 + i];
    sv[i] = scores[comp_pose[a0 + i]];
  }
  __syncthreads();
  double sr = 0, er = 0, srr = 0, err2 = 0, ser = 0;
  for (int i = threadIdx.x; i < na; i += blockDim.x) {
    float rs = 0.f, re = 0.f;
    for (int j = 0; j < na; ++j) {
      rs += (sv[j] < sv[i]) ? 1.f : (sv[j] == sv[i] && j != i ? 0.5f : 0.f);
      re += (ev[j] < ev[i]) ? 1.f : (ev[j] == ev[i] && j != i ? 0.5f : 0.f);
    }
    sr += rs;
    er += re;
    srr += (double)rs * rs;
    err2 += (double)re * re;
    ser += (double)rs * re;
  }
  red[0][threadIdx.x] = sr;
  red[1][threadIdx.x] = er;
  red[2][threadIdx.x] = srr;
  red[3][threadIdx.x] = err2;
  red[4][threadIdx.x] = ser;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int q = 0; q < 5; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (na < 3) {
      err[l] = 0.f; // too few audit poses to measure the error: keep the picks
    } else {
      const double n = na;
      const double cov = red[4][0] / n - (red[0][0] / n) * (red[1][0] / n);
      const double vs = red[2][0] / n - (red[0][0] / n) * (red[0][0] / n);
      const double ve = red[3][0] / n - (red[1][0] / n) * (red[1][0] / n);
      const double rho = (vs > 0 && ve > 0) ? cov / sqrt(vs * ve) : 0.0;
      err[l] = (float)(1.0 - rho);
    }
  }
}

// final[p] = surrogate score; then exact values scattered over the rescored poses.
__global__ void scatter_kernel(const int *comp_pose, const float *comp_exact, long long n, float *final_e,
                               unsigned char *rescored) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  final_e[comp_pose[i]] = comp_exact[i];
  rescored[comp_pose[i]] = 1;
}

// Exhaustive exact energies of the fallback ligands' poses replace their final energies.
__global__ void fallback_copy_kernel(const long long *pose_off, const int *fallback_ligs, const float *exact,
                                     float *final_e, unsigned char *rescored) {
  const int l = fallback_ligs[blockIdx.x];
  for (long long p = pose_off[l] + threadIdx.x; p < pose_off[l + 1]; p += blockDim.x) {
    final_e[p] = exact[p];
    rescored[p] = 1;
  }
}

struct ScreenState {
  DevBuf pose_off, flag, counts, comp_off, comp_pose, comp_xform, comp_exact, err, final_e, rescored, items, fb;
  DevBuf partial;             // slice sums of split exact evaluations
  cudaStream_t side = nullptr; // the exact rescoring beside the surrogate
  long long result_for = -1;   // Context::batch_uploads of the batch the stored result belongs to
};

void release_screen(Context &c) {
  if (!c.screen) return;
  ScreenState &s = *c.screen;
  for (DevBuf *b : {&s.pose_off, &s.flag, &s.counts, &s.comp_off, &s.comp_pose, &s.comp_xform, &s.comp_exact,
                    &s.err, &s.final_e, &s.rescored, &s.items, &s.fb, &s.partial})
    b->release();
  if (s.side) cudaStreamDestroy(s.side);
  delete c.screen;
  c.screen = nullptr;
}

// Batch-kernel items (for_each_item) over pose ranges [first[i], first[i] + count[i]) of ligand
// lig[i], longest ligand first.
static std::vector<int4> range_items(const Context &c, const std::vector<int> &lig, const std::vector<long long> &first,
                                     const std::vector<int> &count, const bude_launch_cfg &shape) {
  const int ppb = shape.ppwi * shape.wgsize;
  std::vector<int> order(lig.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return c.lig_off[lig[x] + 1] - c.lig_off[lig[x]] > c.lig_off[lig[y] + 1] - c.lig_off[lig[y]];
  });
  std::vector<int4> items;
  for (int i : order) {
    const int l = lig[i];
    for_each_item(count[i], shape.ppwi, ppb, [&](long long p, int n) {
      items.push_back(make_int4(c.lig_off[l], c.lig_off[l + 1] - c.lig_off[l], (int)(first[i] + p), n));
    });
  }
  return items;
}

// Exact energies of the items' poses (pose indices in [0, npose_space) of xform / energies).
static int run_items(Context &c, ScreenState &s, const bude_launch_cfg &cfg, const std::vector<int4> &items,
                     const float4 *xform, float *energies, long long npose_space) {
  if (items.empty()) return BUDE_OK;
  int rc = s.items.reserve(items.size() * sizeof(int4), "screen items");
  if (!rc && cfg.split > 1)
    rc = s.partial.reserve((size_t)cfg.split * (size_t)std::max(npose_space, 1LL) * sizeof(float), "screen slice sums");
  if (rc) return rc;
  cudaMemcpyAsync(s.items.ptr, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice, c.stream);
  rc = batch_items_enqueue(c, cfg, s.items.as<int4>(), (int)items.size(), xform, energies, s.partial.as<float>(),
                           npose_space);
  if (rc) return rc;
  // the host item vector must outlive the copy
  cudaError_t e = cudaStreamSynchronize(c.stream);
  return e == cudaSuccess ? BUDE_OK : cuda_error(e, "screen exact rescoring");
}

int screen_run(Context &c, const bude_screen_cfg &sc, bude_screen_stats *stats) {
  if (!c.have_batch) return set_error(BUDE_ERR_STATE, "no batch uploaded");
  if (!(sc.top_frac >= 0.f && sc.top_frac <= 1.f) || !(sc.audit_frac >= 0.f && sc.audit_frac <= 1.f))
    return set_error(BUDE_ERR_ARG, "fractions must lie in [0, 1]");
  if (!c.screen) c.screen = new ScreenState();
  ScreenState &s = *c.screen;
  s.result_for = -1; // a run that fails leaves no result behind
  const long long np = c.batch_poses;
  const int nl = c.nligands;
  int rc = s.pose_off.reserve((size_t)(nl + 1) * 8, "screen offsets");
  if (!rc) rc = s.flag.reserve((size_t)std::max(np, 1LL), "screen flags");
  if (!rc) rc = s.counts.reserve((size_t)std::max(nl, 1) * 8, "screen counts");
  if (!rc) rc = s.comp_off.reserve((size_t)(nl + 1) * 8, "screen compact offsets");
  if (!rc) rc = s.err.reserve((size_t)std::max(nl, 1) * 4, "audit errors");
  if (!rc) rc = s.final_e.reserve((size_t)std::max(np, 1LL) * 4, "final energies");
  if (!rc) rc = s.rescored.reserve((size_t)std::max(np, 1LL), "rescored flags");
  if (rc) return rc;
  bude_launch_cfg cfg = sc.exact;
  cfg.cluster = 0;
  rc = check_cfg(c, cfg);
  if (rc) return rc;
  // The picks and audit counts per ligand depend only on its pose count, so the compacted layout
  // and the rescoring items are known before any kernel runs.
  std::vector<int> counts((size_t)2 * nl);
  std::vector<long long> comp_off((size_t)nl + 1, 0);
  for (int l = 0; l < nl; ++l) {
    const int n = (int)(c.pose_off[l + 1] - c.pose_off[l]);
    counts[2 * l] = screen_top_count(sc.top_frac, n);
    counts[2 * l + 1] = screen_audit_count(sc.audit_frac, n, counts[2 * l]);
    comp_off[l + 1] = comp_off[l] + counts[2 * l] + counts[2 * l + 1];
  }
  const long long ncomp = comp_off[nl];
  rc = s.comp_pose.reserve((size_t)std::max(ncomp, 1LL) * 4, "compact poses");
  if (!rc) rc = s.comp_xform.reserve((size_t)std::max(ncomp, 1LL) * 48, "compact transforms");
  if (!rc) rc = s.comp_exact.reserve((size_t)std::max(ncomp, 1LL) * 4, "compact energies");
  if (!rc && cfg.split > 1)
    rc = s.partial.reserve((size_t)cfg.split * (size_t)std::max(ncomp, 1LL) * sizeof(float), "screen slice sums");
  if (rc) return rc;
  // Ligand chunks (sc.chunks > 1): the surrogate scores chunk j+1 (3 tile groups per block) while
  // the exact kernel rescores chunk j's picks beside it on a second stream, two blocks per SM.
  // Measured on 1,024 ligands x 16,384 poses it is slower (126 ms against 106 ms): the rescoring
  // blocks slow the scorer more than they hide, so one chunk (no overlap, 4 groups) is the default.
  const int nchunks = nl == 0 ? 0 : std::max(1, std::min(nl, sc.chunks > 0 ? sc.chunks : 1));
  const bool overlap = nchunks > 1;
  // Each ligand contributes only a few hundred picks: rescore them in small items so blocks are
  // not mostly empty, with the fallback's protein slices (the pose shape does not change the
  // arithmetic of a pose, the slices do).  One-warp blocks of 8 poses per thread (256-pose
  // items) measured fastest on 410 picks per ligand (8 slices: 27.9 ms against 30.5 for 64
  // threads x 4 poses, before the short-item cut); fewer picks per ligand get 128-pose items.
  int with_picks = 0;
  for (int l = 0; l < nl; ++l) with_picks += counts[2 * l] + counts[2 * l + 1] > 0;
  const long long per_lig = with_picks ? ncomp / with_picks : 0;
  bude_launch_cfg small = overlap                          ? bude_launch_cfg{4, 128, cfg.split, cfg.tile, 2, 0}
                          : (per_lig > 256 && per_lig <= 448) ? bude_launch_cfg{14, 32, cfg.split, cfg.tile, 2, 0}
                          : per_lig >= 128                  ? bude_launch_cfg{8, 32, cfg.split, cfg.tile, 4, 0}
                                                            : bude_launch_cfg{4, 32, cfg.split, cfg.tile, 2, 0};
  if (sc.rescore.ppwi != 0) {
    small = bude_launch_cfg{sc.rescore.ppwi, sc.rescore.wgsize, cfg.split, sc.rescore.tile > 0 ? sc.rescore.tile : cfg.tile,
                            sc.rescore.unroll, 0};
    const bool rescore_only = small.ppwi == 14 && small.unroll == 2; // a batch-kernel shape of the rescoring
    bude_launch_cfg chk = small;
    if (rescore_only) chk.ppwi = 16;
    rc = check_cfg(c, chk);
    if (rc) return rc;
    if (cfg.tile % small.tile) return set_error(BUDE_ERR_ARG, "the rescoring tile must divide the exact tile");
  }
  std::vector<int> chunk_lig(nchunks + 1, nl), chunk_item(nchunks + 1, 0);
  std::vector<int4> items;
  for (int j = 0; j < nchunks; ++j) {
    chunk_lig[j] = (int)((long long)nl * j / nchunks);
    std::vector<int> lig, cnt;
    std::vector<long long> first;
    for (int l = (int)((long long)nl * j / nchunks); l < (int)((long long)nl * (j + 1) / nchunks); ++l) {
      const int k = counts[2 * l] + counts[2 * l + 1];
      if (k == 0) continue;
      lig.push_back(l);
      first.push_back(comp_off[l]);
      cnt.push_back(k);
    }
    chunk_item[j] = (int)items.size();
    const std::vector<int4> its = range_items(c, lig, first, cnt, small);
    items.insert(items.end(), its.begin(), its.end());
  }
  if (nchunks > 0) chunk_item[nchunks] = (int)items.size();
  rc = s.items.reserve(std::max<size_t>(items.size(), 1) * sizeof(int4), "screen items");
  if (rc) return rc;
  if (overlap && !s.side) {
    cudaError_t es = cudaStreamCreateWithFlags(&s.side, cudaStreamNonBlocking);
    if (es != cudaSuccess) return cuda_error(es, "screen rescoring stream");
  }
  EventSet ready((size_t)nchunks, cudaEventDisableTiming), ev(5);
  if (!ready.ok() || !ev.ok()) return set_error(BUDE_ERR_CUDA, "could not create the screen's events");
  cudaEventRecord(ev[0], c.stream);
  cudaEventRecord(ev[1], c.stream); // re-recorded after each chunk's surrogate
  cudaMemcpyAsync(s.pose_off.ptr, c.pose_off.data(), (size_t)(nl + 1) * 8, cudaMemcpyHostToDevice, c.stream);
  cudaMemcpyAsync(s.comp_off.ptr, comp_off.data(), comp_off.size() * 8, cudaMemcpyHostToDevice, c.stream);
  if (!items.empty())
    cudaMemcpyAsync(s.items.ptr, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice, c.stream);
  rc = surrogate_prepare(c, false); // pose transforms of every pose
  if (rc) return rc;
  const float *scores = surrogate_scores(c);
  cudaStream_t rs = overlap ? s.side : c.stream;
  // 1-3. per chunk: surrogate, picks and audit sample, compaction; exact rescoring on `rs`
  for (int j = 0; j < nchunks && !rc; ++j) {
    const int l0 = chunk_lig[j], l1 = chunk_lig[j + 1];
    rc = surrogate_score_range(c, l0, l1, overlap ? 3 : 4, c.stream);
    if (rc) break;
    cudaEventRecord(ev[1], c.stream); // after the last chunk's surrogate: the end of the surrogate phase
    if (l1 > l0) {
      select_kernel<<<l1 - l0, kSelThreads, 0, c.stream>>>(scores, s.pose_off.as<long long>(), l0, sc.top_frac,
                                                           sc.audit_frac, (uint32_t)sc.seed,
                                                           s.flag.as<unsigned char>(), s.counts.as<int>());
      compact_kernel<<<l1 - l0, kSelThreads, 0, c.stream>>>(s.pose_off.as<long long>(), l0,
                                                            s.flag.as<unsigned char>(), s.comp_off.as<long long>(),
                                                            s.counts.as<int>(), c.b_xform.as<float4>(),
                                                            s.comp_pose.as<int>(), s.comp_xform.as<float4>());
      c.launches += 2;
    }
    cudaEventRecord(ready[j], c.stream);
    if (overlap) cudaStreamWaitEvent(rs, ready[j], 0);
    const int n_it = chunk_item[j + 1] - chunk_item[j];
    if (n_it > 0)
      rc = batch_items_enqueue(c, small, s.items.as<int4>() + chunk_item[j], n_it, s.comp_xform.as<float4>(),
                               s.comp_exact.as<float>(), s.partial.as<float>(), ncomp, rs, overlap ? 2 : 0, cfg.tile);
  }
  if (overlap) {
    cudaEvent_t joined = nchunks > 0 ? ready[0] : nullptr;
    if (joined) {
      cudaEventRecord(joined, rs);
      cudaStreamWaitEvent(c.stream, joined, 0);
    }
  }
  cudaEventRecord(ev[2], c.stream);
  if (rc) {
    cudaStreamSynchronize(c.stream);
    return rc;
  }
  // 4. audit and fallback (the audit follows the rescoring on the stream; one wait for both)
  if (nl > 0)
    audit_kernel<<<nl, 256, 0, c.stream>>>(s.comp_off.as<long long>(), s.counts.as<int>(), s.comp_pose.as<int>(),
                                           s.comp_exact.as<float>(), scores, s.err.as<float>());
  c.launches += nl > 0;
  std::vector<float> err((size_t)nl);
  if (nl > 0) cudaMemcpyAsync(err.data(), s.err.ptr, (size_t)nl * 4, cudaMemcpyDeviceToHost, c.stream);
  cudaError_t e = cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) return cuda_error(e, "screen audit");
  std::vector<int> fb_lig, fb_cnt;
  std::vector<long long> fb_first;
  for (int l = 0; l < nl; ++l)
    if (err[l] > sc.audit_tol) {
      fb_lig.push_back(l);
      fb_first.push_back(c.pose_off[l]);
      fb_cnt.push_back((int)(c.pose_off[l + 1] - c.pose_off[l]));
    }
  rc = run_items(c, s, cfg, range_items(c, fb_lig, fb_first, fb_cnt, cfg), c.b_xform.as<float4>(),
                 c.b_energies.as<float>(), np);
  if (rc) return rc;
  cudaEventRecord(ev[3], c.stream);
  // 5. final energies
  if (np > 0) {
    cudaMemcpyAsync(s.final_e.ptr, scores, (size_t)np * 4, cudaMemcpyDeviceToDevice, c.stream);
    cudaMemsetAsync(s.rescored.ptr, 0, (size_t)np, c.stream);
  }
  if (ncomp > 0)
    scatter_kernel<<<(unsigned)((ncomp + 255) / 256), 256, 0, c.stream>>>(
        s.comp_pose.as<int>(), s.comp_exact.as<float>(), ncomp, s.final_e.as<float>(), s.rescored.as<unsigned char>());
  if (!fb_lig.empty()) {
    rc = s.fb.reserve(fb_lig.size() * 4, "fallback ligands");
    if (rc) return rc;
    cudaMemcpyAsync(s.fb.ptr, fb_lig.data(), fb_lig.size() * 4, cudaMemcpyHostToDevice, c.stream);
    fallback_copy_kernel<<<(unsigned)fb_lig.size(), 256, 0, c.stream>>>(
        s.pose_off.as<long long>(), s.fb.as<int>(), c.b_energies.as<float>(), s.final_e.as<float>(),
        s.rescored.as<unsigned char>());
  }
  // Irregular poses (edge_pose.cuh) get the reference's arithmetic in the final list, flagged as
  // rescored, whatever the surrogate made of them.
  rc = enqueue_edge_batch(c, c.b_xform.as<float>(), s.final_e.as<float>(), s.rescored.as<unsigned char>(), c.stream);
  if (rc) return rc;
  cudaEventRecord(ev[4], c.stream);
  e = cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) return cuda_error(e, "screen");
  rc = check_device_error(c);
  if (rc) return rc;
  if (stats) {
    cudaEventElapsedTime(&stats->total_ms, ev[0], ev[4]);
    cudaEventElapsedTime(&stats->surrogate_ms, ev[0], ev[1]);
    cudaEventElapsedTime(&stats->rescore_ms, ev[1], ev[2]);
    cudaEventElapsedTime(&stats->fallback_ms, ev[2], ev[3]);
    stats->rescored_poses = ncomp;
    stats->fallback_ligands = (int32_t)fb_lig.size();
    long long fbp = 0;
    for (int v : fb_cnt) fbp += v;
    stats->fallback_poses = fbp;
    float mx = 0.f;
    for (float v : err) mx = std::max(mx, v);
    stats->max_audit_error = mx;
  }
  s.result_for = c.batch_uploads;
  return BUDE_OK;
}

} // namespace bude

using namespace bude;

extern "C" {

int bude_screen_run(bude_gpu_ctx *ctx, const bude_screen_cfg *cfg, bude_screen_stats *stats) {
  if (!ctx || !cfg) return set_error(BUDE_ERR_ARG, "NULL argument");
  cudaSetDevice(ctx->device);
  return screen_run(*ctx, *cfg, stats);
}

int bude_screen_download(bude_gpu_ctx *ctx, float *final_energies, uint8_t *rescored, float *audit_error,
                         int64_t total_poses) {
  if (!ctx || !ctx->screen || !ctx->have_batch || ctx->screen->result_for != ctx->batch_uploads ||
      total_poses != ctx->batch_poses)
    return set_error(BUDE_ERR_STATE, "no screen result of the uploaded batch for %lld poses", (long long)total_poses);
  cudaSetDevice(ctx->device);
  cudaError_t e = cudaSuccess;
  if (final_energies && total_poses > 0)
    e = copy_sync(*ctx, final_energies, ctx->screen->final_e.ptr, (size_t)total_poses * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && rescored && total_poses > 0)
    e = copy_sync(*ctx, rescored, ctx->screen->rescored.ptr, (size_t)total_poses, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && audit_error && ctx->nligands > 0)
    e = copy_sync(*ctx, audit_error, ctx->screen->err.ptr, (size_t)ctx->nligands * 4, cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? BUDE_OK : cuda_error(e, "screen download");
}

} // extern "C"
