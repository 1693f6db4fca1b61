// screen.cu -- surrogate-screened virtual screening of a batch (no counterpart in the reference).
//
// For every ligand of the uploaded batch:
//   1. the surrogate scores all poses (surrogate.cu);
//   2. select_kernel picks the top `top_frac` of poses by surrogate energy (lowest first; an exact
//      radix select with ties taken in pose order, so the pick is deterministic) and an audit
//      sample of about `audit_frac` of all poses, uniformly from the rest (a hash of the seed and
//      the pose index decides);
//   3. the picked poses are compacted and rescored by the exact kernel (batch_kernel over the
//      compact transforms);
//   4. audit_kernel measures the surrogate's ordering error on the audit sample,
//      1 - Spearman(surrogate, exact); a ligand whose error exceeds `audit_tol` is rescored
//      exhaustively with the exact kernel;
//   5. final energies: exact where rescored, the surrogate's elsewhere.
// The exact kernel is the judge throughout: everything the screen reports as an energy of a
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

// Flags per pose: 1 = top pick, 2 = audit, 0 = neither.  counts[2l] = picks, counts[2l+1] = audit.
__global__ void __launch_bounds__(kSelThreads) select_kernel(const float *scores, const long long *pose_off,
                                                             float top_frac, float audit_frac, uint32_t seed,
                                                             unsigned char *flag, int *counts) {
  __shared__ int hist[2048];
  __shared__ int warp_sums[32];
  __shared__ uint32_t s_prefix, s_mask;
  __shared__ int s_need;
  const int l = blockIdx.x;
  const long long off = pose_off[l];
  const int n = (int)(pose_off[l + 1] - off);
  int k = (int)ceilf(top_frac * (float)n);
  k = max(0, min(n, k));
  if (threadIdx.x == 0) {
    s_prefix = 0;
    s_mask = 0;
    s_need = k;
  }
  __syncthreads();
  const int shifts[3] = {21, 10, 0};
  const int widths[3] = {11, 11, 10};
  for (int pass = 0; pass < 3 && k > 0; ++pass) {
    const int sh = shifts[pass];
    const uint32_t bm = (1u << widths[pass]) - 1u;
    for (int i = threadIdx.x; i < 2048; i += blockDim.x) hist[i] = 0;
    __syncthreads();
    const uint32_t prefix = s_prefix, mask = s_mask;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const uint32_t key = order_key(scores[off + i]);
      if ((key & mask) == prefix) atomicAdd(&hist[(key >> sh) & bm], 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int need = s_need, cum = 0;
      uint32_t b = 0;
      for (; b < bm; ++b) {
        if (cum + hist[b] >= need) break;
        cum += hist[b];
      }
      s_need = need - cum;
      s_prefix = prefix | (b << sh);
      s_mask = mask | (bm << sh);
    }
    __syncthreads();
  }
  const uint32_t T = s_prefix; // key of the k-th smallest score
  const int ties_needed = s_need;
  // Flags in pose order: keys < T, then the first `ties_needed` keys == T.
  const uint32_t audit_thr =
      (uint32_t)fminf(4294967295.f, 4294967296.f * (k < n ? audit_frac * n / (float)(n - k) : 0.f));
  int tie_base = 0, audit_count = 0;
  for (int c0 = 0; c0 < n; c0 += blockDim.x) {
    const int i = c0 + threadIdx.x;
    uint32_t key = 0xffffffffu;
    if (i < n) key = order_key(scores[off + i]);
    const int is_tie = (k > 0 && i < n && key == T) ? 1 : 0;
    int tot = 0;
    const int rank = block_scan(is_tie, warp_sums, &tot);
    if (i < n) {
      unsigned char f = 0;
      if (k > 0 && (key < T || (is_tie && tie_base + rank < ties_needed))) f = 1;
      else if (mix_hash(seed, (uint32_t)(off + i)) < audit_thr) f = 2;
      flag[off + i] = f;
      audit_count += (f == 2);
    }
    tie_base += tot;
  }
  // block sum of audit picks
  int tot = 0;
  (void)block_scan(audit_count, warp_sums, &tot);
  if (threadIdx.x == 0) {
    counts[2 * l] = k;
    counts[2 * l + 1] = tot;
  }
}

// Write the picked poses of ligand l (picks first, then audit, each in pose order) from
// comp_off[l] on, and gather their transforms.
__global__ void __launch_bounds__(kSelThreads) compact_kernel(const long long *pose_off, const unsigned char *flag,
                                                              const long long *comp_off, const int *counts,
                                                              const float4 *xform, int *comp_pose,
                                                              float4 *comp_xform) {
  __shared__ int warp_sums[32];
  const int l = blockIdx.x;
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
      err[l] = 0.f; // too few audit poses to judge: keep the picks
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
  DevBuf partial; // slice sums of split exact evaluations
};

void release_screen(Context &c) {
  if (!c.screen) return;
  ScreenState &s = *c.screen;
  for (DevBuf *b : {&s.pose_off, &s.flag, &s.counts, &s.comp_off, &s.comp_pose, &s.comp_xform, &s.comp_exact,
                    &s.err, &s.final_e, &s.rescored, &s.items, &s.fb, &s.partial})
    b->release();
  delete c.screen;
  c.screen = nullptr;
}

// Items of ppb poses over pose ranges [first[i], first[i] + count[i]) of ligand lig[i].
static std::vector<int4> range_items(const Context &c, const std::vector<int> &lig, const std::vector<long long> &first,
                                     const std::vector<int> &count, int ppb) {
  std::vector<int> order(lig.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return c.lig_off[lig[x] + 1] - c.lig_off[lig[x]] > c.lig_off[lig[y] + 1] - c.lig_off[lig[y]];
  });
  std::vector<int4> items;
  for (int i : order) {
    const int l = lig[i];
    for (int p = 0; p < count[i]; p += ppb)
      items.push_back(make_int4(c.lig_off[l], c.lig_off[l + 1] - c.lig_off[l], (int)(first[i] + p),
                                std::min(ppb, count[i] - p)));
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
  cudaEvent_t ev[5];
  for (auto &e : ev) cudaEventCreate(&e);
  cudaEventRecord(ev[0], c.stream);
  cudaMemcpyAsync(s.pose_off.ptr, c.pose_off.data(), (size_t)(nl + 1) * 8, cudaMemcpyHostToDevice, c.stream);
  // 1. surrogate over every pose (computes the pose transforms first)
  rc = surrogate_score_enqueue(c, nullptr);
  if (rc) return rc;
  const float *scores = surrogate_scores(c);
  cudaEventRecord(ev[1], c.stream);
  // 2. picks and audit sample
  if (nl > 0)
    select_kernel<<<nl, kSelThreads, 0, c.stream>>>(scores, s.pose_off.as<long long>(), sc.top_frac, sc.audit_frac,
                                                    (uint32_t)sc.seed, s.flag.as<unsigned char>(), s.counts.as<int>());
  c.launches += nl > 0;
  std::vector<int> counts((size_t)2 * nl);
  if (nl > 0) cudaMemcpyAsync(counts.data(), s.counts.ptr, counts.size() * 4, cudaMemcpyDeviceToHost, c.stream);
  cudaError_t e = cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) return cuda_error(e, "screen selection");
  std::vector<long long> comp_off((size_t)nl + 1, 0);
  for (int l = 0; l < nl; ++l) comp_off[l + 1] = comp_off[l] + counts[2 * l] + counts[2 * l + 1];
  const long long ncomp = comp_off[nl];
  rc = s.comp_pose.reserve((size_t)std::max(ncomp, 1LL) * 4, "compact poses");
  if (!rc) rc = s.comp_xform.reserve((size_t)std::max(ncomp, 1LL) * 48, "compact transforms");
  if (!rc) rc = s.comp_exact.reserve((size_t)std::max(ncomp, 1LL) * 4, "compact energies");
  if (rc) return rc;
  cudaMemcpyAsync(s.comp_off.ptr, comp_off.data(), comp_off.size() * 8, cudaMemcpyHostToDevice, c.stream);
  if (nl > 0)
    compact_kernel<<<nl, kSelThreads, 0, c.stream>>>(s.pose_off.as<long long>(), s.flag.as<unsigned char>(),
                                                     s.comp_off.as<long long>(), s.counts.as<int>(),
                                                     c.b_xform.as<float4>(), s.comp_pose.as<int>(),
                                                     s.comp_xform.as<float4>());
  c.launches += nl > 0;
  // 3. exact rescoring of picks + audit
  std::vector<int> lig, cnt;
  std::vector<long long> first;
  for (int l = 0; l < nl; ++l) {
    const int k = counts[2 * l] + counts[2 * l + 1];
    if (k == 0) continue;
    lig.push_back(l);
    first.push_back(comp_off[l]);
    cnt.push_back(k);
  }
  // Each ligand contributes only a few hundred picks: rescore them in 256-pose items so blocks are
  // not mostly empty, with the fallback's protein slices (the pose shape does not change the
  // arithmetic of a pose, the slices do).
  const bude_launch_cfg small{4, 64, cfg.split, cfg.tile, 2, 0};
  rc = run_items(c, s, small, range_items(c, lig, first, cnt, small.ppwi * small.wgsize), s.comp_xform.as<float4>(),
                 s.comp_exact.as<float>(), ncomp);
  if (rc) return rc;
  cudaEventRecord(ev[2], c.stream);
  // 4. audit and fallback
  if (nl > 0)
    audit_kernel<<<nl, 256, 0, c.stream>>>(s.comp_off.as<long long>(), s.counts.as<int>(), s.comp_pose.as<int>(),
                                           s.comp_exact.as<float>(), scores, s.err.as<float>());
  c.launches += nl > 0;
  std::vector<float> err((size_t)nl);
  if (nl > 0) cudaMemcpyAsync(err.data(), s.err.ptr, (size_t)nl * 4, cudaMemcpyDeviceToHost, c.stream);
  e = cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) return cuda_error(e, "screen audit");
  std::vector<int> fb_lig, fb_cnt;
  std::vector<long long> fb_first;
  for (int l = 0; l < nl; ++l)
    if (err[l] > sc.audit_tol) {
      fb_lig.push_back(l);
      fb_first.push_back(c.pose_off[l]);
      fb_cnt.push_back((int)(c.pose_off[l + 1] - c.pose_off[l]));
    }
  rc = run_items(c, s, cfg, range_items(c, fb_lig, fb_first, fb_cnt, cfg.ppwi * cfg.wgsize), c.b_xform.as<float4>(),
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
  for (auto &x : ev) cudaEventDestroy(x);
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
  if (!ctx || !ctx->screen || !ctx->have_batch || total_poses != ctx->batch_poses)
    return set_error(BUDE_ERR_STATE, "no screen result for %lld poses", (long long)total_poses);
  cudaSetDevice(ctx->device);
  cudaError_t e = cudaSuccess;
  if (final_energies && total_poses > 0)
    e = cudaMemcpy(final_energies, ctx->screen->final_e.ptr, (size_t)total_poses * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && rescored && total_poses > 0)
    e = cudaMemcpy(rescored, ctx->screen->rescored.ptr, (size_t)total_poses, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && audit_error && ctx->nligands > 0)
    e = cudaMemcpy(audit_error, ctx->screen->err.ptr, (size_t)ctx->nligands * 4, cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? BUDE_OK : cuda_error(e, "screen download");
}

} // extern "C"
