// autotune.cu -- launch-shape selection for the exact kernel.
//
// Replaces the reference driver's brute-force PPWI x wgsize sweep (src/main.cpp:517-541) with
//   * a wave model: for a (poses per thread, block size, unroll) shape it reads the kernel's
//     resident blocks per SM from the CUDA occupancy API and picks the protein split whose block
//     count fills the last wave best (choose_split), and
//   * a short measured search over the shapes the model ranks best, timed with CUDA events on a
//     ligand prefix (time is linear in ligand atoms, the wave structure is unchanged).
// The pick is cached per deck shape in the context.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "exact_shape.h"
#include "internal.h"

namespace bude {

static int ppwi_to_p(int ppwi) {
  if (ppwi >= 16) return 16;
  if (ppwi >= 8) return 8;
  if (ppwi >= 4) return 4;
  if (ppwi >= 2) return 2;
  return 1;
}

// Pick cfg.split (and keep cfg.cluster) so that pose blocks x slices fill whole waves of the
// device's resident block slots.  Cost model, in units of one block's full-protein time:
//   rounds(S) / S * (1 + 0.01 * (S - 1))
// (rounds = ceil(blocks * S / slots); the small per-slice term covers the reduction and the
// shorter protein loop of thin slices).  Slices keep at least 64 protein atoms here; the measured
// search below also tries thinner slices.
int choose_split(const Context &c, bude_launch_cfg &cfg) {
  return choose_split_for(c.num_sms, c.natpro_pad, c.nposes, cfg);
}

int choose_split_for(int num_sms, int natpro_pad, long long nposes, bude_launch_cfg &cfg) {
  cfg.split = 1;
  int per_sm = 0;
  int rc = exact_blocks_per_sm(cfg, &per_sm);
  if (rc) return rc;
  if (per_sm <= 0) return set_error(BUDE_ERR_ARG, "launch shape cannot be resident on an SM");
  const long long slots = (long long)per_sm * std::max(num_sms, 1);
  const long long ppb = (long long)cfg.ppwi * cfg.wgsize;
  const long long blocks = std::max<long long>(1, (nposes + ppb - 1) / ppb);
  const int smax = std::max(1, std::min(cfg.cluster ? 8 : 64, natpro_pad / 64));
  double best = 1e300;
  for (int s = 1; s <= smax; ++s) {
    const long long rounds = (blocks * s + slots - 1) / slots;
    const double cost = double(rounds) / s * (1.0 + 0.01 * (s - 1));
    if (cost < best - 1e-12) {
      best = cost;
      cfg.split = s;
    }
  }
  return BUDE_OK;
}

int default_cfg(const Context &c, int ppwi, int wgsize, bude_launch_cfg &cfg) {
  cfg.ppwi = ppwi_to_p(std::max(ppwi, 1));
  const int w = wgsize < 32 ? 128 : (wgsize + 31) / 32 * 32;
  cfg.wgsize = std::min(w, kMaxThreads);
  cfg.tile = 64;
  cfg.unroll = cfg.ppwi >= 16 ? 1 : 2;
  cfg.cluster = 0;
  cfg.split = 1;
  if (c.num_sms <= 0 || !c.have_deck) return BUDE_OK;
  return choose_split(c, cfg);
}

// Time one shape: one untimed evaluation, then the mean of `reps` event-timed ones.
static int time_cfg(Context &c, const bude_launch_cfg &cfg, int reps, float *ms) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int rc = enqueue_eval(c, cfg);
  if (!rc) {
    cudaEventRecord(e0, c.stream);
    for (int i = 0; i < reps && !rc; ++i) rc = enqueue_eval(c, cfg);
    cudaEventRecord(e1, c.stream);
  }
  cudaError_t e = cudaStreamSynchronize(c.stream);
  if (!rc && e != cudaSuccess) rc = cuda_error(e, "autotune timing");
  if (!rc) {
    cudaEventElapsedTime(ms, e0, e1);
    *ms /= reps;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (!rc) rc = check_device_error(c);
  return rc;
}

int autotune(Context &c, int max_ms, bude_launch_cfg &best, float *best_ms) {
  if (!c.have_deck) return set_error(BUDE_ERR_STATE, "no deck uploaded");
  const long long key[3] = {c.natpro_pad, c.natlig, c.nposes};
  if (key[0] == c.tuned_key[0] && key[1] == c.tuned_key[1] && key[2] == c.tuned_key[2]) {
    best = c.tuned;
    if (best_ms) *best_ms = c.tuned_ms;
    return BUDE_OK;
  }
  // Candidate shapes: poses per thread x block size x unroll, each with its model split, in
  // both reduction modes.
  struct Shape { int p, w, u; };
  const Shape shapes[] = {{4, 64, 2},  {4, 128, 4}, {4, 256, 4}, {8, 64, 2},   {8, 128, 2},
                          {8, 256, 2}, {16, 64, 1}, {16, 128, 1}, {16, 256, 1}, {2, 128, 2}};
  std::vector<bude_launch_cfg> cands;
  for (const Shape &s : shapes)
    for (int cl = 0; cl < 2; ++cl) {
      bude_launch_cfg cfg{s.p, s.w, 1, 64, s.u, cl};
      if (choose_split(c, cfg)) continue;
      if (cl == 1 && cfg.split == 1) continue; // same launch as cluster 0
      cands.push_back(cfg);
    }
  if (cands.empty()) return set_error(BUDE_ERR_ARG, "no launch shape fits this device");

  // Time on a ligand prefix so one evaluation takes about a millisecond or more.
  const int natlig_full = c.natlig;
  const double inter_per_lig = double(c.nposes) * c.natpro;
  int lig = natlig_full;
  const double target = 2.0e9; // interactions per timed evaluation (~1 ms at the kernel's rate)
  if (inter_per_lig * natlig_full > target) lig = std::max(1, (int)std::ceil(target / std::max(inter_per_lig, 1.0)));
  lig = std::min(lig, natlig_full);
  c.natlig = lig;
  int rc = BUDE_OK;
  float best_t = 1e30f;
  float budget = (float)std::max(max_ms, 1);
  float spent = 0.f;
  auto trial = [&](const bude_launch_cfg &cfg, float *ms) {
    rc = time_cfg(c, cfg, 2, ms);
    if (rc) return false;
    spent += 3.f * *ms;
    if (*ms < best_t) {
      best_t = *ms;
      best = cfg;
    }
    return spent <= budget;
  };
  // Phase 1: every shape with the wave model's split.
  std::vector<std::pair<float, bude_launch_cfg>> timed;
  for (const bude_launch_cfg &cfg : cands) {
    float ms = 0.f;
    const bool more = trial(cfg, &ms);
    if (rc) break;
    timed.push_back({ms, cfg});
    if (!more) break;
  }
  // Phase 2: the four fastest global-reduce shapes over every distinct slice width from half to
  // two and a half times the model's split (slices down to 32 atoms).  The model's rounds of
  // resident blocks do not capture how much more resident warps per SM help: on 938 atoms x 65,536
  // poses, 8 poses per thread, 128 threads, it picks 12 slices where 20 (48-atom slices) measured
  // 6% faster.
  if (!rc && spent <= budget) {
    std::sort(timed.begin(), timed.end(), [](const auto &a, const auto &b) { return a.first < b.first; });
    // Splits whose slice sums ([split][nposes] floats) would pass 512 MB are not tried.
    const long long split_cap = std::max(1LL, (512LL << 20) / (4LL * std::max(c.nposes, 1LL)));
    const int smax_thin = (int)std::max(1LL, std::min({64LL, (long long)c.natpro_pad / 32, split_cap}));
    int widened = 0;
    for (const auto &t : timed) {
      if (widened == 4 || rc || spent > budget) break;
      const bude_launch_cfg base = t.second;
      if (base.cluster != 0) continue;
      ++widened;
      int last_slice = -1;
      for (int sp = std::max(2, base.split / 2); sp <= std::min(smax_thin, base.split * 5 / 2); ++sp) {
        const int slice = (c.natpro_pad + sp - 1) / sp;
        const int width = (slice + kAtomAlign - 1) / kAtomAlign * kAtomAlign;
        if (width == last_slice || sp == base.split) continue;
        // The fewest slices of this width (more would only add empty blocks).
        if ((c.natpro_pad + width - 1) / width != sp) continue;
        last_slice = width;
        bude_launch_cfg cfg = base;
        cfg.split = sp;
        float ms = 0.f;
        if (!trial(cfg, &ms) || rc) break;
      }
    }
    // A shape of this pass whose slice sums did not fit in device memory (a failed allocation)
    // ends the pass; the pick stays the best shape timed so far.  Other errors are returned.
    if (rc == BUDE_ERR_CUDA) {
      (void)cudaGetLastError();
      rc = BUDE_OK;
    }
  }
  c.natlig = natlig_full;
  if (rc) return rc;
  const float scale = float(natlig_full) / float(lig);
  c.tuned = best;
  c.tuned_ms = best_t * scale;
  for (int i = 0; i < 3; ++i) c.tuned_key[i] = key[i];
  if (best_ms) *best_ms = c.tuned_ms;
  return BUDE_OK;
}

} // namespace bude

extern "C" int bude_gpu_autotune(bude_gpu_ctx *ctx, int32_t max_ms, bude_launch_cfg *best, float *best_ms) {
  if (!ctx || !best) return bude::set_error(BUDE_ERR_ARG, "NULL argument");
  cudaSetDevice(ctx->device);
  return bude::autotune(*ctx, max_ms, *best, best_ms);
}
