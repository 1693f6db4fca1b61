// batch_kernel.cuh -- persistent exact scoring of many ligands, each with its own poses.
//
// The work of a batch (ligand l has natlig_l atoms and nposes_l poses, all against one protein)
// is cut into items of one pose block each: (first ligand atom, natlig, first pose, pose count),
// with at most P * blockDim poses per item.  The host orders items longest first (natlig
// descending).  A grid of exactly the resident block slots loops: one thread takes the next item
// from a global counter (atomicAdd), the block scores it with the exact kernel's arithmetic
// (PosePairs::transform / tile, exact_kernel.cuh) over the whole protein, writes 0.5 * etot for
// its poses and takes the next item.  The shared-memory ring and its mbarrier phases run on across
// items (a global step counter), so no barrier is re-initialised.
//
// With split > 1 the protein is cut into `split` slices of `slice` records and every item is
// scored once per slice (work unit v = item * split + slice, so the slices of an item follow each
// other in the queue); each unit writes its slice sum to partial[slice][pose] and
// batch_reduce_kernel folds the slices in slice order.  Many small items of uneven ligand size then
// still spread evenly over the block slots.  The result is deterministic for a given split and
// slice length.
#pragma once
#include "exact_kernel.cuh"

namespace bude {

struct BatchArgs {
  const float4 *ligands; // all ligands' atoms: {x, y, z, __int_as_float(type)}
  const float4 *slab;    // ntypes x natpro_pad x kRecF4
  const float *xform;    // total poses x 12
  float *energies;       // total poses
  const int4 *items;     // {first ligand atom, natlig, first pose, pose count}
  unsigned int *counter; // next item; zero before the launch
  unsigned int *err;     // bit 0: a bounded wait ran out
  int n_items;
  int natpro_pad;
  int tile;
  int split;             // protein slices per item (1: energies written directly)
  int slice;             // records per slice (a multiple of tile)
  float *partial;        // split x npose_space slice sums when split > 1
  long long npose_space; // pose index range of energies / partial rows
};

// Fold the slice sums of a split evaluation for the poses of each item (one block per item):
// energies[p] = 0.5 * sum_s partial[s][p], summed in slice order (as slice_reduce_kernel does).
// Poses outside the items keep their energies.
static __global__ void __launch_bounds__(256) batch_reduce_kernel(const int4 *__restrict__ items,
                                                            const float *__restrict__ partial, int split,
                                                            long long npose_space, float *__restrict__ energies) {
  const int4 it = items[blockIdx.x];
  for (int i = threadIdx.x; i < it.w; i += blockDim.x) {
    const long long p = (long long)it.z + i;
    float acc = partial[p];
    for (int s = 1; s < split; ++s) acc += partial[(long long)s * npose_space + p];
    energies[p] = 0.5f * acc;
  }
}

template <int P, int U>
__global__ void __launch_bounds__(kMaxThreads) batch_kernel(const BatchArgs a) {
  extern __shared__ __align__(128) unsigned char smem[];
  float4 *stages = reinterpret_cast<float4 *>(smem);
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + (size_t)kStages * a.tile * kRecF4 * sizeof(float4));
  __shared__ int s_item;

  const int tid = threadIdx.x;
  const int nthr = blockDim.x;
  const int n_units = a.n_items * a.split;

  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) mbar_init(&full[s], 1);
    mbar_fence_init();
  }
  __syncthreads();

  long long qg = 0; // steps already run by this block (stage = step % kStages, phase from step / kStages)
  bool failed = false;
  for (;;) {
    if (tid == 0) s_item = (int)atomicAdd(a.counter, 1u);
    __syncthreads();
    const int unit = s_item;
    __syncthreads(); // s_item is rewritten only after every thread has read it
    if (unit >= n_units) break;
    const int item = unit / a.split, sl = unit - item * a.split;
    const int4 it = __ldg(&a.items[item]);
    const float4 *lig = a.ligands + it.x;
    // Protein records [a0, a1) of this unit's slice (empty past the end of the protein).
    const int a0 = min(sl * a.slice, a.natpro_pad);
    const int a1 = min(a.natpro_pad, a0 + a.slice);
    const int ntile = (a1 - a0 + a.tile - 1) / a.tile;
    const int Q = it.y * ntile;
    const long long base = (long long)it.z + tid;
    const long long end = (long long)it.z + it.w;

    auto issue = [&](int q) {
      const int il = q / ntile;
      const int k = q - il * ntile;
      const int lt = __float_as_int(__ldg(&lig[il]).w);
      const int first = a0 + k * a.tile;
      const int cnt = min(a.tile, a1 - first);
      const int s = (int)((qg + q) % kStages);
      const uint32_t bytes = (uint32_t)cnt * kRecF4 * sizeof(float4);
      mbar_arrive_expect_tx(&full[s], bytes);
      bulk_g2s(stages + (size_t)s * a.tile * kRecF4, a.slab + ((size_t)lt * a.natpro_pad + first) * kRecF4, bytes,
               &full[s]);
    };
    if (tid == 0)
      for (int q = 0; q < min(kStages - 1, Q); ++q) issue(q);

    // The last item of a ligand is usually short: an item that fits in P/2 or P/4 poses per thread
    // runs with that many (a pose's arithmetic does not depend on the poses per thread).
    auto run = [&](auto pp) -> bool {
      pp.clear();
      int q = 0;
      for (; q < Q; ++q) {
        const int il = q / ntile;
        const int k = q - il * ntile;
        if (k == 0) pp.transform(__ldg(&lig[il]), a.xform, base, nthr, end);
        if (__syncthreads_or(failed)) break;
        if (tid == 0 && q + kStages - 1 < Q) issue(q + kStages - 1);
        const long long step = qg + q;
        const int s = (int)(step % kStages);
        if (!mbar_wait_bounded(&full[s], (uint32_t)(step / kStages) & 1u)) {
          failed = true;
          continue;
        }
        pp.template tile<U>(stages + (size_t)s * a.tile * kRecF4, min(a.tile, a1 - (a0 + k * a.tile)));
      }
      const bool ok = !__syncthreads_or(failed || q < Q);
      if (!ok) {
        if (tid == 0) {
          // Record the timeout and wait (bounded) for this block's copies still in flight.
          atomicOr(a.err, 1u);
          for (int d = max(0, q - 1); d < min(Q, q + kStages - 1); ++d)
            (void)mbar_wait_bounded(&full[(qg + d) % kStages], (uint32_t)((qg + d) / kStages) & 1u);
        }
        return false;
      }
      float *out = a.split > 1 ? a.partial + (long long)sl * a.npose_space : a.energies;
      const float scale = a.split > 1 ? 1.f : 0.5f;
#pragma unroll
      for (int i = 0; i < decltype(pp)::kP; ++i) {
        const long long pi = base + (long long)i * nthr;
        if (pi < end) out[pi] = scale * pp.energy(i);
      }
      return true;
    };
    constexpr int P2 = P >= 4 ? P / 2 : P, P4 = P >= 8 ? P / 4 : P2;
    const bool done = it.w <= P4 * nthr   ? run(PosePairs<P4>{})
                      : it.w <= P2 * nthr ? run(PosePairs<P2>{})
                                          : run(PosePairs<P>{});
    if (!done) return;
    qg += Q;
  }
}

} // namespace bude
