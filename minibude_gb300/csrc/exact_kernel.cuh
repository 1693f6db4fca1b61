// exact_kernel.cuh -- the exact miniBUDE energy kernel for sm_103a.
//
// Computes, for every pose, the energy of reference `fasten_main` (src/cuda/fasten.hpp:20-161,
// src/serial/fasten.hpp:18-132): the 3x4 pose transform, every ligand atom x every protein atom
// steric + electrostatic + desolvation term, and 0.5 * the FP32 sum.
//
// Restatement of the pair energy.  For a ligand atom of type L and a protein atom of type P at
// distance r (radij = radius_L + radius_P), the reference's three terms are piecewise linear in r
// and each one is zero past its cut-off:
//   steric   76 * (1 - r/radij)                      for r < radij
//   charge   45*c * clamp(1 - (r - radij)/elcdst, 0, 1)  (c = elsc_L*elsc_P, sign forced negative
//                                                    when either type is 'E'; elcdst 4 or 2)
//   desolv   d * clamp(1 - (r - radij)/distdslv, 0, 1)   (d = signed hphb sum; zero unless the
//                                                    protein hphb is non-zero and distdslv > 0)
// The steric factor lies in [0, 1] as well (r >= 0), so all three are one `fma.rn.sat` each with
// per-type-pair constants.  Those constants are folded into a per-ligand-type "slab" of protein
// records built once per deck on the host (64 bytes per protein atom and ligand type; the values
// used by the paired instructions below are stored twice):
//   {px, px, py, py,  pz, pz, 45*c', 45*c',  d', d', -1/radij, -1/elcdst,
//    1 + radij/elcdst, -1/distdslv, 1 + radij/distdslv, 0}
// One interaction is 3 FADD + FMUL + 2 FFMA (distance^2), one MUFU square root, 3 FFMA.SAT and
// 3 FFMA (accumulate): 12 FP32 operations against the reference's ~30.  Two poses share each
// distance and accumulate instruction through the packed `f32x2` forms, so a pose pair costs
// 9 paired + 6 saturating scalar FP32 instructions and 2 MUFU.
//
// Work decomposition.
//   * each thread holds `P` poses (poses base + i*blockDim.x, i < P, strided like the reference,
//     src/cuda/fasten.hpp:28,48,158): their transformed ligand atom and energy live in registers;
//   * every warp walks the same (ligand atom, protein atom) sequence, so each protein record is a
//     warp-uniform shared-memory broadcast (4 x LDS.128);
//   * protein records stream through a `kStages`-deep ring of shared-memory stages filled by 1-D
//     TMA bulk copies (cp.async.bulk) that complete on mbarriers, prefetched kStages-1 ahead;
//   * blockIdx.y selects a protein slice.  With split > 1 slices the partial energies are summed in
//     slice order either inside a thread-block cluster along y (rank 0 reads the other blocks'
//     partials from distributed shared memory) or, without clusters, through a global
//     [split][nposes] buffer that slice_reduce_kernel folds afterwards.  Both are deterministic.
#pragma once
#include <cooperative_groups.h>
#include <cstdint>

#include "edge_pose.cuh"
#include "exact_shape.h"
#include "ptx.cuh"

namespace bude {

constexpr float kSteric = 76.f; // 2 * HARDNESS (src/bude.h:33, serial/fasten.hpp:107)

struct ExactArgs {
  const float4 *ligand;   // natlig x {x, y, z, __int_as_float(type)}
  const float4 *slab;     // ntypes x natpro_pad x kRecF4
  const float *xform;     // nposes x 12 pose transforms (row-major 3x4, 48 bytes per pose)
  float *energies;        // nposes
  float *partial;         // split x nposes slice sums (global-reduce split), else unused
  unsigned int *err;      // bit 0: a bounded wait ran out
  long long nposes;
  int natlig;
  int natpro_pad;         // multiple of kAtomAlign
  int tile;               // atoms per stage, multiple of kAtomAlign
  int split;              // protein slices (blockIdx.y)
  int cluster;            // 1: slices reduced across a cluster; 0: through `partial`
  int slice;              // atoms per slice, multiple of kAtomAlign
};

// Pose transforms: src/cuda/fasten.hpp:45-71 / serial/fasten.hpp:28-53, one thread per pose.
// Output: three float4 rows per pose, {r00, r01, r02, tx}, {r10, r11, r12, ty}, {r20, r21, r22, tz}.
// With edge_mask, bit (i & 31) of word i >> 5 is set when pose i is irregular (edge_pose.cuh), so
// edge_pose_kernel rescores it afterwards; blockDim must be a multiple of 32.
// (Internal linkage, like slice_reduce_kernel, so several translation units may include this file.)
static __global__ void __launch_bounds__(256) pose_xform_kernel(const float *__restrict__ poses, long long pstride,
                                                         long long nposes, float4 *__restrict__ xform,
                                                         unsigned *__restrict__ edge_mask) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  bool irregular = false;
  if (i < nposes) {
    float sx, cx, sy, cy, sz, cz;
    sincosf(poses[i], &sx, &cx);
    sincosf(poses[pstride + i], &sy, &cy);
    sincosf(poses[2 * pstride + i], &sz, &cz);
    const float4 r0 = make_float4(cy * cz, sx * sy * cz - cx * sz, cx * sy * cz + sx * sz, poses[3 * pstride + i]);
    const float4 r1 = make_float4(cy * sz, sx * sy * sz + cx * cz, cx * sy * sz - sx * cz, poses[4 * pstride + i]);
    const float4 r2 = make_float4(-sy, sx * cy, cx * cy, poses[5 * pstride + i]);
    xform[3 * i + 0] = r0;
    xform[3 * i + 1] = r1;
    xform[3 * i + 2] = r2;
    irregular = !pose_regular(r0, r1, r2);
  }
  if (edge_mask) {
    const unsigned bits = __ballot_sync(0xffffffffu, irregular);
    if ((threadIdx.x & 31) == 0 && i < nposes) edge_mask[i >> 5] = bits;
  }
}


// Fold the slice sums of the global-reduce split: energies[i] = 0.5 * sum_s partial[s][i], summed
// in slice order.
static __global__ void __launch_bounds__(256) slice_reduce_kernel(const float *__restrict__ partial, int split,
                                                           long long nposes, float *__restrict__ energies) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nposes) return;
  float acc = partial[i];
  for (int s = 1; s < split; ++s) acc += partial[(long long)s * nposes + i];
  energies[i] = 0.5f * acc;
}

// Poses are processed in pairs (i = 2j, 2j+1) so the distance and accumulate steps use the packed
// f32x2 instructions; with P == 1 the second lane duplicates the first and is dropped.
template <int P> struct PosePairs {
  static constexpr int kP = P;
  static constexpr int NP = (P + 1) / 2;
  float2 e[NP], lx[NP], ly[NP], lz[NP];

  __device__ __forceinline__ void clear() {
#pragma unroll
    for (int j = 0; j < NP; ++j) e[j] = make_float2(0.f, 0.f);
  }
  __device__ __forceinline__ float energy(int i) const { return (i & 1) ? e[i / 2].y : e[i / 2].x; }

  // Transform ligand atom `la` for the thread's poses base + i*stride (serial/fasten.hpp:66-73);
  // pose indices at or past `end` read pose end-1 instead.  The transforms are re-read per ligand
  // atom (volatile loads: the compiler must not keep 12*P values live across the protein loop);
  // a block's transforms stay in L1.
  __device__ __forceinline__ void transform(float4 la, const float *xform, long long base, int stride,
                                            long long end) {
#pragma unroll
    for (int i = 0; i < 2 * NP; ++i) {
      long long pi = base + (long long)(i < P ? i : P - 1) * stride;
      pi = pi < end ? pi : end - 1;
      const float4 *t = reinterpret_cast<const float4 *>(xform) + pi * 3;
      const float4 r0 = ldg_stream(t + 0), r1 = ldg_stream(t + 1), r2 = ldg_stream(t + 2);
      const float x = r0.w + la.x * r0.x + la.y * r0.y + la.z * r0.z;
      const float y = r1.w + la.x * r1.x + la.y * r1.y + la.z * r1.z;
      const float z = r2.w + la.x * r2.x + la.y * r2.y + la.z * r2.z;
      if (i & 1) {
        lx[i / 2].y = x;
        ly[i / 2].y = y;
        lz[i / 2].y = z;
      } else {
        lx[i / 2].x = x;
        ly[i / 2].x = y;
        lz[i / 2].x = z;
      }
    }
  }

  // Accumulate the interactions with `cnt` protein records staged at `sp` (cnt a multiple of U):
  // the restated pair energy of the file comment, src/serial/fasten.hpp:98-124.
  template <int U> __device__ __forceinline__ void tile(const float4 *sp, int cnt) {
    static_assert(kAtomAlign % U == 0, "the unroll must divide the atom padding");
    const float2 steric2 = make_float2(kSteric, kSteric);
#pragma unroll 1
    for (int j0 = 0; j0 < cnt; j0 += U) {
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const float4 A = sp[(j0 + u) * kRecF4 + 0]; // px px py py
        const float4 B = sp[(j0 + u) * kRecF4 + 1]; // pz pz k_chrg k_chrg
        const float4 C = sp[(j0 + u) * kRecF4 + 2]; // k_dslv k_dslv -1/radij -1/elcdst
        const float4 D = sp[(j0 + u) * kRecF4 + 3]; // b_chrg -1/distdslv b_dslv 0
        const float2 px = make_float2(A.x, A.y), py = make_float2(A.z, A.w), pz = make_float2(B.x, B.y);
        const float2 kc = make_float2(B.z, B.w), kd = make_float2(C.x, C.y);
#pragma unroll
        for (int j = 0; j < NP; ++j) {
          const float2 dx = sub2(lx[j], px);
          const float2 dy = sub2(ly[j], py);
          const float2 dz = sub2(lz[j], pz);
          float2 d2 = mul2(dx, dx);
          d2 = fma2(dy, dy, d2);
          d2 = fma2(dz, dz, d2);
          const float2 r = make_float2(sqrt_approx(d2.x), sqrt_approx(d2.y));
          const float2 fs = make_float2(fma_sat(r.x, C.z, 1.f), fma_sat(r.y, C.z, 1.f));
          const float2 fc = make_float2(fma_sat(r.x, C.w, D.x), fma_sat(r.y, C.w, D.x));
          const float2 fd = make_float2(fma_sat(r.x, D.y, D.z), fma_sat(r.y, D.y, D.z));
          e[j] = fma2(fs, steric2, e[j]);
          e[j] = fma2(fc, kc, e[j]);
          e[j] = fma2(fd, kd, e[j]);
        }
      }
    }
  }
};

// P poses per thread; U protein atoms per unrolled inner-loop body.
template <int P, int U> __device__ __forceinline__ void exact_body(const ExactArgs &a) {
  extern __shared__ __align__(128) unsigned char smem[];
  float4 *stages = reinterpret_cast<float4 *>(smem);
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + (size_t)kStages * a.tile * kRecF4 * sizeof(float4));
  float *red = reinterpret_cast<float *>(full + kStages);

  const int tid = threadIdx.x;
  const int nthr = blockDim.x;
  const long long base = (long long)blockIdx.x * nthr * P + tid;

  // Protein slice [a0, a1) of this block.
  const int a0 = blockIdx.y * a.slice;
  const int a1 = min(a.natpro_pad, a0 + a.slice);
  const int natoms = max(0, a1 - a0);
  const int ntile = (natoms + a.tile - 1) / a.tile;
  const int Q = a.natlig * ntile; // (ligand atom, tile) steps

  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) mbar_init(&full[s], 1);
    mbar_fence_init();
  }
  __syncthreads();

  // Step q = il*ntile + k stages tile k of ligand atom il's slab row into stage q % kStages.
  auto issue = [&](int q) {
    const int il = q / ntile;
    const int k = q - il * ntile;
    const int lt = __float_as_int(__ldg(&a.ligand[il]).w);
    const int first = a0 + k * a.tile;
    const int cnt = min(a.tile, a1 - first);
    const int s = q % kStages;
    const uint32_t bytes = (uint32_t)cnt * kRecF4 * sizeof(float4);
    mbar_arrive_expect_tx(&full[s], bytes);
    bulk_g2s(stages + (size_t)s * a.tile * kRecF4, a.slab + ((size_t)lt * a.natpro_pad + first) * kRecF4, bytes,
             &full[s]);
  };
  if (tid == 0)
    for (int q = 0; q < min(kStages - 1, Q); ++q) issue(q);

  PosePairs<P> pp;
  pp.clear();

  bool failed = false;
  int q = 0;
  for (; q < Q; ++q) {
    const int il = q / ntile;
    const int k = q - il * ntile;
    if (k == 0) pp.transform(__ldg(&a.ligand[il]), a.xform, base, nthr, a.nposes);
    // Everyone is done with step q-1, so its stage may be refilled; agree on failure first.
    if (__syncthreads_or(failed)) break;
    if (tid == 0 && q + kStages - 1 < Q) issue(q + kStages - 1);
    const int s = q % kStages;
    if (!mbar_wait_bounded(&full[s], (uint32_t)(q / kStages) & 1u)) {
      failed = true;
      continue;
    }
    pp.template tile<U>(stages + (size_t)s * a.tile * kRecF4, min(a.tile, a1 - (a0 + k * a.tile)));
  }

  // A wait that ran out on any thread (including in the last step) fails the whole block.
  const bool ok = !__syncthreads_or(failed || q < Q);
  if (!ok && tid == 0) {
    // Record it, then wait (bounded) for this block's copies that may still be in flight -- steps
    // q-1 .. q+kStages-2 -- so no bulk copy lands in shared memory after the block has exited.
    atomicOr(a.err, 1u);
    for (int d = max(0, q - 1); d < min(Q, q + kStages - 1); ++d)
      (void)mbar_wait_bounded(&full[d % kStages], (uint32_t)(d / kStages) & 1u);
  }

  auto energy = [&](int i) { return pp.energy(i); };
  if (a.split == 1) {
    if (!ok) return;
#pragma unroll
    for (int i = 0; i < P; ++i) {
      const long long pi = base + (long long)i * nthr;
      if (pi < a.nposes) a.energies[pi] = 0.5f * energy(i);
    }
    return;
  }

  if (!a.cluster) {
    if (!ok) return;
    float *out = a.partial + (long long)blockIdx.y * a.nposes;
#pragma unroll
    for (int i = 0; i < P; ++i) {
      const long long pi = base + (long long)i * nthr;
      if (pi < a.nposes) out[pi] = energy(i);
    }
    return;
  }

  // Cluster reduction over protein slices (every block of the cluster reaches both barriers).
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
#pragma unroll
  for (int i = 0; i < P; ++i) red[i * nthr + tid] = energy(i);
  cluster.sync();
  if (blockIdx.y == 0 && ok) {
#pragma unroll
    for (int i = 0; i < P; ++i) {
      float acc = red[i * nthr + tid];
      for (int r = 1; r < a.split; ++r) acc += cluster.map_shared_rank(red, r)[i * nthr + tid];
      const long long pi = base + (long long)i * nthr;
      if (pi < a.nposes) a.energies[pi] = 0.5f * acc;
    }
  }
  cluster.sync();
}

// The kernel for every block size up to kMaxThreads (128 registers per thread), and the same
// kernel compiled for blocks of at most kNarrowThreads threads, kNarrowBlocks per SM (170).
template <int P, int U> __global__ void __launch_bounds__(kMaxThreads) exact_kernel(const ExactArgs a) {
  exact_body<P, U>(a);
}
template <int P, int U>
__global__ void __launch_bounds__(kNarrowThreads, kNarrowBlocks) exact_kernel_narrow(const ExactArgs a) {
  exact_body<P, U>(a);
}

} // namespace bude
