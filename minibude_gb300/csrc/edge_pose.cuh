// edge_pose.cuh -- poses and decks outside the range where exact_kernel's restated pair energy is
// the reference's, and the kernel that scores them with the reference's own arithmetic.
//
// exact_kernel.cuh evaluates each pair term as one saturating FMA (fma.rn.sat.f32), which turns a
// NaN into +0 and relies on radij > 0.  The reference (src/serial/fasten.hpp:98-124) instead
// propagates non-finite values: a NaN or infinite pose, a translation large enough that
// x*x + y*y + z*z overflows (|d| > ~1.8e19 A), or a radius sum of zero gives a NaN energy, and a
// negative radius sum gives a different steric term.  The saturating form is exact only inside
// these bounds, which are checked once per pose and once per deck:
//
//   regular pose   its transform is finite (sin/cos of finite angles) and every translation
//                  component satisfies |t| < 2^38 A                    (pose_xform_kernel)
//   regular deck   every protein coordinate |p| <= 2^37 A, every ligand atom |x|+|y|+|z| <= 2^36 A,
//                  every forcefield radius, hphb and elsc in use finite with magnitude <= 2^20,
//                  and every FP32 radius sum radius_L + radius_P >= 2^-20     (host or device check)
//
// Inside them every ligand-protein distance is below 2^39 A (no overflow, nothing non-finite) and
// the padding records at 1e15 A stay out of reach, so the saturating form equals the reference's
// piecewise terms.  Everything else -- the irregular poses (one bit each in a mask written by the
// transform pass), or every pose of an irregular deck or ligand -- is rescored afterwards by
// edge_pose_kernel: one warp per pose, the reference's pair set-up and interaction body in FP32
// over the raw protein and forcefield records, lanes striding over protein atoms, and a fixed-order
// warp reduction.  It overwrites those poses' energies, so NaN and infinity come out where the
// reference's serial model gives them.  Regular decks of regular poses (every deck the reference
// ships) never take this path; it costs one launch that reads the mask.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>

#include <cuda_runtime.h>

#include "../../include/minibude_gb300.h"

namespace bude {

constexpr float kPoseReach = 0x1p38f;    // |translation| bound of a regular pose
constexpr float kProteinReach = 0x1p37f;  // |coordinate| bound of a protein atom in a regular deck
constexpr float kLigandReach = 0x1p36f;   // |x|+|y|+|z| bound of a ligand atom in a regular deck
constexpr float kParamReach = 0x1p20f;    // |radius|, |hphb|, |elsc| bound in a regular deck
constexpr float kMinRadiusSum = 0x1p-20f; // smallest FP32 radius sum of a regular deck

// A pose whose transform rows {r00, r01, r02, tx}, ... keep exact_kernel exact (NaN fails every
// comparison, so a non-finite transform is irregular).
__host__ __device__ __forceinline__ bool pose_regular(float4 r0, float4 r1, float4 r2) {
  const float rs = fabsf(r0.x) + fabsf(r0.y) + fabsf(r0.z) + fabsf(r1.x) + fabsf(r1.y) + fabsf(r1.z) + fabsf(r2.x) +
                   fabsf(r2.y) + fabsf(r2.z);
  return rs < 64.f && fabsf(r0.w) < kPoseReach && fabsf(r1.w) < kPoseReach && fabsf(r2.w) < kPoseReach;
}

// Deck bounds of one forcefield record in use, one protein atom, one ligand atom.
__host__ __device__ __forceinline__ bool param_regular(const bude_ffparams &f) {
  return fabsf(f.radius) <= kParamReach && fabsf(f.hphb) <= kParamReach && fabsf(f.elsc) <= kParamReach;
}
__host__ __device__ __forceinline__ bool protein_atom_regular(const bude_atom &a) {
  return fabsf(a.x) <= kProteinReach && fabsf(a.y) <= kProteinReach && fabsf(a.z) <= kProteinReach;
}
__host__ __device__ __forceinline__ bool ligand_atom_regular(float x, float y, float z) {
  return fabsf(x) + fabsf(y) + fabsf(z) <= kLigandReach;
}

// One ligand-protein term of the reference, src/serial/fasten.hpp:80-124 (pair set-up and
// interaction body), in FP32 with the reference's constants (src/bude.h:22-35).
__device__ __forceinline__ float ref_pair_energy(const bude_ffparams &l, float lx, float ly, float lz,
                                                 const bude_atom &pa, const bude_ffparams &p) {
  const bool l_ltz = l.hphb < 0.f, l_gtz = l.hphb > 0.f;
  const float radij = p.radius + l.radius;
  const float r_radij = 1.f / radij;
  const bool both_f = p.hbtype == 70 && l.hbtype == 70;
  const float elcdst = both_f ? 4.f : 2.f;
  const float elcdst1 = both_f ? 0.25f : 0.5f;
  const bool type_e = p.hbtype == 69 || l.hbtype == 69;
  const bool p_ltz = p.hphb < 0.f, p_gtz = p.hphb > 0.f, p_nz = p.hphb != 0.f;
  const float p_hphb = p.hphb * ((p_ltz && l_gtz) ? -1.f : 1.f);
  const float l_hphb = l.hphb * ((p_gtz && l_ltz) ? -1.f : 1.f);
  const float distdslv = p_ltz ? (l_ltz ? 5.5f : 1.f) : (l_ltz ? 1.f : -3.40282347e38f);
  const float r_distdslv = 1.f / distdslv;
  const float chrg_init = l.elsc * p.elsc;
  const float dslv_init = p_hphb + l_hphb;

  const float x = lx - pa.x, y = ly - pa.y, z = lz - pa.z;
  const float distij = sqrtf(x * x + y * y + z * z);
  const float distbb = distij - radij;
  const bool zone1 = distbb < 0.f;
  float e = (1.f - distij * r_radij) * (zone1 ? 76.f : 0.f);
  float chrg_e = chrg_init * ((zone1 ? 1.f : (1.f - distbb * elcdst1)) * (distbb < elcdst ? 1.f : 0.f));
  chrg_e = type_e ? -fabsf(chrg_e) : chrg_e;
  e += chrg_e * 45.f;
  const float coeff = 1.f - distbb * r_distdslv;
  float dslv_e = dslv_init * ((distbb < distdslv && p_nz) ? 1.f : 0.f);
  dslv_e *= zone1 ? 1.f : coeff;
  return e + dslv_e;
}

struct EdgeArgs {
  const unsigned *mask;         // bit (p & 31) of word p >> 5: pose p is irregular (pose_xform_kernel)
  int all;                      // 1: every pose is rescored (the deck is irregular)
  long long nposes;
  // Batches: pose_off / lig_off (nlig + 1 entries, device) give each ligand's poses and atoms;
  // lig_any (device) counts the irregular ligands and lig_all (device, nlig bytes) marks them.
  // One ligand: pose_off == nullptr, its atoms are ligand[0, natlig).
  const long long *pose_off;
  const int *lig_off;
  const int *lig_any;
  const unsigned char *lig_all;
  int nlig;
  const float4 *ligand; // {x, y, z, __int_as_float(type)}
  int natlig;
  const bude_atom *protein; // raw records
  int natpro;
  const bude_ffparams *ff;
  const float *xform;     // 12 floats per pose
  float *energies;        // overwritten for the rescored poses
  unsigned char *flag;    // optional: set to 1 for the rescored poses
};

// Ligand of pose p in a batch (pose_off ascending; ligands without poses are skipped).
static __device__ __forceinline__ int edge_ligand_of(const long long *pose_off, int nlig, long long p) {
  int lo = 0, hi = nlig - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (pose_off[mid] <= p) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Energy of pose p by the reference's arithmetic, computed by the whole warp; valid in lane 0.
static __device__ float edge_energy(const EdgeArgs &a, long long p) {
  const int lane = threadIdx.x & 31;
  int l0 = 0, nl = a.natlig;
  if (a.pose_off) {
    const int l = edge_ligand_of(a.pose_off, a.nlig, p);
    l0 = a.lig_off[l];
    nl = a.lig_off[l + 1] - l0;
  }
  const float4 *t = reinterpret_cast<const float4 *>(a.xform) + p * 3;
  const float4 r0 = t[0], r1 = t[1], r2 = t[2];
  float acc = 0.f;
  for (int il = 0; il < nl; ++il) {
    const float4 la = a.ligand[l0 + il];
    const bude_ffparams lp = a.ff[__float_as_int(la.w)];
    // serial/fasten.hpp:66-73
    const float lx = r0.w + la.x * r0.x + la.y * r0.y + la.z * r0.z;
    const float ly = r1.w + la.x * r1.x + la.y * r1.y + la.z * r1.z;
    const float lz = r2.w + la.x * r2.x + la.y * r2.y + la.z * r2.z;
    for (int ip = lane; ip < a.natpro; ip += 32) {
      const bude_atom pa = a.protein[ip];
      acc += ref_pair_energy(lp, lx, ly, lz, pa, a.ff[pa.type]);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  return 0.5f * acc;
}

// Rescore the irregular poses: warp w takes mask words w, w + warps, ...; every set bit (and, for
// an irregular deck or ligand, every pose) is one warp-wide evaluation.
static __global__ void __launch_bounds__(256) edge_pose_kernel(const EdgeArgs a) {
  const int lane = threadIdx.x & 31;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  const long long nwords = (a.nposes + 31) >> 5;
  const bool any_lig = a.pose_off && a.lig_all && a.lig_any && *a.lig_any > 0;
  for (long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nwords; w += nwarps) {
    const long long first = w << 5;
    const int valid = (int)min(32LL, a.nposes - first);
    const unsigned vmask = valid == 32 ? 0xffffffffu : ((1u << valid) - 1u);
    unsigned bits = a.all ? vmask : (a.mask[w] & vmask);
    if (any_lig) {
      // Poses of irregular ligands inside this word.
      int l = edge_ligand_of(a.pose_off, a.nlig, first);
      for (; l < a.nlig && a.pose_off[l] < first + valid; ++l) {
        if (!a.lig_all[l]) continue;
        const long long b0 = max(a.pose_off[l], first) - first, b1 = min(a.pose_off[l + 1], first + valid) - first;
        for (long long b = b0; b < b1; ++b) bits |= 1u << b;
      }
    }
    while (bits) {
      const int b = __ffs(bits) - 1;
      bits &= bits - 1u;
      const long long p = first + b;
      const float e = edge_energy(a, p);
      if (lane == 0) {
        a.energies[p] = e;
        if (a.flag) a.flag[p] = 1;
      }
    }
  }
}

// Grid of edge_pose_kernel for n poses on `sms` SMs.
inline unsigned edge_grid(long long n, int sms) {
  const long long words = (n + 31) / 32;
  const long long blocks = (words + 7) / 8; // 8 warps per block
  return (unsigned)std::max(1LL, std::min(blocks, 8LL * std::max(sms, 1)));
}

} // namespace bude
