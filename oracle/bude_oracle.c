/*
 * bude_oracle.c -- CPU restatement of miniBUDE's energy kernel `fasten_main`.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: the test suite, the smoke check and the
 * `cpu_baseline` / `--impl reference` legs of bench.py load it as the checker and as the timed
 * CPU baseline.  The product path (minibude_gb300/csrc, the C-ABI library) never links, loads or
 * calls it, and there is no CPU fallback built on it.
 *
 * What it restates (reference paths are relative to the miniBUDE project root):
 *   - per-group body: src/serial/fasten.hpp:18-132 (identical arithmetic to src/omp/fasten.hpp:19-137
 *     and makedeck/ref-kernel.cpp:15-139):
 *       transform build        serial/fasten.hpp:28-53
 *       ligand atom transform  serial/fasten.hpp:56-73
 *       pair set-up            serial/fasten.hpp:75-96
 *       interaction body       serial/fasten.hpp:98-124
 *       output (0.5 * etot)    serial/fasten.hpp:129-131
 *   - parallel driver: src/omp/fasten.hpp:235-254 (`omp parallel for` over nposes/PPWI groups, each
 *     group vectorised over PPWI poses with `omp simd`).
 *   - constants: src/bude.h:22-35; record layouts: src/bude.h:39-49.
 *
 * Two precisions:
 *   oracle_fasten_f32  FP32, same expression order as the reference (the parity oracle and the
 *                      timed CPU baseline when built with the reference's release flags).
 *   oracle_fasten_f64  the same kernel in double, keeping the FP32 constants and the -FLT_MAX
 *                      sentinel (the "FP64 rerun" used to state each configuration's error).
 *
 * Differences from the reference driver, all on the caller's side:
 *   - a trailing partial group (nposes % PPWI != 0) is computed with masked lanes; the reference
 *     driver instead refuses such pose counts (src/main.cpp:525-530);
 *   - poses are passed as one SoA block with a field stride, the on-disk layout of poses.in
 *     (src/main.cpp:296-311), instead of six separate vectors.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* src/bude.h:39-42 and :44-49: packed 16-byte records. */
typedef struct {
  float x, y, z;
  int32_t type;
} oracle_atom;

typedef struct {
  int32_t hbtype;
  float radius, hphb, elsc;
} oracle_ff;

/* src/bude.h:22-35 */
#define OR_ZERO 0.0f
#define OR_QUARTER 0.25f
#define OR_HALF 0.5f
#define OR_ONE 1.0f
#define OR_TWO 2.0f
#define OR_FOUR 4.0f
#define OR_CNSTNT 45.0f
#define OR_HBTYPE_F 70
#define OR_HBTYPE_E 69
#define OR_HARDNESS 38.0f
#define OR_NPNPDIST 5.5f
#define OR_NPPDIST 1.0f

/* Poses per group; the reference's omp model is templated on this (PPWI).  Per-pose results do
 * not depend on it: every pose accumulates its own terms in the same (il, ip) order. */
#define OR_PPWI 16

#define OR_DEFINE_KERNEL(NAME, REAL, SQRT, SIN, COS, FABS)                                          \
  static void NAME##_group(int64_t first, int64_t nposes, int natlig, int natpro,                    \
                           const oracle_atom *protein, const oracle_atom *ligand,                    \
                           const float *poses, int64_t stride, const oracle_ff *ff, REAL *energies) { \
    REAL transform[3][4][OR_PPWI];                                                                   \
    REAL etot[OR_PPWI];                                                                              \
    /* serial/fasten.hpp:28-53; lanes past the end reuse the last pose and are not written. */      \
    _Pragma("omp simd") for (int l = 0; l < OR_PPWI; l++) {                                                              \
      int64_t ix = first + l < nposes ? first + l : nposes - 1;                                      \
      const REAL sx = SIN((REAL)poses[0 * stride + ix]);                                             \
      const REAL cx = COS((REAL)poses[0 * stride + ix]);                                             \
      const REAL sy = SIN((REAL)poses[1 * stride + ix]);                                             \
      const REAL cy = COS((REAL)poses[1 * stride + ix]);                                             \
      const REAL sz = SIN((REAL)poses[2 * stride + ix]);                                             \
      const REAL cz = COS((REAL)poses[2 * stride + ix]);                                             \
      transform[0][0][l] = cy * cz;                                                                  \
      transform[0][1][l] = sx * sy * cz - cx * sz;                                                   \
      transform[0][2][l] = cx * sy * cz + sx * sz;                                                   \
      transform[0][3][l] = (REAL)poses[3 * stride + ix];                                             \
      transform[1][0][l] = cy * sz;                                                                  \
      transform[1][1][l] = sx * sy * sz + cx * cz;                                                   \
      transform[1][2][l] = cx * sy * sz - sx * cz;                                                   \
      transform[1][3][l] = (REAL)poses[4 * stride + ix];                                             \
      transform[2][0][l] = -sy;                                                                      \
      transform[2][1][l] = sx * cy;                                                                  \
      transform[2][2][l] = cx * cy;                                                                  \
      transform[2][3][l] = (REAL)poses[5 * stride + ix];                                             \
      etot[l] = 0;                                                                                   \
    }                                                                                                \
    for (int il = 0; il < natlig; il++) {                                                            \
      /* serial/fasten.hpp:56-73 */                                                                 \
      const oracle_atom l_atom = ligand[il];                                                         \
      const oracle_ff l_params = ff[l_atom.type];                                                    \
      const int lhphb_ltz = l_params.hphb < 0.f;                                                     \
      const int lhphb_gtz = l_params.hphb > 0.f;                                                     \
      REAL lpos_x[OR_PPWI], lpos_y[OR_PPWI], lpos_z[OR_PPWI];                                        \
      _Pragma("omp simd") for (int l = 0; l < OR_PPWI; l++) {                                                            \
        lpos_x[l] = transform[0][3][l] + l_atom.x * transform[0][0][l] +                             \
                    l_atom.y * transform[0][1][l] + l_atom.z * transform[0][2][l];                   \
        lpos_y[l] = transform[1][3][l] + l_atom.x * transform[1][0][l] +                             \
                    l_atom.y * transform[1][1][l] + l_atom.z * transform[1][2][l];                   \
        lpos_z[l] = transform[2][3][l] + l_atom.x * transform[2][0][l] +                             \
                    l_atom.y * transform[2][1][l] + l_atom.z * transform[2][2][l];                   \
      }                                                                                              \
      for (int ip = 0; ip < natpro; ip++) {                                                          \
        /* pair set-up, serial/fasten.hpp:75-96 */                                                  \
        const oracle_atom p_atom = protein[ip];                                                      \
        const oracle_ff p_params = ff[p_atom.type];                                                  \
        const REAL radij = (REAL)p_params.radius + (REAL)l_params.radius;                            \
        const REAL r_radij = (REAL)1 / radij;                                                        \
        const int both_f = p_params.hbtype == OR_HBTYPE_F && l_params.hbtype == OR_HBTYPE_F;         \
        const REAL elcdst = both_f ? (REAL)OR_FOUR : (REAL)OR_TWO;                                   \
        const REAL elcdst1 = both_f ? (REAL)OR_QUARTER : (REAL)OR_HALF;                              \
        const int type_E = p_params.hbtype == OR_HBTYPE_E || l_params.hbtype == OR_HBTYPE_E;         \
        const int phphb_ltz = p_params.hphb < 0.f;                                                   \
        const int phphb_gtz = p_params.hphb > 0.f;                                                   \
        const int phphb_nz = p_params.hphb != 0.f;                                                   \
        const REAL p_hphb = (REAL)p_params.hphb * (phphb_ltz && lhphb_gtz ? -(REAL)1 : (REAL)1);     \
        const REAL l_hphb = (REAL)l_params.hphb * (phphb_gtz && lhphb_ltz ? -(REAL)1 : (REAL)1);     \
        const REAL distdslv =                                                                        \
            phphb_ltz ? (lhphb_ltz ? (REAL)OR_NPNPDIST : (REAL)OR_NPPDIST)                           \
                      : (lhphb_ltz ? (REAL)OR_NPPDIST : -(REAL)FLT_MAX);                             \
        const REAL r_distdslv = (REAL)1 / distdslv;                                                  \
        const REAL chrg_init = (REAL)l_params.elsc * (REAL)p_params.elsc;                            \
        const REAL dslv_init = p_hphb + l_hphb;                                                      \
        /* interaction body, serial/fasten.hpp:98-124 */                                            \
        _Pragma("omp simd") for (int l = 0; l < OR_PPWI; l++) {                                                          \
          const REAL x = lpos_x[l] - (REAL)p_atom.x;                                                 \
          const REAL y = lpos_y[l] - (REAL)p_atom.y;                                                 \
          const REAL z = lpos_z[l] - (REAL)p_atom.z;                                                 \
          const REAL distij = SQRT(x * x + y * y + z * z);                                           \
          const REAL distbb = distij - radij;                                                        \
          const int zone1 = distbb < (REAL)0;                                                        \
          etot[l] += ((REAL)1 - distij * r_radij) * (zone1 ? (REAL)2 * (REAL)OR_HARDNESS : (REAL)0); \
          REAL chrg_e = chrg_init * ((zone1 ? (REAL)1 : ((REAL)1 - distbb * elcdst1)) *              \
                                     (distbb < elcdst ? (REAL)1 : (REAL)0));                         \
          const REAL neg_chrg_e = -FABS(chrg_e);                                                     \
          chrg_e = type_E ? neg_chrg_e : chrg_e;                                                     \
          etot[l] += chrg_e * (REAL)OR_CNSTNT;                                                       \
          const REAL coeff = (REAL)1 - distbb * r_distdslv;                                          \
          REAL dslv_e = dslv_init * ((distbb < distdslv && phphb_nz) ? (REAL)1 : (REAL)0);           \
          dslv_e *= zone1 ? (REAL)1 : coeff;                                                         \
          etot[l] += dslv_e;                                                                         \
        }                                                                                            \
      }                                                                                              \
    }                                                                                                \
    /* serial/fasten.hpp:129-131 */                                                                 \
    for (int l = 0; l < OR_PPWI; l++)                                                                \
      if (first + l < nposes) energies[first + l] = etot[l] * (REAL)OR_HALF;                         \
  }

OR_DEFINE_KERNEL(or_f32, float, sqrtf, sinf, cosf, fabsf)
OR_DEFINE_KERNEL(or_f64, double, sqrt, sin, cos, fabs)

static int or_check(int natlig, int natpro, int ntypes, int64_t nposes, int64_t stride,
                    const oracle_atom *protein, const oracle_atom *ligand, const oracle_ff *ff) {
  if (natlig < 0 || natpro < 0 || ntypes <= 0 || nposes < 0 || stride < nposes) return -1;
  for (int i = 0; i < natlig; i++)
    if (ligand[i].type < 0 || ligand[i].type >= ntypes) return -2;
  for (int i = 0; i < natpro; i++)
    if (protein[i].type < 0 || protein[i].type >= ntypes) return -2;
  (void)ff;
  return 0;
}

/* Energies of `nposes` poses, FP32.  `poses` holds six float fields (tilt, roll, pan, x, y, z)
 * at `poses + k*stride`.  `nthreads` <= 0 uses the OpenMP default.  Returns 0, or a negative code
 * for bad sizes (-1) or an atom type outside the forcefield (-2). */
int oracle_fasten_f32(int natlig, int natpro, int ntypes, int64_t nposes,
                      const oracle_atom *protein, const oracle_atom *ligand, const oracle_ff *ff,
                      const float *poses, int64_t stride, float *energies, int nthreads) {
  int rc = or_check(natlig, natpro, ntypes, nposes, stride, protein, ligand, ff);
  if (rc) return rc;
  const int64_t ngroups = (nposes + OR_PPWI - 1) / OR_PPWI;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
  for (int64_t g = 0; g < ngroups; g++)
    or_f32_group(g * OR_PPWI, nposes, natlig, natpro, protein, ligand, poses, stride, ff, energies);
  (void)nthreads;
  return 0;
}

/* The same kernel evaluated in double (the FP64 rerun). */
int oracle_fasten_f64(int natlig, int natpro, int ntypes, int64_t nposes,
                      const oracle_atom *protein, const oracle_atom *ligand, const oracle_ff *ff,
                      const float *poses, int64_t stride, double *energies, int nthreads) {
  int rc = or_check(natlig, natpro, ntypes, nposes, stride, protein, ligand, ff);
  if (rc) return rc;
  const int64_t ngroups = (nposes + OR_PPWI - 1) / OR_PPWI;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
  for (int64_t g = 0; g < ngroups; g++)
    or_f64_group(g * OR_PPWI, nposes, natlig, natpro, protein, ligand, poses, stride, ff, energies);
  (void)nthreads;
  return 0;
}

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
