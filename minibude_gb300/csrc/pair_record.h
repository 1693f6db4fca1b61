// pair_record.h -- the per-(ligand type, protein atom) record the exact kernel streams.
//
// Restates the reference's pair set-up (src/serial/fasten.hpp:80-96, constants src/bude.h:22-35)
// as the constants of the three saturating FMAs of exact_kernel.cuh.  Usable from host and device
// code; the derived constants are evaluated in double with explicit fma and rounded to float once,
// so host and device builds of a record are bit-identical.
#pragma once
#include <cfloat>
#include <cmath>

#include "../../include/minibude_gb300.h"

#ifdef __CUDACC__
#define BUDE_HD __host__ __device__
#else
#define BUDE_HD
#endif

namespace bude {

constexpr int kHbtypeF = 70;      // 'F' (src/bude.h:31)
constexpr int kHbtypeE = 69;      // 'E' (src/bude.h:32)
constexpr float kCnstnt = 45.0f; // src/bude.h:28
constexpr float kNpNpDist = 5.5f; // src/bude.h:34
constexpr float kNpPDist = 1.0f;  // src/bude.h:35
constexpr int kRecFloats = 16;    // floats per record (exact_shape.h: kRecF4 * 4)

// rec[0..15] = {px, px, py, py, pz, pz, k_chrg, k_chrg, k_dslv, k_dslv, -1/radij, -1/elcdst,
//               1 + radij/elcdst, -1/distdslv, 1 + radij/distdslv, 0}
BUDE_HD inline void pair_record(const bude_ffparams &L, const bude_ffparams &Pp, float px, float py, float pz,
                                float *rec) {
  const float radij = Pp.radius + L.radius; // FP32 sum, as the reference
  const bool both_f = Pp.hbtype == kHbtypeF && L.hbtype == kHbtypeF;
  const double elcdst1 = both_f ? 0.25 : 0.5;
  const bool type_e = Pp.hbtype == kHbtypeE || L.hbtype == kHbtypeE;
  const bool p_ltz = Pp.hphb < 0.f, p_gtz = Pp.hphb > 0.f, p_nz = Pp.hphb != 0.f;
  const bool l_ltz = L.hphb < 0.f, l_gtz = L.hphb > 0.f;
  const float p_hphb = Pp.hphb * ((p_ltz && l_gtz) ? -1.f : 1.f);
  const float l_hphb = L.hphb * ((p_gtz && l_ltz) ? -1.f : 1.f);
  const float distdslv = p_ltz ? (l_ltz ? kNpNpDist : kNpPDist) : (l_ltz ? kNpPDist : -FLT_MAX);
  const bool dslv_on = p_nz && distdslv > 0.f; // -FLT_MAX distance: the term can never fire
  const double r_distdslv = dslv_on ? 1.0 / (double)distdslv : 1.0;
  const float chrg_init = L.elsc * Pp.elsc;
  const float dslv_init = p_hphb + l_hphb;
  const float k_chrg = kCnstnt * (type_e ? -fabsf(chrg_init) : chrg_init);
  const float k_dslv = dslv_on ? dslv_init : 0.f;
  rec[0] = rec[1] = px;
  rec[2] = rec[3] = py;
  rec[4] = rec[5] = pz;
  rec[6] = rec[7] = k_chrg;
  rec[8] = rec[9] = k_dslv;
  rec[10] = (float)(-1.0 / (double)radij);
  rec[11] = (float)(-elcdst1);
  rec[12] = (float)fma((double)radij, elcdst1, 1.0);
  rec[13] = (float)(-r_distdslv);
  rec[14] = dslv_on ? (float)fma((double)radij, r_distdslv, 1.0) : 0.f;
  rec[15] = 0.f;
}

// A padding atom: far away (every saturating factor is 0) with zero charge/desolvation weights.
BUDE_HD inline void null_record(float *rec) {
  const float far = 1.0e15f;
  for (int i = 0; i < 6; ++i) rec[i] = far;
  for (int i = 6; i < 10; ++i) rec[i] = 0.f;
  rec[10] = rec[11] = rec[13] = -1.f;
  rec[12] = rec[14] = rec[15] = 0.f;
}

} // namespace bude
