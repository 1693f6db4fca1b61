// ref_harness_omp.cpp -- TEST INFRASTRUCTURE ONLY (builds oracle/_ref/libref.so).
//
// Exposes the reference's own OpenMP model, OmpBude<PPWI>::fasten (src/omp/fasten.hpp:182-264),
// behind a C symbol so the test-fixture script can produce golden energies from the unmodified
// reference code.  The reference headers are included from where they lie in the reference tree
// (the include path is set by oracle/Makefile); nothing of them is copied here.
// The reference headers rely on the includer for these.
#include <cmath>
#include <limits>
#include <stdexcept>
#include <string>
#include "bude.h"
#include "omp/fasten.hpp"

#include <cstring>
#include <stdexcept>

template <size_t P>
static int run_ref(const Params &p, float *energies) {
  OmpBude<P> bude;
  Sample s = bude.fasten(p, 1, 0);
  std::memcpy(energies, s.energies.data(), sizeof(float) * s.energies.size());
  return 0;
}

static Params make_params(const Atom *protein, int natpro, const Atom *ligand, int natlig,
                          const FFParams *ff, int ntypes, const float *poses, long stride, long nposes) {
  Params p{};
  p.protein.assign(protein, protein + natpro);
  p.ligand.assign(ligand, ligand + natlig);
  p.forcefield.assign(ff, ff + ntypes);
  for (int k = 0; k < 6; k++) p.poses[k].assign(poses + k * stride, poses + k * stride + nposes);
  p.iterations = 1;
  p.warmupIterations = 0;
  return p;
}

// Energies from the reference OpenMP model for one PPWI.  nposes must be a multiple of ppwi (the
// reference driver's own rule, src/main.cpp:525-530).  Returns 0, -1 for a bad ppwi/size, -3 if the
// reference threw.
extern "C" int ref_omp_fasten(int ppwi, const Atom *protein, int natpro, const Atom *ligand, int natlig,
                              const FFParams *ff, int ntypes, const float *poses, long stride, long nposes,
                              float *energies) {
  if (nposes <= 0 || ppwi <= 0 || nposes % ppwi != 0) return -1;
  try {
    Params p = make_params(protein, natpro, ligand, natlig, ff, ntypes, poses, stride, nposes);
    switch (ppwi) {
    case 1: return run_ref<1>(p, energies);
    case 4: return run_ref<4>(p, energies);
    case 16: return run_ref<16>(p, energies);
    case 64: return run_ref<64>(p, energies);
    default: return -1;
    }
  } catch (const std::exception &) {
    return -3;
  }
}
