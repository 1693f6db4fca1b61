// ref_harness_serial.cpp -- TEST INFRASTRUCTURE ONLY (builds into oracle/_ref/libref.so).
//
// Exposes the reference's serial model, SerialBude<PPWI>::fasten (src/serial/fasten.hpp:145-211),
// behind a C symbol.  Reference headers are included in place through the include path set by
// oracle/Makefile.
// The reference headers rely on the includer for these.
#include <cmath>
#include <limits>
#include <stdexcept>
#include <string>
#include "bude.h"
#include "serial/fasten.hpp"

#include <cstring>
#include <stdexcept>

extern "C" int ref_serial_fasten(const Atom *protein, int natpro, const Atom *ligand, int natlig,
                                 const FFParams *ff, int ntypes, const float *poses, long stride, long nposes,
                                 float *energies) {
  if (nposes <= 0) return -1;
  try {
    Params p{};
    p.protein.assign(protein, protein + natpro);
    p.ligand.assign(ligand, ligand + natlig);
    p.forcefield.assign(ff, ff + ntypes);
    for (int k = 0; k < 6; k++) p.poses[k].assign(poses + k * stride, poses + k * stride + nposes);
    p.iterations = 1;
    p.warmupIterations = 0;
    SerialBude<1> bude;
    Sample s = bude.fasten(p, 1, 0);
    std::memcpy(energies, s.energies.data(), sizeof(float) * s.energies.size());
    return 0;
  } catch (const std::exception &) {
    return -3;
  }
}
