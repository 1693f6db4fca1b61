// deck_builder.h -- building miniBUDE input decks from BUDE forcefield (.bhff) and Tripos mol2
// files, with the seeded pose grid of the reference's deck generator (makedeck/).
//
// The file formats and the deck layout are the reference's (makedeck/input-utils.cpp:73-263,
// makedeck/main.cpp:12-23, 160-190); a deck written here is byte-identical to the one the
// reference's makedeck writes from the same inputs, seed and pose count, so the existing decks
// (data/bm2 was made this way) can be regenerated and new ones made from makedeck/raw.
//
// Host-only code (no CUDA); the pose energies of a deck come from the GPU library (main.cpp).
#pragma once

#include <array>
#include <cstddef>
#include <map>
#include <string>
#include <vector>

#include "minibude_gb300.h"

namespace bude_deck {

// One atom type of a forcefield residue.  `index` is the type's position inside its residue,
// which is the type index the reference writes into the atom records.
struct FFEntry {
  std::size_t index = 0;
  std::string residue;
  std::string atom_type;
  bude_ffparams params{};
};

// Residue id -> its atom types, in file order (std::map: residues sorted by id, the order in
// which the reference concatenates them into forcefield.in).
using ForceField = std::map<std::string, std::vector<FFEntry>>;

struct Molecule {
  std::vector<bude_atom> atoms;                     // heavy atoms (hydrogens skipped)
  std::vector<std::vector<bude_atom>> conformations; // @<BUDE>CONF blocks, same atom types
};

// Six pose fields: tilt, roll, pan (radians) and x, y, z translation (Angstrom).
using PoseFields = std::array<std::vector<float>, 6>;

// The reference's default pose grid: angles -170..180 step 10 degrees, translations -7..7 step 1.
PoseFields default_pose_ranges();

// Parse a .bhff forcefield.  Throws std::runtime_error naming file and line on malformed input.
ForceField read_forcefield(const std::string &path);

// The forcefield table of a deck: every residue's entries, residues in id order.
std::vector<bude_ffparams> forcefield_table(const ForceField &ff);

// Parse the atoms (and @<BUDE>CONF conformations) of a mol2 file against a forcefield.  With a
// single-residue forcefield atoms are matched by their Sybyl type (column 6, 9 columns per atom
// line); otherwise by residue (first 3 characters of column 8) and atom name (column 2), 10
// columns per line.  Throws std::runtime_error on malformed input or unknown atom types.
Molecule read_mol2(const std::string &path, const ForceField &ff);

// The order in which the six grid indices of a candidate pose are drawn.  The reference draws them
// as the arguments of one function call, an order C++ leaves to the compiler: the reference's own
// decks (data/bm2) were drawn tilt first; its generator built with GCC on x86-64 draws z first.
enum class DrawOrder { TiltFirst, ZFirst };

// `count` distinct poses drawn from the grid `ranges` (degrees for the angle fields) with a
// Mersenne-Twister seeded with `seed`; angles converted to radians.  Same draws, same
// de-duplication and same output order as the reference for the same count, seed and draw
// order.  Throws std::invalid_argument if the grid has fewer than `count` combinations.
PoseFields generate_poses(std::size_t count, std::size_t seed, const PoseFields &ranges,
                          DrawOrder order = DrawOrder::TiltFirst);

} // namespace bude_deck
