// deck_builder.cpp -- see deck_builder.h.
#include "deck_builder.h"

#include <algorithm>
#include <cmath>
#include <fstream>
#include <locale>
#include <random>
#include <sstream>
#include <stdexcept>
#include <tuple>
#include <unordered_set>

namespace bude_deck {
namespace {

struct Line {
  std::size_t number; // 1-based line number in the file
  std::string text;   // trimmed
};

bool is_space(char c) { return std::isspace<char>(c, std::locale::classic()); }

std::string trimmed(const std::string &s) {
  std::size_t b = 0, e = s.size();
  while (b < e && is_space(s[b])) ++b;
  while (e > b && is_space(s[e - 1])) --e;
  return s.substr(b, e - b);
}

std::vector<std::string> fields_of(const std::string &s) {
  std::istringstream in(s);
  std::vector<std::string> out;
  for (std::string w; in >> w;) out.push_back(w);
  return out;
}

// Non-empty lines that are not '#' or '%' comments, trimmed, with their line numbers
// (makedeck/input-utils.cpp:39-54).
std::vector<Line> data_lines(const std::string &path) {
  std::ifstream in(path);
  if (!in) throw std::runtime_error("Unable to open " + path);
  std::vector<Line> out;
  std::string raw;
  std::size_t n = 0;
  while (std::getline(in, raw)) {
    ++n;
    std::string t = trimmed(raw);
    if (t.empty() || t[0] == '#' || t[0] == '%') continue;
    out.push_back({n, std::move(t)});
  }
  return out;
}

// Run `parse` on the whitespace fields of line i; any exception becomes a parse error that names
// the file, the line and its text.
template <class F> void parse_line(const std::string &path, const std::vector<Line> &lines, std::size_t i, F &&parse) {
  if (i >= lines.size()) throw std::runtime_error("Parse error at " + path + ": unexpected end of file");
  try {
    parse(fields_of(lines[i].text));
  } catch (const std::exception &e) {
    throw std::runtime_error("Parse error at " + path + ":" + std::to_string(lines[i].number) + ": " + e.what() +
                             "(Source line: `" + lines[i].text + "`)");
  }
}

} // namespace

PoseFields default_pose_ranges() {
  std::vector<float> degs, trans;
  for (int d = -170; d <= 180; d += 10) degs.push_back((float)d);
  for (int t = -7; t <= 7; ++t) trans.push_back((float)t);
  return {degs, degs, degs, trans, trans, trans};
}

ForceField read_forcefield(const std::string &path) {
  const std::vector<Line> lines = data_lines(path);
  ForceField ff;
  // A line of exactly two fields is a residue header "<id> <count>"; the next <count> lines
  // are its atom types: name, electrostatic type (one character, stored as its ASCII code),
  // radius, hydrophobic potential, two distances (unused), radius scaling, electrostatic
  // potential.  The stored radius is radius * scaling (makedeck/input-utils.cpp:73-123).
  for (std::size_t r = 0; r < lines.size(); ++r) {
    parse_line(path, lines, r, [&](const std::vector<std::string> &head) {
      if (head.size() != 2) return;
      const std::string residue = head[0];
      const unsigned long count = std::stoul(head[1]);
      for (unsigned long b = 0; b < count; ++b)
        parse_line(path, lines, r + 1 + b, [&](const std::vector<std::string> &c) {
          if (c.size() != 9)
            throw std::runtime_error("ball row requires 9 columns, got `" + std::to_string(c.size()) + "`");
          if (c[1].size() != 1)
            throw std::runtime_error("column 2 should be a single character column, got `" + c[1] + "`");
          std::vector<FFEntry> &group = ff[residue];
          FFEntry e;
          e.index = group.size();
          e.residue = residue;
          e.atom_type = c[0];
          e.params.hbtype = static_cast<int32_t>(static_cast<unsigned char>(c[1][0]));
          const float radius = std::stof(c[2]), scaling = std::stof(c[7]);
          e.params.radius = radius * scaling;
          e.params.hphb = std::stof(c[3]);
          e.params.elsc = std::stof(c[8]);
          group.push_back(e);
        });
    });
  }
  return ff;
}

std::vector<bude_ffparams> forcefield_table(const ForceField &ff) {
  std::vector<bude_ffparams> out;
  for (const auto &kv : ff)
    for (const FFEntry &e : kv.second) out.push_back(e.params);
  return out;
}

Molecule read_mol2(const std::string &path, const ForceField &ff) {
  static const std::string kAtoms = "@<TRIPOS>ATOM", kSection = "@<TRIPOS>", kConf = "@<BUDE>CONF";
  const std::vector<Line> lines = data_lines(path);
  std::size_t begin = 0;
  while (begin < lines.size() && lines[begin].text != kAtoms) ++begin;
  if (begin == lines.size()) throw std::runtime_error("Begin atom marker(`" + kAtoms + "`) missing");
  ++begin;
  std::size_t end = begin;
  while (end < lines.size() && lines[end].text.compare(0, kSection.size(), kSection) != 0) ++end;
  if (end == lines.size()) throw std::runtime_error("End atom marker(`" + kSection + "`) missing");
  if (ff.empty()) throw std::runtime_error("empty forcefield");

  // One residue: match atoms by Sybyl type (column 6); several: by residue and atom name.
  const bool by_type = ff.size() == 1;
  Molecule mol;
  for (std::size_t i = begin; i < end; ++i)
    parse_line(path, lines, i, [&](const std::vector<std::string> &c) {
      if (by_type && c.size() != 9)
        throw std::runtime_error("forcefield contains only 1 group but " + path + " doesn't have 9 columns");
      if (!by_type && c.size() != 10)
        throw std::runtime_error("forcefield contains > 1 group but " + path + " doesn't have 10 columns");
      if (c[5] == "H" || c[5] == "h") return; // hydrogens are not scored
      const std::string type = by_type ? c[5] : c[1];
      const std::string residue = (by_type ? ff.begin()->first : c[7]).substr(0, 3);
      const float x = std::stof(c[2]), y = std::stof(c[3]), z = std::stof(c[4]);
      const auto group = ff.find(residue);
      if (group == ff.end()) throw std::runtime_error("Cannot match key " + residue + "." + type + " in forcefield.");
      const auto hit = std::find_if(group->second.begin(), group->second.end(),
                                    [&](const FFEntry &e) { return e.atom_type == type; });
      if (hit == group->second.end())
        throw std::runtime_error("Cannot match key " + residue + "." + type + " in forcefield.");
      mol.atoms.push_back(bude_atom{x, y, z, static_cast<int32_t>(hit->index)});
    });
  // "@<BUDE>CONF <n>" blocks after the atom section: one "x y z" line per parsed atom.
  for (std::size_t i = end; i < lines.size(); ++i)
    parse_line(path, lines, i, [&](const std::vector<std::string> &c) {
      if (c.size() != 2 || c[0] != kConf) return;
      std::vector<bude_atom> conf;
      for (std::size_t a = 0; a < mol.atoms.size(); ++a)
        parse_line(path, lines, i + 1 + a, [&](const std::vector<std::string> &p) {
          if (p.size() != 3) throw std::runtime_error("Conformation requires 3 columns, got " + std::to_string(p.size()));
          conf.push_back(bude_atom{std::stof(p[0]), std::stof(p[1]), std::stof(p[2]), mol.atoms[a].type});
        });
      mol.conformations.push_back(std::move(conf));
    });
  return mol;
}

PoseFields generate_poses(std::size_t count, std::size_t seed, const PoseFields &ranges, DrawOrder order) {
  std::size_t combos = 1;
  for (const auto &r : ranges) combos *= r.size();
  if (combos < count)
    throw std::invalid_argument("poseSize exceeds maximum possible pose combinations of " + std::to_string(combos));

  // Grid indices of a pose; the reference keys its de-duplicating hash set with this decimal
  // packing and iterates the set for the output order (makedeck/input-utils.cpp:205-261), so
  // the same container with the same key, hash, bucket hint and insertion sequence reproduces
  // its decks.
  using Key = std::tuple<std::size_t, std::size_t, std::size_t, std::size_t, std::size_t, std::size_t>;
  auto hash = [](const Key &k) -> std::size_t {
    return std::get<0>(k) * 100000 + std::get<1>(k) * 10000 + std::get<2>(k) * 1000 + std::get<3>(k) * 100 +
           std::get<4>(k) * 10 + std::get<5>(k);
  };
  auto equal = [](const Key &a, const Key &b) { return a == b; };
  std::unordered_set<Key, decltype(hash), decltype(equal)> picked(count, hash, equal);

  std::mt19937 gen(static_cast<std::mt19937::result_type>(seed));
  std::array<std::uniform_int_distribution<std::size_t>, 6> dist;
  for (int f = 0; f < 6; ++f) dist[f] = std::uniform_int_distribution<std::size_t>(0, ranges[f].size() - 1);
  // Tilt first reproduces data/bm2/poses.in byte for byte; z first reproduces the reference
  // generator built with GCC on x86-64.
  while (picked.size() < count) {
    std::size_t idx[6];
    if (order == DrawOrder::TiltFirst)
      for (int f = 0; f < 6; ++f) idx[f] = dist[f](gen);
    else
      for (int f = 5; f >= 0; --f) idx[f] = dist[f](gen);
    picked.emplace(idx[0], idx[1], idx[2], idx[3], idx[4], idx[5]);
  }

  const double deg_to_rad = M_PI / 180.0;
  PoseFields out;
  for (auto &v : out) v.reserve(count);
  for (const Key &k : picked) {
    out[0].push_back(static_cast<float>(ranges[0][std::get<0>(k)] * deg_to_rad));
    out[1].push_back(static_cast<float>(ranges[1][std::get<1>(k)] * deg_to_rad));
    out[2].push_back(static_cast<float>(ranges[2][std::get<2>(k)] * deg_to_rad));
    out[3].push_back(ranges[3][std::get<3>(k)]);
    out[4].push_back(ranges[4][std::get<4>(k)]);
    out[5].push_back(ranges[5][std::get<5>(k)]);
  }
  return out;
}

} // namespace bude_deck
