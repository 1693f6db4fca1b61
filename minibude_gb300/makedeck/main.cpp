// gb300-makedeck -- input decks for miniBUDE from a .bhff forcefield and protein/ligand mol2
// files, with the command line of the reference's deck generator (makedeck/main.cpp:40-150):
//
//   gb300-makedeck -f FF.bhff -p PROTEIN.mol2 -l LIGAND.mol2 -o DECK [-s SEED] [-n POSES] [--force]
//
// It writes forcefield.in, protein.in, ligand.in, poses.in and params.txt exactly as the
// reference does, and ref_energies.out (`%.5f` per pose, pose order) with the energies of the
// GPU library's exact kernel.  Options the reference does not have:
//   --no-energies       write no ref_energies.out (no GPU needed)
//   --conformations     also write ligand_conformations.in: every @<BUDE>CONF block of the ligand
//                       as natlig packed atom records, block after block (the reference parses
//                       and drops them)
//   --draw-order ORDER  `tilt-first` (default: the reference's committed decks, data/bm2) or
//                       `z-first` (the reference generator built with GCC on x86-64); the
//                       reference draws the six grid indices in its compiler's argument order
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "deck_builder.h"
#include "minibude_gb300.h"

namespace fs = std::filesystem;

namespace {

constexpr std::size_t kPoseMultiple = 256; // the reference generator's work-group size (makedeck/ref-kernel.h)

[[noreturn]] void fail(const std::string &why) {
  std::cerr << why << std::endl;
  std::exit(EXIT_FAILURE);
}

template <class T> void append_records(const fs::path &path, const std::vector<T> &xs) {
  std::ofstream out(path, std::ios::binary | std::ios::app);
  out.write(reinterpret_cast<const char *>(xs.data()), (std::streamsize)(xs.size() * sizeof(T)));
  if (!out) fail("Unable to write " + path.string());
}

void usage() {
  std::cout << "Generates input decks for miniBUDE (GB300).\n"
               "Usage: gb300-makedeck [OPTIONS]\n\n"
               "Options:\n"
               "  -h  --help           Print this message\n"
               "  -f  --forcefield     Path to a forcefield bhff file\n"
               "  -p  --protein        Path to a protein mol2 file\n"
               "  -l  --ligand         Path to a ligand mol2 file\n"
               "  -s  --pose-seed      The random seed used to generate pose combinations (default: 42)\n"
               "  -n  --pose-length    The amount of poses to generate (default: 65536)\n"
               "  -o  --out            The output directory of the deck\n"
               "      --force          Delete/overwrite an existing output path\n"
               "      --no-energies    Do not compute ref_energies.out (no GPU needed)\n"
               "      --conformations  Also write the ligand's conformations to ligand_conformations.in\n"
               "      --draw-order O   tilt-first (default, the reference's decks) or z-first (x86-64 GCC build)\n"
            << std::endl;
}

} // namespace

int main(int argc, char **argv) {
  const std::vector<std::string> args(argv + 1, argv + argc);
  std::string ff_path, protein_path, ligand_path, out_dir;
  std::size_t seed = 42, nposes = 65536;
  bool force = false, energies = true, conformations = false;
  bude_deck::DrawOrder order = bude_deck::DrawOrder::TiltFirst;

  auto value = [&](std::size_t &i, const std::string &name) -> std::string {
    if (i + 1 >= args.size()) fail("[" + name + "] specified but no value was given");
    return args[++i];
  };
  auto readable = [](const std::string &p, const std::string &what) {
    std::ifstream in(p);
    if (!in.good()) fail("Unable to open " + what + " file: `" + p + "`, is the path valid?");
    return p;
  };
  auto count = [](const std::string &v, const std::string &what) -> std::size_t {
    long long x = 0;
    try {
      x = std::stoll(v);
    } catch (...) {
      fail("malformed value, integer required for <" + what + ">: `" + v + "`");
    }
    if (x < 0) fail("positive integer required for " + what + ": `" + std::to_string(x) + "`");
    return (std::size_t)x;
  };
  for (std::size_t i = 0; i < args.size(); ++i) {
    const std::string &a = args[i];
    if (a == "-f" || a == "--forcefield") ff_path = readable(value(i, a), "forceFieldBhff");
    else if (a == "-p" || a == "--protein") protein_path = readable(value(i, a), "proteinMol2");
    else if (a == "-l" || a == "--ligand") ligand_path = readable(value(i, a), "ligandMol2");
    else if (a == "-s" || a == "--pose-seed") seed = count(value(i, a), "poseSeed");
    else if (a == "-n" || a == "--pose-length") nposes = count(value(i, a), "nPoses");
    else if (a == "-o" || a == "--out") out_dir = value(i, a);
    else if (a == "--force") force = true;
    else if (a == "--no-energies") energies = false;
    else if (a == "--conformations") conformations = true;
    else if (a == "--draw-order") {
      const std::string v = value(i, a);
      if (v == "tilt-first") order = bude_deck::DrawOrder::TiltFirst;
      else if (v == "z-first") order = bude_deck::DrawOrder::ZFirst;
      else fail("--draw-order must be tilt-first or z-first, got `" + v + "`");
    }
    else if (a == "-h" || a == "--help") {
      usage();
      return EXIT_SUCCESS;
    } else fail("Unrecognized argument '" + a + "' (try '--help')");
  }
  if (nposes % kPoseMultiple != 0)
    fail("poseSize(" + std::to_string(nposes) + ") cannot be divided by WGSIZE(" + std::to_string(kPoseMultiple) + ")");
  if (ff_path.empty()) fail("--forcefield is a required parameter");
  if (protein_path.empty()) fail("--protein is a required parameter");
  if (ligand_path.empty()) fail("--ligand is a required parameter");
  if (out_dir.empty()) fail("--out is a required parameter");

  const fs::path out(out_dir);
  if (fs::is_regular_file(out) || fs::is_directory(out)) {
    if (!force) fail("Output path already exists (either a file or directory), pass --force to delete/overwrite them");
    fs::remove_all(out);
  }
  if (!fs::create_directories(out)) fail("Unable to create output directory: " + out.string());

  try {
    const bude_deck::ForceField ff = bude_deck::read_forcefield(ff_path);
    const std::vector<bude_ffparams> table = bude_deck::forcefield_table(ff);
    const bude_deck::Molecule protein = bude_deck::read_mol2(protein_path, ff);
    const bude_deck::Molecule ligand = bude_deck::read_mol2(ligand_path, ff);
    append_records(out / "forcefield.in", table);
    append_records(out / "protein.in", protein.atoms);
    append_records(out / "ligand.in", ligand.atoms);
    const bude_deck::PoseFields poses = bude_deck::generate_poses(nposes, seed, bude_deck::default_pose_ranges(), order);
    for (const auto &f : poses) append_records(out / "poses.in", f);
    if (conformations)
      for (const auto &c : ligand.conformations) append_records(out / "ligand_conformations.in", c);

    {
      std::ofstream params(out / "params.txt");
      for (const std::string &a : args) params << a << " ";
      params << std::endl;
    }
    std::cout << "- Forcefield: " << ff.size() << " residue(s), " << table.size() << " atom type(s)\n"
              << "- Protein: " << protein.atoms.size() << " atom(s), " << protein.conformations.size()
              << " conformation(s)\n"
              << "- Ligand: " << ligand.atoms.size() << " atom(s), " << ligand.conformations.size()
              << " conformation(s)\n"
              << "- Poses: " << nposes << " (seed=" << seed << ")" << std::endl;

    if (energies) {
      // The six pose fields back to back: the SoA layout of poses.in, stride nposes.
      std::vector<float> soa;
      soa.reserve(6 * nposes);
      for (const auto &f : poses) soa.insert(soa.end(), f.begin(), f.end());
      std::vector<float> e(nposes);
      bude_launch_cfg cfg{};
      bude_gpu_ctx *ctx = nullptr;
      int rc = bude_gpu_create(0, &ctx);
      if (!rc) rc = bude_gpu_upload(ctx, protein.atoms.data(), (int32_t)protein.atoms.size(), ligand.atoms.data(),
                                    (int32_t)ligand.atoms.size(), table.data(), (int32_t)table.size(), soa.data(),
                                    (int64_t)nposes, (int64_t)nposes);
      if (!rc) rc = bude_gpu_default_cfg(ctx, 16, 256, &cfg);
      if (!rc) rc = bude_gpu_run(ctx, &cfg, nullptr);
      if (!rc) rc = bude_gpu_download(ctx, e.data(), (int64_t)nposes);
      if (ctx) bude_gpu_destroy(ctx);
      if (rc) fail(std::string("Energy evaluation failed: ") + bude_gpu_last_error());
      std::ofstream ref(out / "ref_energies.out");
      ref << std::fixed << std::setprecision(5);
      for (float v : e) ref << v << "\n";
      std::cout << "- Reference energy: " << e.size() << " lines (GPU exact kernel)" << std::endl;
    }
  } catch (const std::exception &ex) {
    fail(ex.what());
  }
  std::cout << "Done" << std::endl;
  return EXIT_SUCCESS;
}
