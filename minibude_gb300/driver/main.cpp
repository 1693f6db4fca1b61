// main.cpp -- the gb300-bude driver: the reference driver's command line, deck loader, PPWI x
// wgsize sweep, validation and YAML/CSV report (reference src/main.cpp:153-655), written for the
// GB300 model (gb300/fasten.hpp) and its C-ABI library.
//
// Contract kept from the reference:
//   options   -d/--device -i/--iter -n/--poses -p/--ppwi (CSV or `all`) -w/--wgsize (CSV) --deck
//             -o/--out -r/--rows --csv -l/--list -h/--help, defaults 8 iterations, 2 warm-ups,
//             ../data/bm1, ppwi 1, wgsize 1 (src/main.cpp:153-281)
//   deck      readNStruct semantics (a trailing partial record is dropped), poses.in as six
//             blocks of maxPoses floats, `-n` truncation, ref_energies.out one value per line,
//             and the same std::invalid_argument cases (src/main.cpp:138-151, 283-322)
//   checks    max_diff_% with the signed-reference difference and the |x| < 1 skip, valid below
//             DIFF_TOLERANCE_PCT (src/main.cpp:329-342, 371)
//   report    the YAML keys outcome/param/raw_iterations/context_ms/sum..stddev_ms/
//             giga_interactions/s/gflop/s/gfinst/s/energies/best and the CSV columns
//             (src/main.cpp:431-476, 550-559); exit status = all results valid
// Additions: `max_diff_abs_%` (the validator with |ref| in the denominator), `fp32_peak_%` (the
// reference's per-interaction operation count over the device's FP32 peak) and `-w 0` for the
// library's automatic launch shape.  Pose counts that are not a multiple of ppwi*wgsize run
// (the kernel handles ragged tails) instead of being skipped.
#include "bude.h"
#include "gb300/fasten.hpp"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <ctime>
#include <fstream>
#include <functional>
#include <iomanip>
#include <iostream>
#include <map>
#include <memory>
#include <numeric>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#if __has_include("meta_build.h")
#include "meta_build.h" // written by the build: version, compile commands, git state
#endif
#ifndef GB300_BUDE_VERSION
#define GB300_BUDE_VERSION "0.1"
#define GB300_BUDE_COMPILE_COMMANDS {}
#define GB300_BUDE_VCS_RETRIEVED_STATE 0
#endif

namespace {

constexpr size_t kPPWIs[] = {1, 2, 4, 8, 16, 32, 64, 128};

struct Stats {
  double min = 0, max = 0, sum = 0, mean = 0, stddev = 0;
  static Stats of(const std::vector<double> &v) {
    Stats s;
    if (v.empty()) return s;
    s.min = *std::min_element(v.begin(), v.end());
    s.max = *std::max_element(v.begin(), v.end());
    s.sum = std::accumulate(v.begin(), v.end(), 0.0);
    s.mean = s.sum / double(v.size());
    double var = 0;
    for (double x : v) var += (x - s.mean) * (x - s.mean);
    s.stddev = std::sqrt(var / double(v.size()));
    return s;
  }
};

struct Outcome {
  bool valid = false;
  double maxDiffPct = 0, maxDiffAbsPct = 0;
  Sample sample;
  Stats ms;
  double gflops = 0, ginsts = 0, interactionsPerSec = 0, fp32PeakPct = 0;
  explicit Outcome(Sample s) : sample(std::move(s)) {}
};

[[noreturn]] void die(const std::string &msg) {
  std::cerr << msg << std::endl;
  std::exit(EXIT_FAILURE);
}

size_t parseCount(const std::string &text, const std::string &what) {
  long v = 0;
  try {
    size_t used = 0;
    v = std::stol(text, &used);
  } catch (...) {
    die("malformed value, integer required for <" + what + ">: `" + text + "`");
  }
  if (v < 0) die("positive integer required for <" + what + ">: `" + text + "`");
  return size_t(v);
}

std::vector<size_t> parseCounts(const std::string &text, const std::string &what) {
  std::vector<size_t> out;
  std::stringstream ss(text);
  std::string item;
  while (std::getline(ss, item, ',')) out.push_back(parseCount(item, what));
  return out;
}

template <typename T> std::vector<T> readRecords(const std::string &path) {
  std::ifstream in(path, std::ios::binary);
  if (!in.good()) throw std::invalid_argument("Bad file: " + path);
  std::vector<char> bytes((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
  std::vector<T> out(bytes.size() / sizeof(T));
  if (!out.empty()) std::memcpy(out.data(), bytes.data(), out.size() * sizeof(T));
  return out;
}

template <typename C> std::string joined(const C &xs, const std::string &sep = ",") {
  std::ostringstream o;
  bool first = true;
  for (const auto &x : xs) {
    if (!first) o << sep;
    o << x;
    first = false;
  }
  return o.str();
}

void usage() {
  std::cout << "\nUsage: ./gb300-bude [COMMAND|OPTIONS]\n\n"
            << "Commands:\n"
            << "  help -h --help       Print this message\n"
            << "  list -l --list       List available devices\n"
            << "Options:\n"
            << "  -d --device  INDEX   Device index from --list, or a substring of its name [default 0]\n"
            << "  -i --iter    I       Repeat the kernel I times [default " << DEFAULT_ITERS << "]\n"
            << "  -n --poses   N       Compute energies for only N poses, 0 for the whole deck [default 0]\n"
            << "  -p --ppwi    PPWI    CSV list of poses per work-item, or `all` [default 1; available "
            << joined(kPPWIs) << "]\n"
            << "  -w --wgsize  WGSIZE  CSV list of work-group sizes, 0 = automatic launch shape [default 1]\n"
            << "     --deck    DIR     Input deck directory [default `" << DATA_DIR << "`]\n"
            << "  -o --out     PATH    Save energies of the first result to PATH\n"
            << "  -r --rows    N       Show the first N energies of each result [default " << DEFAULT_ENERGY_ENTRIES
            << "]\n"
            << "     --csv             CSV output\n"
            << std::endl;
}

struct Cli {
  Params params{};
  std::vector<size_t> ppwis, wgsizes;
};

Cli parse(const std::vector<std::string> &args) {
  Cli cli;
  Params &p = cli.params;
  p.iterations = DEFAULT_ITERS;
  p.warmupIterations = 2;
  p.deckDir = DATA_DIR;
  p.outRows = DEFAULT_ENERGY_ENTRIES;
  p.csv = false;
  p.list = false;
  size_t nposes = 0;
  for (size_t i = 0; i < args.size(); ++i) {
    const std::string &a = args[i];
    auto value = [&](std::initializer_list<const char *> names) -> const std::string * {
      for (const char *n : names)
        if (a == n) {
          if (i + 1 >= args.size()) die("[" + a + "] specified but no value was given");
          return &args[++i];
        }
      return nullptr;
    };
    if (auto v = value({"--iter", "-i"})) p.iterations = parseCount(*v, "iter");
    else if (auto v = value({"--poses", "-n"})) nposes = parseCount(*v, "poses");
    else if (auto v = value({"--device", "-d"})) p.deviceSelector = *v;
    else if (auto v = value({"--deck"})) p.deckDir = *v;
    else if (auto v = value({"--out", "-o"})) p.output = *v;
    else if (auto v = value({"--rows", "-r"})) p.outRows = parseCount(*v, "rows");
    else if (auto v = value({"--wgsize", "-w"})) cli.wgsizes = parseCounts(*v, "wgsize");
    else if (auto v = value({"--ppwi", "-p"})) {
      if (*v == "all") cli.ppwis.assign(std::begin(kPPWIs), std::end(kPPWIs));
      else {
        cli.ppwis = parseCounts(*v, "ppwi");
        for (size_t x : cli.ppwis)
          if (std::find(std::begin(kPPWIs), std::end(kPPWIs), x) == std::end(kPPWIs))
            die("PPWI " + std::to_string(x) + " is not a supported value, should be one of `" + joined(kPPWIs) + "`");
      }
    } else if (a == "--csv") p.csv = true;
    else if (a == "list" || a == "--list" || a == "-l") p.list = true;
    else if (a == "help" || a == "--help" || a == "-h") {
      usage();
      std::exit(EXIT_SUCCESS);
    } else {
      std::cout << "Unrecognized argument '" << a << "' (try '--help')" << std::endl;
      std::exit(EXIT_FAILURE);
    }
  }
  if (cli.ppwis.empty()) cli.ppwis = {kPPWIs[0]};
  if (cli.wgsizes.empty()) cli.wgsizes = {1};
  if (p.list) return cli;

  p.ligand = readRecords<Atom>(p.deckDir + FILE_LIGAND);
  p.protein = readRecords<Atom>(p.deckDir + FILE_PROTEIN);
  p.forcefield = readRecords<FFParams>(p.deckDir + FILE_FORCEFIELD);
  const std::vector<float> flat = readRecords<float>(p.deckDir + FILE_POSES);
  if (flat.size() % 6 != 0)
    throw std::invalid_argument("Pose size (" + std::to_string(flat.size()) + ") not divisible my 6!");
  p.maxPoses = flat.size() / 6;
  if (nposes == 0) nposes = p.maxPoses;
  if (nposes > p.maxPoses)
    throw std::invalid_argument("Requested poses (" + std::to_string(nposes) + ") exceeded max poses (" +
                                std::to_string(p.maxPoses) + ") for deck");
  for (size_t k = 0; k < 6; ++k)
    p.poses[k].assign(flat.begin() + long(k * p.maxPoses), flat.begin() + long(k * p.maxPoses + nposes));
  std::ifstream refs(p.deckDir + FILE_REF_ENERGIES);
  std::string line;
  while (std::getline(refs, line)) p.refEnergies.push_back(std::stof(line));
  if (p.nposes() > p.refEnergies.size())
    throw std::invalid_argument("Size of reference energies (" + std::to_string(p.refEnergies.size()) +
                                ") is less than poses (" + std::to_string(p.nposes()) + ")");
  return cli;
}

// The reference's difference: signed reference in the denominator.
double signedDiff(float ref, float e) { return std::fabs(double(ref) - e) / ref; }

void check(const Params &p, Outcome &r, std::vector<size_t> &failed) {
  double maxDiff = 0, maxAbs = 0;
  for (size_t i = 0; i < r.sample.energies.size(); ++i) {
    const float ref = p.refEnergies[i], e = r.sample.energies[i];
    if (std::fabs(ref) < 1.f && std::fabs(e) < 1.f) continue;
    const double d = signedDiff(ref, e);
    if (d > maxDiff) maxDiff = d;
    const double da = std::fabs(double(ref) - e) / std::fabs(double(ref));
    if (da > maxAbs) maxAbs = da;
    if (100.0 * d > DIFF_TOLERANCE_PCT) failed.push_back(i);
  }
  r.maxDiffPct = 100.0 * maxDiff;
  r.maxDiffAbsPct = 100.0 * maxAbs;
  r.valid = r.maxDiffPct < DIFF_TOLERANCE_PCT;
}

double fp32PeakFlops(size_t device) {
  int sms = 0;
  if (bude_gpu_sm_count(int(device), &sms) != BUDE_OK) return 0;
  return double(sms) * 128.0 * 2.0 * 2070e6; // nominal: 128 FP32 lanes per SM at the 2070 MHz max clock
}

Outcome evaluate(const Params &p, Sample s, size_t device, bool verbose) {
  if (s.kernelTimes.empty()) throw std::logic_error("Sample size is 0, this implementation did not measure kernel runtime!");
  Outcome r(std::move(s));
  std::vector<double> ms;
  for (size_t i = p.warmupIterations; i < r.sample.kernelTimes.size(); ++i)
    ms.push_back(elapsedMillis(r.sample.kernelTimes[i].first, r.sample.kernelTimes[i].second));
  std::vector<size_t> failed;
  check(p, r, failed);
  if (!r.valid) {
    if (verbose) {
      std::cerr << "# Verification failed for ppwi=" << r.sample.ppwi << ", wgsize=" << r.sample.wgsize
                << "; difference exceeded tolerance (" << DIFF_TOLERANCE_PCT << "%)\n"
                << "# Bad energies (failed/total=" << failed.size() << "/" << r.sample.energies.size()
                << ", showing first " << std::min(failed.size(), p.outRows) << "): \n"
                << "# index,actual,expected,difference_%\n";
      for (size_t i = 0; i < std::min(failed.size(), p.outRows); ++i) {
        const size_t idx = failed[i];
        std::cerr << "# " << idx << "," << r.sample.energies[idx] << "," << p.refEnergies[idx] << ","
                  << signedDiff(p.refEnergies[idx], r.sample.energies[idx]) * 100.0 << "\n";
      }
      std::cerr << std::flush;
    }
    r.ms = Stats::of({std::numeric_limits<double>::max()});
    return r;
  }
  r.ms = Stats::of(ms);
  const double runtime = (r.ms.sum / double(p.iterations)) * 1e-3;
  const double P = double(r.sample.ppwi), L = double(p.natlig()), R = double(p.natpro()), N = double(p.nposes());
  const double opsPerWg = P * 27 + L * (2 + P * 18 + R * (10 + P * 30)) + P; // src/main.cpp:359
  r.gflops = opsPerWg * (N / P) / runtime / 1e9;
  r.ginsts = 25.0 * R * L * N / runtime / 1e9;
  r.interactionsPerSec = N * L * R / runtime;
  const double peak = fp32PeakFlops(device);
  if (peak > 0) r.fp32PeakPct = 100.0 * (30.0 * N * L * R + 18.0 * N * L + 28.0 * N) / runtime / peak;
  return r;
}

void writeEnergies(const Params &p, const Outcome &r) {
  if (p.output.empty()) return;
  std::ofstream out(p.output, std::ios::trunc);
  for (float e : r.sample.energies) out << std::setw(7) << std::setprecision(2) << e << "\n";
}

void showYaml(const Params &p, const Outcome &r) {
  std::vector<double> raw;
  for (auto &t : r.sample.kernelTimes) raw.push_back(elapsedMillis(t.first, t.second));
  const std::string ctx = r.sample.contextTime
                              ? std::to_string(elapsedMillis(r.sample.contextTime->first, r.sample.contextTime->second))
                              : "~";
  std::cout.precision(3);
  std::cout << std::fixed << "  - outcome:             { valid: " << (r.valid ? "true" : "false")
            << ", max_diff_%: " << r.maxDiffPct << ", max_diff_abs_%: " << r.maxDiffAbsPct << " }\n"
            << "    param:               { ppwi: " << r.sample.ppwi << ", wgsize: " << r.sample.wgsize << " }\n"
            << "    raw_iterations:      [" << joined(raw) << "]\n"
            << "    context_ms:          " << ctx << "\n"
            << "    sum_ms:              " << r.ms.sum << "\n"
            << "    avg_ms:              " << r.ms.mean << "\n"
            << "    min_ms:              " << r.ms.min << "\n"
            << "    max_ms:              " << r.ms.max << "\n"
            << "    stddev_ms:           " << r.ms.stddev << "\n"
            << "    giga_interactions/s: " << r.interactionsPerSec / 1e9 << "\n"
            << "    gflop/s:             " << r.gflops << "\n"
            << "    gfinst/s:            " << r.ginsts << "\n"
            << "    fp32_peak_%:         " << r.fp32PeakPct << "\n"
            << "    energies:            \n";
  for (size_t i = 0; i < std::min(p.outRows, r.sample.energies.size()); ++i)
    std::cout << "      - " << std::setprecision(2) << r.sample.energies[i] << "\n";
  std::cout << std::flush;
}

void showCsv(const Outcome &r, bool header) {
  if (header) std::cout << "ppwi,wgsize,sum_ms,avg_ms,min_ms,max_ms,stddev_ms,interactions/s,gflops/s,gfinst/s\n";
  std::cout.precision(3);
  std::cout << std::fixed << r.sample.ppwi << "," << r.sample.wgsize << "," << r.ms.sum << "," << r.ms.mean << ","
            << r.ms.min << "," << r.ms.max << "," << r.ms.stddev << "," << r.interactionsPerSec << "," << r.gflops
            << "," << r.ginsts << std::endl;
}

// Device by index, else by name substring, else the only device (src/main.cpp:398-419).
int selectDevice(const std::string &needle, const std::vector<Device> &devices) {
  if (devices.empty()) return -1;
  if (needle.empty()) return int(devices[0].first);
  try {
    size_t idx = std::stoul(needle);
    if (idx < devices.size()) return int(devices[idx].first);
  } catch (...) {
  }
  std::cerr << "# Attempting to match device with substring  `" << needle << "`" << std::endl;
  for (auto &d : devices)
    if (d.second.find(needle) != std::string::npos) return int(d.first);
  if (devices.size() == 1) {
    std::cerr << "# No matching device but there's only one device, using it anyway" << std::endl;
    return int(devices[0].first);
  }
  std::cerr << "# No matching devices" << std::endl;
  return -1;
}

template <size_t... Ns> struct Models {
  static Sample fasten(size_t ppwi, const Params &p, size_t wgsize, size_t device) {
    Sample out(0, 0, 0);
    bool found = ((ppwi == Ns ? (out = run<Ns>(p, wgsize, device), true) : false) || ...);
    if (!found) throw std::invalid_argument("unsupported ppwi " + std::to_string(ppwi));
    return out;
  }
  template <size_t N> static Sample run(const Params &p, size_t wgsize, size_t device) {
    Gb300Bude<N> bude;
    if (!bude.compatible(p, wgsize, device))
      std::cerr << "Selected device is not compatible with this implementation, results may not be correct!"
                << std::endl;
    return bude.fasten(p, wgsize, device);
  }
};
using AllModels = Models<1, 2, 4, 8, 16, 32, 64, 128>;

bool runAll(const Cli &cli) {
  const Params &p = cli.params;
  auto devices = Gb300Bude<1>().enumerateDevices();
  if (devices.empty()) std::cerr << " # (no devices available)" << std::endl;
  if (p.list) {
    std::cout << (p.csv ? "index,name" : "devices:") << std::endl;
    for (size_t j = 0; j < devices.size(); ++j) {
      if (p.csv) std::cout << j << "," << devices[j].second << std::endl;
      else std::cout << "  " << j << ": \"" << devices[j].second << "\"" << std::endl;
    }
    return true;
  }
  const int dev = selectDevice(p.deviceSelector, devices);
  if (dev < 0) return false;
  if (!p.csv) std::cout << "device: { index: " << dev << ", name: \"" << devices[size_t(dev)].second << "\" }" << std::endl;
  std::vector<Outcome> results;
  bool dumped = false;
  for (size_t ppwi : cli.ppwis)
    for (size_t wgsize : cli.wgsizes) {
      Outcome r = evaluate(p, AllModels::fasten(ppwi, p, wgsize, size_t(dev)), size_t(dev), true);
      std::cout << "# (ppwi=" << ppwi << ",wgsize=" << wgsize << ",valid=" << r.valid << ")" << std::endl;
      if (!dumped || !r.valid) {
        dumped = true;
        writeEnergies(p, r);
      }
      results.push_back(std::move(r));
    }
  if (!p.csv) std::cout << "results:" << std::endl;
  for (size_t i = 0; i < results.size(); ++i) {
    if (p.csv) showCsv(results[i], i == 0);
    else showYaml(p, results[i]);
  }
  if (results.empty()) return false;
  const Outcome &best = *std::min_element(results.begin(), results.end(),
                                          [](const Outcome &a, const Outcome &b) { return a.ms.sum < b.ms.sum; });
  std::cout << (p.csv ? "# " : "") << "best: { min_ms: " << best.ms.min << ", max_ms: " << best.ms.max
            << ", sum_ms: " << best.ms.sum << ", avg_ms: " << best.ms.mean << ", ppwi: " << best.sample.ppwi
            << ", wgsize: " << best.sample.wgsize << " }\n";
  return std::all_of(results.begin(), results.end(), [](const Outcome &r) { return r.valid; });
}

// The host CPU block of the YAML header (src/main.cpp:588-631 prints it through the cpu_features
// library): the same keys, read here from /proc/cpuinfo; "~" where it has none of them.
void print_host_cpu() {
  std::ifstream in("/proc/cpuinfo");
  std::map<std::string, std::string> f;
  for (std::string line; std::getline(in, line);) {
    const auto colon = line.find(':');
    if (colon == std::string::npos) {
      if (!f.empty()) break; // the first processor's block is enough
      continue;
    }
    auto trim = [](std::string x) {
      const auto a = x.find_first_not_of(" \t"), b = x.find_last_not_of(" \t");
      return a == std::string::npos ? std::string() : x.substr(a, b - a + 1);
    };
    f.emplace(trim(line.substr(0, colon)), trim(line.substr(colon + 1)));
  }
  auto num = [&](const char *k) { return std::to_string(std::strtol(f[k].c_str(), nullptr, 0)); };
  std::cout << "host_cpu:\n";
  if (f.count("vendor_id")) {
    std::cout << "  arch:     \"x86 (" << f["vendor_id"] << ")\"\n"
              << "  brand:    \"" << f["model name"] << "\"\n"
              << "  family:   \"" << f["cpu family"] << "\"\n"
              << "  model:    \"" << f["model"] << "\"\n"
              << "  stepping: \"" << f["stepping"] << "\"" << std::endl;
  } else if (f.count("CPU implementer")) {
    std::cout << "  arch:        \"aarch64\"\n"
              << "  implementer: \"" << num("CPU implementer") << "\"\n"
              << "  variant:     \"" << num("CPU variant") << "\"\n"
              << "  part:        \"" << num("CPU part") << "\"\n"
              << "  revision:    \"" << num("CPU revision") << "\"" << std::endl;
  } else {
    std::cout << "  ~" << std::endl;
  }
}

// Version, compile commands and git state of this build (src/main.cpp:570-586).
void print_provenance() {
  const std::vector<std::string> cmds = GB300_BUDE_COMPILE_COMMANDS;
  std::cout << "miniBUDE:  gb300 " GB300_BUDE_VERSION " (" << bude_gpu_version() << ")\n"
            << "compile_commands:\n";
  for (const std::string &c : cmds) std::cout << "   - \"" << c << "\"\n";
  std::cout << "vcs:\n";
#if GB300_BUDE_VCS_RETRIEVED_STATE
  std::cout << "  commit:  " << GB300_BUDE_VCS_HEAD_SHA1 << (GB300_BUDE_VCS_IS_DIRTY ? "*" : "") << "\n"
            << "  author:  \"" << GB300_BUDE_VCS_AUTHOR_NAME << " (" << GB300_BUDE_VCS_AUTHOR_EMAIL << ")\"\n"
            << "  date:    \"" << GB300_BUDE_VCS_COMMIT_DATE_ISO8601 << "\"\n"
            << "  subject: \"" << GB300_BUDE_VCS_COMMIT_SUBJECT << "\"\n";
#else
  std::cout << "   # not built from a git checkout: no commit recorded\n";
#endif
}

} // namespace

int main(int argc, char *argv[]) {
  try {
    const Cli cli = parse(std::vector<std::string>(argv + 1, argv + argc));
    const Params &p = cli.params;
    if (!p.csv) {
      const std::time_t t = std::time(nullptr);
      print_provenance();
      print_host_cpu();
      std::cout << "time: { epoch_s:" << t << ", formatted: \"" << std::put_time(std::gmtime(&t), "%c %Z") << "\" }"
                << std::endl;
      if (!p.list)
        std::cout << "deck:\n"
                  << "  path:         \"" << p.deckDir << "\"\n"
                  << "  poses:        " << p.maxPoses << "\n"
                  << "  proteins:     " << p.natpro() << "\n"
                  << "  ligands:      " << p.natlig() << "\n"
                  << "  forcefields:  " << p.ntypes() << "\n"
                  << "config:\n"
                  << "  iterations:   " << p.iterations << "\n"
                  << "  poses:        " << p.nposes() << "\n"
                  << "  ppwi:\n"
                  << "    available:  [" << joined(kPPWIs) << "]\n"
                  << "    selected:   [" << joined(cli.ppwis) << "]\n"
                  << "  wgsize:       [" << joined(cli.wgsizes) << "]" << std::endl;
    }
    return runAll(cli) ? EXIT_SUCCESS : EXIT_FAILURE;
  } catch (const std::exception &e) {
    std::cerr << "terminate called after throwing an instance of 'std::exception'\n  what():  " << e.what()
              << std::endl;
    return EXIT_FAILURE;
  }
}
