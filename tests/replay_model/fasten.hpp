// fasten.hpp -- TEST HARNESS ONLY: a model for the reference driver's model slot that replays
// energies recorded from the GB300 model on a GB300, so that the reference's own evaluate() and
// validate() (src/main.cpp:329-396) judge them.  tests/test_reference_validator.py compiles the
// reference's unmodified src/main.cpp and src/bude.h with this header in the model slot.
//
// fasten(p, wgsize, device) reads <BUDE_REPLAY_DIR>/p<PPWI>_w<wgsize>.f32 (float32 energies in pose
// order, as bude_gpu_download wrote them) and returns them with one nominal kernel time per
// iteration; a missing recording throws, as a failing model does.
#pragma once

#include "../bude.h"

#include <chrono>
#include <cstdlib>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#ifdef IMPL_CLS
  #error IMPL_CLS was already defined
#endif
#define IMPL_CLS ReplayBude

template <size_t PPWI> class IMPL_CLS final : public Bude<PPWI> {
public:
  IMPL_CLS() = default;
  [[nodiscard]] std::string name() override { return "gb300-replay"; }
  [[nodiscard]] std::vector<Device> enumerateDevices() override { return {{0, "recorded GB300 energies"}}; }
  [[nodiscard]] bool compatible(const Params &, size_t, size_t) const override { return true; }

  [[nodiscard]] Sample fasten(const Params &p, size_t wgsize, size_t) const override {
    const char *dir = std::getenv("BUDE_REPLAY_DIR");
    if (!dir) throw std::runtime_error("BUDE_REPLAY_DIR is not set");
    const std::string path = std::string(dir) + "/p" + std::to_string(PPWI) + "_w" + std::to_string(wgsize) + ".f32";
    std::ifstream in(path, std::ios::binary);
    if (!in) throw std::runtime_error("no recording " + path);
    Sample sample(PPWI, wgsize, p.nposes());
    in.read(reinterpret_cast<char *>(sample.energies.data()), std::streamsize(p.nposes() * sizeof(float)));
    if (in.gcount() != std::streamsize(p.nposes() * sizeof(float)))
      throw std::runtime_error("short recording " + path);
    for (size_t i = 0; i < p.totalIterations(); ++i) {
      auto t0 = std::chrono::high_resolution_clock::now();
      sample.kernelTimes.emplace_back(t0, t0 + std::chrono::microseconds(100));
    }
    return sample;
  }
};
