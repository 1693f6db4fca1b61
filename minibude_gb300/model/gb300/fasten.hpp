// gb300/fasten.hpp -- the GB300 model of miniBUDE, for the reference driver's model slot.
//
// A pure C++ `Bude<PPWI>` subclass (interface: reference src/bude.h:95-101) with no CUDA headers:
// every device operation goes through the C-ABI of libbude_gb300.so (include/minibude_gb300.h).
// It replaces the reference's CudaBude (src/cuda/fasten.hpp:163-306) behind the same contract:
//   * `fasten` owns all device allocations of the call (a library context created and destroyed
//     here), reports the upload as `contextTime`, runs iterations + warm-ups evaluations with a
//     synchronise after each (host-timed like src/cuda/fasten.hpp:277-286) and returns the
//     energies in pose order;
//   * errors become std::runtime_error carrying the library's message (as `checkError` does,
//     src/cuda/fasten.hpp:168-172); `compatible` only reports.
// PPWI keeps its meaning (poses per thread, register-blocked; 32/64/128 use 16) and wgsize is
// the block size (values below 32 become the library's default of 128).  Any pose count is
// accepted: ragged tails are handled by the kernel.
#pragma once

#include "../bude.h"
#include "minibude_gb300.h"

#include <cstring>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#ifdef IMPL_CLS
  #error IMPL_CLS was already defined
#endif
#define IMPL_CLS Gb300Bude

static_assert(sizeof(Atom) == sizeof(bude_atom), "Atom and bude_atom must share the 16-byte deck layout");
static_assert(sizeof(FFParams) == sizeof(bude_ffparams), "FFParams and bude_ffparams must share a layout");

template <size_t PPWI> class IMPL_CLS final : public Bude<PPWI> {

  static void check(int rc, const char *what) {
    if (rc != BUDE_OK) throw std::runtime_error(std::string("gb300 ") + what + ": " + bude_gpu_last_error());
  }

  // Owns one library context for the duration of a call.
  struct Context {
    bude_gpu_ctx *handle = nullptr;
    explicit Context(size_t device) { check(bude_gpu_create(int(device), &handle), "create"); }
    ~Context() {
      if (handle) bude_gpu_destroy(handle);
    }
    Context(const Context &) = delete;
    Context &operator=(const Context &) = delete;
  };

public:
  IMPL_CLS() = default;

  [[nodiscard]] std::string name() override { return "gb300"; }

  [[nodiscard]] std::vector<Device> enumerateDevices() override {
    int count = 0;
    check(bude_gpu_device_count(&count), "device count");
    std::vector<Device> devices;
    for (int i = 0; i < count; ++i) {
      char buf[256];
      check(bude_gpu_device_name(i, buf, sizeof buf), "device name");
      devices.emplace_back(size_t(i), std::string(buf));
    }
    return devices;
  }

  [[nodiscard]] bool compatible(const Params &, size_t, size_t device) const override {
    int kcc = 0, dcc = 0, ok = 0;
    check(bude_gpu_compatible(int(device), &kcc, &dcc, &ok), "compatible");
    if (!ok) {
      std::cerr << "# [WARNING] Device cc (sm_" << dcc << ") != Kernel cc (sm_" << kcc << ")" << std::endl;
      return false;
    }
    std::cout << "# Device and kernel cc: sm_" << dcc << std::endl;
    return true;
  }

  [[nodiscard]] Sample fasten(const Params &p, size_t wgsize, size_t device) const override {
    Sample sample(PPWI, wgsize, p.nposes());
    const size_t n = p.nposes();
    // The six pose fields as one [6][n] block (the layout of poses.in).
    std::vector<float> poses(6 * n);
    for (size_t k = 0; k < 6; ++k) std::memcpy(poses.data() + k * n, p.poses[k].data(), n * sizeof(float));

    Context ctx(device);
    auto contextStart = now();
    check(bude_gpu_upload(ctx.handle, reinterpret_cast<const bude_atom *>(p.protein.data()), int32_t(p.natpro()),
                          reinterpret_cast<const bude_atom *>(p.ligand.data()), int32_t(p.natlig()),
                          reinterpret_cast<const bude_ffparams *>(p.forcefield.data()), int32_t(p.ntypes()),
                          poses.data(), int64_t(n), int64_t(n)),
          "upload");
    auto contextEnd = now();
    sample.contextTime = {contextStart, contextEnd};

    bude_launch_cfg cfg{};
    check(bude_gpu_default_cfg(ctx.handle, int32_t(PPWI), int32_t(wgsize), &cfg), "launch shape");
    for (size_t i = 0; i < p.totalIterations(); ++i) {
      auto kernelStart = now();
      check(bude_gpu_run(ctx.handle, &cfg, nullptr), "run");
      auto kernelEnd = now();
      sample.kernelTimes.emplace_back(kernelStart, kernelEnd);
    }
    check(bude_gpu_download(ctx.handle, sample.energies.data(), int64_t(n)), "download");
    return sample;
  }
};
