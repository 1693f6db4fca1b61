// noalloc.cu -- bude_gpu_fasten_noalloc: one exact evaluation that allocates no device memory.
//
// Some callers of this library may not allocate GPU memory themselves: code running inside
// another framework whose allocator owns the whole device heap and must see every byte, plugin
// hosts that hand a plugin its buffers and forbid it to allocate, and latency-bound loops where
// cudaMalloc/cudaFree (which can synchronise the device) are not allowed.  They pass device
// buffers for the inputs and the output; the working memory the evaluation needs beyond those --
// the per-deck protein slab, the pose transforms and an error word -- comes from one fixed
// file-scope array in device memory, `g_noalloc_scratch`, instead of the cudaMalloc'd buffers of
// a bude_gpu_ctx.
//
// Rules of the array:
//   * its size is fixed at build time (BUDE_NOALLOC_MAX_POSES transforms and
//     BUDE_NOALLOC_MAX_SLAB_RECORDS slab records, about 11 MiB), and every GPU that loads this
//     module holds it until the process exits;
//   * every call on a device shares it and it keeps the last call's contents: the error and check
//     words are reset at the start of each call, the slab, transforms and irregular-pose bits are
//     rewritten in full;
//   * calls whose work overlaps on one GPU (two host threads, or two streams) race on it and
//     must be serialised by the caller;
//   * in host code the array's name is only a stand-in: its device address is looked up once per
//     device with cudaGetSymbolAddress, with that device current, by the first call made on the
//     device, and kept for the life of the process.  A cudaDeviceReset would leave that address
//     stale, so the entry point must not be used on a device after it has been reset.
// Each call reads its error word back and synchronises the stream before it returns.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>

#include "exact_kernel.cuh"
#include "internal.h"
#include "pair_record.h"

namespace bude {
namespace {

constexpr size_t kNaErrBytes = 256;
constexpr size_t kNaXformBytes = (size_t)BUDE_NOALLOC_MAX_POSES * 3 * sizeof(float4);
constexpr size_t kNaSlabBytes = (size_t)BUDE_NOALLOC_MAX_SLAB_RECORDS * kRecF4 * sizeof(float4);
constexpr size_t kNaMaskBytes = (size_t)BUDE_NOALLOC_MAX_POSES / 32 * sizeof(unsigned);
constexpr size_t kNaScratchBytes = kNaErrBytes + kNaXformBytes + kNaSlabBytes + kNaMaskBytes;

// Words of the scratch's first 256 bytes: [0] error bits, [1] and [2] the smallest forcefield
// radius of the protein's and of the ligand's atoms as order-preserving keys (atomicMin).
// Error bits (bit 0 is the exact kernel's bounded-wait timeout):
constexpr unsigned kNaErrProteinType = 2u;
constexpr unsigned kNaErrLigandType = 4u;
constexpr unsigned kNaIrregular = 8u; // an atom or forcefield record outside the regular-deck bounds

// The working memory of bude_gpu_fasten_noalloc:
// [error and check words | pose transforms | protein slab | irregular-pose bits].
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaScratchBytes];

constexpr int kNaMaxDevices = 64;
std::mutex g_na_mutex;
unsigned char *g_na_scratch[kNaMaxDevices]; // device address of g_noalloc_scratch, per device

// Device address of the scratch array on `device` (the current device); looked up on first use.
int na_scratch(int device, unsigned char **out) {
  if (device < 0 || device >= kNaMaxDevices)
    return set_error(BUDE_ERR_ARG, "no-alloc entry point supports device ordinals below %d (got %d)", kNaMaxDevices,
                     device);
  std::lock_guard<std::mutex> lock(g_na_mutex);
  if (!g_na_scratch[device]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(no-alloc scratch)");
    g_na_scratch[device] = static_cast<unsigned char *>(p);
  }
  *out = g_na_scratch[device];
  return BUDE_OK;
}

// The per-ligand-type protein slab, built on the device from device-resident protein and
// forcefield (the same records as the host build: pair_record is shared).  Atom types outside
// the forcefield set an error bit and get a padding record instead of being read.
__global__ void __launch_bounds__(256) na_slab_kernel(const bude_atom *__restrict__ protein, int natpro,
                                                      const bude_ffparams *__restrict__ ff, int ntypes, int natpro_pad,
                                                      float4 *__restrict__ slab, unsigned *err) {
  const long long n = (long long)ntypes * natpro_pad;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < n;
       idx += (long long)gridDim.x * blockDim.x) {
    const int t = (int)(idx / natpro_pad);
    const int j = (int)(idx - (long long)t * natpro_pad);
    float rec[kRecFloats];
    if (j < natpro) {
      const bude_atom a = protein[j];
      if (a.type >= 0 && a.type < ntypes) {
        pair_record(ff[t], ff[a.type], a.x, a.y, a.z, rec);
      } else {
        null_record(rec);
        atomicOr(err, kNaErrProteinType);
      }
    } else {
      null_record(rec);
    }
    float4 *dst = slab + idx * kRecF4;
#pragma unroll
    for (int k = 0; k < kRecF4; ++k) dst[k] = make_float4(rec[4 * k], rec[4 * k + 1], rec[4 * k + 2], rec[4 * k + 3]);
  }
}

__device__ __forceinline__ unsigned radius_key(float f) {
  const unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u); // ascending float order as unsigned order
}

// Per atom: ligand atom types must index the slab (the exact kernel reads them unchecked), and
// the atoms and their forcefield records are checked against the regular-deck bounds
// (edge_pose.cuh); the smallest radii of both sides go to words [1] and [2].  Atoms with a type
// outside the forcefield are only flagged.
__global__ void na_deck_check_kernel(const bude_atom *__restrict__ protein, int natpro,
                                     const bude_atom *__restrict__ ligand, int natlig,
                                     const bude_ffparams *__restrict__ ff, int ntypes, unsigned *words) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < natpro + natlig; i += gridDim.x * blockDim.x) {
    const bool is_lig = i >= natpro;
    const bude_atom a = is_lig ? ligand[i - natpro] : protein[i];
    if (a.type < 0 || a.type >= ntypes) {
      if (is_lig) atomicOr(&words[0], kNaErrLigandType); // protein types: na_slab_kernel
      continue;
    }
    const bude_ffparams f = ff[a.type];
    const bool ok = param_regular(f) && (is_lig ? ligand_atom_regular(a.x, a.y, a.z) : protein_atom_regular(a));
    if (!ok) atomicOr(&words[0], kNaIrregular);
    atomicMin(&words[is_lig ? 2 : 1], radius_key(f.radius));
  }
}

float key_radius(unsigned k) {
  const unsigned u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
  float f;
  std::memcpy(&f, &u, sizeof f);
  return f;
}

// Read n words from the device into a caller-provided host array (no allocation) and wait.
int na_read_words(const unsigned *words, int n, cudaStream_t st, unsigned *out) {
  cudaError_t e = cudaMemcpyAsync(out, words, (size_t)n * sizeof(unsigned), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? BUDE_OK : cuda_error(e, "no-alloc error word");
}

// Device memory of `device` (the current device), or managed memory.  Another GPU's memory is
// refused: the kernels would read it over the interconnect or fault when peer access is off.
bool is_device_memory(const void *p, int device) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return (at.type == cudaMemoryTypeDevice && at.device == device) || at.type == cudaMemoryTypeManaged;
}

} // namespace
} // namespace bude

extern "C" int bude_gpu_fasten_noalloc(const bude_atom *protein, int32_t natpro, const bude_atom *ligand,
                                       int32_t natlig, const bude_ffparams *forcefield, int32_t ntypes,
                                       const float *poses, int64_t pose_stride, int64_t nposes, float *energies,
                                       void *stream) {
  using namespace bude;
  // Sizes against the fixed scratch.
  if (natpro < 0 || natlig < 0 || ntypes <= 0 || nposes < 0 || pose_stride < nposes)
    return set_error(BUDE_ERR_ARG, "bad sizes (natpro %d, natlig %d, ntypes %d, nposes %lld, pose_stride %lld)",
                     natpro, natlig, ntypes, (long long)nposes, (long long)pose_stride);
  if (nposes > BUDE_NOALLOC_MAX_POSES)
    return set_error(BUDE_ERR_ARG, "no-alloc entry point takes at most %d poses per call (got %lld)",
                     BUDE_NOALLOC_MAX_POSES, (long long)nposes);
  const int natpro_pad = std::max((natpro + kAtomAlign - 1) / kAtomAlign * kAtomAlign, kAtomAlign);
  if ((long long)ntypes * natpro_pad > BUDE_NOALLOC_MAX_SLAB_RECORDS)
    return set_error(BUDE_ERR_ARG,
                     "no-alloc entry point holds at most %d slab records; forcefield types x padded protein atoms = "
                     "%d x %d",
                     BUDE_NOALLOC_MAX_SLAB_RECORDS, ntypes, natpro_pad);
  if (nposes == 0) return BUDE_OK;
  // Inputs and output must be device memory; the ligand is read as 16-byte vectors.
  if (!forcefield || !poses || !energies || (natpro > 0 && !protein) || (natlig > 0 && !ligand))
    return set_error(BUDE_ERR_ARG, "NULL input or output buffer");
  if (reinterpret_cast<uintptr_t>(ligand) % 16 != 0)
    return set_error(BUDE_ERR_ARG, "ligand must be 16-byte aligned");
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
  if (!is_device_memory(forcefield, device) || !is_device_memory(poses, device) ||
      !is_device_memory(energies, device) || (natpro > 0 && !is_device_memory(protein, device)) ||
      (natlig > 0 && !is_device_memory(ligand, device)))
    return set_error(BUDE_ERR_ARG, "no-alloc entry point takes buffers in the current device's memory only "
                                   "(device %d)", device);

  unsigned char *scratch = nullptr;
  int rc = na_scratch(device, &scratch);
  if (rc) return rc;
  unsigned *err = reinterpret_cast<unsigned *>(scratch);
  float4 *xform = reinterpret_cast<float4 *>(scratch + kNaErrBytes);
  float4 *slab = reinterpret_cast<float4 *>(scratch + kNaErrBytes + kNaXformBytes);
  unsigned *mask = reinterpret_cast<unsigned *>(scratch + kNaErrBytes + kNaXformBytes + kNaSlabBytes);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);

  // 1. reset the error word and the two radius minima; slab and deck checks.
  e = cudaMemsetAsync(err, 0, sizeof(unsigned), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(err + 1, 0xff, 2 * sizeof(unsigned), st);
  if (e != cudaSuccess) return cuda_error(e, "no-alloc error word clear");
  {
    const long long n = (long long)ntypes * natpro_pad;
    const int blocks = (int)std::min<long long>((n + 255) / 256, 8LL * std::max(sms, 1));
    na_slab_kernel<<<blocks, 256, 0, st>>>(protein, natpro, forcefield, ntypes, natpro_pad, slab, err);
    if (natpro + natlig > 0)
      na_deck_check_kernel<<<(unsigned)std::min((natpro + natlig + 255) / 256, 4 * std::max(sms, 1)), 256, 0, st>>>(
          protein, natpro, ligand, natlig, forcefield, ntypes, err);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(e, "no-alloc slab launch");
  }
  unsigned h[3] = {0, 0, 0};
  rc = na_read_words(err, 3, st, h);
  if (rc) return rc;
  if (h[0] & (kNaErrProteinType | kNaErrLigandType))
    return set_error(BUDE_ERR_TYPE, "%s atom type outside the forcefield (%d types)",
                     (h[0] & kNaErrLigandType) ? "a ligand" : "a protein", ntypes);
  // The deck is irregular when an atom or record is out of bounds or the smallest FP32 radius sum
  // is below the bound (FP32 addition is monotone); with no ligand-protein pair every energy is 0.
  const float min_sum = key_radius(h[1]) + key_radius(h[2]);
  const bool irregular = natpro > 0 && natlig > 0 && ((h[0] & kNaIrregular) || !(min_sum >= kMinRadiusSum));

  // 2. pose transforms and the exact kernel; protein slices (if any) are summed in a cluster, so
  //    no slice buffer is needed.
  pose_xform_kernel<<<(unsigned)((nposes + 255) / 256), 256, 0, st>>>(poses, pose_stride, nposes, xform, mask);
  constexpr int P = 8, U = 2, W = 128, T = 64;
  const long long blocks = (nposes + (long long)P * W - 1) / ((long long)P * W);
  int split = 1;
  while (split < 8 && blocks * split < 4LL * std::max(sms, 1) && natpro_pad / (split * 2) >= 64) split *= 2;
  ExactArgs a;
  a.ligand = reinterpret_cast<const float4 *>(ligand);
  a.slab = slab;
  a.xform = reinterpret_cast<const float *>(xform);
  a.energies = energies;
  a.partial = nullptr;
  a.err = err;
  a.nposes = nposes;
  a.natlig = natlig;
  a.natpro_pad = natpro_pad;
  a.tile = T;
  a.split = split;
  a.cluster = 1;
  a.slice = ((natpro_pad + split - 1) / split + kAtomAlign - 1) / kAtomAlign * kAtomAlign;
  const size_t smem = exact_smem_bytes(P, W, T, split, 1);
  e = cudaFuncSetAttribute(exact_kernel<P, U>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) {
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3((unsigned)blocks, (unsigned)split, 1);
    lc.blockDim = dim3(W, 1, 1);
    lc.dynamicSmemBytes = smem;
    lc.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 1;
    attr[0].val.clusterDim.y = split;
    attr[0].val.clusterDim.z = 1;
    lc.attrs = attr;
    lc.numAttrs = 1;
    e = cudaLaunchKernelEx(&lc, exact_kernel<P, U>, a);
  }
  if (e != cudaSuccess) return cuda_error(e, "no-alloc exact_kernel launch");
  // 3. irregular poses (or every pose of an irregular deck) by the reference's arithmetic.
  EdgeArgs ea{};
  ea.mask = mask;
  ea.all = irregular ? 1 : 0;
  ea.nposes = nposes;
  ea.nlig = 1;
  ea.ligand = reinterpret_cast<const float4 *>(ligand);
  ea.natlig = natlig;
  ea.protein = protein;
  ea.natpro = natpro;
  ea.ff = forcefield;
  ea.xform = reinterpret_cast<const float *>(xform);
  ea.energies = energies;
  edge_pose_kernel<<<edge_grid(nposes, sms), 256, 0, st>>>(ea);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "no-alloc edge_pose_kernel launch");
  rc = na_read_words(err, 1, st, h);
  if (rc) return rc;
  if (h[0] & 1u) return set_error(BUDE_ERR_TIMEOUT, "a bounded device wait ran out; energies are invalid");
  return BUDE_OK;
}
