// bude_gb300.cu -- host side of libbude_gb300.so: the C-ABI declared in include/minibude_gb300.h.
//
// It owns what the reference's CudaBude owns (src/cuda/fasten.hpp:174-305): device selection,
// device buffers for the deck, kernel launches, per-iteration timing and the copy back -- plus
// the per-deck slab of protein records the exact kernel streams (see exact_kernel.cuh).
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/minibude_gb300.h"
#include "exact_kernel.cuh"
#include "internal.h"
#include "pair_record.h"

namespace bude {

// ---------------------------------------------------------------------------------------------
// Errors: the text lives in a fixed per-thread buffer, so reporting an error never allocates.
static thread_local char g_last_error[512];

int set_error(int code, const char *fmt, ...) {
  char buf[sizeof g_last_error];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  std::memcpy(g_last_error, buf, sizeof buf);
  return code;
}

cudaError_t copy_sync(const Context &c, void *dst, const void *src, size_t bytes, cudaMemcpyKind kind) {
  if (bytes == 0) return cudaSuccess;
  cudaError_t e = cudaMemcpyAsync(dst, src, bytes, kind, c.stream);
  return e == cudaSuccess ? cudaStreamSynchronize(c.stream) : e;
}

cudaError_t copy2d_sync(const Context &c, void *dst, size_t dpitch, const void *src, size_t spitch, size_t width,
                        size_t height, cudaMemcpyKind kind) {
  if (width == 0 || height == 0) return cudaSuccess;
  cudaError_t e = cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, height, kind, c.stream);
  return e == cudaSuccess ? cudaStreamSynchronize(c.stream) : e;
}

cudaError_t fill_sync(const Context &c, void *dst, int value, size_t bytes) {
  if (bytes == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(dst, value, bytes, c.stream);
  return e == cudaSuccess ? cudaStreamSynchronize(c.stream) : e;
}

int cuda_error(cudaError_t e, const char *what) {
  return set_error(BUDE_ERR_CUDA, "%s: %s: %s", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

const char *last_error() { return g_last_error; }

// ---------------------------------------------------------------------------------------------
// slab[t][j] = record for ligand type t against protein atom j; rows padded to natpro_pad.
void build_slab(const bude_atom *protein, int natpro, const bude_ffparams *ff, int ntypes, int natpro_pad,
                std::vector<float> &slab) {
  slab.assign((size_t)ntypes * natpro_pad * kRecFloats, 0.f);
  for (int t = 0; t < ntypes; ++t) {
    float *row = slab.data() + (size_t)t * natpro_pad * kRecFloats;
    for (int j = 0; j < natpro; ++j)
      pair_record(ff[t], ff[protein[j].type], protein[j].x, protein[j].y, protein[j].z, row + (size_t)j * kRecFloats);
    for (int j = natpro; j < natpro_pad; ++j) null_record(row + (size_t)j * kRecFloats);
  }
}

int ensure_slab(Context &c, const bude_atom *protein, int natpro, const bude_ffparams *ff, int ntypes, bool *rebuilt) {
  std::vector<unsigned char> key(2 * sizeof(int) + (size_t)natpro * sizeof(bude_atom) +
                                 (size_t)ntypes * sizeof(bude_ffparams));
  std::memcpy(key.data(), &natpro, sizeof(int));
  std::memcpy(key.data() + sizeof(int), &ntypes, sizeof(int));
  if (natpro > 0) std::memcpy(key.data() + 2 * sizeof(int), protein, (size_t)natpro * sizeof(bude_atom));
  std::memcpy(key.data() + 2 * sizeof(int) + (size_t)natpro * sizeof(bude_atom), ff,
              (size_t)ntypes * sizeof(bude_ffparams));
  if (rebuilt) *rebuilt = false;
  if (c.slab.ptr && key == c.slab_key) return BUDE_OK;
  c.slab_key.clear();
  c.ntypes = ntypes;
  c.natpro = natpro;
  c.natpro_pad = std::max((natpro + kAtomAlign - 1) / kAtomAlign * kAtomAlign, kAtomAlign);
  std::vector<float> slab;
  build_slab(protein, natpro, ff, ntypes, c.natpro_pad, slab);
  int rc = c.slab.reserve(slab.size() * sizeof(float), "slab");
  if (!rc) rc = c.raw_protein.reserve((size_t)std::max(natpro, 1) * sizeof(bude_atom), "protein records");
  if (!rc) rc = c.raw_ff.reserve((size_t)ntypes * sizeof(bude_ffparams), "forcefield records");
  if (rc) return rc;
  cudaError_t e = copy_sync(c, c.slab.ptr, slab.data(), slab.size() * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && natpro > 0)
    e = copy_sync(c, c.raw_protein.ptr, protein, (size_t)natpro * sizeof(bude_atom), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = copy_sync(c, c.raw_ff.ptr, ff, (size_t)ntypes * sizeof(bude_ffparams), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_error(e, "slab upload");
  c.host_ff.assign(ff, ff + ntypes);
  // The protein's half of the regular-deck bounds (edge_pose.cuh); types were checked by the caller.
  c.protein_regular = true;
  c.protein_min_radius = FLT_MAX;
  for (int j = 0; j < natpro; ++j) {
    const bude_ffparams &f = ff[protein[j].type];
    c.protein_regular = c.protein_regular && protein_atom_regular(protein[j]) && param_regular(f);
    c.protein_min_radius = std::min(c.protein_min_radius, f.radius);
  }
  c.slab_key = std::move(key);
  if (rebuilt) *rebuilt = true;
  return BUDE_OK;
}

bool ligand_regular(const Context &c, const bude_atom *ligand, int natlig, const bude_ffparams *ff) {
  if (natlig == 0 || c.natpro == 0) return true; // no pairs: every energy is 0, as in the reference
  if (!c.protein_regular) return false;
  float min_radius = FLT_MAX;
  for (int i = 0; i < natlig; ++i) {
    const bude_ffparams &f = ff[ligand[i].type];
    if (!ligand_atom_regular(ligand[i].x, ligand[i].y, ligand[i].z) || !param_regular(f)) return false;
    min_radius = std::min(min_radius, f.radius);
  }
  // FP32 addition is monotone, so this bounds every pair's radius sum (pair_record's radij).
  const float min_sum = c.protein_min_radius + min_radius;
  return min_sum >= kMinRadiusSum;
}

int enqueue_edge_single(Context &c, const float4 *ligand, int natlig, bool all, const unsigned *mask,
                        const float *xform, float *energies, long long n, cudaStream_t st) {
  if (n <= 0) return BUDE_OK;
  EdgeArgs a{};
  a.mask = mask;
  a.all = all ? 1 : 0;
  a.nposes = n;
  a.nlig = 1;
  a.ligand = ligand;
  a.natlig = natlig;
  a.protein = c.raw_protein.as<bude_atom>();
  a.natpro = c.natpro;
  a.ff = c.raw_ff.as<bude_ffparams>();
  a.xform = xform;
  a.energies = energies;
  edge_pose_kernel<<<edge_grid(n, c.num_sms), 256, 0, st>>>(a);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "edge_pose_kernel launch");
  c.launches++;
  return BUDE_OK;
}

int enqueue_edge_batch(Context &c, const float *xform, float *energies, unsigned char *flag, cudaStream_t st) {
  if (c.batch_poses <= 0) return BUDE_OK;
  EdgeArgs a{};
  a.mask = c.b_edge_mask.as<unsigned>();
  a.nposes = c.batch_poses;
  a.pose_off = c.b_pose_off.as<long long>();
  a.lig_off = c.b_lig_off.as<int>();
  a.lig_any = c.b_lig_any.as<int>();
  a.lig_all = c.b_lig_all.as<unsigned char>();
  a.nlig = c.nligands;
  a.ligand = c.b_ligands.as<float4>();
  a.protein = c.raw_protein.as<bude_atom>();
  a.natpro = c.natpro;
  a.ff = c.raw_ff.as<bude_ffparams>();
  a.xform = xform;
  a.energies = energies;
  a.flag = flag;
  edge_pose_kernel<<<edge_grid(c.batch_poses, c.num_sms), 256, 0, st>>>(a);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "edge_pose_kernel launch");
  c.launches++;
  return BUDE_OK;
}

// ---------------------------------------------------------------------------------------------
// Device buffers
int DevBuf::reserve(size_t nbytes, const char *what) {
  if (nbytes <= cap) return BUDE_OK;
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  cap = 0;
  cudaError_t e = cudaMalloc(&ptr, std::max<size_t>(nbytes, 256));
  if (e != cudaSuccess) return cuda_error(e, what);
  cap = nbytes;
  return BUDE_OK;
}

void DevBuf::release() {
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  cap = 0;
}

} // namespace bude

using namespace bude;


// ---------------------------------------------------------------------------------------------
// Launch helpers

namespace bude {

static int round_up(int v, int m) { return (v + m - 1) / m * m; }

int check_cfg(const Context &c, const bude_launch_cfg &cfg) {
  const int p = cfg.ppwi;
  if (p != 1 && p != 2 && p != 4 && p != 8 && p != 16)
    return set_error(BUDE_ERR_ARG, "ppwi must be 1, 2, 4, 8 or 16 (got %d)", p);
  if (cfg.wgsize < 32 || cfg.wgsize > kMaxThreads || cfg.wgsize % 32)
    return set_error(BUDE_ERR_ARG, "wgsize must be a multiple of 32 in [32, %d] (got %d)", kMaxThreads, cfg.wgsize);
  if (cfg.cluster != 0 && cfg.cluster != 1) return set_error(BUDE_ERR_ARG, "cluster must be 0 or 1 (got %d)", cfg.cluster);
  if (cfg.split < 1 || cfg.split > (cfg.cluster ? 8 : 64))
    return set_error(BUDE_ERR_ARG, "split must be in [1, %d] (got %d)", cfg.cluster ? 8 : 64, cfg.split);
  if (cfg.tile < kAtomAlign || cfg.tile > 512 || cfg.tile % kAtomAlign)
    return set_error(BUDE_ERR_ARG, "tile must be a multiple of %d in [%d, 512] (got %d)", kAtomAlign, kAtomAlign,
                     cfg.tile);
  if (cfg.unroll != 1 && cfg.unroll != 2 && cfg.unroll != 4)
    return set_error(BUDE_ERR_ARG, "unroll must be 1, 2 or 4 (got %d)", cfg.unroll);
  if (exact_smem_bytes(p, cfg.wgsize, cfg.tile, cfg.split, cfg.cluster) > 200 * 1024)
    return set_error(BUDE_ERR_ARG, "launch shape needs too much shared memory");
  (void)c;
  return BUDE_OK;
}

// The compilation of exact_kernel<P, U> a block size runs: the narrow one (170 registers) for
// blocks of at most kNarrowThreads threads.
template <int P, int U> static decltype(&exact_kernel<P, U>) exact_entry(int wgsize) {
  return wgsize <= kNarrowThreads ? exact_kernel_narrow<P, U> : exact_kernel<P, U>;
}

template <int P, int U>
static cudaError_t launch_exact_pu(const ExactArgs &a, dim3 grid, int wgsize, size_t smem, int split,
                                   cudaStream_t st) {
  const auto kernel = exact_entry<P, U>(wgsize);
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (split == 1 || !a.cluster) {
    kernel<<<grid, wgsize, smem, st>>>(a);
    return cudaGetLastError();
  }
  cudaLaunchConfig_t lc = {};
  lc.gridDim = grid;
  lc.blockDim = dim3(wgsize, 1, 1);
  lc.dynamicSmemBytes = smem;
  lc.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 1;
  attr[0].val.clusterDim.y = split;
  attr[0].val.clusterDim.z = 1;
  lc.attrs = attr;
  lc.numAttrs = 1;
  return cudaLaunchKernelEx(&lc, kernel, a);
}

template <int P>
static cudaError_t launch_exact_p(const ExactArgs &a, dim3 grid, const bude_launch_cfg &cfg, size_t smem,
                                  cudaStream_t st) {
  switch (cfg.unroll) {
  case 1: return launch_exact_pu<P, 1>(a, grid, cfg.wgsize, smem, cfg.split, st);
  case 2: return launch_exact_pu<P, 2>(a, grid, cfg.wgsize, smem, cfg.split, st);
  default: return launch_exact_pu<P, 4>(a, grid, cfg.wgsize, smem, cfg.split, st);
  }
}

template <int P, int U> static int blocks_per_sm_pu(int wgsize, size_t smem, int *out) {
  const auto kernel = exact_entry<P, U>(wgsize);
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, kernel, wgsize, smem);
  return e == cudaSuccess ? BUDE_OK : cuda_error(e, "occupancy query");
}

template <int P> static int blocks_per_sm_p(const bude_launch_cfg &cfg, size_t smem, int *out) {
  switch (cfg.unroll) {
  case 1: return blocks_per_sm_pu<P, 1>(cfg.wgsize, smem, out);
  case 2: return blocks_per_sm_pu<P, 2>(cfg.wgsize, smem, out);
  default: return blocks_per_sm_pu<P, 4>(cfg.wgsize, smem, out);
  }
}

int exact_blocks_per_sm(const bude_launch_cfg &cfg, int *out) {
  const size_t smem = exact_smem_bytes(cfg.ppwi, cfg.wgsize, cfg.tile, cfg.split, cfg.cluster);
  switch (cfg.ppwi) {
  case 1: return blocks_per_sm_p<1>(cfg, smem, out);
  case 2: return blocks_per_sm_p<2>(cfg, smem, out);
  case 4: return blocks_per_sm_p<4>(cfg, smem, out);
  case 8: return blocks_per_sm_p<8>(cfg, smem, out);
  default: return blocks_per_sm_p<16>(cfg, smem, out);
  }
}

// Enqueue one evaluation (pose transforms + exact kernel) on the context's stream; `mid`, when
// given, is recorded between the two kernels.
int enqueue_eval(Context &c, const bude_launch_cfg &cfg, cudaEvent_t mid) {
  if (!c.have_deck) return set_error(BUDE_ERR_STATE, "no deck uploaded");
  int rc = check_cfg(c, cfg);
  if (rc) return rc;
  if (c.nposes == 0) {
    if (mid) cudaEventRecord(mid, c.stream);
    return BUDE_OK;
  }
  {
    const int tb = 256;
    const long long nb = (c.nposes + tb - 1) / tb;
    pose_xform_kernel<<<(unsigned)nb, tb, 0, c.stream>>>(c.poses.as<float>(), c.pose_stride, c.nposes,
                                                         c.xform.as<float4>(), c.edge_mask.as<unsigned>());
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(e, "pose_xform_kernel launch");
    c.launches++;
  }
  if (mid) cudaEventRecord(mid, c.stream);
  rc = launch_exact_range(c, cfg, c.ligand.as<float4>(), c.natlig, c.xform.as<float>(), c.energies.as<float>(),
                          c.nposes);
  if (rc) return rc;
  return enqueue_edge_single(c, c.ligand.as<float4>(), c.natlig, c.deck_irregular, c.edge_mask.as<unsigned>(),
                             c.xform.as<float>(), c.energies.as<float>(), c.nposes, c.stream);
}

// The exact kernel (and, for a global-reduce split, slice_reduce_kernel) over `nposes` poses whose
// transforms are at `xform`, for the ligand at `ligand`; energies land at `energies`.
int launch_exact_range(Context &c, const bude_launch_cfg &cfg, const float4 *ligand, int natlig, const float *xform,
                       float *energies, long long nposes) {
  if (nposes == 0) return BUDE_OK;
  ExactArgs a;
  a.ligand = ligand;
  a.slab = c.slab.as<float4>();
  a.xform = xform;
  a.energies = energies;
  a.partial = nullptr;
  a.err = c.err.as<unsigned int>();
  a.nposes = nposes;
  a.natlig = natlig;
  a.natpro_pad = c.natpro_pad;
  a.tile = cfg.tile;
  a.split = cfg.split;
  a.cluster = cfg.cluster;
  const bool global_reduce = cfg.split > 1 && !cfg.cluster;
  if (global_reduce) {
    // Slice sums go through a [split][nposes] buffer owned by the context.
    int rc2 = c.partial.reserve((size_t)cfg.split * nposes * sizeof(float), "slice partial sums");
    if (rc2) return rc2;
    a.partial = c.partial.as<float>();
  }
  a.slice = round_up((c.natpro_pad + cfg.split - 1) / cfg.split, kAtomAlign);
  const long long ppb = (long long)cfg.ppwi * cfg.wgsize;
  const long long nbx = (nposes + ppb - 1) / ppb;
  if (nbx > 0x7fffffffLL) return set_error(BUDE_ERR_ARG, "too many poses for one launch");
  dim3 grid((unsigned)nbx, (unsigned)cfg.split, 1);
  const size_t smem = exact_smem_bytes(cfg.ppwi, cfg.wgsize, cfg.tile, cfg.split, cfg.cluster);
  cudaError_t e;
  switch (cfg.ppwi) {
  case 1: e = launch_exact_p<1>(a, grid, cfg, smem, c.stream); break;
  case 2: e = launch_exact_p<2>(a, grid, cfg, smem, c.stream); break;
  case 4: e = launch_exact_p<4>(a, grid, cfg, smem, c.stream); break;
  case 8: e = launch_exact_p<8>(a, grid, cfg, smem, c.stream); break;
  default: e = launch_exact_p<16>(a, grid, cfg, smem, c.stream); break;
  }
  if (e != cudaSuccess) return cuda_error(e, "exact_kernel launch");
  c.launches++;
  if (global_reduce) {
    const int tb = 256;
    slice_reduce_kernel<<<(unsigned)((nposes + tb - 1) / tb), tb, 0, c.stream>>>(a.partial, cfg.split, nposes,
                                                                               a.energies);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(e, "slice_reduce_kernel launch");
    c.launches++;
  }
  return BUDE_OK;
}

// Self-test of the bounded wait: one thread waits on an mbarrier that nothing arrives on, with a
// limit of limit_ns, and sets bit 0 of the error word when the wait runs out -- the path every
// kernel of the library takes when one of its waits gives up.
static __global__ void wait_selftest_kernel(unsigned int *err, unsigned long long limit_ns) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_fence_init();
    if (!mbar_wait_bounded(&bar, 0, limit_ns)) atomicOr(err, 1u);
    mbar_inval(&bar);
  }
}

// Read (and clear) the device error word after the stream has drained.
int check_device_error(Context &c) {
  unsigned int h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, c.err.ptr, sizeof h, cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) return cuda_error(e, "device error word");
  if (h) {
    cudaMemsetAsync(c.err.ptr, 0, sizeof(unsigned int), c.stream);
    cudaStreamSynchronize(c.stream);
    return set_error(BUDE_ERR_TIMEOUT, "a bounded device wait ran out (error word 0x%x); energies are invalid", h);
  }
  return BUDE_OK;
}

static int upload_ligand(Context &c, const bude_atom *ligand, int natlig) {
  for (int i = 0; i < natlig; ++i)
    if (ligand[i].type < 0 || ligand[i].type >= c.ntypes)
      return set_error(BUDE_ERR_TYPE, "ligand atom %d has type %d outside the forcefield (%d types)", i,
                       ligand[i].type, c.ntypes);
  int rc = c.ligand.reserve((size_t)std::max(natlig, 1) * 16, "ligand");
  if (rc) return rc;
  c.deck_irregular = !ligand_regular(c, ligand, natlig, c.host_ff.data());
  if (natlig > 0) {
    // bude_atom is {x, y, z, int32 type}: the same 16 bytes as the kernel's float4 view.
    cudaError_t e = cudaMemcpyAsync(c.ligand.ptr, ligand, (size_t)natlig * 16, cudaMemcpyHostToDevice, c.stream);
    if (e != cudaSuccess) return cuda_error(e, "ligand upload");
  }
  c.natlig = natlig;
  return BUDE_OK;
}

static int upload_poses(Context &c, const float *poses, long long stride, long long nposes) {
  if (nposes < 0 || (nposes > 0 && (!poses || stride < nposes)))
    return set_error(BUDE_ERR_ARG, "bad pose block (nposes %lld, stride %lld)", nposes, stride);
  const long long n = std::max(nposes, 1LL);
  int rc = c.poses.reserve((size_t)6 * n * sizeof(float), "poses");
  if (!rc) rc = c.xform.reserve((size_t)12 * n * sizeof(float), "transforms");
  if (!rc) rc = c.energies.reserve((size_t)n * sizeof(float), "energies");
  if (!rc) rc = c.edge_mask.reserve((size_t)(n + 31) / 32 * sizeof(unsigned), "irregular-pose bits");
  if (rc) return rc;
  if (nposes > 0) {
    cudaError_t e = cudaMemcpy2DAsync(c.poses.ptr, (size_t)nposes * sizeof(float), poses, (size_t)stride * sizeof(float),
                                      (size_t)nposes * sizeof(float), 6, cudaMemcpyHostToDevice, c.stream);
    if (e != cudaSuccess) return cuda_error(e, "pose upload");
  }
  c.nposes = nposes;
  c.pose_stride = nposes;
  return BUDE_OK;
}

int upload_deck(Context &c, const bude_atom *protein, int natpro, const bude_atom *ligand, int natlig,
                const bude_ffparams *ff, int ntypes, const float *poses, long long stride, long long nposes) {
  c.have_deck = false; // a failed upload leaves no deck behind
  c.have_batch = false; // the slab now belongs to this deck
  if (natpro < 0 || natlig < 0 || ntypes <= 0 || !ff || (natpro > 0 && !protein) || (natlig > 0 && !ligand))
    return set_error(BUDE_ERR_ARG, "bad deck sizes or pointers (natpro %d, natlig %d, ntypes %d)", natpro, natlig,
                     ntypes);
  for (int i = 0; i < natpro; ++i)
    if (protein[i].type < 0 || protein[i].type >= ntypes)
      return set_error(BUDE_ERR_TYPE, "protein atom %d has type %d outside the forcefield (%d types)", i,
                       protein[i].type, ntypes);
  int rc = ensure_slab(c, protein, natpro, ff, ntypes);
  if (rc) return rc;
  rc = upload_ligand(c, ligand, natlig);
  if (!rc) rc = upload_poses(c, poses, stride, nposes);
  if (rc) return rc;
  cudaError_t e = cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) return cuda_error(e, "deck upload");
  c.have_deck = true;
  return BUDE_OK;
}

int set_poses(Context &c, const bude_atom *ligand, int natlig, const float *poses, long long stride,
              long long nposes) {
  if (!c.have_deck) return set_error(BUDE_ERR_STATE, "no deck uploaded");
  int rc = BUDE_OK;
  if (ligand) rc = upload_ligand(c, ligand, natlig);
  if (!rc) rc = upload_poses(c, poses, stride, nposes);
  return rc;
}

int make_context(int device, Context **out) {
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetDeviceCount");
  if (device < 0 || device >= count) return set_error(BUDE_ERR_ARG, "device %d out of range (%d devices)", device, count);
  e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
  auto *c = new bude_gpu_ctx();
  c->device = device;
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
  if (e != cudaSuccess) {
    destroy_context(c);
    return cuda_error(e, "stream/event creation");
  }
  int rc = c->err.reserve(sizeof(unsigned int) * 4, "error word");
  if (!rc) {
    e = cudaMemsetAsync(c->err.ptr, 0, sizeof(unsigned int) * 4, c->stream);
    if (e != cudaSuccess) rc = cuda_error(e, "error word");
  }
  if (rc) {
    destroy_context(c);
    return rc;
  }
  *out = c;
  return BUDE_OK;
}

void destroy_context(Context *c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  c->ligand.release();
  c->slab.release();
  c->poses.release();
  c->xform.release();
  c->energies.release();
  c->err.release();
  c->flush.release();
  c->partial.release();
  c->raw_protein.release();
  c->raw_ff.release();
  c->edge_mask.release();
  release_batch(*c);
  release_surrogate(*c);
  release_screen(*c);
  release_streamer(*c);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete static_cast<bude_gpu_ctx *>(c);
}

int flush_l2(Context &c) {
  const size_t bytes = 512ull << 20; // well above the 126 MB L2
  int rc = c.flush.reserve(bytes, "L2 flush buffer");
  if (rc) return rc;
  c.flush_gen = (c.flush_gen + 1) & 0xff;
  cudaError_t e = cudaMemsetAsync(c.flush.ptr, c.flush_gen, bytes, c.stream);
  if (e != cudaSuccess) return cuda_error(e, "L2 flush");
  return BUDE_OK;
}

} // namespace bude

// ---------------------------------------------------------------------------------------------
// C-ABI

extern "C" {

const char *bude_gpu_last_error(void) { return bude::last_error(); }

const char *bude_gpu_version(void) { return "minibude-gb300 0.1 (sm_103a)"; }

int bude_gpu_device_count(int *count) {
  if (!count) return set_error(BUDE_ERR_ARG, "count is NULL");
  cudaError_t e = cudaGetDeviceCount(count);
  if (e != cudaSuccess) {
    *count = 0;
    return cuda_error(e, "cudaGetDeviceCount");
  }
  return BUDE_OK;
}

int bude_gpu_device_name(int device, char *buf, size_t buflen) {
  if (!buf || buflen == 0) return set_error(BUDE_ERR_ARG, "empty name buffer");
  cudaDeviceProp p{};
  cudaError_t e = cudaGetDeviceProperties(&p, device);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetDeviceProperties");
  snprintf(buf, buflen, "%s (%zuMB;sm_%d%d)", p.name, (size_t)(p.totalGlobalMem / 1024 / 1024), p.major, p.minor);
  return BUDE_OK;
}

int bude_gpu_sm_count(int device, int *sms) {
  if (!sms) return set_error(BUDE_ERR_ARG, "sms is NULL");
  cudaError_t e = cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, device);
  return e == cudaSuccess ? BUDE_OK : cuda_error(e, "cudaDeviceGetAttribute");
}

int bude_gpu_compatible(int device, int *kernel_cc, int *device_cc, int *ok) {
  int kcc = 0;
  int rc = bude::probe_kernel_arch(device, &kcc);
  if (rc) return rc;
  cudaDeviceProp p{};
  cudaError_t e = cudaGetDeviceProperties(&p, device);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetDeviceProperties");
  const int dcc = p.major * 10 + p.minor;
  if (kernel_cc) *kernel_cc = kcc;
  if (device_cc) *device_cc = dcc;
  if (ok) *ok = kcc == dcc;
  return BUDE_OK;
}

int bude_gpu_create(int device, bude_gpu_ctx **out) {
  if (!out) return set_error(BUDE_ERR_ARG, "out is NULL");
  bude::Context *c = nullptr;
  int rc = bude::make_context(device, &c);
  *out = static_cast<bude_gpu_ctx *>(c);
  return rc;
}

int bude_gpu_destroy(bude_gpu_ctx *ctx) {
  bude::destroy_context(ctx);
  return BUDE_OK;
}

int bude_gpu_upload(bude_gpu_ctx *ctx, const bude_atom *protein, int32_t natpro, const bude_atom *ligand,
                    int32_t natlig, const bude_ffparams *forcefield, int32_t ntypes, const float *poses,
                    int64_t pose_stride, int64_t nposes) {
  if (!ctx) return set_error(BUDE_ERR_ARG, "ctx is NULL");
  cudaSetDevice(ctx->device);
  return bude::upload_deck(*ctx, protein, natpro, ligand, natlig, forcefield, ntypes, poses, pose_stride, nposes);
}

int bude_gpu_set_poses(bude_gpu_ctx *ctx, const bude_atom *ligand, int32_t natlig, const float *poses,
                       int64_t pose_stride, int64_t nposes) {
  if (!ctx) return set_error(BUDE_ERR_ARG, "ctx is NULL");
  cudaSetDevice(ctx->device);
  int rc = bude::set_poses(*ctx, ligand, natlig, poses, pose_stride, nposes);
  if (rc) return rc;
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  return e == cudaSuccess ? BUDE_OK : cuda_error(e, "pose upload");
}

int bude_gpu_default_cfg(const bude_gpu_ctx *ctx, int32_t ppwi, int32_t wgsize, bude_launch_cfg *cfg) {
  if (!ctx || !cfg) return set_error(BUDE_ERR_ARG, "NULL argument");
  return bude::default_cfg(*ctx, ppwi, wgsize, *cfg);
}

int bude_gpu_run(bude_gpu_ctx *ctx, const bude_launch_cfg *cfg, float *kernel_ms) {
  if (!ctx || !cfg) return set_error(BUDE_ERR_ARG, "NULL argument");
  cudaSetDevice(ctx->device);
  cudaError_t e = cudaEventRecord(ctx->ev0, ctx->stream);
  if (e != cudaSuccess) return cuda_error(e, "event record");
  int rc = bude::enqueue_eval(*ctx, *cfg);
  if (rc) return rc;
  e = cudaEventRecord(ctx->ev1, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_error(e, "evaluation");
  if (kernel_ms) {
    e = cudaEventElapsedTime(kernel_ms, ctx->ev0, ctx->ev1);
    if (e != cudaSuccess) return cuda_error(e, "event timing");
  }
  return bude::check_device_error(*ctx);
}

int bude_gpu_run_many(bude_gpu_ctx *ctx, const bude_launch_cfg *cfg, int32_t iterations, int32_t flush_l2,
                      float *ms_per_iter, float *exact_ms_per_iter) {
  if (!ctx || !cfg || iterations < 0) return set_error(BUDE_ERR_ARG, "bad argument");
  cudaSetDevice(ctx->device);
  // Three events per iteration: start, after the pose transforms, after the exact kernel.
  std::vector<cudaEvent_t> ev((size_t)iterations * 3, nullptr);
  int rc = BUDE_OK;
  cudaError_t e = cudaSuccess;
  for (auto &x : ev)
    if ((e = cudaEventCreate(&x)) != cudaSuccess) break;
  if (e != cudaSuccess) rc = cuda_error(e, "event creation");
  for (int i = 0; i < iterations && !rc; ++i) {
    if (flush_l2) rc = bude::flush_l2(*ctx);
    if (rc) break;
    cudaEventRecord(ev[3 * i], ctx->stream);
    rc = bude::enqueue_eval(*ctx, *cfg, ev[3 * i + 1]);
    cudaEventRecord(ev[3 * i + 2], ctx->stream);
  }
  e = cudaStreamSynchronize(ctx->stream);
  if (!rc && e != cudaSuccess) rc = cuda_error(e, "evaluation");
  for (int i = 0; i < iterations && !rc; ++i) {
    if (ms_per_iter) e = cudaEventElapsedTime(&ms_per_iter[i], ev[3 * i], ev[3 * i + 2]);
    if (e == cudaSuccess && exact_ms_per_iter) e = cudaEventElapsedTime(&exact_ms_per_iter[i], ev[3 * i + 1], ev[3 * i + 2]);
    if (e != cudaSuccess) rc = cuda_error(e, "event timing");
  }
  for (auto &x : ev)
    if (x) cudaEventDestroy(x);
  if (rc) return rc;
  return bude::check_device_error(*ctx);
}

int bude_gpu_download(bude_gpu_ctx *ctx, float *energies, int64_t nposes) {
  if (!ctx || (!energies && nposes > 0)) return set_error(BUDE_ERR_ARG, "NULL argument");
  if (!ctx->have_deck) return set_error(BUDE_ERR_STATE, "no deck uploaded");
  if (nposes != ctx->nposes)
    return set_error(BUDE_ERR_ARG, "download of %lld energies but %lld poses are uploaded", (long long)nposes,
                     ctx->nposes);
  if (nposes == 0) return BUDE_OK;
  cudaSetDevice(ctx->device);
  cudaError_t e = cudaMemcpyAsync(energies, ctx->energies.ptr, (size_t)nposes * sizeof(float), cudaMemcpyDeviceToHost,
                                  ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  return e == cudaSuccess ? BUDE_OK : cuda_error(e, "energy download");
}

int bude_gpu_score_host(bude_gpu_ctx *ctx, const bude_launch_cfg *cfg, const bude_atom *ligand, int32_t natlig,
                        const float *poses, int64_t pose_stride, int64_t nposes, float *energies) {
  if (!ctx || !cfg || (!energies && nposes > 0)) return set_error(BUDE_ERR_ARG, "NULL argument");
  cudaSetDevice(ctx->device);
  int rc = bude::set_poses(*ctx, ligand, natlig, poses, pose_stride, nposes);
  if (!rc) rc = bude::enqueue_eval(*ctx, *cfg);
  if (rc) return rc;
  if (nposes > 0) {
    cudaError_t e = cudaMemcpyAsync(energies, ctx->energies.ptr, (size_t)nposes * sizeof(float),
                                    cudaMemcpyDeviceToHost, ctx->stream);
    if (e != cudaSuccess) return cuda_error(e, "energy download");
  }
  return bude::check_device_error(*ctx); // synchronises the stream
}

int bude_gpu_fasten(int device, int32_t ppwi, int32_t wgsize, const bude_atom *protein, int32_t natpro,
                    const bude_atom *ligand, int32_t natlig, const bude_ffparams *forcefield, int32_t ntypes,
                    const float *poses, int64_t pose_stride, int64_t nposes, int32_t iterations, float *energies,
                    float *kernel_ms, float *context_ms) {
  if (iterations < 1) return set_error(BUDE_ERR_ARG, "iterations must be >= 1");
  bude_gpu_ctx *ctx = nullptr;
  int rc = bude_gpu_create(device, &ctx);
  if (rc) return rc;
  auto t0 = std::chrono::steady_clock::now();
  rc = bude_gpu_upload(ctx, protein, natpro, ligand, natlig, forcefield, ntypes, poses, pose_stride, nposes);
  auto t1 = std::chrono::steady_clock::now();
  if (context_ms) *context_ms = std::chrono::duration<float, std::milli>(t1 - t0).count();
  bude_launch_cfg cfg;
  if (!rc) rc = bude_gpu_default_cfg(ctx, ppwi, wgsize, &cfg);
  for (int i = 0; i < iterations && !rc; ++i) rc = bude_gpu_run(ctx, &cfg, kernel_ms ? &kernel_ms[i] : nullptr);
  if (!rc) rc = bude_gpu_download(ctx, energies, nposes);
  std::string keep = rc ? bude::last_error() : "";
  bude_gpu_destroy(ctx);
  if (rc) bude::set_error(rc, "%s", keep.c_str());
  return rc;
}

int bude_gpu_selftest_wait(bude_gpu_ctx *ctx, int32_t limit_us, float *elapsed_ms) {
  if (!ctx) return set_error(BUDE_ERR_ARG, "NULL context");
  if (limit_us < 1 || limit_us > 1000000) return set_error(BUDE_ERR_ARG, "limit_us must be in [1, 1000000]");
  bude::Context &c = *ctx;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, c.stream);
  bude::wait_selftest_kernel<<<1, 32, 0, c.stream>>>(c.err.as<unsigned>(), 1000ull * (unsigned long long)limit_us);
  cudaError_t e = cudaGetLastError();
  cudaEventRecord(e1, c.stream);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  if (e == cudaSuccess && elapsed_ms) cudaEventElapsedTime(elapsed_ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return cuda_error(e, "wait_selftest_kernel");
  c.launches++;
  return bude::check_device_error(c);
}

int bude_gpu_launch_count(const bude_gpu_ctx *ctx, int64_t *count) {
  if (!ctx || !count) return set_error(BUDE_ERR_ARG, "NULL argument");
  *count = ctx->launches;
  return BUDE_OK;
}

int bude_host_alloc(size_t bytes, void **ptr) {
  if (!ptr) return set_error(BUDE_ERR_ARG, "ptr is NULL");
  cudaError_t e = cudaMallocHost(ptr, std::max<size_t>(bytes, 1));
  return e == cudaSuccess ? BUDE_OK : cuda_error(e, "cudaMallocHost");
}

int bude_host_free(void *ptr) {
  cudaError_t e = cudaFreeHost(ptr);
  return e == cudaSuccess ? BUDE_OK : cuda_error(e, "cudaFreeHost");
}

} // extern "C"
