// surrogate.cu -- host side of the learned pre-screen (kernels in surrogate_kernels.cuh).
//
// No counterpart in the reference.  A per-protein MLP is trained on exact energies of the
// context's uploaded batch (computed here with the batched exact kernel) and then scores poses
// for the screening pipeline (screen.cu), where the exact kernel rescores its picks and remains
// the arbiter of its error.  Forward, backward and Adam are hand-written kernels driven from this file; every
// reduction (weight, bias and embedding gradients, the loss) is summed in a fixed order, so a
// training run is deterministic for a given seed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <random>
#include <utility>
#include <vector>

#include "exact_kernel.cuh"
#include "internal.h"
#include "score_tc.cuh"
#include "surrogate_kernels.cuh"
#include "wgrad_tc.cuh"

namespace bude {

// FP32 parameter layout (masters, Adam moments and gradients share it).
constexpr long long kOffEmb = 0;
constexpr long long kOffW1 = kOffEmb + kMaxTypes * kEmb;
constexpr long long kOffB1 = kOffW1 + kHid * kFeat;
constexpr long long kOffW2 = kOffB1 + kHid;
constexpr long long kOffB2 = kOffW2 + kHid * kHid;
constexpr long long kOffW3 = kOffB2 + kHid;
constexpr long long kOffB3 = kOffW3 + kHid * kHid;
constexpr long long kOffW4 = kOffB3 + kHid;
constexpr long long kOffB4 = kOffW4 + kHid;
constexpr long long kNParams = kOffB4 + 4;

static_assert(kNParams == BUDE_SURROGATE_NPARAMS, "parameter count in the header must match");

struct Surrogate {
  bool ready = false;
  int ntypes = 0;
  DevBuf params, adam_m, adam_v, grads;
  DevBuf emb_bf, w1_bf, w2_bf, w3_bf, w2t_bf, w3t_bf; // w2t, w3t: transposed copies (backward pass)
  DevBuf emb_h, w1_h, w2_h, w3_h; // FP16 copies for the tcgen05 scorer
  float w4_host[kHid] = {};        // host copy of the output weights (scorer launch parameters)
  bool w4_host_valid = false;      // false whenever the weights may have changed
  DevBuf grid, protein4;
  cudaArray_t tex_arr[4] = {};
  cudaTextureObject_t tex[4] = {};
  FieldGrid fg{};
  long long step = 0;
  // training scratch
  DevBuf X, row_type, Z1, Z2, Z3, dZ1, dZ2, dZ3, y, dy, pred, loss, dsum, part_w, S_sum;
  DevBuf labels, pose_lig_first, pose_lig_n, epoch_pose, epoch_rowoff, epoch_pose2, epoch_rowoff2, epoch_loss;
  long long rows_cap = 0;
  // scoring
  DevBuf items, scores, next;
  std::vector<int> item_lig_off; // nligands + 1: first scoring item of each ligand
  long long items_for = -1; // Context::batch_gen the items were built for
  int n_items = 0;
  int scorer = BUDE_SCORER_TCGEN05;
};

static Surrogate &sur(Context &c) {
  if (!c.surrogate) c.surrogate = new Surrogate();
  return *c.surrogate;
}

static void release_textures(Surrogate &s) {
  for (int q = 0; q < 4; ++q) {
    if (s.tex[q]) cudaDestroyTextureObject(s.tex[q]);
    if (s.tex_arr[q]) cudaFreeArray(s.tex_arr[q]);
    s.tex[q] = 0;
    s.tex_arr[q] = nullptr;
  }
}

void release_surrogate(Context &c) {
  if (!c.surrogate) return;
  Surrogate &s = *c.surrogate;
  release_textures(s);
  DevBuf *all[] = {&s.params, &s.adam_m, &s.adam_v, &s.grads, &s.emb_bf, &s.w1_bf, &s.w2_bf, &s.w3_bf,
                   &s.w2t_bf, &s.w3t_bf, &s.emb_h, &s.w1_h, &s.w2_h, &s.w3_h, &s.grid, &s.protein4, &s.X, &s.row_type, &s.Z1,
                   &s.Z2, &s.Z3, &s.dZ1, &s.dZ2, &s.dZ3, &s.y, &s.dy, &s.pred, &s.loss, &s.dsum,
                   &s.part_w, &s.S_sum, &s.labels, &s.pose_lig_first, &s.pose_lig_n,
                   &s.epoch_pose, &s.epoch_rowoff, &s.epoch_pose2, &s.epoch_rowoff2, &s.epoch_loss, &s.items,
                   &s.scores, &s.next};
  for (DevBuf *b : all) b->release();
  delete c.surrogate;
  c.surrogate = nullptr;
}

static MlpWeights weights(Surrogate &s) {
  MlpWeights W;
  W.emb = s.emb_bf.as<__nv_bfloat16>();
  W.w1 = s.w1_bf.as<__nv_bfloat16>();
  W.w2 = s.w2_bf.as<__nv_bfloat16>();
  W.w3 = s.w3_bf.as<__nv_bfloat16>();
  const float *p = s.params.as<float>();
  W.b1 = p + kOffB1;
  W.b2 = p + kOffB2;
  W.b3 = p + kOffB3;
  W.w4 = p + kOffW4;
  W.b4 = p + kOffB4;
  return W;
}

// The BF16 copies of the weights (plain, and transposed for the backward pass).
static BfCopies bf_copies(Surrogate &s) {
  BfCopies c{};
  auto add = [&](long long off, int rows, int cols, DevBuf *plain, DevBuf *trans, DevBuf *half) {
    const int k = c.n++;
    c.off[k] = off;
    c.rows[k] = rows;
    c.cols[k] = cols;
    c.plain[k] = plain ? plain->as<__nv_bfloat16>() : nullptr;
    c.trans[k] = trans ? trans->as<__nv_bfloat16>() : nullptr;
    c.half[k] = half ? half->as<__half>() : nullptr;
  };
  add(kOffEmb, kMaxTypes, kEmb, &s.emb_bf, nullptr, &s.emb_h);
  add(kOffW1, kHid, kFeat, &s.w1_bf, nullptr, &s.w1_h);
  add(kOffW2, kHid, kHid, &s.w2_bf, &s.w2t_bf, &s.w2_h);
  add(kOffW3, kHid, kHid, &s.w3_bf, &s.w3t_bf, &s.w3_h);
  return c;
}

// Refresh the BF16 copies of the weights from the FP32 masters.
static int publish(Context &c, Surrogate &s) {
  s.w4_host_valid = false;
  publish_kernel<<<(unsigned)((kOffW3 + kHid * kHid + 255) / 256), 256, 0, c.stream>>>(s.params.as<float>(),
                                                                                      kOffW3 + kHid * kHid, bf_copies(s));
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? BUDE_OK : cuda_error(e, "surrogate publish");
}

static int set_smem_limits() {
  static bool done = false;
  if (done) return BUDE_OK;
  cudaError_t e = cudaFuncSetAttribute(score_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(MlpSmem));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(score_tc_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TcSmem<4>));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(score_tc_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TcSmem<3>));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(wgrad_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(WgTcSmem));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(train_forward_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sizeof(TcSmem<kTcGroups>));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(train_backward_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sizeof(TcBwdSmem<kBwdGroups>));
  if (e != cudaSuccess) return cuda_error(e, "surrogate shared-memory limits");
  done = true;
  return BUDE_OK;
}

// The scaled FP32 grid (s.grid, n^3 voxels x 16) as four FP16 3-D textures with trilinear
// filtering, clamped addressing and unnormalised coordinates.
static int make_textures(Context &c, Surrogate &s, int n) {
  release_textures(s);
  const long long nvox = (long long)n * n * n;
  DevBuf lin;
  int rc = lin.reserve((size_t)nvox * 13 * sizeof(__half), "texture staging");
  if (rc) return rc;
  __half *t0 = lin.as<__half>(), *t1 = t0 + nvox * 4, *t2 = t1 + nvox * 4, *t3 = t2 + nvox * 4;
  grid_pack_kernel<<<(unsigned)((nvox + 255) / 256), 256, 0, c.stream>>>(s.grid.as<float>(), nvox, t0, t1, t2, t3);
  cudaError_t e = cudaStreamSynchronize(c.stream);
  const __half *src[4] = {t0, t1, t2, t3};
  for (int q = 0; q < 4 && e == cudaSuccess; ++q) {
    const int ch = q < 3 ? 4 : 1;
    cudaChannelFormatDesc fd = cudaCreateChannelDesc(16, ch > 1 ? 16 : 0, ch > 1 ? 16 : 0, ch > 1 ? 16 : 0,
                                                     cudaChannelFormatKindFloat);
    e = cudaMalloc3DArray(&s.tex_arr[q], &fd, make_cudaExtent(n, n, n));
    if (e != cudaSuccess) break;
    cudaMemcpy3DParms cp = {};
    cp.srcPtr = make_cudaPitchedPtr(const_cast<__half *>(src[q]), (size_t)n * ch * sizeof(__half), n, n);
    cp.dstArray = s.tex_arr[q];
    cp.extent = make_cudaExtent(n, n, n);
    cp.kind = cudaMemcpyDeviceToDevice;
    e = cudaMemcpy3D(&cp);
    if (e != cudaSuccess) break;
    cudaResourceDesc rd = {};
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = s.tex_arr[q];
    cudaTextureDesc td = {};
    td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 0;
    e = cudaCreateTextureObject(&s.tex[q], &rd, &td, nullptr);
  }
  lin.release();
  if (e != cudaSuccess) {
    release_textures(s);
    return cuda_error(e, "field grid textures");
  }
  return BUDE_OK;
}

// The protein of the context (kept from the last upload) as float4 records for the grid kernel.
int surrogate_init(Context &c, const bude_atom *protein, int natpro, const bude_ffparams *ff, int ntypes, float extent,
                   float spacing, unsigned long long seed) {
  if (ntypes <= 0 || ntypes > kMaxTypes)
    return set_error(BUDE_ERR_ARG, "the surrogate supports 1..%d forcefield types (got %d)", kMaxTypes, ntypes);
  if (!(extent > 0.f) || !(spacing > 0.f) || extent / spacing > 200.f)
    return set_error(BUDE_ERR_ARG, "bad grid extent %g / spacing %g (at most 400 points a side)", extent, spacing);
  if (natpro < 0 || (natpro > 0 && !protein) || !ff) return set_error(BUDE_ERR_ARG, "bad protein");
  for (int i = 0; i < natpro; ++i)
    if (protein[i].type < 0 || protein[i].type >= ntypes)
      return set_error(BUDE_ERR_TYPE, "protein atom %d has type %d outside the forcefield", i, protein[i].type);
  int rc = set_smem_limits();
  if (rc) return rc;
  Surrogate &s = sur(c);
  s.ready = false;
  s.ntypes = ntypes;
  s.step = 0;
  // Parameters: torch-Linear-style uniform(+-1/sqrt(fan_in)) weights and biases, N(0,1) embedding.
  std::vector<float> p(kNParams, 0.f);
  std::mt19937_64 rng(seed);
  std::normal_distribution<float> nd(0.f, 1.f);
  for (long long i = 0; i < kMaxTypes * kEmb; ++i) p[kOffEmb + i] = nd(rng);
  auto uni = [&](long long off, long long n, int fan_in) {
    std::uniform_real_distribution<float> ud(-1.f / std::sqrt((float)fan_in), 1.f / std::sqrt((float)fan_in));
    for (long long i = 0; i < n; ++i) p[off + i] = ud(rng);
  };
  uni(kOffW1, kHid * kFeat, kFeat);
  uni(kOffB1, kHid, kFeat);
  uni(kOffW2, kHid * kHid, kHid);
  uni(kOffB2, kHid, kHid);
  uni(kOffW3, kHid * kHid, kHid);
  uni(kOffB3, kHid, kHid);
  uni(kOffW4, kHid, kHid);
  uni(kOffB4, 1, kHid);
  const size_t pb = kNParams * sizeof(float);
  rc = s.params.reserve(pb, "surrogate params");
  if (!rc) rc = s.adam_m.reserve(pb, "adam m");
  if (!rc) rc = s.adam_v.reserve(pb, "adam v");
  if (!rc) rc = s.grads.reserve(pb, "surrogate grads");
  if (!rc) rc = s.emb_bf.reserve(kMaxTypes * kEmb * 2, "emb bf16");
  if (!rc) rc = s.w1_bf.reserve(kHid * kFeat * 2, "w1 bf16");
  if (!rc) rc = s.w2_bf.reserve(kHid * kHid * 2, "w2 bf16");
  if (!rc) rc = s.w2t_bf.reserve(kHid * kHid * 2, "w2t bf16");
  if (!rc) rc = s.w3_bf.reserve(kHid * kHid * 2, "w3 bf16");
  if (!rc) rc = s.w3t_bf.reserve(kHid * kHid * 2, "w3t bf16");
  if (!rc) rc = s.emb_h.reserve(kMaxTypes * kEmb * 2, "emb fp16");
  if (!rc) rc = s.w1_h.reserve(kHid * kFeat * 2, "w1 fp16");
  if (!rc) rc = s.w2_h.reserve(kHid * kHid * 2, "w2 fp16");
  if (!rc) rc = s.w3_h.reserve(kHid * kHid * 2, "w3 fp16");
  if (rc) return rc;
  cudaError_t e = copy_sync(c, s.params.ptr, p.data(), pb, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = fill_sync(c, s.adam_m.ptr, 0, pb);
  if (e == cudaSuccess) e = fill_sync(c, s.grads.ptr, 0, pb); // the padding after b4 is never written
  if (e == cudaSuccess) e = fill_sync(c, s.adam_v.ptr, 0, pb);
  if (e != cudaSuccess) return cuda_error(e, "surrogate init");

  // Field grid over [-extent, extent]^3.
  const int n = (int)std::ceil(2.f * extent / spacing) + 1;
  const long long nvox = (long long)n * n * n;
  rc = s.grid.reserve((size_t)nvox * 16 * sizeof(float), "field grid");
  if (!rc) rc = s.protein4.reserve((size_t)std::max(natpro, 1) * 16, "grid protein");
  DevBuf dff, inv;
  if (!rc) rc = dff.reserve((size_t)ntypes * sizeof(bude_ffparams), "grid forcefield");
  if (!rc) rc = inv.reserve(16 * sizeof(float), "grid scales");
  if (rc) return rc;
  e = copy_sync(c, s.protein4.ptr, protein, (size_t)natpro * 16, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = copy_sync(c, dff.ptr, ff, (size_t)ntypes * sizeof(bude_ffparams), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    dff.release();
    inv.release();
    return cuda_error(e, "grid inputs");
  }
  GridBuild gb;
  gb.protein = s.protein4.as<float4>();
  gb.ff = dff.as<bude_ffparams>();
  gb.natpro = natpro;
  gb.ox = gb.oy = gb.oz = -extent;
  gb.h = spacing;
  gb.nx = gb.ny = gb.nz = n;
  gb.out = s.grid.as<float>();
  grid_kernel<<<(unsigned)((nvox + 127) / 128), 128, 0, c.stream>>>(gb);
  e = cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) {
    dff.release();
    inv.release();
    return cuda_error(e, "field grid");
  }
  // Unit standard deviation per channel (a zero channel keeps scale 1).
  std::vector<float> h((size_t)nvox * 16);
  e = copy_sync(c, h.data(), s.grid.ptr, h.size() * sizeof(float), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    dff.release();
    inv.release();
    return cuda_error(e, "field grid read-back");
  }
  float scale[16];
  for (int k = 0; k < 16; ++k) {
    double m = 0, m2 = 0;
    for (long long v = 0; v < nvox; ++v) {
      const double x = h[(size_t)v * 16 + k];
      m += x;
      m2 += x * x;
    }
    m /= (double)nvox;
    const double var = std::max(0.0, m2 / (double)nvox - m * m);
    scale[k] = var > 1e-12 ? (float)(1.0 / std::sqrt(var)) : 1.f;
  }
  e = copy_sync(c, inv.ptr, scale, sizeof scale, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    dff.release();
    inv.release();
    return cuda_error(e, "grid scales");
  }
  grid_scale_kernel<<<(unsigned)((nvox * 16 + 255) / 256), 256, 0, c.stream>>>(s.grid.as<float>(), nvox,
                                                                             inv.as<float>());
  e = cudaStreamSynchronize(c.stream);
  dff.release();
  inv.release();
  if (e != cudaSuccess) return cuda_error(e, "field grid scaling");
  rc = make_textures(c, s, n);
  s.grid.release();
  if (rc) return rc;
  for (int q = 0; q < 4; ++q) s.fg.tex[q] = s.tex[q];
  s.fg.ox = s.fg.oy = s.fg.oz = -extent;
  s.fg.inv_h = 1.f / spacing;
  s.fg.xyz_scale = 0.1f;
  rc = publish(c, s);
  if (rc) return rc;
  s.ready = true;
  return BUDE_OK;
}

static int ensure_train_scratch(Surrogate &s, long long rows, int batch, int wg_blocks) {
  int rc = BUDE_OK;
  if (rows > s.rows_cap) {
    // The row-tiled arrays (tc.cuh: tiled_offset) hold whole 128-row tiles.
    const size_t r = (size_t)tiled_rows(rows);
    rc = s.X.reserve(r * kFeat * 2, "X");
    if (!rc) rc = s.row_type.reserve(r * 4, "row types");
    for (DevBuf *b : {&s.Z1, &s.Z2, &s.Z3, &s.dZ1, &s.dZ2, &s.dZ3})
      if (!rc) rc = b->reserve(r * kHid * 2, "activations");
    if (!rc) rc = s.y.reserve(r * 4, "y");
    if (!rc) rc = s.dy.reserve(r * 4, "dy");
    if (rc) return rc;
    s.rows_cap = (long long)r;
  }
  if (!rc) rc = s.pred.reserve((size_t)batch * 4, "pred");
  if (!rc) rc = s.loss.reserve((size_t)batch * 4, "loss");
  if (!rc) rc = s.dsum.reserve((size_t)batch * 4, "per-pose dy sums");
  if (!rc) rc = s.part_w.reserve((size_t)std::max(wg_blocks, 1) * kWgPart * 4, "gradient parts");
  if (!rc) rc = s.S_sum.reserve((size_t)kHid * kMaxTypes * 4, "per-type dz1 sums");
  return rc;
}

// Launch one kernel of a training step with programmatic stream serialisation: its blocks are
// scheduled as the kernel before it finishes, and run their setup (barriers, TMEM allocation) until
// grid_dep_wait (ptx.cuh) while that kernel's completion is processed.  Every kernel launched this
// way waits before it touches the step's buffers.  80 epochs of 512 ligands x 4096 poses: 6.03 s
// this way, 6.48 s in plain stream order.
template <class... KArgs, class... Args>
static cudaError_t launch_chained(void (*kernel)(KArgs...), unsigned grid, unsigned block, size_t smem,
                                  cudaStream_t st, Args &&...args) {
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// One optimisation step on `nb` poses whose indices/row offsets are at dpose/drowoff; the poses'
// squared errors go to loss_out (device, nb floats; nullptr: the scratch array s.loss).
static int train_step(Context &c, Surrogate &s, const int *dpose, const int *drowoff, int nb, long long rows, float lr,
                      float *loss_out) {
  const float *p = s.params.as<float>();
  float *gr = s.grads.as<float>();
  RowMap m;
  m.pose = dpose;
  m.row_off = drowoff;
  m.lig_first = s.pose_lig_first.as<int>();
  m.lig_n = s.pose_lig_n.as<int>();
  m.nposes = nb;
  const MlpWeights W = weights(s);
  // One gradient block per SM, each with at least one 128-row tile.
  const int wg_grid = (int)std::min<long long>((rows + kWgTile - 1) / kWgTile, std::max(c.num_sms, 1));
  int rc = ensure_train_scratch(s, rows, nb, wg_grid);
  if (!rc) rc = s.next.reserve(256, "work counters");
  if (rc) return rc;
  // The step's kernels run as one chain of programmatic dependent launches (launch_chained); the
  // features kernel zeroes the forward (next[0]) and backward (next[1]) tile counters.
  unsigned int *counters = s.next.as<unsigned int>();
  cudaError_t le = launch_chained(train_features_kernel, (unsigned)((nb * 32 + 255) / 256), 256u, 0, c.stream, W,
                                  s.fg, c.b_ligands.as<float4>(), c.b_xform.as<float4>(), m,
                                  s.X.as<__nv_bfloat16>(), s.row_type.as<int>(), counters);
  {
    // Forward on the tensor cores (score_tc.cuh): z1, z2, z3 as BF16 and y per row.
    TrainFwdTcArgs f;
    f.W = W;
    f.X = s.X.as<__nv_bfloat16>();
    f.rows = (int)rows;
    f.Z1 = s.Z1.as<__nv_bfloat16>();
    f.Z2 = s.Z2.as<__nv_bfloat16>();
    f.Z3 = s.Z3.as<__nv_bfloat16>();
    f.y = s.y.as<float>();
    f.err = c.err.as<unsigned int>();
    f.next = counters;
    const int ftiles = (int)((rows + kTcGroupThreads - 1) / kTcGroupThreads);
    const int grid = std::max(1, std::min((ftiles + kTcGroups - 1) / kTcGroups, std::max(c.num_sms, 1)));
    if (le == cudaSuccess)
      le = launch_chained(train_forward_tc_kernel, (unsigned)grid, (unsigned)(kTcGroups * kTcGroupThreads),
                          sizeof(TcSmem<kTcGroups>), c.stream, f);
  }
  if (le == cudaSuccess)
    le = launch_chained(train_loss_kernel, (unsigned)((nb + kLossPoses - 1) / kLossPoses), 32u * kLossPoses, 0,
                        c.stream, m, s.y.as<float>(), p + kOffB4, s.labels.as<float>(), s.pred.as<float>(),
                        loss_out ? loss_out : s.loss.as<float>(), s.dy.as<float>(), s.dsum.as<float>(),
                        1.f / (float)nb);
  {
    // Backward through the hidden layers on the tensor cores (score_tc.cuh): dz3, dz2, dz1 as BF16.
    TrainBwdTcArgs b;
    b.w3t = s.w3t_bf.as<__nv_bfloat16>();
    b.w2t = s.w2t_bf.as<__nv_bfloat16>();
    b.w4 = p + kOffW4;
    b.Z1 = s.Z1.as<__nv_bfloat16>();
    b.Z2 = s.Z2.as<__nv_bfloat16>();
    b.Z3 = s.Z3.as<__nv_bfloat16>();
    b.dy = s.dy.as<float>();
    b.rows = (int)rows;
    b.dZ1 = s.dZ1.as<__nv_bfloat16>();
    b.dZ2 = s.dZ2.as<__nv_bfloat16>();
    b.dZ3 = s.dZ3.as<__nv_bfloat16>();
    b.err = c.err.as<unsigned int>();
    b.next = counters + 1;
    const int btiles = (int)((rows + kTcGroupThreads - 1) / kTcGroupThreads);
    const int grid = std::max(1, std::min((btiles + kBwdGroups - 1) / kBwdGroups, std::max(c.num_sms, 1)));
    if (le == cudaSuccess)
      le = launch_chained(train_backward_tc_kernel, (unsigned)grid, (unsigned)(kBwdGroups * kTcGroupThreads),
                          sizeof(TcBwdSmem<kBwdGroups>), c.stream, b);
  }
  // Weight, bias and embedding gradients on the tensor cores (wgrad_tc.cuh): per-block partial
  // sums over contiguous row tiles, folded in block order.
  WgTcArgs w;
  w.X = s.X.as<__nv_bfloat16>();
  w.row_type = s.row_type.as<int>();
  w.Z1 = s.Z1.as<__nv_bfloat16>();
  w.Z2 = s.Z2.as<__nv_bfloat16>();
  w.Z3 = s.Z3.as<__nv_bfloat16>();
  w.dZ1 = s.dZ1.as<__nv_bfloat16>();
  w.dZ2 = s.dZ2.as<__nv_bfloat16>();
  w.dZ3 = s.dZ3.as<__nv_bfloat16>();
  w.dy = s.dy.as<float>();
  w.rows = (int)rows;
  w.part = s.part_w.as<float>();
  w.err = c.err.as<unsigned int>();
  if (le == cudaSuccess)
    le = launch_chained(wgrad_tc_kernel, (unsigned)wg_grid, (unsigned)(kWgThreads + 64), sizeof(WgTcSmem), c.stream,
                        w);
  ReduceSegs red{};
  // Matrix segments come column by column from the gradient kernel (wgrad_tc.cuh) and go back
  // row-major ([out][in]) into the gradient vector.
  auto reduce = [&](const float *part, int nparts, long long n, long long stride, float *dst, int tr_cols = 0) {
    const int k = red.nseg++;
    red.part[k] = part;
    red.dst[k] = dst;
    red.stride[k] = stride;
    red.n[k] = (int)n;
    red.nparts[k] = nparts;
    red.tr_rows[k] = tr_cols > 0 ? kHid : 0;
    red.tr_cols[k] = tr_cols;
    red.first[k + 1] = red.first[k] + (int)n;
  };
  const float *part = s.part_w.as<float>();
  reduce(part + kWgOffW3, wg_grid, kHid * kHid, kWgPart, gr + kOffW3, kHid);
  reduce(part + kWgOffB3, wg_grid, kHid, kWgPart, gr + kOffB3);
  reduce(part + kWgOffW2, wg_grid, kHid * kHid, kWgPart, gr + kOffW2, kHid);
  reduce(part + kWgOffB2, wg_grid, kHid, kWgPart, gr + kOffB2);
  reduce(part + kWgOffW1, wg_grid, kHid * kFeat, kWgPart, gr + kOffW1, kFeat);
  reduce(part + kWgOffB1, wg_grid, kHid, kWgPart, gr + kOffB1);
  reduce(part + kWgOffW4, wg_grid, kHid, kWgPart, gr + kOffW4);
  reduce(part + kWgOffS, wg_grid, kHid * kMaxTypes, kWgPart, s.S_sum.as<float>(), kMaxTypes);
  reduce(s.dsum.as<float>(), (nb + kLossPoses - 1) / kLossPoses, 1, 1, gr + kOffB4);
  if (le == cudaSuccess)
    le = launch_chained(reduce_segments_kernel, (unsigned)((red.first[red.nseg] + 31) / 32), 32u * kReduceWarps, 0,
                        c.stream, red);
  if (le == cudaSuccess)
    le = launch_chained(emb_grad_kernel, (unsigned)((kMaxTypes * kEmb * 32 + 255) / 256), 256u, 0, c.stream,
                        s.S_sum.as<float>(), s.w1_bf.as<__nv_bfloat16>(), gr + kOffEmb);
  if (lr > 0.f) {
    s.step++;
    s.w4_host_valid = false;
    const float b1 = 0.9f, b2 = 0.999f;
    const double bc1 = 1.0 - std::pow((double)b1, (double)s.step), bc2 = 1.0 - std::pow((double)b2, (double)s.step);
    if (le == cudaSuccess)
      le = launch_chained(adam_kernel, (unsigned)((kNParams + 255) / 256), 256u, 0, c.stream, s.params.as<float>(),
                          s.adam_m.as<float>(), s.adam_v.as<float>(), (const float *)gr, (long long)kNParams,
                          (float)(lr / bc1), (float)std::sqrt(bc2), b1, b2, 1e-8f, bf_copies(s));
  }
  if (le != cudaSuccess) return cuda_error(le, "surrogate training step launch");
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "surrogate training step");
  return BUDE_OK;
}

// Pose -> (first ligand atom, natlig) for every pose of the uploaded batch.
static int upload_pose_ligands(Context &c, Surrogate &s, std::vector<int> &lig_n) {
  const long long np = c.batch_poses;
  std::vector<int> first((size_t)np);
  lig_n.assign((size_t)np, 0);
  for (int l = 0; l < c.nligands; ++l)
    for (long long p = c.pose_off[l]; p < c.pose_off[l + 1]; ++p) {
      first[(size_t)p] = c.lig_off[l];
      lig_n[(size_t)p] = c.lig_off[l + 1] - c.lig_off[l];
    }
  int rc = s.pose_lig_first.reserve((size_t)std::max(np, 1LL) * 4, "pose ligands");
  if (!rc) rc = s.pose_lig_n.reserve((size_t)std::max(np, 1LL) * 4, "pose ligands");
  if (rc) return rc;
  if (np > 0) {
    cudaError_t e = copy_sync(c, s.pose_lig_first.ptr, first.data(), (size_t)np * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = copy_sync(c, s.pose_lig_n.ptr, lig_n.data(), (size_t)np * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_error(e, "pose ligands");
  }
  return BUDE_OK;
}

static int batch_transforms(Context &c) {
  if (c.batch_poses == 0) return BUDE_OK;
  const int tb = 256;
  pose_xform_kernel<<<(unsigned)((c.batch_poses + tb - 1) / tb), tb, 0, c.stream>>>(
      c.b_poses.as<float>(), c.batch_poses, c.batch_poses, c.b_xform.as<float4>(), c.b_edge_mask.as<unsigned>());
  c.launches++;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? BUDE_OK : cuda_error(e, "pose transforms");
}

// The batch's atom types index the surrogate's embedding table.
static int check_batch_types(const Context &c) {
  if (c.ntypes > kMaxTypes)
    return set_error(BUDE_ERR_ARG, "the uploaded batch has %d forcefield types; the surrogate embeds at most %d",
                     c.ntypes, kMaxTypes);
  return BUDE_OK;
}

int surrogate_train(Context &c, int epochs, int batch, float lr, const float *labels, float *final_loss,
                    float *train_ms, unsigned long long seed) {
  Surrogate &s = sur(c);
  if (!s.ready) return set_error(BUDE_ERR_STATE, "surrogate not initialised");
  if (!c.have_batch) return set_error(BUDE_ERR_STATE, "no batch uploaded");
  if (check_batch_types(c)) return BUDE_ERR_ARG;
  if (epochs < 0 || batch <= 0) return set_error(BUDE_ERR_ARG, "bad epochs/batch");
  const long long np = c.batch_poses;
  if (np == 0) return set_error(BUDE_ERR_ARG, "empty batch");
  int rc = s.labels.reserve((size_t)np * 4, "labels");
  if (rc) return rc;
  if (labels) {
    const cudaError_t e = copy_sync(c, s.labels.ptr, labels, (size_t)np * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_error(e, "labels");
  } else {
    // Labels: exact energies of every pose from the batched exact kernel.
    bude_launch_cfg cfg{16, 128, 1, 64, 1, 0};
    rc = enqueue_batch(c, cfg, 0);
    if (!rc) rc = check_device_error(c);
    if (rc) return rc;
    cudaMemcpyAsync(s.labels.ptr, c.b_energies.ptr, (size_t)np * 4, cudaMemcpyDeviceToDevice, c.stream);
  }
  std::vector<int> lig_n;
  rc = upload_pose_ligands(c, s, lig_n);
  if (!rc) rc = batch_transforms(c);
  if (rc) return rc;
  // The poses learnt from: regular ones (edge_pose.cuh: finite transforms, translations and atoms
  // within bounds) with finite labels.  Every pose of an ordinary batch qualifies.
  std::vector<float> hl((size_t)np);
  std::vector<unsigned> edge((size_t)(np + 31) / 32);
  cudaError_t e = copy_sync(c, hl.data(), s.labels.ptr, (size_t)np * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = copy_sync(c, edge.data(), c.b_edge_mask.ptr, edge.size() * 4, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_error(e, "labels read-back");
  std::vector<int> order;
  order.reserve((size_t)np);
  for (int l = 0; l < c.nligands; ++l) {
    if (c.b_lig_all_host[(size_t)l]) continue;
    for (long long p = c.pose_off[l]; p < c.pose_off[l + 1]; ++p)
      if (!((edge[(size_t)(p >> 5)] >> (p & 31)) & 1u) && std::isfinite(hl[(size_t)p])) order.push_back((int)p);
  }
  const long long n_used = (long long)order.size();
  if (n_used == 0) return set_error(BUDE_ERR_ARG, "the batch has no regular pose with a finite label to train on");
  // b4 starts at the mean label per ligand atom.
  if (s.step == 0) {
    double sl = 0, sa = 0;
    for (int p : order) {
      sl += std::asinh(hl[(size_t)p] / kLossScale) * kLossScale;
      sa += lig_n[(size_t)p];
    }
    const float b4 = (float)(sl / std::max(sa, 1.0));
    e = copy_sync(c, s.params.as<float>() + kOffB4, &b4, sizeof b4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_error(e, "output bias");
  }
  const int nb_full = (int)std::min<long long>(batch, n_used);
  const int steps_per_epoch = (int)((n_used + nb_full - 1) / nb_full);
  const long long total_steps = (long long)epochs * steps_per_epoch;
  const size_t nrow_off = (size_t)(n_used + steps_per_epoch);
  std::mt19937_64 rng(seed);
  // Epochs are double-buffered: while the GPU runs epoch e from one pair of device arrays (pose
  // order, row offsets), the host shuffles epoch e + 1 into pinned memory and a copy stream moves
  // it into the other pair once the kernels of epoch e - 1 have finished with it.  The last
  // epoch's per-pose losses collect on the device and are read once.
  DevBuf *dpose[2] = {&s.epoch_pose, &s.epoch_pose2}, *drow[2] = {&s.epoch_rowoff, &s.epoch_rowoff2};
  for (int k = 0; k < 2 && !rc; ++k) {
    rc = dpose[k]->reserve((size_t)np * 4, "epoch poses");
    if (!rc) rc = drow[k]->reserve(nrow_off * 4, "epoch row offsets");
  }
  if (!rc) rc = s.epoch_loss.reserve((size_t)n_used * 4, "last-epoch losses");
  if (rc) return rc;
  int *hpose[2] = {}, *hrow[2] = {};
  cudaStream_t cs = nullptr;
  cudaEvent_t copied[2] = {}, used[2] = {}, e0 = nullptr, e1 = nullptr;
  bool setup_ok = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) == cudaSuccess;
  for (int k = 0; k < 2 && setup_ok; ++k)
    setup_ok = cudaMallocHost((void **)&hpose[k], (size_t)n_used * 4) == cudaSuccess &&
               cudaMallocHost((void **)&hrow[k], nrow_off * 4) == cudaSuccess &&
               cudaEventCreateWithFlags(&copied[k], cudaEventDisableTiming) == cudaSuccess &&
               cudaEventCreateWithFlags(&used[k], cudaEventDisableTiming) == cudaSuccess;
  setup_ok = setup_ok && cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess;
  std::vector<long long> rows_of[2] = {std::vector<long long>(steps_per_epoch),
                                       std::vector<long long>(steps_per_epoch)};
  // Shuffle epoch `ep` into host buffer k and queue its copy into device pair k.
  auto prepare = [&](int ep, int k) -> int {
    std::shuffle(order.begin(), order.end(), rng);
    // Row offsets of every batch of the epoch, one block of (batch + 1) entries per step.
    size_t w = 0;
    for (int st = 0; st < steps_per_epoch; ++st) {
      const long long a = (long long)st * nb_full, b = std::min(n_used, a + nb_full);
      int r = 0;
      for (long long i = a; i < b; ++i) {
        hrow[k][w++] = r;
        r += lig_n[(size_t)order[(size_t)i]];
      }
      hrow[k][w++] = r;
      rows_of[k][(size_t)st] = r;
    }
    std::memcpy(hpose[k], order.data(), (size_t)n_used * 4);
    cudaError_t ce = ep >= 2 ? cudaStreamWaitEvent(cs, used[k], 0) : cudaSuccess;
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(dpose[k]->ptr, hpose[k], (size_t)n_used * 4, cudaMemcpyHostToDevice, cs);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(drow[k]->ptr, hrow[k], w * 4, cudaMemcpyHostToDevice, cs);
    if (ce == cudaSuccess) ce = cudaEventRecord(copied[k], cs);
    return ce == cudaSuccess ? BUDE_OK : cuda_error(ce, "epoch order copy");
  };
  if (!setup_ok) rc = set_error(BUDE_ERR_CUDA, "training pipeline setup (stream, events, pinned buffers)");
  if (!rc) cudaEventRecord(e0, c.stream);
  if (!rc && epochs > 0) rc = prepare(0, 0);
  long long done = 0;
  for (int ep = 0; ep < epochs && !rc; ++ep) {
    const int k = ep & 1;
    cudaError_t ce = cudaStreamWaitEvent(c.stream, copied[k], 0);
    if (ce != cudaSuccess) rc = cuda_error(ce, "epoch order wait");
    long long ro = 0;
    for (int st = 0; st < steps_per_epoch && !rc; ++st) {
      const long long a = (long long)st * nb_full, b = std::min(n_used, a + nb_full);
      const int nb = (int)(b - a);
      // Cosine decay from lr to lr / 20 over the run.
      const double frac = total_steps > 1 ? (double)done / (double)(total_steps - 1) : 0.0;
      const float lr_now = (float)(lr * (0.05 + 0.95 * 0.5 * (1.0 + std::cos(M_PI * frac))));
      rc = train_step(c, s, dpose[k]->as<int>() + a, drow[k]->as<int>() + ro, nb, rows_of[k][(size_t)st], lr_now,
                      ep == epochs - 1 ? s.epoch_loss.as<float>() + a : nullptr);
      ro += nb + 1;
      ++done;
    }
    if (!rc) {
      ce = cudaEventRecord(used[k], c.stream);
      if (ce != cudaSuccess) rc = cuda_error(ce, "epoch event");
    }
    if (!rc && ep + 1 < epochs) {
      // Host buffer k ^ 1 last fed epoch ep - 1, whose copy finished before that epoch ran.
      ce = cudaEventSynchronize(copied[k ^ 1]);
      rc = ce == cudaSuccess ? prepare(ep + 1, k ^ 1) : cuda_error(ce, "epoch order copy");
    }
  }
  if (e1) cudaEventRecord(e1, c.stream);
  e = cudaStreamSynchronize(c.stream);
  if (!rc && e != cudaSuccess) rc = cuda_error(e, "surrogate training");
  double last_loss = 0;
  if (!rc && epochs > 0) {
    // The last epoch's losses in pose order, summed in that order.
    std::vector<float> lh((size_t)n_used);
    e = copy_sync(c, lh.data(), s.epoch_loss.ptr, (size_t)n_used * 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = cuda_error(e, "loss read-back");
    double loss_sum = 0;
    for (float v : lh) loss_sum += v;
    last_loss = loss_sum / (double)n_used;
  }
  if (cs) {
    cudaStreamSynchronize(cs);
    cudaStreamDestroy(cs);
  }
  for (int k = 0; k < 2; ++k) {
    if (hpose[k]) cudaFreeHost(hpose[k]);
    if (hrow[k]) cudaFreeHost(hrow[k]);
    if (copied[k]) cudaEventDestroy(copied[k]);
    if (used[k]) cudaEventDestroy(used[k]);
  }
  if (!rc && train_ms) cudaEventElapsedTime(train_ms, e0, e1);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (!rc && final_loss) *final_loss = (float)last_loss;
  return rc;
}

// One gradient of the loss over the given poses of the batch (no update); for tests.
int surrogate_gradient(Context &c, const int *poses, int n, const float *labels, float *grad_out, float *pred_out) {
  Surrogate &s = sur(c);
  if (!s.ready || !c.have_batch) return set_error(BUDE_ERR_STATE, "surrogate or batch missing");
  if (check_batch_types(c)) return BUDE_ERR_ARG;
  const long long np = c.batch_poses;
  std::vector<int> lig_n;
  int rc = upload_pose_ligands(c, s, lig_n);
  if (!rc) rc = batch_transforms(c);
  if (!rc) rc = s.labels.reserve((size_t)np * 4, "labels");
  if (!rc) rc = s.epoch_pose.reserve((size_t)n * 4, "poses");
  if (!rc) rc = s.epoch_rowoff.reserve((size_t)(n + 1) * 4, "row offsets");
  if (rc) return rc;
  cudaError_t e = copy_sync(c, s.labels.ptr, labels, (size_t)np * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_error(e, "labels");
  std::vector<int> ro(n + 1, 0);
  for (int i = 0; i < n; ++i) {
    if (poses[i] < 0 || poses[i] >= np) return set_error(BUDE_ERR_ARG, "pose index out of range");
    ro[i + 1] = ro[i] + lig_n[(size_t)poses[i]];
  }
  e = copy_sync(c, s.epoch_pose.ptr, poses, (size_t)n * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = copy_sync(c, s.epoch_rowoff.ptr, ro.data(), ro.size() * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_error(e, "gradient rows");
  rc = train_step(c, s, s.epoch_pose.as<int>(), s.epoch_rowoff.as<int>(), n, ro[n], 0.f, nullptr);
  e = cudaStreamSynchronize(c.stream);
  if (!rc && e != cudaSuccess) rc = cuda_error(e, "surrogate gradient");
  if (rc) return rc;
  if (grad_out) e = copy_sync(c, grad_out, s.grads.ptr, kNParams * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && pred_out) e = copy_sync(c, pred_out, s.pred.ptr, (size_t)n * 4, cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? BUDE_OK : cuda_error(e, "gradient read-back");
}

// Features (as floats) and atom types of the rows of the given poses; for inspection and tests.
int surrogate_features(Context &c, const int *poses, int n, float *X, int *types) {
  Surrogate &s = sur(c);
  if (!s.ready || !c.have_batch) return set_error(BUDE_ERR_STATE, "surrogate or batch missing");
  if (check_batch_types(c)) return BUDE_ERR_ARG;
  std::vector<int> lig_n;
  int rc = upload_pose_ligands(c, s, lig_n);
  if (!rc) rc = batch_transforms(c);
  if (rc) return rc;
  std::vector<int> ro(n + 1, 0);
  for (int i = 0; i < n; ++i) {
    if (poses[i] < 0 || poses[i] >= c.batch_poses) return set_error(BUDE_ERR_ARG, "pose index out of range");
    ro[i + 1] = ro[i] + lig_n[(size_t)poses[i]];
  }
  const long long rows = ro[n];
  rc = s.epoch_pose.reserve((size_t)n * 4, "poses");
  if (!rc) rc = s.epoch_rowoff.reserve((size_t)(n + 1) * 4, "row offsets");
  if (!rc) rc = ensure_train_scratch(s, std::max(rows, 1LL), n, 1);
  if (rc) return rc;
  cudaError_t e = copy_sync(c, s.epoch_pose.ptr, poses, (size_t)n * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = copy_sync(c, s.epoch_rowoff.ptr, ro.data(), ro.size() * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_error(e, "feature rows");
  RowMap m;
  m.pose = s.epoch_pose.as<int>();
  m.row_off = s.epoch_rowoff.as<int>();
  m.lig_first = s.pose_lig_first.as<int>();
  m.lig_n = s.pose_lig_n.as<int>();
  m.nposes = n;
  train_features_kernel<<<(n * 32 + 255) / 256, 256, 0, c.stream>>>(weights(s), s.fg, c.b_ligands.as<float4>(),
                                                                      c.b_xform.as<float4>(), m,
                                                                      s.X.as<__nv_bfloat16>(), s.row_type.as<int>(),
                                                                      nullptr);
  e = cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) return cuda_error(e, "surrogate features");
  std::vector<uint16_t> xb((size_t)tiled_rows(rows) * kFeat);
  e = copy_sync(c, xb.data(), s.X.ptr, xb.size() * 2, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_error(e, "feature read-back");
  for (long long r = 0; r < rows; ++r)
    for (int k = 0; k < kFeat; ++k) {
      const uint32_t u = (uint32_t)xb[(size_t)(tiled_offset(r, k, kFeat) / 2)] << 16;
      std::memcpy(&X[(size_t)r * kFeat + k], &u, 4);
    }
  if (types) e = copy_sync(c, types, s.row_type.ptr, (size_t)rows * 4, cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? BUDE_OK : cuda_error(e, "row type read-back");
}

// Scoring items (128 poses of one ligand each, ligand by ligand) and, unless the caller already
// computed them, the pose transforms of the uploaded batch.
int surrogate_prepare(Context &c, bool xform_ready) {
  Surrogate &s = sur(c);
  if (!s.ready) return set_error(BUDE_ERR_STATE, "surrogate not initialised");
  if (!c.have_batch) return set_error(BUDE_ERR_STATE, "no batch uploaded");
  if (check_batch_types(c)) return BUDE_ERR_ARG;
  const long long np = c.batch_poses;
  int rc = s.scores.reserve((size_t)std::max(np, 1LL) * 4, "surrogate scores");
  if (rc) return rc;
  if (s.items_for != c.batch_gen) {
    std::vector<int4> items;
    s.item_lig_off.assign(1, 0);
    for (int l = 0; l < c.nligands; ++l) {
      for (long long p = c.pose_off[l]; p < c.pose_off[l + 1]; p += kRowsPerCta)
        items.push_back(make_int4(c.lig_off[l], c.lig_off[l + 1] - c.lig_off[l], (int)p,
                                  (int)std::min<long long>(kRowsPerCta, c.pose_off[l + 1] - p)));
      s.item_lig_off.push_back((int)items.size());
    }
    rc = s.items.reserve(std::max<size_t>(items.size(), 1) * sizeof(int4), "surrogate items");
    if (rc) return rc;
    const cudaError_t e = copy_sync(c, s.items.ptr, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_error(e, "surrogate items");
    s.n_items = (int)items.size();
    s.items_for = c.batch_gen;
  }
  if (!xform_ready) {
    rc = batch_transforms(c);
    if (rc) return rc;
  }
  return set_smem_limits();
}

// Surrogate energies of the poses of ligands [lig0, lig1) into s.scores, on `st`.  The tcgen05
// scorer runs `groups` tile groups per block (4 alone; 3 leaves room for exact-kernel blocks).
int surrogate_score_range(Context &c, int lig0, int lig1, int groups, cudaStream_t st) {
  Surrogate &s = sur(c);
  const int i0 = s.item_lig_off[lig0], n_items = s.item_lig_off[lig1] - i0;
  if (n_items <= 0) return BUDE_OK;
  ScoreArgs a;
  a.W = weights(s);
  a.g = s.fg;
  a.ligands = c.b_ligands.as<float4>();
  a.xform = c.b_xform.as<float4>();
  a.items = s.items.as<int4>() + i0;
  a.scores = s.scores.as<float>();
  a.n_items = n_items;
  int per_sm = 0;
  cudaError_t e;
  if (s.scorer == BUDE_SCORER_TCGEN05) {
    if (!s.w4_host_valid) {
      // The weights changed since the last launch (they change on the context's stream).
      e = copy_sync(c, s.w4_host, a.W.w4, sizeof s.w4_host, cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) return cuda_error(e, "output weights");
      s.w4_host_valid = true;
    }
    ScoreTcArgs t;
    t.s = a;
    std::memcpy(t.w4, s.w4_host, sizeof t.w4);
    t.w = TcWeights{s.emb_h.ptr, s.w1_h.ptr, s.w2_h.ptr, s.w3_h.ptr, a.W.b1, a.W.b2, a.W.b3, a.W.w4, a.W.b4};
    t.err = c.err.as<unsigned int>();
    // One block per SM: a block holds all of its SM's TMEM it allocates.
    const int g = groups == 3 ? 3 : 4;
    const int grid = std::min((n_items + g - 1) / g, std::max(c.num_sms, 1));
    if (g == 3) score_tc_kernel<3><<<grid, 3 * kTcGroupThreads, sizeof(TcSmem<3>), st>>>(t);
    else score_tc_kernel<4><<<grid, 4 * kTcGroupThreads, sizeof(TcSmem<4>), st>>>(t);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(e, "score_tc_kernel launch");
  } else {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, score_kernel, kMlpThreads, sizeof(MlpSmem));
    const int grid = std::min(n_items, std::max(1, per_sm) * std::max(c.num_sms, 1));
    score_kernel<<<grid, kMlpThreads, sizeof(MlpSmem), st>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(e, "score_kernel launch");
  }
  c.launches++;
  return BUDE_OK;
}

// Surrogate energies of every pose of the uploaded batch into s.scores (device).
int surrogate_score_enqueue(Context &c, const float4 *xform_ready) {
  int rc = surrogate_prepare(c, xform_ready != nullptr);
  if (!rc) rc = surrogate_score_range(c, 0, c.nligands, kTcGroups, c.stream);
  return rc;
}

float *surrogate_scores(Context &c) { return c.surrogate ? c.surrogate->scores.as<float>() : nullptr; }

int surrogate_io(Context &c, float *out, const float *in, long long n) {
  Surrogate &s = sur(c);
  if (!s.ready) return set_error(BUDE_ERR_STATE, "surrogate not initialised");
  if (n != kNParams) return set_error(BUDE_ERR_ARG, "parameter vector has %lld values, not %lld", n, kNParams);
  cudaError_t e = cudaSuccess;
  if (out) e = copy_sync(c, out, s.params.ptr, kNParams * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && in) e = copy_sync(c, s.params.ptr, in, kNParams * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_error(e, "surrogate parameters");
  if (in) {
    int rc = publish(c, s);
    if (rc) return rc;
  }
  e = cudaStreamSynchronize(c.stream);
  return e == cudaSuccess ? BUDE_OK : cuda_error(e, "surrogate parameters");
}

// Checkpoint: magic, version, step, then masters, Adam m and Adam v (FP32).
int surrogate_save(Context &c, const char *path) {
  Surrogate &s = sur(c);
  if (!s.ready) return set_error(BUDE_ERR_STATE, "surrogate not initialised");
  std::vector<float> buf(3 * kNParams);
  cudaError_t e = copy_sync(c, buf.data(), s.params.ptr, kNParams * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = copy_sync(c, buf.data() + kNParams, s.adam_m.ptr, kNParams * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = copy_sync(c, buf.data() + 2 * kNParams, s.adam_v.ptr, kNParams * 4, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_error(e, "checkpoint read-back");
  FILE *f = std::fopen(path, "wb");
  if (!f) return set_error(BUDE_ERR_ARG, "cannot write %s", path);
  const unsigned long long hdr[3] = {0x4255444553555231ull /* "BUDESUR1" */, (unsigned long long)kNParams,
                                     (unsigned long long)s.step};
  bool ok = std::fwrite(hdr, sizeof hdr, 1, f) == 1 && std::fwrite(buf.data(), 4, buf.size(), f) == buf.size();
  ok = (std::fclose(f) == 0) && ok;
  return ok ? BUDE_OK : set_error(BUDE_ERR_ARG, "short write to %s", path);
}

int surrogate_load(Context &c, const char *path) {
  Surrogate &s = sur(c);
  if (!s.ready) return set_error(BUDE_ERR_STATE, "initialise the surrogate (grid) before loading weights");
  FILE *f = std::fopen(path, "rb");
  if (!f) return set_error(BUDE_ERR_ARG, "cannot read %s", path);
  unsigned long long hdr[3];
  std::vector<float> buf(3 * kNParams);
  bool ok = std::fread(hdr, sizeof hdr, 1, f) == 1 && hdr[0] == 0x4255444553555231ull &&
            hdr[1] == (unsigned long long)kNParams && std::fread(buf.data(), 4, buf.size(), f) == buf.size();
  std::fclose(f);
  if (!ok) return set_error(BUDE_ERR_ARG, "%s is not a surrogate checkpoint of this model", path);
  cudaError_t e = copy_sync(c, s.params.ptr, buf.data(), kNParams * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = copy_sync(c, s.adam_m.ptr, buf.data() + kNParams, kNParams * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = copy_sync(c, s.adam_v.ptr, buf.data() + 2 * kNParams, kNParams * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_error(e, "checkpoint upload");
  s.step = (long long)hdr[2];
  return publish(c, s);
}

} // namespace bude

using namespace bude;

extern "C" {

int bude_surrogate_init(bude_gpu_ctx *ctx, const bude_atom *protein, int32_t natpro, const bude_ffparams *forcefield,
                        int32_t ntypes, float extent, float spacing, uint64_t seed) {
  if (!ctx) return set_error(BUDE_ERR_ARG, "ctx is NULL");
  cudaSetDevice(ctx->device);
  return surrogate_init(*ctx, protein, natpro, forcefield, ntypes, extent, spacing, seed);
}

int bude_surrogate_train(bude_gpu_ctx *ctx, int32_t epochs, int32_t batch_poses, float lr, const float *labels,
                         uint64_t seed, float *final_loss, float *train_ms) {
  if (!ctx) return set_error(BUDE_ERR_ARG, "ctx is NULL");
  cudaSetDevice(ctx->device);
  return surrogate_train(*ctx, epochs, batch_poses, lr, labels, final_loss, train_ms, seed);
}

int bude_surrogate_score(bude_gpu_ctx *ctx, float *ms) {
  if (!ctx) return set_error(BUDE_ERR_ARG, "ctx is NULL");
  cudaSetDevice(ctx->device);
  cudaEventRecord(ctx->ev0, ctx->stream);
  int rc = surrogate_score_enqueue(*ctx, nullptr);
  if (rc) return rc;
  cudaEventRecord(ctx->ev1, ctx->stream);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_error(e, "surrogate scoring");
  if (ms) cudaEventElapsedTime(ms, ctx->ev0, ctx->ev1);
  return check_device_error(*ctx);
}

int bude_surrogate_set_scorer(bude_gpu_ctx *ctx, int32_t scorer) {
  if (!ctx) return set_error(BUDE_ERR_ARG, "ctx is NULL");
  if (scorer != BUDE_SCORER_TCGEN05 && scorer != BUDE_SCORER_MMA_SYNC)
    return set_error(BUDE_ERR_ARG, "unknown surrogate scorer %d", (int)scorer);
  sur(*ctx).scorer = scorer;
  return BUDE_OK;
}

int bude_surrogate_download(bude_gpu_ctx *ctx, float *scores, int64_t n) {
  if (!ctx || (!scores && n > 0)) return set_error(BUDE_ERR_ARG, "NULL argument");
  float *d = surrogate_scores(*ctx);
  if (!d || !ctx->have_batch || n != ctx->batch_poses)
    return set_error(BUDE_ERR_ARG, "no surrogate scores for %lld poses", (long long)n);
  cudaSetDevice(ctx->device);
  cudaError_t e = copy_sync(*ctx, scores, d, (size_t)n * 4, cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? BUDE_OK : cuda_error(e, "score download");
}

int bude_surrogate_gradient(bude_gpu_ctx *ctx, const int32_t *poses, int32_t n, const float *labels, float *grads,
                            float *pred) {
  if (!ctx || !poses || !labels || n <= 0) return set_error(BUDE_ERR_ARG, "bad argument");
  cudaSetDevice(ctx->device);
  return surrogate_gradient(*ctx, poses, n, labels, grads, pred);
}

int bude_surrogate_features(bude_gpu_ctx *ctx, const int32_t *poses, int32_t n, float *features, int32_t *types) {
  if (!ctx || !poses || !features || n <= 0) return set_error(BUDE_ERR_ARG, "bad argument");
  cudaSetDevice(ctx->device);
  return surrogate_features(*ctx, poses, n, features, types);
}

int bude_surrogate_params(bude_gpu_ctx *ctx, float *out, const float *in, int64_t n) {
  if (!ctx) return set_error(BUDE_ERR_ARG, "ctx is NULL");
  cudaSetDevice(ctx->device);
  return surrogate_io(*ctx, out, in, n);
}

int bude_surrogate_save(bude_gpu_ctx *ctx, const char *path) {
  if (!ctx || !path) return set_error(BUDE_ERR_ARG, "NULL argument");
  cudaSetDevice(ctx->device);
  return surrogate_save(*ctx, path);
}

int bude_surrogate_load(bude_gpu_ctx *ctx, const char *path) {
  if (!ctx || !path) return set_error(BUDE_ERR_ARG, "NULL argument");
  cudaSetDevice(ctx->device);
  return surrogate_load(*ctx, path);
}

} // extern "C"
