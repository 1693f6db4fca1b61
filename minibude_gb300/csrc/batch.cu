// batch.cu -- host side of batched ragged scoring: many ligands with uneven atom and pose counts
// against one protein, in one persistent CUDA-graph-captured launch (batch_kernel.cuh), or, for
// comparison, one plain exact-kernel launch per ligand.
//
// The reference scores one ligand per run of its driver (src/main.cpp); a virtual screen runs it
// once per ligand.  Here the batch shares the protein slab and the pose-transform pass, and the
// persistent kernel load-balances pose blocks of all ligands over the resident block slots.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "batch_kernel.cuh"
#include "internal.h"

namespace bude {

void release_batch(Context &c) {
  if (c.graph) cudaGraphExecDestroy(c.graph);
  c.graph = nullptr;
  c.b_ligands.release();
  c.b_poses.release();
  c.b_xform.release();
  c.b_energies.release();
  c.b_items.release();
  c.b_counter.release();
  c.b_partial.release();
  c.b_edge_mask.release();
  c.b_pose_off.release();
  c.b_lig_off.release();
  c.b_lig_all.release();
  c.b_lig_any.release();
  c.b_irregular_ligands = 0;
  c.b_lig_all_host.clear();
  c.have_batch = false;
  c.items_ppb = 0;
  c.items_ppwi = 0;
  c.n_items = 0;
}

static void drop_graph(Context &c) {
  if (c.graph) cudaGraphExecDestroy(c.graph);
  c.graph = nullptr;
}

int upload_batch(Context &c, const bude_atom *protein, int natpro, const bude_ffparams *ff, int ntypes, int nligands,
                 const bude_atom *atoms, const int32_t *lig_off, const float *poses, long long pose_stride,
                 const int64_t *pose_off) {
  // A batch of the same shape as the uploaded one (same ligand sizes and pose counts, same protein
  // and forcefield) keeps its work items, captured graph and tuned launch shape: only the atoms and
  // poses are copied.
  const bool same_shape = c.have_batch && nligands == c.nligands && lig_off && pose_off &&
                          std::equal(lig_off, lig_off + nligands + 1, c.lig_off.begin()) &&
                          std::equal(pose_off, pose_off + nligands + 1, c.pose_off.begin());
  c.have_batch = false;
  c.have_deck = false;
  if (nligands < 0 || !lig_off || !pose_off || ntypes <= 0 || !ff || natpro < 0 || (natpro > 0 && !protein))
    return set_error(BUDE_ERR_ARG, "bad batch sizes or pointers");
  if (lig_off[0] != 0 || pose_off[0] != 0) return set_error(BUDE_ERR_ARG, "batch offsets must start at 0");
  for (int l = 0; l < nligands; ++l)
    if (lig_off[l + 1] < lig_off[l] || pose_off[l + 1] < pose_off[l])
      return set_error(BUDE_ERR_ARG, "batch offsets must not decrease (ligand %d)", l);
  const int total_atoms = lig_off[nligands];
  const long long total_poses = pose_off[nligands];
  if ((total_atoms > 0 && !atoms) || (total_poses > 0 && (!poses || pose_stride < total_poses)))
    return set_error(BUDE_ERR_ARG, "bad batch atoms or poses");
  // Work items (batch, screen and surrogate) carry pose indices as 32-bit integers.
  if (total_poses > 0x7fffffffLL)
    return set_error(BUDE_ERR_ARG, "a batch holds at most 2^31 - 1 poses (got %lld)", total_poses);
  for (int i = 0; i < natpro; ++i)
    if (protein[i].type < 0 || protein[i].type >= ntypes)
      return set_error(BUDE_ERR_TYPE, "protein atom %d has type %d outside the forcefield (%d types)", i,
                       protein[i].type, ntypes);
  for (int i = 0; i < total_atoms; ++i)
    if (atoms[i].type < 0 || atoms[i].type >= ntypes)
      return set_error(BUDE_ERR_TYPE, "ligand atom %d of the batch has type %d outside the forcefield (%d types)", i,
                       atoms[i].type, ntypes);
  // Protein slab (shared with the single-deck path; rebuilt only for another protein/forcefield).
  bool rebuilt = false;
  int rc = ensure_slab(c, protein, natpro, ff, ntypes, &rebuilt);
  if (rc) return rc;
  const bool keep = same_shape && !rebuilt;
  if (!keep) drop_graph(c);
  const long long np = std::max(total_poses, 1LL);
  rc = c.b_ligands.reserve((size_t)std::max(total_atoms, 1) * 16, "batch ligands");
  if (!rc) rc = c.b_poses.reserve((size_t)6 * np * sizeof(float), "batch poses");
  if (!rc) rc = c.b_xform.reserve((size_t)12 * np * sizeof(float), "batch transforms");
  if (!rc) rc = c.b_energies.reserve((size_t)np * sizeof(float), "batch energies");
  if (!rc) rc = c.b_counter.reserve(256, "batch work counter");
  if (!rc) rc = c.b_edge_mask.reserve((size_t)(np + 31) / 32 * sizeof(unsigned), "batch irregular-pose bits");
  if (!rc) rc = c.b_pose_off.reserve((size_t)(nligands + 1) * sizeof(long long), "batch pose offsets");
  if (!rc) rc = c.b_lig_off.reserve((size_t)(nligands + 1) * sizeof(int), "batch atom offsets");
  if (!rc) rc = c.b_lig_all.reserve((size_t)std::max(nligands, 1), "batch irregular ligands");
  if (!rc) rc = c.b_lig_any.reserve(sizeof(int), "batch irregular ligand count");
  if (rc) return rc;
  // Ligands outside the regular-deck bounds (edge_pose.cuh): all their poses go to edge_pose_kernel.
  std::vector<unsigned char> lig_all((size_t)std::max(nligands, 1), 0);
  int n_irregular = 0;
  for (int l = 0; l < nligands; ++l) {
    lig_all[(size_t)l] = !ligand_regular(c, atoms + lig_off[l], lig_off[l + 1] - lig_off[l], ff);
    n_irregular += lig_all[(size_t)l];
  }
  cudaError_t e = cudaSuccess;
  if (total_atoms > 0) e = copy_sync(c, c.b_ligands.ptr, atoms, (size_t)total_atoms * 16, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && total_poses > 0)
    e = copy2d_sync(c, c.b_poses.ptr, (size_t)total_poses * sizeof(float), poses, (size_t)pose_stride * sizeof(float),
                    (size_t)total_poses * sizeof(float), 6, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = copy_sync(c, c.b_pose_off.ptr, pose_off, (size_t)(nligands + 1) * sizeof(long long), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = copy_sync(c, c.b_lig_off.ptr, lig_off, (size_t)(nligands + 1) * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && nligands > 0)
    e = copy_sync(c, c.b_lig_all.ptr, lig_all.data(), (size_t)nligands, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = copy_sync(c, c.b_lig_any.ptr, &n_irregular, sizeof(int), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_error(e, "batch upload");
  c.b_irregular_ligands = n_irregular;
  c.b_lig_all_host.assign(lig_all.begin(), lig_all.begin() + nligands);
  c.have_batch = true;
  ++c.batch_uploads;
  if (keep) return BUDE_OK;
  ++c.batch_gen;
  c.nligands = nligands;
  c.lig_off.assign(lig_off, lig_off + nligands + 1);
  c.pose_off.assign(pose_off, pose_off + nligands + 1);
  c.batch_poses = total_poses;
  c.items_ppb = 0;
  c.items_ppwi = 0;
  c.batch_tuned_key = -1;
  return BUDE_OK;
}

// Items of at most P*W poses (for_each_item), longest (most ligand atoms) first; uploaded when the
// launch shape changes.
static int build_items(Context &c, int ppwi, int wgsize, std::vector<int4> *keep = nullptr) {
  const int ppb = ppwi * wgsize;
  if (c.items_ppb == ppb && c.items_ppwi == ppwi && !keep) return BUDE_OK;
  std::vector<int> order(c.nligands);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return c.lig_off[x + 1] - c.lig_off[x] > c.lig_off[y + 1] - c.lig_off[y];
  });
  std::vector<int4> items;
  for (int l : order) {
    const int natlig = c.lig_off[l + 1] - c.lig_off[l];
    for_each_item(c.pose_off[l + 1] - c.pose_off[l], ppwi, ppb, [&](long long p, int n) {
      items.push_back(make_int4(c.lig_off[l], natlig, (int)(c.pose_off[l] + p), n));
    });
  }
  if (c.batch_poses > 0x7fffffffLL) return set_error(BUDE_ERR_ARG, "batch too large for 32-bit pose indices");
  if (keep) {
    *keep = std::move(items);
    return BUDE_OK;
  }
  int rc = c.b_items.reserve(std::max<size_t>(items.size(), 1) * sizeof(int4), "batch items");
  if (rc) return rc;
  if (!items.empty()) {
    cudaError_t e = copy_sync(c, c.b_items.ptr, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_error(e, "batch item upload");
  }
  c.n_items = (int)items.size();
  c.items_ppb = ppb;
  c.items_ppwi = ppwi;
  return BUDE_OK;
}

template <int P, int U> static cudaError_t batch_launch_pu(const BatchArgs &a, int grid, int w, size_t smem,
                                                         cudaStream_t st) {
  batch_kernel<P, U><<<grid, w, smem, st>>>(a);
  return cudaGetLastError();
}

template <int P, int U> static int batch_prepare_pu(int w, size_t smem, int *per_sm) {
  cudaError_t e = cudaFuncSetAttribute(batch_kernel<P, U>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, batch_kernel<P, U>, w, smem);
  return e == cudaSuccess ? BUDE_OK : cuda_error(e, "batch kernel set-up");
}

#define BUDE_BATCH_DISPATCH(CFG, CALL)                                                                                 \
  switch ((CFG).ppwi * 10 + (CFG).unroll) {                                                                            \
  case 11: CALL(1, 1); break;                                                                                          \
  case 12: CALL(1, 2); break;                                                                                          \
  case 14: CALL(1, 4); break;                                                                                          \
  case 21: CALL(2, 1); break;                                                                                          \
  case 22: CALL(2, 2); break;                                                                                          \
  case 24: CALL(2, 4); break;                                                                                          \
  case 41: CALL(4, 1); break;                                                                                          \
  case 42: CALL(4, 2); break;                                                                                          \
  case 44: CALL(4, 4); break;                                                                                          \
  case 81: CALL(8, 1); break;                                                                                          \
  case 82: CALL(8, 2); break;                                                                                          \
  case 84: CALL(8, 4); break;                                                                                          \
  case 142: CALL(14, 2); break;                                                                                        \
  case 161: CALL(16, 1); break;                                                                                        \
  case 162: CALL(16, 2); break;                                                                                        \
  default: CALL(16, 4); break;                                                                                         \
  }

static size_t batch_smem(const bude_launch_cfg &cfg) { return exact_smem_bytes(cfg.ppwi, cfg.wgsize, cfg.tile, 1, 0); }

// Resident blocks per SM of batch_kernel for the shape (also sets its shared-memory limit).
static int batch_blocks_per_sm(const bude_launch_cfg &cfg, int *per_sm) {
  const size_t smem = batch_smem(cfg);
  int rc = BUDE_OK;
#define BUDE_PREP(P, U) rc = batch_prepare_pu<P, U>(cfg.wgsize, smem, per_sm)
  BUDE_BATCH_DISPATCH(cfg, BUDE_PREP)
#undef BUDE_PREP
  return rc;
}

// Records per protein slice of a split evaluation: ceil(natpro_pad / split) in whole tiles.
static int batch_slice(const Context &c, int split, int tile) {
  const int per = (c.natpro_pad + split - 1) / split;
  return (per + tile - 1) / tile * tile;
}

// The context's slice-sum buffer for a split evaluation of the whole batch.  Growing it moves the
// buffer, so a captured graph that points at it is dropped first.
static int reserve_batch_partial(Context &c, const bude_launch_cfg &cfg) {
  if (cfg.split <= 1) return BUDE_OK;
  const size_t bytes = (size_t)cfg.split * (size_t)std::max(c.batch_poses, 1LL) * sizeof(float);
  if (bytes > c.b_partial.cap) drop_graph(c);
  return c.b_partial.reserve(bytes, "batch slice sums");
}

// Enqueue the batch kernel over `items` (counter reset first): energies of the items' poses from
// the transforms at `xform` into `energies` (through `partial` and a slice reduction when split).
static int enqueue_items(Context &c, const bude_launch_cfg &cfg, int grid, const int4 *items, int n_items,
                         const float4 *xform, float *energies, float *partial, long long npose_space,
                         cudaStream_t st = nullptr, int slice_tile = 0) {
  if (!st) st = c.stream;
  if (slice_tile <= 0) slice_tile = cfg.tile;
  if (slice_tile % cfg.tile) return set_error(BUDE_ERR_ARG, "the stage tile must divide the slice tile");
  if (cfg.split > 1 && !partial) return set_error(BUDE_ERR_STATE, "split batch evaluation without a slice buffer");
  cudaError_t e = cudaMemsetAsync(c.b_counter.ptr, 0, sizeof(unsigned), st);
  if (e != cudaSuccess) return cuda_error(e, "batch counter reset");
  BatchArgs a;
  a.ligands = c.b_ligands.as<float4>();
  a.slab = c.slab.as<float4>();
  a.xform = reinterpret_cast<const float *>(xform);
  a.energies = energies;
  a.items = items;
  a.counter = c.b_counter.as<unsigned>();
  a.err = c.err.as<unsigned>();
  a.n_items = n_items;
  a.natpro_pad = c.natpro_pad;
  a.tile = cfg.tile;
  a.split = std::max(cfg.split, 1);
  a.slice = a.split > 1 ? batch_slice(c, a.split, slice_tile) : c.natpro_pad;
  a.partial = partial;
  a.npose_space = npose_space;
  const size_t smem = batch_smem(cfg);
#define BUDE_LAUNCH(P, U) e = batch_launch_pu<P, U>(a, grid, cfg.wgsize, smem, st)
  BUDE_BATCH_DISPATCH(cfg, BUDE_LAUNCH)
#undef BUDE_LAUNCH
  if (e != cudaSuccess) return cuda_error(e, "batch_kernel launch");
  c.launches++;
  if (a.split > 1 && n_items > 0) {
    batch_reduce_kernel<<<(unsigned)n_items, 256, 0, st>>>(items, partial, a.split, npose_space, energies);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(e, "batch_reduce_kernel launch");
    c.launches++;
  }
  return BUDE_OK;
}

// Enqueue one persistent evaluation of the whole batch (transforms, then the batch kernel) for
// items already on the device.
static int enqueue_persistent(Context &c, const bude_launch_cfg &cfg, int grid, const int4 *items, int n_items) {
  if (c.batch_poses > 0) {
    const int tb = 256;
    pose_xform_kernel<<<(unsigned)((c.batch_poses + tb - 1) / tb), tb, 0, c.stream>>>(
        c.b_poses.as<float>(), c.batch_poses, c.batch_poses, c.b_xform.as<float4>(), c.b_edge_mask.as<unsigned>());
    c.launches++;
  }
  int rc = enqueue_items(c, cfg, grid, items, n_items, c.b_xform.as<float4>(), c.b_energies.as<float>(),
                         c.b_partial.as<float>(), c.batch_poses);
  if (rc) return rc;
  return enqueue_edge_batch(c, c.b_xform.as<float>(), c.b_energies.as<float>(), nullptr, c.stream);
}

static int persistent_grid(Context &c, const bude_launch_cfg &cfg, int *grid) {
  int per_sm = 0;
  int rc = batch_blocks_per_sm(cfg, &per_sm);
  if (rc) return rc;
  if (per_sm <= 0) return set_error(BUDE_ERR_ARG, "batch launch shape cannot be resident on an SM");
  *grid = per_sm * std::max(c.num_sms, 1);
  return BUDE_OK;
}

// The persistent evaluation as a CUDA graph, captured once per launch shape.
static int ensure_graph(Context &c, const bude_launch_cfg &cfg) {
  int rc = reserve_batch_partial(c, cfg); // may drop the graph
  if (rc) return rc;
  const bool same = c.graph && c.graph_cfg.ppwi == cfg.ppwi && c.graph_cfg.wgsize == cfg.wgsize &&
                    c.graph_cfg.tile == cfg.tile && c.graph_cfg.unroll == cfg.unroll &&
                    c.graph_cfg.split == cfg.split;
  if (same) return BUDE_OK;
  drop_graph(c);
  rc = build_items(c, cfg.ppwi, cfg.wgsize);
  int grid = 0;
  if (!rc) rc = persistent_grid(c, cfg, &grid); // also sets the kernel's shared-memory limit
  if (rc) return rc;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_error(e, "graph capture begin");
  const long long launches0 = c.launches;
  rc = enqueue_persistent(c, cfg, grid, c.b_items.as<int4>(), c.n_items);
  c.launches = launches0; // captured, not launched
  e = cudaStreamEndCapture(c.stream, &g);
  if (!rc && e != cudaSuccess) rc = cuda_error(e, "graph capture end");
  if (!rc) {
    e = cudaGraphInstantiate(&c.graph, g, 0);
    if (e != cudaSuccess) rc = cuda_error(e, "graph instantiate");
  }
  if (g) cudaGraphDestroy(g);
  if (rc) {
    c.graph = nullptr;
    return rc;
  }
  c.graph_cfg = cfg;
  return BUDE_OK;
}

int batch_items_enqueue(Context &c, const bude_launch_cfg &cfg, const int4 *items, int n_items, const float4 *xform,
                        float *energies, float *partial, long long npose_space, cudaStream_t st,
                        int max_blocks_per_sm, int slice_tile) {
  int grid = 0;
  int rc = persistent_grid(c, cfg, &grid);
  if (rc) return rc;
  if (max_blocks_per_sm > 0) grid = std::min(grid, max_blocks_per_sm * std::max(c.num_sms, 1));
  return enqueue_items(c, cfg, grid, items, n_items, xform, energies, partial, npose_space, st, slice_tile);
}

int enqueue_batch(Context &c, const bude_launch_cfg &cfg, int per_ligand) {
  if (!c.have_batch) return set_error(BUDE_ERR_STATE, "no batch uploaded");
  bude_launch_cfg shape = cfg;
  shape.cluster = 0;
  int rc = check_cfg(c, shape);
  if (rc) return rc;
  if (!per_ligand) {
    rc = ensure_graph(c, shape);
    if (rc) return rc;
    cudaError_t e = cudaGraphLaunch(c.graph, c.stream);
    if (e != cudaSuccess) return cuda_error(e, "graph launch");
    c.launches += (c.batch_poses > 0 ? 3 : 1) + (shape.split > 1 && c.n_items > 0 ? 1 : 0);
    return BUDE_OK;
  }
  // One plain exact-kernel launch per ligand, each with its own wave-model split (cluster
  // reduction, so no slice buffer), after one transform pass over all poses.
  if (c.batch_poses > 0) {
    const int tb = 256;
    pose_xform_kernel<<<(unsigned)((c.batch_poses + tb - 1) / tb), tb, 0, c.stream>>>(
        c.b_poses.as<float>(), c.batch_poses, c.batch_poses, c.b_xform.as<float4>(), c.b_edge_mask.as<unsigned>());
    c.launches++;
  }
  for (int l = 0; l < c.nligands; ++l) {
    const long long n = c.pose_off[l + 1] - c.pose_off[l];
    if (n == 0) continue;
    bude_launch_cfg lc = cfg;
    lc.cluster = 1;
    rc = choose_split_for(c.num_sms, c.natpro_pad, n, lc);
    if (rc) return rc;
    rc = launch_exact_range(c, lc, c.b_ligands.as<float4>() + c.lig_off[l], c.lig_off[l + 1] - c.lig_off[l],
                            c.b_xform.as<float>() + c.pose_off[l] * 12, c.b_energies.as<float>() + c.pose_off[l], n);
    if (rc) return rc;
  }
  return enqueue_edge_batch(c, c.b_xform.as<float>(), c.b_energies.as<float>(), nullptr, c.stream);
}

int autotune_batch(Context &c, int max_ms, bude_launch_cfg &best, float *best_ms) {
  if (!c.have_batch) return set_error(BUDE_ERR_STATE, "no batch uploaded");
  if (c.batch_tuned_key == c.batch_poses) {
    best = c.batch_tuned;
    if (best_ms) *best_ms = c.batch_tuned_ms;
    return BUDE_OK;
  }
  struct Shape { int p, w, u; };
  // Short items run with P/2 or P/4 poses per thread, so P = 16 no longer loses a ligand's last
  // pose block to padding and leads the list.
  const Shape shapes[] = {{16, 128, 1}, {16, 256, 1}, {16, 64, 1}, {8, 128, 2}, {8, 64, 2}, {8, 256, 2}};
  // Time each shape on every k-th item of its own item list so one timing covers about 2e10
  // interactions (the mix of ligand sizes is kept) while still giving every resident block slot
  // at least 8 items (a subset smaller than the grid would time latency, not throughput).
  double work = 0;
  for (int l = 0; l < c.nligands; ++l)
    work += double(c.lig_off[l + 1] - c.lig_off[l]) * double(c.pose_off[l + 1] - c.pose_off[l]) * c.natpro_pad;
  const int stride_work = std::max(1, (int)std::ceil(work / 2e10));
  DevBuf sub;
  float best_t = 1e30f;
  float spent = 0.f;
  int rc = BUDE_OK;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // Shapes at split 1 first; then the best of them with its protein cut into 2, 4 and 8 slices,
  // which pays off when the batch is too small to keep every block slot busy to the end.
  std::vector<bude_launch_cfg> cands;
  for (const Shape &sh : shapes) cands.push_back(bude_launch_cfg{sh.p, sh.w, 1, 64, sh.u, 0});
  const size_t n_shapes = cands.size();
  for (size_t ci = 0; ci < cands.size(); ++ci) {
    if (ci == n_shapes && best_t < 1e30f)
      for (int sp : {2, 4, 8}) {
        bude_launch_cfg v = best;
        v.split = sp;
        cands.push_back(v);
      }
    const bude_launch_cfg cfg = cands[ci];
    if (check_cfg(c, cfg)) continue;
    rc = reserve_batch_partial(c, cfg);
    if (rc) break;
    std::vector<int4> items;
    rc = build_items(c, cfg.ppwi, cfg.wgsize, &items);
    if (rc) break;
    int grid = 0;
    rc = persistent_grid(c, cfg, &grid);
    if (rc) break;
    const int stride = std::max(1, std::min(stride_work, (int)(items.size() / (8 * (size_t)std::max(grid, 1)))));
    std::vector<int4> picked;
    for (size_t i = 0; i < items.size(); i += stride) picked.push_back(items[i]);
    if (picked.empty()) continue;
    rc = sub.reserve(picked.size() * sizeof(int4), "autotune items");
    if (rc) break;
    const cudaError_t ec = copy_sync(c, sub.ptr, picked.data(), picked.size() * sizeof(int4), cudaMemcpyHostToDevice);
    if (ec != cudaSuccess) {
      rc = cuda_error(ec, "autotune item upload");
      break;
    }
    rc = enqueue_persistent(c, cfg, grid, sub.as<int4>(), (int)picked.size()); // warm-up
    cudaEventRecord(e0, c.stream);
    if (!rc) rc = enqueue_persistent(c, cfg, grid, sub.as<int4>(), (int)picked.size());
    cudaEventRecord(e1, c.stream);
    cudaError_t e = cudaStreamSynchronize(c.stream);
    if (!rc && e != cudaSuccess) rc = cuda_error(e, "batch autotune");
    if (rc) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const float full = ms * stride;
    spent += 2.f * ms;
    if (full < best_t) {
      best_t = full;
      best = cfg;
    }
    if (spent > (float)std::max(max_ms, 1)) break;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  sub.release();
  if (!rc) rc = check_device_error(c);
  if (rc) return rc;
  if (best_t >= 1e30f) return set_error(BUDE_ERR_ARG, "no batch launch shape fits this device");
  c.batch_tuned = best;
  c.batch_tuned_ms = best_t;
  c.batch_tuned_key = c.batch_poses;
  if (best_ms) *best_ms = best_t;
  return BUDE_OK;
}

} // namespace bude

using namespace bude;

extern "C" {

int bude_gpu_upload_batch(bude_gpu_ctx *ctx, const bude_atom *protein, int32_t natpro,
                          const bude_ffparams *forcefield, int32_t ntypes, int32_t nligands,
                          const bude_atom *ligand_atoms, const int32_t *ligand_offsets, const float *poses,
                          int64_t pose_stride, const int64_t *pose_offsets) {
  if (!ctx) return set_error(BUDE_ERR_ARG, "ctx is NULL");
  cudaSetDevice(ctx->device);
  return upload_batch(*ctx, protein, natpro, forcefield, ntypes, nligands, ligand_atoms, ligand_offsets, poses,
                      pose_stride, pose_offsets);
}

int bude_gpu_autotune_batch(bude_gpu_ctx *ctx, int32_t max_ms, bude_launch_cfg *best, float *best_ms) {
  if (!ctx || !best) return set_error(BUDE_ERR_ARG, "NULL argument");
  cudaSetDevice(ctx->device);
  return autotune_batch(*ctx, max_ms, *best, best_ms);
}

int bude_gpu_run_batch(bude_gpu_ctx *ctx, const bude_launch_cfg *cfg, int32_t per_ligand, float *ms) {
  if (!ctx || !cfg) return set_error(BUDE_ERR_ARG, "NULL argument");
  cudaSetDevice(ctx->device);
  if (ctx->have_batch && !per_ligand) {
    // Capture (or re-capture) before timing so the first timed launch is the graph itself.
    bude_launch_cfg shape = *cfg;
    shape.cluster = 0;
    int rc = check_cfg(*ctx, shape);
    if (!rc) rc = ensure_graph(*ctx, shape);
    if (rc) return rc;
  }
  cudaEventRecord(ctx->ev0, ctx->stream);
  int rc = enqueue_batch(*ctx, *cfg, per_ligand);
  if (rc) return rc;
  cudaEventRecord(ctx->ev1, ctx->stream);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_error(e, "batch evaluation");
  if (ms) cudaEventElapsedTime(ms, ctx->ev0, ctx->ev1);
  return check_device_error(*ctx);
}

int bude_gpu_download_batch(bude_gpu_ctx *ctx, float *energies, int64_t total_poses) {
  if (!ctx || (!energies && total_poses > 0)) return set_error(BUDE_ERR_ARG, "NULL argument");
  if (!ctx->have_batch || total_poses != ctx->batch_poses)
    return set_error(BUDE_ERR_ARG, "download of %lld energies but the batch has %lld poses", (long long)total_poses,
                     ctx->have_batch ? ctx->batch_poses : 0LL);
  if (total_poses == 0) return BUDE_OK;
  cudaSetDevice(ctx->device);
  cudaError_t e = cudaMemcpyAsync(energies, ctx->b_energies.ptr, (size_t)total_poses * sizeof(float),
                                  cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  return e == cudaSuccess ? BUDE_OK : cuda_error(e, "batch energy download");
}

} // extern "C"
