// internal.h -- shared host-side declarations of libbude_gb300.so (not part of the C-ABI).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <vector>

#include "../../include/minibude_gb300.h"

namespace bude {


struct Surrogate;
struct ScreenState;
struct StreamState;

// CUDA events owned by one host call: created together, destroyed when the call returns by any
// path.  ok() is false when a creation failed.
struct EventSet {
  std::vector<cudaEvent_t> ev;
  explicit EventSet(size_t n, unsigned flags = cudaEventDefault) : ev(n, nullptr) {
    for (auto &e : ev)
      if (cudaEventCreateWithFlags(&e, flags) != cudaSuccess) e = nullptr;
  }
  ~EventSet() {
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
  }
  EventSet(const EventSet &) = delete;
  EventSet &operator=(const EventSet &) = delete;
  cudaEvent_t operator[](size_t i) const { return ev[i]; }
  bool ok() const {
    for (cudaEvent_t e : ev)
      if (!e) return false;
    return true;
  }
};

// A growable device allocation.
struct DevBuf {
  void *ptr = nullptr;
  size_t cap = 0;
  int reserve(size_t nbytes, const char *what);
  void release();
  template <class T> T *as() const { return static_cast<T *>(ptr); }
};

// State behind a bude_gpu_ctx handle.
struct Context {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // deck
  bool have_deck = false;
  int natpro = 0, natpro_pad = 0, natlig = 0, ntypes = 0;
  long long nposes = 0, pose_stride = 0;
  DevBuf ligand, slab, poses, xform, energies, err, flush, partial;
  // Irregular poses and decks (edge_pose.cuh): the raw protein and forcefield records, the
  // transform pass's irregular-pose bits of the deck's poses, and whether the deck is irregular.
  DevBuf raw_protein, raw_ff, edge_mask;
  std::vector<bude_ffparams> host_ff; // the forcefield the slab was built from
  bool protein_regular = true;      // every protein atom and its forcefield record within bounds
  float protein_min_radius = 0.f;   // smallest radius of the protein's atom types
  bool deck_irregular = false;      // the uploaded deck (protein + ligand) is scored by edge_pose_kernel
  int flush_gen = 0;
  long long launches = 0;
  // batch of ligands (bude_gpu_upload_batch); shares the protein slab with the deck fields above
  bool have_batch = false;
  int nligands = 0;
  std::vector<int> lig_off;        // nligands + 1 atom offsets
  std::vector<long long> pose_off; // nligands + 1 pose offsets
  long long batch_poses = 0;
  DevBuf b_ligands, b_poses, b_xform, b_energies, b_items, b_counter;
  DevBuf b_partial; // split x batch_poses slice sums of a split batch evaluation (graph-owned)
  // Irregular poses of the batch: transform-pass bits, device pose/atom offsets, and the ligands
  // whose every pose goes to edge_pose_kernel (lig_all flags and their count, both on the device).
  DevBuf b_edge_mask, b_pose_off, b_lig_off, b_lig_all, b_lig_any;
  int b_irregular_ligands = 0;
  std::vector<unsigned char> b_lig_all_host; // host copy of the lig_all flags
  int items_ppb = 0;  // poses per item the device item list was built for
  int items_ppwi = 0; // and poses per thread (the cut of a ligand's last block depends on it)
  int n_items = 0;
  cudaGraphExec_t graph = nullptr;
  bude_launch_cfg graph_cfg{};
  long long batch_gen = 0; // bumped whenever the batch's shape (ligand sizes, pose counts) changes
  long long batch_uploads = 0; // bumped by every successful batch upload
  long long batch_tuned_key = -1;
  bude_launch_cfg batch_tuned{};
  float batch_tuned_ms = 0.f;
  Surrogate *surrogate = nullptr; // learned pre-screen (surrogate.cu)
  ScreenState *screen = nullptr;  // last screening run (screen.cu)
  StreamState *streamer = nullptr; // chunked evaluation of host-resident poses (stream.cu)
  // autotuner cache: the deck shape it was tuned for and the pick
  long long tuned_key[3] = {-1, -1, -1};
  bude_launch_cfg tuned{};
  float tuned_ms = 0.f;
  // the protein and forcefield the slab on the device was built from (ensure_slab)
  std::vector<unsigned char> slab_key;
};

// Copies and fills ordered on the context's stream and finished on return.  The context's stream
// is non-blocking, so plain cudaMemcpy / cudaMemset (the legacy default stream) would be ordered
// neither after the kernels already on it nor before the ones launched next.
cudaError_t copy_sync(const Context &c, void *dst, const void *src, size_t bytes, cudaMemcpyKind kind);
cudaError_t copy2d_sync(const Context &c, void *dst, size_t dpitch, const void *src, size_t spitch, size_t width,
                        size_t height, cudaMemcpyKind kind);
cudaError_t fill_sync(const Context &c, void *dst, int value, size_t bytes);

int set_error(int code, const char *fmt, ...);
int cuda_error(cudaError_t e, const char *what);
const char *last_error();

void build_slab(const bude_atom *protein, int natpro, const bude_ffparams *ff, int ntypes, int natpro_pad,
                std::vector<float> &slab);
// Build and upload the protein slab for (protein, forcefield) unless the device already holds the
// slab of exactly these records; sets natpro, natpro_pad and ntypes.  *rebuilt (optional) tells
// whether it was rebuilt.
int ensure_slab(Context &c, const bude_atom *protein, int natpro, const bude_ffparams *ff, int ntypes,
                bool *rebuilt = nullptr);

int make_context(int device, Context **out);
void destroy_context(Context *c);
int upload_deck(Context &c, const bude_atom *protein, int natpro, const bude_atom *ligand, int natlig,
                const bude_ffparams *ff, int ntypes, const float *poses, long long stride, long long nposes);
int set_poses(Context &c, const bude_atom *ligand, int natlig, const float *poses, long long stride,
              long long nposes);
int check_cfg(const Context &c, const bude_launch_cfg &cfg);
int exact_blocks_per_sm(const bude_launch_cfg &cfg, int *out);
int choose_split(const Context &c, bude_launch_cfg &cfg);
int choose_split_for(int num_sms, int natpro_pad, long long nposes, bude_launch_cfg &cfg);
void release_batch(Context &c);
int enqueue_batch(Context &c, const bude_launch_cfg &cfg, int per_ligand);
// Cut a ligand's n poses into batch-kernel items of at most ppb = ppwi * wgsize poses: full blocks,
// then the remainder r.  The batch kernel runs an item of at most ppb/2 or ppb/4 poses with half or
// a quarter of the poses per thread (a quarter from 8 poses per thread up), so with ppwi 8 or 16 a
// remainder ppb/2 < r <= 3ppb/4 is cut into ppb/2 + the rest: 3/4 of a full item's work.  (With 14
// poses per thread, a shape sized for one item per ligand, halves would run 7 poses in 4 pairs.)
// f(first pose offset within the ligand, pose count) is called per item, in pose order.
template <class F> inline void for_each_item(long long n, int ppwi, int ppb, F &&f) {
  long long p = 0;
  for (; n - p >= ppb; p += ppb) f(p, ppb);
  const int r = (int)(n - p);
  if ((ppwi == 8 || ppwi == 16) && 2 * r > ppb && 4 * r <= 3 * ppb) {
    f(p, ppb / 2);
    f(p + ppb / 2, r - ppb / 2);
  } else if (r > 0) {
    f(p, r);
  }
}

// Batch kernel over `items` (energies of the items' poses from the transforms at `xform`).  With
// cfg.split > 1 the slice sums go through `partial` (at least cfg.split * npose_space floats) and a
// per-item slice reduction.  On stream `st` (nullptr: the context's stream); max_blocks_per_sm > 0
// caps the persistent grid, leaving room on each SM for kernels running beside it.  slice_tile > 0
// cuts the protein slices as a launch with that tile would (cfg.tile, the records per shared-memory
// stage, must divide it): the slices alone fix a pose's arithmetic.
int batch_items_enqueue(Context &c, const bude_launch_cfg &cfg, const int4 *items, int n_items, const float4 *xform,
                        float *energies, float *partial, long long npose_space, cudaStream_t st = nullptr,
                        int max_blocks_per_sm = 0, int slice_tile = 0);
void release_surrogate(Context &c);
void release_streamer(Context &c);
void release_screen(Context &c);
int surrogate_score_enqueue(Context &c, const float4 *xform_ready);
int surrogate_prepare(Context &c, bool xform_ready);
int surrogate_score_range(Context &c, int lig0, int lig1, int groups, cudaStream_t st);
float *surrogate_scores(Context &c);
int autotune(Context &c, int max_ms, bude_launch_cfg &best, float *best_ms);
int default_cfg(const Context &c, int ppwi, int wgsize, bude_launch_cfg &cfg);
int enqueue_eval(Context &c, const bude_launch_cfg &cfg, cudaEvent_t mid = nullptr);
int launch_exact_range(Context &c, const bude_launch_cfg &cfg, const float4 *ligand, int natlig, const float *xform,
                       float *energies, long long nposes);
// Whether a ligand of natlig atoms keeps the uploaded protein's deck regular (edge_pose.cuh).
bool ligand_regular(const Context &c, const bude_atom *ligand, int natlig, const bude_ffparams *ff);
// Enqueue edge_pose_kernel for the deck's single ligand over n poses (mask and transforms of
// those poses; energies overwritten where irregular, or everywhere when `all`).
int enqueue_edge_single(Context &c, const float4 *ligand, int natlig, bool all, const unsigned *mask,
                        const float *xform, float *energies, long long n, cudaStream_t st);
// Enqueue edge_pose_kernel over the uploaded batch's poses (flag: optional per-pose marks).
int enqueue_edge_batch(Context &c, const float *xform, float *energies, unsigned char *flag, cudaStream_t st);
int check_device_error(Context &c);
int flush_l2(Context &c);
int probe_kernel_arch(int device, int *cc);

} // namespace bude

// The opaque handle of the C-ABI is the context itself.
struct bude_gpu_ctx : public bude::Context {};
