/*
 * minibude_gb300.h -- C-ABI of the GB300 (sm_103a) miniBUDE energy-evaluation library
 * (libbude_gb300.so).
 *
 * Plain C types, integer status codes and caller-owned buffers only.  Every entry point is the
 * replacement for one piece of the reference's CUDA model, src/cuda/fasten.hpp (the `CudaBude`
 * class behind the `Bude<PPWI>` interface of src/bude.h:95-101); each declaration below names the
 * reference lines it replaces.  The C++ `Bude<PPWI>` model in minibude_gb300/model/gb300/fasten.hpp
 * and the Python host (minibude_gb300/__init__.py) are thin wrappers over these symbols.
 *
 * Threading: a context is used from one host thread at a time (the reference calls `fasten`
 * sequentially from one thread, src/main.cpp:517-541).  Error text is per host thread.
 */
#ifndef MINIBUDE_GB300_H
#define MINIBUDE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Record layouts of the deck files; byte-identical to the reference's packed structs
 * `Atom` (src/bude.h:39-42) and `FFParams` (src/bude.h:44-49). */
typedef struct bude_atom {
  float x, y, z;
  int32_t type; /* index into the forcefield table */
} bude_atom;

typedef struct bude_ffparams {
  int32_t hbtype; /* ASCII code of the bhff electrostatic type: '-' 45, 'D' 68, 'E' 69, 'F' 70 */
  float radius, hphb, elsc;
} bude_ffparams;

/* Status codes.  The C++ model turns any non-zero code into std::runtime_error with the text of
 * bude_gpu_last_error(), as the reference's checkError does (src/cuda/fasten.hpp:168-172). */
#define BUDE_OK 0
#define BUDE_ERR_ARG (-1)     /* bad size, pointer or launch shape */
#define BUDE_ERR_CUDA (-2)    /* a CUDA runtime call failed */
#define BUDE_ERR_STATE (-3)   /* call out of order (e.g. run before upload) */
#define BUDE_ERR_TIMEOUT (-4) /* a bounded device-side wait ran out; the kernel returned early */
#define BUDE_ERR_TYPE (-5)    /* an atom type index lies outside the forcefield table */

/* Kernel launch shape of the exact kernel.  The reference exposes two knobs, PPWI (poses per work
 * item, a template parameter, src/main.cpp:48-53) and wgsize (threads per block,
 * src/cuda/fasten.hpp:272-275); this kernel adds the protein split and the shared-memory tile. */
typedef struct bude_launch_cfg {
  int32_t ppwi;    /* poses per thread, held in registers: 1, 2, 4, 8 or 16 */
  int32_t wgsize;  /* threads per block: a multiple of 32 in [32, 512] */
  int32_t split;   /* protein slices per pose block: 1..8 with cluster = 1, 1..64 with cluster = 0 */
  int32_t tile;    /* protein atoms per shared-memory stage (TMA bulk copy): multiple of 8, 8..512 */
  int32_t unroll;  /* protein atoms per unrolled inner-loop body: 1, 2 or 4 */
  int32_t cluster; /* split > 1: 1 = slices summed inside a thread-block cluster (distributed shared
                      memory), 0 = through a context-owned [split][nposes] buffer and a second kernel */
} bude_launch_cfg;

typedef struct bude_gpu_ctx bude_gpu_ctx;

/* Text of the last error raised on this host thread ("" if none). */
const char *bude_gpu_last_error(void);

/* Library version string, e.g. "minibude-gb300 0.1 (sm_103a)". */
const char *bude_gpu_version(void);

/* Device enumeration; replaces CudaBude::enumerateDevices (src/cuda/fasten.hpp:181-196).
 * The name has the reference's form "<name> (<MB>MB;sm_<cc>)". */
int bude_gpu_device_count(int *count);
int bude_gpu_device_name(int device, char *buf, size_t buflen);
/* Streaming multiprocessors of the device (sizes launch grids and the FP32 peak). */
int bude_gpu_sm_count(int device, int *sms);

/* Architecture check; replaces CudaBude::compatible and its `version` probe kernel
 * (src/cuda/fasten.hpp:12-18, 218-248).  Writes the compute capability the kernels were built
 * for and the device's own (both as 10*major+minor) and sets *ok to 1 when they match. */
int bude_gpu_compatible(int device, int *kernel_cc, int *device_cc, int *ok);

/* Context: device selection and the library's stream (src/cuda/fasten.hpp:252). */
int bude_gpu_create(int device, bude_gpu_ctx **out);
/* Frees every device buffer of the context (src/cuda/fasten.hpp:291-301). */
int bude_gpu_destroy(bude_gpu_ctx *ctx);

/* Upload a deck: protein, ligand, forcefield and poses; replaces the "context" allocation and
 * copies of src/cuda/fasten.hpp:256-270.  `poses` holds six float fields (tilt, roll, pan in
 * radians; x, y, z translation) at poses + k*pose_stride, the layout of poses.in
 * (src/main.cpp:296-311).  Atom types are checked against ntypes (BUDE_ERR_TYPE).  Buffers grow
 * as needed and are reused by later uploads. */
int bude_gpu_upload(bude_gpu_ctx *ctx, const bude_atom *protein, int32_t natpro, const bude_atom *ligand,
                    int32_t natlig, const bude_ffparams *forcefield, int32_t ntypes, const float *poses,
                    int64_t pose_stride, int64_t nposes);

/* Replace only the poses (and, when ligand != NULL, the ligand) of an uploaded deck. */
int bude_gpu_set_poses(bude_gpu_ctx *ctx, const bude_atom *ligand, int32_t natlig, const float *poses,
                       int64_t pose_stride, int64_t nposes);

/* Map the reference's (PPWI, wgsize) pair onto this kernel's launch shape, choosing split and tile
 * for the uploaded deck.  PPWI above 16 uses 16 poses per thread; wgsize 0 or below 32 is rounded
 * up to a multiple of 32.  Results do not depend on the shape beyond FP32 summation order. */
int bude_gpu_default_cfg(const bude_gpu_ctx *ctx, int32_t ppwi, int32_t wgsize, bude_launch_cfg *cfg);

/* Choose a launch shape for the uploaded deck by measurement; replaces the reference driver's
 * brute-force PPWI x wgsize sweep (src/main.cpp:517-541).  Candidate shapes get their protein
 * split from a wave model (resident blocks per SM from the occupancy API) and are timed with CUDA
 * events on a ligand prefix, within about max_ms of GPU time.  The pick is cached per deck shape
 * in the context.  best_ms (optional) receives the predicted time of one full evaluation. */
int bude_gpu_autotune(bude_gpu_ctx *ctx, int32_t max_ms, bude_launch_cfg *best, float *best_ms);

/* One evaluation of all uploaded poses (one iteration of the reference's hot loop,
 * src/cuda/fasten.hpp:277-286): pose transforms and the exact kernel on the context's stream,
 * then a stream synchronise.  *kernel_ms (optional) receives the CUDA-event time of the two
 * kernels.  Energies stay on the device. */
int bude_gpu_run(bude_gpu_ctx *ctx, const bude_launch_cfg *cfg, float *kernel_ms);

/* `iterations` back-to-back evaluations, each timed with CUDA events on the context's stream;
 * with flush_l2 != 0 a buffer larger than L2 is rewritten before each timed evaluation (outside
 * the timed span).  ms_per_iter (optional) receives the time of each evaluation (both kernels),
 * exact_ms_per_iter (optional) that of the exact kernel alone. */
int bude_gpu_run_many(bude_gpu_ctx *ctx, const bude_launch_cfg *cfg, int32_t iterations, int32_t flush_l2,
                      float *ms_per_iter, float *exact_ms_per_iter);

/* Copy the energies of the last evaluation to the host (src/cuda/fasten.hpp:288-289).
 * BUDE_ERR_STATE when no deck is uploaded (a failed upload or a batch upload leaves none). */
int bude_gpu_download(bude_gpu_ctx *ctx, float *energies, int64_t nposes);

/* End-to-end evaluation from host buffers: copies `poses` (and the ligand, when not NULL) to the
 * device, evaluates, and copies the energies back, all on the context's stream. */
int bude_gpu_score_host(bude_gpu_ctx *ctx, const bude_launch_cfg *cfg, const bude_atom *ligand, int32_t natlig,
                        const float *poses, int64_t pose_stride, int64_t nposes, float *energies);

/* Evaluate poses that stay in host memory, `chunk` poses at a time, against the uploaded deck's
 * protein and ligand: chunk i+1's poses are copied in and chunk i-1's energies copied out while
 * chunk i is evaluated (two copy streams beside the context's stream).  Replaces the whole-deck
 * H2D copy of src/cuda/fasten.hpp:256-270 for decks too large to stage at once or produced on the
 * host.  poses: six fields at poses + k*pose_stride (poses.in layout); energies: nposes floats.
 * Pinned host buffers (bude_host_alloc) let the copies overlap.  The energies equal those of
 * bude_gpu_run with the same cfg over all poses, bit for bit, for any chunk.  The chunk is rounded
 * up to whole waves of the launch shape's resident blocks (so each chunk's launch fills the GPU).
 * *ms (optional): CUDA-event time of the whole call.  No counterpart in the reference. */
int bude_gpu_score_stream(bude_gpu_ctx *ctx, const bude_launch_cfg *cfg, const float *poses, int64_t pose_stride,
                          int64_t nposes, int64_t chunk, float *energies, float *ms);

/* The whole of CudaBude<PPWI>::fasten (src/cuda/fasten.hpp:250-305) in one call: create a context
 * on `device`, upload, run `iterations` times, download, destroy.  kernel_ms (optional) receives
 * `iterations` per-iteration times, context_ms (optional) the upload time. */
int bude_gpu_fasten(int device, int32_t ppwi, int32_t wgsize, const bude_atom *protein, int32_t natpro,
                    const bude_atom *ligand, int32_t natlig, const bude_ffparams *forcefield, int32_t ntypes,
                    const float *poses, int64_t pose_stride, int64_t nposes, int32_t iterations, float *energies,
                    float *kernel_ms, float *context_ms);

/* Batched ragged scoring: many ligands, each with its own atoms and poses, against one protein.
 * No counterpart in the reference's CUDA model, which scores one ligand per run; it replaces a
 * loop of CudaBude::fasten calls (src/cuda/fasten.hpp:250-305), one per ligand.  Ligand l owns
 * atoms [ligand_offsets[l], ligand_offsets[l+1]) of ligand_atoms and poses
 * [pose_offsets[l], pose_offsets[l+1]) of the [6][pose_stride] pose block; both offset arrays
 * have nligands+1 entries starting at 0.  A batch replaces any deck uploaded to the context (and
 * vice versa); energies come out in the concatenated pose order.  A batch holds at most
 * 2^31 - 1 poses (work items index poses with 32-bit integers): BUDE_ERR_ARG beyond that. */
int bude_gpu_upload_batch(bude_gpu_ctx *ctx, const bude_atom *protein, int32_t natpro,
                          const bude_ffparams *forcefield, int32_t ntypes, int32_t nligands,
                          const bude_atom *ligand_atoms, const int32_t *ligand_offsets, const float *poses,
                          int64_t pose_stride, const int64_t *pose_offsets);

/* Launch shape for the batch (ppwi, wgsize, tile, unroll, split; cluster is not used): each
 * candidate is timed on a strided subset of the batch's work items, the best pose shape also with
 * its protein cut into 2, 4 and 8 slices.  Cached per batch. */
int bude_gpu_autotune_batch(bude_gpu_ctx *ctx, int32_t max_ms, bude_launch_cfg *best, float *best_ms);

/* One evaluation of the whole batch, then a stream synchronise.  per_ligand = 0: one persistent
 * kernel over all (ligand, pose block) items, longest first, taken from an atomic work counter,
 * launched as a CUDA graph (counter reset + pose transforms + persistent kernel) captured on first
 * use of a launch shape.  With cfg->split > 1 (cluster ignored) every item is scored once per
 * protein slice and a reduction kernel sums the slices in order; the energies then differ from
 * split = 1 by FP32 summation order only.  per_ligand = 1: one plain exact-kernel launch per
 * ligand, for comparison.  *ms (optional) receives the CUDA-event time. */
int bude_gpu_run_batch(bude_gpu_ctx *ctx, const bude_launch_cfg *cfg, int32_t per_ligand, float *ms);

/* Energies of the last batch evaluation, in concatenated pose order. */
int bude_gpu_download_batch(bude_gpu_ctx *ctx, float *energies, int64_t total_poses);

/* ---- Learned pre-screen (no counterpart in the reference) --------------------------------
 * A per-protein MLP estimates pose energies: per (pose, ligand atom) features -- a 16-wide
 * learned type embedding, the transformed atom position and 13 protein-field channels sampled
 * from a grid precomputed for the protein -- go through 32 -> 128 -> 128 -> 128 -> 1 with
 * hard-swish activations (h = z * sat(z/6 + 1/2), the piecewise-polynomial form of SiLU); the
 * outputs are summed per pose.  Training runs BF16 tensor-core GEMMs (tcgen05) with FP32
 * accumulation, FP32 master weights and Adam state; the default scorer runs FP16 tensor-core GEMMs
 * with FP32 accumulation. */
#define BUDE_SURROGATE_NPARAMS 38404

/* Create (or reset) the context's surrogate for a protein: builds the field grid over
 * [-extent, extent]^3 with `spacing` (at most 400 points a side) and seeds the weights.  At most
 * 64 forcefield types.  A 1.0 A spacing keeps the accuracy of finer grids on the reference's
 * proteins and samples faster than they do (the grid stays in the texture cache). */
int bude_surrogate_init(bude_gpu_ctx *ctx, const bude_atom *protein, int32_t natpro, const bude_ffparams *forcefield,
                        int32_t ntypes, float extent, float spacing, uint64_t seed);

/* Train on every pose of the uploaded batch (bude_gpu_upload_batch) for `epochs` epochs of
 * shuffled batches of `batch_poses` poses with Adam (learning rate `lr`, cosine decay to lr/20).
 * labels (NULL: exact energies computed here with the batched exact kernel) are per pose in batch
 * order.  The loss is the mean squared error on the compressed scale 20*asinh(E/20).  final_loss
 * (optional): mean loss of the last epoch; train_ms (optional): elapsed time of the epochs on the
 * context's stream (CUDA events from before the first epoch's shuffle to after the last step). */
int bude_surrogate_train(bude_gpu_ctx *ctx, int32_t epochs, int32_t batch_poses, float lr, const float *labels,
                         uint64_t seed, float *final_loss, float *train_ms);

/* Surrogate energies of every pose of the uploaded batch (kept on the device; see
 * bude_surrogate_download).  *ms (optional): CUDA-event time including the pose transforms. */
int bude_surrogate_score(bude_gpu_ctx *ctx, float *ms);
int bude_surrogate_download(bude_gpu_ctx *ctx, float *scores, int64_t n);

/* Which kernel scores poses (bude_surrogate_score and the screening pipeline):
 * BUDE_SCORER_TCGEN05 (default) runs the three hidden layers as tcgen05 UMMAs with TMEM
 * accumulators, in FP16; BUDE_SCORER_MMA_SYNC runs them as warp-level mma.sync in BF16, the
 * roundings of the training pass.  Both evaluate the same network and accumulate in FP32; their
 * scores differ by the 16-bit roundings of the activations (a few tenths of a per cent). */
#define BUDE_SCORER_TCGEN05 0
#define BUDE_SCORER_MMA_SYNC 1
int bude_surrogate_set_scorer(bude_gpu_ctx *ctx, int32_t scorer);

/* Loss gradient (no update) over the given batch poses with the given per-pose labels:
 * grads[BUDE_SURROGATE_NPARAMS] in the parameter layout, pred[n] the predicted energies. */
int bude_surrogate_gradient(bude_gpu_ctx *ctx, const int32_t *poses, int32_t n, const float *labels, float *grads,
                            float *pred);

/* Features of the (pose, ligand atom) rows of the given batch poses, rows laid out pose by pose:
 * features[rows][32] as the BF16 values the MLP sees (widened to float), types[rows] (optional)
 * the atoms' forcefield types. */
int bude_surrogate_features(bude_gpu_ctx *ctx, const int32_t *poses, int32_t n, float *features, int32_t *types);

/* Read (out != NULL) and/or replace (in != NULL) the FP32 parameters, n = BUDE_SURROGATE_NPARAMS.
 * Layout: embedding [64][16], W1 [128][32], b1, W2 [128][128], b2, W3 [128][128], b3, w4 [128],
 * b4 (+3 unused). */
int bude_surrogate_params(bude_gpu_ctx *ctx, float *out, const float *in, int64_t n);

/* Checkpoint of the weights and the Adam state (flat binary file). */
int bude_surrogate_save(bude_gpu_ctx *ctx, const char *path);
int bude_surrogate_load(bude_gpu_ctx *ctx, const char *path);

/* ---- Surrogate-screened scoring of the uploaded batch (no counterpart in the reference) ---- */
typedef struct bude_screen_cfg {
  float top_frac;     /* fraction of each ligand's poses rescored by the exact kernel (best surrogate) */
  float audit_frac;   /* fraction of each ligand's poses rescored at random (audit sample) */
  float audit_tol;    /* audit error above which a ligand is rescored exhaustively */
  uint32_t seed;      /* audit sample */
  bude_launch_cfg exact; /* exact kernel of the exhaustive fallback (cluster unused); its split and
                          * tile also cut the protein for the rescoring, so every exact energy the
                          * screen reports equals bude_gpu_run_batch's with this shape, bit for bit */
  int32_t chunks;     /* ligand chunks (0 or 1: none): with more, the exact rescoring of chunk j
                       * runs beside the surrogate of chunk j+1 (slower on the 1,024-ligand
                       * screen: the rescoring blocks slow the surrogate more than they hide) */
  bude_launch_cfg rescore; /* shape of the exact rescoring: ppwi, wgsize, unroll and tile, the
                            * records per shared-memory stage (0: exact's; it must divide exact's
                            * tile); split and cluster are ignored: the protein slices are exact's.
                            * ppwi 0 picks the shape from the number of poses rescored per ligand */
} bude_screen_cfg;

/* total_ms: the whole call; surrogate_ms: pose transforms and surrogate scoring (until the last
 * chunk's scorer has finished); rescore_ms: selection, compaction and exact rescoring after that;
 * fallback_ms: the audit and the exhaustive fallback. */
typedef struct bude_screen_stats {
  float total_ms, surrogate_ms, rescore_ms, fallback_ms;
  int64_t rescored_poses;  /* picks + audit */
  int32_t fallback_ligands;
  int64_t fallback_poses;
  float max_audit_error;
} bude_screen_stats;

/* Surrogate scores every pose; per ligand the exact kernel rescores the ceil(top_frac * n)
 * best-scored poses and an audit sample of ceil(audit_frac * n) of the others (uniform, seeded);
 * a ligand whose audit error -- 1 - Spearman rank correlation of surrogate and
 * exact energies over its audit poses (at most 2048) -- exceeds audit_tol is rescored exhaustively.
 * Needs a trained (or loaded) surrogate and an uploaded batch. */
int bude_screen_run(bude_gpu_ctx *ctx, const bude_screen_cfg *cfg, bude_screen_stats *stats);

/* Final energies (exact where rescored, surrogate elsewhere), rescored flags (per pose) and the
 * per-ligand audit errors of the last screen; any output may be NULL.  BUDE_ERR_STATE when the
 * last screen failed or a batch was uploaded after it (its result belongs to the earlier batch). */
int bude_screen_download(bude_gpu_ctx *ctx, float *final_energies, uint8_t *rescored, float *audit_error,
                         int64_t total_poses);

/* Number of kernels this library launched on the context since it was created (the transform
 * and exact kernels count one each). */
int bude_gpu_launch_count(const bude_gpu_ctx *ctx, int64_t *count);

/* Self-test of the failure path (no counterpart in the reference): runs one kernel that waits on
 * an mbarrier nothing arrives on, bounded to limit_us microseconds (1..1e6), exactly as every
 * device wait of the library is bounded.  Returns BUDE_ERR_TIMEOUT with the error text of a real
 * timeout, clears the error word, and leaves the context usable.  elapsed_ms (optional) receives
 * the kernel's time. */
int bude_gpu_selftest_wait(bude_gpu_ctx *ctx, int32_t limit_us, float *elapsed_ms);

/* One exact evaluation that allocates no device memory.  This entry point has no counterpart in
 * the reference.  It is for callers that may not allocate GPU memory themselves: code running
 * inside another framework whose allocator owns the device heap, plugin hosts that hand a plugin
 * its buffers, and loops where cudaMalloc/cudaFree and their device synchronisation are not
 * allowed.  Every pointer is a buffer in the current device's own memory (or managed memory):
 * protein, ligand (16-byte aligned) and forcefield records, poses as six float fields at
 * poses + k*pose_stride, and the output energies[nposes]; host memory and other GPUs' memory give
 * BUDE_ERR_ARG.  `stream` is a cudaStream_t (NULL: the default stream); the call reads a status
 * word back and returns after `stream` has drained, with the energies written.  The working
 * memory (per-deck protein slab, pose transforms, irregular-pose bits, status words) is one fixed
 * device array inside the library of about 11 MiB, held by every GPU that loads it until the
 * process exits: sizes above BUDE_NOALLOC_MAX_POSES poses or BUDE_NOALLOC_MAX_SLAB_RECORDS slab
 * records (forcefield types x protein atoms rounded up to 8) are rejected with BUDE_ERR_ARG.
 * Calls share that array: calls whose work overlaps on one GPU race and must be serialised by the
 * caller.  Every call is synchronous: it reads its status word back and waits for `stream`, so it
 * cannot be recorded into a CUDA graph (inside a stream capture it fails and invalidates the
 * capture).  The first call on a device looks up the array's device address (cudaGetSymbolAddress)
 * and keeps it for the process: do not use the entry point on a device after cudaDeviceReset.
 * Atom types outside the forcefield give BUDE_ERR_TYPE and leave energies unwritten. */
#define BUDE_NOALLOC_MAX_POSES 65536
#define BUDE_NOALLOC_MAX_SLAB_RECORDS 131072
int bude_gpu_fasten_noalloc(const bude_atom *protein, int32_t natpro, const bude_atom *ligand, int32_t natlig,
                            const bude_ffparams *forcefield, int32_t ntypes, const float *poses, int64_t pose_stride,
                            int64_t nposes, float *energies, void *stream);

/* Page-locked host buffers for callers that time host<->device copies. */
int bude_host_alloc(size_t bytes, void **ptr);
int bude_host_free(void *ptr);

#ifdef __cplusplus
}
#endif

#endif /* MINIBUDE_GB300_H */
