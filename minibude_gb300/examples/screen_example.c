/* screen_example.c -- the screening pipeline from C, through the C-ABI alone.
 *
 * Builds a seeded synthetic problem (a protein of random atoms, ligands of uneven size, random
 * poses), then: uploads the batch, scores it exhaustively with the persistent batch kernel, trains
 * the surrogate on a second batch, screens the first batch (surrogate over every pose, exact
 * rescoring of the top 2% + 0.5% audit) and checks that every rescored energy equals the
 * exhaustive one (same launch shape) and that each ligand's best exact pose was found.
 *
 *   cc -std=c11 -I include minibude_gb300/examples/screen_example.c -L minibude_gb300 -lbude_gb300 \
 *      -Wl,-rpath,minibude_gb300 -lm -o screen_example && ./screen_example
 *
 * Exit status 0 when every check holds. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "minibude_gb300.h"

#define CHECK(call)                                                                                \
  do {                                                                                             \
    int rc_ = (call);                                                                              \
    if (rc_ != BUDE_OK) {                                                                          \
      fprintf(stderr, "%s failed (%d): %s\n", #call, rc_, bude_gpu_last_error());                   \
      return 1;                                                                                    \
    }                                                                                              \
  } while (0)

static uint64_t rng_state = 0x9E3779B97F4A7C15ull;
static double uniform(double lo, double hi) { /* xorshift64* */
  rng_state ^= rng_state >> 12;
  rng_state ^= rng_state << 25;
  rng_state ^= rng_state >> 27;
  const uint64_t r = rng_state * 0x2545F4914F6CDD1Dull;
  return lo + (hi - lo) * (double)(r >> 11) * (1.0 / 9007199254740992.0);
}

typedef struct {
  int32_t nligands;
  int32_t *lig_off;   /* nligands + 1 */
  int64_t *pose_off;  /* nligands + 1 */
  bude_atom *atoms;
  float *poses;       /* [6][total] */
} batch_t;

static void make_batch(batch_t *b, int nligands, int ntypes, int poses_per_ligand) {
  b->nligands = nligands;
  b->lig_off = calloc((size_t)nligands + 1, sizeof(int32_t));
  b->pose_off = calloc((size_t)nligands + 1, sizeof(int64_t));
  for (int l = 0; l < nligands; ++l) {
    b->lig_off[l + 1] = b->lig_off[l] + 12 + (int32_t)uniform(0, 40);
    b->pose_off[l + 1] = b->pose_off[l] + poses_per_ligand;
  }
  const int32_t natoms = b->lig_off[nligands];
  const int64_t n = b->pose_off[nligands];
  b->atoms = calloc((size_t)natoms, sizeof(bude_atom));
  for (int i = 0; i < natoms; ++i) {
    b->atoms[i].x = (float)uniform(-4, 4);
    b->atoms[i].y = (float)uniform(-4, 4);
    b->atoms[i].z = (float)uniform(-4, 4);
    b->atoms[i].type = (int32_t)uniform(0, ntypes);
  }
  b->poses = calloc((size_t)n * 6, sizeof(float));
  for (int64_t i = 0; i < n; ++i) {
    for (int k = 0; k < 3; ++k) b->poses[k * n + i] = (float)uniform(0, 6.283185307179586);
    for (int k = 3; k < 6; ++k) b->poses[k * n + i] = (float)uniform(-3, 3);
  }
}

static void free_batch(batch_t *b) {
  free(b->lig_off);
  free(b->pose_off);
  free(b->atoms);
  free(b->poses);
}

int main(void) {
  enum { NATPRO = 900, NTYPES = 24, NLIG = 12, NPOSES = 4096 };
  bude_atom protein[NATPRO];
  bude_ffparams ff[NTYPES];
  for (int i = 0; i < NATPRO; ++i) {
    protein[i].x = (float)uniform(-18, 18);
    protein[i].y = (float)uniform(-18, 18);
    protein[i].z = (float)uniform(-18, 18);
    protein[i].type = (int32_t)uniform(0, NTYPES);
  }
  const int32_t hbtypes[3] = {45, 69, 70}; /* '-', 'E', 'F' */
  for (int t = 0; t < NTYPES; ++t) {
    ff[t].hbtype = hbtypes[(int)uniform(0, 3)];
    ff[t].radius = (float)uniform(1.0, 2.5);
    ff[t].hphb = (float)uniform(-3, 3);
    ff[t].elsc = (float)uniform(-1, 1);
  }
  batch_t screen, train;
  make_batch(&screen, NLIG, NTYPES, NPOSES);
  make_batch(&train, 4 * NLIG, NTYPES, 2048);
  const int64_t n = screen.pose_off[NLIG];

  bude_gpu_ctx *ctx = NULL;
  CHECK(bude_gpu_create(0, &ctx));
  /* exhaustive exact scoring of the screen batch, with the shape the screen's fallback uses */
  const bude_launch_cfg exact = {8, 128, 4, 64, 2, 0};
  CHECK(bude_gpu_upload_batch(ctx, protein, NATPRO, ff, NTYPES, NLIG, screen.atoms, screen.lig_off, screen.poses,
                              n, screen.pose_off));
  float ms = 0.f;
  CHECK(bude_gpu_run_batch(ctx, &exact, 0, &ms));
  float *full = malloc((size_t)n * sizeof(float));
  CHECK(bude_gpu_download_batch(ctx, full, n));
  /* the surrogate, trained on the other batch (labels from the exact kernel) */
  CHECK(bude_surrogate_init(ctx, protein, NATPRO, ff, NTYPES, 11.0f, 1.25f, 1));
  CHECK(bude_gpu_upload_batch(ctx, protein, NATPRO, ff, NTYPES, train.nligands, train.atoms, train.lig_off,
                              train.poses, train.pose_off[train.nligands], train.pose_off));
  float loss = 0.f, train_ms = 0.f;
  CHECK(bude_surrogate_train(ctx, 60, 4096, 3e-3f, NULL, 2, &loss, &train_ms));
  /* the screen */
  CHECK(bude_gpu_upload_batch(ctx, protein, NATPRO, ff, NTYPES, NLIG, screen.atoms, screen.lig_off, screen.poses,
                              n, screen.pose_off));
  bude_screen_cfg sc;
  memset(&sc, 0, sizeof sc);
  sc.top_frac = 0.02f;
  sc.audit_frac = 0.005f;
  sc.audit_tol = 0.05f;
  sc.seed = 7;
  sc.exact = exact;
  bude_screen_stats st;
  CHECK(bude_screen_run(ctx, &sc, &st));
  float *final = malloc((size_t)n * sizeof(float));
  uint8_t *rescored = malloc((size_t)n);
  CHECK(bude_screen_download(ctx, final, rescored, NULL, n));

  int bad = 0, best_found = 0;
  int64_t nres = 0;
  for (int l = 0; l < NLIG; ++l) {
    int64_t best = screen.pose_off[l];
    for (int64_t p = screen.pose_off[l]; p < screen.pose_off[l + 1]; ++p) {
      if (full[p] < full[best]) best = p;
      if (rescored[p]) {
        ++nres;
        if (final[p] != full[p]) ++bad; /* the rescoring's energies are the exhaustive ones, bit for bit */
      }
    }
    best_found += rescored[best] != 0;
  }
  printf("training loss %.2f (%.0f ms); screen %.2f ms: %lld of %lld poses rescored, %d fallback ligand(s); "
         "best exact pose found for %d of %d ligands; %d mismatching energies\n",
         loss, train_ms, st.total_ms, (long long)nres, (long long)n, st.fallback_ligands, best_found, NLIG, bad);
  CHECK(bude_gpu_destroy(ctx));
  free(full);
  free(final);
  free(rescored);
  free_batch(&screen);
  free_batch(&train);
  return (bad == 0 && nres >= st.rescored_poses && best_found >= NLIG - 1) ? 0 : 2;
}
