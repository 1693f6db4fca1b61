// stream.cu -- evaluation of a pose set that lives in host memory, in chunks, with the copies
// overlapped with the kernels (bude_gpu_score_stream).
//
// For decks whose poses are produced or kept on the host (the 1,048,576-pose bm2_long deck is
// 24 MB of poses and 7.5e12 interactions per evaluation), the poses go to the device chunk by
// chunk: chunk i+1's poses are copied on one stream and chunk i-1's energies copied back on
// another while chunk i is evaluated on the context's stream.  Two staging slots per direction;
// events keep a slot from being refilled before its consumer has finished.  Every chunk runs the
// same launch shape as one bude_gpu_run over all poses would, so the energies are identical to it,
// bit for bit, whatever the chunk size.
#include <cuda_runtime.h>

#include <algorithm>

#include "exact_kernel.cuh"
#include "internal.h"

namespace bude {

struct StreamState {
  cudaStream_t h2d = nullptr, d2h = nullptr;
  DevBuf poses[2], energies[2], xform, edge_mask;
  cudaEvent_t copied[2] = {}, consumed[2] = {}, computed[2] = {}, returned[2] = {};
};

void release_streamer(Context &c) {
  if (!c.streamer) return;
  StreamState &s = *c.streamer;
  if (s.h2d) cudaStreamSynchronize(s.h2d);
  if (s.d2h) cudaStreamSynchronize(s.d2h);
  for (int b = 0; b < 2; ++b) {
    s.poses[b].release();
    s.energies[b].release();
    for (cudaEvent_t ev : {s.copied[b], s.consumed[b], s.computed[b], s.returned[b]})
      if (ev) cudaEventDestroy(ev);
  }
  s.xform.release();
  s.edge_mask.release();
  if (s.h2d) cudaStreamDestroy(s.h2d);
  if (s.d2h) cudaStreamDestroy(s.d2h);
  delete c.streamer;
  c.streamer = nullptr;
}

// The context's streaming state, created on first use, with slots for `chunk` poses.
static int streamer(Context &c, long long chunk, StreamState **out) {
  if (!c.streamer) {
    c.streamer = new StreamState();
    StreamState &s = *c.streamer;
    cudaError_t e = cudaStreamCreateWithFlags(&s.h2d, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s.d2h, cudaStreamNonBlocking);
    for (int b = 0; b < 2 && e == cudaSuccess; ++b)
      for (cudaEvent_t *ev : {&s.copied[b], &s.consumed[b], &s.computed[b], &s.returned[b]})
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
    if (e != cudaSuccess) {
      release_streamer(c);
      return cuda_error(e, "stream set-up");
    }
  }
  StreamState &s = *c.streamer;
  int rc = BUDE_OK;
  for (int b = 0; b < 2 && !rc; ++b) {
    rc = s.poses[b].reserve((size_t)chunk * 6 * sizeof(float), "streamed poses");
    if (!rc) rc = s.energies[b].reserve((size_t)chunk * sizeof(float), "streamed energies");
  }
  if (!rc) rc = s.xform.reserve((size_t)chunk * 12 * sizeof(float), "streamed transforms");
  if (!rc) rc = s.edge_mask.reserve((size_t)(chunk + 31) / 32 * sizeof(unsigned), "streamed irregular-pose bits");
  if (rc) return rc;
  *out = &s;
  return BUDE_OK;
}

static int score_stream(Context &c, const bude_launch_cfg &cfg, const float *poses, long long stride,
                        long long nposes, long long chunk, float *energies, float *ms) {
  if (!c.have_deck) return set_error(BUDE_ERR_STATE, "no deck uploaded");
  if (nposes < 0 || (nposes > 0 && (!poses || !energies)) || stride < nposes)
    return set_error(BUDE_ERR_ARG, "bad poses, stride or energies");
  if (chunk <= 0) return set_error(BUDE_ERR_ARG, "chunk must be positive (got %lld)", chunk);
  int rc = check_cfg(c, cfg);
  if (rc) return rc;
  {
    // Round the chunk up to whole waves of the launch shape's resident blocks, so that no chunk's
    // launch leaves SMs idle in a partial last wave (131,072 poses at 16 poses per thread, 128
    // threads and 8 slices fill 0.84 of one wave of 608 blocks; 155,648 fill it).
    int per_sm = 0;
    if (exact_blocks_per_sm(cfg, &per_sm) == BUDE_OK && per_sm > 0) {
      const long long slots = (long long)per_sm * std::max(c.num_sms, 1);
      const long long ppw = std::max(1LL, slots / std::max(cfg.split, 1)) * cfg.ppwi * cfg.wgsize;
      chunk = (chunk + ppw - 1) / ppw * ppw;
    }
  }
  chunk = std::min(chunk, std::max(nposes, 1LL));
  StreamState *sp = nullptr;
  rc = streamer(c, chunk, &sp);
  if (rc) return rc;
  StreamState &s = *sp;
  const long long nchunks = (nposes + chunk - 1) / chunk;
  cudaEventRecord(c.ev0, c.stream);
  // Host -> device copy of chunk i's six pose fields into slot i % 2 (rows of n floats).
  auto upload = [&](long long i) -> cudaError_t {
    const int b = (int)(i & 1);
    const long long first = i * chunk, n = std::min(chunk, nposes - first);
    if (i >= 2) cudaStreamWaitEvent(s.h2d, s.consumed[b], 0); // slot read by chunk i-2's transforms
    cudaError_t e = cudaMemcpy2DAsync(s.poses[b].ptr, (size_t)n * sizeof(float), poses + first,
                                      (size_t)stride * sizeof(float), (size_t)n * sizeof(float), 6,
                                      cudaMemcpyHostToDevice, s.h2d);
    if (e == cudaSuccess) e = cudaEventRecord(s.copied[b], s.h2d);
    return e;
  };
  cudaError_t e = nposes > 0 ? upload(0) : cudaSuccess;
  for (long long i = 0; i < nchunks && e == cudaSuccess && !rc; ++i) {
    const int b = (int)(i & 1);
    const long long first = i * chunk, n = std::min(chunk, nposes - first);
    if (i + 1 < nchunks) e = upload(i + 1);
    if (e != cudaSuccess) break;
    cudaStreamWaitEvent(c.stream, s.copied[b], 0);
    if (i >= 2) cudaStreamWaitEvent(c.stream, s.returned[b], 0); // energies slot copied back
    const int tb = 256;
    pose_xform_kernel<<<(unsigned)((n + tb - 1) / tb), tb, 0, c.stream>>>(s.poses[b].as<float>(), n, n,
                                                                          s.xform.as<float4>(),
                                                                          s.edge_mask.as<unsigned>());
    c.launches++;
    e = cudaEventRecord(s.consumed[b], c.stream);
    if (e != cudaSuccess) break;
    rc = launch_exact_range(c, cfg, c.ligand.as<float4>(), c.natlig, s.xform.as<float>(), s.energies[b].as<float>(), n);
    if (!rc)
      rc = enqueue_edge_single(c, c.ligand.as<float4>(), c.natlig, c.deck_irregular, s.edge_mask.as<unsigned>(),
                               s.xform.as<float>(), s.energies[b].as<float>(), n, c.stream);
    if (rc) break;
    e = cudaEventRecord(s.computed[b], c.stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s.d2h, s.computed[b], 0);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(energies + first, s.energies[b].ptr, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost,
                          s.d2h);
    if (e == cudaSuccess) e = cudaEventRecord(s.returned[b], s.d2h);
  }
  // Drain both copy streams into the context's stream, then time and check.
  cudaEvent_t done = nullptr;
  if (cudaEventCreateWithFlags(&done, cudaEventDisableTiming) == cudaSuccess) {
    cudaEventRecord(done, s.d2h);
    cudaStreamWaitEvent(c.stream, done, 0);
    cudaEventRecord(done, s.h2d);
    cudaStreamWaitEvent(c.stream, done, 0);
  }
  cudaEventRecord(c.ev1, c.stream);
  const cudaError_t es = cudaStreamSynchronize(c.stream);
  if (done) cudaEventDestroy(done);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_error(e, "streamed evaluation");
  if (es != cudaSuccess) return cuda_error(es, "streamed evaluation");
  if (ms) cudaEventElapsedTime(ms, c.ev0, c.ev1);
  return check_device_error(c);
}

} // namespace bude

using namespace bude;

extern "C" int bude_gpu_score_stream(bude_gpu_ctx *ctx, const bude_launch_cfg *cfg, const float *poses,
                                     int64_t pose_stride, int64_t nposes, int64_t chunk, float *energies, float *ms) {
  if (!ctx || !cfg) return set_error(BUDE_ERR_ARG, "NULL argument");
  cudaSetDevice(ctx->device);
  return score_stream(*ctx, *cfg, poses, pose_stride, nposes, chunk, energies, ms);
}
