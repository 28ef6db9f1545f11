// or3_internal.h -- the context and helpers shared by the host translation
// units (or3_api.cu: plain render and queries; or3_batch.cu: batched and
// served forms).  Not part of the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "or3.h"
#include "or3_kernels.cuh"

namespace or3 {

struct SceneGPU {
  DevScene view{};
  std::vector<void *> allocs;       // cudaMalloc'd (the device BVH build's nodes, the 8-wide tree)
  std::vector<void *> pool_allocs;  // from the context's scene pool, freed on `stream`
  cudaStream_t stream = nullptr;
  or3_scene_info info{};
  bool has_split = false;  // a refractive layer exists: paths can split at depth <= 2
  // ray queue capacity per camera path for or3_render where paths can split:
  // kSplitQueueFactor, doubled (up to 8) after a render whose waves overflowed
  uint32_t split_factor = kSplitQueueFactor;
};

struct BatchBuffers;  // or3_batch.cu
struct Server;        // or3_batch.cu

}  // namespace or3

// extra wave lanes a context can hold (or3_render uses two by default)
constexpr int kExtraLanes = 3;

struct or3_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  std::map<int32_t, or3::SceneGPU *> scenes;
  int32_t next_scene = 1;
  int num_sms = 0;
  // resident 256-thread blocks per SM: extend; shade without / with the light sample
  int occ_extend = 1, occ_shade = 1, occ_shade_nee = 1;

  // queues
  size_t cap_rays = 0, cap_paths = 0;
  float4 *qorig[2] = {nullptr, nullptr}, *qdir[2] = {nullptr, nullptr}, *qbeta[2] = {nullptr, nullptr};
  float4 *hits = nullptr, *pathL = nullptr;
  float4 *sorig = nullptr, *sdir = nullptr, *scontrib = nullptr;  // shadow queue (cap_rays entries)
  uint32_t *slist = nullptr;  // sorted shade: hit indices by material class (cap_rays entries)
  uint32_t *counters = nullptr;
  unsigned long long *dstats = nullptr;
  uint32_t *host_counters = nullptr;  // pinned

  // accumulation + frames
  size_t cap_pixels = 0;
  double *pix_sum = nullptr, *pix_sumsq = nullptr;
  size_t cap_frame = 0;
  double *frame_dev = nullptr;
  uint32_t *wave_fail = nullptr;  // waves of a pass whose queue overflowed: [0] count, then indices
  size_t cap_wave_fail = 0;
  // pinned host frames: the pass's copy lands in the back buffer, which then
  // becomes the front (last completed frame, Renderer::GetResult) by a
  // pointer swap under frame_mu
  double *frame_pinned = nullptr, *frame_front = nullptr;
  size_t cap_back = 0, cap_front = 0, front_doubles = 0;
  std::mutex frame_mu;
  int32_t frame_samples = 0;

  std::atomic<bool> stop{false};
  or3_render_stats last{};
  uint32_t last_W = 0, last_H = 0;
  uint64_t last_count = 0;  // paths per pixel in the moments
  bool moments_valid = false;
  uint64_t last_wave_paths = 0;
  bool last_kept_paths = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // per-kernel timing events of one pass (4 per bounce: before extend, shade,
  // shadow and after), created on first use and kept for later renders
  std::vector<cudaEvent_t> kpool;
  // pinned staging of flattened primitives for device BVH builds (grown on demand)
  void *stage = nullptr;
  size_t stage_bytes = 0;
  // stream-ordered pool for the temporaries of a scene upload (keeps up to
  // 1 GiB cached between uploads)
  cudaMemPool_t tmp_pool = nullptr;
  // a scene's records, materials, sky and light tables: kept by the pool when
  // a scene is released, so the next upload maps no new memory
  cudaMemPool_t scene_pool = nullptr;

  // or3_render's extra wave lanes (two by default): waves are dealt round robin to lane 0
  // (the buffers above) and these, each on its own stream with its own
  // queues, counters and pixel sums (merged into lane 0's at the end of each
  // pass), so one wave's latency-bound shading overlaps another's traversal
  struct Lane {
    cudaStream_t stream = nullptr;
    float4 *qorig[2] = {nullptr, nullptr}, *qdir[2] = {nullptr, nullptr}, *qbeta[2] = {nullptr, nullptr};
    float4 *hits = nullptr, *pathL = nullptr, *sorig = nullptr, *sdir = nullptr, *scontrib = nullptr;
    uint32_t *slist = nullptr;
    uint32_t *counters = nullptr;
    unsigned long long *dstats = nullptr;
    double *pix_sum = nullptr, *pix_sumsq = nullptr;
    size_t cap_paths = 0, cap_rays = 0, cap_pixels = 0;
  } xl[kExtraLanes];
  cudaEvent_t ev_fork = nullptr, ev_join[kExtraLanes] = {};
  cudaEvent_t ev_poll[1 + kExtraLanes] = {};  // a lane's queue-count read-back has landed

  or3::BatchBuffers *batch = nullptr;  // batched form state (or3_batch.cu)
  or3::Server *server = nullptr;       // served form state (or3_batch.cu)
};

namespace or3 {

inline int fail(or3_context *ctx, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (ctx) ctx->err = buf;
  return code;
}

#define OR3_CUDA(ctx, call)                                                                      \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess) {                                                                     \
      return ::or3::fail(ctx, e_ == cudaErrorMemoryAllocation ? OR3_ERR_OUT_OF_MEMORY : OR3_ERR_CUDA, \
                         "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    }                                                                                            \
  } while (0)

// or3_api.cu
int ensure_queues(or3_context *ctx, size_t paths, size_t rays);
Queues make_queues(or3_context *ctx);
// extra wave lane k (0 or 1): stream, queues, counters, pixel sums
int ensure_lane(or3_context *ctx, int k, size_t paths, size_t rays, size_t pixels);
Queues lane_queues(const or3_context::Lane &L);
void camera_basis(const or3_camera *c, Camera32 &out);
int validate_render(or3_context *ctx, const or3_camera *cam, const or3_render_params *prm);
void fill_render_const(const or3_camera *cam, const or3_render_params *prm, RenderConst &rc);

// or3_batch.cu
void destroy_batch_state(or3_context *ctx);
// or3_server.cu
void destroy_server_state(or3_context *ctx);

}  // namespace or3
