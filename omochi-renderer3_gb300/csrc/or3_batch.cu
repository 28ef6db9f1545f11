// or3_batch.cu -- the batched form: many renders in one wavefront.
//
// The reference renders one scene per RenderScene call
// (src/renderer/PathTracer.cpp:55-85).  Small renders leave a GB300 mostly
// idle: a 128x128, 16-spp job is 262k camera paths, a few bounce waves of
// short kernels.  Here every job's path space (its samples in pass order,
// pixels, sub-pixels) is cut into segments aligned to whole pixel-samples,
// and a planner packs segments of all jobs into waves of up to `wave_paths`
// camera paths.  Rays carry their segment index, so the multi-job kernels
// (raygen/extend/shade/accumulate *_batch) pick scene, camera, depth policy and
// RNG numbering per ray.
//
// By default the device runs the whole batch: all planned waves sit in one
// device table, and each wave lane (stream and ray queues) is ONE launch of a
// graph whose single node is a while loop.  Its body takes the next wave from
// the shared head counter when the lane is idle, writes the wave's camera
// rays, runs `graph_bounces` extend/shade/shadow iterations, accumulates a
// wave whose queue ran empty, and ends the loop when the queue of waves is
// empty, with no host round trip in between.  OR3_FLAG_HOST_LOOP keeps the
// host-driven form: the host hands each wave to a free lane and replays the
// wave's captured bounce graph until its queue is empty.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include "or3_internal.h"

namespace or3 {

struct BatchBuffers {
  double *sum = nullptr, *sumsq = nullptr;
  size_t cap_pixels = 0, cap_sumsq = 0;
  size_t cap_frame_pinned = 0;
  DevScene *scenes = nullptr;
  size_t cap_scenes = 0;
  JobDev *jobs = nullptr;
  size_t cap_jobs = 0;
  // per wave lane (lane 0: the context's stream and queues; 1, 2: its extra
  // lanes): the wave's segment table, pinned staging, read-back counters
  struct Lane {
    Segment *segs = nullptr;
    size_t cap_segs = 0;
    WaveInfo *info = nullptr;
    Segment *segs_host = nullptr;  // pinned staging
    size_t cap_segs_host = 0;
    WaveInfo *info_host = nullptr;  // pinned
    uint32_t *hc = nullptr;         // pinned
    cudaEvent_t ev = nullptr;
  } lanes[3];
  double *frame_dev = nullptr, *frame_pinned = nullptr;
  size_t cap_frame = 0;
  // the device loop: every wave's segments, the wave table, the loop state
  Segment *segs_all = nullptr;
  size_t cap_segs_all = 0;
  WaveDesc *wdesc = nullptr;
  size_t cap_wdesc = 0;
  uint32_t *fail = nullptr;  // waves a glass split overflowed
  size_t cap_fail = 0;
  BatchLoop *loop = nullptr;
  struct JobOut {
    uint64_t pix_base;
    uint32_t W, H;
    uint64_t count;  // paths per pixel
  };
  std::vector<JobOut> last;
  bool valid = false;
};

void destroy_batch_state(or3_context *ctx) {
  BatchBuffers *b = ctx->batch;
  if (!b) return;
  cudaFree(b->sum);
  cudaFree(b->sumsq);
  cudaFree(b->scenes);
  cudaFree(b->jobs);
  for (BatchBuffers::Lane &L : b->lanes) {
    cudaFree(L.segs);
    cudaFree(L.info);
    cudaFreeHost(L.segs_host);
    cudaFreeHost(L.info_host);
    cudaFreeHost(L.hc);
    if (L.ev) cudaEventDestroy(L.ev);
  }
  cudaFree(b->frame_dev);
  cudaFreeHost(b->frame_pinned);
  cudaFree(b->segs_all);
  cudaFree(b->wdesc);
  cudaFree(b->fail);
  cudaFree(b->loop);
  delete b;
  ctx->batch = nullptr;
}

namespace {

template <class T>
int grow_dev(or3_context *ctx, T *&p, size_t &cap, size_t n) {
  if (n <= cap && p) return OR3_OK;
  cudaFree(p);
  p = nullptr;
  cap = 0;
  OR3_CUDA(ctx, cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
  cap = std::max<size_t>(n, 1);
  return OR3_OK;
}

template <class T>
int grow_pinned(or3_context *ctx, T *&p, size_t &cap, size_t n) {
  if (n <= cap && p) return OR3_OK;
  cudaFreeHost(p);
  p = nullptr;
  cap = 0;
  OR3_CUDA(ctx, cudaMallocHost(&p, std::max<size_t>(n, 1) * sizeof(T)));
  cap = std::max<size_t>(n, 1);
  return OR3_OK;
}

struct JobPlan {
  uint64_t per_sample;  // W*H*ss2
  uint32_t ss2;
  int32_t min_s, max_s, step;
  int32_t samples;  // samples the schedule renders (its last pass end)
};

struct PlannedWave {
  std::vector<Segment> segs;
  uint32_t num_paths = 0;
  uint32_t ngroups = 0;
};

// Cuts every job's passes into segments of whole pixel-samples and packs them
// into waves of at most `cap` paths, jobs in order.
void plan_waves(const std::vector<JobPlan> &jp, uint64_t cap, std::vector<PlannedWave> &waves) {
  waves.clear();
  PlannedWave cur;
  auto flush = [&]() {
    if (cur.num_paths) waves.push_back(cur);
    cur = PlannedWave();
  };
  for (uint32_t j = 0; j < jp.size(); j++) {
    const JobPlan &p = jp[j];
    int32_t prev = 0;
    for (int32_t next = p.min_s; next <= p.max_s; next += p.step) {
      uint64_t g = (uint64_t)prev * p.per_sample;
      const uint64_t end = (uint64_t)next * p.per_sample;
      while (g < end) {
        const uint64_t room = cap - cur.num_paths;
        const uint64_t take = std::min<uint64_t>(end - g, room) / p.ss2 * p.ss2;
        if (take == 0) {
          flush();
          continue;
        }
        Segment s{};
        s.g_first = g;
        s.job = j;
        s.wave_first = cur.num_paths;
        s.count = (uint32_t)take;
        s.pass_first = (uint32_t)prev;
        s.group_first = cur.ngroups;
        cur.segs.push_back(s);
        cur.num_paths += (uint32_t)take;
        cur.ngroups += (uint32_t)(take / p.ss2);
        g += take;
      }
      prev = next;
    }
  }
  flush();
}

// The segments of the waves `ids` of `src` cut into waves of at most `cap`
// paths (whole pixel-samples of each job; cap >= every job's ss2), for a
// re-render of waves whose ray queue a glass split overflowed.
void replan_waves(const std::vector<PlannedWave> &src, const std::vector<uint32_t> &ids,
                  const std::vector<JobPlan> &jp, uint64_t cap, std::vector<PlannedWave> &out) {
  out.clear();
  PlannedWave cur;
  auto flush = [&]() {
    if (cur.num_paths) out.push_back(cur);
    cur = PlannedWave();
  };
  for (uint32_t id : ids) {
    for (const Segment &s : src[id].segs) {
      const uint32_t ss2 = jp[s.job].ss2;
      uint64_t g = s.g_first;
      const uint64_t end = s.g_first + s.count;
      while (g < end) {
        const uint64_t take = std::min<uint64_t>(end - g, cap - cur.num_paths) / ss2 * ss2;
        if (take == 0) {
          flush();
          continue;
        }
        Segment t{};
        t.g_first = g;
        t.job = s.job;
        t.wave_first = cur.num_paths;
        t.count = (uint32_t)take;
        t.pass_first = s.pass_first;
        t.group_first = cur.ngroups;
        cur.segs.push_back(t);
        cur.num_paths += (uint32_t)take;
        cur.ngroups += (uint32_t)(take / ss2);
        g += take;
      }
    }
  }
  flush();
}

int run_batch(or3_context *ctx, const or3_batch_job *jobs, size_t n, const or3_batch_params *bp,
              or3_render_stats *out, bool write_frames) {
  if (!ctx || (n && !jobs)) return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "null argument");
  if (n == 0) return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "empty batch");
  if (n > (1u << 20)) return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "too many jobs");
  or3_batch_params defaults{};
  if (!bp) bp = &defaults;
  cudaSetDevice(ctx->device);
  if (!ctx->batch) ctx->batch = new BatchBuffers();
  BatchBuffers &B = *ctx->batch;
  B.valid = false;

  // scenes and jobs
  std::map<int32_t, uint32_t> scene_index;
  std::vector<DevScene> scenes;
  bool split = false;
  bool shadows = false;  // some job samples lights: the bounce loop runs the shadow kernel
  std::vector<JobDev> jd(n);
  std::vector<JobPlan> jp(n);
  std::vector<BatchBuffers::JobOut> outs(n);
  uint64_t pixels = 0, total_paths = 0, max_ss2 = 1;
  for (size_t j = 0; j < n; j++) {
    const or3_batch_job &job = jobs[j];
    auto it = ctx->scenes.find(job.scene);
    if (it == ctx->scenes.end()) return fail(ctx, OR3_ERR_NOT_FOUND, "job %zu: scene %d not found", j, job.scene);
    if (int v = validate_render(ctx, &job.camera, &job.params)) return v;
    if (!scene_index.count(job.scene)) {
      scene_index[job.scene] = (uint32_t)scenes.size();
      scenes.push_back(it->second->view);
      split = split || it->second->has_split;
    }
    const DevScene &sv = it->second->view;
    shadows = shadows || (job.params.next_event_estimation && (sv.num_lights > 0 || sv.env_light != 0));
    fill_render_const(&job.camera, &job.params, jd[j].rc);
    jd[j].scene = scene_index[job.scene];
    const uint64_t npix = (uint64_t)job.camera.width * job.camera.height;
    JobPlan &p = jp[j];
    p.ss2 = jd[j].rc.ss2;
    p.per_sample = npix * p.ss2;
    p.min_s = job.params.min_samples;
    p.max_s = job.params.max_samples;
    p.step = job.params.step_samples;
    p.samples = p.min_s + (p.max_s - p.min_s) / p.step * p.step;
    outs[j] = {pixels, job.camera.width, job.camera.height, (uint64_t)p.samples * p.ss2};
    pixels += npix;
    total_paths += (uint64_t)p.samples * p.per_sample;
    max_ss2 = std::max<uint64_t>(max_ss2, p.ss2);
  }
  const bool use_graph = !(bp->flags & OR3_FLAG_NO_GRAPH);
  const bool device_loop = use_graph && !(bp->flags & OR3_FLAG_HOST_LOOP);
  // Glass (a split makes up to 8 rays of a path): the device loop's queues
  // hold kSplitQueueFactor rays per path and a wave that overflows them is
  // rendered again in smaller waves after the loop; the host loop keeps 8.
  const uint64_t qfactor = !split ? 1 : device_loop ? kSplitQueueFactor : 8;
  uint64_t cap = bp->wave_paths ? bp->wave_paths : (split && !device_loop ? (1ull << 23) : (1ull << 25));
  cap = std::max<uint64_t>(cap, max_ss2);
  cap = std::min<uint64_t>(cap, (1ull << 31) / qfactor);  // queue capacities stay 32-bit
  cap = std::min<uint64_t>(cap, std::max<uint64_t>(total_paths, max_ss2));
  const uint64_t rays = std::max<uint64_t>(cap * qfactor, split ? 8 * max_ss2 : 1);
  const uint64_t safe_cap = std::max<uint64_t>(max_ss2, rays / 8);  // a wave this size cannot overflow
  std::vector<PlannedWave> waves;
  plan_waves(jp, cap, waves);
  size_t max_segs = 1;
  for (const PlannedWave &w : waves) max_segs = std::max(max_segs, w.segs.size());

  // device state
  int rc = ensure_queues(ctx, cap, rays);
  if (rc) return rc;
  if ((rc = grow_dev(ctx, B.sum, B.cap_pixels, 3 * pixels))) return rc;
  if ((rc = grow_dev(ctx, B.sumsq, B.cap_sumsq, 3 * pixels))) return rc;
  if ((rc = grow_dev(ctx, B.scenes, B.cap_scenes, scenes.size()))) return rc;
  if ((rc = grow_dev(ctx, B.jobs, B.cap_jobs, n))) return rc;
  // wave lanes (three unless OR3_FLAG_ONE_LANE): each runs its own waves on
  // its own stream and queues; the lanes' pixel sums are the jobs' (atomic adds)
  const int nl = (bp->flags & OR3_FLAG_ONE_LANE) || waves.size() < 2 ? 1 : (int)std::min<size_t>(3, waves.size());
  Queues ql[3];
  cudaStream_t sl[3];
  for (int l = 0; l < nl; l++) {
    BatchBuffers::Lane &L = B.lanes[l];
    if (l == 0) {
      ql[0] = make_queues(ctx);
      sl[0] = ctx->stream;
    } else {
      if ((rc = ensure_lane(ctx, l - 1, cap, rays, 1))) return rc;
      ql[l] = lane_queues(ctx->xl[l - 1]);
      sl[l] = ctx->xl[l - 1].stream;
    }
    ql[l].capacity = (uint32_t)std::min<uint64_t>(ql[l].capacity, rays);  // this batch's sizing
    if ((rc = grow_dev(ctx, L.segs, L.cap_segs, max_segs))) return rc;
    if ((rc = grow_pinned(ctx, L.segs_host, L.cap_segs_host, max_segs))) return rc;
    if (!L.info) OR3_CUDA(ctx, cudaMalloc(&L.info, sizeof(WaveInfo)));
    if (!L.info_host) OR3_CUDA(ctx, cudaMallocHost(&L.info_host, sizeof(WaveInfo)));
    if (!L.hc) OR3_CUDA(ctx, cudaMallocHost(&L.hc, 4 * sizeof(uint32_t)));
    if (!L.ev) OR3_CUDA(ctx, cudaEventCreateWithFlags(&L.ev, cudaEventDisableTiming));
  }
  cudaStream_t st = ctx->stream;
  for (size_t j = 0; j < n; j++) {
    jd[j].sum = B.sum + 3 * outs[j].pix_base;
    jd[j].sumsq = B.sumsq + 3 * outs[j].pix_base;
  }
  OR3_CUDA(ctx, cudaMemcpyAsync(B.scenes, scenes.data(), scenes.size() * sizeof(DevScene), cudaMemcpyHostToDevice, st));
  OR3_CUDA(ctx, cudaMemcpyAsync(B.jobs, jd.data(), n * sizeof(JobDev), cudaMemcpyHostToDevice, st));
  OR3_CUDA(ctx, cudaMemsetAsync(B.sum, 0, 3 * pixels * sizeof(double), st));
  OR3_CUDA(ctx, cudaMemsetAsync(B.sumsq, 0, 3 * pixels * sizeof(double), st));
  for (int l = 0; l < nl; l++) {
    OR3_CUDA(ctx, cudaMemsetAsync(ql[l].counters, 0, 16 * sizeof(uint32_t), st));
    OR3_CUDA(ctx, cudaMemsetAsync(ql[l].stats, 0, 8 * sizeof(unsigned long long), st));
  }

  const int bps_ext = bp->blocks_per_sm ? std::min<int>((int)bp->blocks_per_sm, ctx->occ_extend) : ctx->occ_extend;
  const int occ_sh = shadows ? ctx->occ_shade_nee : ctx->occ_shade;  // the instance launch_shade_batch picks
  const int bps_sh = bp->blocks_per_sm ? std::min<int>((int)bp->blocks_per_sm, occ_sh) : occ_sh;
  const int grid_ext = ctx->num_sms * std::max(bps_ext, 1);
  const int grid_sh = ctx->num_sms * std::max(bps_sh, 1);
  const bool count = (bp->flags & OR3_FLAG_COUNT_TRAVERSAL) != 0;
  int unroll = bp->graph_bounces ? (int)bp->graph_bounces : 8;
  unroll = std::max(2, std::min(unroll, 64));
  unroll += unroll & 1;  // even: the live queue is queue 0 after every replay

  // the bounce loop, captured once per call and lane
  auto lane_batch = [&](int l) { return Batch{B.scenes, B.jobs, B.lanes[l].segs, B.lanes[l].info}; };
  // traversal variant: node layout and how a ray's node array is reached
  const int tvar = ((bp->flags & OR3_FLAG_QUANTISED_NODES) ? 1 : 0) | ((bp->flags & OR3_FLAG_HOIST_NODES) ? 0 : 2);
  // material-sorted shade where the batch samples lights (as or3_render)
  const bool sorted_shade = shadows && !(bp->flags & OR3_FLAG_UNSORTED_SHADE);
  auto launch_bounces = [&](int l) {
    const Batch b = lane_batch(l);
    for (int k = 0; k < unroll; k++) {
      const int in = k & 1;
      launch_extend_batch(b, ql[l], in, grid_ext, count, tvar, sl[l]);
      if (sorted_shade)
        launch_shade_batch_sorted(b, ql[l], in, true, ctx->num_sms * 8, ctx->num_sms * ctx->occ_shade_nee,
                                  ctx->num_sms * ctx->occ_shade, sl[l]);
      else
        launch_shade_batch(b, ql[l], in, grid_sh, shadows, sl[l]);
      if (shadows) launch_shadow_batch(b, ql[l], grid_ext, tvar, sl[l]);
      launch_reset_count(ql[l], in, sl[l]);
    }
  };
  struct GraphGuard {
    cudaGraphExec_t g[3] = {nullptr, nullptr, nullptr};
    ~GraphGuard() {
      for (cudaGraphExec_t x : g)
        if (x) cudaGraphExecDestroy(x);
    }
  } guard;
  struct LoopGraphs {
    cudaGraph_t g[3] = {nullptr, nullptr, nullptr};
    ~LoopGraphs() {
      for (cudaGraph_t x : g)
        if (x) cudaGraphDestroy(x);
    }
  } lg;
  or3_render_stats stats{};
  // Device loop, one round over a wave list: the waves' segments go to the
  // device in one table, read by the lanes' loop heads as they take waves;
  // per lane a graph whose one node is a while loop, whose body takes a wave
  // when the lane is idle, runs `unroll` bounces and completes the wave when
  // its queue is empty.  (Re)captured per round: a round's tables may have
  // moved.
  auto prepare_round = [&](const std::vector<PlannedWave> &wv) -> int {
    std::vector<Segment> all;
    std::vector<WaveDesc> wd(wv.size());
    size_t msegs = 1;
    for (size_t w = 0; w < wv.size(); w++) {
      wd[w] = WaveDesc{(uint32_t)all.size(), (uint32_t)wv[w].segs.size(), wv[w].ngroups, wv[w].num_paths};
      all.insert(all.end(), wv[w].segs.begin(), wv[w].segs.end());
      msegs = std::max(msegs, wv[w].segs.size());
    }
    int r = OR3_OK;
    if ((r = grow_dev(ctx, B.segs_all, B.cap_segs_all, all.size()))) return r;
    if ((r = grow_dev(ctx, B.wdesc, B.cap_wdesc, wd.size()))) return r;
    if ((r = grow_dev(ctx, B.fail, B.cap_fail, wd.size()))) return r;
    for (int l = 0; l < nl; l++)
      if ((r = grow_dev(ctx, B.lanes[l].segs, B.lanes[l].cap_segs, msegs))) return r;
    if (!B.loop) OR3_CUDA(ctx, cudaMalloc(&B.loop, sizeof(BatchLoop)));
    BatchLoop hl{};
    hl.nwaves = (uint32_t)wd.size();
    hl.max_iters = 1u << 16;  // per wave, as the host loop's replay bound
    hl.fail_cap = (uint32_t)wd.size();
    if (!all.empty())
      OR3_CUDA(ctx, cudaMemcpyAsync(B.segs_all, all.data(), all.size() * sizeof(Segment), cudaMemcpyHostToDevice, st));
    if (!wd.empty())
      OR3_CUDA(ctx, cudaMemcpyAsync(B.wdesc, wd.data(), wd.size() * sizeof(WaveDesc), cudaMemcpyHostToDevice, st));
    OR3_CUDA(ctx, cudaMemcpyAsync(B.loop, &hl, sizeof(hl), cudaMemcpyHostToDevice, st));
    OR3_CUDA(ctx, cudaStreamSynchronize(st));
    for (int l = 0; l < nl; l++) {
      if (guard.g[l]) cudaGraphExecDestroy(guard.g[l]);
      guard.g[l] = nullptr;
      if (lg.g[l]) cudaGraphDestroy(lg.g[l]);
      lg.g[l] = nullptr;
      OR3_CUDA(ctx, cudaGraphCreate(&lg.g[l], 0));
      cudaGraphConditionalHandle h{};
      OR3_CUDA(ctx, cudaGraphConditionalHandleCreate(&h, lg.g[l], 1u, cudaGraphCondAssignDefault));
      cudaGraphNodeParams cp{};
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = h;
      cp.conditional.type = cudaGraphCondTypeWhile;
      cp.conditional.size = 1;
      cudaGraphNode_t node = nullptr;
      OR3_CUDA(ctx, cudaGraphAddNode(&node, lg.g[l], nullptr, nullptr, 0, &cp));
      cudaGraph_t body = cp.conditional.phGraph_out[0];
      OR3_CUDA(ctx, cudaStreamBeginCaptureToGraph(sl[l], body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
      BatchBuffers::Lane &L = B.lanes[l];
      const Batch b = lane_batch(l);
      launch_wave_take(B.loop, l, B.wdesc, B.segs_all, L.segs, L.info, ql[l].counters, h, sl[l]);
      launch_raygen_batch_loop(b, ql[l], B.loop, l, ctx->num_sms * 8, sl[l]);
      launch_bounces(l);
      launch_accumulate_batch_loop(b, ql[l], B.loop, l, ctx->num_sms * 8, sl[l]);
      launch_wave_finish(B.loop, l, L.info, ql[l].counters, B.fail, sl[l]);
      cudaGraph_t captured = nullptr;
      const cudaError_t ce = cudaStreamEndCapture(sl[l], &captured);
      if (ce != cudaSuccess) return fail(ctx, OR3_ERR_CUDA, "device loop capture: %s", cudaGetErrorString(ce));
      const cudaError_t ie = cudaGraphInstantiate(&guard.g[l], lg.g[l], 0);
      if (ie != cudaSuccess) return fail(ctx, OR3_ERR_CUDA, "device loop instantiate: %s", cudaGetErrorString(ie));
    }
    return OR3_OK;
  };
  // Runs a prepared round to its end; adds its completed waves and paths to
  // the stats and returns the waves a glass split overflowed in `failed`.
  auto run_round = [&](std::vector<uint32_t> &failed) -> int {
    if (nl > 1) {
      OR3_CUDA(ctx, cudaEventRecord(ctx->ev_fork, st));
      for (int l = 1; l < nl; l++) OR3_CUDA(ctx, cudaStreamWaitEvent(sl[l], ctx->ev_fork, 0));
    }
    for (int l = 0; l < nl; l++) OR3_CUDA(ctx, cudaGraphLaunch(guard.g[l], sl[l]));
    for (int l = 1; l < nl; l++) {
      OR3_CUDA(ctx, cudaEventRecord(B.lanes[l].ev, sl[l]));
      OR3_CUDA(ctx, cudaStreamWaitEvent(st, B.lanes[l].ev, 0));
    }
    OR3_CUDA(ctx, cudaStreamSynchronize(st));
    BatchLoop hl{};
    OR3_CUDA(ctx, cudaMemcpy(&hl, B.loop, sizeof(hl), cudaMemcpyDeviceToHost));
    uint32_t bits = 0;
    for (int l = 0; l < nl; l++) {
      uint32_t c[4];
      OR3_CUDA(ctx, cudaMemcpy(c, ql[l].counters, sizeof(c), cudaMemcpyDeviceToHost));
      bits |= c[2];
    }
    if (bits || (hl.abort & 2u)) return fail(ctx, OR3_ERR_DEVICE_REPORTED, "kernel reported error bits 0x%x in a batch", bits);
    if (hl.abort & 1u) return fail(ctx, OR3_ERR_DEVICE_REPORTED, "bounce loop did not end");
    if (hl.nfail > hl.fail_cap) return fail(ctx, OR3_ERR_DEVICE_REPORTED, "overflow list full (%u waves)", hl.nfail);
    uint32_t done = 0;
    for (int l = 0; l < nl; l++) {
      done += hl.lane[l].waves;
      stats.camera_paths += hl.lane[l].paths;
    }
    stats.waves += done;
    if (done + hl.nfail != hl.nwaves)
      return fail(ctx, OR3_ERR_DEVICE_REPORTED, "device loop completed %u of %u waves", done + hl.nfail, hl.nwaves);
    failed.resize(hl.nfail);
    if (hl.nfail)
      OR3_CUDA(ctx, cudaMemcpy(failed.data(), B.fail, hl.nfail * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    return OR3_OK;
  };
  if (device_loop) {
    OR3_CUDA(ctx, cudaStreamSynchronize(st));
    if ((rc = prepare_round(waves))) return rc;
  } else if (use_graph) {
    OR3_CUDA(ctx, cudaStreamSynchronize(st));
    for (int l = 0; l < nl; l++) {
      cudaGraph_t graph = nullptr;
      OR3_CUDA(ctx, cudaStreamBeginCapture(sl[l], cudaStreamCaptureModeThreadLocal));
      launch_bounces(l);
      OR3_CUDA(ctx, cudaStreamEndCapture(sl[l], &graph));
      cudaError_t e = cudaGraphInstantiate(&guard.g[l], graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) return fail(ctx, OR3_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    }
  }

  OR3_CUDA(ctx, cudaEventRecord(ctx->ev0, st));
  if (nl > 1 && !device_loop) {  // the extra lanes start after the tables and sums above
    OR3_CUDA(ctx, cudaEventRecord(ctx->ev_fork, st));
    for (int l = 1; l < nl; l++) OR3_CUDA(ctx, cudaStreamWaitEvent(sl[l], ctx->ev_fork, 0));
  }
  auto replay = [&](int l) -> int {
    BatchBuffers::Lane &L = B.lanes[l];
    if (use_graph) OR3_CUDA(ctx, cudaGraphLaunch(guard.g[l], sl[l]));
    else launch_bounces(l);
    OR3_CUDA(ctx, cudaMemcpyAsync(L.hc, ql[l].counters, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, sl[l]));
    OR3_CUDA(ctx, cudaEventRecord(L.ev, sl[l]));
    return OR3_OK;
  };
  // waves in plan order, each to the next free lane; the lanes are visited in turn
  size_t next_wave = 0;
  int wave_of[3] = {-1, -1, -1}, reps[3] = {0, 0, 0};
  auto start = [&](int l) -> int {
    if (next_wave >= waves.size()) return OR3_OK;
    const PlannedWave &w = waves[next_wave];
    BatchBuffers::Lane &L = B.lanes[l];
    std::memcpy(L.segs_host, w.segs.data(), w.segs.size() * sizeof(Segment));
    L.info_host->nseg = (uint32_t)w.segs.size();
    L.info_host->ngroups = w.ngroups;
    L.info_host->num_paths = w.num_paths;
    OR3_CUDA(ctx, cudaMemcpyAsync(L.segs, L.segs_host, w.segs.size() * sizeof(Segment), cudaMemcpyHostToDevice, sl[l]));
    OR3_CUDA(ctx, cudaMemcpyAsync(L.info, L.info_host, sizeof(WaveInfo), cudaMemcpyHostToDevice, sl[l]));
    launch_raygen_batch(lane_batch(l), w.num_paths, ql[l], 0, sl[l]);
    wave_of[l] = (int)next_wave++;
    reps[l] = 0;
    return replay(l);
  };
  int live = 0;
  if (device_loop) {  // the lanes' loops run the whole batch
    std::vector<uint32_t> failed;
    if ((rc = run_round(failed))) return rc;
    if (!failed.empty()) {
      // waves a glass split overflowed were not accumulated: their paths
      // again, in waves that cannot overflow (the same paths, the same image)
      stats.waves_rerun = (uint32_t)failed.size();
      std::vector<PlannedWave> sub;
      replan_waves(waves, failed, jp, safe_cap, sub);
      if ((rc = prepare_round(sub))) return rc;
      if ((rc = run_round(failed))) return rc;
      if (!failed.empty()) return fail(ctx, OR3_ERR_DEVICE_REPORTED, "ray queue capacity exceeded by a sub-wave");
    }
  } else {
    for (int l = 0; l < nl; l++) {
      if ((rc = start(l))) return rc;
      if (wave_of[l] >= 0) live++;
    }
  }
  while (live > 0) {
    for (int l = 0; l < nl; l++) {
      if (wave_of[l] < 0) continue;
      BatchBuffers::Lane &L = B.lanes[l];
      OR3_CUDA(ctx, cudaEventSynchronize(L.ev));
      if (L.hc[2]) {
        const uint32_t bits = L.hc[2];
        for (int k = 0; k < nl; k++) cudaStreamSynchronize(sl[k]);
        for (int k = 0; k < nl; k++) cudaMemsetAsync(ql[k].counters, 0, 16 * sizeof(uint32_t), st);
        cudaStreamSynchronize(st);
        return fail(ctx, OR3_ERR_DEVICE_REPORTED, "kernel reported error bits 0x%x in a batch", bits);
      }
      if (L.hc[0] != 0) {
        if (++reps[l] > (1 << 16)) return fail(ctx, OR3_ERR_DEVICE_REPORTED, "bounce loop did not end");
        if ((rc = replay(l))) return rc;
        continue;
      }
      const PlannedWave &w = waves[(size_t)wave_of[l]];
      launch_accumulate_batch(lane_batch(l), w.ngroups, ql[l], sl[l]);
      stats.waves++;
      stats.camera_paths += w.num_paths;
      wave_of[l] = -1;
      live--;
      if ((rc = start(l))) return rc;
      if (wave_of[l] >= 0) live++;
    }
  }
  for (int l = 1; l < nl; l++) {  // join the extra lanes
    OR3_CUDA(ctx, cudaEventRecord(B.lanes[l].ev, sl[l]));
    OR3_CUDA(ctx, cudaStreamWaitEvent(st, B.lanes[l].ev, 0));
  }
  OR3_CUDA(ctx, cudaEventRecord(ctx->ev1, st));
  OR3_CUDA(ctx, cudaEventSynchronize(ctx->ev1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  stats.render_ms = ms;
  if (write_frames) {
    size_t need = 0;
    for (size_t j = 0; j < n; j++)
      if (jobs[j].frame_host)
        need = std::max(need, (size_t)(jobs[j].params.output_layout == OR3_LAYOUT_REFERENCE ? 2 : 1) *
                                  jobs[j].camera.width * jobs[j].camera.height * 3);
    if (need) {
      if ((rc = grow_dev(ctx, B.frame_dev, B.cap_frame, need))) return rc;
      if ((rc = grow_pinned(ctx, B.frame_pinned, B.cap_frame_pinned, B.cap_frame))) return rc;
    }
    for (size_t j = 0; j < n; j++) {
      const or3_batch_job &job = jobs[j];
      if (!job.frame_host) continue;
      const size_t doubles = (size_t)(job.params.output_layout == OR3_LAYOUT_REFERENCE ? 2 : 1) * job.camera.width *
                             job.camera.height * 3;
      if (job.frame_capacity < doubles)
        return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "job %zu: frame needs %zu doubles", j, doubles);
      OR3_CUDA(ctx, cudaMemsetAsync(B.frame_dev, 0, doubles * sizeof(double), st));
      launch_frame(B.sum + 3 * outs[j].pix_base, job.camera.width, job.camera.height, job.params.output_layout,
                   1.0 / (double)outs[j].count, B.frame_dev, st);
      OR3_CUDA(ctx, cudaMemcpyAsync(B.frame_pinned, B.frame_dev, doubles * sizeof(double), cudaMemcpyDeviceToHost, st));
      OR3_CUDA(ctx, cudaStreamSynchronize(st));
      std::memcpy(job.frame_host, B.frame_pinned, doubles * sizeof(double));
    }
  }
  unsigned long long hs[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int l = 0; l < nl; l++) {
    unsigned long long h1[8];
    OR3_CUDA(ctx, cudaMemcpy(h1, ql[l].stats, sizeof(h1), cudaMemcpyDeviceToHost));
    for (int k = 0; k < 8; k++) hs[k] += h1[k];
  }
  stats.lanes = (uint32_t)nl;
  stats.extension_rays = hs[0];
  stats.shadow_rays = hs[1];
  stats.bounces = hs[2];
  stats.nodes_visited = hs[3];
  stats.tris_tested = hs[4];
  stats.spheres_tested = hs[5];
  stats.passes = 1;
  if (out) *out = stats;
  B.last = outs;
  B.valid = true;
  return OR3_OK;
}

}  // namespace
}  // namespace or3

using namespace or3;

extern "C" {

int or3_render_batch(or3_context *ctx, const or3_batch_job *jobs, size_t n_jobs, const or3_batch_params *params,
                     or3_render_stats *stats_out) {
  return run_batch(ctx, jobs, n_jobs, params, stats_out, true);
}

int or3_get_batch_moments(or3_context *ctx, size_t job, double *sum, double *sumsq, size_t capacity,
                          uint64_t *count_out) {
  if (!ctx) return OR3_ERR_INVALID_ARGUMENT;
  if (!ctx->batch || !ctx->batch->valid) return fail(ctx, OR3_ERR_NOT_FOUND, "no completed batch");
  BatchBuffers &B = *ctx->batch;
  if (job >= B.last.size()) return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "job %zu out of range", job);
  const BatchBuffers::JobOut &o = B.last[job];
  const size_t nd = (size_t)o.W * o.H * 3;
  if (capacity < nd) return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "moments need %zu doubles", nd);
  cudaSetDevice(ctx->device);
  double *tmp = nullptr;
  OR3_CUDA(ctx, cudaMalloc(&tmp, 2 * nd * sizeof(double)));
  launch_moments(B.sum + 3 * o.pix_base, B.sumsq + 3 * o.pix_base, o.W, o.H, tmp, tmp + nd, ctx->stream);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e == cudaSuccess && sum) e = cudaMemcpy(sum, tmp, nd * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && sumsq) e = cudaMemcpy(sumsq, tmp + nd, nd * sizeof(double), cudaMemcpyDeviceToHost);
  cudaFree(tmp);
  if (e != cudaSuccess) return fail(ctx, OR3_ERR_CUDA, "batch moments: %s", cudaGetErrorString(e));
  if (count_out) *count_out = o.count;
  return OR3_OK;
}

int or3_autotune_batch(or3_context *ctx, const or3_batch_job *jobs, size_t n, uint64_t sample_paths,
                       or3_batch_params *best, double *best_mpaths) {
  if (!ctx || !jobs || !best || n == 0) return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "null argument");
  // reduced copy: every job keeps its image and sub-pixel grid, its sample
  // budget is cut so the whole copy is about sample_paths camera paths
  uint64_t total = 0;
  for (size_t j = 0; j < n; j++)
    total += (uint64_t)jobs[j].camera.width * jobs[j].camera.height * jobs[j].params.supersamples *
             jobs[j].params.supersamples * (uint64_t)std::max(jobs[j].params.max_samples, 1);
  const double f = sample_paths && total > sample_paths ? (double)sample_paths / (double)total : 1.0;
  std::vector<or3_batch_job> small(jobs, jobs + n);
  for (or3_batch_job &j : small) {
    const int32_t s = std::max<int32_t>(1, (int32_t)std::lround(j.params.max_samples * f));
    j.params.min_samples = s;
    j.params.max_samples = s;
    j.params.step_samples = 1;
    j.frame_host = nullptr;
  }
  const uint64_t waves[] = {1ull << 21, 1ull << 22, 1ull << 23, 1ull << 24, 1ull << 25};
  const uint32_t unrolls[] = {4, 8, 16};
  double best_rate = -1.0;
  or3_batch_params bestp{};
  for (uint64_t wv : waves) {
    for (uint32_t un : unrolls) {
      for (uint32_t bps : {0u, 2u}) {
        or3_batch_params p{};
        p.wave_paths = wv;
        p.graph_bounces = un;
        p.blocks_per_sm = bps;
        or3_render_stats s{};
        int rc = run_batch(ctx, small.data(), n, &p, &s, false);  // warm-up
        if (rc == OR3_OK) rc = run_batch(ctx, small.data(), n, &p, &s, false);
        if (rc != OR3_OK) return rc;
        const double rate = (double)s.camera_paths / (s.render_ms * 1e3);
        if (rate > best_rate) {
          best_rate = rate;
          bestp = p;
        }
      }
    }
  }
  *best = bestp;
  if (best_mpaths) *best_mpaths = best_rate;
  return OR3_OK;
}

}  // extern "C"
