// or3_server.cu -- the served form: continuous batching of render jobs.
//
// One worker thread owns the context's stream.  Submitted jobs wait in a FIFO
// until a slot and their device memory (pixel sums, frame) fit in the budget;
// admitted jobs share every wave fairly (each gets wave/active paths, leftover
// room goes to whoever still has paths), so a job that arrives while others
// run starts at the next wave instead of after them.  Waves use the batched
// kernels and the captured bounce-loop graph of or3_batch.cu's design; a job's
// paths keep or3_render's numbering and seeds, so its image is the same alone
// or in any mix.  After each wave, jobs that crossed a frame boundary get a
// progressive frame; the last one is final and closes the job's latency
// (submission to final frame).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "or3_internal.h"

namespace or3 {

namespace {

using Clock = std::chrono::steady_clock;

struct SJob {
  uint64_t id = 0;
  or3_batch_job job{};
  uint64_t per_sample = 0;
  uint32_t ss2 = 1;
  int32_t samples = 0;   // samples of the schedule
  uint64_t total = 0;    // camera paths
  uint64_t cursor = 0;   // next path to schedule
  uint64_t done = 0;     // paths accumulated
  uint64_t next_frame = 0;
  double *sum = nullptr, *sumsq = nullptr;
  size_t bytes = 0;
  int32_t state = OR3_JOB_QUEUED;
  int32_t samples_done = 0;
  double t_submit = 0, t_admit = -1, t_first = -1, t_done = -1;
  bool cancel = false;
  uint32_t scene_slot = 0;
  std::vector<double> host_sum, host_sumsq;  // kept moments
};

}  // namespace

struct Server {
  or3_server_params p{};
  or3_job_frame_callback cb = nullptr;
  or3_job_frame8_callback cb8 = nullptr;  // frames encoded to 8-bit on the device (or3_server_start8)
  void *user = nullptr;
  std::thread th;
  std::mutex mu;
  std::condition_variable cv;   // wakes the worker
  std::condition_variable idle; // wakes drain()
  bool quit = false;
  std::deque<SJob *> pending;
  std::vector<SJob *> active;
  std::map<uint64_t, SJob *> all;
  uint64_t next_id = 1;
  uint64_t budget = 0, in_use = 0, peak_in_use = 0, peak_active = 0;
  Clock::time_point t0;
  uint64_t cap = 0;
  bool split = false;
  uint64_t rays = 0;  // a lane's queue capacity (kSplitQueueFactor rays per path where glass can split)
  // stats
  uint64_t paths = 0, waves = 0, submitted = 0, finished = 0, cancelled = 0, waves_rerun = 0;
  double device_ms = 0, busy_s = 0;
  int error = OR3_OK;
  std::string error_msg;
  // device tables (fixed capacity: the captured graphs hold their addresses)
  std::map<int32_t, uint32_t> scene_index;
  DevScene *scenes_dev = nullptr;
  JobDev *jobs_dev = nullptr;
  JobDev *jobs_host = nullptr;
  uint32_t cap_segs = 0;
  // Wave lanes: a wave's segments are dealt to the lanes, each with its own
  // stream, ray queues, segment table and captured bounce loop; the lanes run
  // at once and join before the frames.  Lane 0 is the context's stream and
  // queues, lanes 1.. the context's extra lanes.
  struct Lane {
    cudaStream_t st = nullptr;
    Queues q{};
    Segment *segs_dev = nullptr, *segs_host = nullptr;
    WaveInfo *info_dev = nullptr, *info_host = nullptr;
    uint32_t *hc = nullptr;  // pinned: the lane's queue counters, read back per replay
    cudaGraphExec_t graph = nullptr;
    cudaEvent_t ev = nullptr;
    std::vector<Segment> segs;
    uint64_t used = 0, groups = 0;
    bool live = false;
  };
  std::vector<Lane> lanes;
  cudaEvent_t ev_jobs = nullptr;
  double *frame_dev = nullptr, *frame_pinned = nullptr;
  size_t cap_frame = 0;
  uint8_t *frame8_dev = nullptr, *frame8_pinned = nullptr;  // 8-bit frames (3 bytes per pixel)
  int unroll = 8;
  cudaEvent_t e0 = nullptr, e1 = nullptr;

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

size_t frame_doubles(const or3_batch_job &j) {
  return (size_t)(j.params.output_layout == OR3_LAYOUT_REFERENCE ? 2 : 1) * j.camera.width * j.camera.height * 3;
}

void free_job_device(SJob *j) {
  cudaFree(j->sum);
  cudaFree(j->sumsq);
  j->sum = j->sumsq = nullptr;
}

// End of the pass holding path g, as a path count (segments never straddle passes).
uint64_t pass_end(const SJob &j, uint64_t g, uint32_t *pass_first) {
  const uint64_t s = g / j.per_sample;
  int32_t prev = 0;
  for (int32_t next = j.job.params.min_samples; next <= j.job.params.max_samples;
       next += j.job.params.step_samples) {
    if ((int64_t)s < next) {
      *pass_first = (uint32_t)prev;
      return (uint64_t)next * j.per_sample;
    }
    prev = next;
  }
  *pass_first = (uint32_t)prev;
  return j.total;
}

int emit_frame(or3_context *ctx, Server &S, SJob &j, bool final) {
  cudaStream_t st = ctx->stream;
  const size_t nd = frame_doubles(j.job);
  if (nd > S.cap_frame) {  // staging is the worker's own; grows to the largest frame seen
    OR3_CUDA(ctx, cudaStreamSynchronize(st));
    cudaFree(S.frame_dev);
    cudaFreeHost(S.frame_pinned);
    cudaFree(S.frame8_dev);
    cudaFreeHost(S.frame8_pinned);
    S.frame_dev = nullptr;
    S.frame_pinned = nullptr;
    S.frame8_dev = nullptr;
    S.frame8_pinned = nullptr;
    S.cap_frame = 0;
    OR3_CUDA(ctx, cudaMalloc(&S.frame_dev, nd * sizeof(double)));
    if (S.cb8) {
      OR3_CUDA(ctx, cudaMalloc(&S.frame8_dev, nd));
      OR3_CUDA(ctx, cudaMallocHost(&S.frame8_pinned, nd));
    } else {
      OR3_CUDA(ctx, cudaMallocHost(&S.frame_pinned, nd * sizeof(double)));
    }
    S.cap_frame = nd;
  }
  OR3_CUDA(ctx, cudaMemsetAsync(S.frame_dev, 0, nd * sizeof(double), st));
  launch_frame(j.sum, j.job.camera.width, j.job.camera.height, j.job.params.output_layout,
               1.0 / ((double)j.samples_done * j.ss2), S.frame_dev, st);
  const size_t w = (j.job.params.output_layout == OR3_LAYOUT_REFERENCE ? 2 : 1) * (size_t)j.job.camera.width;
  if (S.cb8) {
    // 8-bit on the device: 3 bytes per pixel cross to the host instead of 24
    launch_encode_rgb8(S.frame_dev, nd, 1, S.frame8_dev, st);
    OR3_CUDA(ctx, cudaMemcpyAsync(S.frame8_pinned, S.frame8_dev, nd, cudaMemcpyDeviceToHost, st));
    OR3_CUDA(ctx, cudaStreamSynchronize(st));
    if (j.t_first < 0) j.t_first = S.now();
    S.cb8(S.user, j.id, j.samples_done, S.frame8_pinned, w, j.job.camera.height, final ? 1 : 0);
    return OR3_OK;
  }
  OR3_CUDA(ctx, cudaMemcpyAsync(S.frame_pinned, S.frame_dev, nd * sizeof(double), cudaMemcpyDeviceToHost, st));
  OR3_CUDA(ctx, cudaStreamSynchronize(st));
  if (j.t_first < 0) j.t_first = S.now();
  if (j.job.frame_host && j.job.frame_capacity >= nd) std::memcpy(j.job.frame_host, S.frame_pinned, nd * sizeof(double));
  if (S.cb) S.cb(S.user, j.id, j.samples_done, S.frame_pinned, w, j.job.camera.height, final ? 1 : 0);
  return OR3_OK;
}

int keep_moments(or3_context *ctx, SJob &j) {
  const size_t nd = (size_t)j.job.camera.width * j.job.camera.height * 3;
  double *tmp = nullptr;
  OR3_CUDA(ctx, cudaMalloc(&tmp, 2 * nd * sizeof(double)));
  launch_moments(j.sum, j.sumsq, j.job.camera.width, j.job.camera.height, tmp, tmp + nd, ctx->stream);
  j.host_sum.resize(nd);
  j.host_sumsq.resize(nd);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpy(j.host_sum.data(), tmp, nd * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(j.host_sumsq.data(), tmp + nd, nd * sizeof(double), cudaMemcpyDeviceToHost);
  cudaFree(tmp);
  if (e != cudaSuccess) return fail(ctx, OR3_ERR_CUDA, "keep moments: %s", cudaGetErrorString(e));
  return OR3_OK;
}

// One wave over the active jobs.  Returns an OR3 status.
int run_wave(or3_context *ctx, Server &S, std::vector<SJob *> &act) {
  cudaStream_t st = ctx->stream;
  const size_t na = act.size();
  // job table
  for (size_t k = 0; k < na; k++) {
    SJob &j = *act[k];
    JobDev &d = S.jobs_host[k];
    fill_render_const(&j.job.camera, &j.job.params, d.rc);
    d.scene = j.scene_slot;
    d.sum = j.sum;
    d.sumsq = j.sumsq;
  }
  // Segments, lane by lane: each lane takes up to cap paths (its queues are
  // sized for a whole wave: larger waves make every kernel cheaper per ray),
  // fair shares of the active jobs first, then leftover room.
  const size_t nl = S.lanes.size();
  const uint64_t cap_l = std::max<uint64_t>(S.cap, 1);
  std::vector<uint64_t> taken(na, 0);
  uint64_t used_all = 0;
  for (size_t l = 0; l < nl; l++) {
    Server::Lane &L = S.lanes[l];
    std::vector<Segment> &segs = L.segs;
    segs.clear();
    uint64_t used = 0, groups = 0;
    auto give = [&](size_t k, uint64_t want) {
      SJob &j = *act[k];
      while (want >= j.ss2 && j.cursor < j.total && used + j.ss2 <= cap_l && segs.size() < S.cap_segs) {
        uint32_t pf = 0;
        const uint64_t pend = pass_end(j, j.cursor, &pf);
        uint64_t take = std::min<uint64_t>({want, pend - j.cursor, cap_l - used});
        take = take / j.ss2 * j.ss2;
        if (take == 0) break;
        Segment s{};
        s.g_first = j.cursor;
        s.job = (uint32_t)k;
        s.wave_first = (uint32_t)used;
        s.count = (uint32_t)take;
        s.pass_first = pf;
        s.group_first = (uint32_t)groups;
        segs.push_back(s);
        used += take;
        groups += take / j.ss2;
        j.cursor += take;
        taken[k] += take;
        want -= take;
      }
    };
    const uint64_t share = std::max<uint64_t>(cap_l / std::max<size_t>(na, 1), 1);
    for (size_t k = 0; k < na; k++) give(k, share);
    for (size_t k = 0; k < na && used < cap_l; k++) give(k, cap_l - used);
    L.used = used;
    L.groups = groups;
    used_all += used;
  }
  if (used_all == 0) return OR3_OK;

  OR3_CUDA(ctx, cudaEventRecord(S.e0, st));
  OR3_CUDA(ctx, cudaMemcpyAsync(S.jobs_dev, S.jobs_host, na * sizeof(JobDev), cudaMemcpyHostToDevice, st));
  OR3_CUDA(ctx, cudaEventRecord(S.ev_jobs, st));
  int live = 0;
  for (size_t l = 0; l < nl; l++) {
    Server::Lane &L = S.lanes[l];
    L.live = false;
    if (L.segs.empty()) continue;
    if (l) OR3_CUDA(ctx, cudaStreamWaitEvent(L.st, S.ev_jobs, 0));
    std::memcpy(L.segs_host, L.segs.data(), L.segs.size() * sizeof(Segment));
    L.info_host->nseg = (uint32_t)L.segs.size();
    L.info_host->ngroups = (uint32_t)L.groups;
    L.info_host->num_paths = (uint32_t)L.used;
    OR3_CUDA(ctx, cudaMemcpyAsync(L.segs_dev, L.segs_host, L.segs.size() * sizeof(Segment), cudaMemcpyHostToDevice,
                                  L.st));
    OR3_CUDA(ctx, cudaMemcpyAsync(L.info_dev, L.info_host, sizeof(WaveInfo), cudaMemcpyHostToDevice, L.st));
    const Batch b{S.scenes_dev, S.jobs_dev, L.segs_dev, L.info_dev};
    launch_raygen_batch(b, (uint32_t)L.used, L.q, 0, L.st);
    OR3_CUDA(ctx, cudaGraphLaunch(L.graph, L.st));
    OR3_CUDA(ctx, cudaMemcpyAsync(L.hc, L.q.counters, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, L.st));
    OR3_CUDA(ctx, cudaEventRecord(L.ev, L.st));
    L.live = true;
    live++;
  }
  // replay each lane's bounce loop until its queue is empty, visiting the
  // lanes in turn (the others keep running meanwhile)
  std::vector<Segment> redo;  // segments of lanes whose queue overflowed
  for (int rep = 0; live > 0; rep++) {
    if (rep > (1 << 18)) return fail(ctx, OR3_ERR_DEVICE_REPORTED, "bounce loop did not end");
    for (size_t l = 0; l < nl; l++) {
      Server::Lane &L = S.lanes[l];
      if (!L.live) continue;
      OR3_CUDA(ctx, cudaEventSynchronize(L.ev));
      if (L.hc[2] & ~kErrQueue) return fail(ctx, OR3_ERR_DEVICE_REPORTED, "kernel error bits 0x%x", L.hc[2]);
      if (L.hc[0] == 0) {
        const Batch b{S.scenes_dev, S.jobs_dev, L.segs_dev, L.info_dev};
        if (L.hc[2] & kErrQueue) {  // a glass split overflowed the queue: rendered again below
          redo.insert(redo.end(), L.segs.begin(), L.segs.end());
          OR3_CUDA(ctx, cudaMemsetAsync(L.q.counters + 2, 0, sizeof(uint32_t), L.st));
        } else {
          launch_accumulate_batch(b, (uint32_t)L.groups, L.q, L.st);
        }
        if (l) {
          OR3_CUDA(ctx, cudaEventRecord(L.ev, L.st));
          OR3_CUDA(ctx, cudaStreamWaitEvent(st, L.ev, 0));
        }
        L.live = false;
        live--;
        continue;
      }
      OR3_CUDA(ctx, cudaGraphLaunch(L.graph, L.st));
      OR3_CUDA(ctx, cudaMemcpyAsync(L.hc, L.q.counters, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, L.st));
      OR3_CUDA(ctx, cudaEventRecord(L.ev, L.st));
    }
  }
  // Overflowed lanes: their segments again, on lane 0, in pieces of at most
  // a queue's capacity / 8 paths, one piece per sub-wave (the same paths).
  if (!redo.empty()) {
    Server::Lane &L = S.lanes[0];
    const Batch b{S.scenes_dev, S.jobs_dev, L.segs_dev, L.info_dev};
    for (const Segment &sg : redo) {
      const uint64_t ss2 = act[sg.job]->ss2;
      const uint64_t piece = std::max<uint64_t>(ss2, S.rays / 8 / ss2 * ss2);
      for (uint64_t off = 0; off < sg.count; off += piece) {
        Segment t = sg;
        t.g_first = sg.g_first + off;
        t.count = (uint32_t)std::min<uint64_t>(piece, sg.count - off);
        t.wave_first = 0;
        t.group_first = 0;
        L.segs_host[0] = t;
        L.info_host->nseg = 1;
        L.info_host->ngroups = (uint32_t)(t.count / ss2);
        L.info_host->num_paths = t.count;
        OR3_CUDA(ctx, cudaMemcpyAsync(L.segs_dev, L.segs_host, sizeof(Segment), cudaMemcpyHostToDevice, L.st));
        OR3_CUDA(ctx, cudaMemcpyAsync(L.info_dev, L.info_host, sizeof(WaveInfo), cudaMemcpyHostToDevice, L.st));
        launch_raygen_batch(b, t.count, L.q, 0, L.st);
        for (int rep = 0;; rep++) {
          if (rep > (1 << 18)) return fail(ctx, OR3_ERR_DEVICE_REPORTED, "bounce loop did not end");
          OR3_CUDA(ctx, cudaGraphLaunch(L.graph, L.st));
          OR3_CUDA(ctx, cudaMemcpyAsync(L.hc, L.q.counters, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, L.st));
          OR3_CUDA(ctx, cudaStreamSynchronize(L.st));
          if (L.hc[2]) return fail(ctx, OR3_ERR_DEVICE_REPORTED, "kernel error bits 0x%x in a re-rendered piece", L.hc[2]);
          if (L.hc[0] == 0) break;
        }
        launch_accumulate_batch(b, t.count / (uint32_t)ss2, L.q, L.st);
      }
    }
    S.waves_rerun++;
  }
  OR3_CUDA(ctx, cudaEventRecord(S.e1, st));
  OR3_CUDA(ctx, cudaEventSynchronize(S.e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, S.e0, S.e1);
  S.device_ms += ms;
  S.paths += used_all;
  S.waves++;
  // progressive and final frames
  const uint64_t every = S.p.frame_every_samples ? S.p.frame_every_samples : 16;
  for (size_t k = 0; k < na; k++) {
    SJob &j = *act[k];
    if (!taken[k]) continue;
    j.done += taken[k];
    const bool final = j.done >= j.total;
    if (final || j.done >= j.next_frame) {
      j.samples_done = (int32_t)(j.done / j.per_sample);
      while (j.next_frame <= j.done) j.next_frame += every * j.per_sample;
      if (j.samples_done > 0)
        if (int rc = emit_frame(ctx, S, j, final)) return rc;
    }
  }
  return OR3_OK;
}

void worker(or3_context *ctx) {
  Server &S = *ctx->server;
  cudaSetDevice(ctx->device);
  for (;;) {
    std::vector<SJob *> act;
    {
      std::unique_lock<std::mutex> lk(S.mu);
      // cancellations of running jobs
      for (size_t k = 0; k < S.active.size();) {
        SJob *j = S.active[k];
        if (j->cancel) {
          free_job_device(j);
          S.in_use -= j->bytes;
          j->state = OR3_JOB_CANCELLED;
          j->t_done = S.now();
          S.cancelled++;
          S.active.erase(S.active.begin() + k);
        } else {
          k++;
        }
      }
      // admission: FIFO, by slots and device-memory budget
      const size_t maxa = S.p.max_active_jobs ? S.p.max_active_jobs : 64;
      while (!S.pending.empty() && S.active.size() < maxa) {
        SJob *j = S.pending.front();
        if (j->cancel) {
          S.pending.pop_front();
          j->state = OR3_JOB_CANCELLED;
          S.cancelled++;
          continue;
        }
        if (S.in_use + j->bytes > S.budget && !S.active.empty()) break;
        const size_t nd = (size_t)j->job.camera.width * j->job.camera.height * 3;
        if (cudaMalloc(&j->sum, nd * sizeof(double)) != cudaSuccess ||
            cudaMalloc(&j->sumsq, nd * sizeof(double)) != cudaSuccess) {
          cudaGetLastError();
          free_job_device(j);
          if (S.active.empty()) {  // cannot ever fit
            S.pending.pop_front();
            j->state = OR3_JOB_FAILED;
            S.cancelled++;
            continue;
          }
          break;
        }
        cudaMemsetAsync(j->sum, 0, nd * sizeof(double), ctx->stream);
        cudaMemsetAsync(j->sumsq, 0, nd * sizeof(double), ctx->stream);
        S.pending.pop_front();
        S.in_use += j->bytes;
        S.peak_in_use = std::max(S.peak_in_use, S.in_use);
        j->state = OR3_JOB_RUNNING;
        j->t_admit = S.now();
        S.active.push_back(j);
      }
      S.peak_active = std::max<uint64_t>(S.peak_active, S.active.size());
      if (S.active.empty()) {
        S.idle.notify_all();
        if (S.quit || S.error) return;
        S.cv.wait(lk);
        continue;
      }
      act = S.active;
    }
    const double w0 = S.now();
    int rc = run_wave(ctx, S, act);
    {
      std::lock_guard<std::mutex> lk(S.mu);
      S.busy_s += S.now() - w0;
      if (rc != OR3_OK) {
        S.error = rc;
        S.error_msg = ctx->err;
        for (SJob *j : S.active) {
          free_job_device(j);
          j->state = OR3_JOB_FAILED;
        }
        S.in_use = 0;
        S.active.clear();
        S.idle.notify_all();
        return;
      }
      for (size_t k = 0; k < S.active.size();) {
        SJob *j = S.active[k];
        if (j->done >= j->total) {
          if (S.p.flags & OR3_SERVER_KEEP_MOMENTS) keep_moments(ctx, *j);
          free_job_device(j);
          S.in_use -= j->bytes;
          j->state = OR3_JOB_DONE;
          j->t_done = S.now();
          S.finished++;
          S.active.erase(S.active.begin() + k);
        } else {
          k++;
        }
      }
    }
  }
}

double percentile(std::vector<double> v, double p) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const double idx = p * (double)(v.size() - 1);
  const size_t lo = (size_t)idx, hi = std::min(v.size() - 1, lo + 1);
  return v[lo] + (v[hi] - v[lo]) * (idx - (double)lo);
}

}  // namespace

void destroy_server_state(or3_context *ctx) {
  Server *S = ctx->server;
  if (!S) return;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->quit = true;
    for (SJob *j : S->pending) j->cancel = true;
    for (SJob *j : S->active) j->cancel = true;
  }
  S->cv.notify_all();
  if (S->th.joinable()) S->th.join();
  for (auto &kv : S->all) {
    free_job_device(kv.second);
    delete kv.second;
  }
  for (Server::Lane &L : S->lanes) {
    if (L.st) cudaStreamSynchronize(L.st);
    if (L.graph) cudaGraphExecDestroy(L.graph);
    cudaFree(L.segs_dev);
    cudaFreeHost(L.segs_host);
    cudaFree(L.info_dev);
    cudaFreeHost(L.info_host);
    cudaFreeHost(L.hc);
    if (L.ev) cudaEventDestroy(L.ev);
  }
  if (S->ev_jobs) cudaEventDestroy(S->ev_jobs);
  cudaFree(S->scenes_dev);
  cudaFree(S->jobs_dev);
  cudaFreeHost(S->jobs_host);
  cudaFree(S->frame_dev);
  cudaFreeHost(S->frame_pinned);
  cudaFree(S->frame8_dev);
  cudaFreeHost(S->frame8_pinned);
  if (S->e0) cudaEventDestroy(S->e0);
  if (S->e1) cudaEventDestroy(S->e1);
  delete S;
  ctx->server = nullptr;
}

}  // namespace or3

using namespace or3;

extern "C" {

static int server_start(or3_context *ctx, const or3_server_params *params, or3_job_frame_callback cb,
                        or3_job_frame8_callback cb8, void *user) {
  if (!ctx) return OR3_ERR_INVALID_ARGUMENT;
  if (ctx->server) return fail(ctx, OR3_ERR_BUSY, "server already running");
  cudaSetDevice(ctx->device);
  if (cb8) {
    if (int e = ensure_gamma_table(ctx->device))
      return fail(ctx, OR3_ERR_CUDA, "gamma table: %s", cudaGetErrorString((cudaError_t)e));
  }
  Server *S = new Server();
  ctx->server = S;
  if (params) S->p = *params;
  S->cb = cb;
  S->cb8 = cb8;
  S->user = user;
  S->t0 = Clock::now();
  auto bail = [&](int rc) {
    destroy_server_state(ctx);
    return rc;
  };
  // resident scenes
  std::vector<DevScene> scenes;
  bool shadows = false;  // a resident scene has lights: NEE jobs queue shadow rays
  for (auto &kv : ctx->scenes) {
    S->scene_index[kv.first] = (uint32_t)scenes.size();
    scenes.push_back(kv.second->view);
    S->split = S->split || kv.second->has_split;
    shadows = shadows || kv.second->view.num_lights > 0 || kv.second->view.env_light != 0;
  }
  if (scenes.empty()) return bail(fail(ctx, OR3_ERR_NOT_FOUND, "upload scenes before starting the server"));
  // Glass: the queues hold kSplitQueueFactor rays per path, and a lane whose
  // wave a split overflows is rendered again in pieces that cannot overflow
  // (run_wave), so waves need not shrink to 1/8 of the queues.
  const uint64_t qfactor = S->split ? kSplitQueueFactor : 1;
  S->cap = S->p.wave_paths ? S->p.wave_paths : (S->split ? (1ull << 25) : (1ull << 24));
  S->cap = std::max<uint64_t>(S->cap, 1u << 16);
  S->cap = std::min<uint64_t>(S->cap, (1ull << 31) / qfactor);
  S->rays = S->cap * qfactor;
  const uint32_t maxa = S->p.max_active_jobs ? S->p.max_active_jobs : 64;
  S->cap_segs = 4 * maxa + 64;
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  int rc = ensure_queues(ctx, S->cap, S->rays);
  if (rc) return bail(rc);
  S->budget = S->p.hbm_budget_bytes ? S->p.hbm_budget_bytes : free_b / 2;
  if (cudaMalloc(&S->scenes_dev, scenes.size() * sizeof(DevScene)) != cudaSuccess ||
      cudaMalloc(&S->jobs_dev, maxa * sizeof(JobDev)) != cudaSuccess ||
      cudaMallocHost(&S->jobs_host, maxa * sizeof(JobDev)) != cudaSuccess)
    return bail(fail(ctx, OR3_ERR_OUT_OF_MEMORY, "server tables"));
  cudaEventCreate(&S->e0);
  cudaEventCreate(&S->e1);
  cudaEventCreateWithFlags(&S->ev_jobs, cudaEventDisableTiming);
  const int nl = (S->p.flags & OR3_SERVER_ONE_LANE) ? 1 : 3;
  S->lanes.resize(nl);
  for (int l = 0; l < nl; l++) {
    Server::Lane &L = S->lanes[l];
    if (l == 0) {
      L.st = ctx->stream;
      L.q = make_queues(ctx);
    } else {
      if ((rc = ensure_lane(ctx, l - 1, S->cap, S->rays, 1))) return bail(rc);
      L.st = ctx->xl[l - 1].stream;
      L.q = lane_queues(ctx->xl[l - 1]);
    }
    L.q.capacity = (uint32_t)std::min<uint64_t>(L.q.capacity, S->rays);  // the server's sizing
    if (cudaMalloc(&L.segs_dev, S->cap_segs * sizeof(Segment)) != cudaSuccess ||
        cudaMallocHost(&L.segs_host, S->cap_segs * sizeof(Segment)) != cudaSuccess ||
        cudaMalloc(&L.info_dev, sizeof(WaveInfo)) != cudaSuccess ||
        cudaMallocHost(&L.info_host, sizeof(WaveInfo)) != cudaSuccess ||
        cudaMallocHost(&L.hc, 4 * sizeof(uint32_t)) != cudaSuccess ||
        cudaEventCreateWithFlags(&L.ev, cudaEventDisableTiming) != cudaSuccess)
      return bail(fail(ctx, OR3_ERR_OUT_OF_MEMORY, "server lane tables"));
    cudaMemsetAsync(L.q.counters, 0, 16 * sizeof(uint32_t), L.st);
    cudaMemsetAsync(L.q.stats, 0, 8 * sizeof(unsigned long long), L.st);
  }
  cudaStream_t st = ctx->stream;
  if (cudaMemcpy(S->scenes_dev, scenes.data(), scenes.size() * sizeof(DevScene), cudaMemcpyHostToDevice) != cudaSuccess)
    return bail(fail(ctx, OR3_ERR_CUDA, "scene table upload"));
  // one captured bounce loop per lane (its queues and segment table)
  S->unroll = S->p.graph_bounces ? (int)S->p.graph_bounces : 8;
  S->unroll = std::max(2, std::min(S->unroll, 64));
  S->unroll += S->unroll & 1;
  for (Server::Lane &L : S->lanes) {
    const Batch b{S->scenes_dev, S->jobs_dev, L.segs_dev, L.info_dev};
    cudaGraph_t graph = nullptr;
    if (cudaStreamSynchronize(L.st) != cudaSuccess ||
        cudaStreamBeginCapture(L.st, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
      return bail(fail(ctx, OR3_ERR_CUDA, "graph capture"));
    for (int k = 0; k < S->unroll; k++) {
      const int in = k & 1;
      launch_extend_batch(b, L.q, in, ctx->num_sms * ctx->occ_extend, false, 0, L.st);
      if (shadows && !(S->p.flags & OR3_SERVER_UNSORTED_SHADE))  // material-sorted shade, as or3_render
        launch_shade_batch_sorted(b, L.q, in, true, ctx->num_sms * 8, ctx->num_sms * ctx->occ_shade_nee,
                                  ctx->num_sms * ctx->occ_shade, L.st);
      else
        launch_shade_batch(b, L.q, in, ctx->num_sms * (shadows ? ctx->occ_shade_nee : ctx->occ_shade), shadows,
                           L.st);
      if (shadows) launch_shadow_batch(b, L.q, ctx->num_sms * ctx->occ_extend, 0, L.st);
      launch_reset_count(L.q, in, L.st);
    }
    if (cudaStreamEndCapture(L.st, &graph) != cudaSuccess || cudaGraphInstantiate(&L.graph, graph, 0) != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return bail(fail(ctx, OR3_ERR_CUDA, "graph instantiate"));
    }
    cudaGraphDestroy(graph);
  }
  if (cudaStreamSynchronize(st) != cudaSuccess) return bail(fail(ctx, OR3_ERR_CUDA, "server start"));
  S->th = std::thread(worker, ctx);
  return OR3_OK;
}

int or3_server_start(or3_context *ctx, const or3_server_params *params, or3_job_frame_callback cb, void *user) {
  return server_start(ctx, params, cb, nullptr, user);
}

int or3_server_start8(or3_context *ctx, const or3_server_params *params, or3_job_frame8_callback cb, void *user) {
  if (!cb) return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "or3_server_start8 needs a frame callback");
  return server_start(ctx, params, nullptr, cb, user);
}

int or3_server_submit(or3_context *ctx, const or3_batch_job *job, uint64_t *id_out) {
  if (!ctx || !job) return OR3_ERR_INVALID_ARGUMENT;
  Server *S = ctx->server;
  if (!S) return fail(ctx, OR3_ERR_NOT_FOUND, "server not running");
  if (int v = validate_render(ctx, &job->camera, &job->params)) return v;
  std::lock_guard<std::mutex> lk(S->mu);
  if (S->error) return fail(ctx, S->error, "server stopped after an error: %s", S->error_msg.c_str());
  auto it = S->scene_index.find(job->scene);
  if (it == S->scene_index.end()) return fail(ctx, OR3_ERR_NOT_FOUND, "scene %d was not resident at start", job->scene);
  SJob *j = new SJob();
  j->id = S->next_id++;
  j->job = *job;
  j->scene_slot = it->second;
  j->ss2 = (uint32_t)(job->params.supersamples * job->params.supersamples);
  j->per_sample = (uint64_t)job->camera.width * job->camera.height * j->ss2;
  j->samples = job->params.min_samples +
               (job->params.max_samples - job->params.min_samples) / job->params.step_samples * job->params.step_samples;
  j->total = (uint64_t)j->samples * j->per_sample;
  const uint64_t every = S->p.frame_every_samples ? S->p.frame_every_samples : 16;
  j->next_frame = every * j->per_sample;
  j->bytes = (size_t)job->camera.width * job->camera.height * 3 * sizeof(double) * 2;
  j->t_submit = S->now();
  S->all[j->id] = j;
  S->pending.push_back(j);
  S->submitted++;
  if (id_out) *id_out = j->id;
  S->cv.notify_all();
  return OR3_OK;
}

int or3_server_poll(or3_context *ctx, uint64_t id, or3_job_status *out) {
  if (!ctx || !out) return OR3_ERR_INVALID_ARGUMENT;
  Server *S = ctx->server;
  if (!S) return fail(ctx, OR3_ERR_NOT_FOUND, "server not running");
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->all.find(id);
  if (it == S->all.end()) return fail(ctx, OR3_ERR_NOT_FOUND, "job %llu not found", (unsigned long long)id);
  const SJob &j = *it->second;
  out->state = j.state;
  out->samples_done = j.samples_done;
  out->submit_s = j.t_submit;
  out->admit_s = j.t_admit;
  out->first_frame_s = j.t_first;
  out->done_s = j.t_done;
  return OR3_OK;
}

int or3_server_cancel(or3_context *ctx, uint64_t id) {
  if (!ctx) return OR3_ERR_INVALID_ARGUMENT;
  Server *S = ctx->server;
  if (!S) return fail(ctx, OR3_ERR_NOT_FOUND, "server not running");
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->all.find(id);
  if (it == S->all.end()) return fail(ctx, OR3_ERR_NOT_FOUND, "job %llu not found", (unsigned long long)id);
  it->second->cancel = true;
  S->cv.notify_all();
  return OR3_OK;
}

int or3_server_drain(or3_context *ctx, double timeout_s) {
  if (!ctx) return OR3_ERR_INVALID_ARGUMENT;
  Server *S = ctx->server;
  if (!S) return fail(ctx, OR3_ERR_NOT_FOUND, "server not running");
  std::unique_lock<std::mutex> lk(S->mu);
  const auto deadline = Clock::now() + std::chrono::duration<double>(timeout_s > 0 ? timeout_s : 1e9);
  while (!(S->pending.empty() && S->active.empty()) && !S->error) {
    if (S->idle.wait_until(lk, deadline) == std::cv_status::timeout)
      return fail(ctx, OR3_ERR_BUSY, "drain timed out with %zu queued and %zu running jobs", S->pending.size(),
                  S->active.size());
  }
  if (S->error) return fail(ctx, S->error, "server stopped after an error: %s", S->error_msg.c_str());
  return OR3_OK;
}

int or3_server_get_stats(or3_context *ctx, or3_server_stats *out) {
  if (!ctx || !out) return OR3_ERR_INVALID_ARGUMENT;
  Server *S = ctx->server;
  if (!S) return fail(ctx, OR3_ERR_NOT_FOUND, "server not running");
  std::lock_guard<std::mutex> lk(S->mu);
  std::vector<double> lat, queue, first;
  for (auto &kv : S->all) {
    const SJob &j = *kv.second;
    if (j.state == OR3_JOB_DONE) {
      lat.push_back(j.t_done - j.t_submit);
      queue.push_back(j.t_admit - j.t_submit);
      first.push_back(j.t_first - j.t_submit);
    }
  }
  *out = or3_server_stats{};
  out->jobs_submitted = S->submitted;
  out->jobs_done = S->finished;
  out->jobs_cancelled = S->cancelled;
  out->camera_paths = S->paths;
  out->waves = S->waves;
  out->waves_rerun = S->waves_rerun;
  out->busy_s = S->busy_s;
  out->device_ms = S->device_ms;
  out->latency_p50_s = percentile(lat, 0.5);
  out->latency_p99_s = percentile(lat, 0.99);
  out->queue_p50_s = percentile(queue, 0.5);
  out->queue_p99_s = percentile(queue, 0.99);
  out->first_frame_p50_s = percentile(first, 0.5);
  out->peak_active_jobs = S->peak_active;
  out->peak_budget_bytes = S->peak_in_use;
  return OR3_OK;
}

int or3_server_get_moments(or3_context *ctx, uint64_t id, double *sum, double *sumsq, size_t capacity,
                           uint64_t *count_out) {
  if (!ctx) return OR3_ERR_INVALID_ARGUMENT;
  Server *S = ctx->server;
  if (!S) return fail(ctx, OR3_ERR_NOT_FOUND, "server not running");
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->all.find(id);
  if (it == S->all.end()) return fail(ctx, OR3_ERR_NOT_FOUND, "job %llu not found", (unsigned long long)id);
  const SJob &j = *it->second;
  if (j.state != OR3_JOB_DONE || j.host_sum.empty())
    return fail(ctx, OR3_ERR_NOT_FOUND, "job %llu has no kept moments (finished with OR3_SERVER_KEEP_MOMENTS?)",
                (unsigned long long)id);
  if (capacity < j.host_sum.size()) return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "moments need %zu doubles", j.host_sum.size());
  if (sum) std::memcpy(sum, j.host_sum.data(), j.host_sum.size() * sizeof(double));
  if (sumsq) std::memcpy(sumsq, j.host_sumsq.data(), j.host_sumsq.size() * sizeof(double));
  if (count_out) *count_out = (uint64_t)j.samples * j.ss2;
  return OR3_OK;
}

int or3_server_stop(or3_context *ctx) {
  if (!ctx) return OR3_ERR_INVALID_ARGUMENT;
  if (!ctx->server) return OR3_OK;
  destroy_server_state(ctx);
  return OR3_OK;
}

}  // extern "C"
