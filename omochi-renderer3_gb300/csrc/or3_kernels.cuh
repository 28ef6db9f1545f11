// or3_kernels.cuh -- launch interface between the host runtime and the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "or3_device.cuh"

namespace or3 {

// Camera basis (Camera::Camera, src/renderer/Camera.h:12-43), built in double on
// the host and used in FP32 on the device.
struct Camera32 {
  float pos[3];
  float center[3];
  float xaxis[3];  // scaled by the screen width in world units
  float yaxis[3];  // scaled by the screen height in world units
  float focal;
  float aperture;  // 0 = pinhole
};

struct RenderConst {
  Camera32 cam;
  uint32_t W, H, ss, ss2;
  int32_t nee, rr_min_depth, max_depth, pad;
  uint32_t seed_lo, seed_hi;
};

// One wave = a contiguous range of camera paths g in [g_first, g_first + num_paths)
// with g = ((s * H + y) * W + x) * ss2 + sub.  Waves never straddle passes.
struct Wave {
  uint64_t g_first;
  uint32_t num_paths;
  uint32_t pass_first;  // first sample index of the pass (lens sample key)
  uint32_t pix0, npix;  // pixel range touched (camera order y*W+x)
  uint32_t ns;          // samples per pixel in the wave
  uint32_t pad;
};

// Ray queues in HBM (structure of arrays, ping-pong).
//   orig: (o.xyz, path index in wave)   dir: (d.xyz, depth | leaf << 16 | spec << 24)
//   beta: (throughput.xyz, segment)     hits: (t, record, u, v)
// Shadow queue (next-event estimation), filled by shade, drained by k_shadow:
//   sorig: (o.xyz, path index)  sdir: (d.xyz, tmax)  scontrib: (radiance if unoccluded, segment)
struct Queues {
  float4 *orig[2];
  float4 *dir[2];
  float4 *beta[2];
  float4 *hits;
  float4 *pathL;  // per camera path radiance of the wave
  float4 *sorig, *sdir, *scontrib;
  uint32_t *slist;            // sorted shade: indices of this bounce's hits by material class
                              // (light-sampling surfaces from the front, the rest from the back);
                              // null where the sorted shade is not used
  uint32_t *counters;         // [0],[1] queue lengths, [2] error bits, [3] shadow queue length,
                              // [4],[5] extend fetch counters, [6] shadow fetch counter,
                              // [10],[11] sorted shade: front and back list lengths
  unsigned long long *stats;  // [0] extension rays [1] shadow rays [2] bounces [3] nodes [4] tris [5] spheres
  uint32_t capacity;          // entries per queue (the shadow queue too)
  uint32_t pad;
};

// dir.w bit: the ray leaves a mirror/glass vertex (no light sample was taken
// there, so next-event estimation still counts the emission it reaches)
constexpr uint32_t kMetaSpec = 1u << 24;

constexpr uint32_t kErrStack = 1u;
constexpr uint32_t kErrQueue = 2u;
// Ray queue capacity per camera path of a wave where glass can split paths.
// A split (depth <= 2) can make up to 8 rays of one path; a wave whose queue
// overflows is rendered again in sub-waves of capacity / 8 paths, which
// cannot overflow, and the same paths give the same image.
constexpr uint32_t kSplitQueueFactor = 2;

// ---- batched form: one wave holds path ranges ("segments") of many jobs.
// A job is one render (scene, camera, sample budget); its camera paths keep
// the plain render's numbering and RNG keys, so a job renders the same paths
// alone or in a batch.  Rays carry their segment index in beta.w.
struct JobDev {
  RenderConst rc;
  uint32_t scene;     // index into Batch::scenes
  uint32_t pad;
  double *sum;        // the job's per-pixel sums (3 per pixel, camera order y*W+x)
  double *sumsq;
};

struct Segment {
  uint64_t g_first;      // first job path index (a multiple of ss2)
  uint32_t job;
  uint32_t wave_first;   // wave path index of the segment's first path
  uint32_t count;        // paths (a multiple of ss2)
  uint32_t pass_first;   // first sample of the pass (lens key)
  uint32_t group_first;  // first pixel-sample group of the segment in the wave
  uint32_t pad;
};

// Wave description read by the kernels from device memory, so one captured
// graph of the bounce loop serves every wave.
struct WaveInfo {
  uint32_t nseg;
  uint32_t ngroups;   // pixel-sample groups (ss2 paths each) in the wave
  uint32_t num_paths;
  uint32_t pad;
};

struct Batch {
  const DevScene *scenes;
  const JobDev *jobs;
  const Segment *segs;
  const WaveInfo *info;
};

// The device-driven batch loop: every planned wave of the batch sits in one
// table, and the lanes' looping graphs take waves from a shared head counter
// until none is left (no host round trip between waves or bounces).
struct WaveDesc {
  uint32_t seg_first;  // the wave's first entry in the batch's segment table
  uint32_t nseg;
  uint32_t ngroups;
  uint32_t num_paths;
};

struct BatchLoop {
  uint32_t next_wave;  // head of the shared wave queue
  uint32_t nwaves;
  uint32_t abort;      // bit 0: a wave's bounce loop passed max_iters; bit 1: a kernel set error bits
  uint32_t max_iters;  // loop iterations one wave may take
  uint32_t nfail;      // waves whose ray queue a glass split overflowed (their indices in the fail list)
  uint32_t fail_cap;
  struct Lane {
    uint32_t active;   // the lane holds a wave
    uint32_t fresh;    // the wave was taken in this iteration: camera rays pending
    uint32_t iters;    // iterations of the current wave
    uint32_t waves;    // waves completed
    unsigned long long paths;  // camera paths completed
    uint32_t wave;     // the wave the lane holds
    uint32_t pad;
  } lane[3];
};

void launch_raygen_batch(const Batch &b, uint32_t num_paths, const Queues &q, int out, cudaStream_t st);
// One iteration of a lane's device loop around its bounces: take a wave when
// idle (ending the loop through `h` when the queue is empty), then camera
// rays for a fresh wave; after the bounces, accumulate a finished wave and
// free the lane.  `segs` / `info` are the lane's (b.segs, b.info).
void launch_wave_take(BatchLoop *L, int lane, const WaveDesc *waves, const Segment *segs_all, Segment *segs,
                      WaveInfo *info, const uint32_t *counters, cudaGraphConditionalHandle h, cudaStream_t st);
void launch_raygen_batch_loop(const Batch &b, const Queues &q, const BatchLoop *L, int lane, int grid,
                              cudaStream_t st);
void launch_accumulate_batch_loop(const Batch &b, const Queues &q, const BatchLoop *L, int lane, int grid,
                                  cudaStream_t st);
// fail: the overflowed waves' indices (L->fail_cap entries); their queue
// error bit is cleared and they count as neither done nor accumulated.
void launch_wave_finish(BatchLoop *L, int lane, const WaveInfo *info, uint32_t *counters, uint32_t *fail,
                        cudaStream_t st);
void launch_extend_batch(const Batch &b, const Queues &q, int in, int grid, bool count, int variant,
                         cudaStream_t st);
// nee: some job samples lights (the light-sampling instance of the kernel)
void launch_shade_batch(const Batch &b, const Queues &q, int in, int grid, bool nee, cudaStream_t st);
void launch_accumulate_batch(const Batch &b, uint32_t max_groups, const Queues &q, cudaStream_t st);

struct LaunchCfg {
  int grid_extend, grid_shade, grid_raygen, grid_accum;
  int block;
};

// host launchers (or3_kernels.cu)
void launch_raygen(const RenderConst &rc, const Wave &w, const Queues &q, int out, int grid, int block,
                   cudaStream_t st);
// variant: 0 one thread per ray over a grid-stride loop, 1 and 2 persistent
// lane-refilled traversal (see persistent_trace)
// Maps OR3_TUNE_EXTEND_MASK to a kernel variant (0 = default = 2, 3 = grid-stride).
inline int extend_variant(uint32_t tuning) {
  const uint32_t v = tuning & 0x7u;
  return v == 0 ? 2 : v == 3 ? 0 : (int)v;  // 4, 5: refill thresholds; 6: quantised nodes; 7: nearest first
}
void launch_extend(const DevScene &S, const Queues &q, int in, int grid, int block, int smem_nodes, bool count,
                   int variant, cudaStream_t st);
// nee4: the light-sampling instance limited to 64 registers (4 blocks per SM)
// nee4: the light-sampling instance at 4 blocks/SM; blk: block-aggregated
// queue appends (256-thread blocks)
void launch_shade(const DevScene &S, const RenderConst &rc, const Wave &w, const Queues &q, int in,
                  int grid, int block, cudaStream_t st, bool nee4 = false, bool blk = false);
void launch_reset_count(const Queues &q, int which, cudaStream_t st);
// a += b, b = 0 over n doubles (sums and sums of squares)
// Material-sorted shade (k_classify, then k_shade_list per class list):
// replaces launch_shade when chosen; 2 or 3 launches.
void launch_shade_sorted(const DevScene &S, const RenderConst &rc, const Wave &w, const Queues &q, int in,
                         int grid_classify, int grid_nee, int grid_plain, cudaStream_t st);
// The same for the batched and served forms (nee: the batch's light-sampling
// instance, as launch_shade_batch picks it).
void launch_shade_batch_sorted(const Batch &b, const Queues &q, int in, bool nee, int grid_classify, int grid_nee,
                               int grid_plain, cudaStream_t st);
void launch_merge_sums(size_t n, double *a, double *aq, double *b, double *bq, int max_grid, cudaStream_t st);
// any-hit test of the shadow queue; unoccluded samples add to their path's radiance
void launch_shadow(const DevScene &S, const Queues &q, int grid, bool unsorted, bool quantised, cudaStream_t st,
                   bool wide8 = false, bool refill8 = false);
void launch_shadow_batch(const Batch &b, const Queues &q, int grid, int variant, cudaStream_t st);
void launch_accumulate(const Queues &q, const Wave &w, uint32_t ss2, double *sum, double *sumsq, int grid,
                       int block, cudaStream_t st);
// After launch_accumulate: files the wave in fail when its queue overflowed
// (and clears the bit); fail[0] counts, fail[1..cap] hold wave indices.
void launch_wave_check(const Queues &q, uint32_t *fail, uint32_t cap, uint32_t wave, cudaStream_t st);
void launch_frame(const double *sum, uint32_t W, uint32_t H, int layout, double scale, double *out,
                  cudaStream_t st);
void launch_moments(const double *sum, const double *sumsq, uint32_t W, uint32_t H, double *sum_out,
                    double *sumsq_out, cudaStream_t st);
// counters: the context's counter block ([2] error bits, [8] query fetch counter)
void launch_trace_closest(const DevScene &S, size_t n, const float *orig, const float *dir, int32_t *prim,
                          float *t, float *normal, uint32_t *counters, cudaStream_t st);
void launch_env_sample(const DevScene &S, uint32_t n, const float *dir, float *rgb, cudaStream_t st);
void launch_texture_sample(const DevScene &S, int tex, uint32_t n, const float *uv, float *rgb, cudaStream_t st);
void launch_trace_occluded(const DevScene &S, size_t n, const float *orig, const float *dir,
                           const float *tmax, uint8_t *occ, uint32_t *counters, cudaStream_t st);
void set_query_grid(int grid);

// or3_image.cu: image output/input and the environment CDF
int ensure_gamma_table(int device);  // per device, before launch_encode_rgb8 with gamma; 0 or a cudaError_t
void launch_encode_rgb8(const double *in, size_t nvals, int gamma, uint8_t *out, cudaStream_t st);
void launch_encode_rgbe(const double *in, size_t npix, uint8_t *out, cudaStream_t st);
void launch_decode_rgbe(const uint8_t *in, size_t npix, float *out, cudaStream_t st);
// rows: H + 1 doubles of scratch; rows[H] receives the map's total weight.
// gmarg [H + 1] and gcond [H * (W + 1)]: guide tables of marg and of each cond row.
void launch_env_cdf(const float *env, uint32_t W, uint32_t H, float *marg, float *cond, double *rows,
                    uint32_t *gmarg, uint32_t *gcond, cudaStream_t st);

// or3_noalloc.cu: the bounce loop on the static scratch array
int render_paths_noalloc(const DevScene &S, bool has_split, const RenderConst &rc, uint64_t first,
                         uint32_t num_paths, uint32_t pass_first, int device, int grid_ext, int grid_sh,
                         float *out, cudaStream_t st, std::string *err);

// kernel handles for occupancy queries
const void *kernel_extend_ptr();
const void *kernel_shade_ptr(bool batch, bool nee);

}  // namespace or3
