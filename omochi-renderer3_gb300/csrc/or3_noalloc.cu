// or3_noalloc.cu -- or3_render_paths_noalloc: the wavefront path loop on a
// fixed, statically allocated scratch area instead of cudaMalloc'd queues.
//
// Some callers cannot allocate device memory when they render: engines that
// hand the whole device to their own memory pool up front (cudaMalloc would
// fail or fragment the pool), and frame loops with a latency budget
// (cudaMalloc/cudaFree can synchronise the device).  For them this entry
// point keeps every queue of the bounce loop in one file-scope __device__
// array, sized for kMaxPaths camera paths; the scene must already be
// resident (or3_scene_upload, done at set-up) and the caller passes the
// output buffer.  It is called from ordinary host code and blocks: it
// launches kernels, copies counters to the host and synchronises its stream,
// none of which CUDA allows inside a host function enqueued on a stream.
#include <cuda_runtime.h>

#include <mutex>

#include "or3.h"
#include "or3_kernels.cuh"

namespace or3 {
namespace {

constexpr uint32_t kMaxPaths = OR3_NOALLOC_MAX_PATHS;
constexpr uint32_t kMaxRays = 8u * kMaxPaths;  // glass splits at depth <= 2: <= 8 rays per path

struct Scratch {
  float4 orig[2][kMaxRays];
  float4 dir[2][kMaxRays];
  float4 beta[2][kMaxRays];
  float4 hits[kMaxRays];
  float4 pathL[kMaxPaths];
  float4 sorig[kMaxRays], sdir[kMaxRays], scontrib[kMaxRays];  // shadow queue
  uint32_t counters[16];
  unsigned long long stats[8];
};

// Every GPU that loads libor3.so holds this array (about 5.3 MB) until exit.
// All calls share it and it keeps the last call's contents.
static __device__ __align__(256) Scratch g_scratch;

constexpr int kMaxDevices = 64;
std::mutex g_mu;
Scratch *g_addr[kMaxDevices] = {};

__global__ void k_copy_radiance(uint32_t n, float *out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 L = g_scratch.pathL[i];
  out[3 * i] = L.x;
  out[3 * i + 1] = L.y;
  out[3 * i + 2] = L.z;
}

// Per-device set-up: the array's device address, taken once with the device
// current.  (In host code `g_scratch` names a host-side stand-in, not device
// memory, so it must never be passed to a kernel.)  The address is cached for
// the life of the process; a cudaDeviceReset (a new primary context) would
// make it stale, which the entry point's documentation states.
cudaError_t scratch_for(int device, Scratch **out) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[device]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess) return e;
    g_addr[device] = static_cast<Scratch *>(p);
  }
  *out = g_addr[device];
  return cudaSuccess;
}

}  // namespace

int render_paths_noalloc(const DevScene &S, bool has_split, const RenderConst &rc, uint64_t first,
                         uint32_t num_paths, uint32_t pass_first, int device, int grid_ext, int grid_sh,
                         float *out, cudaStream_t st, std::string *err) {
  (void)has_split;
  Scratch *sc = nullptr;
  cudaError_t e = scratch_for(device, &sc);
  if (e != cudaSuccess) {
    *err = std::string("no-alloc scratch set-up: ") + cudaGetErrorString(e);
    return OR3_ERR_CUDA;
  }
  Queues q{};
  for (int k = 0; k < 2; k++) {
    q.orig[k] = sc->orig[k];
    q.dir[k] = sc->dir[k];
    q.beta[k] = sc->beta[k];
  }
  q.hits = sc->hits;
  q.pathL = sc->pathL;
  q.sorig = sc->sorig;
  q.sdir = sc->sdir;
  q.scontrib = sc->scontrib;
  q.counters = sc->counters;
  q.stats = sc->stats;
  q.capacity = kMaxRays;
  // queue lengths, error bits and statistics start at zero; pathL is cleared by ray-gen
  e = cudaMemsetAsync(sc->counters, 0, sizeof(sc->counters) + sizeof(sc->stats), st);
  if (e != cudaSuccess) {
    *err = std::string("no-alloc clear: ") + cudaGetErrorString(e);
    return OR3_ERR_CUDA;
  }
  Wave w{};
  w.g_first = first;
  w.num_paths = num_paths;
  w.pass_first = pass_first;
  launch_raygen(rc, w, q, 0, 0, 256, st);
  int in = 0;
  uint32_t count = num_paths, errbits = 0;
  const bool shadows = rc.nee && (S.num_lights > 0 || S.env_light != 0);
  // bounces in chunks without a host round trip (kernels read their queue
  // length on the device): the whole path under a depth bound of at most 32
  const bool whole = rc.max_depth > 0 && rc.max_depth <= 32;
  const int chunk = whole ? rc.max_depth : 8;
  for (int chunks = 0; count > 0 && chunks < 1 << 20; chunks++) {
    for (int b = 0; b < chunk; b++) {
      launch_extend(S, q, in, grid_ext, 256, 0, false, extend_variant(0), st);
      launch_shade(S, rc, w, q, in, grid_sh, 256, st);
      if (shadows) launch_shadow(S, q, grid_ext, false, false, st);
      launch_reset_count(q, in, st);
      in ^= 1;
    }
    uint32_t hc[3] = {0, 0, 0};
    e = cudaMemcpyAsync(hc, sc->counters, sizeof(hc), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      *err = std::string("no-alloc bounce: ") + cudaGetErrorString(e);
      return OR3_ERR_CUDA;
    }
    count = whole ? 0u : hc[in];
    errbits = hc[2];
    if (errbits) break;
  }
  if (errbits) {
    *err = "kernel reported error bits in the no-alloc path";
    return OR3_ERR_DEVICE_REPORTED;
  }
  k_copy_radiance<<<(num_paths + 255) / 256, 256, 0, st>>>(num_paths, out);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    *err = std::string("no-alloc output: ") + cudaGetErrorString(e);
    return OR3_ERR_CUDA;
  }
  return OR3_OK;
}

}  // namespace or3
