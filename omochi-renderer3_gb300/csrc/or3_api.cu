// or3_api.cu -- the C ABI (include/or3.h): contexts, scene upload, render loop,
// ray-set queries.  Host side of the GB300 path-tracing hot path.
#include <cuda_runtime.h>

#include <algorithm>
#include <thread>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "bvh_build.h"
#include "bvh_build_gpu.h"
#include "or3.h"
#include "or3_internal.h"
#include "or3_kernels.cuh"

using namespace or3;

namespace {

template <class T>
int dev_upload(or3_context *ctx, SceneGPU *sg, const std::vector<T> &v, const T **out) {
  *out = nullptr;
  if (v.empty()) return OR3_OK;
  void *p = nullptr;
  OR3_CUDA(ctx, cudaMallocFromPoolAsync(&p, v.size() * sizeof(T), ctx->scene_pool, ctx->stream));
  sg->pool_allocs.push_back(p);
  OR3_CUDA(ctx, cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
  sg->info.device_bytes += v.size() * sizeof(T);
  *out = static_cast<const T *>(p);
  return OR3_OK;
}

template <class T>
int dev_alloc(or3_context *ctx, SceneGPU *sg, T **out, size_t n) {
  *out = nullptr;
  void *p = nullptr;
  OR3_CUDA(ctx, cudaMallocFromPoolAsync(&p, std::max<size_t>(n, 1) * sizeof(T), ctx->scene_pool, ctx->stream));
  sg->pool_allocs.push_back(p);
  sg->info.device_bytes += n * sizeof(T);
  *out = static_cast<T *>(p);
  return OR3_OK;
}

// Device buffers that live only during one upload.
// Temporaries of one upload, stream-ordered from the context's pool (freed
// on the stream when the upload returns).
struct DeviceTemps {
  or3_context *ctx = nullptr;
  std::vector<void *> p;
  explicit DeviceTemps(or3_context *c) : ctx(c) {}
  template <class T>
  int alloc(or3_context *c, T **out, size_t n) {
    *out = nullptr;
    void *q = nullptr;
    OR3_CUDA(c, cudaMallocFromPoolAsync(&q, std::max<size_t>(n, 1) * sizeof(T), c->tmp_pool, c->stream));
    p.push_back(q);
    *out = static_cast<T *>(q);
    return OR3_OK;
  }
  ~DeviceTemps() {
    for (void *q : p) cudaFreeAsync(q, ctx->stream);
  }
};

// The scene's 8-wide tree (WideNode8F) for OR3_TUNE_WIDE8, made on the host
// from its 4-wide FP32-box nodes the first time it is asked for.
int ensure_wide8(or3_context *ctx, SceneGPU *sg) {
  if (sg->view.fnodes8 || sg->view.num_nodes == 0) return OR3_OK;
  std::vector<WideNodeF> n4(sg->view.num_nodes);
  OR3_CUDA(ctx, cudaMemcpy(n4.data(), sg->view.fnodes, n4.size() * sizeof(WideNodeF), cudaMemcpyDeviceToHost));
  std::vector<WideNode8F> n8;
  int pushes = 0;
  if (!make_wide8_nodes(n4, n8, &pushes))
    return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "8-wide tree: a ray could need %d stack entries (limit %d)", pushes,
                kStackSize8);
  void *d = nullptr;
  OR3_CUDA(ctx, cudaMalloc(&d, n8.size() * sizeof(WideNode8F)));
  sg->allocs.push_back(d);
  OR3_CUDA(ctx, cudaMemcpy(d, n8.data(), n8.size() * sizeof(WideNode8F), cudaMemcpyHostToDevice));
  sg->view.fnodes8 = static_cast<const float4 *>(d);
  return OR3_OK;
}

// Callers make sure no kernel still reads the scene (the pool's memory is
// handed out again in the stream's order).
void free_scene(SceneGPU *sg) {
  for (void *p : sg->pool_allocs) cudaFreeAsync(p, sg->stream);
  for (void *p : sg->allocs) cudaFree(p);
  delete sg;
}

float down(double x) {
  float f = (float)x;
  if ((double)f > x) f = std::nextafter(f, -INFINITY);
  return f;
}
float up(double x) {
  float f = (float)x;
  if ((double)f < x) f = std::nextafter(f, INFINITY);
  return f;
}

int check_layers(or3_context *ctx, const or3_scene_desc *d, const uint32_t *lay, const char *what, uint32_t i) {
  if (lay[1] == 0 || (uint64_t)lay[0] + lay[1] > d->num_layers)
    return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "%s %u: layer range [%u,+%u) outside %u layers", what, i, lay[0],
                lay[1], d->num_layers);
  return OR3_OK;
}

uint32_t layer_flags(const or3_scene_desc *d, const uint32_t *lay) {
  uint32_t f = 0;
  for (uint32_t k = 0; k < lay[1]; k++) {
    const or3_material &m = d->materials[d->layer_material[lay[0] + k]];
    if (m.texture >= 0) f |= kFlagTexturedUV;
    if (m.emission[0] * m.emission[0] + m.emission[1] * m.emission[1] + m.emission[2] * m.emission[2] != 0)
      f |= kFlagEmissive;
  }
  return f;
}

// Probability that the layer roulette (PathTracer.cpp:370-382) picks layer k.
double layer_prob(const or3_scene_desc *d, const uint32_t *lay, uint32_t k) {
  double lo = 0;
  for (uint32_t j = 0; j < k; j++) lo += d->layer_rate[lay[0] + j];
  lo = std::min(1.0, std::max(0.0, lo));
  double hi = k + 1 == lay[1] ? 1.0 : lo + d->layer_rate[lay[0] + k];
  hi = std::min(1.0, std::max(0.0, hi));
  return hi > lo ? hi - lo : 0.0;
}

constexpr double kPiD = 3.14159265358979323846264338327950288419716939;

// Next-event light tables.  Local lights are the in-BVH objects with an
// emissive layer (triangles, then spheres, in description order), chosen with
// probability proportional to area * sum(p_layer * |emission|) (the power
// measure of SphereLight::TotalPower, src/renderer/SphereLight.h:71-78).  The
// environment is sampled through a piecewise-constant marginal/conditional CDF
// over max(r, g, b) * sin(theta) per texel (the reference's importance map,
// src/renderer/IBL.h:104-189, is a stub; the CDF is built on the device), or
// cosine-weighted about the receiver's normal when it is a constant background.
struct LightTables {
  std::vector<LightDev> lights;
  std::vector<float> cdf, pdf;
  int env_light = 0;
  float env_prob = 0.f;
};

void build_light_tables(const or3_scene_desc *d, const float *geom, LightTables &T) {
  const uint32_t nt = d->num_triangles, nsph = d->num_spheres;
  std::vector<double> power;
  double total = 0;
  auto add_light = [&](const uint32_t *lay, double area, LightDev L) {
    double le[3] = {0, 0, 0}, mag = 0;
    for (uint32_t k = 0; k < lay[1]; k++) {
      const double p = layer_prob(d, lay, k);
      const double *e = d->materials[d->layer_material[lay[0] + k]].emission;
      for (int a = 0; a < 3; a++) le[a] += e[a] * p;
      mag += p * std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
    }
    for (int a = 0; a < 3; a++) L.le[a] = (float)le[a];
    T.lights.push_back(L);
    power.push_back(area * mag);
    total += area * mag;
  };
  for (uint32_t i = 0; i < nt; i++) {
    const uint32_t *lay = d->tri_layers + 2 * i;
    if (!(layer_flags(d, lay) & kFlagEmissive)) continue;
    const double *v = d->tri_vertices + 9 * (size_t)i;
    const double e1[3] = {v[3] - v[0], v[4] - v[1], v[5] - v[2]};
    const double e2[3] = {v[6] - v[0], v[7] - v[1], v[8] - v[2]};
    const double c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    LightDev L{};
    const float *g = &geom[12 * (size_t)i];
    for (int a = 0; a < 3; a++) {
      L.p[a] = g[a];
      L.e1[a] = g[3 + a];
      L.e2[a] = g[6 + a];
    }
    L.kind = kLightTriangle;
    add_light(lay, 0.5 * std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]), L);
  }
  for (uint32_t j = 0; j < nsph; j++) {
    const uint32_t *lay = d->sphere_layers + 2 * j;
    if (!(layer_flags(d, lay) & kFlagEmissive)) continue;
    const double r = d->spheres[4 * (size_t)j + 3];
    LightDev L{};
    const float *g = &geom[12 * (size_t)(nt + j)];
    for (int a = 0; a < 3; a++) L.p[a] = g[a];
    L.r = g[3];
    L.kind = kLightSphere;
    add_light(lay, 4 * kPiD * r * r, L);
  }
  if (!(total > 0)) T.lights.clear();
  const size_t nl = T.lights.size();
  T.cdf.resize(nl);
  T.pdf.resize(nl);
  double run = 0;
  for (size_t k = 0; k < nl; k++) {
    run += power[k];
    T.cdf[k] = k + 1 == nl ? 1.0f : (float)(run / total);
    T.pdf[k] = (float)(power[k] / total);
  }
  if (!d->env_rgb && !d->env_rgbe) {
    const double *b = d->background;
    T.env_light = (b[0] * b[0] + b[1] * b[1] + b[2] * b[2]) != 0 ? 2 : 0;
  }
  // an equirect map's CDF is built on the device (launch_env_cdf); the upload
  // sets env_light = 1 there once the map's total weight is known
}

}  // namespace

namespace or3 {

// The ray queues are large: memory the pools keep from released scenes and
// finished uploads goes back to the device before they grow.
static void trim_pools(or3_context *ctx) {
  cudaStreamSynchronize(ctx->stream);
  if (ctx->tmp_pool) cudaMemPoolTrimTo(ctx->tmp_pool, 0);
  if (ctx->scene_pool) cudaMemPoolTrimTo(ctx->scene_pool, 0);
}

int ensure_queues(or3_context *ctx, size_t paths, size_t rays) {
  if (paths <= ctx->cap_paths && rays <= ctx->cap_rays) return OR3_OK;
  for (int k = 0; k < 2; k++) {
    cudaFree(ctx->qorig[k]);
    cudaFree(ctx->qdir[k]);
    cudaFree(ctx->qbeta[k]);
    ctx->qorig[k] = ctx->qdir[k] = ctx->qbeta[k] = nullptr;
  }
  cudaFree(ctx->hits);
  cudaFree(ctx->pathL);
  cudaFree(ctx->sorig);
  cudaFree(ctx->sdir);
  cudaFree(ctx->scontrib);
  cudaFree(ctx->slist);
  ctx->hits = ctx->pathL = ctx->sorig = ctx->sdir = ctx->scontrib = nullptr;
  ctx->slist = nullptr;
  ctx->cap_paths = ctx->cap_rays = 0;
  trim_pools(ctx);
  for (int k = 0; k < 2; k++) {
    OR3_CUDA(ctx, cudaMalloc(&ctx->qorig[k], rays * sizeof(float4)));
    OR3_CUDA(ctx, cudaMalloc(&ctx->qdir[k], rays * sizeof(float4)));
    OR3_CUDA(ctx, cudaMalloc(&ctx->qbeta[k], rays * sizeof(float4)));
  }
  OR3_CUDA(ctx, cudaMalloc(&ctx->hits, rays * sizeof(float4)));
  OR3_CUDA(ctx, cudaMalloc(&ctx->pathL, paths * sizeof(float4)));
  OR3_CUDA(ctx, cudaMalloc(&ctx->sorig, rays * sizeof(float4)));
  OR3_CUDA(ctx, cudaMalloc(&ctx->sdir, rays * sizeof(float4)));
  OR3_CUDA(ctx, cudaMalloc(&ctx->scontrib, rays * sizeof(float4)));
  OR3_CUDA(ctx, cudaMalloc(&ctx->slist, rays * sizeof(uint32_t)));
  ctx->cap_paths = paths;
  ctx->cap_rays = rays;
  return OR3_OK;
}

int ensure_pixels(or3_context *ctx, size_t pixels, size_t frame_doubles) {
  if (pixels > ctx->cap_pixels) {
    cudaFree(ctx->pix_sum);
    cudaFree(ctx->pix_sumsq);
    ctx->pix_sum = ctx->pix_sumsq = nullptr;
    ctx->cap_pixels = 0;
    OR3_CUDA(ctx, cudaMalloc(&ctx->pix_sum, pixels * 3 * sizeof(double)));
    OR3_CUDA(ctx, cudaMalloc(&ctx->pix_sumsq, pixels * 3 * sizeof(double)));
    ctx->cap_pixels = pixels;
  }
  if (frame_doubles > ctx->cap_frame) {
    cudaFree(ctx->frame_dev);
    ctx->frame_dev = nullptr;
    ctx->cap_frame = 0;
    OR3_CUDA(ctx, cudaMalloc(&ctx->frame_dev, frame_doubles * sizeof(double)));
    ctx->cap_frame = frame_doubles;
  }
  return OR3_OK;
}

Queues make_queues(or3_context *ctx) {
  Queues q{};
  for (int k = 0; k < 2; k++) {
    q.orig[k] = ctx->qorig[k];
    q.dir[k] = ctx->qdir[k];
    q.beta[k] = ctx->qbeta[k];
  }
  q.hits = ctx->hits;
  q.pathL = ctx->pathL;
  q.sorig = ctx->sorig;
  q.sdir = ctx->sdir;
  q.scontrib = ctx->scontrib;
  q.slist = ctx->slist;
  q.counters = ctx->counters;
  q.stats = ctx->dstats;
  q.capacity = (uint32_t)ctx->cap_rays;
  return q;
}

// An extra wave lane: stream, events and counters once; queues and pixel
// sums grown like lane 0's.
int ensure_lane(or3_context *ctx, int k, size_t paths, size_t rays, size_t pixels) {
  or3_context::Lane &L = ctx->xl[k];
  if (!ctx->ev_fork) OR3_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming));
  if (!L.stream) {
    OR3_CUDA(ctx, cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking));
    OR3_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_join[k], cudaEventDisableTiming));
    OR3_CUDA(ctx, cudaMalloc(&L.counters, 16 * sizeof(uint32_t)));
    OR3_CUDA(ctx, cudaMalloc(&L.dstats, 8 * sizeof(unsigned long long)));
  }
  if (paths > L.cap_paths || rays > L.cap_rays) {
    for (int k = 0; k < 2; k++) {
      cudaFree(L.qorig[k]);
      cudaFree(L.qdir[k]);
      cudaFree(L.qbeta[k]);
      L.qorig[k] = L.qdir[k] = L.qbeta[k] = nullptr;
    }
    for (float4 **p : {&L.hits, &L.pathL, &L.sorig, &L.sdir, &L.scontrib}) {
      cudaFree(*p);
      *p = nullptr;
    }
    cudaFree(L.slist);
    L.slist = nullptr;
    L.cap_paths = L.cap_rays = 0;
    trim_pools(ctx);
    for (int k = 0; k < 2; k++) {
      OR3_CUDA(ctx, cudaMalloc(&L.qorig[k], rays * sizeof(float4)));
      OR3_CUDA(ctx, cudaMalloc(&L.qdir[k], rays * sizeof(float4)));
      OR3_CUDA(ctx, cudaMalloc(&L.qbeta[k], rays * sizeof(float4)));
    }
    OR3_CUDA(ctx, cudaMalloc(&L.hits, rays * sizeof(float4)));
    OR3_CUDA(ctx, cudaMalloc(&L.pathL, paths * sizeof(float4)));
    OR3_CUDA(ctx, cudaMalloc(&L.sorig, rays * sizeof(float4)));
    OR3_CUDA(ctx, cudaMalloc(&L.sdir, rays * sizeof(float4)));
    OR3_CUDA(ctx, cudaMalloc(&L.scontrib, rays * sizeof(float4)));
    OR3_CUDA(ctx, cudaMalloc(&L.slist, rays * sizeof(uint32_t)));
    L.cap_paths = paths;
    L.cap_rays = rays;
  }
  if (pixels > L.cap_pixels) {
    cudaFree(L.pix_sum);
    cudaFree(L.pix_sumsq);
    L.pix_sum = L.pix_sumsq = nullptr;
    L.cap_pixels = 0;
    OR3_CUDA(ctx, cudaMalloc(&L.pix_sum, pixels * 3 * sizeof(double)));
    OR3_CUDA(ctx, cudaMalloc(&L.pix_sumsq, pixels * 3 * sizeof(double)));
    L.cap_pixels = pixels;
  }
  return OR3_OK;
}

void free_lane_buffers(or3_context::Lane &L) {
  for (int k = 0; k < 2; k++) {
    cudaFree(L.qorig[k]);
    cudaFree(L.qdir[k]);
    cudaFree(L.qbeta[k]);
    L.qorig[k] = L.qdir[k] = L.qbeta[k] = nullptr;
  }
  for (float4 **p : {&L.hits, &L.pathL, &L.sorig, &L.sdir, &L.scontrib}) {
    cudaFree(*p);
    *p = nullptr;
  }
  cudaFree(L.slist);
  L.slist = nullptr;
  cudaFree(L.pix_sum);
  cudaFree(L.pix_sumsq);
  L.pix_sum = L.pix_sumsq = nullptr;
  L.cap_paths = L.cap_rays = L.cap_pixels = 0;
}

Queues lane_queues(const or3_context::Lane &L) {
  Queues q{};
  for (int k = 0; k < 2; k++) {
    q.orig[k] = L.qorig[k];
    q.dir[k] = L.qdir[k];
    q.beta[k] = L.qbeta[k];
  }
  q.hits = L.hits;
  q.pathL = L.pathL;
  q.sorig = L.sorig;
  q.sdir = L.sdir;
  q.scontrib = L.scontrib;
  q.slist = L.slist;
  q.counters = L.counters;
  q.stats = L.dstats;
  q.capacity = (uint32_t)L.cap_rays;
  return q;
}

// Camera::Camera (src/renderer/Camera.h:12-43) in double.
int validate_render(or3_context *ctx, const or3_camera *cam, const or3_render_params *prm) {
  if (cam->width == 0 || cam->height == 0) return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "empty image");
  if ((uint64_t)cam->width * cam->height > (1ull << 28))
    return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "image too large");
  if (prm->supersamples < 1 || prm->supersamples > 256)
    return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "supersamples must be in [1,256]");
  if (prm->min_samples < 1 || prm->max_samples < prm->min_samples || prm->step_samples < 1)
    return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "sample schedule must satisfy 1 <= min <= max, step >= 1");
  if (prm->output_layout != OR3_LAYOUT_REFERENCE && prm->output_layout != OR3_LAYOUT_COMPACT)
    return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "unknown output layout");
  return OR3_OK;
}

void fill_render_const(const or3_camera *cam, const or3_render_params *prm, RenderConst &rc) {
  camera_basis(cam, rc.cam);
  rc.W = cam->width;
  rc.H = cam->height;
  rc.ss = (uint32_t)prm->supersamples;
  rc.ss2 = rc.ss * rc.ss;
  rc.nee = prm->next_event_estimation;
  rc.rr_min_depth = prm->rr_min_depth;
  rc.max_depth = prm->max_depth;
  rc.seed_lo = (uint32_t)prm->seed;
  rc.seed_hi = (uint32_t)(prm->seed >> 32);
}

void camera_basis(const or3_camera *c, Camera32 &out) {
  double dir[3] = {c->direction[0], c->direction[1], c->direction[2]};
  double upv[3] = {c->up[0], c->up[1], c->up[2]};
  auto nrm = [](double *v) {
    const double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] /= l; v[1] /= l; v[2] /= l;
  };
  auto crs = [](const double *a, const double *b, double *r) {
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
  };
  nrm(dir);
  nrm(upv);
  const double sh = c->screen_height_world;
  const double sw = c->screen_height_world * (double)c->width / (double)c->height;
  double X[3], Y[3];
  crs(dir, upv, X);
  nrm(X);
  crs(X, dir, Y);
  nrm(Y);
  for (int a = 0; a < 3; a++) {
    out.pos[a] = (float)c->position[a];
    out.center[a] = (float)(c->position[a] + dir[a] * c->distance_to_screen);
    out.xaxis[a] = (float)(X[a] * sw);
    out.yaxis[a] = (float)(Y[a] * sh);
  }
  out.focal = (float)c->focal_distance;
  out.aperture = (float)c->aperture_radius;
}

}  // namespace

extern "C" {

int or3_api_version(void) { return OR3_API_VERSION; }

const char *or3_last_error(const or3_context *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int or3_context_create(int device, or3_context **out) {
  if (!out) return OR3_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return OR3_ERR_NO_DEVICE;
  if (device < 0 || device >= n) return OR3_ERR_INVALID_ARGUMENT;
  or3_context *ctx = new or3_context();
  ctx->device = device;
  auto bail = [&](int code) {
    delete ctx;
    return code;
  };
  if (cudaSetDevice(device) != cudaSuccess) return bail(OR3_ERR_CUDA);
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(OR3_ERR_CUDA);
  cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ctx->occ_extend, kernel_extend_ptr(), 256, 0);
  ctx->occ_extend = std::max(ctx->occ_extend, 1);
  // the shade instances differ in registers (the light sample): a grid sized
  // for the wrong one leaves a tail of blocks that wait for a free slot
  for (int nee = 0; nee < 2; nee++) {
    int o = 64;
    for (int batch = 0; batch < 2; batch++) {
      int ob = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ob, kernel_shade_ptr(batch, nee), 256, 0);
      o = std::min(o, ob);
    }
    (nee ? ctx->occ_shade_nee : ctx->occ_shade) = std::max(o, 1);
  }
  set_query_grid(ctx->num_sms * ctx->occ_extend);
  {
    cudaMemPoolProps pp{};
    pp.allocType = cudaMemAllocationTypePinned;
    pp.location.type = cudaMemLocationTypeDevice;
    pp.location.id = device;
    if (cudaMemPoolCreate(&ctx->tmp_pool, &pp) != cudaSuccess) return bail(OR3_ERR_CUDA);
    uint64_t keep = uint64_t(1) << 30;
    cudaMemPoolSetAttribute(ctx->tmp_pool, cudaMemPoolAttrReleaseThreshold, &keep);
    if (cudaMemPoolCreate(&ctx->scene_pool, &pp) != cudaSuccess) {
      cudaMemPoolDestroy(ctx->tmp_pool);
      return bail(OR3_ERR_CUDA);
    }
    cudaMemPoolSetAttribute(ctx->scene_pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  if (cudaMalloc(&ctx->counters, 16 * sizeof(uint32_t)) != cudaSuccess) return bail(OR3_ERR_OUT_OF_MEMORY);
  if (cudaMalloc(&ctx->dstats, 8 * sizeof(unsigned long long)) != cudaSuccess) return bail(OR3_ERR_OUT_OF_MEMORY);
  // pinned read-back counters: lane 0 at [0, 4), extra lane k at [8 + 4k, 12 + 4k)
  if (cudaMallocHost(&ctx->host_counters, 32 * sizeof(uint32_t)) != cudaSuccess) return bail(OR3_ERR_OUT_OF_MEMORY);
  cudaMemset(ctx->counters, 0, 16 * sizeof(uint32_t));
  cudaMemset(ctx->dstats, 0, 8 * sizeof(unsigned long long));
  cudaEventCreate(&ctx->ev0);
  cudaEventCreate(&ctx->ev1);
  if (cudaDeviceSynchronize() != cudaSuccess) return bail(OR3_ERR_CUDA);
  *out = ctx;
  return OR3_OK;
}

int or3_context_destroy(or3_context *ctx) {
  if (!ctx) return OR3_ERR_INVALID_ARGUMENT;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  destroy_server_state(ctx);
  destroy_batch_state(ctx);
  for (auto &kv : ctx->scenes) free_scene(kv.second);
  for (int k = 0; k < 2; k++) {
    cudaFree(ctx->qorig[k]);
    cudaFree(ctx->qdir[k]);
    cudaFree(ctx->qbeta[k]);
  }
  cudaFree(ctx->hits);
  cudaFree(ctx->pathL);
  cudaFree(ctx->sorig);
  cudaFree(ctx->sdir);
  cudaFree(ctx->scontrib);
  cudaFree(ctx->slist);
  cudaFree(ctx->counters);
  cudaFree(ctx->dstats);
  cudaFreeHost(ctx->host_counters);
  cudaFree(ctx->pix_sum);
  cudaFree(ctx->pix_sumsq);
  cudaFree(ctx->frame_dev);
  cudaFree(ctx->wave_fail);
  cudaFreeHost(ctx->frame_pinned);
  cudaFreeHost(ctx->frame_front);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  for (cudaEvent_t e : ctx->kpool) cudaEventDestroy(e);
  if (ctx->stage) cudaFreeHost(ctx->stage);
  for (int k = 0; k < kExtraLanes; k++) {
    or3_context::Lane &L = ctx->xl[k];
    if (L.stream) cudaStreamSynchronize(L.stream);
    for (int j = 0; j < 2; j++) {
      cudaFree(L.qorig[j]);
      cudaFree(L.qdir[j]);
      cudaFree(L.qbeta[j]);
    }
    for (void *p : {(void *)L.hits, (void *)L.pathL, (void *)L.sorig, (void *)L.sdir, (void *)L.scontrib,
                    (void *)L.counters, (void *)L.dstats, (void *)L.pix_sum, (void *)L.pix_sumsq})
      cudaFree(p);
    if (L.stream) cudaStreamDestroy(L.stream);
    if (ctx->ev_join[k]) cudaEventDestroy(ctx->ev_join[k]);
  }
  if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
  for (cudaEvent_t e : ctx->ev_poll)
    if (e) cudaEventDestroy(e);
  cudaStreamSynchronize(ctx->stream);
  if (ctx->tmp_pool) cudaMemPoolDestroy(ctx->tmp_pool);
  if (ctx->scene_pool) cudaMemPoolDestroy(ctx->scene_pool);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return OR3_OK;
}

namespace {

// Flattened in-BVH primitives in input order (triangles, then spheres):
// the kernels' FP32 geometry (12 floats), build bounds, PrimInfo, TriShade.
struct FlatPrims {
  float *geom = nullptr;
  BuildPrim *bp = nullptr;
  PrimInfo *info = nullptr;
  TriShade *shade = nullptr;
  std::vector<float> vgeom;  // storage unless the context's pinned staging holds them
  std::vector<BuildPrim> vbp;
  std::vector<PrimInfo> vinfo;
  std::vector<TriShade> vshade;
};

constexpr size_t kFlatBytes = 12 * sizeof(float) + sizeof(BuildPrim) + sizeof(PrimInfo) + sizeof(TriShade);
constexpr size_t kStageMax = size_t(4) << 30;  // larger scenes flatten into pageable memory

// Primitives [i0, i1) of the flattening.  Returns the first index whose
// layers (or sphere radius) are invalid, or i1; *bad_bounds is set when a
// finished primitive has an invalid or non-finite box.
uint32_t flatten_range(const or3_scene_desc *d, uint32_t i0, uint32_t i1, FlatPrims &f, bool *bad_bounds) {
  const uint32_t nt = d->num_triangles;
  for (uint32_t i = i0; i < i1; i++) {
    const bool tri = i < nt;
    const uint32_t j = tri ? i : i - nt;
    const uint32_t *lay = tri ? d->tri_layers + 2 * (size_t)i : d->sphere_layers + 2 * (size_t)j;
    if (lay[1] == 0 || (uint64_t)lay[0] + lay[1] > d->num_layers) return i;
    if (!tri && !(d->spheres[4 * (size_t)j + 3] > 0)) return i;
    float *g = f.geom + 12 * (size_t)i;
    BuildPrim &b = f.bp[i];
    TriShade &ts = f.shade[i];
    std::memset(g, 0, 12 * sizeof(float));
    std::memset(&ts, 0, sizeof(ts));
    if (tri) {
      const double *v = d->tri_vertices + 9 * (size_t)i;
      for (int a = 0; a < 3; a++) {
        g[a] = (float)v[a];                   // v0
        g[3 + a] = (float)(v[3 + a] - v[a]);  // e1 = p1 - p0
        g[6 + a] = (float)(v[6 + a] - v[a]);  // e2 = p2 - p0
      }
      for (int a = 0; a < 3; a++) {
        const double p0 = g[a], p1 = (double)g[a] + g[3 + a], p2 = (double)g[a] + g[6 + a];
        b.lo[a] = down(std::min(p0, std::min(p1, p2)));
        b.hi[a] = up(std::max(p0, std::max(p1, p2)));
      }
      b.kind = kPrimTriangle;
      f.info[i] = PrimInfo{d->tri_ids ? d->tri_ids[i] : i, lay[0], lay[1], kPrimTriangle | (layer_flags(d, lay) << 8)};
      double n0[3], n1[3], n2[3];
      if (d->tri_normals) {
        const double *n = d->tri_normals + 9 * (size_t)i;
        for (int a = 0; a < 3; a++) { n0[a] = n[a]; n1[a] = n[3 + a]; n2[a] = n[6 + a]; }
      } else {
        const double e1[3] = {v[3] - v[0], v[4] - v[1], v[5] - v[2]};
        const double e2[3] = {v[6] - v[0], v[7] - v[1], v[8] - v[2]};
        double c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        const double l = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        for (int a = 0; a < 3; a++) n0[a] = n1[a] = n2[a] = l > 0 ? c[a] / l : 0.0;
      }
      for (int a = 0; a < 3; a++) {
        ts.n0[a] = (float)n0[a];
        ts.dn1[a] = (float)(n1[a] - n0[a]);
        ts.dn2[a] = (float)(n2[a] - n0[a]);
      }
      if (d->tri_uvs) {
        const double *u = d->tri_uvs + 6 * (size_t)i;
        for (int a = 0; a < 2; a++) {
          ts.uv0[a] = (float)u[a];
          ts.duv1[a] = (float)(u[2 + a] - u[a]);
          ts.duv2[a] = (float)(u[4 + a] - u[a]);
        }
      }
    } else {
      const double *sp = d->spheres + 4 * (size_t)j;
      g[0] = (float)sp[0]; g[1] = (float)sp[1]; g[2] = (float)sp[2]; g[3] = (float)sp[3];
      for (int a = 0; a < 3; a++) {
        b.lo[a] = down((double)g[a] - (double)g[3]);
        b.hi[a] = up((double)g[a] + (double)g[3]);
      }
      b.kind = kPrimSphere;
      uint32_t fl = layer_flags(d, lay);
      if (d->sphere_flags && (d->sphere_flags[j] & OR3_SPHERE_LIGHT)) fl |= kFlagSphereLight;
      f.info[i] = PrimInfo{d->sphere_ids ? d->sphere_ids[j] : nt + j, lay[0], lay[1], kPrimSphere | (fl << 8)};
    }
    for (int a = 0; a < 3; a++)
      if (!(b.lo[a] <= b.hi[a]) || !std::isfinite(b.lo[a]) || !std::isfinite(b.hi[a])) *bad_bounds = true;
  }
  return i1;
}

}  // namespace

int or3_scene_upload(or3_context *ctx, const or3_scene_desc *d, int32_t *scene_out) {
  if (!ctx || !d || !scene_out) return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "null argument");
  cudaSetDevice(ctx->device);
  *scene_out = -1;
  // ---- validation
  if (d->num_materials == 0 || !d->materials) return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "no materials");
  if (d->num_layers == 0 || !d->layer_material || !d->layer_rate)
    return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "no material layers");
  for (uint32_t i = 0; i < d->num_layers; i++)
    if (d->layer_material[i] >= d->num_materials)
      return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "layer %u: material %u out of range", i, d->layer_material[i]);
  for (uint32_t i = 0; i < d->num_materials; i++) {
    const or3_material &m = d->materials[i];
    if (m.type < OR3_LAMBERT || m.type > OR3_PHONG)
      return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "material %u: unknown type %d", i, m.type);
    if (m.texture >= (int32_t)d->num_textures)
      return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "material %u: texture %d out of range", i, m.texture);
  }
  if (d->num_triangles && (!d->tri_vertices || !d->tri_layers))
    return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "triangles without vertices or layers");
  if (d->num_spheres && (!d->spheres || !d->sphere_layers))
    return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "spheres without data or layers");
  if (d->num_planes && (!d->planes || !d->plane_layers))
    return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "planes without data or layers");
  if ((uint64_t)d->num_triangles + d->num_spheres >= (uint64_t)kPlaneBit)
    return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "too many primitives");
  if ((d->env_rgb || d->env_rgbe) && (d->env_width == 0 || d->env_height == 0))
    return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "environment map with zero size");
  if (d->env_rgb && d->env_rgbe)
    return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "give the environment as env_rgb or env_rgbe, not both");

  auto t0 = std::chrono::steady_clock::now();
  SceneGPU *sg = new SceneGPU();
  sg->stream = ctx->stream;
  const uint32_t nt = d->num_triangles, nsph = d->num_spheres, np = nt + nsph;

  // ---- primitives and their bounds (in the FP32 geometry the kernels test),
  // on all host threads; a device build reads them from pinned staging
  const bool dev_build = np > 0 && np <= (1u << 26) &&
                         (d->build == OR3_BUILD_DEVICE ||
                          (d->build == OR3_BUILD_AUTO && np >= OR3_BUILD_DEVICE_MIN_PRIMS));
  FlatPrims fp;
  // the sky's bytes go through the same pinned staging (copied on the
  // flattening threads) instead of a pageable copy
  const size_t env_bytes = d->env_rgb    ? 3 * sizeof(float) * (size_t)d->env_width * d->env_height
                           : d->env_rgbe ? 4 * (size_t)d->env_width * d->env_height
                                         : 0;
  const void *env_src = d->env_rgb ? (const void *)d->env_rgb : (const void *)d->env_rgbe;
  char *env_stage = nullptr;
  const size_t stage_need = kFlatBytes * (size_t)np + env_bytes + 5 * 64;
  if (dev_build && stage_need <= kStageMax) {
    if (ctx->stage_bytes < stage_need) {
      cudaStreamSynchronize(ctx->stream);
      if (ctx->stage) cudaFreeHost(ctx->stage);
      ctx->stage = nullptr;
      ctx->stage_bytes = 0;
      if (cudaMallocHost(&ctx->stage, stage_need) == cudaSuccess) ctx->stage_bytes = stage_need;
      else ctx->stage = nullptr;
    }
  }
  if (dev_build && ctx->stage && ctx->stage_bytes >= stage_need) {
    cudaStreamSynchronize(ctx->stream);  // no copy out of the staging still in flight
    char *c = static_cast<char *>(ctx->stage);
    auto carve = [&](size_t bytes) {
      char *r = c;
      c += (bytes + 63) & ~size_t(63);
      return r;
    };
    fp.geom = reinterpret_cast<float *>(carve(12 * sizeof(float) * (size_t)np));
    fp.bp = reinterpret_cast<BuildPrim *>(carve(sizeof(BuildPrim) * (size_t)np));
    fp.info = reinterpret_cast<PrimInfo *>(carve(sizeof(PrimInfo) * (size_t)np));
    fp.shade = reinterpret_cast<TriShade *>(carve(sizeof(TriShade) * (size_t)np));
    if (env_bytes) env_stage = carve(env_bytes);
  } else {
    fp.vgeom.resize(12 * (size_t)np);
    fp.vbp.resize(np);
    fp.vinfo.resize(np);
    fp.vshade.resize(np);
    fp.geom = fp.vgeom.data();
    fp.bp = fp.vbp.data();
    fp.info = fp.vinfo.data();
    fp.shade = fp.vshade.data();
  }
  {
    const uint32_t hw = std::max(1u, std::thread::hardware_concurrency());
    const uint32_t nth = std::max(1u, std::min<uint32_t>(hw, np / 8192u));
    std::vector<uint32_t> first_bad(nth, np);
    std::vector<char> bad_bounds(nth, 0);
    auto work = [&](uint32_t t) {
      const uint32_t a = (uint32_t)((uint64_t)np * t / nth), b = (uint32_t)((uint64_t)np * (t + 1) / nth);
      bool bb = false;
      const uint32_t r = flatten_range(d, a, b, fp, &bb);
      first_bad[t] = r < b ? r : np;
      bad_bounds[t] = bb;
      if (env_stage) {
        const size_t e0 = env_bytes * t / nth, e1 = env_bytes * (t + 1) / nth;
        std::memcpy(env_stage + e0, static_cast<const char *>(env_src) + e0, e1 - e0);
      }
    };
    std::vector<std::thread> pool;
    for (uint32_t t = 1; t < nth; t++) pool.emplace_back(work, t);
    work(0);
    for (std::thread &th : pool) th.join();
    const uint32_t bad = *std::min_element(first_bad.begin(), first_bad.end());
    if (bad < np) {
      // the message of the first invalid primitive, as a sequential check gives it
      int rc = bad < nt ? check_layers(ctx, d, d->tri_layers + 2 * (size_t)bad, "triangle", bad)
                        : check_layers(ctx, d, d->sphere_layers + 2 * (size_t)(bad - nt), "sphere", bad - nt);
      if (!rc) rc = fail(ctx, OR3_ERR_INVALID_ARGUMENT, "sphere %u: radius <= 0", bad - nt);
      free_scene(sg);
      return rc;
    }
    if (dev_build && std::find(bad_bounds.begin(), bad_bounds.end(), 1) != bad_bounds.end()) {
      free_scene(sg);
      return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "build_wide_bvh: primitive with invalid or non-finite bounds");
    }
  }
  auto tf = std::chrono::steady_clock::now();

  // ---- BVH: host threads, or the device for large scenes (same tree rules)
  if (d->build > OR3_BUILD_DEVICE) {
    free_scene(sg);
    return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "unknown build location %u", d->build);
  }
  const int leaf_max = d->leaf_max ? (int)d->leaf_max : 4;
  const double trav_cost = d->traversal_cost > 0 ? d->traversal_cost : 1.0;
  if (leaf_max > 8) {
    free_scene(sg);
    return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "leaf_max %d: at most 8", leaf_max);
  }
  const bool on_device = dev_build;
  WideBVH bvh;
  DeviceBVH dbvh;
  DeviceTemps tmp(ctx);  // freed on the stream when the upload returns
  std::string berr;
  if (!on_device) {
    if (!build_wide_bvh(fp.vbp, 16, leaf_max, bvh, &berr, trav_cost)) {
      free_scene(sg);
      return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "%s", berr.c_str());
    }
  } else {
    BuildPrim *bp_dev = nullptr;
    if (int rc = tmp.alloc(ctx, &bp_dev, np)) { free_scene(sg); return rc; }
    const cudaError_t ce = cudaMemcpyAsync(bp_dev, fp.bp, np * sizeof(BuildPrim), cudaMemcpyHostToDevice,
                                           ctx->stream);
    if (ce != cudaSuccess) {
      free_scene(sg);
      return fail(ctx, OR3_ERR_CUDA, "scene upload: %s", cudaGetErrorString(ce));
    }
    if (!build_wide_bvh_device(bp_dev, np, leaf_max, ctx->stream, dbvh, &berr, trav_cost, ctx->tmp_pool)) {
      free_scene(sg);
      return fail(ctx, OR3_ERR_CUDA, "%s", berr.c_str());
    }
    sg->allocs.push_back(dbvh.nodes);
    sg->allocs.push_back(dbvh.fnodes);
    tmp.p.push_back(dbvh.order);
  }
  // the traversal stack (kStackSize entries, at most 3 pushed per wide level)
  // relies on the builders' depth bound
  if ((on_device ? dbvh.wide_depth : bvh.wide_depth) > kMaxBinaryDepth / 2) {
    free_scene(sg);
    return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "BVH deeper than the traversal stack allows (%d wide levels)",
                on_device ? dbvh.wide_depth : bvh.wide_depth);
  }
  auto t1 = std::chrono::steady_clock::now();

  // ---- records in leaf order (the device build gathers them on the device)
  const uint32_t nrec = on_device ? 0u : np;
  std::vector<float4> prims(3 * (size_t)nrec);
  std::vector<PrimInfo> info(nrec);
  std::vector<TriShade> shade(nrec);
  for (uint32_t r = 0; r < nrec; r++) {
    const uint32_t src = bvh.order[r];
    const float *g = fp.geom + 12 * (size_t)src;
    if (src < nt) {
      prims[3 * r + 0] = make_float4(g[0], g[1], g[2], g[3]);
      prims[3 * r + 1] = make_float4(g[4], g[5], g[6], g[7]);
      prims[3 * r + 2] = make_float4(g[8], 0.f, 0.f, 0.f);
    } else {
      prims[3 * r + 0] = make_float4(g[0], g[1], g[2], g[3]);
      prims[3 * r + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
      prims[3 * r + 2] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    info[r] = fp.info[src];
    shade[r] = fp.shade[src];
  }
  std::vector<PlaneRec> planes(d->num_planes);
  for (uint32_t i = 0; i < d->num_planes; i++) {
    int rc = check_layers(ctx, d, d->plane_layers + 2 * i, "plane", i);
    if (rc) { free_scene(sg); return rc; }
    const double *p = d->planes + 4 * (size_t)i;
    PlaneRec &pr = planes[i];
    pr.kind = (int)p[0] == OR3_PLANE_INFINITE_FLOOR ? kPrimFloor : kPrimPlane;
    pr.axis = (uint32_t)p[1];
    if (pr.axis > 2) { free_scene(sg); return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "plane %u: axis %u", i, pr.axis); }
    pr.offset = (float)p[2];
    pr.normal_sign = p[3] != 0.0 ? -1.f : 1.f;
    pr.object_id = d->plane_ids ? d->plane_ids[i] : np + i;
    pr.layer_begin = d->plane_layers[2 * i];
    pr.layer_count = d->plane_layers[2 * i + 1];
    pr.flags = layer_flags(d, d->plane_layers + 2 * i);
  }
  std::vector<MaterialDev> mats(d->num_materials);
  bool split = false;
  for (uint32_t i = 0; i < d->num_materials; i++) {
    const or3_material &m = d->materials[i];
    MaterialDev &o = mats[i];
    std::memset(&o, 0, sizeof(o));
    for (int a = 0; a < 3; a++) {
      o.emission[a] = (float)m.emission[a];
      o.color[a] = (float)m.color[a];
    }
    o.ior = (float)m.ior;
    o.phong_exponent = (float)m.phong_exponent;
    o.type = m.type;
    o.texture = m.texture;
    o.emissive = (m.emission[0] * m.emission[0] + m.emission[1] * m.emission[1] + m.emission[2] * m.emission[2]) != 0;
  }
  std::vector<LayerDev> layers(d->num_layers);
  for (uint32_t i = 0; i < d->num_layers; i++) {
    layers[i].material = d->layer_material[i];
    layers[i].rate = (float)d->layer_rate[i];
    if (d->materials[d->layer_material[i]].type == OR3_REFRACTION) split = true;
  }
  sg->has_split = split;

  DevScene &S = sg->view;
  S.num_nodes = on_device ? dbvh.num_nodes : (uint32_t)bvh.nodes.size();
  S.num_prims = np;
  S.num_planes = d->num_planes;
  S.bg[0] = (float)d->background[0];
  S.bg[1] = (float)d->background[1];
  S.bg[2] = (float)d->background[2];
  int rc = OR3_OK;
  if (!on_device) {
    const WideNode *nodes_dev = nullptr;
    if ((rc = dev_upload(ctx, sg, bvh.nodes, &nodes_dev))) { free_scene(sg); return rc; }
    S.nodes = reinterpret_cast<const uint4 *>(nodes_dev);
    std::vector<WideNodeF> fnodes;
    make_float_nodes(bvh, fnodes);
    const WideNodeF *fnodes_dev = nullptr;
    if ((rc = dev_upload(ctx, sg, fnodes, &fnodes_dev))) { free_scene(sg); return rc; }
    S.fnodes = reinterpret_cast<const float4 *>(fnodes_dev);
    if ((rc = dev_upload(ctx, sg, prims, &S.prims))) { free_scene(sg); return rc; }
    if ((rc = dev_upload(ctx, sg, info, &S.info))) { free_scene(sg); return rc; }
    if ((rc = dev_upload(ctx, sg, shade, &S.tri_shade))) { free_scene(sg); return rc; }
  } else {
    S.nodes = reinterpret_cast<const uint4 *>(dbvh.nodes);
    S.fnodes = reinterpret_cast<const float4 *>(dbvh.fnodes);
    sg->info.device_bytes += (size_t)dbvh.num_nodes * (sizeof(WideNode) + sizeof(WideNodeF));
    // input-order records (temporary) gathered into leaf order
    float4 *geom_in = nullptr;
    PrimInfo *info_in = nullptr;
    TriShade *shade_in = nullptr;
    if ((rc = tmp.alloc(ctx, &geom_in, 3 * (size_t)np)) || (rc = tmp.alloc(ctx, &info_in, np)) ||
        (rc = tmp.alloc(ctx, &shade_in, np))) {
      free_scene(sg);
      return rc;
    }
    cudaError_t ce = cudaMemcpyAsync(geom_in, fp.geom, 12 * sizeof(float) * (size_t)np, cudaMemcpyHostToDevice,
                                     ctx->stream);
    if (ce == cudaSuccess)
      ce = cudaMemcpyAsync(info_in, fp.info, np * sizeof(PrimInfo), cudaMemcpyHostToDevice, ctx->stream);
    if (ce == cudaSuccess)
      ce = cudaMemcpyAsync(shade_in, fp.shade, np * sizeof(TriShade), cudaMemcpyHostToDevice, ctx->stream);
    if (ce != cudaSuccess) {
      free_scene(sg);
      return fail(ctx, OR3_ERR_CUDA, "scene upload: %s", cudaGetErrorString(ce));
    }
    float4 *prims_d = nullptr;
    PrimInfo *info_d = nullptr;
    TriShade *shade_d = nullptr;
    if ((rc = dev_alloc(ctx, sg, &prims_d, 3 * (size_t)np)) || (rc = dev_alloc(ctx, sg, &info_d, np)) ||
        (rc = dev_alloc(ctx, sg, &shade_d, np))) {
      free_scene(sg);
      return rc;
    }
    gather_leaf_order(np, dbvh.order, geom_in, info_in, shade_in, prims_d, info_d, shade_d, ctx->stream);
    S.prims = prims_d;
    S.info = info_d;
    S.tri_shade = shade_d;
  }
  if ((rc = dev_upload(ctx, sg, planes, &S.planes))) { free_scene(sg); return rc; }
  if ((rc = dev_upload(ctx, sg, mats, &S.materials))) { free_scene(sg); return rc; }
  if ((rc = dev_upload(ctx, sg, layers, &S.layers))) { free_scene(sg); return rc; }
  double *env_total = nullptr;  // device: [H] row totals, [H] the map's total
  if (d->env_rgb || d->env_rgbe) {
    const uint32_t W = d->env_width, H = d->env_height;
    const size_t texels = (size_t)W * H;
    float *env_d = nullptr, *marg_d = nullptr, *cond_d = nullptr;
    uint32_t *gmarg_d = nullptr, *gcond_d = nullptr;
    if ((rc = dev_alloc(ctx, sg, &env_d, 3 * texels)) || (rc = dev_alloc(ctx, sg, &marg_d, H)) ||
        (rc = dev_alloc(ctx, sg, &cond_d, texels)) || (rc = dev_alloc(ctx, sg, &gmarg_d, (size_t)H + 1)) ||
        (rc = dev_alloc(ctx, sg, &gcond_d, (size_t)H * (W + 1))) ||
        (rc = tmp.alloc(ctx, &env_total, (size_t)H + 1))) {
      free_scene(sg);
      return rc;
    }
    cudaError_t ce;
    if (d->env_rgb) {
      ce = cudaMemcpyAsync(env_d, env_stage ? (const void *)env_stage : (const void *)d->env_rgb,
                           3 * texels * sizeof(float), cudaMemcpyHostToDevice, ctx->stream);
    } else {
      // RGBE bytes (a third of the float map's size) decoded on the device
      uint8_t *rgbe_d = nullptr;
      if ((rc = tmp.alloc(ctx, &rgbe_d, 4 * texels))) { free_scene(sg); return rc; }
      ce = cudaMemcpyAsync(rgbe_d, env_stage ? (const void *)env_stage : (const void *)d->env_rgbe, 4 * texels,
                           cudaMemcpyHostToDevice, ctx->stream);
      if (ce == cudaSuccess) launch_decode_rgbe(rgbe_d, texels, env_d, ctx->stream);
    }
    if (ce != cudaSuccess) {
      free_scene(sg);
      return fail(ctx, OR3_ERR_CUDA, "environment upload: %s", cudaGetErrorString(ce));
    }
    launch_env_cdf(env_d, W, H, marg_d, cond_d, env_total, gmarg_d, gcond_d, ctx->stream);
    S.env = env_d;
    S.env_marg = marg_d;
    S.env_cond = cond_d;
    S.env_gmarg = gmarg_d;
    S.env_gcond = gcond_d;
    S.env_w = W;
    S.env_h = H;
  }
  LightTables T;
  build_light_tables(d, fp.geom, T);
  if ((rc = dev_upload(ctx, sg, T.lights, &S.lights))) { free_scene(sg); return rc; }
  if ((rc = dev_upload(ctx, sg, T.cdf, &S.light_cdf))) { free_scene(sg); return rc; }
  if ((rc = dev_upload(ctx, sg, T.pdf, &S.light_pdf))) { free_scene(sg); return rc; }
  S.num_lights = (uint32_t)T.lights.size();
  S.env_light = T.env_light;
  sg->info.num_lights = (int32_t)S.num_lights;
  if (d->num_textures) {
    std::vector<TextureDev> tex(d->num_textures);
    uint64_t total = 0;
    for (uint32_t i = 0; i < d->num_textures; i++) {
      tex[i].offset = d->texture_offsets[i];
      tex[i].width = d->texture_dims[2 * i];
      tex[i].height = d->texture_dims[2 * i + 1];
      total = std::max<uint64_t>(total, tex[i].offset + 3ull * tex[i].width * tex[i].height);
    }
    std::vector<float> texels(d->texture_rgb, d->texture_rgb + total);
    if ((rc = dev_upload(ctx, sg, tex, &S.textures))) { free_scene(sg); return rc; }
    if ((rc = dev_upload(ctx, sg, texels, &S.texels))) { free_scene(sg); return rc; }
    S.num_textures = d->num_textures;
  }
  double env_sum = 0.0;
  if (env_total) cudaMemcpyAsync(&env_sum, env_total + S.env_h, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    free_scene(sg);
    return fail(ctx, OR3_ERR_CUDA, "scene upload: %s", cudaGetErrorString(e));
  }
  if (env_total) S.env_light = env_sum > 0 ? 1 : 0;
  S.env_prob = S.env_light ? (S.num_lights ? 0.5f : 1.0f) : 0.0f;
  auto t2 = std::chrono::steady_clock::now();
  sg->info.num_primitives = np + d->num_planes;
  sg->info.num_nodes = S.num_nodes;
  sg->info.build_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  sg->info.flatten_ms = std::chrono::duration<double, std::milli>(tf - t0).count();
  sg->info.upload_ms = std::chrono::duration<double, std::milli>(t2 - t1).count();
  sg->info.tree_depth = on_device ? dbvh.wide_depth : bvh.wide_depth;
  const int32_t id = ctx->next_scene++;
  ctx->scenes[id] = sg;
  *scene_out = id;
  return OR3_OK;
}

int or3_scene_release(or3_context *ctx, int32_t scene) {
  if (!ctx) return OR3_ERR_INVALID_ARGUMENT;
  auto it = ctx->scenes.find(scene);
  if (it == ctx->scenes.end()) return fail(ctx, OR3_ERR_NOT_FOUND, "scene %d not found", scene);
  cudaSetDevice(ctx->device);
  // every stream of the device (wave lanes, a running server) is past the
  // scene's last use before its memory goes back to the pool
  cudaDeviceSynchronize();
  free_scene(it->second);
  ctx->scenes.erase(it);
  return OR3_OK;
}

int or3_scene_get_info(or3_context *ctx, int32_t scene, or3_scene_info *out) {
  if (!ctx || !out) return OR3_ERR_INVALID_ARGUMENT;
  auto it = ctx->scenes.find(scene);
  if (it == ctx->scenes.end()) return fail(ctx, OR3_ERR_NOT_FOUND, "scene %d not found", scene);
  *out = it->second->info;
  return OR3_OK;
}

int or3_stop(or3_context *ctx) {
  if (!ctx) return OR3_ERR_INVALID_ARGUMENT;
  ctx->stop.store(true);
  return OR3_OK;
}

int or3_reset_stop(or3_context *ctx) {
  if (!ctx) return OR3_ERR_INVALID_ARGUMENT;
  ctx->stop.store(false);
  return OR3_OK;
}

int or3_render(or3_context *ctx, int32_t scene, const or3_camera *cam, const or3_render_params *prm,
               or3_frame_callback cb, void *user) {
  if (!ctx || !cam || !prm) return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "null argument");
  auto it = ctx->scenes.find(scene);
  if (it == ctx->scenes.end()) return fail(ctx, OR3_ERR_NOT_FOUND, "scene %d not found", scene);
  SceneGPU *sg = it->second;
  if (int v = validate_render(ctx, cam, prm)) return v;
  cudaSetDevice(ctx->device);

  const uint32_t W = cam->width, H = cam->height, ss = (uint32_t)prm->supersamples, ss2 = ss * ss;
  const uint64_t npix = (uint64_t)W * H;
  const uint64_t paths_per_sample = npix * ss2;
  // Default waves: 2^25 camera paths.  Fewer, larger waves mean fewer bounce
  // iterations and kernel tails (measured on the mesh workload: 4M-path waves
  // 1007 Mpaths/s, 32M-path waves 1285; the terrain 2440 / 2659 / 2774 / 2829
  // at 2^22 / 2^23 / 2^24 / 2^25).
  // Where glass can split paths the queues hold the scene's split_factor
  // rays per path (kSplitQueueFactor at first), and a wave that overflows
  // them is rendered again in sub-waves (see the end of the pass); after such
  // a render the scene's factor doubles, up to 8, and its default waves
  // shrink to keep the queues' size (2^26 rays).  OR3_FLAG_KEEP_PATHS reads
  // the last wave's per-path radiance, so it keeps queues no split can
  // overflow (8 rays per path) and 2^23-path waves.
  const bool keep_paths = (prm->flags & OR3_FLAG_KEEP_PATHS) != 0;
  const uint64_t qfactor = !sg->has_split ? 1 : keep_paths ? 8 : std::min<uint32_t>(sg->split_factor, 8u);
  const bool optimistic = sg->has_split && qfactor < 8;  // a wave's queue can overflow: re-render it
  uint64_t wave = prm->wave_paths ? prm->wave_paths : std::min<uint64_t>(1ull << 25, (1ull << 26) / qfactor);
  wave = std::max<uint64_t>(wave, ss2);
  wave = std::min<uint64_t>(wave, (1ull << 31) / qfactor);  // queue capacities stay 32-bit
  // Waves: whole samples of the full image when one fits, else row chunks of one sample.
  uint64_t ns_per_wave = 1, npix_per_wave = npix;
  if (paths_per_sample <= wave) {
    ns_per_wave = wave / paths_per_sample;
  } else {
    npix_per_wave = std::max<uint64_t>(1, wave / ss2);
  }
  const uint64_t max_wave_paths = ns_per_wave * npix_per_wave * ss2;
  // a split scene's queues hold at least 8 rays per path of one pixel, so a
  // one-pixel sub-wave always fits
  const uint64_t rays = std::max<uint64_t>(max_wave_paths * qfactor, sg->has_split ? 8 * (uint64_t)ss2 : 1);
  // sub-waves of an overflowed wave: whole pixels, at most rays / 8 paths
  const uint64_t safe_pix = std::max<uint64_t>(1, rays / 8 / ss2);
  // the overflow list holds every wave of a pass
  const uint64_t max_pass_waves =
      (((uint64_t)prm->max_samples + ns_per_wave - 1) / ns_per_wave) * ((npix + npix_per_wave - 1) / npix_per_wave);
  int rc = ensure_queues(ctx, max_wave_paths, rays);
  if (rc) return rc;
  const size_t frame_doubles = (prm->output_layout == OR3_LAYOUT_REFERENCE ? 2 : 1) * npix * 3;
  if ((rc = ensure_pixels(ctx, npix, frame_doubles))) return rc;
  if (max_pass_waves + 1 > ctx->cap_wave_fail) {
    cudaFree(ctx->wave_fail);
    ctx->wave_fail = nullptr;
    ctx->cap_wave_fail = 0;
    OR3_CUDA(ctx, cudaMalloc(&ctx->wave_fail, (max_pass_waves + 1) * sizeof(uint32_t)));
    ctx->cap_wave_fail = max_pass_waves + 1;
  }
  const uint32_t fail_cap = (uint32_t)std::min<uint64_t>(ctx->cap_wave_fail - 1, UINT32_MAX);

  RenderConst rcst{};
  fill_render_const(cam, prm, rcst);

  cudaStream_t st = ctx->stream;
  OR3_CUDA(ctx, cudaMemsetAsync(ctx->pix_sum, 0, npix * 3 * sizeof(double), st));
  OR3_CUDA(ctx, cudaMemsetAsync(ctx->pix_sumsq, 0, npix * 3 * sizeof(double), st));
  OR3_CUDA(ctx, cudaMemsetAsync(ctx->frame_dev, 0, frame_doubles * sizeof(double), st));
  OR3_CUDA(ctx, cudaMemsetAsync(ctx->counters, 0, 16 * sizeof(uint32_t), st));
  OR3_CUDA(ctx, cudaMemsetAsync(ctx->dstats, 0, 8 * sizeof(unsigned long long), st));
  OR3_CUDA(ctx, cudaMemsetAsync(ctx->wave_fail, 0, sizeof(uint32_t), st));

  // the render's own capacity, not the allocation's (which earlier, larger
  // renders may have grown): whether a wave overflows depends on the wave only
  Queues q = make_queues(ctx);
  q.capacity = (uint32_t)std::min<uint64_t>(q.capacity, rays);
  const int block = 256;
  const int grid_ext = ctx->num_sms * ctx->occ_extend;
  const int smem_nodes =
      (prm->tuning & OR3_TUNE_SMEM_NODES) ? (int)std::min<uint64_t>(256, sg->view.num_nodes) : 0;
  // the 8-wide traversal variant: its tree is made from the 4-wide one on first use
  const bool wide8 = (prm->tuning & OR3_TUNE_WIDE8) != 0;
  if (wide8) {
    if (int r = ensure_wide8(ctx, sg)) return r;
  }
  const int variant = wide8 ? 8 : extend_variant(prm->tuning);
  // L2 persisting window over the BVH nodes (a context setting, restored below)
  const bool l2win = (prm->tuning & OR3_TUNE_L2_PERSIST) != 0;
  if (l2win) {
    int maxp = 0, maxw = 0;
    cudaDeviceGetAttribute(&maxp, cudaDevAttrMaxPersistingL2CacheSize, ctx->device);
    cudaDeviceGetAttribute(&maxw, cudaDevAttrMaxAccessPolicyWindowSize, ctx->device);
    const bool fn = variant == 2 || variant == 4 || variant == 5;
    const size_t bytes =
        std::min<size_t>((size_t)sg->view.num_nodes * (fn ? sizeof(WideNodeF) : sizeof(WideNode)), (size_t)maxw);
    if (maxp > 0 && bytes > 0) {
      cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, std::min<size_t>(bytes, (size_t)maxp));
      cudaStreamAttrValue a{};
      a.accessPolicyWindow.base_ptr = fn ? (void *)sg->view.fnodes : (void *)sg->view.nodes;
      a.accessPolicyWindow.num_bytes = bytes;
      a.accessPolicyWindow.hitRatio = std::min(1.0f, (float)maxp / (float)bytes);
      a.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
      a.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
      cudaStreamSetAttribute(st, cudaStreamAttributeAccessPolicyWindow, &a);
    }
  }
  struct L2Restore {
    bool on;
    cudaStream_t st;
    ~L2Restore() {
      if (!on) return;
      cudaStreamAttrValue a{};
      a.accessPolicyWindow.num_bytes = 0;
      cudaStreamSetAttribute(st, cudaStreamAttributeAccessPolicyWindow, &a);
      cudaCtxResetPersistingL2Cache();
      cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, 0);
    }
  } l2restore{l2win, st};
  const bool timek = (prm->flags & OR3_FLAG_TIME_KERNELS) != 0;
  const bool countk = (prm->flags & OR3_FLAG_COUNT_TRAVERSAL) != 0;
  const bool shadows = prm->next_event_estimation && (sg->view.num_lights > 0 || sg->view.env_light != 0);
  // sized for the shade instance launch_shade picks
  const bool nee4 = (prm->tuning & OR3_TUNE_SHADE_NEE_OCC4) != 0;
  const int grid_sh = ctx->num_sms * (shadows && !nee4 ? ctx->occ_shade_nee : ctx->occ_shade);
  // material-sorted shade (classify, then one kernel instance per class
  // list): the default where vertices sample lights, whose shade kernel then
  // no longer carries the misses (measured +3.2% on the terrain); without
  // light sampling it costs more than it saves (-5.6% on the mesh)
  const bool sorted_shade = (prm->tuning & OR3_TUNE_SORTED_SHADE) != 0 ||
                            (shadows && !(prm->tuning & OR3_TUNE_UNSORTED_SHADE));

  // a depth bound of at most 32 enqueues every bounce of a wave at once
  const bool whole = prm->max_depth > 0 && prm->max_depth <= 32;
  const int chunk = whole ? prm->max_depth : 8;
  // extra wave lanes: waves round robin over 1 + nx streams (not where a
  // wave's paths or per-kernel times are read back)
  const bool multi = !(prm->tuning & OR3_TUNE_ONE_LANE) &&
                     !(prm->flags & (OR3_FLAG_KEEP_PATHS | OR3_FLAG_TIME_KERNELS | OR3_FLAG_COUNT_TRAVERSAL));
  int nx = !multi ? 0 : (prm->tuning & OR3_TUNE_TWO_LANES) ? 1 : (prm->tuning & OR3_TUNE_FOUR_LANES) ? 3 : 2;
  Queues qx[kExtraLanes] = {};
  for (int k = 0; k < nx; k++) {
    or3_context::Lane &L = ctx->xl[k];
    if ((rc = ensure_lane(ctx, k, max_wave_paths, rays, npix))) {
      if (rc != OR3_ERR_OUT_OF_MEMORY) return rc;
      // no room for another lane's queues: render on the lanes that fit
      cudaGetLastError();
      free_lane_buffers(L);
      ctx->err.clear();
      nx = k;
      break;
    }
    qx[k] = lane_queues(L);
    qx[k].capacity = (uint32_t)std::min<uint64_t>(qx[k].capacity, rays);
    OR3_CUDA(ctx, cudaMemsetAsync(L.pix_sum, 0, npix * 3 * sizeof(double), st));
    OR3_CUDA(ctx, cudaMemsetAsync(L.pix_sumsq, 0, npix * 3 * sizeof(double), st));
    OR3_CUDA(ctx, cudaMemsetAsync(L.counters, 0, 16 * sizeof(uint32_t), st));
    OR3_CUDA(ctx, cudaMemsetAsync(L.dstats, 0, 8 * sizeof(unsigned long long), st));
  }

  const bool two = nx > 0;

  or3_render_stats stats{};
  ctx->moments_valid = false;
  ctx->last_kept_paths = (prm->flags & OR3_FLAG_KEEP_PATHS) != 0;
  std::memset(ctx->host_counters, 0, 32 * sizeof(uint32_t));  // no stale error bits from an earlier render
  auto wall0 = std::chrono::steady_clock::now();
  int32_t prev = 0;
  int passes = 0;
  bool stopped = false;
  for (int32_t next = prm->min_samples; next <= prm->max_samples; next += prm->step_samples) {
    if (ctx->stop.load()) { stopped = true; break; }
    size_t kused = 0;  // timing events used in this pass
    OR3_CUDA(ctx, cudaEventRecord(ctx->ev0, st));
    if (two) {
      OR3_CUDA(ctx, cudaEventRecord(ctx->ev_fork, st));
      for (int k = 0; k < nx; k++) OR3_CUDA(ctx, cudaStreamWaitEvent(ctx->xl[k].stream, ctx->ev_fork, 0));
    }
    // The pass's waves: whole samples of the image, or row chunks of one sample.
    std::vector<Wave> pw;
    for (uint32_t s = (uint32_t)prev; s < (uint32_t)next;) {
      const uint32_t ns = (uint32_t)std::min<uint64_t>(ns_per_wave, (uint64_t)next - s);
      for (uint64_t p0 = 0; p0 < npix; p0 += npix_per_wave) {
        const uint64_t np = std::min<uint64_t>(npix_per_wave, npix - p0);
        Wave w{};
        w.g_first = ((uint64_t)s * npix + p0) * ss2;
        w.num_paths = (uint32_t)(ns * np * ss2);
        w.pass_first = (uint32_t)prev;
        w.pix0 = (uint32_t)p0;
        w.npix = (uint32_t)np;
        w.ns = ns;
        pw.push_back(w);
      }
      s += ns;
    }
    // Waves go round robin to the lanes.  Bounces are enqueued in chunks
    // without a host round trip: every kernel reads its queue length on the
    // device, so a bounce after the last ray is a few empty launches.  With a
    // depth bound of at most 32 the chunk is the whole path and nothing is
    // read back; without one each lane's live count is read after each chunk
    // of 8, the host visiting the lanes in turn while the others run.
    const int nlanes = 1 + nx;
    struct LaneRun {
      int wave = -1, in = 0, chunks = 0;
    } lr[1 + kExtraLanes];
    size_t next_wave = 0;
    auto lane_q = [&](int l) -> const Queues & { return l ? qx[l - 1] : q; };
    auto lane_st = [&](int l) { return l ? ctx->xl[l - 1].stream : st; };
    auto lane_hc = [&](int l) { return l ? ctx->host_counters + 8 + 4 * (l - 1) : ctx->host_counters; };
    auto enqueue_chunk = [&](int l) -> int {
      const Queues &ql = lane_q(l);
      cudaStream_t sl = lane_st(l);
      const Wave &w = pw[(size_t)lr[l].wave];
      for (int b = 0; b < chunk; b++) {
        cudaEvent_t e4[4] = {};
        if (timek) {  // one lane only
          while (ctx->kpool.size() < kused + 4) {
            cudaEvent_t e;
            OR3_CUDA(ctx, cudaEventCreate(&e));
            ctx->kpool.push_back(e);
          }
          for (int k = 0; k < 4; k++) e4[k] = ctx->kpool[kused + k];
          kused += 4;
        }
        const int in = lr[l].in;
        if (timek) OR3_CUDA(ctx, cudaEventRecord(e4[0], st));
        launch_extend(sg->view, ql, in, grid_ext, block, smem_nodes, countk, variant, sl);
        if (timek) OR3_CUDA(ctx, cudaEventRecord(e4[1], st));
        if (sorted_shade) {
          launch_shade_sorted(sg->view, rcst, w, ql, in, ctx->num_sms * 8, ctx->num_sms * ctx->occ_shade_nee,
                              ctx->num_sms * ctx->occ_shade, sl);
          stats.kernel_launches += shadows ? 2 : 1;
        } else {
          launch_shade(sg->view, rcst, w, ql, in, grid_sh, block, sl, nee4,
                       (prm->tuning & OR3_TUNE_BLOCK_APPEND) != 0);
        }
        if (timek) OR3_CUDA(ctx, cudaEventRecord(e4[2], st));
        if (shadows)
          launch_shadow(sg->view, ql, grid_ext, (prm->tuning & OR3_TUNE_SHADOW_UNSORTED) != 0, variant == 6, sl,
                        wide8, (prm->tuning & OR3_TUNE_SHADOW_REFILL8) != 0);
        if (timek) OR3_CUDA(ctx, cudaEventRecord(e4[3], st));
        launch_reset_count(ql, in, sl);
        lr[l].in ^= 1;
        stats.kernel_launches += shadows ? 4 : 3;
        stats.extend_launches++;
        stats.shade_launches++;
        if (shadows) stats.shadow_launches++;
      }
      lr[l].chunks++;
      if (!whole) {
        OR3_CUDA(ctx, cudaMemcpyAsync(lane_hc(l), ql.counters, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, sl));
        OR3_CUDA(ctx, cudaEventRecord(ctx->ev_poll[l], sl));
      }
      return OR3_OK;
    };
    auto finish_wave = [&](int l) {
      const Wave &w = pw[(size_t)lr[l].wave];
      const uint64_t np = w.npix;
      double *lsum = l ? ctx->xl[l - 1].pix_sum : ctx->pix_sum;
      double *lsq = l ? ctx->xl[l - 1].pix_sumsq : ctx->pix_sumsq;
      launch_accumulate(lane_q(l), w, ss2, lsum, lsq, (int)std::min<uint64_t>((np + 7) / 8, (uint64_t)ctx->num_sms * 64),
                        block, lane_st(l));
      stats.kernel_launches++;
      if (optimistic) {
        launch_wave_check(lane_q(l), ctx->wave_fail, fail_cap, (uint32_t)lr[l].wave, lane_st(l));
        stats.kernel_launches++;
      }
      stats.waves++;
      stats.camera_paths += w.num_paths;
      ctx->last_wave_paths = w.num_paths;
      lr[l].wave = -1;
    };
    // starts the next wave on lane l (whole mode: the wave in full); false when none is left
    auto start_wave = [&](int l, int *rc_out) -> bool {
      *rc_out = OR3_OK;
      if (next_wave >= pw.size()) return false;
      if (next_wave > 0 && ctx->stop.load()) {
        stopped = true;
        return false;
      }
      lr[l].wave = (int)next_wave++;
      lr[l].in = 0;
      lr[l].chunks = 0;
      launch_raygen(rcst, pw[(size_t)lr[l].wave], lane_q(l), 0, 0, block, lane_st(l));
      stats.kernel_launches++;
      if ((*rc_out = enqueue_chunk(l))) return false;
      if (whole) finish_wave(l);
      return true;
    };
    if (!whole) {
      for (int l = 0; l < nlanes; l++)
        if (!ctx->ev_poll[l]) OR3_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_poll[l], cudaEventDisableTiming));
    }
    int live = 0;
    for (int l = 0; l < nlanes; l++) {
      int r = OR3_OK;
      if (start_wave(l, &r)) live++;
      if (r) return r;
    }
    if (whole) {
      for (int l = 0;; l = (l + 1) % nlanes) {
        int r = OR3_OK;
        if (!start_wave(l, &r)) {
          if (r) return r;
          break;
        }
      }
    } else {
      bool dev_error = false;
      while (live > 0) {
        for (int l = 0; l < nlanes; l++) {
          if (lr[l].wave < 0) continue;
          OR3_CUDA(ctx, cudaEventSynchronize(ctx->ev_poll[l]));
          const uint32_t *hc = lane_hc(l);
          // a queue overflow only spoils its own wave (re-rendered at the end of the pass)
          if (hc[2] & (optimistic ? ~kErrQueue : ~0u)) dev_error = true;
          if (!dev_error && hc[lr[l].in] != 0 && lr[l].chunks < 100000) {
            if (int r = enqueue_chunk(l)) return r;
            continue;
          }
          finish_wave(l);
          live--;
          int r = OR3_OK;
          if (!dev_error && start_wave(l, &r)) live++;
          if (r) return r;
        }
      }
    }
    for (int k = 0; k < nx; k++) {  // join the extra lanes and fold their pixel sums into lane 0's
      or3_context::Lane &L = ctx->xl[k];
      OR3_CUDA(ctx, cudaEventRecord(ctx->ev_join[k], L.stream));
      OR3_CUDA(ctx, cudaStreamWaitEvent(st, ctx->ev_join[k], 0));
      launch_merge_sums(npix * 3, ctx->pix_sum, ctx->pix_sumsq, L.pix_sum, L.pix_sumsq, ctx->num_sms * 16, st);
      stats.kernel_launches++;
      OR3_CUDA(ctx, cudaMemcpyAsync(ctx->host_counters + 8 + 4 * k, L.counters, 4 * sizeof(uint32_t),
                                    cudaMemcpyDeviceToHost, st));
    }
    // Waves whose ray queue overflowed (glass splits beyond kSplitQueueFactor
    // rays per path) were not accumulated: each is rendered again, on lane 0,
    // in sub-waves of whole pixels and one sample that cannot overflow.  The
    // paths and their random numbers are the same, so is the image.
    if (optimistic && !stopped) {
      uint32_t *hf = ctx->host_counters + 28;
      OR3_CUDA(ctx, cudaMemcpyAsync(hf, ctx->wave_fail, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
      OR3_CUDA(ctx, cudaStreamSynchronize(st));
      const uint32_t nf = *hf;
      if (nf > fail_cap) return fail(ctx, OR3_ERR_DEVICE_REPORTED, "overflow list full (%u waves)", nf);
      if (nf) {
        std::vector<uint32_t> ids(nf);
        OR3_CUDA(ctx, cudaMemcpy(ids.data(), ctx->wave_fail + 1, nf * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        OR3_CUDA(ctx, cudaMemsetAsync(ctx->wave_fail, 0, sizeof(uint32_t), st));
        const size_t first_sub = pw.size();
        for (uint32_t id : ids) {
          const Wave w = pw[id];
          stats.camera_paths -= w.num_paths;
          stats.waves--;
          stats.waves_rerun++;
          const uint64_t s0 = w.g_first / (npix * ss2);
          for (uint32_t j = 0; j < w.ns; j++) {
            for (uint64_t a = w.pix0; a < (uint64_t)w.pix0 + w.npix; a += safe_pix) {
              Wave sw = w;
              sw.ns = 1;
              sw.pix0 = (uint32_t)a;
              sw.npix = (uint32_t)std::min<uint64_t>(safe_pix, (uint64_t)w.pix0 + w.npix - a);
              sw.g_first = ((s0 + j) * npix + a) * ss2;
              sw.num_paths = sw.npix * ss2;
              pw.push_back(sw);
            }
          }
        }
        for (size_t k = first_sub; k < pw.size(); k++) {
          lr[0].wave = (int)k;
          lr[0].in = 0;
          lr[0].chunks = 0;
          launch_raygen(rcst, pw[k], q, 0, 0, block, st);
          stats.kernel_launches++;
          for (;;) {
            if (int r = enqueue_chunk(0)) return r;
            if (whole) break;
            OR3_CUDA(ctx, cudaEventSynchronize(ctx->ev_poll[0]));
            const uint32_t *hc = lane_hc(0);
            if (hc[2] || hc[lr[0].in] == 0 || lr[0].chunks >= 100000) break;  // other errors: reported below
          }
          finish_wave(0);
        }
        OR3_CUDA(ctx, cudaMemcpyAsync(hf, ctx->wave_fail, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        OR3_CUDA(ctx, cudaStreamSynchronize(st));
        if (*hf) return fail(ctx, OR3_ERR_DEVICE_REPORTED, "ray queue capacity exceeded by a sub-wave");
      }
    }
    // error bits of the pass (queue capacity, traversal stack)
    OR3_CUDA(ctx, cudaMemcpyAsync(ctx->host_counters, ctx->counters, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                  st));
    OR3_CUDA(ctx, cudaEventRecord(ctx->ev1, st));
    OR3_CUDA(ctx, cudaEventSynchronize(ctx->ev1));
    for (size_t k = 0; k + 3 < kused; k += 4) {
      float e = 0.f, s2 = 0.f, s3 = 0.f;
      cudaEventElapsedTime(&e, ctx->kpool[k], ctx->kpool[k + 1]);
      cudaEventElapsedTime(&s2, ctx->kpool[k + 1], ctx->kpool[k + 2]);
      cudaEventElapsedTime(&s3, ctx->kpool[k + 2], ctx->kpool[k + 3]);
      stats.extend_ms += e;
      stats.shade_ms += s2;
      if (shadows) stats.shadow_ms += s3;
    }
    uint32_t errbits = ctx->host_counters[2];
    for (int k = 0; k < nx; k++) errbits |= ctx->host_counters[8 + 4 * k + 2];
    if (errbits) {
      const uint32_t bits = errbits;
      cudaMemsetAsync(ctx->counters, 0, 16 * sizeof(uint32_t), st);
      for (int k = 0; k < nx; k++) cudaMemsetAsync(ctx->xl[k].counters, 0, 16 * sizeof(uint32_t), st);
      cudaStreamSynchronize(st);
      return fail(ctx, OR3_ERR_DEVICE_REPORTED, "kernel reported error bits 0x%x (%s)", bits,
                  (bits & kErrQueue) ? "ray queue capacity" : "traversal stack");
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    stats.render_ms += ms;
    if (stopped) break;
    passes++;
    // frame = running mean over `next` samples (PathTracer.cpp:169-170)
    const double scale = 1.0 / ((double)next * ss2);
    launch_frame(ctx->pix_sum, W, H, prm->output_layout, scale, ctx->frame_dev, st);
    stats.kernel_launches++;
    if (frame_doubles > ctx->cap_back) {  // the back buffer is never read by another thread
      cudaStreamSynchronize(st);
      cudaFreeHost(ctx->frame_pinned);
      ctx->frame_pinned = nullptr;
      ctx->cap_back = 0;
      OR3_CUDA(ctx, cudaMallocHost(&ctx->frame_pinned, frame_doubles * sizeof(double)));
      ctx->cap_back = frame_doubles;
    }
    OR3_CUDA(ctx, cudaMemcpyAsync(ctx->frame_pinned, ctx->frame_dev, frame_doubles * sizeof(double),
                                  cudaMemcpyDeviceToHost, st));
    OR3_CUDA(ctx, cudaStreamSynchronize(st));
    {
      std::lock_guard<std::mutex> lk(ctx->frame_mu);
      std::swap(ctx->frame_pinned, ctx->frame_front);
      std::swap(ctx->cap_back, ctx->cap_front);
      ctx->front_doubles = frame_doubles;
      ctx->frame_samples = next;
    }
    ctx->last_count = (uint64_t)next * ss2;
    prev = next;
    if (cb) {  // the front frame changes only in this thread, after the callback returns
      const double minutes =
          std::chrono::duration<double>(std::chrono::steady_clock::now() - wall0).count() / 60.0;
      cb(user, next, ctx->frame_front, (prm->output_layout == OR3_LAYOUT_REFERENCE ? 2 : 1) * (size_t)W,
         (size_t)H, minutes);
    }
  }
  unsigned long long hs[8];
  OR3_CUDA(ctx, cudaMemcpy(hs, ctx->dstats, sizeof(hs), cudaMemcpyDeviceToHost));
  for (int k = 0; k < nx; k++) {
    unsigned long long h1[8];
    OR3_CUDA(ctx, cudaMemcpy(h1, ctx->xl[k].dstats, sizeof(h1), cudaMemcpyDeviceToHost));
    for (int j = 0; j < 8; j++) hs[j] += h1[j];
  }
  stats.lanes = (uint32_t)(1 + nx);
  stats.extension_rays = hs[0];
  stats.shadow_rays = hs[1];
  stats.bounces = hs[2];
  stats.nodes_visited = hs[3];
  stats.tris_tested = hs[4];
  stats.spheres_tested = hs[5];
  stats.samples = prev;
  if (stats.waves_rerun && sg->split_factor < 8u) sg->split_factor *= 2u;  // the scene's next renders
  stats.passes = passes;
  stats.upload_ms = sg->info.build_ms + sg->info.upload_ms;
  ctx->last = stats;
  ctx->last_W = W;
  ctx->last_H = H;
  ctx->moments_valid = !stopped;
  return OR3_OK;
}

namespace {
// Host copy of a frame: large frames (a 1024x768 reference-layout frame is
// 37.7 MB) are cut into 64-byte-aligned pieces copied on up to 8 host threads.
void copy_frame(void *dst, const void *src, size_t bytes) {
  constexpr size_t kPiece = 4u << 20;
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const unsigned nt = (unsigned)std::min<size_t>({(size_t)8, (size_t)hw, bytes / kPiece});
  if (nt <= 1) {
    std::memcpy(dst, src, bytes);
    return;
  }
  const size_t per = (bytes / nt + 63) & ~(size_t)63;
  auto part = [&](unsigned k) {
    const size_t b = std::min(bytes, per * k), e = std::min(bytes, b + per);
    std::memcpy(static_cast<char *>(dst) + b, static_cast<const char *>(src) + b, e - b);
  };
  std::vector<std::thread> th;
  th.reserve(nt - 1);
  for (unsigned k = 1; k < nt; k++) th.emplace_back(part, k);
  part(0);
  for (auto &t : th) t.join();
}
}  // namespace

int or3_get_frame(or3_context *ctx, double *rgb, size_t capacity, int32_t *samples_out) {
  if (!ctx) return OR3_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(ctx->frame_mu);
  if (samples_out) *samples_out = ctx->frame_samples;
  if (ctx->front_doubles == 0) return fail(ctx, OR3_ERR_NOT_FOUND, "no frame rendered yet");
  if (!rgb || capacity < ctx->front_doubles)
    return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "frame needs %zu doubles", ctx->front_doubles);
  copy_frame(rgb, ctx->frame_front, ctx->front_doubles * sizeof(double));
  return OR3_OK;
}

int or3_get_stats(or3_context *ctx, or3_render_stats *out) {
  if (!ctx || !out) return OR3_ERR_INVALID_ARGUMENT;
  *out = ctx->last;
  return OR3_OK;
}

int or3_get_moments(or3_context *ctx, double *sum, double *sumsq, size_t capacity, uint64_t *count_out) {
  if (!ctx) return OR3_ERR_INVALID_ARGUMENT;
  if (!ctx->moments_valid) return fail(ctx, OR3_ERR_NOT_FOUND, "no completed render");
  const size_t n = (size_t)ctx->last_W * ctx->last_H * 3;
  if (capacity < n) return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "moments need %zu doubles", n);
  cudaSetDevice(ctx->device);
  double *tmp = nullptr;
  OR3_CUDA(ctx, cudaMalloc(&tmp, 2 * n * sizeof(double)));
  launch_moments(ctx->pix_sum, ctx->pix_sumsq, ctx->last_W, ctx->last_H, tmp, tmp + n, ctx->stream);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e == cudaSuccess && sum) e = cudaMemcpy(sum, tmp, n * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && sumsq) e = cudaMemcpy(sumsq, tmp + n, n * sizeof(double), cudaMemcpyDeviceToHost);
  cudaFree(tmp);
  if (e != cudaSuccess) return fail(ctx, OR3_ERR_CUDA, "moments: %s", cudaGetErrorString(e));
  if (count_out) *count_out = ctx->last_count;
  return OR3_OK;
}

int or3_get_path_radiance(or3_context *ctx, float *rgb, size_t capacity, uint64_t *paths_out) {
  if (!ctx) return OR3_ERR_INVALID_ARGUMENT;
  if (!ctx->last_kept_paths || ctx->last_wave_paths == 0)
    return fail(ctx, OR3_ERR_NOT_FOUND, "render with OR3_FLAG_KEEP_PATHS first");
  const size_t n = ctx->last_wave_paths;
  if (paths_out) *paths_out = n;
  if (!rgb) return OR3_OK;
  if (capacity < 3 * n) return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "path radiance needs %zu floats", 3 * n);
  std::vector<float4> tmp(n);
  OR3_CUDA(ctx, cudaMemcpy(tmp.data(), ctx->pathL, n * sizeof(float4), cudaMemcpyDeviceToHost));
  for (size_t i = 0; i < n; i++) {
    rgb[3 * i] = tmp[i].x;
    rgb[3 * i + 1] = tmp[i].y;
    rgb[3 * i + 2] = tmp[i].z;
  }
  return OR3_OK;
}

int or3_trace_closest_device(or3_context *ctx, int32_t scene, size_t n, const float *o, const float *d,
                             int32_t *prim, float *t, float *normal, void *stream) {
  if (!ctx || (n && (!o || !d || !prim || !t))) return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "null argument");
  auto it = ctx->scenes.find(scene);
  if (it == ctx->scenes.end()) return fail(ctx, OR3_ERR_NOT_FOUND, "scene %d not found", scene);
  if (n == 0) return OR3_OK;
  cudaSetDevice(ctx->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  launch_trace_closest(it->second->view, n, o, d, prim, t, normal, ctx->counters, st);
  OR3_CUDA(ctx, cudaGetLastError());
  return OR3_OK;
}

int or3_trace_closest(or3_context *ctx, int32_t scene, size_t n, const float *o, const float *d, int32_t *prim,
                      float *t, float *normal) {
  if (!ctx || (n && (!o || !d || !prim || !t))) return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "null argument");
  if (ctx->scenes.find(scene) == ctx->scenes.end()) return fail(ctx, OR3_ERR_NOT_FOUND, "scene %d not found", scene);
  if (n == 0) return OR3_OK;
  cudaSetDevice(ctx->device);
  char *buf = nullptr;
  const size_t bytes = n * (3 + 3 + 1 + 1 + 3) * 4;
  OR3_CUDA(ctx, cudaMalloc(&buf, bytes));
  float *od = (float *)buf, *dd = od + 3 * n, *td = dd + 3 * n, *nd = td + n;
  int32_t *pd = (int32_t *)(nd + 3 * n);
  cudaStream_t st = ctx->stream;
  cudaMemcpyAsync(od, o, 3 * n * 4, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dd, d, 3 * n * 4, cudaMemcpyHostToDevice, st);
  int rc = or3_trace_closest_device(ctx, scene, n, od, dd, pd, td, nd, st);
  if (rc == OR3_OK) {
    cudaMemcpyAsync(prim, pd, n * 4, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(t, td, n * 4, cudaMemcpyDeviceToHost, st);
    if (normal) cudaMemcpyAsync(normal, nd, 3 * n * 4, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(ctx->host_counters, ctx->counters, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = fail(ctx, OR3_ERR_CUDA, "trace: %s", cudaGetErrorString(e));
    else if (ctx->host_counters[2]) rc = fail(ctx, OR3_ERR_DEVICE_REPORTED, "traversal stack overflow");
  }
  cudaFree(buf);
  return rc;
}

int or3_render_paths_noalloc(or3_context *ctx, int32_t scene, const or3_camera *cam, const or3_render_params *prm,
                             uint64_t first, uint32_t num_paths, float *radiance_dev, void *stream) {
  if (!ctx || !cam || !prm || (num_paths && !radiance_dev))
    return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "null argument");
  if (num_paths > OR3_NOALLOC_MAX_PATHS)
    return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "num_paths %u exceeds the no-alloc scratch limit of %u paths",
                num_paths, OR3_NOALLOC_MAX_PATHS);
  auto it = ctx->scenes.find(scene);
  if (it == ctx->scenes.end()) return fail(ctx, OR3_ERR_NOT_FOUND, "scene %d not found", scene);
  if (cam->width == 0 || cam->height == 0 || prm->supersamples < 1 || prm->supersamples > 256 ||
      prm->min_samples < 1 || prm->max_samples < prm->min_samples || prm->step_samples < 1)
    return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "invalid camera or sample schedule");
  if (num_paths == 0) return OR3_OK;
  const uint64_t ss2 = (uint64_t)prm->supersamples * prm->supersamples;
  const uint64_t per_sample = (uint64_t)cam->width * cam->height * ss2;
  const uint64_t total = per_sample * (uint64_t)prm->max_samples;
  if (first + num_paths > total)
    return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "paths [%llu, +%u) outside the %llu paths of the render",
                (unsigned long long)first, num_paths, (unsigned long long)total);
  // the pass [prev, next) holding the first path; the range must not leave it
  const uint64_t s0 = first / per_sample, s1 = (first + num_paths - 1) / per_sample;
  int32_t prev = 0, next = prm->min_samples;
  while ((uint64_t)next <= s0 && next + prm->step_samples <= prm->max_samples) {
    prev = next;
    next += prm->step_samples;
  }
  if (s1 >= (uint64_t)next) return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "path range spans two passes");
  RenderConst rc{};
  camera_basis(cam, rc.cam);
  rc.W = cam->width;
  rc.H = cam->height;
  rc.ss = (uint32_t)prm->supersamples;
  rc.ss2 = (uint32_t)ss2;
  rc.nee = prm->next_event_estimation;
  rc.rr_min_depth = prm->rr_min_depth;
  rc.max_depth = prm->max_depth;
  rc.seed_lo = (uint32_t)prm->seed;
  rc.seed_hi = (uint32_t)(prm->seed >> 32);
  // the caller's current device is put back before returning
  int caller_device = -1;
  if (cudaGetDevice(&caller_device) != cudaSuccess) caller_device = -1;
  cudaSetDevice(ctx->device);
  std::string err;
  const int rcode = render_paths_noalloc(it->second->view, it->second->has_split, rc, first, num_paths,
                                         (uint32_t)prev, ctx->device, ctx->num_sms * ctx->occ_extend,
                                         ctx->num_sms * (rc.nee ? ctx->occ_shade_nee : ctx->occ_shade), radiance_dev,
                                         stream ? (cudaStream_t)stream : ctx->stream, &err);
  if (caller_device >= 0 && caller_device != ctx->device) cudaSetDevice(caller_device);
  if (rcode != OR3_OK) return fail(ctx, rcode, "%s", err.c_str());
  return OR3_OK;
}

}  // extern "C"

// Shared by or3_env_sample / or3_texture_sample: n inputs of `in_floats`
// floats each to the device, one lookup kernel, 3 floats each back.
template <class Launch>
static int lookup_query(or3_context *ctx, size_t n, const float *in, size_t in_floats, float *rgb, Launch launch) {
  char *buf = nullptr;
  OR3_CUDA(ctx, cudaMalloc(&buf, n * (in_floats + 3) * sizeof(float)));
  float *ind = (float *)buf, *outd = ind + in_floats * n;
  cudaStream_t st = ctx->stream;
  cudaError_t e = cudaMemcpyAsync(ind, in, n * in_floats * sizeof(float), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    launch((uint32_t)n, ind, outd, st);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(rgb, outd, n * 3 * sizeof(float), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(buf);
  if (e != cudaSuccess) return fail(ctx, OR3_ERR_CUDA, "lookup: %s", cudaGetErrorString(e));
  return OR3_OK;
}

extern "C" {

int or3_env_sample(or3_context *ctx, int32_t scene, size_t n, const float *dirs, float *rgb) {
  if (!ctx || (n && (!dirs || !rgb))) return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "null argument");
  auto it = ctx->scenes.find(scene);
  if (it == ctx->scenes.end()) return fail(ctx, OR3_ERR_NOT_FOUND, "scene %d not found", scene);
  if (n >= ((size_t)1 << 31)) return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "n too large");
  if (n == 0) return OR3_OK;
  cudaSetDevice(ctx->device);
  const DevScene S = it->second->view;
  return lookup_query(ctx, n, dirs, 3, rgb, [&](uint32_t m, const float *i, float *o, cudaStream_t st) {
    launch_env_sample(S, m, i, o, st);
  });
}

int or3_texture_sample(or3_context *ctx, int32_t scene, int32_t texture, size_t n, const float *uv, float *rgb) {
  if (!ctx || (n && (!uv || !rgb))) return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "null argument");
  auto it = ctx->scenes.find(scene);
  if (it == ctx->scenes.end()) return fail(ctx, OR3_ERR_NOT_FOUND, "scene %d not found", scene);
  const DevScene S = it->second->view;
  if (texture < 0 || (uint32_t)texture >= S.num_textures)
    return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "texture %d not in the scene (%u textures)", texture, S.num_textures);
  if (n >= ((size_t)1 << 31)) return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "n too large");
  if (n == 0) return OR3_OK;
  cudaSetDevice(ctx->device);
  return lookup_query(ctx, n, uv, 2, rgb, [&](uint32_t m, const float *i, float *o, cudaStream_t st) {
    launch_texture_sample(S, texture, m, i, o, st);
  });
}

int or3_trace_occluded(or3_context *ctx, int32_t scene, size_t n, const float *o, const float *d,
                       const float *tmax, uint8_t *occ) {
  if (!ctx || (n && (!o || !d || !tmax || !occ))) return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "null argument");
  auto it = ctx->scenes.find(scene);
  if (it == ctx->scenes.end()) return fail(ctx, OR3_ERR_NOT_FOUND, "scene %d not found", scene);
  if (n == 0) return OR3_OK;
  cudaSetDevice(ctx->device);
  char *buf = nullptr;
  OR3_CUDA(ctx, cudaMalloc(&buf, n * 7 * 4 + n));
  float *od = (float *)buf, *dd = od + 3 * n, *tm = dd + 3 * n;
  uint8_t *oc = (uint8_t *)(tm + n);
  cudaStream_t st = ctx->stream;
  cudaMemcpyAsync(od, o, 3 * n * 4, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dd, d, 3 * n * 4, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(tm, tmax, n * 4, cudaMemcpyHostToDevice, st);
  launch_trace_occluded(it->second->view, n, od, dd, tm, oc, ctx->counters, st);
  cudaMemcpyAsync(occ, oc, n, cudaMemcpyDeviceToHost, st);
  cudaError_t e = cudaStreamSynchronize(st);
  cudaFree(buf);
  if (e != cudaSuccess) return fail(ctx, OR3_ERR_CUDA, "occluded: %s", cudaGetErrorString(e));
  return OR3_OK;
}

}  // extern "C"
