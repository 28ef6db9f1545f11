/*
 * or3.h -- C ABI of the GB300 path-tracing hot path (libor3.so).
 *
 * This is the drop-in boundary for omochi-renderer3's render call.  The
 * reference renders through the abstract `Renderer` interface
 * (src/renderer/Renderer.h:10-23), implemented by `PathTracer`
 * (src/renderer/PathTracer.h:18-88).  A C++ host class mirrors that interface
 * on top of the functions below (omochi-renderer3_gb300/host/GpuPathTracer.hpp),
 * so the reference's `main` changes by one line.
 *
 * Conventions
 *   - Every function returns an int status: OR3_OK (0) or a negative OR3_ERR_*
 *     code.  No exception or abort crosses the ABI; or3_last_error() gives the
 *     message of the last failure on a context.
 *   - Scene data enters in the reference's own precision (double) and layout
 *     conventions; the library flattens and converts it (FP32 on the device).
 *   - Pointers named *_host are host memory, *_dev are device memory of the
 *     context's GPU.
 *   - A context is used from one host thread at a time, except or3_stop() and
 *     or3_get_frame(), which may be called from other threads while
 *     or3_render() runs (the reference's timer and saver threads do this:
 *     src/tools/StopRendererWithTimer.cpp:38-40,
 *     src/tools/FileSaverCallerWithTimer.cpp:59-66).
 */
#ifndef OR3_H_
#define OR3_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OR3_API_VERSION 1

/* ---- status codes ------------------------------------------------------ */
#define OR3_OK 0
#define OR3_ERR_INVALID_ARGUMENT (-1)
#define OR3_ERR_CUDA (-2)
#define OR3_ERR_OUT_OF_MEMORY (-3)
#define OR3_ERR_NO_DEVICE (-4)
#define OR3_ERR_NOT_FOUND (-5)
/* A kernel reported an internal limit (traversal stack, queue capacity,
   bounded wait); the context stays usable. */
#define OR3_ERR_DEVICE_REPORTED (-6)
#define OR3_ERR_BUSY (-7)

/* ---- materials (src/renderer/Material.h:9-36) --------------------------- */
#define OR3_LAMBERT 0    /* REFLECTION_TYPE_LAMBERT */
#define OR3_SPECULAR 1   /* REFLECTION_TYPE_SPECULAR */
#define OR3_REFRACTION 2 /* REFLECTION_TYPE_REFRACTION */
#define OR3_PHONG 3      /* glossy lobe; no counterpart in the reference */

typedef struct or3_material {
  int32_t type;          /* OR3_LAMBERT .. OR3_PHONG */
  int32_t texture;       /* index into or3_scene_desc textures, -1 = none */
  double emission[3];    /* Material::emission */
  double color[3];       /* Material::color */
  double ior;            /* Material::refraction_rate */
  double phong_exponent; /* OR3_PHONG only */
} or3_material;

/* ---- flattened scene ---------------------------------------------------
 * One record per reference SceneObject.  `id` fields give the object's
 * insertion index in the reference Scene (AddObject order,
 * src/scenes/Scene.h:48-59); closest-hit queries return these ids, so they
 * compare one-to-one with the reference's `IntersectionInformation::object`.
 * If an id array is NULL the ids are 0..n-1 per primitive class, offset by
 * the counts of the classes before it (triangles, spheres, planes).
 *
 * Each object has a list of material layers chosen by roulette with the
 * given rates (SceneObject::MultiMaterialElem, src/renderer/SceneObject.h:17-67);
 * `*_layers` holds [begin, count] into layer_material/layer_rate.
 */
#define OR3_SPHERE_LIGHT 1u   /* sphere_flags bit: a SphereLight (src/renderer/SphereLight.h:8) */

#define OR3_PLANE_AXIS_ALIGNED 0 /* AxisAlignedPlane (src/renderer/AxisAlignedPlane.h:9-70) */
#define OR3_PLANE_INFINITE_FLOOR 1 /* InfiniteFloor (src/renderer/InfiniteFloor.h:11-42) */

typedef struct or3_scene_desc {
  uint32_t num_materials;
  const or3_material *materials;
  uint32_t num_layers;
  const uint32_t *layer_material; /* [num_layers] */
  const double *layer_rate;       /* [num_layers], normalised per object */

  /* Polygon (src/renderer/Polygon.h:11-136), in BVH */
  uint32_t num_triangles;
  const double *tri_vertices; /* [n][3][3] world positions (pos_i + position_) */
  const double *tri_normals;  /* [n][3][3] per-vertex normals, NULL = face normal */
  const double *tri_uvs;      /* [n][3][2], NULL = zero */
  const uint32_t *tri_layers; /* [n][2] */
  const uint32_t *tri_ids;    /* [n] or NULL */

  /* Sphere / SphereLight (src/renderer/Sphere.h:11-82), in BVH */
  uint32_t num_spheres;
  const double *spheres;         /* [n][4] center xyz, radius */
  const uint32_t *sphere_layers; /* [n][2] */
  const uint32_t *sphere_flags;  /* [n] OR3_SPHERE_LIGHT, or NULL */
  const uint32_t *sphere_ids;    /* [n] or NULL */

  /* objects kept out of the BVH (Scene::m_notInBVHObjects) */
  uint32_t num_planes;
  const double *planes;         /* [n][4] kind, axis(0=XY,1=XZ,2=YZ), offset, flip */
  const uint32_t *plane_layers; /* [n][2] */
  const uint32_t *plane_ids;    /* [n] or NULL */

  /* IBL equirect image (src/renderer/IBL.h:30-45), row-major: RGB float, or
     RGBE bytes (4 per texel, HDRImage's encoding, decoded on the device; see
     or3_read_hdr).  Both NULL = no IBL: misses return `background`. */
  uint32_t env_width, env_height;
  const float *env_rgb;
  const uint8_t *env_rgbe;
  double background[3];  /* Scene::Background() (src/scenes/Scene.h:40) */

  /* textures (src/tools/Image.h:20-31): RGB float, linear */
  uint32_t num_textures;
  const uint32_t *texture_dims;    /* [n][2] width, height */
  const uint64_t *texture_offsets; /* [n] float offset into texture_rgb */
  const float *texture_rgb;

  /* where the BVH is built (OR3_BUILD_*); zero-initialised = automatic */
  uint32_t build;
  /* BVH build: primitives per leaf at most (0 = 4, up to 8); SAH cost of a
     node visit relative to a primitive test (0 = 1, the reference's) */
  uint32_t leaf_max;
  double traversal_cost;
} or3_scene_desc;

/* BVH build location.  Both build the same kind of tree (binned SAH, 16 bins,
   leaves <= 4, 4-wide, 8-bit child boxes); closest hits are the same. */
#define OR3_BUILD_AUTO 0u    /* device for >= OR3_BUILD_DEVICE_MIN_PRIMS in-BVH primitives, else host */
#define OR3_BUILD_HOST 1u    /* host threads (bvh_build.cpp) */
#define OR3_BUILD_DEVICE 2u  /* the GPU (bvh_build_gpu.cu), up to 2^26 primitives */
#define OR3_BUILD_DEVICE_MIN_PRIMS 16384u

/* ---- camera (src/renderer/Camera.h:12-43, :65-93; Aperture.h:23-35) ---- */
typedef struct or3_camera {
  uint32_t width, height;
  double position[3];
  double direction[3];
  double up[3];
  double screen_height_world; /* Camera::m_nearScreenHeight */
  double distance_to_screen;  /* Camera::m_distToScreen */
  double focal_distance;      /* Camera::m_focalDistance */
  double aperture_radius;     /* CircleAperture radius, 0 = pinhole (no aperture) */
} or3_camera;

/* ---- render parameters (PathTracer ctor, src/renderer/PathTracer.h:25-37) */
#define OR3_LAYOUT_REFERENCE 0 /* 2W x H doubles, image in the left viewport, rows top-down
                                  (ScreenPixels with 2x1 viewports, src/renderer/ScreenPixels.cpp:37-65) */
#define OR3_LAYOUT_COMPACT 1   /* W x H doubles, rows top-down */

#define OR3_FLAG_KEEP_PATHS 1u   /* keep per-path radiance of the last wave (testing) */
/* bits 2 and 8 are reserved */
#define OR3_FLAG_NO_GRAPH 4u     /* batched/served forms: launch the bounce loop without a CUDA graph */
#define OR3_FLAG_TIME_KERNELS 16u      /* CUDA events around every extend/shade launch */
#define OR3_FLAG_COUNT_TRAVERSAL 32u   /* count nodes and primitives visited (slower) */
#define OR3_FLAG_ONE_LANE 64u          /* batched form: every wave on one stream (default: three that overlap) */
#define OR3_FLAG_QUANTISED_NODES 128u  /* batched form: traverse the 64-byte nodes with 8-bit child boxes
                                          (default: the 128-byte FP32-box nodes) */
#define OR3_FLAG_HOIST_NODES 256u      /* batched form: copy each ray's node array into registers when a
                                          lane takes the ray (default: read it through the ray's scene
                                          descriptor every step, which frees the registers for two node
                                          steps per warp vote) */
#define OR3_FLAG_UNSORTED_SHADE 512u   /* batched form: one shade kernel for every hit and miss (default where
                                          the batch samples lights: the material-sorted shade) */
#define OR3_FLAG_HOST_LOOP 1024u       /* batched form: the host hands out waves and replays each wave's
                                          bounce graph (default: the device runs the whole batch, each lane
                                          one graph launch whose while loop takes waves from a shared
                                          device queue); with glass it keeps queues of 8 rays per path
                                          and 2^23-path waves */

typedef struct or3_render_params {
  int32_t min_samples;   /* PathTracer m_min_samples */
  int32_t max_samples;   /* m_max_samples */
  int32_t step_samples;  /* m_step_samples */
  int32_t supersamples;  /* m_supersamples (ss x ss fixed grid per pixel) */
  int32_t next_event_estimation; /* 0 = off (the reference default);
                                    1 = one light sample per Lambert/Phong vertex with an
                                    any-hit shadow ray: emissive triangles and spheres by
                                    power, the environment by its marginal/conditional CDF.
                                    The reference's own NEE weights by the receiver's
                                    emission (PathTracer.cpp:311-314) and renders black;
                                    this is the estimator it describes, not its output. */
  int32_t rr_min_depth;  /* Russian roulette for depth > this; reference MinDepth = 5 */
  int32_t max_depth;     /* rays at depth >= max_depth are not traced; 0 = unbounded (reference) */
  int32_t output_layout; /* OR3_LAYOUT_* */
  uint64_t seed;         /* counter-based RNG key */
  uint64_t wave_paths;   /* camera paths per wave, 0 = automatic */
  uint32_t flags;        /* OR3_FLAG_* */
  uint32_t tuning;       /* 0 = defaults; OR3_TUNE_* (kernel choices, set by the autotuner) */
} or3_render_params;

#define OR3_TUNE_EXTEND_MASK 0x7u  /* extend kernel: 0 default (= 2); 1 persistent, one node or leaf per step;
                                      2 persistent, node steps with leaves in place, lanes refilled once
                                      16 are idle; 3 one ray per thread; 4, 5 as 2 refilling at 8 / 24
                                      idle lanes; 6 as 2 over the 8-bit quantised child boxes (shadow
                                      rays too); 7 as 2 with the nearest internal child next and
                                      its siblings pushed unsorted.  2, 4, 5, 7 test FP32 child
                                      boxes; 1, 3, 6 the quantised ones */
#define OR3_TUNE_SMEM_NODES 0x10u  /* stage the top quantised BVH nodes in shared memory (variants 1, 3, 6) */
#define OR3_TUNE_SHADOW_UNSORTED 0x20u /* shadow rays take children in slot order (no distance sort) */
#define OR3_TUNE_L2_PERSIST 0x40u      /* or3_render: L2 persisting access window over the BVH nodes */
#define OR3_TUNE_SHADE_NEE_OCC4 0x80u  /* or3_render: light-sampling shade kernel at 64 registers, 4 blocks/SM */
#define OR3_TUNE_ONE_LANE 0x100u       /* or3_render: all waves on one stream (no overlap of waves) */
#define OR3_TUNE_TWO_LANES 0x200u      /* or3_render: waves round robin over two streams instead of three */
#define OR3_TUNE_FOUR_LANES 0x400u     /* or3_render: waves round robin over four streams instead of three */
#define OR3_TUNE_SORTED_SHADE 0x800u   /* or3_render: material-sorted shade (misses shaded while the hits are
                                          filed by material class, then one shade kernel per class) also
                                          without light sampling; with it, it is the default */
#define OR3_TUNE_UNSORTED_SHADE 0x2000u /* or3_render: one shade kernel for every hit and miss even where
                                          vertices sample lights */
#define OR3_TUNE_WIDE8 0x4000u         /* or3_render: extension and shadow rays traverse an 8-wide tree made
                                          from the scene's 4-wide one on first use (kept with the scene) */
#define OR3_TUNE_SHADOW_REFILL8 0x8000u /* or3_render: shadow-ray warps fetch new rays once 8 lanes are idle
                                          (default 24) */
#define OR3_TUNE_BLOCK_APPEND 0x1000u  /* or3_render: the shade kernel appends rays with one atomic per block
                                          instead of one per warp */

/* Called after each pass, like PathTracer's RenderingFinishCallbackFunction
   (src/renderer/PathTracer.h:21): samples so far, the frame in the requested
   layout, its width/height in doubles-per-row / rows, accumulated minutes. */
typedef void (*or3_frame_callback)(void *user, int32_t samples, const double *rgb,
                                   size_t width, size_t height, double minutes);

typedef struct or3_render_stats {
  uint64_t camera_paths;   /* W*H*ss*ss*samples rendered */
  uint64_t extension_rays; /* closest-hit queries */
  uint64_t shadow_rays;    /* any-hit queries */
  uint64_t bounces;        /* bounce iterations launched */
  uint64_t waves;
  double render_ms;        /* device time of the passes (CUDA events) */
  double upload_ms;        /* scene upload + BVH build of the rendered scene */
  int32_t samples;         /* samples per subpixel accumulated */
  int32_t passes;
  /* OR3_FLAG_TIME_KERNELS: summed device time and launch counts */
  double extend_ms;
  double shade_ms;         /* the shade kernel (shadow rays are in shadow_ms) */
  uint64_t extend_launches;
  uint64_t shade_launches;
  /* OR3_FLAG_COUNT_TRAVERSAL: totals over all extension rays */
  uint64_t nodes_visited;  /* wide nodes fetched (128 bytes with FP32 child boxes, 64 quantised) */
  uint64_t tris_tested;    /* 48-byte triangle records tested */
  uint64_t spheres_tested; /* sphere records tested */
  /* OR3_FLAG_TIME_KERNELS: the shadow-ray (any-hit) kernel, next-event estimation only */
  double shadow_ms;
  uint64_t shadow_launches;
  uint32_t lanes;          /* wave lanes (streams) the render used */
  uint32_t waves_rerun;    /* waves whose ray queue a glass split overflowed, rendered again in sub-waves */
  uint64_t kernel_launches; /* kernels this call launched (every kind, counted at each launch) */
} or3_render_stats;

typedef struct or3_scene_info {
  uint64_t num_primitives;
  uint64_t num_nodes;      /* wide nodes */
  uint64_t device_bytes;
  double build_ms;         /* flattening + BVH build (host or device) */
  double upload_ms;        /* records, materials, environment, lights to the device */
  int32_t tree_depth;
  int32_t num_lights;      /* next-event lights: in-BVH objects with an emissive layer */
  double flatten_ms;       /* the part of build_ms spent flattening the primitives (host threads) */
} or3_scene_info;

typedef struct or3_context or3_context;

/* ---- context ----------------------------------------------------------- */
int or3_context_create(int device, or3_context **out);
int or3_context_destroy(or3_context *ctx);
const char *or3_last_error(const or3_context *ctx);
int or3_api_version(void);

/* ---- scenes (replaces Scene::ConstructBVH/ConstructQBVH,
        src/scenes/Scene.cpp:27-49, and the data Scene::CheckIntersection walks) */
int or3_scene_upload(or3_context *ctx, const or3_scene_desc *desc, int32_t *scene_out);
int or3_scene_release(or3_context *ctx, int32_t scene);
int or3_scene_get_info(or3_context *ctx, int32_t scene, or3_scene_info *out);

/* ---- render (replaces PathTracer::RenderScene, src/renderer/PathTracer.cpp:55-85)
   Blocking.  Calls `cb` (may be NULL) after every pass. */
int or3_render(or3_context *ctx, int32_t scene, const or3_camera *camera,
               const or3_render_params *params, or3_frame_callback cb, void *user);
/* Renderer::StopRendering (src/renderer/Renderer.h:22); safe from any thread. */
int or3_stop(or3_context *ctx);
/* Clears the stop request so the next or3_render runs. */
int or3_reset_stop(or3_context *ctx);
/* Last completed frame (Renderer::GetResult): `capacity` doubles. */
int or3_get_frame(or3_context *ctx, double *rgb_host, size_t capacity, int32_t *samples_out);
int or3_get_stats(or3_context *ctx, or3_render_stats *out);
/* Per-pixel sums of path radiance and of its square, rows top-down, W*H*3
   doubles each (either may be NULL); count = paths per pixel. */
int or3_get_moments(or3_context *ctx, double *sum_host, double *sumsq_host, size_t capacity,
                    uint64_t *count_out);
/* Per-path radiance of the last wave when OR3_FLAG_KEEP_PATHS was set:
   3 floats per path, in camera-path order
   g = ((s * H + y) * W + x) * ss*ss + sy*ss + sx, counted from the wave's first
   path (s = sample index from 0, y = camera row with 0 at the bottom as in
   PathTracer::scanPixelsOnYAndCastRays, src/renderer/PathTracer.cpp:143-175). */
int or3_get_path_radiance(or3_context *ctx, float *rgb_host, size_t capacity, uint64_t *paths_out);

/* ---- ray queries (replaces Scene::CheckIntersection, src/scenes/Scene.cpp:51-85)
   Closest hit of n rays: prim id (object id, -1 = miss), distance t, and the
   shading normal as the reference reports it (interpolated for triangles). */
int or3_trace_closest(or3_context *ctx, int32_t scene, size_t n, const float *origins_host,
                      const float *dirs_host, int32_t *prim_host, float *t_host,
                      float *normal_host);
int or3_trace_closest_device(or3_context *ctx, int32_t scene, size_t n, const float *origins_dev,
                             const float *dirs_dev, int32_t *prim_dev, float *t_dev,
                             float *normal_dev, void *stream);
/* Any hit in (EPS, tmax) for shadow rays: 1 = occluded. */
int or3_trace_occluded(or3_context *ctx, int32_t scene, size_t n, const float *origins_host,
                       const float *dirs_host, const float *tmax_host, uint8_t *occluded_host);

/* ---- lookups the shading uses, for n inputs at a time --------------------
   or3_env_sample: IBL::Sample(dir) (src/renderer/IBL.h:30-45), the
   nearest-texel equirect lookup a missed ray returns (the scene's background
   colour when it has no environment map); dirs are unit vectors.
   or3_texture_sample: Image::GetPixelByUV(u, v) (src/tools/Image.h:21-31) of
   the scene's texture `texture` (clamp to [0, 1], x 0.99999, nearest texel),
   the factor GetTexturedColor (src/renderer/PathTracer.cpp:327-346) applies
   to a textured layer's colour.  3 floats out per input.  Both run the
   device functions of the render's shade kernel.  n < 2^31. */
int or3_env_sample(or3_context *ctx, int32_t scene, size_t n, const float *dirs_host, float *rgb_host);
int or3_texture_sample(or3_context *ctx, int32_t scene, int32_t texture, size_t n, const float *uv_host,
                       float *rgb_host);

/* ---- batched form (no counterpart in the reference) ----------------------
 * Many renders ("jobs": scene, camera, sample budget) traced together: every
 * wave of the wavefront holds camera paths of several jobs, so small jobs fill
 * the GPU together instead of one after another.  A job's paths are numbered
 * and seeded exactly as in or3_render with the same camera and params, so a
 * job gives the same image alone or in a batch.  Scenes must be uploaded. */
typedef struct or3_batch_job {
  int32_t scene;
  uint32_t reserved;
  or3_camera camera;
  or3_render_params params; /* supersamples, sample schedule, depth policy, seed, output layout */
  double *frame_host;       /* final frame (params.output_layout), NULL = none */
  size_t frame_capacity;    /* doubles */
} or3_batch_job;

typedef struct or3_batch_params {
  uint64_t wave_paths;     /* camera paths per wave, 0 = automatic */
  uint32_t flags;          /* OR3_FLAG_NO_GRAPH, OR3_FLAG_COUNT_TRAVERSAL, OR3_FLAG_ONE_LANE, OR3_FLAG_HOST_LOOP, ... */
  uint32_t graph_bounces;  /* bounce iterations per loop iteration / graph replay, 0 = 8 */
  uint32_t blocks_per_sm;  /* persistent kernel blocks per SM, 0 = occupancy limit */
  uint32_t reserved;
} or3_batch_params;

int or3_render_batch(or3_context *ctx, const or3_batch_job *jobs, size_t n_jobs,
                     const or3_batch_params *params, or3_render_stats *stats_out);
/* Per-pixel path-radiance sums of job `job` of the last batch (rows top-down,
   W*H*3 doubles each, either may be NULL); count = paths per pixel. */
int or3_get_batch_moments(or3_context *ctx, size_t job, double *sum_host, double *sumsq_host,
                          size_t capacity, uint64_t *count_out);
/* Autotuner: renders a reduced copy of the batch (every job's sample budget cut
   so the copy holds about `sample_paths` camera paths) under candidate wave
   sizes, graph depths and block counts, and writes the fastest to *best. */
int or3_autotune_batch(or3_context *ctx, const or3_batch_job *jobs, size_t n_jobs, uint64_t sample_paths,
                       or3_batch_params *best, double *best_mpaths_out);

/* ---- served form (no counterpart in the reference) -----------------------
 * A request loop on its own host thread.  Jobs (or3_batch_job) are submitted
 * from any thread; the loop admits them as slots and device memory free up
 * (accumulation and frame buffers counted against hbm_budget_bytes), gives
 * every admitted job a fair share of each wave so new work overlaps running
 * work on the device, delivers a progressive frame every frame_every_samples
 * samples and a final frame, and records latency from submission to the final
 * frame.  Scenes stay resident (or3_scene_upload before submitting); while the
 * server runs, no other call may use the context except the or3_server_*
 * functions and or3_stop. */
typedef struct or3_server_params {
  uint64_t wave_paths;          /* camera paths per wave, 0 = automatic */
  uint64_t hbm_budget_bytes;    /* admitted jobs' buffers, 0 = half of the free device memory */
  uint32_t max_active_jobs;     /* 0 = 64 */
  uint32_t frame_every_samples; /* progressive frame cadence, 0 = 16 */
  uint32_t graph_bounces;       /* 0 = 8 */
  uint32_t flags;               /* OR3_SERVER_KEEP_MOMENTS, OR3_SERVER_ONE_LANE */
} or3_server_params;

#define OR3_SERVER_KEEP_MOMENTS 1u /* keep finished jobs' pixel sums on the host for or3_server_get_moments */
#define OR3_SERVER_ONE_LANE 2u     /* each wave on one stream (default: split over three streams that overlap) */
#define OR3_SERVER_UNSORTED_SHADE 4u /* one shade kernel for every hit and miss (default where jobs sample lights:
                                        the material-sorted shade) */

/* frame of job `job_id`: samples so far, frame in the job's output layout,
   final = 1 for the last one.  Called on the server thread. */
typedef void (*or3_job_frame_callback)(void *user, uint64_t job_id, int32_t samples, const double *rgb,
                                       size_t width, size_t height, int32_t final_frame);

#define OR3_JOB_QUEUED 0
#define OR3_JOB_RUNNING 1
#define OR3_JOB_DONE 2
#define OR3_JOB_CANCELLED 3
#define OR3_JOB_FAILED 4

typedef struct or3_job_status {
  int32_t state;           /* OR3_JOB_* */
  int32_t samples_done;
  double submit_s;         /* seconds since the server started */
  double admit_s;
  double first_frame_s;
  double done_s;
} or3_job_status;

typedef struct or3_server_stats {
  uint64_t jobs_submitted, jobs_done, jobs_cancelled;
  uint64_t camera_paths;
  uint64_t waves;
  double busy_s;           /* wall time with admitted work */
  double device_ms;        /* device time of the waves (CUDA events) */
  double latency_p50_s, latency_p99_s;   /* submit -> final frame, completed jobs */
  double queue_p50_s, queue_p99_s;       /* submit -> admission */
  double first_frame_p50_s;
  uint64_t peak_active_jobs;
  uint64_t peak_budget_bytes;
  uint64_t waves_rerun;    /* waves with a lane a glass split overflowed (rendered again in pieces) */
} or3_server_stats;

int or3_server_start(or3_context *ctx, const or3_server_params *params, or3_job_frame_callback cb, void *user);
int or3_server_submit(or3_context *ctx, const or3_batch_job *job, uint64_t *job_id_out);
int or3_server_poll(or3_context *ctx, uint64_t job_id, or3_job_status *status_out);
int or3_server_cancel(or3_context *ctx, uint64_t job_id);
/* Blocks until every submitted job has finished, or timeout_s passes (OR3_ERR_BUSY). */
int or3_server_drain(or3_context *ctx, double timeout_s);
int or3_server_get_stats(or3_context *ctx, or3_server_stats *stats_out);
/* Per-pixel sums of a finished job (kept until or3_server_stop). */
int or3_server_get_moments(or3_context *ctx, uint64_t job_id, double *sum_host, double *sumsq_host,
                           size_t capacity, uint64_t *count_out);
int or3_server_stop(or3_context *ctx);

/* Served form with progressive frames encoded on the device to 8-bit RGB
   (or3_encode_rgb8 with gamma: what the reference's PNG saver writes), 3
   bytes per pixel in the job's layout, so a frame crosses to the host at an
   eighth of the FP64 frame's size.  Jobs' frame_host buffers are not used. */
typedef void (*or3_job_frame8_callback)(void *user, uint64_t job_id, int32_t samples, const uint8_t *rgb,
                                        size_t width, size_t height, int32_t final_frame);
int or3_server_start8(or3_context *ctx, const or3_server_params *params, or3_job_frame8_callback cb, void *user);

/* ---- image output and input on the device (the reference's savers and HDR
 * loader stay the file writers and readers; these replace their per-pixel
 * conversions, src/tools/FileSaver.h:49-120, src/tools/HDRImage.h:10-38) ---- */

/* 8-bit RGB as the reference's PNG/PPM savers produce it: clamp to [0, 1],
   pow(x, 1/2.2) when gamma (FileSaver::CopyColorArrayToImage, Utils::GammaRev),
   then (int)(v * 255 + 0.5) (Utils::ToRgb).  n pixels, 3 doubles each. */
int or3_encode_rgb8(or3_context *ctx, const double *rgb, size_t n, int32_t gamma, uint8_t *out);
/* HDRImage::Color2RGBE: 4 bytes per pixel. */
int or3_encode_rgbe(or3_context *ctx, const double *rgb, size_t n, uint8_t *out);
/* HDRImage::RGBE2Color: 3 floats per pixel. */
int or3_decode_rgbe(or3_context *ctx, const uint8_t *rgbe, size_t n, float *out);
/* The last frame of or3_render (the layout it was rendered in), encoded on
   the device; capacity in bytes (3 or 4 per pixel). */
int or3_get_frame_rgb8(or3_context *ctx, int32_t gamma, uint8_t *rgb, size_t capacity, int32_t *samples_out);
int or3_get_frame_rgbe(or3_context *ctx, uint8_t *rgbe, size_t capacity, int32_t *samples_out);
/* A Radiance .hdr file in memory (HDRImage::ReadFromRadianceFile,
   src/tools/HDRImage.cpp:12-186: "#?" header, "-Y h +X w", run-length or flat
   scanlines) to flat RGBE bytes, row-major, on the host.  rgbe NULL returns
   the size only.  No context or GPU needed; decode with or3_decode_rgbe or
   pass the bytes as or3_scene_desc.env_rgbe. */
int or3_read_hdr(const uint8_t *file, size_t length, uint32_t *width_out, uint32_t *height_out, uint8_t *rgbe,
                 size_t capacity);

/* ---- mesh ingest: Wavefront .obj/.mtl to arrays (Model::ReadFromObj,
 * src/renderer/Model.cpp:50-182; Model::LoadMaterialFile, :184-292), without
 * a per-triangle object; the arrays plug into or3_scene_desc's triangle
 * fields.  Material 0 is the reference's default (Lambert, colour 0.99); the
 * rest come from the .mtl files in order.  Triangles are in file order. */
typedef struct or3_mesh {
  uint32_t num_triangles;
  double *vertices;        /* [n][3][3] */
  double *normals;         /* [n][3][3]; the face normal where the file gives none */
  double *uvs;             /* [n][3][2] */
  uint32_t *material;      /* [n] index into materials */
  uint32_t num_materials;
  or3_material *materials; /* texture = -1: textures are listed by path */
  char **material_names;   /* [num_materials] */
  char **texture_paths;    /* [num_materials] map_Kd path, or NULL */
} or3_mesh;
/* threads 0 = all host threads.  OR3_ERR_NOT_FOUND for a missing .obj/.mtl,
   OR3_ERR_INVALID_ARGUMENT for a malformed line or index. */
int or3_mesh_load_obj(const char *path, int32_t flip_v, uint32_t threads, or3_mesh **mesh_out);
/* Model::Transform as SceneFromExternalFile::ReadMesh applies it (rotation in
   radians, Rz * Ry * Rx; per-axis scale; then translation; normals rotated). */
int or3_mesh_transform(or3_mesh *mesh, const double position[3], const double scaling[3],
                       const double rotation[3]);
void or3_mesh_free(or3_mesh *mesh);

/* ---- scene files: the reference's text scene format to a scene descriptor
 * (SceneFromExternalFile::ReadFromFile, src/scenes/SceneFromExternalFile.cpp:
 * 66-182, and its object readers, :214-529).  Header "Base Dir", "IBL",
 * "Space Partitioning" up to "Objects:", then "Obj Mesh", "Sphere",
 * "SphereLight", "Floor" and "InfiniteFloor" blocks.  Meshes are read with
 * or3_mesh_load_obj (flip_v 0) and placed with or3_mesh_transform; the IBL
 * .hdr is read with or3_read_hdr into desc.env_rgbe.  Object ids follow the
 * file (a mesh's triangles in file order).  Every sphere and triangle goes in
 * the BVH ("Space Partitioning: False" objects are tested after the BVH by
 * the reference, which differs only for hits at exactly equal distance).
 * Materials with a texture keep texture = -1 and name the image in
 * texture_paths[material] (loading it stays with the caller).  The descriptor
 * and everything it points to live until or3_scene_file_free. */
typedef struct or3_scene_file {
  or3_scene_desc desc;
  uint32_t num_meshes;          /* "Obj Mesh" blocks read */
  char space_partitioning[16];  /* the header's value ("BVH", "QBVH", or "") */
  char **texture_paths;         /* [desc.num_materials] image path, or NULL */
  char *ibl_path;               /* the IBL file read, or NULL */
} or3_scene_file;
/* threads: for the .obj files (0 = all host threads).  OR3_ERR_NOT_FOUND for
   a missing scene, mesh or IBL file, OR3_ERR_INVALID_ARGUMENT for anything the
   reference's reader rejects, or an object without a Material; err (may be
   NULL) gets a one-line reason. */
int or3_scene_load_file(const char *path, uint32_t threads, or3_scene_file **file_out, char *err, size_t err_len);
void or3_scene_file_free(or3_scene_file *file);

/* ---- rendering without allocating (no counterpart in the reference) ------
 * For callers that must not allocate device memory while they render:
 * engines that give the whole device to their own pool at start-up (a
 * cudaMalloc would fail or fragment that pool), and frame loops that cannot
 * afford cudaMalloc/cudaFree synchronising the device.  Call it from ordinary
 * host code: it launches kernels, copies and waits, so it must not be called
 * from a host function or callback enqueued on a CUDA stream (CUDA forbids
 * CUDA calls there).
 *
 * Traces camera paths g in [first_path, first_path + num_paths) of the render
 * that `camera` and `params` describe (the path order of or3_get_path_radiance;
 * all paths must lie in one pass of the sample schedule) and writes 3 floats
 * of radiance per path to radiance_dev (device memory of the context's GPU,
 * provided by the caller).  The scene must already be uploaded.
 *
 * The ray queues live in one file-scope device array sized for
 * OR3_NOALLOC_MAX_PATHS paths (about 5.3 MB, held by every GPU that loads the
 * library until the process exits); larger num_paths is rejected with
 * OR3_ERR_INVALID_ARGUMENT.  The call allocates nothing.  Its first call on a
 * device looks up that array's device address, so make that first call before
 * any stream capture.  The address is kept for the life of the process: after
 * cudaDeviceReset (or any reset of the device's primary context) it is stale,
 * so do not call this entry again in that process.  Every call shares the
 * array and it keeps the previous call's contents (the call clears what must
 * start at zero); calls that overlap on the GPU -- from two host threads, or
 * on two streams -- race on it.
 * Blocks: every call synchronises `stream` (several times: it reads the queue
 * lengths back to the host between bounce chunks) and returns once the
 * result is in radiance_dev.  It makes the context's GPU current while it
 * runs and restores the caller's current device before it returns.
 * stream NULL = the context's. */
#define OR3_NOALLOC_MAX_PATHS 4096u
int or3_render_paths_noalloc(or3_context *ctx, int32_t scene, const or3_camera *camera,
                             const or3_render_params *params, uint64_t first_path, uint32_t num_paths,
                             float *radiance_dev, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* OR3_H_ */
