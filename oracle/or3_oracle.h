/*
 * or3_oracle.h -- TEST INFRASTRUCTURE ONLY: the CPU oracle for the GPU path.
 *
 * A plain-C, FP64 restatement of omochi-renderer3's render path.  It is the
 * checker for the CUDA kernels (tests, __graft_entry__.smoke) and the CPU
 * baseline timed by bench.py; the product never links or loads it.
 *
 * Pinning: tests/test_oracle_pin.py checks it against the reference's own
 * compiled code (oracle/_ref, built from the reference sources) -- closest
 * hits on seeded ray sets must agree exactly, rendered images statistically
 * (3 standard errors) -- and against the committed golden vectors in
 * tests/golden/ generated from the reference by tests/golden/make_golden.py.
 */
#ifndef OR3_ORACLE_H_
#define OR3_ORACLE_H_

#include <stddef.h>
#include <stdint.h>

#include "or3.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_scene orc_scene;

typedef struct orc_params {
  int32_t supersamples;
  int32_t min_samples, max_samples, step_samples;
  int32_t next_event_estimation;
  int32_t rr_min_depth;
  int32_t max_depth;
  int32_t pad;
  uint64_t seed;
} orc_params;

/* use_bvh: 1 = the reference's binary SAH BVH (src/renderer/BVH.cpp), 0 = the
   reference's brute-force loop over the in-BVH objects (src/scenes/Scene.cpp:60-70). */
orc_scene *orc_scene_create(const or3_scene_desc *d, int use_bvh);
void orc_scene_destroy(orc_scene *s);
int orc_scene_bvh_nodes(const orc_scene *s);

/* Scene::CheckIntersection on n rays: object id (-1 miss), t, shading normal. */
int orc_closest(const orc_scene *s, size_t n, const double *orig, const double *dir, int32_t *id, double *t,
                double *normal);

/* Distance at which ray i hits object id[i] alone (INF = no hit), to tell
   ties from real disagreements. */
int orc_object_distance(const orc_scene *s, size_t n, const int32_t *id, const double *orig, const double *dir,
                        double *t);

/* Radiance of camera paths g in [first, first + count) (the GPU's path order,
   include/or3.h), written to out[3 * (g - first)]. */
int orc_path_radiance(const orc_scene *s, const or3_camera *cam, const orc_params *p, uint64_t first,
                      uint64_t count, int nthreads, double *out);

/* Full render: per-pixel sums / sums of squares of path radiance (rows
   top-down, W*H*3 each) over the sample schedule; wall seconds. */
int orc_render(const orc_scene *s, const or3_camera *cam, const orc_params *p, int nthreads, double *sum,
               double *sumsq, double *seconds);

/* Image conversions of the reference's savers and HDR loader:
   8-bit: FileSaver::CopyColorArrayToImage + Utils::ToRgb (gamma 1/2.2 or none);
   RGBE: HDRImage::Color2RGBE / RGBE2Color.  n pixels, RGB doubles. */
void orc_encode_rgb8(size_t n, const double *rgb, int gamma, uint8_t *out);
void orc_encode_rgbe(size_t n, const double *rgb, uint8_t *out);
void orc_decode_rgbe(size_t n, const uint8_t *rgbe, double *out);

/* Philox4x32-10 as the kernels use it (for the RNG known-answer test). */
/* IBL::Sample(dir) and Image::GetPixelByUV of texture `tex`, 3 doubles out per input. */
void orc_env_sample(const orc_scene *s, size_t n, const double *dir, double *rgb);
int orc_texel(const orc_scene *s, int tex, size_t n, const double *uv, double *rgb);
void orc_philox(const uint32_t ctr[4], uint32_t k0, uint32_t k1, uint32_t out[4]);

#ifdef __cplusplus
}
#endif
#endif
