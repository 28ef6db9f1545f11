/*
 * or3_oracle.c -- TEST INFRASTRUCTURE ONLY (see or3_oracle.h).
 *
 * FP64 restatement of the reference render path, function by function:
 *   obj_hit_triangle   Polygon::CheckIntersection       src/renderer/Polygon.h:63-106
 *   obj_hit_sphere     Sphere::CheckIntersection        src/renderer/Sphere.h:21-78
 *   obj_hit_plane      AxisAlignedPlane / InfiniteFloor src/renderer/AxisAlignedPlane.h:38-64,
 *                                                       src/renderer/InfiniteFloor.h:19-37
 *   box_hit_f          BoundingBox::CheckIntersection<float> src/renderer/BoundingBox.h:96-123
 *   bvh_build          BVH::Construct_internal (SAH)    src/renderer/BVH.cpp:164-312
 *   bvh_closest        BVH::CheckIntersection           src/renderer/BVH.cpp:19-88
 *   scene_closest      Scene::CheckIntersection         src/scenes/Scene.cpp:51-85
 *   camera_ray         Camera::SampleRayForPixel        src/renderer/Camera.h:65-93
 *   radiance           PathTracer::Radiance/_internal/_Lambert/_Specular/_Refraction
 *                                                       src/renderer/PathTracer.cpp:180-591
 *   env_sample         IBL::Sample(dir)                 src/renderer/IBL.h:30-45
 *   orc_encode_rgb8    FileSaver::CopyColorArrayToImage + Utils::ToRgb
 *                                                       src/tools/FileSaver.h:49-120,
 *                                                       src/tools/Utils.h:93-109
 *   orc_encode_rgbe    HDRImage::Color2RGBE             src/tools/HDRImage.h:10-25
 *   orc_decode_rgbe    HDRImage::RGBE2Color             src/tools/HDRImage.h:27-38
 * The random numbers are the GPU's counter-based Philox draws (not the
 * reference's per-row xorshift), so a path can be replayed exactly; the
 * estimator and its expectation are the reference's.
 */
#include "or3_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define EPS 0.0005
#define INF ((FLT_MAX - 1) / 2)
#define PI 3.14159265358979323846264338327950288419716939

typedef struct { double x, y, z; } v3;
static inline v3 mk(double x, double y, double z) { v3 r = {x, y, z}; return r; }
static inline v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 mul(v3 a, double s) { return mk(a.x * s, a.y * s, a.z * s); }
static inline v3 mulv(v3 a, v3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline double dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 cross(v3 a, v3 b) {
  return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline v3 nrm(v3 a) { double l = sqrt(dot(a, a)); return mk(a.x / l, a.y / l, a.z / l); }
static inline v3 ld(const double *p) { return mk(p[0], p[1], p[2]); }

/* ------------------------------------------------------------------ RNG */
void orc_philox(const uint32_t ctr[4], uint32_t k0, uint32_t k1, uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  for (int r = 0; r < 10; r++) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c0 = hi1 ^ c1 ^ k0;
    c1 = lo1;
    c2 = hi0 ^ c3 ^ k1;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}
static inline double u01(uint32_t x) { return (double)(x >> 8) * (1.0 / 16777216.0); }
static void path_rand(uint64_t seed, uint64_t g, uint32_t leaf, uint32_t depth, uint32_t call, double r[4]) {
  uint32_t c[4] = {(uint32_t)g, (uint32_t)(g >> 32), (depth & 0xFFFFu) | (leaf << 16) | (call << 24), 0u}, o[4];
  orc_philox(c, (uint32_t)seed, (uint32_t)(seed >> 32), o);
  for (int k = 0; k < 4; k++) r[k] = u01(o[k]);
}

/* ------------------------------------------------------------------ scene */
enum { K_TRI = 0, K_SPHERE = 1, K_PLANE = 2, K_FLOOR = 3 };

typedef struct {
  int kind, in_bvh;
  uint32_t id, lb, lc, textured;
  v3 p0, e1, e2, n0, dn1, dn2;
  double uv0[2], duv1[2], duv2[2];
  v3 c;
  double r;
  int axis;
  double offset, nsign;
  v3 bmin, bmax, bcen;
  int light;  /* in-BVH object with an emissive layer: a next-event light */
} obj;

typedef struct {
  int type, texture, emissive;
  v3 emission, color;
  double ior, phong;
} mat;

typedef struct {
  float box[2][3];
  int child[2];   /* -1 = leaf */
  int first, count;
} bnode;

struct orc_scene {
  obj *o;
  int n;          /* objects in id order */
  int *inbvh;     /* in-BVH objects in insertion order */
  int nin;
  int *outbvh;
  int nout;
  mat *m;
  uint32_t *lmat;
  double *lrate;
  int use_bvh;
  bnode *nodes;
  int nnodes, capnodes;
  int *leafobj;   /* leaf object lists */
  int nleaf, capleaf;
  float *env;
  int envw, envh;
  v3 bg;
  const float **tex;
  uint32_t *texw, *texh;
  int ntex;
  /* next-event estimation: local lights (emissive triangles, then emissive
     spheres, in description order) chosen by power, and the environment */
  int nlights;
  int *light_obj;
  v3 *light_le;       /* emission expected over the layer roulette */
  float *light_cdf;   /* inclusive, last = 1 */
  float *light_pdf;
  int env_light;      /* 0 none, 1 equirect map, 2 constant background */
  float *env_marg;    /* [envh] inclusive marginal CDF over rows */
  float *env_cond;    /* [envh * envw] inclusive conditional CDF per row */
  double env_prob;    /* probability of sampling the environment */
  int *order;         /* object index of description entry i (triangles, spheres, planes) */
};

typedef struct {
  double t;
  v3 pos, normal;
  double u, v;
  int obj;
} hitrec;

static int obj_hit_triangle(const obj *o, v3 org, v3 dir, hitrec *h) {
  v3 P = cross(dir, o->e2);
  double det = dot(P, o->e1);
  if (det > EPS) {
    v3 T = sub(org, o->p0);
    double u = dot(P, T);
    if (u >= 0 && u <= det) {
      v3 Q = cross(T, o->e1);
      double v = dot(Q, dir);
      if (v >= 0 && u + v <= det) {
        double t = dot(Q, o->e2) / det;
        if (t >= EPS) {
          double ur = u / det, vr = v / det;
          h->t = t;
          h->pos = add(org, mul(dir, t));
          h->normal = nrm(add(add(mul(o->dn1, ur), mul(o->dn2, vr)), o->n0));
          h->u = o->uv0[0] + o->duv1[0] * ur + o->duv2[0] * vr;
          h->v = o->uv0[1] + o->duv1[1] * ur + o->duv2[1] * vr;
          return 1;
        }
      }
    }
  }
  return 0;
}

static int obj_hit_sphere(const obj *o, v3 x, v3 v, hitrec *h) {
  v3 cmx = sub(o->c, x);
  double b = dot(v, cmx);
  double D1 = b * b;
  double D2 = dot(v, v) * (dot(cmx, cmx) - o->r * o->r);
  double D = D1 - D2;
  if (D < 0) return 0;
  double sq = sqrt(D);
  double t1 = sq + b, t2 = -sq + b;
  if (t1 <= EPS && t2 <= EPS) return 0;
  h->t = t2 > EPS ? t2 : t1;
  h->pos = add(x, mul(v, h->t));
  h->normal = nrm(sub(h->pos, o->c));
  h->u = h->v = 0;
  if (o->textured) {
    double vv = (asin(h->normal.y) + PI * 0.5) / PI;
    while (vv > 1) vv -= 1;
    while (vv < 0) vv += 1;
    double uu = (atan2(h->normal.z, h->normal.x) + PI) / (2 * PI);
    while (uu > 1) uu -= 1;
    while (uu < 0) uu += 1;
    h->u = uu;
    h->v = 1 - vv;
  }
  return 1;
}

static int obj_hit_plane(const obj *o, v3 org, v3 dir, hitrec *h) {
  double t;
  if (o->kind == K_FLOOR) {
    if (fabs(dir.y) < EPS) return 0;
    t = (o->offset - org.y) / dir.y;
    if (t < EPS) return 0;
    h->normal = mk(0, dir.y < 0 ? 1 : -1, 0);
  } else {
    double dd = o->axis == 0 ? dir.z : o->axis == 1 ? dir.y : dir.x;
    double oo = o->axis == 0 ? org.z : o->axis == 1 ? org.y : org.x;
    t = -INF;
    if (dd != 0) t = (o->offset - oo) / dd;
    if (t < EPS) return 0;
    h->normal = o->axis == 0 ? mk(0, 0, o->nsign) : o->axis == 1 ? mk(0, o->nsign, 0) : mk(o->nsign, 0, 0);
  }
  h->t = t;
  h->pos = add(org, mul(dir, t));
  h->u = h->v = 0;
  return 1;
}

static int obj_hit(const obj *o, v3 org, v3 dir, hitrec *h) {
  switch (o->kind) {
    case K_TRI: return obj_hit_triangle(o, org, dir, h);
    case K_SPHERE: return obj_hit_sphere(o, org, dir, h);
    default: return obj_hit_plane(o, org, dir, h);
  }
}

/* BoundingBox::CheckIntersection<float> */
static int box_hit_f(const float dir[3], const float org[3], const float mn[3], const float mx[3], float *dist) {
  float fastest_out = (float)INF, latest_in = -(float)INF;
  for (int i = 0; i < 3; i++) {
    float inv = dir[i] != 0 ? 1.0f / dir[i] : (float)INF;
    float t1 = (mn[i] - org[i]) * inv;
    float t2 = (mx[i] - org[i]) * inv;
    if (fabsf(inv) > 999999.0f) {
      t1 = (mn[i] - org[i]) > 0 ? (float)INF : -(float)INF;
      t2 = (mx[i] - org[i]) > 0 ? (float)INF : -(float)INF;
    }
    float tmin = t1 < t2 ? t1 : t2, tmax = t1 < t2 ? t2 : t1;
    if (tmax < fastest_out) fastest_out = tmax;
    if (tmin > latest_in) latest_in = tmin;
    if (latest_in > fastest_out) return 0;
  }
  *dist = latest_in > 0 ? latest_in : 0;
  return 1;
}

/* ------------------------------------------------------------------ BVH build (reference SAH) */
static const orc_scene *g_sort_scene;
static int g_sort_axis;
static int cmp_center(const void *a, const void *b) {
  const obj *oa = &g_sort_scene->o[*(const int *)a], *ob = &g_sort_scene->o[*(const int *)b];
  double ca = g_sort_axis == 0 ? oa->bcen.x : g_sort_axis == 1 ? oa->bcen.y : oa->bcen.z;
  double cb = g_sort_axis == 0 ? ob->bcen.x : g_sort_axis == 1 ? ob->bcen.y : ob->bcen.z;
  return ca < cb ? -1 : ca > cb ? 1 : 0;
}

static double box_area(v3 mn, v3 mx) {
  double dx = mx.x - mn.x, dy = mx.y - mn.y, dz = mx.z - mn.z;
  return dx * dy + dx * dz + dy * dz;
}

static int new_node(orc_scene *s) {
  if (s->nnodes == s->capnodes) {
    s->capnodes = s->capnodes ? 2 * s->capnodes : 64;
    s->nodes = (bnode *)realloc(s->nodes, sizeof(bnode) * s->capnodes);
  }
  memset(&s->nodes[s->nnodes], 0, sizeof(bnode));
  return s->nnodes++;
}

static void float_box(const orc_scene *s, const int *objs, int n, float mn[3], float mx[3]) {
  /* CalcBoundingBoxOfObjects<float> (src/renderer/BVH.cpp:197-215) */
  const obj *o0 = &s->o[objs[0]];
  mn[0] = (float)o0->bmin.x; mn[1] = (float)o0->bmin.y; mn[2] = (float)o0->bmin.z;
  mx[0] = (float)o0->bmax.x; mx[1] = (float)o0->bmax.y; mx[2] = (float)o0->bmax.z;
  for (int i = 0; i < n; i++) {
    const obj *a = &s->o[objs[i]];
    if (a->bmin.x < mn[0]) mn[0] = (float)a->bmin.x;
    if (a->bmin.y < mn[1]) mn[1] = (float)a->bmin.y;
    if (a->bmin.z < mn[2]) mn[2] = (float)a->bmin.z;
    if (a->bmax.x > mx[0]) mx[0] = (float)a->bmax.x;
    if (a->bmax.y > mx[1]) mx[1] = (float)a->bmax.y;
    if (a->bmax.z > mx[2]) mx[2] = (float)a->bmax.z;
  }
}

static void bvh_build(orc_scene *s, int node, int *objs, int n) {
  float mn[3], mx[3];
  float_box(s, objs, n, mn, mx);
  memcpy(s->nodes[node].box[0], mn, sizeof(mn));
  memcpy(s->nodes[node].box[1], mx, sizeof(mx));
  float fd[3] = {mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]};
  const double area = (double)(fd[0] * fd[1] + fd[1] * fd[2] + fd[0] * fd[2]);
  const double inv = 1.0 / area;
  int best_axis = -1, best_index = -1;
  double best_cost = -1;
  int *sorted = (int *)malloc(sizeof(int) * n);
  double *left = (double *)malloc(sizeof(double) * n), *right = (double *)malloc(sizeof(double) * n);
  for (int axis = 0; axis < 3; axis++) {
    memcpy(sorted, objs, sizeof(int) * n);
    g_sort_scene = s;
    g_sort_axis = axis;
    qsort(sorted, n, sizeof(int), cmp_center);
    /* right areas: right[i] = area of objects i+1..n-1 */
    v3 bmn = s->o[sorted[n - 1]].bmin, bmx = s->o[sorted[n - 1]].bmax;
    right[n - 1] = INF;
    for (int i = n - 2; i >= 0; i--) {
      right[i] = box_area(bmn, bmx);
      const obj *a = &s->o[sorted[i]];
      bmn = mk(fmin(bmn.x, a->bmin.x), fmin(bmn.y, a->bmin.y), fmin(bmn.z, a->bmin.z));
      bmx = mk(fmax(bmx.x, a->bmax.x), fmax(bmx.y, a->bmax.y), fmax(bmx.z, a->bmax.z));
    }
    bmn = s->o[sorted[0]].bmin;
    bmx = s->o[sorted[0]].bmax;
    const double leaf_cost = (double)n;
    for (int c = 0; c <= n - 2; c++) {
      left[c] = box_area(bmn, bmx);
      const obj *a = &s->o[sorted[c + 1]];
      bmn = mk(fmin(bmn.x, a->bmin.x), fmin(bmn.y, a->bmin.y), fmin(bmn.z, a->bmin.z));
      bmx = mk(fmax(bmx.x, a->bmax.x), fmax(bmx.y, a->bmax.y), fmax(bmx.z, a->bmax.z));
      /* the reference weighs the areas with the set sizes after moving one
         more object left (src/renderer/BVH.cpp:312-331) */
      const double nl = (double)(c + 2), nr = (double)(n - c - 2);
      const double cost = 2.0 + (left[c] * nl + right[c] * nr) * inv;
      if ((cost < best_cost || best_cost == -1) && cost < leaf_cost) {
        best_cost = cost;
        best_index = c;
        best_axis = axis;
      }
    }
  }
  free(left);
  free(right);
  if (best_axis == -1) {
    free(sorted);
    if (s->nleaf + n > s->capleaf) {
      s->capleaf = 2 * (s->nleaf + n) + 64;
      s->leafobj = (int *)realloc(s->leafobj, sizeof(int) * s->capleaf);
    }
    s->nodes[node].child[0] = s->nodes[node].child[1] = -1;
    s->nodes[node].first = s->nleaf;
    s->nodes[node].count = n;
    memcpy(s->leafobj + s->nleaf, objs, sizeof(int) * n);
    s->nleaf += n;
    return;
  }
  memcpy(sorted, objs, sizeof(int) * n);
  g_sort_scene = s;
  g_sort_axis = best_axis;
  qsort(sorted, n, sizeof(int), cmp_center);
  const int c0 = new_node(s);
  const int c1 = new_node(s);
  s->nodes[node].child[0] = c0;
  s->nodes[node].child[1] = c1;
  bvh_build(s, c0, sorted, best_index + 1);
  bvh_build(s, c1, sorted + best_index + 1, n - best_index - 1);
  free(sorted);
}

typedef struct { int index; } stackent;

static void bvh_closest(const orc_scene *s, v3 org, v3 dir, hitrec *best) {
  int stack[256];
  int sp = 0;
  stack[sp++] = 0;
  const float fd[3] = {(float)dir.x, (float)dir.y, (float)dir.z};
  const float fo[3] = {(float)org.x, (float)org.y, (float)org.z};
  int *heap = NULL;
  int cap = 256;
  int *st = stack;
  while (sp > 0) {
    const bnode *nd = &s->nodes[st[--sp]];
    if (nd->child[0] == -1) {
      for (int i = 0; i < nd->count; i++) {
        hitrec h;
        const int oi = s->leafobj[nd->first + i];
        if (obj_hit(&s->o[oi], org, dir, &h) && best->t > h.t) {
          *best = h;
          best->obj = oi;
        }
      }
    } else {
      float d1 = (float)INF, d2 = (float)INF;
      const bnode *n1 = &s->nodes[nd->child[0]], *n2 = &s->nodes[nd->child[1]];
      int h1 = box_hit_f(fd, fo, n1->box[0], n1->box[1], &d1);
      int h2 = box_hit_f(fd, fo, n2->box[0], n2->box[1], &d2);
      if (sp + 2 > cap) {
        cap *= 2;
        if (st == stack) {
          heap = (int *)malloc(sizeof(int) * cap);
          memcpy(heap, stack, sizeof(stack));
        } else {
          heap = (int *)realloc(heap, sizeof(int) * cap);
        }
        st = heap;
      }
      if (h1 && h2) {
        if (d1 < d2 && best->t >= d1) {
          st[sp++] = nd->child[1];
          st[sp++] = nd->child[0];
        } else if (d1 >= d2 && best->t >= d2) {
          st[sp++] = nd->child[0];
          st[sp++] = nd->child[1];
        }
      } else if (h1) {
        st[sp++] = nd->child[0];
      } else if (h2) {
        st[sp++] = nd->child[1];
      }
    }
  }
  free(heap);
}

static int scene_closest(const orc_scene *s, v3 org, v3 dir, hitrec *best) {
  best->t = INF;
  best->obj = -1;
  if (s->use_bvh && s->nnodes > 0) {
    bvh_closest(s, org, dir, best);
  } else {
    for (int i = 0; i < s->nin; i++) {
      hitrec h;
      if (obj_hit(&s->o[s->inbvh[i]], org, dir, &h) && best->t > h.t) {
        *best = h;
        best->obj = s->inbvh[i];
      }
    }
  }
  for (int i = 0; i < s->nout; i++) {
    hitrec h;
    if (obj_hit(&s->o[s->outbvh[i]], org, dir, &h) && best->t > h.t) {
      *best = h;
      best->obj = s->outbvh[i];
    }
  }
  return best->t != INF;
}

/* ------------------------------------------------------------------ lights
 * Next-event estimation has no working reference counterpart: the
 * reference's DirectRadiance_Lambert (src/renderer/PathTracer.cpp:239-323)
 * weights the light sample by the receiving surface's emission (always 0
 * there), and its IBL importance map (src/renderer/IBL.h:104-189) is a stub.
 * This restates the estimator the GPU implements:
 *   - lights: every in-BVH object with an emissive layer (triangles by area,
 *     spheres by SphereLight::SampleOnePointWithTargetPoint's visible-cap
 *     sampling, src/renderer/SphereLight.h:39-69), chosen with probability
 *     proportional to area * sum(p_layer * |emission|) (SphereLight::TotalPower,
 *     :71-78), and the environment (equirect map by a piecewise-constant
 *     marginal/conditional CDF over max(r,g,b) * sin(theta), or a constant
 *     background by cosine-weighted directions about the receiver's normal);
 *     when both kinds exist, each half;
 *   - at a Lambert or Phong vertex that survived Russian roulette, one light
 *     sample with an any-hit shadow ray, weighted like the reference's
 *     direct term: brdf * Le * cos * G / (pdf * p_select) / p_rr;
 *   - emission reached by a BSDF ray is counted only after the camera or a
 *     mirror/glass vertex, or from an object that is not a light (planes).
 */
static double layer_prob(const orc_scene *s, const obj *o, uint32_t k) {
  double lo = 0;
  for (uint32_t j = 0; j < k; j++) lo += s->lrate[o->lb + j];
  lo = lo < 0 ? 0 : lo > 1 ? 1 : lo;
  double hi = k + 1 == o->lc ? 1.0 : lo + s->lrate[o->lb + k];
  hi = hi < 0 ? 0 : hi > 1 ? 1 : hi;
  return hi > lo ? hi - lo : 0.0;
}

static void build_lights(orc_scene *s) {
  double *power = (double *)malloc(sizeof(double) * (s->n > 0 ? s->n : 1));
  s->light_obj = (int *)malloc(sizeof(int) * (s->n > 0 ? s->n : 1));
  s->light_le = (v3 *)malloc(sizeof(v3) * (s->n > 0 ? s->n : 1));
  double total = 0;
  /* description order: triangles, then spheres (object ids may be permuted) */
  for (int pass = 0; pass < 2; pass++)
    for (int i = 0; i < s->n; i++) {
      obj *o = &s->o[s->order[i]];
      if (!o->in_bvh || o->kind != (pass == 0 ? K_TRI : K_SPHERE)) continue;
      o->light = 0;
      for (uint32_t k = 0; k < o->lc; k++)
        if (s->m[s->lmat[o->lb + k]].emissive) o->light = 1;
      if (!o->light) continue;
      v3 le = mk(0, 0, 0);
      double mag = 0;
      for (uint32_t k = 0; k < o->lc; k++) {
        const double p = layer_prob(s, o, k);
        const v3 e = s->m[s->lmat[o->lb + k]].emission;
        le = add(le, mul(e, p));
        mag += p * sqrt(dot(e, e));
      }
      const double area = o->kind == K_TRI ? 0.5 * sqrt(dot(cross(o->e1, o->e2), cross(o->e1, o->e2)))
                                           : 4 * PI * o->r * o->r;
      s->light_obj[s->nlights] = s->order[i];
      s->light_le[s->nlights] = le;
      power[s->nlights] = area * mag;
      total += area * mag;
      s->nlights++;
    }
  if (!(total > 0)) s->nlights = 0;
  s->light_cdf = (float *)malloc(sizeof(float) * (s->nlights > 0 ? s->nlights : 1));
  s->light_pdf = (float *)malloc(sizeof(float) * (s->nlights > 0 ? s->nlights : 1));
  double run = 0;
  for (int k = 0; k < s->nlights; k++) {
    run += power[k];
    s->light_cdf[k] = k + 1 == s->nlights ? 1.0f : (float)(run / total);
    s->light_pdf[k] = (float)(power[k] / total);
  }
  free(power);
  /* environment */
  if (s->env) {
    const int W = s->envw, H = s->envh;
    double *rows = (double *)malloc(sizeof(double) * H);
    s->env_cond = (float *)malloc(sizeof(float) * (size_t)W * H);
    s->env_marg = (float *)malloc(sizeof(float) * H);
    double etot = 0;
    for (int i = 0; i < H; i++) {
      const double st = sin(PI * (i + 0.5) / H);
      double r = 0;
      for (int j = 0; j < W; j++) {
        const float *p = s->env + 3 * ((size_t)i * W + j);
        const float mx = p[0] > p[1] ? (p[0] > p[2] ? p[0] : p[2]) : (p[1] > p[2] ? p[1] : p[2]);
        r += (mx > 0 ? mx : 0) * st;
        s->env_cond[(size_t)i * W + j] = (float)r; /* running sum, normalised below */
      }
      rows[i] = r;
      etot += r;
    }
    for (int i = 0; i < H; i++) {
      double r = 0;
      for (int j = 0; j < W; j++) {
        const float *p = s->env + 3 * ((size_t)i * W + j);
        const float mx = p[0] > p[1] ? (p[0] > p[2] ? p[0] : p[2]) : (p[1] > p[2] ? p[1] : p[2]);
        r += (mx > 0 ? mx : 0) * sin(PI * (i + 0.5) / H);
        s->env_cond[(size_t)i * W + j] =
            j + 1 == W ? 1.0f : rows[i] > 0 ? (float)(r / rows[i]) : (float)((j + 1.0) / W);
      }
    }
    double run2 = 0;
    for (int i = 0; i < H; i++) {
      run2 += rows[i];
      s->env_marg[i] = i + 1 == H ? 1.0f : etot > 0 ? (float)(run2 / etot) : (float)((i + 1.0) / H);
    }
    free(rows);
    s->env_light = etot > 0 ? 1 : 0;
  } else {
    s->env_light = dot(s->bg, s->bg) != 0 ? 2 : 0;
  }
  s->env_prob = s->env_light ? (s->nlights ? 0.5 : 1.0) : 0.0;
}

/* first index whose inclusive CDF value exceeds u */
static int cdf_find(const float *cdf, int n, double u) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if ((double)cdf[mid] > u) hi = mid;
    else lo = mid + 1;
  }
  return lo;
}

/* orthonormal basis about unit a (Duff et al., JCGT 2017) */
static void onb(v3 a, v3 *t1, v3 *t2) {
  const double sg = a.z >= 0 ? 1.0 : -1.0;
  const double aa = -1.0 / (sg + a.z), bb = a.x * a.y * aa;
  *t1 = mk(1.0 + sg * a.x * a.x * aa, sg * bb, -sg * a.x);
  *t2 = mk(bb, sg + a.y * a.y * aa, -a.y);
}

static v3 env_sample(const orc_scene *s, v3 d);
static int scene_closest(const orc_scene *s, v3 org, v3 dir, hitrec *best);

/* One light sample seen from x (oriented normal nl).  brdf(d) is the vertex's
   BRDF times its colour; returns brdf * Le * cos * G / (pdf * p_select),
   0 when the sample is occluded or faces away. */
typedef struct {
  int phong;
  double exponent;
  v3 col, mirror;
} brdf_t;

static v3 brdf_eval(const brdf_t *b, v3 d) {
  if (!b->phong) return mul(b->col, 1.0 / PI);
  const double c = dot(d, b->mirror);
  return mul(b->col, (b->exponent + 2.0) / (2.0 * PI) * (c > 0 ? pow(c, b->exponent) : 0.0));
}

static v3 nee_direct(const orc_scene *s, const double r[4], v3 x, v3 nl, const brdf_t *b) {
  const v3 zero = mk(0, 0, 0);
  double usel = r[0];
  v3 d, le;
  double pdf_w, tmax;
  double psel;
  if (usel < s->env_prob) {
    psel = s->env_prob;
    if (s->env_light == 1) {
      const int W = s->envw, H = s->envh;
      const int i = cdf_find(s->env_marg, H, r[1]);
      const double prev = i ? (double)s->env_marg[i - 1] : 0.0, pr = (double)s->env_marg[i] - prev;
      const float *row = s->env_cond + (size_t)i * W;
      const int j = cdf_find(row, W, r[2]);
      const double prevc = j ? (double)row[j - 1] : 0.0, pc = (double)row[j] - prevc;
      const double u = (j + (r[2] - prevc) / pc) / W, v = (i + (r[1] - prev) / pr) / H;
      const double th = v * PI, ph = u * 2 * PI, st = sin(th);
      if (!(st > 0)) return zero;
      d = mk(st * cos(ph), cos(th), st * sin(ph));
      pdf_w = pr * pc * W * H / (2 * PI * PI * st);
      const float *p = s->env + 3 * ((size_t)i * W + j);
      le = mk(p[0], p[1], p[2]);
    } else {
      /* constant background: cosine-weighted about the receiver's normal */
      v3 t1, t2;
      onb(nl, &t1, &t2);
      const double ct = sqrt(r[1]), st = sqrt(1 - r[1]), ph = 2 * PI * r[2];
      d = add(add(mul(t1, st * cos(ph)), mul(t2, st * sin(ph))), mul(nl, ct));
      pdf_w = ct / PI;
      if (!(pdf_w > 0)) return zero;
      le = s->bg;
    }
    const double cs = dot(d, nl);
    if (!(cs > 0)) return zero;
    hitrec h;
    if (scene_closest(s, x, d, &h)) return zero;
    return mul(mulv(brdf_eval(b, d), le), cs / (pdf_w * psel));
  }
  if (s->nlights == 0) return zero;
  const double ul = s->env_prob > 0 ? (usel - s->env_prob) / (1 - s->env_prob) : usel;
  const int k = cdf_find(s->light_cdf, s->nlights, ul);
  psel = (1 - s->env_prob) * (double)s->light_pdf[k];
  const obj *o = &s->o[s->light_obj[k]];
  v3 p;
  double pdf_a, cl;
  if (o->kind == K_TRI) {
    const double su = sqrt(r[1]);
    p = add(o->p0, add(mul(o->e1, su * (1 - r[2])), mul(o->e2, su * r[2])));
    const v3 ng = cross(o->e1, o->e2);
    const double ln = sqrt(dot(ng, ng));
    pdf_a = 2.0 / ln;
    const v3 L = sub(p, x);
    const double dist2 = dot(L, L), dist = sqrt(dist2);
    d = mul(L, 1.0 / dist);
    const double det = -dot(d, ng); /* Polygon::CheckIntersection's det: the face must be hit from its front */
    if (!(det > EPS)) return zero;
    cl = det / ln;
    tmax = dist * (1 - 1e-3);
    const double cs = dot(d, nl);
    if (!(cs > 0)) return zero;
    hitrec h;
    if (scene_closest(s, x, d, &h) && h.t < tmax) return zero;
    return mul(mulv(brdf_eval(b, d), s->light_le[k]), cs * cl / (dist2 * pdf_a * psel));
  }
  /* sphere: uniform over the cap visible from x */
  const v3 diff = sub(x, o->c);
  const double dd = sqrt(dot(diff, diff)), cmax = o->r / dd;
  if (!(cmax < 1)) return zero;
  const v3 ax = mul(diff, 1.0 / dd);
  v3 t1, t2;
  onb(ax, &t1, &t2);
  const double ct = 1 - (1 - cmax) * r[1], st = sqrt(fmax(0.0, 1 - ct * ct)), ph = 2 * PI * r[2];
  const v3 nlight = add(mul(ax, ct), add(mul(t1, st * cos(ph)), mul(t2, st * sin(ph))));
  p = add(o->c, mul(nlight, o->r));
  pdf_a = 1.0 / (2 * PI * o->r * o->r * (1 - cmax));
  const v3 L = sub(p, x);
  const double dist2 = dot(L, L), dist = sqrt(dist2);
  d = mul(L, 1.0 / dist);
  cl = -dot(d, nlight);
  if (!(cl > 0)) return zero;
  tmax = dist * (1 - 1e-3);
  const double cs = dot(d, nl);
  if (!(cs > 0)) return zero;
  hitrec h;
  if (scene_closest(s, x, d, &h) && h.t < tmax) return zero;
  return mul(mulv(brdf_eval(b, d), s->light_le[k]), cs * cl / (dist2 * pdf_a * psel));
}

/* ------------------------------------------------------------------ construction */
orc_scene *orc_scene_create(const or3_scene_desc *d, int use_bvh) {
  orc_scene *s = (orc_scene *)calloc(1, sizeof(orc_scene));
  const int n = (int)(d->num_triangles + d->num_spheres + d->num_planes);
  s->n = n;
  s->o = (obj *)calloc(n > 0 ? n : 1, sizeof(obj));
  s->order = (int *)calloc(n > 0 ? n : 1, sizeof(int));
  s->m = (mat *)calloc(d->num_materials, sizeof(mat));
  for (uint32_t i = 0; i < d->num_materials; i++) {
    const or3_material *a = &d->materials[i];
    s->m[i].type = a->type;
    s->m[i].texture = a->texture;
    s->m[i].emission = ld(a->emission);
    s->m[i].color = ld(a->color);
    s->m[i].ior = a->ior;
    s->m[i].phong = a->phong_exponent;
    s->m[i].emissive = dot(s->m[i].emission, s->m[i].emission) != 0;
  }
  s->lmat = (uint32_t *)malloc(sizeof(uint32_t) * d->num_layers);
  s->lrate = (double *)malloc(sizeof(double) * d->num_layers);
  memcpy(s->lmat, d->layer_material, sizeof(uint32_t) * d->num_layers);
  memcpy(s->lrate, d->layer_rate, sizeof(double) * d->num_layers);
  uint32_t base = 0;
  /* place each object at its id */
  for (uint32_t i = 0; i < d->num_triangles; i++) {
    const uint32_t id = d->tri_ids ? d->tri_ids[i] : base + i;
    obj *o = &s->o[id];
    s->order[base + i] = (int)id;
    const double *v = d->tri_vertices + 9 * (size_t)i;
    o->kind = K_TRI;
    o->in_bvh = 1;
    o->id = id;
    o->lb = d->tri_layers[2 * i];
    o->lc = d->tri_layers[2 * i + 1];
    o->p0 = ld(v);
    o->e1 = sub(ld(v + 3), ld(v));
    o->e2 = sub(ld(v + 6), ld(v));
    if (d->tri_normals) {
      const double *nn = d->tri_normals + 9 * (size_t)i;
      o->n0 = ld(nn);
      o->dn1 = sub(ld(nn + 3), ld(nn));
      o->dn2 = sub(ld(nn + 6), ld(nn));
    } else {
      o->n0 = nrm(cross(sub(ld(v + 3), ld(v)), sub(ld(v + 6), ld(v))));
      o->dn1 = o->dn2 = mk(0, 0, 0);
    }
    if (d->tri_uvs) {
      const double *u = d->tri_uvs + 6 * (size_t)i;
      for (int a = 0; a < 2; a++) {
        o->uv0[a] = u[a];
        o->duv1[a] = u[2 + a] - u[a];
        o->duv2[a] = u[4 + a] - u[a];
      }
    }
    v3 p1 = add(o->e1, o->p0), p2 = add(o->e2, o->p0);
    o->bmin = mk(fmin(fmin(o->p0.x, p1.x), p2.x), fmin(fmin(o->p0.y, p1.y), p2.y), fmin(fmin(o->p0.z, p1.z), p2.z));
    o->bmax = mk(fmax(fmax(o->p0.x, p1.x), p2.x), fmax(fmax(o->p0.y, p1.y), p2.y), fmax(fmax(o->p0.z, p1.z), p2.z));
  }
  base += d->num_triangles;
  for (uint32_t i = 0; i < d->num_spheres; i++) {
    const uint32_t id = d->sphere_ids ? d->sphere_ids[i] : base + i;
    obj *o = &s->o[id];
    s->order[base + i] = (int)id;
    const double *sp = d->spheres + 4 * (size_t)i;
    o->kind = K_SPHERE;
    o->in_bvh = 1;
    o->id = id;
    o->lb = d->sphere_layers[2 * i];
    o->lc = d->sphere_layers[2 * i + 1];
    o->c = ld(sp);
    o->r = sp[3];
    o->bmin = sub(o->c, mk(o->r, o->r, o->r));
    o->bmax = add(o->c, mk(o->r, o->r, o->r));
  }
  base += d->num_spheres;
  for (uint32_t i = 0; i < d->num_planes; i++) {
    const uint32_t id = d->plane_ids ? d->plane_ids[i] : base + i;
    obj *o = &s->o[id];
    s->order[base + i] = (int)id;
    const double *p = d->planes + 4 * (size_t)i;
    o->kind = (int)p[0] == OR3_PLANE_INFINITE_FLOOR ? K_FLOOR : K_PLANE;
    o->in_bvh = 0;
    o->id = id;
    o->axis = (int)p[1];
    o->offset = p[2];
    o->nsign = p[3] != 0 ? -1 : 1;
    o->lb = d->plane_layers[2 * i];
    o->lc = d->plane_layers[2 * i + 1];
  }
  s->inbvh = (int *)malloc(sizeof(int) * (n > 0 ? n : 1));
  s->outbvh = (int *)malloc(sizeof(int) * (n > 0 ? n : 1));
  for (int i = 0; i < n; i++) {
    obj *o = &s->o[i];
    o->bcen = mul(add(o->bmin, o->bmax), 0.5);
    o->textured = 0;
    for (uint32_t k = 0; k < o->lc; k++)
      if (s->m[s->lmat[o->lb + k]].texture >= 0) o->textured = 1;
    if (o->in_bvh) s->inbvh[s->nin++] = i;
    else s->outbvh[s->nout++] = i;
  }
  s->use_bvh = use_bvh;
  if (use_bvh && s->nin > 0) {
    new_node(s);
    int *objs = (int *)malloc(sizeof(int) * s->nin);
    memcpy(objs, s->inbvh, sizeof(int) * s->nin);
    bvh_build(s, 0, objs, s->nin);
    free(objs);
  }
  if (d->env_rgb) {
    s->envw = (int)d->env_width;
    s->envh = (int)d->env_height;
    s->env = (float *)malloc(sizeof(float) * 3 * (size_t)s->envw * s->envh);
    memcpy(s->env, d->env_rgb, sizeof(float) * 3 * (size_t)s->envw * s->envh);
  } else if (d->env_rgbe) { /* RGBE bytes: HDRImage::RGBE2Color per texel (exact in FP32) */
    s->envw = (int)d->env_width;
    s->envh = (int)d->env_height;
    const size_t np = (size_t)s->envw * s->envh;
    double *tmp = (double *)malloc(sizeof(double) * 3 * np);
    orc_decode_rgbe(np, d->env_rgbe, tmp);
    s->env = (float *)malloc(sizeof(float) * 3 * np);
    for (size_t i = 0; i < 3 * np; i++) s->env[i] = (float)tmp[i];
    free(tmp);
  }
  s->bg = ld(d->background);
  s->ntex = (int)d->num_textures;
  if (s->ntex) {
    s->tex = (const float **)malloc(sizeof(float *) * s->ntex);
    s->texw = (uint32_t *)malloc(sizeof(uint32_t) * s->ntex);
    s->texh = (uint32_t *)malloc(sizeof(uint32_t) * s->ntex);
    for (int i = 0; i < s->ntex; i++) {
      s->texw[i] = d->texture_dims[2 * i];
      s->texh[i] = d->texture_dims[2 * i + 1];
      const size_t cnt = 3 * (size_t)s->texw[i] * s->texh[i];
      float *t = (float *)malloc(sizeof(float) * cnt);
      memcpy(t, d->texture_rgb + d->texture_offsets[i], sizeof(float) * cnt);
      s->tex[i] = t;
    }
  }
  build_lights(s);
  return s;
}

void orc_scene_destroy(orc_scene *s) {
  if (!s) return;
  free(s->o);
  free(s->m);
  free(s->lmat);
  free(s->lrate);
  free(s->inbvh);
  free(s->outbvh);
  free(s->nodes);
  free(s->leafobj);
  free(s->env);
  for (int i = 0; i < s->ntex; i++) free((void *)s->tex[i]);
  free(s->tex);
  free(s->texw);
  free(s->texh);
  free(s->order);
  free(s->light_obj);
  free(s->light_le);
  free(s->light_cdf);
  free(s->light_pdf);
  free(s->env_marg);
  free(s->env_cond);
  free(s);
}

int orc_scene_bvh_nodes(const orc_scene *s) { return s->nnodes; }

int orc_object_distance(const orc_scene *s, size_t n, const int32_t *id, const double *orig, const double *dir,
                        double *t) {
  for (size_t i = 0; i < n; i++) {
    hitrec h;
    t[i] = INF;
    if (id[i] >= 0 && id[i] < s->n && obj_hit(&s->o[id[i]], ld(orig + 3 * i), ld(dir + 3 * i), &h)) t[i] = h.t;
  }
  return 0;
}

int orc_closest(const orc_scene *s, size_t n, const double *orig, const double *dir, int32_t *id, double *t,
                double *normal) {
#pragma omp parallel for schedule(dynamic, 256)
  for (long long i = 0; i < (long long)n; i++) {
    hitrec h;
    const int hit = scene_closest(s, ld(orig + 3 * i), ld(dir + 3 * i), &h);
    id[i] = hit ? (int32_t)s->o[h.obj].id : -1;
    t[i] = hit ? h.t : INF;
    if (normal) {
      normal[3 * i] = hit ? h.normal.x : 0;
      normal[3 * i + 1] = hit ? h.normal.y : 0;
      normal[3 * i + 2] = hit ? h.normal.z : 0;
    }
  }
  return 0;
}

/* ------------------------------------------------------------------ shading */
static v3 env_sample(const orc_scene *s, v3 d) {
  if (!s->env) return s->bg;
  const double theta = acos(d.y);
  double phi = acos(d.x / sqrt(d.x * d.x + d.z * d.z));
  if (d.z < 0.0) phi = 2.0 * PI - phi;
  const double u = phi / (2.0 * PI), v = theta / PI;
  const int x = (int)(u * s->envw) % s->envw;
  const int y = (int)(v * s->envh) % s->envh;
  const float *p = s->env + 3 * ((size_t)y * s->envw + x);
  return mk(p[0], p[1], p[2]);
}

static v3 texel(const orc_scene *s, int tex, double u, double v) {
  u = (u < 0 ? 0 : u > 1 ? 1 : u) * 0.99999;
  v = (v < 0 ? 0 : v > 1 ? 1 : v) * 0.99999;
  const int x = (int)(u * s->texw[tex]), y = (int)(v * s->texh[tex]);
  const float *p = s->tex[tex] + 3 * ((size_t)y * s->texw[tex] + x);
  return mk(p[0], p[1], p[2]);
}

/* The two lookups on their own, for the pin tests: IBL::Sample(dir)
   (src/renderer/IBL.h:30-45) and Image::GetPixelByUV (src/tools/Image.h:21-31). */
void orc_env_sample(const orc_scene *s, size_t n, const double *dir, double *rgb) {
  for (size_t i = 0; i < n; i++) {
    const v3 c = env_sample(s, mk(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]));
    rgb[3 * i] = c.x;
    rgb[3 * i + 1] = c.y;
    rgb[3 * i + 2] = c.z;
  }
}

int orc_texel(const orc_scene *s, int tex, size_t n, const double *uv, double *rgb) {
  if (tex < 0 || tex >= s->ntex) return -1;
  for (size_t i = 0; i < n; i++) {
    const v3 c = texel(s, tex, uv[2 * i], uv[2 * i + 1]);
    rgb[3 * i] = c.x;
    rgb[3 * i + 1] = c.y;
    rgb[3 * i + 2] = c.z;
  }
  return 0;
}

typedef struct {
  const orc_scene *s;
  const orc_params *p;
  uint64_t g;
} pathctx;

/* spec: the ray leaves the camera or a mirror/glass vertex (no light sample
   was taken there, so next-event estimation counts the emission it reaches) */
static v3 radiance(const pathctx *c, v3 org, v3 dir, uint32_t leaf, int depth, int spec) {
  const orc_scene *s = c->s;
  const orc_params *p = c->p;
  const int nee = p->next_event_estimation != 0;
  if (p->max_depth > 0 && depth >= p->max_depth) return mk(0, 0, 0);
  hitrec h;
  if (!scene_closest(s, org, dir, &h)) return (!nee || spec) ? env_sample(s, dir) : mk(0, 0, 0);
  const obj *o = &s->o[h.obj];
  const v3 normal = dot(h.normal, dir) < 0.0 ? h.normal : mul(h.normal, -1.0);
  double r[4];
  path_rand(p->seed, c->g, leaf, (uint32_t)depth, 0, r);
  double value = r[0];
  int sel = -1;
  for (uint32_t k = 0; k < o->lc; k++) {
    if (value <= s->lrate[o->lb + k]) { sel = (int)k; break; }
    value -= s->lrate[o->lb + k];
  }
  if (sel == -1) sel = (int)o->lc - 1;
  const mat *m = &s->m[s->lmat[o->lb + sel]];
  v3 col = m->color;
  if (m->texture >= 0) col = mulv(col, texel(s, m->texture, h.u, h.v));
  /* The reference counts emission at the eye vertex only when NEE is on
     (PathTracer.cpp:433-439); with a working light sample the emission a
     BSDF ray reaches is counted after the camera or a delta vertex, or from
     an object that is not a light.  Without NEE this is every vertex. */
  const int add_emission = !nee || spec || !o->light;
  double prr = fmax(col.x, fmax(col.y, col.z));
  if (depth > 64) prr *= pow(0.5, depth - 64);
  if (depth > p->rr_min_depth) {
    /* the reference returns Background() here when NEE is on (:405-411);
       that term has no place in the NEE estimator and is left out */
    if (r[1] >= prr) return add_emission ? m->emission : mk(0, 0, 0);
  } else {
    prr = 1.0;
  }
  v3 income = mk(0, 0, 0);
  const v3 pos = h.pos;
  /* light sample at a Lambert or Phong vertex whose continuation would be traced */
  const int sample_light = nee && (p->max_depth <= 0 || depth + 1 < p->max_depth) &&
                           ((m->type == OR3_LAMBERT && !m->emissive) || m->type == OR3_PHONG);
  v3 direct = mk(0, 0, 0);
  if (sample_light) {
    double rl[4];
    path_rand(p->seed, c->g, leaf, (uint32_t)depth, 2, rl);
    brdf_t b;
    b.phong = m->type == OR3_PHONG;
    b.exponent = m->phong;
    b.col = col;
    b.mirror = nrm(sub(dir, mul(normal, 2 * dot(dir, normal))));
    direct = mul(nee_direct(s, rl, pos, normal, &b), 1.0 / prr);
  }
  switch (m->type) {
    case OR3_LAMBERT: {
      if (!m->emissive) {
        const v3 w = normal;
        const v3 u = fabs(normal.x) > EPS ? cross(mk(0, 1, 0), w) : cross(mk(1, 0, 0), w);
        const v3 v = cross(w, u);
        const double r1 = 2 * PI * r[2], r2 = sqrt(r[3]), r3 = sqrt(1 - r[3]);
        const v3 nd = nrm(add(add(mul(u, r3 * cos(r1)), mul(v, r3 * sin(r1))), mul(w, r2)));
        const v3 in = radiance(c, pos, nd, leaf, depth + 1, 0);
        income = add(mul(mulv(col, in), 1.0 / prr), direct);
      }
      break;
    }
    case OR3_SPECULAR: {
      const v3 rd = nrm(sub(dir, mul(normal, 2 * dot(dir, normal))));
      income = mulv(mul(col, 1.0 / prr), radiance(c, pos, rd, leaf, depth + 1, 1));
      break;
    }
    case OR3_REFRACTION: {
      const int into = dot(h.normal, normal) > 0.0;
      const v3 refl = nrm(sub(dir, mul(normal, 2 * dot(dir, normal))));
      const double nv = 1.0, no = m->ior;
      const double nratio = into ? nv / no : no / nv;
      const double dd = dot(dir, normal);
      const double cos2t = 1 - nratio * nratio * (1 - dd * dd);
      if (cos2t < 0) {
        income = mulv(mul(m->color, 1.0 / prr), radiance(c, pos, refl, leaf, depth + 1, 1));
        break;
      }
      const v3 refr = nrm(sub(mul(dir, nratio), mul(h.normal, (into ? 1.0 : -1.0) * (dd * nratio + sqrt(cos2t)))));
      const double F0 = (no - nv) * (no - nv) / ((no + nv) * (no + nv));
      const double cc = 1 - (into ? -dd : -dot(refr, normal));
      const double Fr = F0 + (1 - F0) * pow(cc, 5.0);
      const double Tr = (1 - Fr) * nratio * nratio;
      if (depth > 2) {
        double r2[4];
        path_rand(p->seed, c->g, leaf, (uint32_t)depth, 1, r2);
        const double pr = 0.1 + 0.8 * Fr;
        if (r2[0] < pr) {
          income = mulv(mul(col, Fr / (prr * pr)), radiance(c, pos, refl, leaf, depth + 1, 1));
        } else {
          income = mulv(mul(col, Tr / (prr * (1 - pr))), radiance(c, pos, refr, leaf, depth + 1, 1));
        }
      } else {
        const v3 a = mul(radiance(c, pos, refl, leaf, depth + 1, 1), Fr);
        const v3 b = mul(radiance(c, pos, refr, leaf | (1u << depth), depth + 1, 1), Tr);
        income = mulv(mul(col, 1.0 / prr), add(a, b));
      }
      break;
    }
    default: {
      /* Phong lobe about the mirror direction (no reference counterpart) */
      const v3 rr = nrm(sub(dir, mul(normal, 2 * dot(dir, normal))));
      const double e = m->phong;
      const double ca = pow(r[2], 1.0 / (e + 1.0));
      const double sa = sqrt(fmax(0.0, 1 - ca * ca));
      const double ph = 2 * PI * r[3];
      const double sg = rr.z >= 0 ? 1.0 : -1.0;
      const double aa = -1.0 / (sg + rr.z), bb = rr.x * rr.y * aa;
      const v3 t1 = mk(1.0 + sg * rr.x * rr.x * aa, sg * bb, -sg * rr.x);
      const v3 t2 = mk(bb, sg + rr.y * rr.y * aa, -rr.y);
      const v3 wi = nrm(add(add(mul(t1, sa * cos(ph)), mul(t2, sa * sin(ph))), mul(rr, ca)));
      const double cosn = dot(wi, normal);
      if (cosn > 0) {
        income = mulv(mul(col, (e + 2.0) / (e + 1.0) * cosn / prr), radiance(c, pos, wi, leaf, depth + 1, 0));
      }
      income = add(income, direct);
      break;
    }
  }
  if (add_emission) income = add(income, m->emission);
  return income;
}

/* ------------------------------------------------------------------ camera */
typedef struct {
  v3 pos, center, X, Y;
  double focal, aperture;
  int W, H;
} cam64;

static void cam_setup(const or3_camera *c, cam64 *k) {
  v3 dir = nrm(ld(c->direction)), up = nrm(ld(c->up));
  const double sh = c->screen_height_world, sw = c->screen_height_world * c->width / (double)c->height;
  k->pos = ld(c->position);
  k->center = add(k->pos, mul(dir, c->distance_to_screen));
  k->X = mul(nrm(cross(dir, up)), sw);
  k->Y = mul(nrm(cross(k->X, dir)), sh);
  k->focal = c->focal_distance;
  k->aperture = c->aperture_radius;
  k->W = (int)c->width;
  k->H = (int)c->height;
}

static void camera_ray(const cam64 *k, const orc_params *p, int x, int y, int sx, int sy, uint32_t lens_key,
                       uint32_t pass_first, v3 *o, v3 *d) {
  const int ss = p->supersamples;
  const double rx = (2.0 * sx + 1.0) / (2 * ss), ry = (2.0 * sy + 1.0) / (2 * ss);
  const v3 target = add(add(k->center, mul(k->X, (x + rx) / k->W - 0.5)), mul(k->Y, (y + ry) / k->H - 0.5));
  *d = nrm(sub(target, k->pos));
  *o = k->pos;
  if (k->aperture > 0) {
    uint32_t c[4] = {lens_key, pass_first, 0u, 1u}, r[4];
    orc_philox(c, (uint32_t)p->seed, (uint32_t)(p->seed >> 32), r);
    const double th = 2 * PI * u01(r[0]), rr = k->aperture * sqrt(u01(r[1]));
    const double tf = k->focal / fabs(d->z);
    const v3 focus = add(k->pos, mul(*d, tf));
    *o = add(k->pos, mk(rr * cos(th), rr * sin(th), 0));
    *d = nrm(sub(focus, *o));
  }
}

static uint32_t pass_first_of(const orc_params *p, uint32_t sidx) {
  int prev = 0;
  for (int next = p->min_samples; next <= p->max_samples; next += p->step_samples) {
    if ((int)sidx < next) return (uint32_t)prev;
    prev = next;
  }
  return (uint32_t)prev;
}

int orc_path_radiance(const orc_scene *s, const or3_camera *cam, const orc_params *p, uint64_t first,
                      uint64_t count, int nthreads, double *out) {
  cam64 k;
  cam_setup(cam, &k);
  const uint64_t ss2 = (uint64_t)p->supersamples * p->supersamples;
  const uint64_t npix = (uint64_t)k.W * k.H;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
#pragma omp parallel for schedule(dynamic, 64)
  for (long long i = 0; i < (long long)count; i++) {
    const uint64_t g = first + (uint64_t)i;
    const uint32_t subi = (uint32_t)(g % ss2);
    const uint64_t pg = g / ss2;
    const uint32_t pix = (uint32_t)(pg % npix);
    const uint32_t sidx = (uint32_t)(pg / npix);
    const int x = (int)(pix % k.W), y = (int)(pix / k.W);
    v3 o, d;
    camera_ray(&k, p, x, y, (int)(subi % p->supersamples), (int)(subi / p->supersamples),
               (uint32_t)(pix * ss2 + subi), pass_first_of(p, sidx), &o, &d);
    pathctx c = {s, p, g};
    const v3 L = radiance(&c, o, d, 0u, 0, 1);
    out[3 * i] = L.x;
    out[3 * i + 1] = L.y;
    out[3 * i + 2] = L.z;
  }
  return 0;
}

int orc_render(const orc_scene *s, const or3_camera *cam, const orc_params *p, int nthreads, double *sum,
               double *sumsq, double *seconds) {
  cam64 k;
  cam_setup(cam, &k);
  const int ss = p->supersamples;
  const uint64_t ss2 = (uint64_t)ss * ss;
  const uint64_t npix = (uint64_t)k.W * k.H;
  memset(sum, 0, sizeof(double) * 3 * npix);
  memset(sumsq, 0, sizeof(double) * 3 * npix);
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
  const double t0 = omp_get_wtime();
#else
  (void)nthreads;
  const clock_t t0 = clock();
#endif
#pragma omp parallel for schedule(dynamic, 16)
  for (long long pix = 0; pix < (long long)npix; pix++) {
    const int x = (int)(pix % k.W), y = (int)(pix / k.W);
    double *S = sum + 3 * ((size_t)(k.H - 1 - y) * k.W + x);
    double *Q = sumsq + 3 * ((size_t)(k.H - 1 - y) * k.W + x);
    int prev = 0;
    for (int next = p->min_samples; next <= p->max_samples; next += p->step_samples) {
      for (int sy = 0; sy < ss; sy++)
        for (int sx = 0; sx < ss; sx++) {
          const uint32_t subi = (uint32_t)(sy * ss + sx);
          v3 o, d;
          camera_ray(&k, p, x, y, sx, sy, (uint32_t)(pix * ss2 + subi), (uint32_t)prev, &o, &d);
          for (int sidx = prev; sidx < next; sidx++) {
            pathctx c = {s, p, ((uint64_t)sidx * npix + (uint64_t)pix) * ss2 + subi};
            const v3 L = radiance(&c, o, d, 0u, 0, 1);
            S[0] += L.x; S[1] += L.y; S[2] += L.z;
            Q[0] += L.x * L.x; Q[1] += L.y * L.y; Q[2] += L.z * L.z;
          }
        }
      prev = next;
    }
  }
#ifdef _OPENMP
  if (seconds) *seconds = omp_get_wtime() - t0;
#else
  if (seconds) *seconds = (double)(clock() - t0) / CLOCKS_PER_SEC;
#endif
  return 0;
}

/* ------------------------------------------------------------------ image conversions */
static double clamp01(double x) { return x < 0.0 ? 0.0 : x > 1.0 ? 1.0 : x; }

void orc_encode_rgb8(size_t n, const double *rgb, int gamma, uint8_t *out) {
  for (size_t i = 0; i < 3 * n; i++) {
    double v = clamp01(rgb[i]);
    if (gamma) v = pow(clamp01(v), 1.0 / 2.2);
    out[i] = (uint8_t)(int)(v * 255 + 0.5);
  }
}

void orc_encode_rgbe(size_t n, const double *rgb, uint8_t *out) {
  for (size_t i = 0; i < n; i++) {
    const double *c = rgb + 3 * i;
    uint8_t *b = out + 4 * i;
    const double mx = fmax(fmax(c[0], c[1]), c[2]);
    float v = (float)mx;
    if (v < 1e-32) {
      b[0] = b[1] = b[2] = b[3] = 0;
    } else {
      int e;
      v = frexpf(v, &e) * 256.0f / v;
      b[0] = (uint8_t)(c[0] * v);
      b[1] = (uint8_t)(c[1] * v);
      b[2] = (uint8_t)(c[2] * v);
      b[3] = (uint8_t)(e + 128);
    }
  }
}

void orc_decode_rgbe(size_t n, const uint8_t *rgbe, double *out) {
  for (size_t i = 0; i < n; i++) {
    const uint8_t *b = rgbe + 4 * i;
    if (b[3]) {
      const float f = (float)ldexp(1.0, (int)b[3] - (128 + 8));
      out[3 * i] = (double)(b[0] * f);
      out[3 * i + 1] = (double)(b[1] * f);
      out[3 * i + 2] = (double)(b[2] * f);
    } else {
      out[3 * i] = out[3 * i + 1] = out[3 * i + 2] = 0.0;
    }
  }
}
