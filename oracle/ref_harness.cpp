// ref_harness.cpp -- TEST INFRASTRUCTURE ONLY (the oracle's reference arm).
//
// Drives the reference's own, unmodified C++ classes (compiled from the
// reference sources by oracle/Makefile into oracle/_ref/) so the test suite can
// pin the oracle and the GPU path against the reference itself:
//   * orref_scene_create  builds a reference `Scene` from the flattened
//     or3_scene_desc through Scene::AddObject (src/scenes/Scene.h:48-59) and,
//     on request, Scene::ConstructBVH (src/scenes/Scene.cpp:27-34);
//   * orref_closest       calls Scene::CheckIntersection (src/scenes/Scene.cpp:51-85);
//   * orref_render_moments calls PathTracer::Radiance (src/renderer/PathTracer.cpp:180-199)
//     per camera sample with the reference's per-row RNG seeding
//     (src/renderer/PathTracer.cpp:151) and records per-pixel sums and sums of
//     squares so the tests have standard errors;
//   * orref_render_scene  runs PathTracer::RenderScene itself
//     (src/renderer/PathTracer.cpp:55-85) and returns its 2W x H buffer.
// Nothing in the product links or loads this file.
//
// The reference keeps Scene's containers protected and PathTracer::Radiance
// private; this one translation unit reaches them by compiling the reference
// headers with `private`/`protected` redefined after all standard headers are
// in, which leaves the class layouts unchanged (GCC lays members out in
// declaration order whatever their access).

#include <algorithm>
#include <atomic>
#include <cassert>
#include <cfloat>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <ctime>
#include <fstream>
#include <functional>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <stack>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#define private public
#define protected public
#include "stdafx.h"
#include "renderer/AxisAlignedPlane.h"
#include "renderer/Camera.h"
#include "renderer/IBL.h"
#include "renderer/InfiniteFloor.h"
#include "renderer/PathTracer.h"
#include "renderer/Polygon.h"
#include "renderer/Sphere.h"
#include "renderer/SphereLight.h"
#include "renderer/Model.h"
#include "scenes/Scene.h"
#include "scenes/SceneFromExternalFile.h"
#include "tools/FileSaver.h"
#include "tools/Matrix.h"
#include "tools/HDRImage.h"
#include "tools/ImageHandler.h"
#undef private
#undef protected

#include "or3.h"

using namespace OmochiRenderer;

#ifdef OR3REF_CFG
// Depth limits of the patched copy of PathTracer.cpp (see oracle/Makefile).
extern "C" {
int or3ref_min_depth = 5;
int or3ref_max_depth = 0;
}
#endif

namespace {

class HarnessScene : public Scene {
 public:
  HarnessScene() : Scene(), m_bg(0, 0, 0) {}
  Color Background() const override { return m_bg; }
  void add(SceneObject *obj, bool inBVH) { AddObject(obj, true, inBVH); }
  Color m_bg;
  std::vector<SceneObject *> byId;  // object id -> object
  std::vector<int> texIds;          // or3 texture index -> ImageHandler id
  std::unordered_map<const SceneObject *, int32_t> idOf;
};

Vector3 V(const double *p) { return Vector3(p[0], p[1], p[2]); }

Material makeMaterial(const or3_material &m, const std::vector<int> &texIds) {
  Material::REFLECTION_TYPE t = Material::REFLECTION_TYPE_LAMBERT;
  if (m.type == OR3_SPECULAR) t = Material::REFLECTION_TYPE_SPECULAR;
  if (m.type == OR3_REFRACTION) t = Material::REFLECTION_TYPE_REFRACTION;
  int tex = ImageHandler::INVALID_IMAGE_ID;
  if (m.texture >= 0 && m.texture < (int)texIds.size()) tex = texIds[m.texture];
  return Material(t, V(m.emission), V(m.color), m.ior, tex);
}

// Reproduces the object's layer list exactly (rates as given, no re-normalisation).
void setLayers(SceneObject *obj, const or3_scene_desc *d, const uint32_t *lay,
               const std::vector<int> &texIds) {
  obj->materials_.clear();
  for (uint32_t k = 0; k < lay[1]; k++) {
    const uint32_t li = lay[0] + k;
    obj->materials_.push_back(SceneObject::MultiMaterialElem(
        makeMaterial(d->materials[d->layer_material[li]], texIds), d->layer_rate[li]));
  }
}

}  // namespace

extern "C" {

void *orref_scene_create(const or3_scene_desc *d, int use_bvh) {
  HarnessScene *s = new HarnessScene();
  s->m_bg = V(d->background);

  std::vector<int> texIds;
  for (uint32_t i = 0; i < d->num_textures; i++) {
    const uint32_t w = d->texture_dims[2 * i], h = d->texture_dims[2 * i + 1];
    int id = ImageHandler::GetInstance().CreateImage(w, h);
    Image *img = ImageHandler::GetInstance().GetImage(id);
    const float *src = d->texture_rgb + d->texture_offsets[i];
    for (size_t p = 0; p < (size_t)w * h; p++)
      img->m_image[p] = Color(src[3 * p], src[3 * p + 1], src[3 * p + 2]);
    texIds.push_back(id);
  }
  s->texIds = texIds;

  // (id, class, index) sorted by id = the reference's insertion order.
  struct Rec { uint32_t id; int cls; uint32_t idx; };
  std::vector<Rec> recs;
  uint32_t base = 0;
  for (uint32_t i = 0; i < d->num_triangles; i++)
    recs.push_back({d->tri_ids ? d->tri_ids[i] : base + i, 0, i});
  base += d->num_triangles;
  for (uint32_t i = 0; i < d->num_spheres; i++)
    recs.push_back({d->sphere_ids ? d->sphere_ids[i] : base + i, 1, i});
  base += d->num_spheres;
  for (uint32_t i = 0; i < d->num_planes; i++)
    recs.push_back({d->plane_ids ? d->plane_ids[i] : base + i, 2, i});
  std::sort(recs.begin(), recs.end(), [](const Rec &a, const Rec &b) { return a.id < b.id; });

  const Material dummy;
  for (const Rec &r : recs) {
    SceneObject *obj = nullptr;
    bool inBVH = true;
    if (r.cls == 0) {
      const double *v = d->tri_vertices + 9 * r.idx;
      Vector3 p0 = V(v), p1 = V(v + 3), p2 = V(v + 6);
      Vector3 n0, n1, n2;
      if (d->tri_normals) {
        const double *n = d->tri_normals + 9 * r.idx;
        n0 = V(n); n1 = V(n + 3); n2 = V(n + 6);
      } else {
        n0 = n1 = n2 = Polygon::CalculateNormal(p0, p1, p2);
      }
      Vector3 uv0, uv1, uv2;
      if (d->tri_uvs) {
        const double *u = d->tri_uvs + 6 * r.idx;
        uv0 = Vector3(u[0], u[1], 0); uv1 = Vector3(u[2], u[3], 0); uv2 = Vector3(u[4], u[5], 0);
      }
      obj = new Polygon(p0, p1, p2, uv0, uv1, uv2, n0, n1, n2, dummy, Vector3(0, 0, 0));
      setLayers(obj, d, d->tri_layers + 2 * r.idx, texIds);
    } else if (r.cls == 1) {
      const double *sp = d->spheres + 4 * r.idx;
      const bool light = d->sphere_flags && (d->sphere_flags[r.idx] & OR3_SPHERE_LIGHT);
      if (light) obj = new SphereLight(sp[3], V(sp), dummy);
      else obj = new Sphere(sp[3], V(sp), dummy);
      setLayers(obj, d, d->sphere_layers + 2 * r.idx, texIds);
    } else {
      const double *pl = d->planes + 4 * r.idx;
      if ((int)pl[0] == OR3_PLANE_INFINITE_FLOOR) {
        obj = new InfiniteFloor(pl[2], dummy);
      } else {
        AxisAlignedPlane::PLANE_AXIS ax = AxisAlignedPlane::PLANE_XY;
        if ((int)pl[1] == 1) ax = AxisAlignedPlane::PLANE_XZ;
        if ((int)pl[1] == 2) ax = AxisAlignedPlane::PLANE_YZ;
        obj = new AxisAlignedPlane(dummy, ax, pl[2], pl[3] != 0.0);
      }
      setLayers(obj, d, d->plane_layers + 2 * r.idx, texIds);
      inBVH = false;
    }
    s->add(obj, inBVH);
    if (s->byId.size() <= r.id) s->byId.resize(r.id + 1, nullptr);
    s->byId[r.id] = obj;
    s->idOf[obj] = (int32_t)r.id;
  }

  if ((d->env_rgb || d->env_rgbe) && d->env_width && d->env_height) {
    // The IBL constructor only reads a .hdr file; feed the float image instead
    // (no RGBE quantisation), or RGBE bytes through HDRImage::RGBE2Color.
    std::streambuf *old = std::cerr.rdbuf(nullptr);
    IBL *ibl = new IBL("");
    std::cerr.rdbuf(old);
    ibl->m_image.m_width = d->env_width;
    ibl->m_image.m_height = d->env_height;
    ibl->m_image.m_image.resize((size_t)d->env_width * d->env_height);
    for (size_t p = 0; p < (size_t)d->env_width * d->env_height; p++) {
      if (d->env_rgb) {
        ibl->m_image.m_image[p] = Color(d->env_rgb[3 * p], d->env_rgb[3 * p + 1], d->env_rgb[3 * p + 2]);
      } else {
        unsigned char b[4] = {d->env_rgbe[4 * p], d->env_rgbe[4 * p + 1], d->env_rgbe[4 * p + 2], d->env_rgbe[4 * p + 3]};
        HDRImage::RGBE2Color(b, ibl->m_image.m_image[p]);
      }
    }
    s->m_ibl.reset(ibl);
  }
  if (use_bvh && !s->m_inBVHObjects.empty()) s->ConstructBVH();
  return s;
}

void orref_scene_destroy(void *p) { delete static_cast<HarnessScene *>(p); }

// IBL::Sample(const Vector3 &) (src/renderer/IBL.h:30-45) of the scene's IBL
// for n directions (used as given, unit length expected); -1 without an IBL.
int orref_ibl_sample(void *p, size_t n, const double *dir, double *rgb) {
  HarnessScene *s = static_cast<HarnessScene *>(p);
  if (!s->m_ibl.get()) return -1;
  for (size_t i = 0; i < n; i++) {
    const Color &c = s->m_ibl->Sample(V(dir + 3 * i));
    rgb[3 * i] = c.x; rgb[3 * i + 1] = c.y; rgb[3 * i + 2] = c.z;
  }
  return 0;
}

// Image::GetPixelByUV (src/tools/Image.h:20-31) of the scene's texture `tex`.
int orref_texel(void *p, int tex, size_t n, const double *uv, double *rgb) {
  HarnessScene *s = static_cast<HarnessScene *>(p);
  if (tex < 0 || tex >= (int)s->texIds.size()) return -1;
  Image *img = ImageHandler::GetInstance().GetImage(s->texIds[tex]);
  if (!img) return -1;
  for (size_t i = 0; i < n; i++) {
    const Color &c = img->GetPixelByUV(uv[2 * i], uv[2 * i + 1]);
    rgb[3 * i] = c.x; rgb[3 * i + 1] = c.y; rgb[3 * i + 2] = c.z;
  }
  return 0;
}

// Closest hit of n rays through Scene::CheckIntersection.
int orref_closest(void *p, size_t n, const double *orig, const double *dir, int32_t *id,
                  double *t, double *normal, double *pos) {
  HarnessScene *s = static_cast<HarnessScene *>(p);
  for (size_t i = 0; i < n; i++) {
    Ray ray(V(orig + 3 * i), V(dir + 3 * i));
    Scene::IntersectionInformation info;
    const bool hit = s->CheckIntersection(ray, info);
    id[i] = hit ? s->idOf[info.object] : -1;
    t[i] = hit ? info.hit.distance : INF;
    for (int k = 0; k < 3; k++) {
      const double nv = k == 0 ? info.hit.normal.x : k == 1 ? info.hit.normal.y : info.hit.normal.z;
      const double pv = k == 0 ? info.hit.position.x : k == 1 ? info.hit.position.y : info.hit.position.z;
      if (normal) normal[3 * i + k] = hit ? nv : 0.0;
      if (pos) pos[3 * i + k] = hit ? pv : 0.0;
    }
  }
  return 0;
}

static Camera makeCamera(const or3_camera *c) {
  Camera cam(c->width, c->height, V(c->position), V(c->direction), V(c->up),
             c->screen_height_world, c->distance_to_screen, c->focal_distance);
  if (c->aperture_radius > 0) cam.SetAperture(std::make_shared<CircleAperture>(c->aperture_radius));
  return cam;
}

#ifdef OR3REF_CFG
void orref_set_depth_limits(int rr_min_depth, int max_depth) {
  or3ref_min_depth = rr_min_depth;
  or3ref_max_depth = max_depth;
}
#endif

// Per-pixel moments of the reference estimator.  Each camera sample is one
// PathTracer::Radiance call, exactly as in scanPixelsOnYAndCastRays
// (src/renderer/PathTracer.cpp:143-175): per (row, pass) Random seed
// y+1+prev*H, fixed ss x ss grid, one camera ray per sub-pixel per pass.
// Rows are spread over `nthreads` threads dynamically.  sum/sumsq: W*H*3,
// rows top-down.  Returns the wall-clock seconds in *seconds.
int orref_render_moments(void *p, const or3_camera *c, int min_s, int max_s, int step, int ss,
                         int nthreads, int nee, double *sum, double *sumsq, double *seconds) {
  HarnessScene *s = static_cast<HarnessScene *>(p);
  Camera cam = makeCamera(c);
  PathTracer pt(cam, min_s, max_s, step, ss, nullptr);
  pt.EnableNextEventEstimation(nee != 0);
  const int W = (int)c->width, H = (int)c->height;
  std::memset(sum, 0, sizeof(double) * 3 * W * H);
  std::memset(sumsq, 0, sizeof(double) * 3 * W * H);
  if (nthreads <= 0) nthreads = (int)std::thread::hardware_concurrency();
  auto t0 = std::chrono::steady_clock::now();
  int prev = 0;
  for (int next = min_s; next <= max_s; next += step) {
    std::atomic<int> row(0);
    auto work = [&]() {
      for (int y = row.fetch_add(1); y < H; y = row.fetch_add(1)) {
        Random rnd(static_cast<unsigned int>(y + 1 + prev * H));
        for (int x = 0; x < W; x++) {
          double *S = sum + 3 * ((size_t)(H - 1 - y) * W + x);
          double *Q = sumsq + 3 * ((size_t)(H - 1 - y) * W + x);
          for (int sy = 0; sy < ss; sy++)
            for (int sx = 0; sx < ss; sx++) {
              const double rx = (2.0 * sx + 1.0) / (2 * ss);
              const double ry = (2.0 * sy + 1.0) / (2 * ss);
              Ray ray(cam.SampleRayForPixel(x + rx, y + ry, rnd));
              for (int k = prev + 1; k <= next; k++) {
                Color L = pt.Radiance(*s, ray, rnd, 0);
                S[0] += L.x; S[1] += L.y; S[2] += L.z;
                Q[0] += L.x * L.x; Q[1] += L.y * L.y; Q[2] += L.z * L.z;
              }
            }
        }
      }
    };
    std::vector<std::thread> th;
    for (int i = 0; i < nthreads; i++) th.emplace_back(work);
    for (auto &t : th) t.join();
    prev = next;
  }
  if (seconds)
    *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return 0;
}

// The reference's own PathTracer::RenderScene.  `out` receives the
// 2W x H result buffer (ScreenPixels::GetScreen); with nthreads <= 2 the whole
// image lies in the left viewport (src/renderer/PathTracer.cpp:104-111).
int orref_render_scene(void *p, const or3_camera *c, int min_s, int max_s, int step, int ss,
                       int nthreads, int nee, double *out, double *seconds) {
  HarnessScene *s = static_cast<HarnessScene *>(p);
  Camera cam = makeCamera(c);
  PathTracer *pt = new PathTracer(cam, min_s, max_s, step, ss, nullptr);
  pt->EnableNextEventEstimation(nee != 0);
  pt->SetMaxThreadCount(nthreads);
  std::streambuf *old = std::cerr.rdbuf(nullptr);
  auto t0 = std::chrono::steady_clock::now();
  pt->RenderScene(*s);
  double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::cerr.rdbuf(old);
  const ScreenPixels *px = pt->GetResult();
  const size_t n = px->CalcScreenWidth() * px->CalcScreenHeight();
  const Color *img = px->GetScreen();
  for (size_t i = 0; i < n; i++) {
    out[3 * i] = img[i].x; out[3 * i + 1] = img[i].y; out[3 * i + 2] = img[i].z;
  }
  if (seconds) *seconds = sec;
  // PathTracer's destructor frees a scalar `new` with delete[]
  // (src/renderer/PathTracer.cpp:52 vs :62); free the result here so that
  // destructor only sees a null pointer.
  delete pt->m_result;
  pt->m_result = nullptr;
  delete pt;
  return 0;
}

// ---- image output and input (the savers' 8-bit conversion, RGBE)

// FileSaver::CopyColorArrayToImage (src/tools/FileSaver.h:49-120, gamma on or
// off) followed by ImageHandler::SaveToPngFile's Utils::ToRgb
// (src/tools/ImageHandler.cpp:133-155): the bytes the reference writes.
void orref_encode_rgb8(size_t n, const double *rgb, int gamma, uint8_t *out) {
  std::vector<Color> img(n), conv;
  for (size_t i = 0; i < n; i++) img[i] = Color(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]);
  FileSaver::CopyColorArrayToImage(img.data(), conv, static_cast<int>(n), 1, gamma != 0);
  for (size_t i = 0; i < n; i++) {
    out[3 * i] = static_cast<unsigned char>(Utils::ToRgb(conv[i].x));
    out[3 * i + 1] = static_cast<unsigned char>(Utils::ToRgb(conv[i].y));
    out[3 * i + 2] = static_cast<unsigned char>(Utils::ToRgb(conv[i].z));
  }
}

// HDRImage::Color2RGBE / RGBE2Color (src/tools/HDRImage.h:10-38).
void orref_encode_rgbe(size_t n, const double *rgb, uint8_t *out) {
  for (size_t i = 0; i < n; i++) HDRImage::Color2RGBE(out + 4 * i, Color(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]));
}

void orref_decode_rgbe(size_t n, const uint8_t *rgbe, double *out) {
  for (size_t i = 0; i < n; i++) {
    unsigned char b[4] = {rgbe[4 * i], rgbe[4 * i + 1], rgbe[4 * i + 2], rgbe[4 * i + 3]};
    Color c;
    HDRImage::RGBE2Color(b, c);
    out[3 * i] = c.x;
    out[3 * i + 1] = c.y;
    out[3 * i + 2] = c.z;
  }
}

// HDRImage::WriteToRadianceFile / ReadFromRadianceFile (src/tools/HDRImage.cpp).
int orref_write_hdr(const char *path, int w, int h, const double *rgb) {
  HDRImage img;
  img.m_width = w;
  img.m_height = h;
  img.m_image.resize((size_t)w * h);
  for (size_t i = 0; i < (size_t)w * h; i++) img.m_image[i] = Color(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]);
  return img.WriteToRadianceFile(path) ? 0 : -1;
}

int orref_read_hdr(const char *path, int *w, int *h, double *out, size_t capacity) {
  HDRImage img;
  if (!img.ReadFromRadianceFile(path)) return -1;
  *w = static_cast<int>(img.GetWidth());
  *h = static_cast<int>(img.GetHeight());
  if (!out) return 0;
  if (capacity < 3 * img.m_image.size()) return -2;
  for (size_t i = 0; i < img.m_image.size(); i++) {
    out[3 * i] = img.m_image[i].x;
    out[3 * i + 1] = img.m_image[i].y;
    out[3 * i + 2] = img.m_image[i].z;
  }
  return 0;
}

// Model::ReadFromObj (src/renderer/Model.cpp:50-182) and the Transform that
// SceneFromExternalFile::ReadMesh applies (src/scenes/SceneFromExternalFile.cpp:518-527);
// every polygon of every material list, as Scene::AddModel would add them.
// tri: [n][3][3] world vertices, nrm: [n][3][3], uv: [n][3][2], mat: [n][5]
// (type, r, g, b, ior).  Returns the triangle count (or -1), filling at most cap.
long orref_load_obj(const char *path, int flip_v, const double *pos, const double *scale, const double *rot,
                    double *tri, double *nrm, double *uv, double *mat, long cap) {
  Model model;
  std::streambuf *old = std::cerr.rdbuf(nullptr);
  const bool ok = model.ReadFromObj(path, flip_v != 0);
  std::cerr.rdbuf(old);
  if (!ok) return -1;
  model.Transform(Vector3(pos[0], pos[1], pos[2]), Vector3(scale[0], scale[1], scale[2]),
                  Matrix::RotateAroundVector(Vector3(0, 0, 1), rot[2]) *
                      Matrix::RotateAroundVector(Vector3(0, 1, 0), rot[1]) *
                      Matrix::RotateAroundVector(Vector3(1, 0, 0), rot[0]));
  long n = 0;
  for (size_t i = 0; i < model.GetMaterialCount(); i++) {
    const Material &m = model.GetMaterial(i);
    const Model::PolygonList &pl = model.GetPolygonList(m);
    for (size_t j = 0; j < pl.size(); j++, n++) {
      if (n >= cap) continue;
      const Polygon *p = pl[j];
      const Vector3 v0 = p->m_posAndEdges[0] + p->position_;
      const Vector3 v[3] = {v0, v0 + p->m_posAndEdges[1], v0 + p->m_posAndEdges[2]};
      const Vector3 n0 = p->m_normalAndDiffs[0];
      const Vector3 nn[3] = {n0, n0 + p->m_normalAndDiffs[1], n0 + p->m_normalAndDiffs[2]};
      const Vector3 u0 = p->m_uvOrigAndEdges[0];
      const Vector3 uu[3] = {u0, u0 + p->m_uvOrigAndEdges[1], u0 + p->m_uvOrigAndEdges[2]};
      for (int k = 0; k < 3; k++) {
        tri[9 * n + 3 * k] = v[k].x; tri[9 * n + 3 * k + 1] = v[k].y; tri[9 * n + 3 * k + 2] = v[k].z;
        nrm[9 * n + 3 * k] = nn[k].x; nrm[9 * n + 3 * k + 1] = nn[k].y; nrm[9 * n + 3 * k + 2] = nn[k].z;
        uv[6 * n + 2 * k] = uu[k].x; uv[6 * n + 2 * k + 1] = uu[k].y;
      }
      mat[5 * n] = (double)m.reflection_type;
      mat[5 * n + 1] = m.color.x; mat[5 * n + 2] = m.color.y; mat[5 * n + 3] = m.color.z;
      mat[5 * n + 4] = m.refraction_rate;
    }
  }
  return n;
}

// SceneFromExternalFile (src/scenes/SceneFromExternalFile.cpp:47-182): the
// scene a text scene file describes, one record of kSceneRec doubles per
// object in Scene::m_objects order: kind (0 polygon, 1 sphere, 2 sphere
// light, 3 infinite floor, 4 other), in BVH, layer count, 24 of geometry
// (polygon: world vertices 9, normals 9, uvs 6; sphere: centre, radius;
// infinite floor: y), then up to 4 layers of (type, emission 3, colour 3,
// ior, rate, has texture).  ibl[0..1] get the IBL image's width and height
// (0 without one) and ibl[2..4] the sum of its texels.  Returns the object
// count, or -1 when the reference rejects the file.
static const int kSceneRec = 67;
long orref_load_scene_file(const char *path, double *rec, long cap, double *ibl) {
  std::streambuf *old = std::cerr.rdbuf(nullptr);
  SceneFromExternalFile scene(path);
  std::cerr.rdbuf(old);
  if (!scene.IsValid()) return -1;
  long n = 0;
  for (const auto &info : scene.m_objects) {
    if (n >= cap) { n++; continue; }
    double *r = rec + (size_t)kSceneRec * n;
    std::fill(r, r + kSceneRec, 0.0);
    const SceneObject *o = info.object;
    r[1] = info.inBVH ? 1 : 0;
    if (const Polygon *p = dynamic_cast<const Polygon *>(o)) {
      r[0] = 0;
      const Vector3 v0 = p->m_posAndEdges[0] + p->position_;
      const Vector3 v[3] = {v0, v0 + p->m_posAndEdges[1], v0 + p->m_posAndEdges[2]};
      const Vector3 n0 = p->m_normalAndDiffs[0];
      const Vector3 nn[3] = {n0, n0 + p->m_normalAndDiffs[1], n0 + p->m_normalAndDiffs[2]};
      const Vector3 u0 = p->m_uvOrigAndEdges[0];
      const Vector3 uu[3] = {u0, u0 + p->m_uvOrigAndEdges[1], u0 + p->m_uvOrigAndEdges[2]};
      for (int k = 0; k < 3; k++) {
        r[3 + 3 * k] = v[k].x; r[4 + 3 * k] = v[k].y; r[5 + 3 * k] = v[k].z;
        r[12 + 3 * k] = nn[k].x; r[13 + 3 * k] = nn[k].y; r[14 + 3 * k] = nn[k].z;
        r[21 + 2 * k] = uu[k].x; r[22 + 2 * k] = uu[k].y;
      }
    } else if (const Sphere *sp = dynamic_cast<const Sphere *>(o)) {
      r[0] = dynamic_cast<const SphereLight *>(o) ? 2 : 1;
      r[3] = sp->position_.x; r[4] = sp->position_.y; r[5] = sp->position_.z; r[6] = sp->m_radius;
    } else if (const InfiniteFloor *f = dynamic_cast<const InfiniteFloor *>(o)) {
      r[0] = 3;
      r[3] = f->y;
    } else {
      r[0] = 4;
    }
    r[2] = (double)o->GetMaterialCount();
    for (size_t l = 0; l < o->GetMaterialCount() && l < 4; l++) {
      const SceneObject::MultiMaterialElem *e = o->GetMaterial(l);
      double *m = r + 27 + 10 * l;
      m[0] = (double)e->material_.reflection_type;
      m[1] = e->material_.emission.x; m[2] = e->material_.emission.y; m[3] = e->material_.emission.z;
      m[4] = e->material_.color.x; m[5] = e->material_.color.y; m[6] = e->material_.color.z;
      m[7] = e->material_.refraction_rate;
      m[8] = e->rate_;
      m[9] = e->material_.texture_id != ImageHandler::INVALID_IMAGE_ID ? 1 : 0;
    }
    n++;
  }
  ibl[0] = ibl[1] = ibl[2] = ibl[3] = ibl[4] = 0;
  if (scene.m_ibl.get()) {
    const Image &im = scene.m_ibl->m_image;
    ibl[0] = (double)im.GetWidth();
    ibl[1] = (double)im.GetHeight();
    for (const Color &c : im.m_image) { ibl[2] += c.x; ibl[3] += c.y; ibl[4] += c.z; }
  }
  return n;
}

}  // extern "C"
