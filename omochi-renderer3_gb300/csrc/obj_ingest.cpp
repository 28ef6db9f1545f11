// obj_ingest.cpp -- Wavefront .obj/.mtl straight to structure-of-arrays
// triangles (or3_mesh_load_obj), without a per-triangle object.
//
// Reads what Model::ReadFromObj and Model::LoadMaterialFile read
// (src/renderer/Model.cpp:50-182 and :184-292), with their rules:
//   * lines split on single spaces; "v x y z" and "vn x y z" need exactly three
//     numbers, "vt u v [w]" at least two (v flipped to 1 - v on request);
//   * "f" with 3 vertices is a triangle, 4 a quad split (0,1,2) (0,2,3), 5 or
//     more a fan (0, i+1, i+2); a vertex is "v", "v/t", "v/t/n" or "v//n",
//     1-based; missing uvs are 0; when no vertex of a face has a normal the
//     face normal normalize((v1 - v0) x (v2 - v0)) goes to all three
//     (Polygon::CalculateNormal, src/renderer/Polygon.h:45-49), otherwise a
//     vertex without one gets (0, 0, 0);
//   * "g" returns to the default material (Lambert, colour 0.99), "usemtl"
//     selects a material of the .mtl ("mtllib", relative to the .obj);
//   * .mtl: "illum" 0-2 Lambert, "illum 3 <ior>" refraction; the colour is Kd
//     (Ks for a specular type); type, Kd, Ks and the IOR carry over from one
//     "newmtl" to the next, as the reference's reader keeps them.
// Differences, on purpose: triangles come in file order (the reference adds
// them grouped by material in hash-map order, and adds a group twice when two
// materials are equal in value); a "map_Kd" belongs to the material it follows
// (the reference gives the last texture read to the last material only).
// Textures are returned as paths; loading the image stays with the caller.
//
// Large files parse on all host threads: the file is cut at line boundaries,
// each chunk counts and then parses its own lines, and face indices resolve
// against the global vertex arrays afterwards.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "or3.h"

namespace {

struct V3d {
  double x, y, z;
};

// single-space split (Utils::split, src/tools/Utils.h:13-35): empty fields kept
// between adjacent spaces, none after a trailing space
int split_spaces(const char *b, const char *e, const char **tok, const char **tend, int max) {
  int n = 0;
  const char *p = b;
  while (p < e) {
    const char *q = p;
    while (q < e && *q != ' ') q++;
    if (n < max) {
      tok[n] = p;
      tend[n] = q;
    }
    n++;
    p = q + (q < e ? 1 : 0);
    if (q == e) break;
  }
  return n;
}

double num(const char *b, const char *e) {  // atof on [b, e)
  char buf[64];
  const size_t n = std::min<size_t>(e - b, sizeof(buf) - 1);
  std::memcpy(buf, b, n);
  buf[n] = 0;
  return std::atof(buf);
}

struct FaceVert {
  int64_t v, t, n;  // 0-based; -1 = absent
};

struct Chunk {
  const char *b, *e;
  std::vector<V3d> v, vt, vn;
  // faces: polygons as runs of vertices, each with the material event index in force
  std::vector<FaceVert> fv;
  std::vector<uint32_t> fstart;  // polygon start in fv (size = polygons + 1)
  std::vector<std::string> events;  // "g" (empty string) or "usemtl name", in order
  std::vector<uint32_t> fevent;     // per polygon: number of events seen in this chunk before it
  std::vector<std::string> mtllibs;
  bool error = false;
  std::string error_line;
};

bool starts(const char *b, const char *e, const char *lit) {
  const size_t n = std::strlen(lit);
  return (size_t)(e - b) >= n && std::memcmp(b, lit, n) == 0;
}

void parse_chunk(Chunk &c, int flip_v) {
  const char *p = c.b;
  const char *tok[64], *te[64];
  c.fstart.push_back(0);
  while (p < c.e && !c.error) {
    const char *le = (const char *)std::memchr(p, '\n', c.e - p);
    if (!le) le = c.e;
    const char *lb = p;
    const char *lend = le;
    if (lend > lb && lend[-1] == '\r') lend--;  // getline keeps '\r'; the number parsers stop at it
    p = le + (le < c.e ? 1 : 0);
    if (lend == lb || *lb == '#') continue;
    if (starts(lb, lend, "mtllib ")) {
      c.mtllibs.emplace_back(lb + 7, lend);
    } else if (starts(lb, lend, "g ")) {
      c.events.emplace_back();
    } else if (starts(lb, lend, "usemtl ")) {
      c.events.emplace_back(std::string("u") + std::string(lb + 7, lend));
    } else if (starts(lb, lend, "v ")) {
      const int n = split_spaces(lb + 2, lend, tok, te, 64);
      if (n != 3) {
        c.error = true;
        c.error_line.assign(lb, lend);
        break;
      }
      c.v.push_back({num(tok[0], te[0]), num(tok[1], te[1]), num(tok[2], te[2])});
    } else if (starts(lb, lend, "vt ")) {
      const int n = split_spaces(lb + 3, lend, tok, te, 64);
      if (n < 2) {
        c.error = true;
        c.error_line.assign(lb, lend);
        break;
      }
      double v = num(tok[1], te[1]);
      if (flip_v) v = 1 - v;
      c.vt.push_back({num(tok[0], te[0]), v, 0.0});
    } else if (starts(lb, lend, "vn ")) {
      const int n = split_spaces(lb + 3, lend, tok, te, 64);
      if (n != 3) {
        c.error = true;
        c.error_line.assign(lb, lend);
        break;
      }
      c.vn.push_back({num(tok[0], te[0]), num(tok[1], te[1]), num(tok[2], te[2])});
    } else if (starts(lb, lend, "f ")) {
      const int n = split_spaces(lb + 2, lend, tok, te, 64);
      if (n < 3 || n > 64) {
        if (n > 64) {
          c.error = true;
          c.error_line.assign(lb, lend);
        }
        continue;  // the reference ignores faces of fewer than 3 vertices
      }
      for (int k = 0; k < n; k++) {
        // "v", "v/t", "v/t/n", "v//n"
        const char *f[3] = {tok[k], nullptr, nullptr}, *fe[3] = {te[k], nullptr, nullptr};
        int parts = 1;
        for (const char *q = tok[k]; q < te[k]; q++)
          if (*q == '/') {
            fe[parts - 1] = q;
            if (parts == 3) break;
            f[parts] = q + 1;
            fe[parts] = te[k];
            parts++;
          }
        FaceVert v{num(f[0], fe[0]) > 0 ? (int64_t)num(f[0], fe[0]) - 1 : -2, -1, -1};
        if (parts >= 2 && fe[1] > f[1]) v.t = (int64_t)num(f[1], fe[1]) - 1;
        if (parts == 3) v.n = (int64_t)num(f[2], fe[2]) - 1;
        c.fv.push_back(v);
      }
      c.fstart.push_back((uint32_t)c.fv.size());
      c.fevent.push_back((uint32_t)c.events.size());
    }
  }
}

struct Mtl {
  or3_material m;
  std::string name, texture;
};

// Model::LoadMaterialFile's reading of a .mtl
bool load_mtl(const std::string &path, std::vector<Mtl> &out) {
  std::ifstream ifs(path.c_str());
  if (!ifs) return false;
  std::string base;
  {
    std::string f = path;
    std::replace(f.begin(), f.end(), '\\', '/');
    const size_t pos = f.find_last_of('/');
    if (pos != std::string::npos && pos > 0) base = f.substr(0, pos);
  }
  std::string name;
  int type = OR3_LAMBERT;
  double ior = 0.0, kd[3] = {0, 0, 0}, ks[3] = {0, 0, 0};
  std::string tex;
  auto reg = [&]() {
    Mtl m{};
    m.m.type = type;
    m.m.texture = -1;
    m.m.ior = ior;
    const double *c = type == OR3_SPECULAR ? ks : kd;
    for (int a = 0; a < 3; a++) m.m.color[a] = c[a];
    m.name = name;
    m.texture = tex;
    out.push_back(m);
  };
  std::string line;
  const char *tok[16], *te[16];
  while (std::getline(ifs, line)) {
    if (!line.empty() && line.back() == '\r') line.pop_back();
    const char *b = line.data(), *e = b + line.size();
    if (line.empty() || line[0] == '#') continue;
    if (starts(b, e, "newmtl ")) {
      if (!name.empty()) reg();
      name.assign(b + 7, e);
      tex.clear();
    } else if (starts(b, e, "illum ")) {
      const int n = split_spaces(b + 6, e, tok, te, 16);
      if (n < 1) continue;
      const int v = (int)num(tok[0], te[0]);
      if (v >= 0 && v <= 2) type = OR3_LAMBERT;
      if (v == 3 && n >= 2) {
        type = OR3_REFRACTION;
        ior = num(tok[1], te[1]);
      }
    } else if (starts(b, e, "Kd ") || starts(b, e, "Ks ")) {
      const int n = split_spaces(b + 3, e, tok, te, 16);
      if (n != 3) continue;
      double *d = line[1] == 'd' ? kd : ks;
      for (int a = 0; a < 3; a++) d[a] = num(tok[a], te[a]);
    } else if (starts(b, e, "map_Kd ")) {
      tex.assign(b + 7, e);
      if (!base.empty()) tex = base + "/" + tex;
    }
  }
  if (!name.empty()) reg();
  return true;
}

char *dup(const std::string &s) {
  char *p = (char *)std::malloc(s.size() + 1);
  std::memcpy(p, s.c_str(), s.size() + 1);
  return p;
}

}  // namespace

extern "C" {

void or3_mesh_free(or3_mesh *m) {
  if (!m) return;
  std::free(m->vertices);
  std::free(m->normals);
  std::free(m->uvs);
  std::free(m->material);
  for (uint32_t i = 0; i < m->num_materials; i++) {
    std::free(m->material_names ? m->material_names[i] : nullptr);
    std::free(m->texture_paths ? m->texture_paths[i] : nullptr);
  }
  std::free(m->materials);
  std::free(m->material_names);
  std::free(m->texture_paths);
  std::free(m);
}

int or3_mesh_load_obj(const char *path, int32_t flip_v, uint32_t threads, or3_mesh **out) {
  if (!path || !out) return OR3_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  std::ifstream ifs(path, std::ios::binary | std::ios::ate);
  if (!ifs) return OR3_ERR_NOT_FOUND;
  std::string text;
  {
    const std::streamoff size = ifs.tellg();
    if (size < 0) return OR3_ERR_NOT_FOUND;
    text.resize((size_t)size);
    ifs.seekg(0);
    if (size > 0 && !ifs.read(&text[0], size)) return OR3_ERR_NOT_FOUND;
  }
  std::string base;
  {
    const std::string f(path);
    const size_t pos = f.find_last_of('/');
    if (pos != std::string::npos) base = f.substr(0, pos);
  }
  // chunks at line boundaries
  unsigned nt = threads ? threads : std::thread::hardware_concurrency();
  nt = std::max(1u, std::min(nt, 64u));
  if (text.size() < (1u << 20)) nt = 1;
  std::vector<Chunk> ch(nt);
  const char *b = text.data(), *e = b + text.size();
  for (unsigned k = 0; k < nt; k++) {
    const char *s = k == 0 ? b : ch[k - 1].e;
    const char *t = k + 1 == nt ? e : b + text.size() * (k + 1) / nt;
    if (t < s) t = s;
    while (t < e && t > s && t[-1] != '\n') t++;  // end after a newline
    ch[k].b = s;
    ch[k].e = t;
  }
  {
    std::vector<std::thread> pool;
    for (unsigned k = 1; k < nt; k++) pool.emplace_back(parse_chunk, std::ref(ch[k]), flip_v);
    parse_chunk(ch[0], flip_v);
    for (auto &t : pool) t.join();
  }
  for (const Chunk &c : ch)
    if (c.error) return OR3_ERR_INVALID_ARGUMENT;
  // materials: index 0 = the default (Lambert 0.99), then every .mtl's in order
  std::vector<Mtl> mats(1);
  mats[0].name = "__default__material__";
  mats[0].m.type = OR3_LAMBERT;
  mats[0].m.texture = -1;
  for (int a = 0; a < 3; a++) mats[0].m.color[a] = 0.99;
  for (const Chunk &c : ch)
    for (const std::string &lib : c.mtllibs)
      if (!load_mtl(base.empty() ? lib : base + "/" + lib, mats)) return OR3_ERR_NOT_FOUND;
  std::map<std::string, uint32_t> by_name;  // a later definition of a name wins, as in the reference's map
  for (uint32_t i = 0; i < mats.size(); i++) by_name[mats[i].name] = i;
  // global vertex arrays and per-chunk offsets
  std::vector<size_t> vo(nt + 1, 0), to(nt + 1, 0), no(nt + 1, 0);
  for (unsigned k = 0; k < nt; k++) {
    vo[k + 1] = vo[k] + ch[k].v.size();
    to[k + 1] = to[k] + ch[k].vt.size();
    no[k + 1] = no[k] + ch[k].vn.size();
  }
  std::vector<V3d> V(vo[nt]), T(to[nt]), N(no[nt]);
  for (unsigned k = 0; k < nt; k++) {
    std::copy(ch[k].v.begin(), ch[k].v.end(), V.begin() + vo[k]);
    std::copy(ch[k].vt.begin(), ch[k].vt.end(), T.begin() + to[k]);
    std::copy(ch[k].vn.begin(), ch[k].vn.end(), N.begin() + no[k]);
  }
  // material in force at each chunk start (events are sequential)
  std::vector<uint32_t> start_mat(nt, 0);
  uint32_t cur = 0;
  auto apply = [&](const std::string &ev, uint32_t) -> uint32_t {
    if (ev.empty()) return 0;  // "g": back to the default material
    auto it = by_name.find(ev.substr(1));
    return it == by_name.end() ? 0u : it->second;
  };
  for (unsigned k = 0; k < nt; k++) {
    start_mat[k] = cur;
    for (const std::string &ev : ch[k].events) cur = apply(ev, cur);
  }
  // triangles: count, then fill per chunk (file order)
  std::vector<size_t> tri_off(nt + 1, 0);
  for (unsigned k = 0; k < nt; k++) {
    size_t t = 0;
    for (size_t f = 0; f + 1 < ch[k].fstart.size(); f++) t += ch[k].fstart[f + 1] - ch[k].fstart[f] - 2;
    tri_off[k + 1] = tri_off[k] + t;
  }
  const size_t ntri = tri_off[nt];
  if (ntri > 0xFFFFFFFFull) return OR3_ERR_INVALID_ARGUMENT;
  or3_mesh *m = (or3_mesh *)std::calloc(1, sizeof(or3_mesh));
  m->num_triangles = (uint32_t)ntri;
  m->vertices = (double *)std::malloc(std::max<size_t>(1, ntri) * 9 * sizeof(double));
  m->normals = (double *)std::malloc(std::max<size_t>(1, ntri) * 9 * sizeof(double));
  m->uvs = (double *)std::malloc(std::max<size_t>(1, ntri) * 6 * sizeof(double));
  m->material = (uint32_t *)std::malloc(std::max<size_t>(1, ntri) * sizeof(uint32_t));
  std::vector<int> bad(nt, 0);
  auto fill = [&](unsigned k) {
    const Chunk &c = ch[k];
    size_t t = tri_off[k];
    uint32_t mat = start_mat[k];
    uint32_t ev = 0;
    for (size_t f = 0; f + 1 < c.fstart.size(); f++) {
      while (ev < c.fevent[f]) mat = apply(c.events[ev++], mat);
      const uint32_t s = c.fstart[f], n = c.fstart[f + 1] - s;
      for (uint32_t i = 0; i + 2 < n; i++) {
        const uint32_t idx[3] = {s, s + i + 1, s + i + 2};
        V3d p[3], nn[3] = {}, uv[3] = {};
        bool has_n = false;
        for (int q = 0; q < 3; q++) {
          const FaceVert &fv = c.fv[idx[q]];
          if (fv.v < 0 || (size_t)fv.v >= V.size() || (fv.t >= 0 && (size_t)fv.t >= T.size()) ||
              (fv.n >= 0 && (size_t)fv.n >= N.size()) || fv.t < -1 || fv.n < -1) {
            bad[k] = 1;
            return;
          }
          p[q] = V[fv.v];
          if (fv.t >= 0) uv[q] = T[fv.t];
          if (fv.n >= 0) {
            nn[q] = N[fv.n];
            has_n = true;
          }
        }
        if (!has_n) {
          const V3d a{p[1].x - p[0].x, p[1].y - p[0].y, p[1].z - p[0].z};
          const V3d bb{p[2].x - p[0].x, p[2].y - p[0].y, p[2].z - p[0].z};
          V3d cn{a.y * bb.z - a.z * bb.y, a.z * bb.x - a.x * bb.z, a.x * bb.y - a.y * bb.x};
          const double l = std::sqrt(cn.x * cn.x + cn.y * cn.y + cn.z * cn.z);
          cn = {cn.x / l, cn.y / l, cn.z / l};
          nn[0] = nn[1] = nn[2] = cn;
        }
        for (int q = 0; q < 3; q++) {
          double *pv = m->vertices + 9 * t + 3 * q, *pn = m->normals + 9 * t + 3 * q, *pu = m->uvs + 6 * t + 2 * q;
          pv[0] = p[q].x; pv[1] = p[q].y; pv[2] = p[q].z;
          pn[0] = nn[q].x; pn[1] = nn[q].y; pn[2] = nn[q].z;
          pu[0] = uv[q].x; pu[1] = uv[q].y;
        }
        m->material[t] = mat;
        t++;
      }
    }
  };
  {
    std::vector<std::thread> pool;
    for (unsigned k = 1; k < nt; k++) pool.emplace_back(fill, k);
    fill(0);
    for (auto &th : pool) th.join();
  }
  m->num_materials = (uint32_t)mats.size();
  m->materials = (or3_material *)std::calloc(mats.size(), sizeof(or3_material));
  m->material_names = (char **)std::calloc(mats.size(), sizeof(char *));
  m->texture_paths = (char **)std::calloc(mats.size(), sizeof(char *));
  for (size_t i = 0; i < mats.size(); i++) {
    m->materials[i] = mats[i].m;
    m->material_names[i] = dup(mats[i].name);
    m->texture_paths[i] = mats[i].texture.empty() ? nullptr : dup(mats[i].texture);
  }
  for (unsigned k = 0; k < nt; k++)
    if (bad[k]) {
      or3_mesh_free(m);
      return OR3_ERR_INVALID_ARGUMENT;
    }
  *out = m;
  return OR3_OK;
}

// Model::Transform as SceneFromExternalFile::ReadMesh applies it
// (src/scenes/SceneFromExternalFile.cpp:518-527, src/renderer/Polygon.h:51-61):
// R = Rz(rz) Ry(ry) Rx(rx) (Matrix::RotateAroundVector, radians) on the first
// vertex and both edges, then the per-axis scale, then the translation; the
// normals are rotated only.
int or3_mesh_transform(or3_mesh *m, const double position[3], const double scaling[3], const double rotation[3]) {
  if (!m || !position || !scaling || !rotation) return OR3_ERR_INVALID_ARGUMENT;
  auto rot = [](int axis, double a, double R[3][3]) {
    const double c = std::cos(a), s = std::sin(a), omc = 1 - c;
    const double v[3] = {axis == 0 ? 1.0 : 0.0, axis == 1 ? 1.0 : 0.0, axis == 2 ? 1.0 : 0.0};
    R[0][0] = v[0] * v[0] * omc + c;    R[0][1] = v[0] * v[1] * omc - v[2] * s; R[0][2] = v[2] * v[0] * omc + v[1] * s;
    R[1][0] = v[0] * v[1] * omc + v[2] * s; R[1][1] = v[1] * v[1] * omc + c;    R[1][2] = v[2] * v[1] * omc - v[0] * s;
    R[2][0] = v[0] * v[2] * omc - v[1] * s; R[2][1] = v[2] * v[1] * omc + v[0] * s; R[2][2] = v[2] * v[2] * omc + c;
  };
  auto mul = [](const double A[3][3], const double B[3][3], double C[3][3]) {
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 3; c++) C[r][c] = A[r][0] * B[0][c] + A[r][1] * B[1][c] + A[r][2] * B[2][c];
  };
  double Rz[3][3], Ry[3][3], Rx[3][3], T[3][3], R[3][3];
  rot(2, rotation[2], Rz);
  rot(1, rotation[1], Ry);
  rot(0, rotation[0], Rx);
  mul(Rz, Ry, T);
  mul(T, Rx, R);
  auto apply = [&](const double *v, double *o) {
    o[0] = R[0][0] * v[0] + R[0][1] * v[1] + R[0][2] * v[2];
    o[1] = R[1][0] * v[0] + R[1][1] * v[1] + R[1][2] * v[2];
    o[2] = R[2][0] * v[0] + R[2][1] * v[1] + R[2][2] * v[2];
  };
  for (uint32_t t = 0; t < m->num_triangles; t++) {
    double *p = m->vertices + 9 * (size_t)t, *n = m->normals + 9 * (size_t)t;
    // the reference keeps (p0, p1 - p0, p2 - p0) and transforms each
    double pe[3][3], ne[3][3];
    for (int a = 0; a < 3; a++) {
      pe[0][a] = p[a];
      pe[1][a] = p[3 + a] - p[a];
      pe[2][a] = p[6 + a] - p[a];
      ne[0][a] = n[a];
      ne[1][a] = n[3 + a] - n[a];
      ne[2][a] = n[6 + a] - n[a];
    }
    double q[3][3], r[3][3];
    for (int k = 0; k < 3; k++) {
      apply(pe[k], q[k]);
      for (int a = 0; a < 3; a++) q[k][a] *= scaling[a];
      apply(ne[k], r[k]);
    }
    for (int a = 0; a < 3; a++) {
      const double v0 = q[0][a] + position[a];
      p[a] = v0;
      p[3 + a] = v0 + q[1][a];
      p[6 + a] = v0 + q[2][a];
      n[a] = r[0][a];
      n[3 + a] = r[0][a] + r[1][a];
      n[6 + a] = r[0][a] + r[2][a];
    }
  }
  return OR3_OK;
}

}  // extern "C"
