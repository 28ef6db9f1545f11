// scene_file.cpp -- the reference's text scene files straight to an
// or3_scene_desc (or3_scene_load_file), without its per-object heap records.
//
// Reads what SceneFromExternalFile::ReadFromFile reads
// (src/scenes/SceneFromExternalFile.cpp:66-182), with its rules:
//   * header lines "Key: Value" up to a line "Objects:" (after left trimming);
//     the keys are "Base Dir" / "BaseDir" (a '/' is appended), "IBL" (the
//     base directory as it stands then, plus the name) and "Space
//     Partitioning"; any other key fails (ReadHeader, :184-212);
//   * blank lines and lines starting with '#' are skipped; a line containing
//     '{' opens an object whose type is the line with "{" and then blanks
//     trimmed from its right: "Obj Mesh", "Sphere", "SphereLight", "Floor" or
//     "InfiniteFloor"; a line starting with '}' closes it; inside, "Key: Value"
//     (a line is cut at ':' and only the first two fields count);
//   * Material: "er, eg, eb, TYPE, r, g, b[, ior][, texture]" with TYPE
//     LAMBERT, SPECULAR or REFRACTION (the IOR only and always for
//     REFRACTION) and an optional texture file under the base directory
//     (ParseMaterial, :214-269);
//   * several Material lines make layers with "MaterialRates" normalised to
//     sum 1; one material is one layer of rate 1; a count mismatch fails
//     (ProcessMaterials, :274-293), except for an InfiniteFloor, which then
//     keeps its first material alone (:426-432);
//   * Sphere / SphereLight: Radius, Position (exactly 3 numbers); Floor: Size
//     (exactly 2), Position, Type XZ_yUp (default), XZ_yDown, XY_zUp,
//     XY_zDown, YZ_xUp, YZ_xDown as two triangles with the vertices, uvs and
//     normals of Scene::AddFloor* (src/scenes/Scene.cpp:88-195) offset by the
//     position; InfiniteFloor: Y; Obj Mesh: FileName under the base
//     directory, Position, Scaling (default 1, 1, 1), Rotation, each
//     component optionally "<number> deg" (parseVector3, :15-43), loaded with
//     or3_mesh_load_obj and placed with or3_mesh_transform (ReadMesh,
//     :489-529);
//   * the IBL is read with or3_read_hdr into the descriptor's RGBE bytes.
// Differences, on purpose: every sphere and triangle goes into the BVH
// ("Space Partitioning: False" objects are tested after the BVH by the
// reference, which differs only for hits at exactly equal distance); an
// object without a Material fails instead of reading past an empty list;
// textures are returned as paths (the loader does not decode images); object
// ids follow the file, a mesh's triangles in file order.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <utility>
#include <vector>

#include "or3.h"

namespace {

constexpr double kPiD = 3.14159265358979323846;

std::vector<std::string> split(const std::string &s, char d) {  // Utils::split: no field after a trailing delimiter
  std::vector<std::string> r;
  size_t i = 0;
  while (i < s.size()) {
    const size_t p = s.find(d, i);
    if (p == std::string::npos) {
      r.push_back(s.substr(i));
      break;
    }
    r.push_back(s.substr(i, p - i));
    i = p + 1;
  }
  return r;
}
std::string ltrim(const std::string &s, const char *ws = " \t") {
  const size_t i = s.find_first_not_of(ws);
  return i == std::string::npos ? std::string() : s.substr(i);
}
std::string rtrim(const std::string &s, const char *ws = " \t") {
  const size_t i = s.find_last_not_of(ws);
  return i == std::string::npos ? std::string() : s.substr(0, i + 1);
}
std::string trim(const std::string &s) { return ltrim(rtrim(s)); }
double num(const std::string &s) { return std::atof(s.c_str()); }

using Lines = std::vector<std::pair<std::string, std::string>>;

void add_line(Lines &out, const std::string &line) {
  const std::vector<std::string> f = split(line, ':');
  if (f.size() == 1) out.emplace_back(trim(f[0]), "");
  else if (f.size() >= 2) out.emplace_back(trim(f[0]), trim(f[1]));
}

// "x[ deg], y[ deg], z[ deg]"; missing components are 0
void vec3_deg(const std::string &s, double v[3]) {
  const std::vector<std::string> c = split(s, ',');
  for (int a = 0; a < 3; a++) {
    v[a] = 0.0;
    if ((size_t)a >= c.size()) continue;
    const std::vector<std::string> t = split(trim(c[a]), ' ');
    if (t.empty()) continue;
    v[a] = num(trim(t[0]));
    if (t.size() >= 2 && t[1] == "deg") v[a] = v[a] * kPiD / 180;
  }
}

bool vec_n(const std::string &s, int n, double *v) {  // exactly n comma-separated numbers
  const std::vector<std::string> c = split(s, ',');
  if ((int)c.size() != n) return false;
  for (int a = 0; a < n; a++) v[a] = num(trim(c[a]));
  return true;
}

struct Mat {
  or3_material m;
  std::string texture;  // full path, or empty
};

struct Builder {
  std::string base, ibl, partitioning, err;
  std::vector<or3_material> mats;
  std::vector<std::string> tex;
  std::vector<uint32_t> layer_mat;
  std::vector<double> layer_rate;
  std::vector<double> tv, tn, tuv;       // triangles: 9, 9, 6 doubles
  std::vector<uint32_t> tl, tid;         // layers (first, count), object id
  std::vector<double> sph;               // x, y, z, r
  std::vector<uint32_t> sl, sflag, sid;
  std::vector<double> pl;                // kind, axis, offset, flip
  std::vector<uint32_t> pll, pid;
  uint32_t next_id = 0;
  uint32_t meshes = 0;
  uint32_t threads = 0;

  bool fail(const char *fmt, ...) {
    char b[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(b, sizeof(b), fmt, ap);
    va_end(ap);
    err = b;
    return false;
  }

  bool material(const std::string &text, Mat &out) {
    const std::vector<std::string> d = split(text, ',');
    if (d.size() < 7) return fail("insufficient material definition: %s", text.c_str());
    std::memset(&out.m, 0, sizeof(out.m));
    out.m.texture = -1;
    for (int a = 0; a < 3; a++) out.m.emission[a] = num(trim(d[a]));
    const std::string t = trim(d[3]);
    if (t == "LAMBERT") out.m.type = OR3_LAMBERT;
    else if (t == "SPECULAR") out.m.type = OR3_SPECULAR;
    else if (t == "REFRACTION") out.m.type = OR3_REFRACTION;
    else return fail("undefined reflection type: %s", t.c_str());
    for (int a = 0; a < 3; a++) out.m.color[a] = num(trim(d[4 + a]));
    const bool refr = out.m.type == OR3_REFRACTION;
    if (refr) {
      if (d.size() < 8) return fail("reflectance is not defined: %s", text.c_str());
      out.m.ior = num(trim(d[7]));
    }
    const size_t ti = refr ? 8 : 7;
    if (d.size() > ti) out.texture = base + trim(d[ti]);
    return true;
  }

  // layers of one object; false on a rate count mismatch
  bool layers(const std::vector<Mat> &ms, std::vector<double> rates, uint32_t lay[2]) {
    if (ms.size() == 1) rates.assign(1, 1.0);
    if (ms.size() != rates.size()) return false;
    double total = 0;
    if (ms.size() > 1)
      for (double r : rates) total += r;
    lay[0] = (uint32_t)layer_mat.size();
    lay[1] = (uint32_t)ms.size();
    for (size_t i = 0; i < ms.size(); i++) {
      layer_mat.push_back((uint32_t)mats.size());
      layer_rate.push_back(ms.size() > 1 ? rates[i] / total : rates[i]);
      mats.push_back(ms[i].m);
      tex.push_back(ms[i].texture);
    }
    return true;
  }

  bool object_materials(const Lines &lines, std::vector<Mat> &ms, std::vector<double> &rates) {
    for (const auto &kv : lines) {
      if (kv.first == "Material") {
        Mat m;
        if (!material(kv.second, m)) return false;
        ms.push_back(m);
      } else if (kv.first == "MaterialRates") {
        for (const std::string &r : split(kv.second, ',')) rates.push_back(num(r));
      }
    }
    if (ms.empty()) return fail("object without a Material");
    return true;
  }

  void triangle(const double v[3][3], const double uv[3][2], const double n[3][3], const uint32_t lay[2]) {
    for (int k = 0; k < 3; k++)
      for (int a = 0; a < 3; a++) {
        tv.push_back(v[k][a]);
        tn.push_back(n[k][a]);
      }
    for (int k = 0; k < 3; k++)
      for (int a = 0; a < 2; a++) tuv.push_back(uv[k][a]);
    tl.push_back(lay[0]);
    tl.push_back(lay[1]);
    tid.push_back(next_id++);
  }

  bool sphere(const Lines &lines, bool light) {
    double radius = 0, pos[3] = {0, 0, 0};
    for (const auto &kv : lines) {
      if (kv.first == "Radius") radius = num(kv.second);
      else if (kv.first == "Position" && !vec_n(kv.second, 3, pos)) return fail("Position needs 3 numbers");
    }
    std::vector<Mat> ms;
    std::vector<double> rates;
    if (!object_materials(lines, ms, rates)) return false;
    uint32_t lay[2];
    if (!layers(ms, rates, lay)) return fail("MaterialRates do not match the materials");
    sph.insert(sph.end(), {pos[0], pos[1], pos[2], radius});
    sl.insert(sl.end(), {lay[0], lay[1]});
    sflag.push_back(light ? OR3_SPHERE_LIGHT : 0u);
    sid.push_back(next_id++);
    return true;
  }

  bool floor(const Lines &lines) {
    double size[2] = {0, 0}, pos[3] = {0, 0, 0};
    std::string type = "XZ_yUp";
    for (const auto &kv : lines) {
      if (kv.first == "Size" && !vec_n(kv.second, 2, size)) return fail("Size needs 2 numbers");
      if (kv.first == "Position" && !vec_n(kv.second, 3, pos)) return fail("Position needs 3 numbers");
      if (kv.first == "Type" && (kv.second == "XZ_yUp" || kv.second == "XZ_yDown" || kv.second == "XY_zUp" ||
                                 kv.second == "XY_zDown" || kv.second == "YZ_xUp" || kv.second == "YZ_xDown"))
        type = kv.second;
    }
    std::vector<Mat> ms;
    std::vector<double> rates;
    if (!object_materials(lines, ms, rates)) return false;
    const double a = size[0] / 2, b = size[1] / 2;
    // Scene::AddFloor*: vertices, uvs, normal of each of the two triangles
    struct Tri {
      double v[3][3], uv[3][2];
    } t[2];
    double n[3] = {0, 0, 0};
    auto set = [](Tri &tr, std::initializer_list<double> v, std::initializer_list<double> uv) {
      auto it = v.begin();
      for (int k = 0; k < 3; k++)
        for (int c = 0; c < 3; c++) tr.v[k][c] = *it++;
      auto iu = uv.begin();
      for (int k = 0; k < 3; k++)
        for (int c = 0; c < 2; c++) tr.uv[k][c] = *iu++;
    };
    if (type == "XZ_yUp") {
      set(t[0], {-a, 0, -b, -a, 0, b, a, 0, -b}, {0, 0, 0, 1, 1, 0});
      set(t[1], {a, 0, -b, -a, 0, b, a, 0, b}, {1, 0, 0, 1, 1, 1});
      n[1] = 1;
    } else if (type == "XY_zUp") {
      set(t[0], {-a, b, 0, -a, -b, 0, a, -b, 0}, {0, 0, 0, 1, 1, 1});
      set(t[1], {a, b, 0, -a, b, 0, a, -b, 0}, {1, 0, 0, 0, 1, 1});
      n[2] = 1;
    } else if (type == "YZ_xUp") {
      set(t[0], {0, a, -b, 0, a, b, 0, -a, b}, {1, 0, 0, 0, 0, 1});
      set(t[1], {0, -a, -b, 0, a, -b, 0, -a, b}, {1, 1, 1, 0, 0, 1});
      n[0] = 1;
    } else if (type == "XZ_yDown") {
      set(t[0], {a, 0, -b, -a, 0, b, -a, 0, -b}, {1, 1, 0, 0, 0, 1});
      set(t[1], {a, 0, b, -a, 0, b, a, 0, -b}, {1, 0, 0, 0, 1, 1});
      n[1] = -1;
    } else if (type == "XY_zDown") {
      set(t[0], {a, -b, 0, -a, -b, 0, -a, b, 0}, {0, 1, 1, 1, 1, 0});
      set(t[1], {a, -b, 0, -a, b, 0, a, b, 0}, {0, 1, 1, 0, 0, 0});
      n[2] = -1;
    } else {  // YZ_xDown
      set(t[0], {0, -a, b, 0, a, b, 0, a, -b}, {1, 1, 1, 0, 0, 0});
      set(t[1], {0, -a, b, 0, a, -b, 0, -a, -b}, {1, 1, 0, 0, 0, 1});
      n[0] = -1;
    }
    for (Tri &tr : t) {
      uint32_t lay[2];
      if (!layers(ms, rates, lay)) return fail("MaterialRates do not match the materials");
      double v[3][3], nn[3][3];
      for (int k = 0; k < 3; k++)
        for (int c = 0; c < 3; c++) {
          v[k][c] = tr.v[k][c] + pos[c];
          nn[k][c] = n[c];
        }
      triangle(v, tr.uv, nn, lay);
    }
    return true;
  }

  bool infinite_floor(const Lines &lines) {
    double y = 0;
    for (const auto &kv : lines)
      if (kv.first == "Y") y = num(kv.second);
    std::vector<Mat> ms;
    std::vector<double> rates;
    if (!object_materials(lines, ms, rates)) return false;
    uint32_t lay[2];
    if (!layers(ms, rates, lay)) {  // the reference ignores the failure: the first material alone
      std::vector<Mat> first(1, ms[0]);
      layers(first, {}, lay);
    }
    pl.insert(pl.end(), {(double)OR3_PLANE_INFINITE_FLOOR, 1.0, y, 0.0});
    pll.insert(pll.end(), {lay[0], lay[1]});
    pid.push_back(next_id++);
    return true;
  }

  bool mesh(const Lines &lines) {
    std::string file;
    double pos[3] = {0, 0, 0}, scale[3] = {1, 1, 1}, rot[3] = {0, 0, 0};
    for (const auto &kv : lines) {
      if (kv.first == "FileName") file = base + kv.second;
      else if (kv.first == "Position") vec3_deg(kv.second, pos);
      else if (kv.first == "Scaling") vec3_deg(kv.second, scale);
      else if (kv.first == "Rotation") vec3_deg(kv.second, rot);
    }
    or3_mesh *m = nullptr;
    const int rc = or3_mesh_load_obj(file.c_str(), 0, threads, &m);
    if (rc != OR3_OK) return fail("cannot read the mesh %s (status %d)", file.c_str(), rc);
    or3_mesh_transform(m, pos, scale, rot);
    // one single-layer material per .mtl material
    const uint32_t lay0 = (uint32_t)layer_mat.size();
    for (uint32_t i = 0; i < m->num_materials; i++) {
      layer_mat.push_back((uint32_t)mats.size());
      layer_rate.push_back(1.0);
      mats.push_back(m->materials[i]);
      tex.push_back(m->texture_paths[i] ? m->texture_paths[i] : "");
    }
    const size_t nt = m->num_triangles;  // whole arrays appended: the mesh is most of a large scene
    tv.insert(tv.end(), m->vertices, m->vertices + 9 * nt);
    tn.insert(tn.end(), m->normals, m->normals + 9 * nt);
    tuv.insert(tuv.end(), m->uvs, m->uvs + 6 * nt);
    const size_t l0 = tl.size(), i0 = tid.size();
    tl.resize(l0 + 2 * nt);
    tid.resize(i0 + nt);
    for (size_t t = 0; t < nt; t++) {
      tl[l0 + 2 * t] = lay0 + m->material[t];
      tl[l0 + 2 * t + 1] = 1;
      tid[i0 + t] = next_id++;
    }
    or3_mesh_free(m);
    meshes++;
    return true;
  }

  bool header(const Lines &lines) {
    for (const auto &kv : lines) {
      if (kv.first == "Base Dir" || kv.first == "BaseDir") {
        base = kv.second;
        if (!base.empty() && base.back() != '/') base.push_back('/');
      } else if (kv.first == "IBL") {
        ibl = base + kv.second;
      } else if (kv.first == "Space Partitioning") {
        partitioning = kv.second;
      } else {
        return fail("undefined header information: %s", kv.first.c_str());
      }
    }
    return true;
  }

  bool read(const char *path) {
    std::ifstream in(path);
    if (!in || in.bad() || in.eof()) return fail("cannot open %s", path);
    Lines lines;
    int number = 1;
    std::string line;
    do {  // header, up to "Objects:"
      std::getline(in, line);
      line = ltrim(line);
      if (line == "Objects:") break;
      if (!line.empty() && line.find('#') != 0) add_line(lines, line);
      number++;
    } while (!in.eof());
    if (in.eof()) return fail("no \"Objects:\" line (or nothing after it)");
    if (!header(lines)) return false;
    enum Kind { NONE, MESH, SPHERE, LIGHT, FLOOR, INF_FLOOR } kind = NONE;
    bool open = false;
    lines.clear();
    do {
      std::getline(in, line);
      line = ltrim(line);
      if (line.empty() || line[0] == '#') {
        number++;
        if (in.eof()) break;
        continue;
      }
      if (line.find('{') != std::string::npos) {
        if (open) return fail("nested object definition: line %d", number);
        const std::string t = rtrim(rtrim(line, "{"));
        kind = t == "Obj Mesh" ? MESH : t == "Sphere" ? SPHERE : t == "Floor" ? FLOOR
             : t == "SphereLight" ? LIGHT : t == "InfiniteFloor" ? INF_FLOOR : NONE;
        if (kind == NONE) return fail("undefined object type: %s line %d", t.c_str(), number);
        open = true;
      } else if (line.find('}') == 0) {
        if (!open) return fail("inconsistent delimiter: line %d", number);
        bool ok = false;
        switch (kind) {
          case MESH: ok = mesh(lines); break;
          case FLOOR: ok = floor(lines); break;
          case SPHERE: ok = sphere(lines, false); break;
          case LIGHT: ok = sphere(lines, true); break;
          case INF_FLOOR: ok = infinite_floor(lines); break;
          default: break;
        }
        if (!ok) return fail("failed to load object ending at line %d: %s", number, err.c_str());
        kind = NONE;
        open = false;
        lines.clear();
      } else if (open) {
        add_line(lines, line);
      }
      number++;
    } while (!in.eof());
    return true;
  }
};

// The loaded file: the public struct first, the arrays it points into after.
struct SceneFileOwned {
  or3_scene_file pub;
  Builder b;
  std::vector<uint8_t> rgbe;
  std::vector<char *> tex_ptrs;
  std::string ibl_path;
};

}  // namespace

extern "C" {

int or3_scene_load_file(const char *path, uint32_t threads, or3_scene_file **out, char *err, size_t err_len) {
  auto report = [&](int rc, const std::string &msg) {
    if (err && err_len) std::snprintf(err, err_len, "%s", msg.c_str());
    return rc;
  };
  if (!path || !out) return report(OR3_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  {
    std::ifstream probe(path);
    if (!probe) return report(OR3_ERR_NOT_FOUND, std::string("cannot open ") + path);
  }
  SceneFileOwned *f = new SceneFileOwned();
  Builder &b = f->b;
  b.threads = threads;
  if (!b.read(path)) {
    const int rc = b.err.find("cannot read the mesh") != std::string::npos ? OR3_ERR_NOT_FOUND : OR3_ERR_INVALID_ARGUMENT;
    const std::string msg = b.err;
    delete f;
    return report(rc, msg);
  }
  if (!b.ibl.empty()) {  // the environment: RGBE bytes of the .hdr
    std::ifstream h(b.ibl, std::ios::binary);
    if (!h) {
      const std::string msg = "cannot open the IBL " + b.ibl;
      delete f;
      return report(OR3_ERR_NOT_FOUND, msg);
    }
    const std::vector<uint8_t> bytes((std::istreambuf_iterator<char>(h)), std::istreambuf_iterator<char>());
    uint32_t w = 0, hh = 0;
    int rc = or3_read_hdr(bytes.data(), bytes.size(), &w, &hh, nullptr, 0);
    if (rc == OR3_OK) {
      f->rgbe.resize(4 * (size_t)w * hh);
      rc = or3_read_hdr(bytes.data(), bytes.size(), &w, &hh, f->rgbe.data(), f->rgbe.size());
    }
    if (rc != OR3_OK) {
      const std::string msg = "cannot read the IBL " + b.ibl;
      delete f;
      return report(rc, msg);
    }
    f->pub.desc.env_rgbe = f->rgbe.data();
    f->pub.desc.env_width = w;
    f->pub.desc.env_height = hh;
    f->ibl_path = b.ibl;
  }
  or3_scene_desc &d = f->pub.desc;
  d.num_materials = (uint32_t)b.mats.size();
  d.materials = b.mats.data();
  d.num_layers = (uint32_t)b.layer_mat.size();
  d.layer_material = b.layer_mat.data();
  d.layer_rate = b.layer_rate.data();
  d.num_triangles = (uint32_t)b.tid.size();
  if (d.num_triangles) {
    d.tri_vertices = b.tv.data();
    d.tri_normals = b.tn.data();
    d.tri_uvs = b.tuv.data();
    d.tri_layers = b.tl.data();
    d.tri_ids = b.tid.data();
  }
  d.num_spheres = (uint32_t)b.sid.size();
  if (d.num_spheres) {
    d.spheres = b.sph.data();
    d.sphere_layers = b.sl.data();
    d.sphere_flags = b.sflag.data();
    d.sphere_ids = b.sid.data();
  }
  d.num_planes = (uint32_t)b.pid.size();
  if (d.num_planes) {
    d.planes = b.pl.data();
    d.plane_layers = b.pll.data();
    d.plane_ids = b.pid.data();
  }
  f->tex_ptrs.resize(b.tex.size());
  for (size_t i = 0; i < b.tex.size(); i++) f->tex_ptrs[i] = b.tex[i].empty() ? nullptr : &b.tex[i][0];
  f->pub.texture_paths = f->tex_ptrs.empty() ? nullptr : f->tex_ptrs.data();
  f->pub.ibl_path = f->ibl_path.empty() ? nullptr : &f->ibl_path[0];
  std::snprintf(f->pub.space_partitioning, sizeof(f->pub.space_partitioning), "%s", b.partitioning.c_str());
  f->pub.num_meshes = b.meshes;
  *out = &f->pub;
  return OR3_OK;
}

void or3_scene_file_free(or3_scene_file *f) {
  delete reinterpret_cast<SceneFileOwned *>(f);  // pub is the first member
}

}  // extern "C"
