// reference_flatten.hpp -- a reference Scene and Camera as the C ABI's
// or3_scene_desc / or3_camera.
//
// Include it after the reference's headers (Scene.h, Polygon.h, Sphere.h,
// SphereLight.h, AxisAlignedPlane.h, InfiniteFloor.h, IBL.h, Camera.h,
// ImageHandler.h) have been included with `private` and `protected`
// redefined to `public`: the reference keeps Scene's object lists protected
// and Polygon's geometry private (src/scenes/Scene.h:110-118,
// src/renderer/Polygon.h:108-111) and has no accessor for them.  Used by the
// drop-in adapter (reference_adapter.cpp) and by the test that compares its
// output with the native scene-file reader.
#pragma once

#include <cstdint>
#include <iostream>
#include <map>
#include <vector>

#include "or3.h"

namespace OmochiRenderer {

// Owning flattened copy of a reference Scene (arrays behind an or3_scene_desc).
struct FlatScene {
  std::vector<or3_material> materials;
  std::vector<uint32_t> layer_material;
  std::vector<double> layer_rate;
  std::vector<double> tri_vertices, tri_normals, tri_uvs, spheres, planes;
  std::vector<uint32_t> tri_layers, tri_ids, sphere_layers, sphere_flags, sphere_ids, plane_layers, plane_ids;
  std::vector<float> env;
  uint32_t env_w = 0, env_h = 0;
  std::vector<uint32_t> tex_dims;
  std::vector<uint64_t> tex_offsets;
  std::vector<float> texels;
  std::map<int, int> tex_index;  // ImageHandler id -> texture index
  double background[3] = {0, 0, 0};

  int texture_of(int image_id) {
    if (image_id == ImageHandler::INVALID_IMAGE_ID) return -1;
    auto it = tex_index.find(image_id);
    if (it != tex_index.end()) return it->second;
    const Image *img = ImageHandler::GetInstance().GetImage(image_id);
    if (!img) return -1;
    const int idx = (int)tex_dims.size() / 2;
    tex_dims.push_back((uint32_t)img->GetWidth());
    tex_dims.push_back((uint32_t)img->GetHeight());
    tex_offsets.push_back(texels.size());
    for (const Color &c : img->m_image) {
      texels.push_back((float)c.x);
      texels.push_back((float)c.y);
      texels.push_back((float)c.z);
    }
    tex_index[image_id] = idx;
    return idx;
  }

  void layers_of(const SceneObject *o, std::vector<uint32_t> &out) {
    out.push_back((uint32_t)layer_material.size());
    out.push_back((uint32_t)o->materials_.size());
    for (const auto &l : o->materials_) {
      const Material &m = l.material_;
      or3_material om{};
      om.type = m.reflection_type == Material::REFLECTION_TYPE_SPECULAR     ? OR3_SPECULAR
                : m.reflection_type == Material::REFLECTION_TYPE_REFRACTION ? OR3_REFRACTION
                                                                            : OR3_LAMBERT;
      om.texture = texture_of(m.texture_id);
      om.emission[0] = m.emission.x; om.emission[1] = m.emission.y; om.emission[2] = m.emission.z;
      om.color[0] = m.color.x; om.color[1] = m.color.y; om.color[2] = m.color.z;
      om.ior = m.refraction_rate;
      layer_material.push_back((uint32_t)materials.size());
      layer_rate.push_back(l.rate_);
      materials.push_back(om);
    }
  }

  static void push3(std::vector<double> &v, const Vector3 &a) {
    v.push_back(a.x); v.push_back(a.y); v.push_back(a.z);
  }

  explicit FlatScene(const Scene &scene) {
    const Color bg = scene.Background();
    background[0] = bg.x; background[1] = bg.y; background[2] = bg.z;
    uint32_t id = 0;
    for (const auto &info : scene.m_objects) {  // AddObject order = object id
      const SceneObject *o = info.object;
      if (const Polygon *p = dynamic_cast<const Polygon *>(o)) {
        const Vector3 p0 = p->m_posAndEdges[0] + p->position_;
        push3(tri_vertices, p0);
        push3(tri_vertices, p0 + p->m_posAndEdges[1]);
        push3(tri_vertices, p0 + p->m_posAndEdges[2]);
        const Vector3 &n0 = p->m_normalAndDiffs[0];
        push3(tri_normals, n0);
        push3(tri_normals, n0 + p->m_normalAndDiffs[1]);
        push3(tri_normals, n0 + p->m_normalAndDiffs[2]);
        const Vector3 &u0 = p->m_uvOrigAndEdges[0];
        const Vector3 u1 = u0 + p->m_uvOrigAndEdges[1], u2 = u0 + p->m_uvOrigAndEdges[2];
        const double uv[6] = {u0.x, u0.y, u1.x, u1.y, u2.x, u2.y};
        tri_uvs.insert(tri_uvs.end(), uv, uv + 6);
        layers_of(o, tri_layers);
        tri_ids.push_back(id);
      } else if (const Sphere *s = dynamic_cast<const Sphere *>(o)) {
        push3(spheres, s->position_);
        spheres.push_back(s->m_radius);
        layers_of(o, sphere_layers);
        sphere_flags.push_back(dynamic_cast<const SphereLight *>(o) ? OR3_SPHERE_LIGHT : 0u);
        sphere_ids.push_back(id);
      } else if (const AxisAlignedPlane *a = dynamic_cast<const AxisAlignedPlane *>(o)) {
        const int axis = a->m_axis == AxisAlignedPlane::PLANE_XY ? 0 : a->m_axis == AxisAlignedPlane::PLANE_XZ ? 1 : 2;
        const double n = axis == 0 ? a->m_normal.z : axis == 1 ? a->m_normal.y : a->m_normal.x;
        planes.push_back(OR3_PLANE_AXIS_ALIGNED);
        planes.push_back(axis);
        planes.push_back(a->m_offset);
        planes.push_back(n < 0 ? 1.0 : 0.0);
        layers_of(o, plane_layers);
        plane_ids.push_back(id);
      } else if (const InfiniteFloor *f = dynamic_cast<const InfiniteFloor *>(o)) {
        planes.push_back(OR3_PLANE_INFINITE_FLOOR);
        planes.push_back(1);
        planes.push_back(f->y);
        planes.push_back(0);
        layers_of(o, plane_layers);
        plane_ids.push_back(id);
      } else {
        std::cerr << "GpuPathTracerAdapter: object " << id << " has a type the GPU path does not know" << std::endl;
      }
      id++;
    }
    if (const IBL *ibl = scene.GetIBL()) {
      env_w = (uint32_t)ibl->m_image.GetWidth();
      env_h = (uint32_t)ibl->m_image.GetHeight();
      for (const Color &c : ibl->m_image.m_image) {
        env.push_back((float)c.x);
        env.push_back((float)c.y);
        env.push_back((float)c.z);
      }
    }
  }

  or3_scene_desc desc() const {
    or3_scene_desc d{};
    d.num_materials = (uint32_t)materials.size();
    d.materials = materials.data();
    d.num_layers = (uint32_t)layer_material.size();
    d.layer_material = layer_material.data();
    d.layer_rate = layer_rate.data();
    d.num_triangles = (uint32_t)tri_ids.size();
    d.tri_vertices = tri_vertices.data();
    d.tri_normals = tri_normals.data();
    d.tri_uvs = tri_uvs.data();
    d.tri_layers = tri_layers.data();
    d.tri_ids = tri_ids.data();
    d.num_spheres = (uint32_t)sphere_ids.size();
    d.spheres = spheres.data();
    d.sphere_layers = sphere_layers.data();
    d.sphere_flags = sphere_flags.data();
    d.sphere_ids = sphere_ids.data();
    d.num_planes = (uint32_t)plane_ids.size();
    d.planes = planes.data();
    d.plane_layers = plane_layers.data();
    d.plane_ids = plane_ids.data();
    d.env_width = env_w;
    d.env_height = env_h;
    d.env_rgb = env.empty() ? nullptr : env.data();
    for (int k = 0; k < 3; k++) d.background[k] = background[k];
    d.num_textures = (uint32_t)tex_offsets.size();
    d.texture_dims = tex_dims.data();
    d.texture_offsets = tex_offsets.data();
    d.texture_rgb = texels.data();
    return d;
  }
};

static or3_camera to_or3(const Camera &c) {
  or3_camera o{};
  o.width = (uint32_t)c.m_width;
  o.height = (uint32_t)c.m_height;
  const Vector3 *v[3] = {&c.m_camPos, &c.m_camDir, &c.m_camUp};
  double *dst[3] = {o.position, o.direction, o.up};
  for (int i = 0; i < 3; i++) {
    dst[i][0] = v[i]->x; dst[i][1] = v[i]->y; dst[i][2] = v[i]->z;
  }
  o.screen_height_world = c.m_nearScreenHeight;
  o.distance_to_screen = c.m_distToScreen;
  o.focal_distance = c.m_focalDistance;
  const CircleAperture *ap = dynamic_cast<const CircleAperture *>(c.m_aperture.get());
  o.aperture_radius = ap ? ap->m_radius : 0.0;
  return o;
}

}  // namespace OmochiRenderer
