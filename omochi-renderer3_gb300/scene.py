"""Flattened scene description (or3_scene_desc) and camera (or3_camera).

A `SceneDesc` is what the reference's Scene holds after its factories have
run (src/scenes/Scene.h:110-118): an ordered list of objects, each with a list
of material layers.  Object ids are insertion order, as Scene::AddObject
assigns them, so closest-hit ids compare one-to-one with the reference.
"""
import ctypes
import math
from dataclasses import dataclass, field

import numpy as np

from . import abi


def _cat(blocks):
    """One contiguous array of the blocks; a single contiguous block is passed through uncopied."""
    if len(blocks) == 1:
        return np.ascontiguousarray(blocks[0])
    return np.ascontiguousarray(np.concatenate(blocks))


def _ptr(a, ctype):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctype))


@dataclass
class Camera:
    """or3_camera; defaults are the reference Camera's (src/renderer/Camera.h:12-20)."""
    width: int
    height: int
    position: tuple = (50.0, 52.0, 220.0)
    direction: tuple = (0.0, -0.04, -1.0)
    up: tuple = (0.0, 1.0, 0.0)
    screen_height_world: float = 30.0
    distance_to_screen: float = 40.0
    focal_distance: float = 200.0
    aperture_radius: float = 0.0

    def to_c(self):
        c = abi.CameraC()
        c.width, c.height = int(self.width), int(self.height)
        c.position = abi.c_double3(*self.position)
        c.direction = abi.c_double3(*self.direction)
        c.up = abi.c_double3(*self.up)
        c.screen_height_world = self.screen_height_world
        c.distance_to_screen = self.distance_to_screen
        c.focal_distance = self.focal_distance
        c.aperture_radius = self.aperture_radius
        return c

    @staticmethod
    def from_fov(width, height, position, target, fov_y_deg, up=(0.0, 1.0, 0.0), distance=40.0):
        d = np.asarray(target, float) - np.asarray(position, float)
        return Camera(width, height, tuple(position), tuple(d / np.linalg.norm(d)), tuple(up),
                      2.0 * distance * math.tan(math.radians(fov_y_deg) / 2.0), distance)


@dataclass
class SceneDesc:
    materials: list = field(default_factory=list)
    layer_material: list = field(default_factory=list)
    layer_rate: list = field(default_factory=list)
    _layer_sets: dict = field(default_factory=dict)
    _next_id: int = 0
    tris: list = field(default_factory=list)      # (verts (n,3,3), normals or None, uvs or None, layers (n,2), ids)
    spheres: list = field(default_factory=list)   # (cx,cy,cz,r, layer_begin, layer_count, flags, id)
    planes: list = field(default_factory=list)    # (kind, axis, offset, flip, layer_begin, layer_count, id)
    env: np.ndarray = None
    env_rgbe: np.ndarray = None  # (H, W, 4) uint8, decoded on the device (alternative to env)
    background: tuple = (0.0, 0.0, 0.0)
    textures: list = field(default_factory=list)
    build: int = 0  # abi.OR3_BUILD_*
    leaf_max: int = 0          # BVH leaf size bound (0 = 4)
    traversal_cost: float = 0.0  # SAH node cost (0 = 1)

    # ---- materials
    def material(self, mtype=abi.OR3_LAMBERT, color=(0, 0, 0), emission=(0, 0, 0), ior=0.0,
                 phong_exponent=0.0, texture=-1):
        self.materials.append((int(mtype), int(texture), tuple(map(float, emission)),
                               tuple(map(float, color)), float(ior), float(phong_exponent)))
        return len(self.materials) - 1

    def layers(self, spec):
        """spec: material index, or list of (material, rate). Returns (begin, count)."""
        if isinstance(spec, (int, np.integer)):
            spec = [(int(spec), 1.0)]
        key = tuple((int(m), float(r)) for m, r in spec)
        if key not in self._layer_sets:
            self._layer_sets[key] = (len(self.layer_material), len(key))
            for m, r in key:
                self.layer_material.append(m)
                self.layer_rate.append(r)
        return self._layer_sets[key]

    def _ids(self, n):
        ids = np.arange(self._next_id, self._next_id + n, dtype=np.uint32)
        self._next_id += n
        return ids

    # ---- objects (insertion order = object id)
    def add_triangles(self, verts, layers, normals=None, uvs=None):
        verts = np.ascontiguousarray(verts, dtype=np.float64).reshape(-1, 3, 3)
        n = verts.shape[0]
        lay = np.asarray(layers, dtype=np.uint32)
        if lay.ndim == 1:
            lay = np.broadcast_to(lay, (n, 2))
        self.tris.append((verts,
                          None if normals is None else np.asarray(normals, np.float64).reshape(n, 3, 3),
                          None if uvs is None else np.asarray(uvs, np.float64).reshape(n, 3, 2),
                          np.ascontiguousarray(lay, dtype=np.uint32), self._ids(n)))
        return self.tris[-1][4]

    def add_sphere(self, center, radius, layers, light=False):
        i = int(self._ids(1)[0])
        self.spheres.append((*map(float, center), float(radius), layers[0], layers[1],
                             abi.OR3_SPHERE_LIGHT if light else 0, i))
        return i

    def add_plane(self, kind, axis, offset, flip, layers):
        i = int(self._ids(1)[0])
        self.planes.append((float(kind), float(axis), float(offset), 1.0 if flip else 0.0, layers[0], layers[1], i))
        return i

    def add_texture(self, rgb):
        rgb = np.ascontiguousarray(rgb, dtype=np.float32)
        self.textures.append(rgb)
        return len(self.textures) - 1

    def set_env(self, rgb):
        self.env = np.ascontiguousarray(rgb, dtype=np.float32)
        self.env_rgbe = None

    def set_env_rgbe(self, rgbe):
        """Environment as RGBE bytes (H, W, 4), e.g. from renderer.read_hdr."""
        self.env_rgbe = np.ascontiguousarray(rgbe, dtype=np.uint8)
        self.env = None

    @property
    def num_objects(self):
        return self._next_id

    def quantized_f32(self):
        """A copy whose geometry is exactly representable in FP32 (vertices,
        sphere centres and radii, plane offsets), so an FP64 reference and the
        FP32 kernels intersect identical primitives."""
        import copy
        q = copy.deepcopy(self)
        q.tris = [(t[0].astype(np.float32).astype(np.float64),) + tuple(t[1:]) for t in q.tris]
        q.spheres = [tuple(float(np.float32(x)) for x in s[:4]) + tuple(s[4:]) for s in q.spheres]
        q.planes = [s[:2] + (float(np.float32(s[2])),) + tuple(s[3:]) for s in q.planes]
        return q

    def digest(self):
        """sha256 of the flattened scene (fixtures record which scene they were made from)."""
        import hashlib
        a = self.arrays()
        h = hashlib.sha256()
        h.update(repr(a["mat"]).encode())
        for k in sorted(a):
            if k == "mat" or a[k] is None:
                continue
            h.update(k.encode())
            h.update(np.ascontiguousarray(a[k]).tobytes())
        if self.env is not None:
            h.update(self.env.tobytes())
        if self.env_rgbe is not None:
            h.update(self.env_rgbe.tobytes())
        return h.hexdigest()

    # ---- flattened arrays
    def arrays(self):
        a = {}
        m = self.materials
        a["mat"] = m
        a["layer_material"] = np.asarray(self.layer_material, np.uint32)
        a["layer_rate"] = np.asarray(self.layer_rate, np.float64)
        if self.tris:
            a["tri_vertices"] = _cat([t[0] for t in self.tris])
            n_tot = a["tri_vertices"].shape[0]
            if any(t[1] is not None for t in self.tris):
                norms = []
                for t in self.tris:
                    if t[1] is not None:
                        norms.append(t[1])
                    else:
                        v = t[0]
                        c = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
                        c /= np.linalg.norm(c, axis=1, keepdims=True)
                        norms.append(np.repeat(c[:, None, :], 3, axis=1))
                a["tri_normals"] = _cat(norms)
            else:
                a["tri_normals"] = None
            if any(t[2] is not None for t in self.tris):
                a["tri_uvs"] = _cat([t[2] if t[2] is not None else np.zeros((t[0].shape[0], 3, 2))
                                     for t in self.tris])
            else:
                a["tri_uvs"] = None
            a["tri_layers"] = _cat([t[3] for t in self.tris])
            a["tri_ids"] = _cat([t[4] for t in self.tris])
            assert a["tri_layers"].shape == (n_tot, 2)
        else:
            for k in ("tri_vertices", "tri_normals", "tri_uvs", "tri_layers", "tri_ids"):
                a[k] = None
        if self.spheres:
            s = np.asarray(self.spheres, dtype=np.float64)
            a["spheres"] = np.ascontiguousarray(s[:, :4])
            a["sphere_layers"] = np.ascontiguousarray(s[:, 4:6].astype(np.uint32))
            a["sphere_flags"] = np.ascontiguousarray(s[:, 6].astype(np.uint32))
            a["sphere_ids"] = np.ascontiguousarray(s[:, 7].astype(np.uint32))
        else:
            a["spheres"] = a["sphere_layers"] = a["sphere_flags"] = a["sphere_ids"] = None
        if self.planes:
            p = np.asarray(self.planes, dtype=np.float64)
            a["planes"] = np.ascontiguousarray(p[:, :4])
            a["plane_layers"] = np.ascontiguousarray(p[:, 4:6].astype(np.uint32))
            a["plane_ids"] = np.ascontiguousarray(p[:, 6].astype(np.uint32))
        else:
            a["planes"] = a["plane_layers"] = a["plane_ids"] = None
        if self.textures:
            dims = np.asarray([[t.shape[1], t.shape[0]] for t in self.textures], np.uint32)
            offs = np.cumsum([0] + [t.size for t in self.textures[:-1]]).astype(np.uint64)
            a["texture_dims"] = dims
            a["texture_offsets"] = offs
            a["texture_rgb"] = np.ascontiguousarray(np.concatenate([t.reshape(-1) for t in self.textures]))
        return a

    def to_c(self):
        """Returns (SceneDescC, keepalive) -- keep both alive while the C side reads them."""
        a = self.arrays()
        keep = [a]
        d = abi.SceneDescC()
        mats = (abi.Material * len(a["mat"]))()
        for i, (t, tex, em, col, ior, pe) in enumerate(a["mat"]):
            mats[i].type = t
            mats[i].texture = tex
            mats[i].emission = abi.c_double3(*em)
            mats[i].color = abi.c_double3(*col)
            mats[i].ior = ior
            mats[i].phong_exponent = pe
        keep.append(mats)
        d.num_materials = len(a["mat"])
        d.materials = ctypes.cast(mats, ctypes.POINTER(abi.Material))
        d.num_layers = len(a["layer_material"])
        d.layer_material = _ptr(a["layer_material"], ctypes.c_uint32)
        d.layer_rate = _ptr(a["layer_rate"], ctypes.c_double)
        if a["tri_vertices"] is not None:
            d.num_triangles = a["tri_vertices"].shape[0]
            d.tri_vertices = _ptr(a["tri_vertices"], ctypes.c_double)
            d.tri_normals = _ptr(a["tri_normals"], ctypes.c_double)
            d.tri_uvs = _ptr(a["tri_uvs"], ctypes.c_double)
            d.tri_layers = _ptr(a["tri_layers"], ctypes.c_uint32)
            d.tri_ids = _ptr(a["tri_ids"], ctypes.c_uint32)
        if a["spheres"] is not None:
            d.num_spheres = a["spheres"].shape[0]
            d.spheres = _ptr(a["spheres"], ctypes.c_double)
            d.sphere_layers = _ptr(a["sphere_layers"], ctypes.c_uint32)
            d.sphere_flags = _ptr(a["sphere_flags"], ctypes.c_uint32)
            d.sphere_ids = _ptr(a["sphere_ids"], ctypes.c_uint32)
        if a["planes"] is not None:
            d.num_planes = a["planes"].shape[0]
            d.planes = _ptr(a["planes"], ctypes.c_double)
            d.plane_layers = _ptr(a["plane_layers"], ctypes.c_uint32)
            d.plane_ids = _ptr(a["plane_ids"], ctypes.c_uint32)
        if self.env is not None:
            d.env_height, d.env_width = self.env.shape[0], self.env.shape[1]
            d.env_rgb = _ptr(self.env, ctypes.c_float)
            keep.append(self.env)
        elif self.env_rgbe is not None:
            d.env_height, d.env_width = self.env_rgbe.shape[0], self.env_rgbe.shape[1]
            d.env_rgbe = _ptr(self.env_rgbe, ctypes.c_uint8)
            keep.append(self.env_rgbe)
        d.background = abi.c_double3(*self.background)
        if self.textures:
            d.num_textures = len(self.textures)
            d.texture_dims = _ptr(a["texture_dims"], ctypes.c_uint32)
            d.texture_offsets = _ptr(a["texture_offsets"], ctypes.c_uint64)
            d.texture_rgb = _ptr(a["texture_rgb"], ctypes.c_float)
        d.build = self.build
        d.leaf_max = self.leaf_max
        d.traversal_cost = self.traversal_cost
        return d, keep


# ---------------------------------------------------------------- geometry helpers

def quad(corners, facing):
    """Two triangles (c0,c1,c2), (c0,c2,c3) wound so their face normal points
    along `facing` (the reference culls back faces: src/renderer/Polygon.h:72)."""
    c = np.asarray(corners, np.float64)
    n = np.cross(c[1] - c[0], c[2] - c[0])
    if np.dot(n, facing) < 0:
        c = c[::-1].copy()
    return np.stack([np.stack([c[0], c[1], c[2]]), np.stack([c[0], c[2], c[3]])])


def _hash3(ix, iy, iz, seed):
    h = (ix.astype(np.uint64) * np.uint64(73856093)) ^ (iy.astype(np.uint64) * np.uint64(19349663)) \
        ^ (iz.astype(np.uint64) * np.uint64(83492791)) ^ np.uint64(seed * 2654435761 & 0xFFFFFFFF)
    h ^= h >> np.uint64(13)
    h *= np.uint64(0x5bd1e995)
    h ^= h >> np.uint64(15)
    return (h & np.uint64(0xFFFFFF)).astype(np.float64) / float(0xFFFFFF) * 2.0 - 1.0


def value_noise3(p, seed):
    """Seeded lattice value noise in [-1, 1] with smoothstep interpolation."""
    p = np.asarray(p, np.float64)
    f = np.floor(p)
    t = p - f
    t = t * t * (3.0 - 2.0 * t)
    i = f.astype(np.int64) + (1 << 20)
    out = 0.0
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                w = (t[..., 0] if dx else 1 - t[..., 0]) * (t[..., 1] if dy else 1 - t[..., 1]) * \
                    (t[..., 2] if dz else 1 - t[..., 2])
                out = out + w * _hash3(i[..., 0] + dx, i[..., 1] + dy, i[..., 2] + dz, seed)
    return out


def fbm3(p, seed, octaves=4, lacunarity=2.0, gain=0.5):
    total, amp, freq = 0.0, 1.0, 1.0
    for o in range(octaves):
        total = total + amp * value_noise3(np.asarray(p) * freq, seed + 101 * o)
        amp *= gain
        freq *= lacunarity
    return total


def icosphere(level):
    """Unit icosphere with faces wound counter-clockwise seen from outside."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    for _ in range(level):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        e.sort(axis=1)
        key = e[:, 0] * (len(v) + 1) + e[:, 1]
        uk, inv = np.unique(key, return_inverse=True)
        a, b = uk // (len(v) + 1), uk % (len(v) + 1)
        mid = v[a] + v[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = len(v)
        v = np.concatenate([v, mid])
        nf = len(f)
        m01, m12, m20 = inv[:nf] + base, inv[nf:2 * nf] + base, inv[2 * nf:] + base
        f = np.concatenate([np.stack([f[:, 0], m01, m20], 1), np.stack([f[:, 1], m12, m01], 1),
                            np.stack([f[:, 2], m20, m12], 1), np.stack([m01, m12, m20], 1)])
    # orient outward
    c = v[f].mean(axis=1)
    n = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    flip = (n * c).sum(1) < 0
    f[flip] = f[flip][:, ::-1]
    return v, f


def vertex_normals(v, f):
    n = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])  # area weighted
    vn = np.zeros_like(v)
    for k in range(3):
        np.add.at(vn, f[:, k], n)
    vn /= np.linalg.norm(vn, axis=1, keepdims=True)
    return vn
