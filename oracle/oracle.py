"""TEST INFRASTRUCTURE ONLY: ctypes access to the two oracle arms.

  CRestatement   oracle/_build/liboracle.so  -- the FP64 C restatement
                 (or3_oracle.c), built on every machine by build()
  Reference      oracle/_ref/libor3ref*.so   -- the reference's own sources plus
                 ref_harness.cpp, built only where the reference sources exist

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this.
"""
import ctypes
import os
import subprocess

import numpy as np

ORACLE_DIR = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(ORACLE_DIR, "_build", "liboracle.so")
REF_LIB = os.path.join(ORACLE_DIR, "_ref", "libor3ref.so")
REF_CFG_LIB = os.path.join(ORACLE_DIR, "_ref", "libor3ref_cfg.so")


def _reference_dir():
    """The reference checkout: $OR3_REFERENCE_DIR, else the one `make ref`
    last compiled (recorded in _ref/source_dir), else none."""
    if os.environ.get("OR3_REFERENCE_DIR"):
        return os.environ["OR3_REFERENCE_DIR"]
    rec = os.path.join(ORACLE_DIR, "_ref", "source_dir")
    if os.path.exists(rec):
        return open(rec).read().strip()
    return ""


REFERENCE_SRC = _reference_dir()

f64p = ctypes.POINTER(ctypes.c_double)
i32p = ctypes.POINTER(ctypes.c_int32)


class OrcParams(ctypes.Structure):
    _fields_ = [("supersamples", ctypes.c_int32), ("min_samples", ctypes.c_int32),
                ("max_samples", ctypes.c_int32), ("step_samples", ctypes.c_int32),
                ("next_event_estimation", ctypes.c_int32), ("rr_min_depth", ctypes.c_int32),
                ("max_depth", ctypes.c_int32), ("pad", ctypes.c_int32), ("seed", ctypes.c_uint64)]


def build_oracle(reference=True, reference_dir=None):
    """make -C oracle (C restatement) and, when a reference checkout is named
    (reference_dir, else $OR3_REFERENCE_DIR) and holds the sources, make ref."""
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)
    ref = reference_dir or REFERENCE_SRC
    if reference and ref and os.path.isdir(os.path.join(ref, "src")):
        subprocess.run(["make", "-s", "-C", ORACLE_DIR, "ref", "REF=%s" % ref, "-j8"], check=True)


def reference_available():
    return os.path.exists(REF_LIB) and os.path.exists(REF_CFG_LIB)


def _np(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def _params(supersamples=1, min_samples=1, max_samples=1, step_samples=1, next_event_estimation=False,
            rr_min_depth=5, max_depth=0, seed=0, **_):
    p = OrcParams()
    p.supersamples, p.min_samples, p.max_samples, p.step_samples = supersamples, min_samples, max_samples, step_samples
    p.next_event_estimation = 1 if next_event_estimation else 0
    p.rr_min_depth, p.max_depth, p.seed = rr_min_depth, max_depth, seed
    return p


class CRestatement:
    def __init__(self):
        if not os.path.exists(LIB):
            build_oracle(reference=False)
        lib = ctypes.CDLL(LIB)
        lib.orc_scene_create.restype = ctypes.c_void_p
        lib.orc_scene_create.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.orc_scene_destroy.argtypes = [ctypes.c_void_p]
        lib.orc_scene_bvh_nodes.argtypes = [ctypes.c_void_p]
        lib.orc_closest.argtypes = [ctypes.c_void_p, ctypes.c_size_t, f64p, f64p, i32p, f64p, f64p]
        lib.orc_object_distance.argtypes = [ctypes.c_void_p, ctypes.c_size_t, i32p, f64p, f64p, f64p]
        lib.orc_path_radiance.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(OrcParams),
                                          ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, f64p]
        u8p = ctypes.POINTER(ctypes.c_uint8)
        lib.orc_encode_rgb8.argtypes = [ctypes.c_size_t, f64p, ctypes.c_int, u8p]
        lib.orc_encode_rgbe.argtypes = [ctypes.c_size_t, f64p, u8p]
        lib.orc_decode_rgbe.argtypes = [ctypes.c_size_t, u8p, f64p]
        lib.orc_render.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(OrcParams), ctypes.c_int,
                                   f64p, f64p, f64p]
        lib.orc_philox.argtypes = [ctypes.POINTER(ctypes.c_uint32), ctypes.c_uint32, ctypes.c_uint32,
                                   ctypes.POINTER(ctypes.c_uint32)]
        lib.orc_env_sample.argtypes = [ctypes.c_void_p, ctypes.c_size_t, f64p, f64p]
        lib.orc_texel.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t, f64p, f64p]
        self.lib = lib

    def encode_rgb8(self, rgb, gamma=True):
        c = np.ascontiguousarray(rgb, np.float64).reshape(-1, 3)
        out = np.zeros((c.shape[0], 3), np.uint8)
        self.lib.orc_encode_rgb8(c.shape[0], _np(c, ctypes.c_double), 1 if gamma else 0, _np(out, ctypes.c_uint8))
        return out

    def encode_rgbe(self, rgb):
        c = np.ascontiguousarray(rgb, np.float64).reshape(-1, 3)
        out = np.zeros((c.shape[0], 4), np.uint8)
        self.lib.orc_encode_rgbe(c.shape[0], _np(c, ctypes.c_double), _np(out, ctypes.c_uint8))
        return out

    def decode_rgbe(self, rgbe):
        b = np.ascontiguousarray(rgbe, np.uint8).reshape(-1, 4)
        out = np.zeros((b.shape[0], 3), np.float64)
        self.lib.orc_decode_rgbe(b.shape[0], _np(b, ctypes.c_uint8), _np(out, ctypes.c_double))
        return out

    def philox(self, ctr, k0, k1):
        c = (ctypes.c_uint32 * 4)(*ctr)
        o = (ctypes.c_uint32 * 4)()
        self.lib.orc_philox(c, k0, k1, o)
        return list(o)

    def scene(self, sd, use_bvh=True):
        return _OracleScene(self, sd, use_bvh)


class _OracleScene:
    def __init__(self, orc, sd, use_bvh):
        self.orc = orc
        d, self._keep = sd.to_c()
        self._desc = d
        self.h = orc.lib.orc_scene_create(ctypes.byref(d), 1 if use_bvh else 0)

    def __del__(self):
        if getattr(self, "h", None):
            self.orc.lib.orc_scene_destroy(self.h)
            self.h = None

    def bvh_nodes(self):
        return self.orc.lib.orc_scene_bvh_nodes(self.h)

    def closest(self, orig, dirs):
        o = np.ascontiguousarray(orig, np.float64)
        d = np.ascontiguousarray(dirs, np.float64)
        n = o.shape[0]
        ids = np.zeros(n, np.int32)
        t = np.zeros(n, np.float64)
        nrm = np.zeros((n, 3), np.float64)
        self.orc.lib.orc_closest(self.h, n, _np(o, ctypes.c_double), _np(d, ctypes.c_double),
                                 _np(ids, ctypes.c_int32), _np(t, ctypes.c_double), _np(nrm, ctypes.c_double))
        return ids, t, nrm

    def object_distance(self, ids, orig, dirs):
        o = np.ascontiguousarray(orig, np.float64)
        d = np.ascontiguousarray(dirs, np.float64)
        i = np.ascontiguousarray(ids, np.int32)
        t = np.zeros(len(i), np.float64)
        self.orc.lib.orc_object_distance(self.h, len(i), _np(i, ctypes.c_int32), _np(o, ctypes.c_double),
                                         _np(d, ctypes.c_double), _np(t, ctypes.c_double))
        return t

    def env_sample(self, dirs):
        d = np.ascontiguousarray(dirs, np.float64).reshape(-1, 3)
        out = np.zeros((d.shape[0], 3), np.float64)
        self.orc.lib.orc_env_sample(self.h, d.shape[0], _np(d, ctypes.c_double), _np(out, ctypes.c_double))
        return out

    def texel(self, tex, uv):
        u = np.ascontiguousarray(uv, np.float64).reshape(-1, 2)
        out = np.zeros((u.shape[0], 3), np.float64)
        if self.orc.lib.orc_texel(self.h, tex, u.shape[0], _np(u, ctypes.c_double), _np(out, ctypes.c_double)):
            raise ValueError("no texture %d" % tex)
        return out

    def path_radiance(self, camera, first, count, nthreads=0, **settings):
        cam = camera.to_c()
        p = _params(**settings)
        out = np.zeros((count, 3), np.float64)
        self.orc.lib.orc_path_radiance(self.h, ctypes.byref(cam), ctypes.byref(p), first, count, nthreads,
                                       _np(out, ctypes.c_double))
        return out

    def render(self, camera, nthreads=0, **settings):
        cam = camera.to_c()
        p = _params(**settings)
        s = np.zeros((camera.height, camera.width, 3), np.float64)
        q = np.zeros_like(s)
        sec = ctypes.c_double()
        self.orc.lib.orc_render(self.h, ctypes.byref(cam), ctypes.byref(p), nthreads, _np(s, ctypes.c_double),
                                _np(q, ctypes.c_double), ctypes.byref(sec))
        return s, q, sec.value


class Reference:
    """The reference's compiled code (unmodified; `cfg=True` = the copy whose
    MinDepth and hard depth cut are runtime settings)."""

    def __init__(self, cfg=False):
        path = REF_CFG_LIB if cfg else REF_LIB
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        lib = ctypes.CDLL(path)
        lib.orref_scene_create.restype = ctypes.c_void_p
        lib.orref_scene_create.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.orref_scene_destroy.argtypes = [ctypes.c_void_p]
        lib.orref_closest.argtypes = [ctypes.c_void_p, ctypes.c_size_t, f64p, f64p, i32p, f64p, f64p, f64p]
        lib.orref_ibl_sample.argtypes = [ctypes.c_void_p, ctypes.c_size_t, f64p, f64p]
        lib.orref_texel.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t, f64p, f64p]
        lib.orref_render_moments.argtypes = [ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_int] * 6 + [f64p, f64p, f64p]
        lib.orref_render_scene.argtypes = [ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_int] * 6 + [f64p, f64p]
        if cfg:
            lib.orref_set_depth_limits.argtypes = [ctypes.c_int, ctypes.c_int]
        u8p = ctypes.POINTER(ctypes.c_uint8)
        lib.orref_encode_rgb8.argtypes = [ctypes.c_size_t, f64p, ctypes.c_int, u8p]
        lib.orref_encode_rgbe.argtypes = [ctypes.c_size_t, f64p, u8p]
        lib.orref_decode_rgbe.argtypes = [ctypes.c_size_t, u8p, f64p]
        lib.orref_write_hdr.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, f64p]
        lib.orref_read_hdr.argtypes = [ctypes.c_char_p, i32p, i32p, f64p, ctypes.c_size_t]
        lib.orref_load_obj.restype = ctypes.c_long
        lib.orref_load_scene_file.restype = ctypes.c_long
        lib.orref_load_scene_file.argtypes = [ctypes.c_char_p, f64p, ctypes.c_long, f64p]
        lib.orref_load_obj.argtypes = [ctypes.c_char_p, ctypes.c_int, f64p, f64p, f64p, f64p, f64p, f64p, f64p,
                                       ctypes.c_long]
        self.lib = lib
        self.cfg = cfg

    # ---- the reference's image conversions (src/tools/FileSaver.h, HDRImage.h/.cpp)
    def encode_rgb8(self, rgb, gamma=True):
        c = np.ascontiguousarray(rgb, np.float64).reshape(-1, 3)
        out = np.zeros((c.shape[0], 3), np.uint8)
        self.lib.orref_encode_rgb8(c.shape[0], _np(c, ctypes.c_double), 1 if gamma else 0, _np(out, ctypes.c_uint8))
        return out

    def encode_rgbe(self, rgb):
        c = np.ascontiguousarray(rgb, np.float64).reshape(-1, 3)
        out = np.zeros((c.shape[0], 4), np.uint8)
        self.lib.orref_encode_rgbe(c.shape[0], _np(c, ctypes.c_double), _np(out, ctypes.c_uint8))
        return out

    def decode_rgbe(self, rgbe):
        b = np.ascontiguousarray(rgbe, np.uint8).reshape(-1, 4)
        out = np.zeros((b.shape[0], 3), np.float64)
        self.lib.orref_decode_rgbe(b.shape[0], _np(b, ctypes.c_uint8), _np(out, ctypes.c_double))
        return out

    def write_hdr(self, path, rgb):
        c = np.ascontiguousarray(rgb, np.float64)
        h, w = c.shape[:2]
        if self.lib.orref_write_hdr(path.encode(), w, h, _np(c, ctypes.c_double)) != 0:
            raise IOError(path)

    def load_obj(self, path, flip_v=False, position=(0, 0, 0), scaling=(1, 1, 1), rotation=(0, 0, 0)):
        """Model::ReadFromObj + Transform: (tri [n,3,3], normals [n,3,3], uvs [n,3,2], mat [n,5])."""
        args = [np.ascontiguousarray(x, np.float64) for x in (position, scaling, rotation)]
        z = np.zeros(1)
        n = self.lib.orref_load_obj(path.encode(), 1 if flip_v else 0, *[_np(a, ctypes.c_double) for a in args],
                                    _np(z, ctypes.c_double), _np(z, ctypes.c_double), _np(z, ctypes.c_double),
                                    _np(z, ctypes.c_double), 0)
        if n < 0:
            raise IOError(path)
        tri, nrm = np.zeros((n, 3, 3)), np.zeros((n, 3, 3))
        uv, mat = np.zeros((n, 3, 2)), np.zeros((n, 5))
        self.lib.orref_load_obj(path.encode(), 1 if flip_v else 0, *[_np(a, ctypes.c_double) for a in args],
                                _np(tri, ctypes.c_double), _np(nrm, ctypes.c_double), _np(uv, ctypes.c_double),
                                _np(mat, ctypes.c_double), n)
        return tri, nrm, uv, mat

    def load_scene_file(self, path):
        """SceneFromExternalFile: (records [n, 67], ibl [5]) or None when the reference rejects the file.
        Record: kind, in BVH, layers, geometry 24, then 4 x (type, emission 3, colour 3, ior, rate, texture)."""
        ibl = np.zeros(5)
        z = np.zeros(1)
        n = self.lib.orref_load_scene_file(path.encode(), _np(z, ctypes.c_double), 0, _np(ibl, ctypes.c_double))
        if n < 0:
            return None
        rec = np.zeros((n, 67))
        self.lib.orref_load_scene_file(path.encode(), _np(rec, ctypes.c_double), n, _np(ibl, ctypes.c_double))
        return rec, ibl

    def read_hdr(self, path):
        w, h = ctypes.c_int32(), ctypes.c_int32()
        if self.lib.orref_read_hdr(path.encode(), ctypes.byref(w), ctypes.byref(h), None, 0) != 0:
            raise IOError(path)
        out = np.zeros((h.value, w.value, 3), np.float64)
        self.lib.orref_read_hdr(path.encode(), ctypes.byref(w), ctypes.byref(h), _np(out, ctypes.c_double), out.size)
        return out

    def set_depth_limits(self, rr_min_depth, max_depth):
        if not self.cfg:
            raise RuntimeError("depth limits need the cfg build")
        self.lib.orref_set_depth_limits(rr_min_depth, max_depth)

    def scene(self, sd, use_bvh=True):
        return _RefScene(self, sd, use_bvh)


class _RefScene:
    def __init__(self, ref, sd, use_bvh):
        self.ref = ref
        d, self._keep = sd.to_c()
        self._desc = d
        self.h = ref.lib.orref_scene_create(ctypes.byref(d), 1 if use_bvh else 0)

    def __del__(self):
        if getattr(self, "h", None):
            self.ref.lib.orref_scene_destroy(self.h)
            self.h = None

    def closest(self, orig, dirs):
        o = np.ascontiguousarray(orig, np.float64)
        d = np.ascontiguousarray(dirs, np.float64)
        n = o.shape[0]
        ids = np.zeros(n, np.int32)
        t = np.zeros(n, np.float64)
        nrm = np.zeros((n, 3), np.float64)
        pos = np.zeros((n, 3), np.float64)
        self.ref.lib.orref_closest(self.h, n, _np(o, ctypes.c_double), _np(d, ctypes.c_double),
                                   _np(ids, ctypes.c_int32), _np(t, ctypes.c_double), _np(nrm, ctypes.c_double),
                                   _np(pos, ctypes.c_double))
        return ids, t, nrm

    def ibl_sample(self, dirs):
        d = np.ascontiguousarray(dirs, np.float64).reshape(-1, 3)
        out = np.zeros((d.shape[0], 3), np.float64)
        if self.ref.lib.orref_ibl_sample(self.h, d.shape[0], _np(d, ctypes.c_double), _np(out, ctypes.c_double)):
            raise ValueError("scene has no IBL")
        return out

    def texel(self, tex, uv):
        u = np.ascontiguousarray(uv, np.float64).reshape(-1, 2)
        out = np.zeros((u.shape[0], 3), np.float64)
        if self.ref.lib.orref_texel(self.h, tex, u.shape[0], _np(u, ctypes.c_double), _np(out, ctypes.c_double)):
            raise ValueError("no texture %d" % tex)
        return out

    def render_moments(self, camera, supersamples=1, min_samples=1, max_samples=1, step_samples=1, nthreads=0,
                       next_event_estimation=False, **_):
        cam = camera.to_c()
        s = np.zeros((camera.height, camera.width, 3), np.float64)
        q = np.zeros_like(s)
        sec = ctypes.c_double()
        self.ref.lib.orref_render_moments(self.h, ctypes.byref(cam), min_samples, max_samples, step_samples,
                                          supersamples, nthreads, 1 if next_event_estimation else 0,
                                          _np(s, ctypes.c_double), _np(q, ctypes.c_double), ctypes.byref(sec))
        return s, q, sec.value

    def render_scene(self, camera, supersamples=1, min_samples=1, max_samples=1, step_samples=1, nthreads=1,
                     next_event_estimation=False, **_):
        cam = camera.to_c()
        out = np.zeros((camera.height, 2 * camera.width, 3), np.float64)
        sec = ctypes.c_double()
        self.ref.lib.orref_render_scene(self.h, ctypes.byref(cam), min_samples, max_samples, step_samples,
                                        supersamples, nthreads, 1 if next_event_estimation else 0,
                                        _np(out, ctypes.c_double), ctypes.byref(sec))
        return out, sec.value
