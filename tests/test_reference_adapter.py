"""The drop-in adapter (omochi-renderer3_gb300/host/reference_adapter.cpp and
its scene flattener host/reference_flatten.hpp) against the reference's own
classes.  Needs the reference sources (marker `reference`); builds with g++.

  * it compiles and links with the reference's objects and libor3.so into a
    program that renders the reference's CornellBoxScene (run only where a
    GPU exists);
  * linked instead with a CPU stand-in for libor3.so (tests/adapter/fake_or3.cpp)
    it keeps the Renderer threading contract (Renderer.h:10-23): StopRendering
    from a timer thread on a second RenderScene, a stopped renderer rendering
    nothing, whole frames for GetResult() readers, exceptions from the frame
    callback leaving no thread behind;
  * its flattener turns scenes the reference builds (SceneFromExternalFile on
    tests/golden/scene/full.scene.in, the built-in CornellBoxScene) into the
    same objects, in AddObject order, as the native scene-file reader and the
    Python scene builders.
"""
import ctypes
import glob
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

sys.path.insert(0, os.path.join(GOLDEN, "scene"))
from cases import stage_scene_dir  # noqa: E402

pytestmark = pytest.mark.reference

HOST = os.path.join(ROOT, "omochi-renderer3_gb300", "host")
ADAPTER_TESTS = os.path.join(ROOT, "tests", "adapter")


def _ref_src(oracle_mod):
    src = os.path.join(oracle_mod.REFERENCE_SRC, "src")
    if not os.path.isdir(src):
        pytest.skip("reference sources not present")
    if not oracle_mod.reference_available():
        oracle_mod.build_oracle(reference=True)
    return src


def _ref_objs():
    # the reference's compiled translation units, without the oracle harness and PathTracer
    return [o for o in glob.glob(os.path.join(ROOT, "oracle", "_ref", "obj", "*.o"))
            if "harness" not in o and "PathTracer" not in o]


def _flags(src):
    return ["-std=c++11", "-O1", "-w", "-I", src, "-I", os.path.join(ROOT, "include"), "-I", HOST,
            "-include", "immintrin.h"]


def _build(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def test_adapter_builds_against_the_reference(pkg, oracle_mod, tmp_path):
    src = _ref_src(oracle_mod)
    lib = pkg.build.build_library()
    exe = str(tmp_path / "gpu_main")
    _build(["g++", *_flags(src), os.path.join(HOST, "reference_adapter.cpp"),
            "-include", os.path.join(src, "stdafx.h"), os.path.join(src, "scenes", "CornellBoxScene.cpp"),
            os.path.join(ROOT, "tests", "adapter_main.cpp"), *_ref_objs(), lib, "-fopenmp", "-lpthread",
            "-Wl,-rpath," + os.path.dirname(lib), "-o", exe])
    if os.path.exists("/dev/nvidia0"):
        out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
        assert out.returncode == 0, out.stdout + out.stderr


def test_adapter_threading_with_a_stand_in_library(pkg, oracle_mod, tmp_path):
    src = _ref_src(oracle_mod)
    exe = str(tmp_path / "threads_main")
    _build(["g++", *_flags(src), "-O2", os.path.join(HOST, "reference_adapter.cpp"),
            os.path.join(ADAPTER_TESTS, "fake_or3.cpp"), "-include", os.path.join(src, "stdafx.h"),
            os.path.join(src, "scenes", "CornellBoxScene.cpp"), os.path.join(ADAPTER_TESTS, "threads_main.cpp"),
            *_ref_objs(), "-fopenmp", "-lpthread", "-o", exe])
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "torn 0" in out.stdout, out.stdout


class _Probe:
    def __init__(self, pkg, src, tmp_path):
        so = str(tmp_path / "libflatten_probe.so")
        _build(["g++", *_flags(src), "-fPIC", "-shared", os.path.join(ADAPTER_TESTS, "flatten_probe.cpp"),
                "-include", os.path.join(src, "stdafx.h"), os.path.join(src, "scenes", "CornellBoxScene.cpp"),
                *_ref_objs(), "-fopenmp", "-lpthread", "-o", so])
        self.lib = ctypes.CDLL(so)
        D = ctypes.POINTER(pkg.abi.SceneDescC)
        self.lib.flat_scene_file.restype = ctypes.c_void_p
        self.lib.flat_scene_file.argtypes = [ctypes.c_char_p, D]
        self.lib.flat_cornell.restype = ctypes.c_void_p
        self.lib.flat_cornell.argtypes = [D]
        self.lib.flat_free.argtypes = [ctypes.c_void_p]
        self.pkg = pkg

    def scene(self, path=None):
        d = self.pkg.abi.SceneDescC()
        h = self.lib.flat_scene_file(path.encode(), ctypes.byref(d)) if path else self.lib.flat_cornell(ctypes.byref(d))
        assert h
        try:
            sd = self.pkg.renderer.scene_from_desc(d)
            textured = [d.materials[i].texture >= 0 for i in range(d.num_materials)]
        finally:
            self.lib.flat_free(h)
        return sd, textured


def _records(sd, textured):
    """One row per object in id order: kind, geometry, then per layer (type,
    emission, colour, ior, rate, textured)."""
    rec = np.zeros((sd.num_objects, 31 + 10 * 4))

    def layers(r, b, c):
        r[1] = c
        for j in range(min(c, 4)):
            mi = sd.layer_material[b + j]
            mt, _tex, em, col, ior, _ph = sd.materials[mi]
            r[31 + 10 * j:41 + 10 * j] = [mt, *em, *col, ior, sd.layer_rate[b + j], textured[mi]]

    for verts, nrm, uv, lay, ids in sd.tris:
        if nrm is None:  # the face normal at every vertex (Polygon::CalculateNormal)
            fn = np.cross(verts[:, 1] - verts[:, 0], verts[:, 2] - verts[:, 0])
            fn /= np.linalg.norm(fn, axis=1, keepdims=True)
            nrm = np.repeat(fn[:, None, :], 3, axis=1)
        if uv is None:
            uv = np.zeros((verts.shape[0], 3, 2))
        for t in range(verts.shape[0]):
            r = rec[ids[t]]
            r[0] = 0
            r[2:11], r[11:20], r[20:26] = verts[t].reshape(9), nrm[t].reshape(9), uv[t].reshape(6)
            layers(r, *lay[t])
    for cx, cy, cz, rad, b, c, flags, i in sd.spheres:
        rec[i][0] = 2 if flags else 1
        rec[i][2:6] = [cx, cy, cz, rad]
        layers(rec[i], b, c)
    for kind, axis, off, flip, b, c, i in sd.planes:
        rec[i][0] = 3 + kind
        rec[i][2:5] = [axis, off, flip]
        layers(rec[i], b, c)
    return rec


def _sorted_rows(x):
    return x[np.lexsort(np.round(x, 9).T[::-1])]


def test_flattener_matches_the_native_scene_reader(pkg, oracle_mod, orc, tmp_path):
    src = _ref_src(oracle_mod)
    probe = _Probe(pkg, src, tmp_path)
    path = stage_scene_dir(str(tmp_path))
    flat, flat_tex = probe.scene(path)
    ours, info = pkg.load_scene_file(path)
    a = _records(flat, flat_tex)
    b = _records(ours, [t is not None for t in info["textures"]])
    assert a.shape == b.shape
    # the reference adds a mesh's triangles grouped by material, the reader in
    # file order: the mesh (ids 0..n-1) compares as a multiset, the rest in order
    n_mesh = ours.tris[0][0].shape[0] - 12
    np.testing.assert_allclose(_sorted_rows(a[:n_mesh]), _sorted_rows(b[:n_mesh]), rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(a[n_mesh:], b[n_mesh:], rtol=1e-12, atol=1e-15)
    # the IBL: the reference's decoded floats against the reader's RGBE bytes
    assert flat.env.shape[:2] == ours.env_rgbe.shape[:2]
    dec = orc.decode_rgbe(ours.env_rgbe.reshape(-1, 4)).reshape(flat.env.shape)
    np.testing.assert_allclose(flat.env, dec.astype(np.float32), rtol=1e-7)
    assert any(flat_tex)  # the file's textured material came through as a texture


def test_flattener_matches_the_python_cornell_builder(pkg, oracle_mod, tmp_path):
    src = _ref_src(oracle_mod)
    probe = _Probe(pkg, src, tmp_path)
    flat, flat_tex = probe.scene()
    ours, _, _ = pkg.workloads.reference_cornell()
    a, b = _records(flat, flat_tex), _records(ours, [False] * len(ours.materials))
    assert not any(flat_tex)
    # Scene::AddFloor* gives its floors uv coordinates (src/scenes/Scene.cpp:88-195)
    # and the Python builder none: uv is read only for textured layers, and
    # this scene has no texture, so the uv columns are left out
    cols = [c for c in range(a.shape[1]) if not 20 <= c < 26]
    np.testing.assert_allclose(a[:, cols], b[:, cols], rtol=1e-12, atol=1e-12)
    assert flat.background == tuple(float(c) for c in ours.background)
