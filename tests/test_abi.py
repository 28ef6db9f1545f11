"""CPU checks of the drop-in boundary: libor3.so builds, exports every
function include/or3.h declares, and the ctypes mirror has the C layouts.
No compute call is made (no GPU needed)."""
import ctypes
import os
import re
import subprocess
import tempfile

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "or3.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(or3_[a-z_]+)\s*\(", src)) - {"or3_frame_callback"})


def test_library_builds_and_exports_every_declared_symbol(pkg):
    path = pkg.build.build_library()
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (or3_\w+)", out))
    missing = [f for f in declared_functions() if f not in exported]
    assert not missing, missing
    # and the Python mirror binds each of them
    assert set(declared_functions()) <= set(pkg.abi.PROTOTYPES), set(declared_functions()) - set(pkg.abi.PROTOTYPES)


def test_python_constants_match_the_header(pkg):
    """Every OR3_* integer constant of include/or3.h has the same value in abi.py."""
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    defines = dict(re.findall(r"#define\s+(OR3_\w+)\s+(0x[0-9a-fA-F]+|\d+)u?\b", src))
    assert len(defines) > 30
    missing = [k for k in defines if not hasattr(pkg.abi, k)]
    assert not missing, missing
    wrong = {k: (v, getattr(pkg.abi, k)) for k, v in defines.items() if int(v, 0) != getattr(pkg.abi, k)}
    assert not wrong, wrong


def test_library_loads_without_a_gpu(pkg):
    lib = ctypes.CDLL(pkg.build.build_library())
    lib.or3_api_version.restype = ctypes.c_int
    assert lib.or3_api_version() == pkg.abi.API_VERSION


LAYOUT_C = r"""
#include <stdio.h>
#include <stddef.h>
#include "or3.h"
#define S(T) printf(#T " %zu\n", sizeof(T));
#define O(T, f) printf(#T "." #f " %zu\n", offsetof(T, f));
int main(void) {
  S(or3_material) O(or3_material, emission) O(or3_material, ior) O(or3_material, phong_exponent)
  S(or3_scene_desc) O(or3_scene_desc, tri_vertices) O(or3_scene_desc, spheres) O(or3_scene_desc, planes)
  O(or3_scene_desc, env_rgb) O(or3_scene_desc, background) O(or3_scene_desc, texture_rgb)
  S(or3_camera) O(or3_camera, position) O(or3_camera, aperture_radius)
  S(or3_render_params) O(or3_render_params, seed) O(or3_render_params, flags)
  S(or3_render_stats) O(or3_render_stats, render_ms) O(or3_render_stats, passes) O(or3_render_stats, lanes) O(or3_render_stats, kernel_launches)
  S(or3_scene_info) O(or3_scene_info, build_ms) O(or3_scene_info, tree_depth) O(or3_scene_info, flatten_ms)
  S(or3_server_stats) O(or3_server_stats, latency_p50_s) O(or3_server_stats, waves_rerun)
  return 0;
}
"""


def test_ctypes_layouts_match_the_header(pkg):
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "layout.c")
        exe = os.path.join(d, "layout")
        open(src, "w").write(LAYOUT_C)
        subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    a = pkg.abi
    py = {"or3_material": a.Material, "or3_scene_desc": a.SceneDescC, "or3_camera": a.CameraC,
          "or3_render_params": a.RenderParamsC, "or3_render_stats": a.RenderStatsC, "or3_scene_info": a.SceneInfoC,
          "or3_server_stats": a.ServerStatsC}
    for line in out.strip().splitlines():
        key, val = line.split()
        if "." in key:
            t, f = key.split(".")
            assert getattr(py[t], f).offset == int(val), key
        else:
            assert ctypes.sizeof(py[key]) == int(val), key


def test_product_code_never_touches_the_oracle():
    """The shipped package and kernels do not import, load or link the oracle."""
    pkg_dir = os.path.join(ROOT, "omochi-renderer3_gb300")
    for dirpath, _, files in os.walk(pkg_dir):
        if "lib" in dirpath.split(os.sep):
            continue
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".cpp", ".h", ".hpp")):
                text = open(os.path.join(dirpath, f)).read()
                assert "or3_oracle" not in text and "liboracle" not in text and "orref_" not in text, f


def test_context_creation_fails_cleanly_without_a_device(pkg):
    if os.path.exists("/dev/nvidia0"):
        pytest.skip("a GPU is present")
    with pytest.raises(pkg.Or3Error) as e:
        pkg.Context(0)
    assert e.value.code == pkg.abi.OR3_ERR_NO_DEVICE
