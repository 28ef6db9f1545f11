"""The drop-in adapter (omochi-renderer3_gb300/host/reference_adapter.cpp)
compiles against the reference's own headers and links with its objects and
libor3.so into a program that renders the reference's CornellBoxScene.
Needs the reference sources (marker `reference`); runs the program only where
a GPU exists."""
import glob
import os
import subprocess
import tempfile

import pytest

from conftest import ROOT

pytestmark = pytest.mark.reference


def test_adapter_builds_against_the_reference(pkg, oracle_mod):
    src = os.path.join(oracle_mod.REFERENCE_SRC, "src")
    if not os.path.isdir(src):
        pytest.skip("reference sources not present")
    if not oracle_mod.reference_available():
        oracle_mod.build_oracle(reference=True)
    lib = pkg.build.build_library()
    host = os.path.join(ROOT, "omochi-renderer3_gb300", "host")
    objs = [o for o in glob.glob(os.path.join(ROOT, "oracle", "_ref", "obj", "*.o"))
            if "harness" not in o and "PathTracer" not in o]
    flags = ["-std=c++11", "-O1", "-w", "-I", src, "-I", os.path.join(ROOT, "include"), "-I", host,
             "-include", "immintrin.h"]
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "gpu_main")
        cmd = ["g++", *flags, os.path.join(host, "reference_adapter.cpp"),
               "-include", os.path.join(src, "stdafx.h"), os.path.join(src, "scenes", "CornellBoxScene.cpp"),
               os.path.join(ROOT, "tests", "adapter_main.cpp"), *objs, lib, "-fopenmp", "-lpthread",
               "-Wl,-rpath," + os.path.dirname(lib), "-o", exe]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
        if os.path.exists("/dev/nvidia0"):
            out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
            assert out.returncode == 0, out.stdout + out.stderr
