"""Seeded mutations of scene, .obj/.mtl and .hdr files through the host readers,
built with AddressSanitizer and UndefinedBehaviorSanitizer (no GPU).

The readers take files from users, so a malformed file must load or fail with a
status: no read past a buffer, no use after free, no undefined arithmetic.
tests/reader_fuzz.cpp drives or3_scene_load_file (which reads the mesh through
or3_mesh_load_obj on 1-4 threads) and or3_read_hdr on exact-size buffers."""
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

sys.path.insert(0, os.path.join(GOLDEN, "scene"))
from cases import stage_scene_dir  # noqa: E402

CSRC = os.path.join(ROOT, "omochi-renderer3_gb300", "csrc")


def test_readers_under_sanitizers(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    exe = str(tmp_path / "reader_fuzz")
    cmd = ["g++", "-std=c++17", "-O1", "-g", "-pthread", "-fsanitize=address,undefined", "-fno-omit-frame-pointer",
           "-fno-sanitize-recover=undefined", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "reader_fuzz.cpp"), os.path.join(CSRC, "scene_file.cpp"),
           os.path.join(CSRC, "obj_ingest.cpp"), os.path.join(CSRC, "hdr_io.cpp"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("sanitizer build unavailable: " + r.stderr[-300:])
    stage = str(tmp_path / "stage")
    os.makedirs(stage)
    stage_scene_dir(stage)
    codec = np.load(os.path.join(GOLDEN, "image_codec.npz"))
    hdrs = []
    for name in ("rle", "flat"):
        p = str(tmp_path / (name + ".hdr"))
        with open(p, "wb") as fh:
            fh.write(codec["hdr_%s_file" % name].tobytes())
        hdrs.append(p)
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="print_stacktrace=1")
    r = subprocess.run([exe, stage, hdrs[0], hdrs[1], "600", "4000"], capture_output=True, text=True, env=env,
                       timeout=600)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-4000:])
    assert "ERROR: AddressSanitizer" not in r.stderr and "runtime error" not in r.stderr, r.stderr[-4000:]
    ok, failed = [int(x) for x in r.stdout.split()[1::2]]
    assert ok > 0 and failed > 0
