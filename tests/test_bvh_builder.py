"""CPU property tests of the host wide-BVH builder (csrc/bvh_build.cpp)."""
import os
import subprocess
import tempfile

import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "omochi-renderer3_gb300", "csrc")


@pytest.fixture(scope="module")
def bvh_check_bin():
    d = tempfile.mkdtemp()
    exe = os.path.join(d, "bvh_check")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", CSRC, "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "bvh_check.cpp"), os.path.join(CSRC, "bvh_build.cpp"), "-o", exe],
                   check=True)
    return exe


@pytest.mark.parametrize("n,seed,mode", [(1, 1, 0), (3, 1, 0), (4, 2, 0), (5, 3, 0), (1000, 4, 0),
                                         (100000, 5, 0), (500, 6, 1), (20000, 7, 2), (3000, 8, 3), (0, 1, 0)])
def test_builder_properties(bvh_check_bin, n, seed, mode):
    r = subprocess.run([bvh_check_bin, str(n), str(seed), str(mode)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
