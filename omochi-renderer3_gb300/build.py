"""In-tree build of libor3.so, the sm_103a CUDA path behind include/or3.h.

    python omochi-renderer3_gb300/build.py      (or __graft_entry__.build())

Sources are compiled in parallel with nvcc (one -gencode, sm_103a) into
omochi-renderer3_gb300/lib/ and linked into one shared library with the CUDA
runtime linked statically.  A rebuild happens only when a source or header is
newer than the library.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)
LIB_DIR = os.path.join(PKG_DIR, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libor3.so")
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(ROOT, "include")

SOURCES = ["or3_kernels.cu", "or3_api.cu", "or3_batch.cu", "or3_server.cu", "or3_noalloc.cu", "bvh_build.cpp", "bvh_wide8.cpp",
           "bvh_build_gpu.cu", "or3_image.cu", "hdr_io.cpp", "obj_ingest.cpp",
           "scene_file.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libor3.so")


def _inputs():
    files = [os.path.join(CSRC, s) for s in SOURCES]
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh", ".hpp")):
                files.append(os.path.join(d, f))
    return files


def needs_build():
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    return any(os.path.getmtime(f) > t for f in _inputs())


def _compile(src, obj, extra):
    nvcc = nvcc_path()
    cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
           "-I", INCLUDE, "-I", CSRC, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stderr


def build_library(force=False, verbose=False, extra_flags=()):
    """Compiles and links libor3.so; returns its path."""
    if not force and not needs_build():
        return LIB_PATH
    obj_dir = os.path.join(LIB_DIR, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    objs = [os.path.join(obj_dir, os.path.splitext(s)[0] + ".o") for s in SOURCES]
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        futs = [ex.submit(_compile, s, o, list(extra_flags)) for s, o in zip(SOURCES, objs)]
        for f in futs:
            log = f.result()
            if verbose and log:
                sys.stderr.write(log)
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc_path(), *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build_library(force="--force" in sys.argv, verbose=True))
