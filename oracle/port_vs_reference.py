"""TEST INFRASTRUCTURE: how fast the FP64 C oracle (the port that bench.py
times as its CPU baseline, oracle/or3_oracle.c) runs compared with the
reference's own integrator compiled from its sources (oracle/_ref:
PathTracer::Radiance per camera sample with the reference's BVH, driven by
ref_harness.cpp's thread pool), on the same scenes, estimator, depth rules and
host threads.

    python oracle/port_vs_reference.py [--threads N]

Both render the whole image with next-event estimation off (the reference's
own NEE does not work) and the reference's binary SAH BVH; the scenes are
reduced-resolution versions of the benchmark workloads that the reference
can render (the mesh with Lambert faces only: the reference has no glossy
lobe).  Prints one JSON line per scene and thread count: Mpaths/s of each
and port / reference.  The port draws its random numbers from Philox and the
reference from its xorshift stream, so their images agree statistically, not
bit for bit.
"""
import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import __graft_entry__ as ge  # noqa: E402


def scenes(W):
    return {
        "cornell": (lambda: W.cornell_box(256, 256), dict(supersamples=8, max_samples=1, rr_min_depth=3,
                                                           max_depth=8)),
        "mesh_lambert": (lambda: W.icosphere_in_box(256, 192, glossy_faces=False),
                         dict(supersamples=4, max_samples=2, rr_min_depth=5, max_depth=10)),
        "terrain_bsdf": (lambda: W.terrain_ibl(240, 136), dict(supersamples=4, max_samples=1, rr_min_depth=5,
                                                                 max_depth=12)),
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, nargs="*", default=[os.cpu_count()])
    ap.add_argument("--only", default="")
    a = ap.parse_args()
    pkg = ge.load_package()
    O = ge.load_oracle()
    if not O.reference_available():
        sys.exit("oracle/_ref is not built (the reference sources are needed)")
    ref = O.Reference(cfg=True)
    orc = O.CRestatement()
    for name, (build, st) in scenes(pkg.workloads).items():
        if a.only and a.only != name:
            continue
        sd, cam, _ = build()
        kw = dict(supersamples=st["supersamples"], min_samples=1, max_samples=st["max_samples"], step_samples=1,
                  next_event_estimation=False, rr_min_depth=st["rr_min_depth"], max_depth=st["max_depth"], seed=3)
        paths = cam.width * cam.height * st["supersamples"] ** 2 * st["max_samples"]
        t0 = time.time()
        rs = ref.scene(sd, use_bvh=True)
        ref_build = time.time() - t0
        t0 = time.time()
        ps = orc.scene(sd, use_bvh=True)
        port_build = time.time() - t0
        ref.set_depth_limits(st["rr_min_depth"], st["max_depth"])
        for n in a.threads:
            _, _, t_ref = rs.render_moments(cam, nthreads=n, **kw)
            _, _, t_port = ps.render(cam, nthreads=n, **kw)
            print(json.dumps({"scene": name, "threads": n, "paths": paths, "reference_mpaths_s": paths / t_ref / 1e6,
                              "port_mpaths_s": paths / t_port / 1e6, "port_over_reference": t_ref / t_port,
                              "reference_bvh_build_s": ref_build, "port_bvh_build_s": port_build}), flush=True)


if __name__ == "__main__":
    main()
