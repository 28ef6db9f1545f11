"""Generates the golden fixtures in tests/golden/ from the reference's own code.

    python tests/golden/make_golden.py [--rmse]

Needs oracle/_ref (the reference sources compiled by `make -C oracle ref`),
so it runs where the reference is present; the fixtures it writes are
committed and are all the GPU tests need.

  closest_<scene>.npz   seeded FP64 ray sets (primary rays from around the
                        scene and secondary rays leaving surfaces) with the
                        reference's Scene::CheckIntersection answers through
                        its BVH (use_bvh=1) and its brute-force loop (use_bvh=0)
  render_<name>.npz     per-pixel mean and standard error of the reference's
                        PathTracer::Radiance estimator (float16), sample counts
  rmse_cornell_cfg.npz  (--rmse) 16384-spp reference render of the Cornell
                        workload, the RMSE target
  obj_ref.npz           the reference's Model::ReadFromObj + Transform of
                        tests/golden/obj/mesh.obj (with and without the v flip)
  image_codec.npz       the reference's 8-bit conversion (gamma on and off),
                        Color2RGBE and RGBE2Color on seeded colours and bytes,
                        and two .hdr files its writer produced (one run-length
                        encoded, one flat) with what its reader decodes
  scene_ref.npz         the reference's SceneFromExternalFile on
                        tests/golden/scene/full.scene.in (one record per
                        scene object, the IBL's size and texel sum) and its
                        accept/reject verdict on each file of scene/cases.py
Each fixture stores a digest of the flattened scene it was made from.
"""
import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
import __graft_entry__ as ge  # noqa: E402

pkg = ge.load_package()
O = ge.load_oracle()
W = pkg.workloads


def scene_digest(sd):
    return sd.digest()


def ico_in_box(level):
    sd, cam, st = W.icosphere_in_box(64, 48, level=level)
    return sd


CLOSEST_SCENES = {
    "cornell": lambda: W.cornell_box()[0],
    "refcornell": lambda: W.reference_cornell()[0],
    "tris3000": lambda: W.random_triangles(3000, 7),
    "ico3": lambda: ico_in_box(3),
    "ico6": lambda: ico_in_box(6),
}


def secondary_rays(o, d, ids, t, seed):
    """Rays leaving the first-hit points in random directions."""
    rng = np.random.default_rng(seed)
    hit = ids >= 0
    p = o[hit] + d[hit] * t[hit][:, None]
    v = rng.normal(size=p.shape)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return p, v


def f32(a):
    return np.asarray(a, np.float64).astype(np.float32).astype(np.float64)


def make_closest(name, nrays=2048, seed=5):
    # scene and rays exactly representable in FP32: the reference (FP64) and
    # the kernels (FP32) then intersect identical rays with identical geometry
    sd = CLOSEST_SCENES[name]().quantized_f32()
    ref = O.Reference()
    rs_bvh = ref.scene(sd, use_bvh=True)
    rs_bf = ref.scene(sd, use_bvh=False)
    o1, d1 = W.random_rays(nrays, seed)
    o1, d1 = f32(o1), f32(d1)
    ids1, t1, _ = rs_bvh.closest(o1, d1)
    o2, d2 = secondary_rays(o1, d1, ids1, t1, seed + 1)
    o = np.concatenate([o1, f32(o2)])
    d = np.concatenate([d1, f32(d2)])
    ids, t, nrm = rs_bvh.closest(o, d)
    ids_bf, t_bf, _ = rs_bf.closest(o, d)
    path = os.path.join(HERE, "closest_%s.npz" % name)
    np.savez_compressed(path, digest=scene_digest(sd), orig=o, dir=d, ids=ids, t=t, normal=nrm.astype(np.float32),
                        ids_bruteforce=ids_bf, t_bruteforce=t_bf, n_primary=len(o1))
    print("%s: %d rays, hit %.3f, bvh==bruteforce %.5f" % (path, len(o), (ids >= 0).mean(), (ids == ids_bf).mean()))


RENDERS = {
    # name: (builder, settings, cfg library (rr, max depth) or None, nthreads)
    "cornell_ref": (lambda: W.cornell_box(256, 256),
                    dict(supersamples=8, min_samples=1, max_samples=16, step_samples=1), None),
    "cornell_cfg": (lambda: W.cornell_box(128, 128),
                    dict(supersamples=8, min_samples=1, max_samples=16, step_samples=1), (3, 8)),
    "refcornell": (lambda: W.reference_cornell(160, 120),
                   dict(supersamples=4, min_samples=1, max_samples=64, step_samples=1), None),
}


def make_render(name):
    build, settings, cfg = RENDERS[name]
    sd, cam, _ = build()
    ref = O.Reference(cfg=cfg is not None)
    if cfg is not None:
        ref.set_depth_limits(*cfg)
    t0 = time.time()
    s, q, sec = ref.scene(sd, use_bvh=False).render_moments(cam, nthreads=os.cpu_count(), **settings)
    n = settings["max_samples"] * settings["supersamples"] ** 2
    mean = s / n
    var = np.maximum(q / n - mean * mean, 0.0) / n
    path = os.path.join(HERE, "render_%s.npz" % name)
    np.savez_compressed(path, digest=scene_digest(sd), mean=mean.astype(np.float16),
                        se=np.sqrt(var).astype(np.float16), n=n, width=cam.width, height=cam.height,
                        rr_min_depth=cfg[0] if cfg else 5, max_depth=cfg[1] if cfg else 0,
                        seconds=sec, **{k: v for k, v in settings.items()})
    print("%s: %dx%d, %d paths/pixel, %.1fs (%.2f Mpaths/s)" % (path, cam.width, cam.height, n, time.time() - t0,
                                                               cam.width * cam.height * n / sec / 1e6))


def make_rmse():
    sd, cam, _ = W.cornell_box(256, 256)
    ref = O.Reference(cfg=True)
    ref.set_depth_limits(3, 8)
    settings = dict(supersamples=8, min_samples=1, max_samples=256, step_samples=1)
    s, q, sec = ref.scene(sd, use_bvh=False).render_moments(cam, nthreads=os.cpu_count(), **settings)
    n = 256 * 64
    path = os.path.join(HERE, "rmse_cornell_cfg.npz")
    np.savez_compressed(path, digest=scene_digest(sd), mean=(s / n).astype(np.float32), n=n, seconds=sec,
                        rr_min_depth=3, max_depth=8, **settings)
    print("%s: %d spp, %.0fs" % (path, n, sec))


OBJ_TRANSFORM = dict(position=(10.0, -5.0, 3.0), scaling=(2.0, 1.0, 0.5), rotation=(0.3, -0.2, 0.7))


def make_obj():
    ref = O.Reference()
    path = os.path.join(HERE, "obj", "mesh.obj")
    out = {}
    for flip in (0, 1):
        tri, nrm, uv, mat = ref.load_obj(path, flip_v=bool(flip), **OBJ_TRANSFORM)
        out.update({"tri_%d" % flip: tri, "nrm_%d" % flip: nrm, "uv_%d" % flip: uv, "mat_%d" % flip: mat})
    dest = os.path.join(HERE, "obj_ref.npz")
    np.savez_compressed(dest, **out)
    print(dest, out["tri_0"].shape)


def make_scene():
    import tempfile
    sys.path.insert(0, os.path.join(HERE, "scene"))
    import cases
    ref = O.Reference()
    with tempfile.TemporaryDirectory() as td:
        rec, ibl = ref.load_scene_file(cases.stage_scene_dir(td))
        verdict = []
        for name in sorted(cases.CASES):
            r = ref.load_scene_file(cases.write(name, td))
            verdict.append(-1 if r is None else r[0].shape[0])
    dest = os.path.join(HERE, "scene_ref.npz")
    np.savez_compressed(dest, records=rec, ibl=ibl, case_names=np.array(sorted(cases.CASES)),
                        case_objects=np.array(verdict))
    print(dest, rec.shape, dict(zip(sorted(cases.CASES), verdict)))


def make_image_codec():
    import tempfile
    ref = O.Reference()
    rng = np.random.default_rng(21)
    n = 20000
    ldr = rng.uniform(-0.1, 1.2, (n, 3))
    ldr[:8] = [[0, 0, 0], [1, 1, 1], [0.5, 0.5, 0.5], [2, -1, 0.999999], [1e-9, 1e-5, 0.0039215],
               [0.99, 0.001, 0.2], [np.nextafter(1.0, 0), 0.25, 0.75], [0.0, 1.0, 0.5]]
    hdr = np.exp(rng.uniform(np.log(1e-6), np.log(1e6), (n, 3)))
    hdr[rng.random(n) < 0.05] = 0.0
    hdr[:6] = [[0, 0, 0], [1e-33, 1e-33, 1e-33], [1, 1, 1], [255.99, 0.5, 1e-3], [1e30, 1e29, 1], [0.5, 0.5, 0.5]]
    rgbe_in = rng.integers(0, 256, (n, 4), dtype=np.uint8)
    rgbe_in[:4, 3] = [0, 1, 128, 255]
    out = dict(ldr=ldr, rgb8_gamma=ref.encode_rgb8(ldr, True), rgb8_linear=ref.encode_rgb8(ldr, False),
               hdr=hdr, rgbe=ref.encode_rgbe(hdr), rgbe_in=rgbe_in, rgbe_decoded=ref.decode_rgbe(rgbe_in))
    with tempfile.TemporaryDirectory() as td:
        for name, (h, w) in (("rle", (23, 37)), ("flat", (4, 5))):
            img = np.exp(rng.uniform(np.log(1e-3), np.log(1e3), (h, w, 3)))
            img[::3] = img[::3, :1]  # constant rows: runs for the run-length encoder
            path = os.path.join(td, name + ".hdr")
            ref.write_hdr(path, img)
            out["hdr_%s_file" % name] = np.frombuffer(open(path, "rb").read(), np.uint8)
            out["hdr_%s_image" % name] = img
            out["hdr_%s_decoded" % name] = ref.read_hdr(path)
    path = os.path.join(HERE, "image_codec.npz")
    np.savez_compressed(path, **out)
    print(path)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--rmse", action="store_true")
    ap.add_argument("--only", default="")
    a = ap.parse_args()
    if not O.reference_available():
        O.build_oracle(reference=True)
    if a.rmse:
        make_rmse()
        sys.exit(0)
    if a.only == "image_codec":
        make_image_codec()
        sys.exit(0)
    if a.only == "obj":
        make_obj()
        sys.exit(0)
    if a.only == "scene":
        make_scene()
        sys.exit(0)
    make_image_codec()
    make_obj()
    make_scene()
    for nm in CLOSEST_SCENES:
        if not a.only or a.only == nm:
            make_closest(nm)
    for nm in RENDERS:
        if not a.only or a.only == nm:
            make_render(nm)
