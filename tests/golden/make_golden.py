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
  rmse_mesh.npz, rmse_terrain.npz, rmse_batched_job0.npz
                        (--only rmse_mesh / rmse_terrain / rmse_batched_job0) 16384-spp
                        FP64 oracle renders of five 32x32 tiles of the mesh and
                        terrain workloads and of the batched workload's first job
                        (their own sub-pixel grids), the RMSE targets of those
                        workloads
  obj_ref.npz           the reference's Model::ReadFromObj + Transform of
                        tests/golden/obj/mesh.obj (with and without the v flip)
  image_codec.npz       the reference's 8-bit conversion (gamma on and off),
                        Color2RGBE and RGBE2Color on seeded colours and bytes,
                        and two .hdr files its writer produced (one run-length
                        encoded, one flat) with what its reader decodes
  ibl_ref.npz           the reference's IBL::Sample(dir) on seeded directions
                        (z < 0, the x axis, near the poles, on texel lines) over
                        two index-coded equirect maps: the texel each one reads
  texel_ref.npz         the reference's Image::GetPixelByUV on the textured
                        scene's textures at seeded and edge (u, v)
  render_textured.npz   the reference's render of the textured scene (no
                        noise: per-pixel means in float32)
  render_lens_*.npz     the Cornell box through the reference's thin lens
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
    # thin lens: the reference main()'s CircleAperture(1.3) at focal distance
    # 300, and a strong depth of field (radius 20, focal plane at the box's
    # front z = 100: the spheres blur over ~5 pixels, the back wall over ~9)
    "lens_main": (lambda: W.cornell_lens(128, 128, 1.3, 300.0),
                  dict(supersamples=4, min_samples=1, max_samples=64, step_samples=1), None),
    "lens_dof": (lambda: W.cornell_lens(128, 128, 20.0, 150.0),
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
                        aperture=cam.aperture_radius, focal=cam.focal_distance,
                        seconds=sec, **{k: v for k, v in settings.items()})
    print("%s: %dx%d, %d paths/pixel, %.1fs (%.2f Mpaths/s)" % (path, cam.width, cam.height, n, time.time() - t0,
                                                               cam.width * cam.height * n / sec / 1e6))


def make_textured():
    """The reference's render of the textured scene.  Every path's radiance is
    colour x texel (no noise), so the per-pixel means are stored in float32 and
    compared by value."""
    sd, cam, st = W.textured_scene()
    ref = O.Reference()
    s, q, sec = ref.scene(sd, use_bvh=False).render_moments(cam, nthreads=os.cpu_count(), **st)
    n = st["supersamples"] ** 2 * st["max_samples"]
    path = os.path.join(HERE, "render_textured.npz")
    np.savez_compressed(path, digest=scene_digest(sd), mean=(s / n).astype(np.float32), n=n,
                        width=cam.width, height=cam.height, **st)
    print(path)


def _unit_f32(v):
    v = np.asarray(v, np.float64)
    v = v / np.linalg.norm(v, axis=1, keepdims=True)
    return v.astype(np.float32).astype(np.float64)


IBL_SIZES = ((64, 32), (37, 19))


def ibl_scene(w, h):
    """A scene with only an index-coded equirect map: texel (x, y) holds
    (x, y, y * w + x), so a lookup's colour names the texel it read."""
    sd = W.SceneDesc()
    m = sd.material(W.abi.OR3_LAMBERT, (0.5, 0.5, 0.5))
    sd.add_sphere((0.0, 0.0, 0.0), 1.0, sd.layers(m))
    yy, xx = np.mgrid[0:h, 0:w]
    sd.set_env(np.stack([xx, yy, yy * w + xx], axis=-1).astype(np.float32))
    return sd


def ibl_directions(seed=31):
    """Seeded unit directions (FP32 values): uniform on the sphere, the z < 0
    half and z = -0.0 (IBL::Sample mirrors phi there), the x axis (phi = 0 and
    pi), near-pole directions, and directions on the texel grid's phi and
    theta lines.  The exact poles are left out: there the reference takes
    acos(0 / 0) and converts the NaN to int, which has no defined value."""
    rng = np.random.default_rng(seed)
    d = [rng.normal(size=(3000, 3))]
    z = rng.normal(size=(500, 3))
    z[:, 2] = -np.abs(z[:, 2])
    d.append(z)
    special = [[1, 0, 0], [-1, 0, 0], [1, 0, -0.0], [-1, 0, -0.0], [0, 0, 1], [0, 0, -1], [1, 1, 0], [1, -1, 0],
               [1, 0.5, -1e-6], [1, 0.5, 1e-6], [-1, 0.5, -1e-6], [-1, -0.5, 1e-6]]
    for e in (1e-3, 1e-4, 1e-5):
        for sy in (1, -1):
            for ang in (0.3, 2.0, 4.0, 5.5):
                special.append([e * np.cos(ang), sy, e * np.sin(ang)])
    d.append(np.asarray(special, np.float64))
    for w, h in IBL_SIZES:  # on phi = 2 pi k / w and theta = pi j / h
        k = np.arange(w)
        ph = 2 * np.pi * k / w
        d.append(np.stack([np.cos(ph) * 0.8, np.full(w, 0.3), np.sin(ph) * 0.8], axis=1))
        j = np.arange(1, h)
        th = np.pi * j / h
        d.append(np.stack([np.sin(th) * 0.6, np.cos(th), np.sin(th) * 0.8], axis=1))
    return _unit_f32(np.concatenate(d))  # the z = -0.0 entries keep their sign


def make_ibl():
    """IBL::Sample(dir) of the reference on index-coded maps of two sizes."""
    ref = O.Reference()
    dirs = ibl_directions()
    out = dict(dirs=dirs.astype(np.float32), sizes=np.asarray(IBL_SIZES, np.int32))
    for w, h in IBL_SIZES:
        c = ref.scene(ibl_scene(w, h), use_bvh=False).ibl_sample(dirs)
        out["texel_%dx%d" % (w, h)] = c[:, :2].astype(np.int32)
        assert np.all(c[:, 2] == c[:, 1] * w + c[:, 0])
    path = os.path.join(HERE, "ibl_ref.npz")
    np.savez_compressed(path, **out)
    print(path, dirs.shape)


def texel_uvs(tex, seed=32):
    """(u, v) pairs: seeded over [-0.3, 1.3]^2 (the clamp), the corners and
    edges 0 and 1 (the x0.99999 rule keeps 1 on the last texel), and the
    texel grid's lines k / w, k / h."""
    rng = np.random.default_rng(seed)
    h, w = tex.shape[:2]
    uv = [rng.uniform(-0.3, 1.3, (3000, 2))]
    e = np.array([0.0, 1.0, np.float32(1.0 - 2.0 ** -24), 1e-7, -0.0])
    uv.append(np.stack(np.meshgrid(e, e), axis=-1).reshape(-1, 2))
    ku = np.arange(w + 1) / w
    kv = np.arange(h + 1) / h
    uv.append(np.stack([ku, np.full(w + 1, 0.37)], axis=1))
    uv.append(np.stack([np.full(h + 1, 0.61), kv], axis=1))
    return np.concatenate(uv).astype(np.float32).astype(np.float64)


def make_texel():
    """Image::GetPixelByUV of the reference on the textured scene's two textures."""
    ref = O.Reference()
    sd, _, _ = W.textured_scene()
    rs = ref.scene(sd, use_bvh=False)
    out = dict(digest=scene_digest(sd))
    for t, tex in enumerate(sd.textures):
        uv = texel_uvs(tex, seed=32 + t)
        out["uv_%d" % t] = uv.astype(np.float32)
        out["rgb_%d" % t] = rs.texel(t, uv).astype(np.float32)
    path = os.path.join(HERE, "texel_ref.npz")
    np.savez_compressed(path, **out)
    print(path)


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


# 16384-spp references of the benchmark workloads, on five 32x32 tiles (the
# four quadrant centres and the image centre), with the workload's own
# sub-pixel grid (the estimator converges to the grid-sampled pixel), from the
# FP64 C oracle: the mesh's Phong lobe and the terrain's light sampling have
# no counterpart in the reference, and the oracle is pinned to the reference
# wherever they overlap.
RMSE_CONFIGS = {"mesh": lambda: W.icosphere_in_box(), "terrain": lambda: W.terrain_ibl(),
                # the batched workload's first job (1.31M-triangle icosphere in the box, NEE)
                "batched_job0": lambda: W.batched_jobs(n=1)[0]}
RMSE_SEED = 0x5EED16


def rmse_tiles(width, height, size=32):
    cs = [(width // 4, height // 4), (3 * width // 4, height // 4), (width // 4, 3 * height // 4),
          (3 * width // 4, 3 * height // 4), (width // 2, height // 2)]
    return np.asarray([(cx - size // 2, cy - size // 2, size, size) for cx, cy in cs], np.int32)


def make_rmse_config(name, spp=16384):
    """Tiles (x0, y0 in camera rows counted from the bottom, w, h) of the
    workload rendered at `spp` samples per pixel: per-pixel FP64 means and
    standard errors, rows of each tile bottom-up."""
    sd, cam, st = RMSE_CONFIGS[name]()
    orc = O.CRestatement()
    scene = orc.scene(sd, use_bvh=True)
    ss2 = st["supersamples"] ** 2
    samples = spp // ss2
    kw = dict(supersamples=st["supersamples"], min_samples=1, max_samples=samples, step_samples=samples,
              rr_min_depth=st["rr_min_depth"], max_depth=st["max_depth"], seed=RMSE_SEED,
              next_event_estimation=st.get("next_event_estimation", False))
    tiles = rmse_tiles(cam.width, cam.height)
    S = np.zeros((len(tiles), 32, 32, 3))
    Q = np.zeros_like(S)
    t0 = time.time()
    for k, (x0, y0, w, h) in enumerate(tiles.tolist()):  # Python ints: path indices pass 2^31
        for j in range(h):
            for s_ in range(samples):
                g = ((s_ * cam.height + y0 + j) * cam.width + x0) * ss2
                r = scene.path_radiance(cam, g, w * ss2, nthreads=os.cpu_count(), **kw).reshape(w, ss2, 3)
                S[k, j] += r.sum(axis=1)
                Q[k, j] += (r * r).sum(axis=1)
    sec = time.time() - t0
    n = samples * ss2
    mean = S / n
    se = np.sqrt(np.maximum(Q / n - mean * mean, 0.0) / n)
    path = os.path.join(HERE, "rmse_%s.npz" % name)
    np.savez_compressed(path, digest=scene_digest(sd), tiles=tiles, mean=mean.astype(np.float32),
                        se=se.astype(np.float32), n=n, seconds=sec, seed=RMSE_SEED, width=cam.width,
                        height=cam.height, **{k: v for k, v in kw.items() if k != "seed"})
    print("%s: %d tiles, %d spp, %.0fs" % (path, len(tiles), n, sec))


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
    if a.only.startswith("rmse_"):
        make_rmse_config(a.only[5:])
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
    if a.only == "lookups":
        make_ibl()
        make_texel()
        make_textured()
        sys.exit(0)
    if not a.only:
        make_image_codec()
        make_obj()
        make_scene()
        make_ibl()
        make_texel()
        make_textured()
    for nm in CLOSEST_SCENES:
        if not a.only or a.only == nm:
            make_closest(nm)
    for nm in RENDERS:
        if not a.only or a.only == nm:
            make_render(nm)
