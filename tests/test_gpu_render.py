"""GPU render parity through the C ABI (or3_render).

Two bars:
  * path by path against the C oracle, which replays the same counter-based
    random numbers in FP64: a path's radiance must agree to 1e-3 relative
    unless FP32 rounding flipped one of its discrete decisions (Russian
    roulette, layer choice, a grazing hit); at most 1% of paths may differ;
  * per pixel against the reference's own renders (golden fixtures): two-sample
    z within 3 standard errors (see conftest.zscores), and image RMSE against
    the 16384-spp reference render consistent with the GPU's own noise.
"""
import os
import threading

import numpy as np
import pytest

from conftest import GOLDEN, golden, moments_to_mean_se, zscores

pytestmark = pytest.mark.gpu


def _path_parity(pkg, ctx, orc, sd, cam, use_bvh=True, **settings):
    sid = ctx.upload(sd)
    try:
        ctx.render(sid, cam, flags=pkg.abi.OR3_FLAG_KEEP_PATHS, **settings)
        gpu = ctx.path_radiance().astype(np.float64)
    finally:
        ctx.release(sid)
    ref = orc.scene(sd, use_bvh=use_bvh).path_radiance(cam, 0, gpu.shape[0], **settings)
    close = (np.abs(gpu - ref) <= 1e-3 * (1.0 + np.abs(ref))).all(axis=1)
    return gpu, ref, close


@pytest.mark.parametrize("case", ["cornell", "cornell_refdepth", "refcornell", "ico_phong", "terrain_env",
                                  "cornell_lens", "textured"])
def test_paths_match_oracle(pkg, ctx, orc, case):
    W = pkg.workloads
    if case == "cornell":
        sd, cam, _ = W.cornell_box(48, 48)
        st = dict(supersamples=4, rr_min_depth=3, max_depth=8)
    elif case == "cornell_refdepth":
        sd, cam, _ = W.cornell_box(48, 48)
        st = dict(supersamples=4, rr_min_depth=5, max_depth=0)
    elif case == "refcornell":
        sd, cam, _ = W.reference_cornell(64, 48)
        st = dict(supersamples=4, rr_min_depth=5, max_depth=0)
    elif case == "cornell_lens":
        sd, cam, _ = W.cornell_lens(48, 48, 20.0, 150.0)
        st = dict(supersamples=4, rr_min_depth=5, max_depth=0)
    elif case == "textured":
        sd, cam, _ = W.textured_scene(48, 32)
        st = dict(supersamples=4, rr_min_depth=5, max_depth=0)
    elif case == "ico_phong":
        sd, cam, _ = W.icosphere_in_box(64, 48, level=4)
        st = dict(supersamples=4, rr_min_depth=5, max_depth=10)
    else:
        sd, cam, _ = W.terrain_ibl(64, 36, cells_x=64, cells_z=32, spheres=16)
        st = dict(supersamples=4, rr_min_depth=5, max_depth=12)
    gpu, ref, close = _path_parity(pkg, ctx, orc, sd, cam, seed=1234, min_samples=1, max_samples=1,
                                   step_samples=1, **st)
    assert gpu.shape[0] == cam.width * cam.height * st["supersamples"] ** 2
    assert np.isfinite(gpu).all()
    assert close.mean() >= 0.99, close.mean()
    # the few paths that diverge do not bias the image
    mg, mr = gpu.mean(), ref.mean()
    assert abs(mg - mr) <= 0.02 * max(mr, 1e-3) + 3 * gpu.std() / np.sqrt(len(gpu)), (mg, mr)


RENDERS = [
    ("render_cornell_ref.npz", lambda W: W.cornell_box(256, 256), 64, dict(rr_min_depth=5, max_depth=0)),
    ("render_cornell_cfg.npz", lambda W: W.cornell_box(128, 128), 64, dict(rr_min_depth=3, max_depth=8)),
    ("render_refcornell.npz", lambda W: W.reference_cornell(160, 120), 64, dict(rr_min_depth=5, max_depth=0)),
]


@pytest.mark.parametrize("fixture,build,samples,depth", RENDERS)
def test_render_statistically_matches_reference(pkg, ctx, fixture, build, samples, depth):
    g = golden(fixture)
    sd, cam, _ = build(pkg.workloads)
    assert sd.digest() == str(g["digest"])
    ss = int(g["supersamples"])
    sid = ctx.upload(sd)
    try:
        ctx.render(sid, cam, supersamples=ss, min_samples=samples, max_samples=samples, step_samples=1, seed=77,
                   **depth)
        s, q, n = ctx.moments(cam.width, cam.height)
    finally:
        ctx.release(sid)
    assert n == samples * ss * ss
    m, se = moments_to_mean_se(s, q, n)
    z = zscores(m, se, n, g["mean"], g["se"], int(g["n"]))
    assert np.mean(np.abs(z) > 3) < 0.01, np.mean(np.abs(z) > 3)
    assert abs(z.mean()) < 0.05, z.mean()
    assert 0.8 < z.var() < 1.25, z.var()
    gm = g["mean"].astype(np.float64).mean()
    assert abs(m.mean() - gm) / gm < 0.01


@pytest.mark.skipif(not os.path.exists(os.path.join(GOLDEN, "rmse_cornell_cfg.npz")), reason="no RMSE fixture")
def test_rmse_against_16k_reference(pkg, ctx):
    g = golden("rmse_cornell_cfg.npz")
    sd, cam, st = pkg.workloads.cornell_box(256, 256)
    assert sd.digest() == str(g["digest"])
    sid = ctx.upload(sd)
    ctx.render(sid, cam, supersamples=8, min_samples=1, max_samples=1, rr_min_depth=3, max_depth=8, seed=5)
    s, q, n = ctx.moments(cam.width, cam.height)
    ctx.release(sid)
    m, se = moments_to_mean_se(s, q, n)
    rmse = np.sqrt(np.mean((m - g["mean"]) ** 2))
    # expected from the GPU's own noise plus the reference render's (n = 16384)
    expect = np.sqrt(np.mean(se ** 2) * (1.0 + n / float(g["n"])))
    assert rmse < 1.1 * expect, (rmse, expect)
    assert rmse > 0.5 * expect, (rmse, expect)


def tile_rmse(fixture, m, se):
    """RMSE of image moments (rows top-down) against a tiled 16384-spp
    reference (tile rows counted from the bottom, as camera rows), and the
    RMSE the two renders' own noise predicts."""
    H = m.shape[0]
    d2, v = [], []
    for k, (x0, y0, w, h) in enumerate(fixture["tiles"].tolist()):
        rows = H - 1 - (y0 + np.arange(h))
        d2.append((m[rows, x0:x0 + w] - fixture["mean"][k]) ** 2)
        v.append(se[rows, x0:x0 + w] ** 2 + fixture["se"][k].astype(np.float64) ** 2)
    return float(np.sqrt(np.mean(d2))), float(np.sqrt(np.mean(v)))


@pytest.mark.parametrize("name", ["mesh", "terrain", "batched_job0"])
def test_rmse_of_benchmark_workloads_against_16k_oracle(pkg, ctx, name):
    # the full benchmark render (its resolution, sub-pixel grid, depth and
    # light sampling) against the FP64 oracle's 16384-spp tiles; batched_job0
    # is the batched workload's first job, rendered plainly (a batch renders
    # the same paths)
    g = golden("rmse_%s.npz" % name)
    W = pkg.workloads
    sd, cam, st = {"mesh": W.icosphere_in_box, "terrain": W.terrain_ibl,
                   "batched_job0": lambda: W.batched_jobs(n=1)[0]}[name]()
    assert sd.digest() == str(g["digest"])
    assert (int(g["width"]), int(g["height"]), int(g["supersamples"])) == (cam.width, cam.height,
                                                                           st["supersamples"])
    sid = ctx.upload(sd)
    try:
        ctx.render(sid, cam, **dict(st, seed=7))
        s, q, n = ctx.moments(cam.width, cam.height)
    finally:
        ctx.release(sid)
    m, se = moments_to_mean_se(s, q, n)
    rmse, expect = tile_rmse(g, m, se)
    assert 0.7 * expect < rmse < 1.3 * expect, (rmse, expect)


def test_frame_layout_and_progressive_callbacks(pkg, ctx):
    sd, cam, _ = pkg.workloads.cornell_box(40, 24)
    sid = ctx.upload(sd)
    frames = []
    ctx.render(sid, cam, supersamples=2, min_samples=1, max_samples=7, step_samples=3, seed=3,
               callback=lambda s, img, w, h, mins: frames.append((s, img, w, h)))
    last, samples = ctx.frame(cam.width, cam.height)
    s, q, n = ctx.moments(cam.width, cam.height)
    ctx.release(sid)
    assert [f[0] for f in frames] == [1, 4, 7]  # PathTracer's pass schedule min..max step
    for f in frames:
        assert f[2] == 2 * cam.width and f[3] == cam.height
        assert np.all(f[1][:, cam.width:] == 0)  # right viewport stays empty
    assert samples == 7
    np.testing.assert_array_equal(last, frames[-1][1])
    # frame rows are top-down (ScreenPixels flips y): equal to the moments' mean
    np.testing.assert_allclose(last[:, :cam.width], s / n, rtol=1e-12, atol=0)
    assert n == 7 * 4


def test_frame_into_the_callers_buffer(pkg, ctx):
    sd, cam, _ = pkg.workloads.cornell_box(16, 12)
    sid = ctx.upload(sd)
    ctx.render(sid, cam, supersamples=2, seed=3)
    ctx.release(sid)
    ref, n = ctx.frame(cam.width, cam.height)
    buf = np.full((cam.height, 2 * cam.width, 3), -1.0)
    out, n2 = ctx.frame(cam.width, cam.height, out=buf)
    assert out is buf and n2 == n
    np.testing.assert_array_equal(buf, ref)
    with pytest.raises(ValueError):
        ctx.frame(cam.width, cam.height, out=np.zeros((cam.height, cam.width, 3)))


def test_compact_layout(pkg, ctx):
    sd, cam, _ = pkg.workloads.cornell_box(20, 10)
    sid = ctx.upload(sd)
    ctx.render(sid, cam, supersamples=1, seed=1, layout=pkg.abi.OR3_LAYOUT_COMPACT)
    img, _ = ctx.frame(cam.width, cam.height, layout=pkg.abi.OR3_LAYOUT_COMPACT)
    ctx.release(sid)
    assert img.shape == (10, 20, 3) and img.sum() > 0


@pytest.mark.parametrize("max_depth,wave_paths", [(0, 0), (8, 2000), (0, 2000)])
def test_stop_rendering_from_another_thread(pkg, ctx, max_depth, wave_paths):
    """wave_paths 2000: many small waves per pass on the three wave lanes."""
    sd, cam, _ = pkg.workloads.cornell_box(64, 64)
    sid = ctx.upload(sd)
    seen = []

    def cb(samples, img, w, h, minutes):
        seen.append(samples)
        if samples >= 2:
            threading.Thread(target=ctx.stop).start()
            threading.Event().wait(0.2)

    ctx.render(sid, cam, supersamples=2, min_samples=1, max_samples=1000, step_samples=1, seed=2, callback=cb,
               max_depth=max_depth, wave_paths=wave_paths)
    ctx.reset_stop()
    _, samples = ctx.frame(cam.width, cam.height)
    ctx.release(sid)
    assert 2 <= len(seen) < 1000
    assert samples == seen[-1]


def test_waves_do_not_change_the_image(pkg, ctx):
    sd, cam, _ = pkg.workloads.icosphere_in_box(48, 32, level=3)
    sid = ctx.upload(sd)
    ctx.render(sid, cam, supersamples=4, min_samples=3, max_samples=3, seed=9, max_depth=10)
    s1, q1, _ = ctx.moments(cam.width, cam.height)
    ctx.render(sid, cam, supersamples=4, min_samples=3, max_samples=3, seed=9, max_depth=10, wave_paths=1000)
    s2, q2, _ = ctx.moments(cam.width, cam.height)
    st = ctx.stats()
    ctx.release(sid)
    assert st["waves"] > 10
    np.testing.assert_allclose(s1, s2, rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("nee,tuning,depth", [(False, 0, 8), (True, 0, 8), (True, 0x200, 8), (True, 0x400, 8),
                                              (False, 0, 0), (True, 0, 0)])
def test_wave_lanes_match_one(pkg, ctx, nee, tuning, depth):
    """Waves run round robin on three (two: 0x200, four: 0x400) streams with their own
    queues and pixel sums, merged at the end of each pass: the image, the moments and the ray counts
    equal the one-stream render's (up to the order of float additions: FP64
    pixel sums, and FP32 atomics of light samples into a path's radiance)."""
    sd, cam = pkg.workloads.sky_floor(48, 32) if nee else pkg.workloads.icosphere_in_box(48, 32, level=3)[:2]
    sid = ctx.upload(sd)
    # depth 0: the reference's rules (Russian roulette only), each lane's live
    # count read back per chunk of bounces
    kw = dict(supersamples=4, min_samples=2, max_samples=6, step_samples=2, seed=5, max_depth=depth,
              wave_paths=3000, next_event_estimation=nee)
    try:
        s2 = ctx.render(sid, cam, tuning=tuning, **kw)
        f2, n2 = ctx.frame(cam.width, cam.height)
        m2 = ctx.moments(cam.width, cam.height)
        s1 = ctx.render(sid, cam, tuning=pkg.abi.OR3_TUNE_ONE_LANE, **kw)
        f1, n1 = ctx.frame(cam.width, cam.height)
        m1 = ctx.moments(cam.width, cam.height)
    finally:
        ctx.release(sid)
    assert s2["waves"] > 10 and n1 == n2 == 6
    assert s1["lanes"] == 1 and s2["lanes"] == {0: 3, 0x200: 2, 0x400: 4}[tuning]
    for k in ("extension_rays", "shadow_rays", "camera_paths"):
        assert s1[k] == s2[k], k
    np.testing.assert_allclose(f2, f1, rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(m2[0], m1[0], rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(m2[1], m1[1], rtol=1e-5, atol=1e-7)
    assert f1.sum() > 0


@pytest.mark.parametrize("depth,wave", [(8, 2048), (0, 2048), (8, 32768)])
def test_split_overflow_renders_waves_again(pkg, ctx, depth, wave):
    """Where glass can split paths the ray queues hold two rays per camera
    path of a wave.  Here a glass sphere in front of the camera fills the
    view: every camera ray splits on entry (depth 0), its refracted ray on
    the far side (depth 1) and the internal reflection again (depth 2), so
    the depth-3 bounce holds three rays per path.  Those waves are not
    accumulated and are rendered again in sub-waves that cannot overflow.
    The image equals a render whose queues no split can overflow
    (OR3_FLAG_KEEP_PATHS keeps eight rays per path), up to the order of
    float additions, and the scene's next render, with its queue factor
    doubled, overflows no wave."""
    A = pkg.abi
    sd, cam, _ = pkg.workloads.cornell_box(48, 36)
    glass = sd.material(A.OR3_REFRACTION, (0.99, 0.99, 0.99), ior=1.5)
    sd.add_sphere((50.0, 50.0, 150.0), 60.0, sd.layers(glass))  # the camera is at z = 250, 100 from its centre
    sid = ctx.upload(sd)
    # wave 2048: passes of one sample in row chunks; 32768: one pass of three
    # samples in one wave (re-rendered one sample at a time)
    kw = dict(supersamples=2, min_samples=1 if wave == 2048 else 3, max_samples=3, step_samples=1, seed=3,
              rr_min_depth=3, max_depth=depth, wave_paths=wave)
    try:
        s_opt = ctx.render(sid, cam, **kw)
        f_opt, n_opt = ctx.frame(cam.width, cam.height)
        m_opt = ctx.moments(cam.width, cam.height)
        s_safe = ctx.render(sid, cam, flags=A.OR3_FLAG_KEEP_PATHS, **kw)
        f_safe, n_safe = ctx.frame(cam.width, cam.height)
        m_safe = ctx.moments(cam.width, cam.height)
        # the overflow doubled the scene's queue factor: its next render fits
        s_again = ctx.render(sid, cam, **kw)
        m_again = ctx.moments(cam.width, cam.height)
    finally:
        ctx.release(sid)
    assert s_opt["waves_rerun"] > 0 and s_safe["waves_rerun"] == 0 and s_again["waves_rerun"] == 0
    np.testing.assert_allclose(m_again[0], m_safe[0], rtol=1e-5, atol=1e-7)
    assert n_opt == n_safe == 3 and s_opt["camera_paths"] == s_safe["camera_paths"]
    np.testing.assert_allclose(m_opt[0], m_safe[0], rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(m_opt[1], m_safe[1], rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(f_opt, f_safe, rtol=1e-5, atol=1e-7)
    assert f_opt.sum() > 0


def test_lanes_fall_back_when_device_memory_is_short(pkg, ctx):
    """When another lane's queues do not fit, the render uses the lanes that do
    (same image) instead of failing."""
    torch = pytest.importorskip("torch")
    sd, cam = pkg.workloads.icosphere_in_box(256, 192, level=3)[:2]
    kw = dict(supersamples=8, min_samples=4, max_samples=4, seed=2, max_depth=8, wave_paths=1 << 22)
    filler = None
    with pkg.Context(0) as c2:  # a fresh context: its extra lanes are not allocated yet
        sid = c2.upload(sd)
        try:
            c2.render(sid, cam, tuning=pkg.abi.OR3_TUNE_ONE_LANE, **kw)
            f1 = c2.frame(cam.width, cam.height)[0]
            wave = cam.width * cam.height * 64  # one sample of the image per wave
            lane = 16 * 11 * wave  # ten ray arrays and pathL of one lane, float4 each
            free = torch.cuda.mem_get_info(0)[0]
            keep = int(0.5 * lane) + (256 << 20)  # not room for the two extra lanes
            if free <= keep:
                pytest.skip("device memory already short")
            filler = torch.empty(free - keep, dtype=torch.uint8, device="cuda:0")
            s = c2.render(sid, cam, **kw)  # three lanes wanted
            f2 = c2.frame(cam.width, cam.height)[0]
        finally:
            del filler
            torch.cuda.empty_cache()
            c2.release(sid)
    # (the CUDA driver may find room for one extra lane by trimming its own pools)
    assert s["waves"] >= 4 and s["lanes"] < 3, s["lanes"]
    np.testing.assert_allclose(f2, f1, rtol=1e-5, atol=1e-7)


def test_invalid_arguments_are_reported(pkg, ctx):
    sd, cam, _ = pkg.workloads.cornell_box(8, 8)
    sid = ctx.upload(sd)
    for bad in (dict(supersamples=0), dict(min_samples=0), dict(min_samples=3, max_samples=2),
                dict(step_samples=0), dict(layout=7)):
        with pytest.raises(pkg.Or3Error) as e:
            ctx.render(sid, cam, **bad)
        assert e.value.code == pkg.abi.OR3_ERR_INVALID_ARGUMENT
    ctx.release(sid)
    bad_scene = pkg.SceneDesc()
    m = bad_scene.material(pkg.abi.OR3_LAMBERT, (1, 1, 1))
    bad_scene.add_sphere((0, 0, 0), -1.0, bad_scene.layers(m))
    with pytest.raises(pkg.Or3Error):
        ctx.upload(bad_scene)


def test_gpu_path_tracer_mirror(pkg):
    """The Renderer-interface mirror renders progressively and exposes GetResult."""
    sd, cam, _ = pkg.workloads.cornell_box(32, 32)
    got = []
    pt = pkg.GpuPathTracer(cam, 1, 3, 1, 2, callback=lambda s, img, w, h, m: got.append(s))
    pt.EnableNextEventEstimation(False)
    pt.SetMaxThreadCount(4)
    pt.RenderScene(sd)
    assert got == [1, 2, 3]
    assert pt.GetCurrentSampleCount() == 3
    r = pt.GetResult()
    assert r.CalcScreenWidth() == 64 and r.CalcScreenHeight() == 32
    assert "samples" in pt.GetCurrentRenderingInfo()
