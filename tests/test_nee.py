"""Next-event estimation (light sampling with any-hit shadow rays).

The reference's own NEE cannot be a pin: DirectRadiance_Lambert weights the
light sample by the receiving surface's emission (src/renderer/PathTracer.cpp:
311-314), which is zero wherever it is called, so its NEE renders black.  What
pins the estimator instead:

  * on the CPU, the oracle's NEE estimator and its BSDF-only estimator (the
    reference's, pinned against the reference's compiled code elsewhere) must
    agree in expectation on the same scene -- emissive triangles, a sphere
    light with a Phong receiver, an equirect sky through its CDF, a constant
    background -- and NEE must cut the noise where lights are small;
  * on the GPU, every path's radiance must match the oracle's FP64 replay of
    the same random numbers (at most 1% of paths may differ), the GPU's NEE
    and BSDF-only renders must agree statistically, and the batched form must
    give a NEE job the same sums as a plain render.
"""
import numpy as np
import pytest


def _scenes(W):
    return {
        "cornell_triangle_light": (W.cornell_box(32, 32)[:2], dict(rr_min_depth=3, max_depth=8)),
        "cornell_reference_depth": (W.cornell_box(32, 32)[:2], dict(rr_min_depth=5, max_depth=0)),
        "sphere_light_phong": (W.sphere_light_box(32, 32), dict(rr_min_depth=3, max_depth=8)),
        "sky_env_cdf": (W.sky_floor(32, 32), dict(rr_min_depth=3, max_depth=6)),
        "constant_background": (W.sky_floor(32, 32, constant=(0.8, 0.9, 1.0)), dict(rr_min_depth=3, max_depth=6)),
    }


NAMES = ["cornell_triangle_light", "cornell_reference_depth", "sphere_light_phong", "sky_env_cdf",
         "constant_background"]
# scenes whose light is small enough that one light sample per vertex must beat BSDF sampling
SMALL_LIGHTS = {"cornell_triangle_light", "cornell_reference_depth", "sphere_light_phong", "sky_env_cdf"}


def block_z(a, b, k=4):
    """z of two estimates of the same image, over k x k pixel blocks.

    a, b: (sum, sum of squares, paths per pixel).  Blocks average out the
    heavy per-pixel tails of the BSDF-only estimator (rare light hits), for
    which a per-pixel sample variance is unreliable at test sample counts.
    """
    (s1, q1, n1), (s2, q2, n2) = a, b
    H, W_, _ = s1.shape

    def agg(x):
        return x[:H // k * k, :W_ // k * k].reshape(H // k, k, W_ // k, k, 3).sum(axis=(1, 3))

    m1, m2 = s1 / n1, s2 / n2
    v1 = np.maximum(q1 / n1 - m1 ** 2, 0) / n1
    v2 = np.maximum(q2 / n2 - m2 ** 2, 0) / n2
    M1, M2, V = agg(m1), agg(m2), agg(v1) + agg(v2)
    return (M1 - M2) / np.sqrt(V + (1e-3 * (np.abs(M1) + np.abs(M2))) ** 2 + 1e-30)


def mean_se(r):
    s, q, n = r
    return float(np.sqrt(np.maximum(q / n - (s / n) ** 2, 0) / n).mean())


@pytest.mark.parametrize("name", NAMES)
def test_oracle_nee_has_the_bsdf_estimators_expectation(pkg, orc, name):
    (sd, cam), st = _scenes(pkg.workloads)[name]
    sc = orc.scene(sd)
    spp = 500
    res = []
    for nee in (False, True):
        s, q, _ = sc.render(cam, supersamples=2, min_samples=spp, max_samples=spp, next_event_estimation=nee,
                            seed=9, **st)
        res.append((s, q, 4 * spp))
    z = block_z(res[0], res[1])
    assert np.abs(z).max() < 4.5, np.abs(z).max()
    assert (np.abs(z) > 3).mean() <= 0.02
    if name in SMALL_LIGHTS:
        assert mean_se(res[1]) < 0.6 * mean_se(res[0])


# ---------------------------------------------------------------- GPU

@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_nee_paths_match_oracle(pkg, ctx, orc, name):
    (sd, cam), st = _scenes(pkg.workloads)[name]
    settings = dict(supersamples=4, min_samples=2, max_samples=2, step_samples=1, seed=4321,
                    next_event_estimation=True, **st)
    sid = ctx.upload(sd)
    try:
        stats = ctx.render(sid, cam, flags=pkg.abi.OR3_FLAG_KEEP_PATHS, **settings)
        gpu = ctx.path_radiance().astype(np.float64)
        assert ctx.scene_info(sid)["num_lights"] == (0 if name.startswith(("sky", "constant")) else
                                                    (1 if name == "sphere_light_phong" else 2))
    finally:
        ctx.release(sid)
    assert stats["shadow_rays"] > 0
    ref = orc.scene(sd).path_radiance(cam, 0, gpu.shape[0], **settings)
    assert np.isfinite(gpu).all()
    close = (np.abs(gpu - ref) <= 1e-3 * (1.0 + np.abs(ref))).all(axis=1)
    assert close.mean() >= 0.99, close.mean()
    mg, mr = gpu.mean(), ref.mean()
    assert abs(mg - mr) <= 0.02 * max(mr, 1e-3) + 3 * gpu.std() / np.sqrt(len(gpu)), (mg, mr)


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_nee_and_bsdf_renders_agree(pkg, ctx, name):
    (sd, cam), st = _scenes(pkg.workloads)[name]
    sid = ctx.upload(sd)
    res = []
    try:
        for nee in (False, True):
            stats = ctx.render(sid, cam, supersamples=4, min_samples=256, max_samples=256, step_samples=1, seed=21,
                               next_event_estimation=nee, **st)
            assert (stats["shadow_rays"] > 0) == nee
            res.append(ctx.moments(cam.width, cam.height))
    finally:
        ctx.release(sid)
    z = block_z(res[0], res[1])
    assert np.abs(z).max() < 4.5, np.abs(z).max()
    assert (np.abs(z) > 3).mean() <= 0.02
    if name in SMALL_LIGHTS:
        assert mean_se(res[1]) < 0.6 * mean_se(res[0])


@pytest.mark.gpu
def test_nee_batch_jobs_equal_plain_renders(pkg, ctx):
    W = pkg.workloads
    scenes = [W.cornell_box(24, 20)[:2], W.sphere_light_box(20, 24), W.sky_floor(28, 16)]
    sids = [ctx.upload(sd) for sd, _ in scenes]
    try:
        jobs = [(sids[k], scenes[k][1], dict(supersamples=2, min_samples=2, max_samples=4, step_samples=2,
                                             rr_min_depth=3, max_depth=8, seed=50 + k,
                                             next_event_estimation=(k != 1)))
                for k in range(3)]
        alone = []
        for sid, cam, st in jobs:
            ctx.render(sid, cam, **st)
            alone.append(ctx.moments(cam.width, cam.height))
        ctx.render_batch(jobs, wave_paths=2000)
        for k, (_, cam, _) in enumerate(jobs):
            s, q, n = ctx.batch_moments(k, cam.width, cam.height)
            assert n == alone[k][2]
            np.testing.assert_allclose(s, alone[k][0], rtol=1e-5, atol=1e-6)
            np.testing.assert_allclose(q, alone[k][1], rtol=1e-5, atol=1e-6)
    finally:
        for s in sids:
            ctx.release(s)
