"""Parity at the benchmark's full sizes.

The per-path parity tests elsewhere use small images.  Here the workloads are
the benchmark's own: the 81,920-triangle icosphere at 1024x768 with a 16x16
sub-pixel grid, and the 1,048,576-triangle terrain with its sky at
1920x1080 with a 32x32 grid.  Three spread ranges of camera paths go through
or3_render_paths_noalloc and are compared path by path with the oracle's
FP64 replay of the same random numbers (the 1% allowance of the small tests
for paths whose discrete decisions FP32 rounding flips).  The whole image is
also rendered with three wave lanes and with one, which must agree.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _workload(W, name):
    if name == "mesh":
        sd, cam, st = W.icosphere_in_box()
    else:
        sd, cam, st = W.terrain_ibl()
    keys = ("supersamples", "rr_min_depth", "max_depth", "next_event_estimation")
    return sd, cam, {k: st[k] for k in keys if k in st}


@pytest.mark.parametrize("name", ["mesh", "terrain"])
def test_full_size_paths_match_the_oracle(pkg, orc, name):
    torch = pytest.importorskip("torch")
    sd, cam, st = _workload(pkg.workloads, name)
    settings = dict(st, min_samples=1, max_samples=1, step_samples=1, seed=7)
    total = cam.width * cam.height * settings["supersamples"] ** 2
    n = pkg.abi.OR3_NOALLOC_MAX_PATHS
    firsts = [0, (total // 3) // n * n, total - n]
    ctx = pkg.Context(0)
    try:
        sid = ctx.upload(sd)
        out = torch.zeros(3 * n, dtype=torch.float32, device="cuda:0")
        got = []
        for first in firsts:
            ctx.render_paths_noalloc(sid, cam, first, n, out.data_ptr(), **settings)
            torch.cuda.synchronize()
            got.append(out.cpu().numpy().reshape(n, 3).astype(np.float64))
        ctx.release(sid)
    finally:
        ctx.close()
    oscene = orc.scene(sd, use_bvh=True)
    for first, g in zip(firsts, got):
        ref = oscene.path_radiance(cam, first, n, **settings)
        assert np.isfinite(g).all()
        close = (np.abs(g - ref) <= 1e-3 * (1.0 + np.abs(ref))).all(axis=1)
        assert close.mean() >= 0.99, (first, close.mean())
        # the few paths that diverge do not bias the estimate
        assert abs(g.mean() - ref.mean()) <= 0.02 * max(ref.mean(), 1e-3) + 4 * g.std() / np.sqrt(n), first


@pytest.mark.parametrize("name", ["mesh", "terrain"])
def test_full_size_wave_lanes_match_one_lane(pkg, ctx, name):
    sd, cam, st = _workload(pkg.workloads, name)
    settings = dict(st, min_samples=1, max_samples=1, step_samples=1, seed=8)
    sid = ctx.upload(sd)
    try:
        s3 = ctx.render(sid, cam, **settings)
        f3 = ctx.frame(cam.width, cam.height)[0]
        s1 = ctx.render(sid, cam, tuning=pkg.abi.OR3_TUNE_ONE_LANE, **settings)
        f1 = ctx.frame(cam.width, cam.height)[0]
    finally:
        ctx.release(sid)
    assert s3["lanes"] == 3 and s1["lanes"] == 1 and s3["waves"] >= 6
    assert s3["extension_rays"] == s1["extension_rays"] and s3["shadow_rays"] == s1["shadow_rays"]
    assert np.isfinite(f3).all() and f3.sum() > 0
    np.testing.assert_allclose(f3, f1, rtol=1e-5, atol=1e-7)
