"""GPU shading lookups and the thin lens against the reference's own code.

  * IBL::Sample(dir) (src/renderer/IBL.h:30-45) through or3_env_sample, which
    runs the shade kernel's env_lookup: the texel index per direction equals
    the reference's, except where the reference's FP64 u*W or v*H lies within
    5e-5 texel of a texel edge (FP32 acos/sqrt can land on either side);
  * Image::GetPixelByUV (src/tools/Image.h:20-31) through or3_texture_sample
    (the kernel's texel()): equal colours except within 2e-5 texel of an edge;
  * GetTexturedColor in the render (src/renderer/PathTracer.cpp:327-346): the
    textured scene has no Monte Carlo noise, so per-pixel means are compared
    by value with the reference's render;
  * Camera::SampleRayForPixel with CircleAperture (Camera.h:65-93,
    Aperture.h:23-35): per-pixel 3-SE agreement with the reference's renders
    through the lens of its main() (radius 1.3, focal distance 300) and a
    strong depth of field (radius 20, focal plane at the box's front, the
    back wall blurred over ~9 pixels), one
    lens sample per sub-pixel per pass as in the reference.
"""
import sys

import numpy as np
import pytest

from conftest import GOLDEN, golden, moments_to_mean_se, zscores

sys.path.insert(0, GOLDEN)
import make_golden as MG  # noqa: E402

pytestmark = pytest.mark.gpu


def _ref_uv(d, w, h):
    x, y, z = d[:, 0], d[:, 1], d[:, 2]
    theta = np.arccos(y)
    with np.errstate(invalid="ignore", divide="ignore"):
        phi = np.arccos(x / np.sqrt(x * x + z * z))
    phi = np.where(z < 0.0, 2.0 * np.pi - phi, phi)
    return phi / (2.0 * np.pi) * w, theta / np.pi * h


def _near_edge(f, tol):
    return np.abs(f - np.round(f)) < tol


def test_env_sample_matches_reference(pkg, ctx):
    g = golden("ibl_ref.npz")
    dirs = g["dirs"]
    for w, h in g["sizes"]:
        w, h = int(w), int(h)
        sid = ctx.upload(MG.ibl_scene(w, h))
        try:
            got = ctx.env_sample(sid, dirs)
        finally:
            ctx.release(sid)
        want = g["texel_%dx%d" % (w, h)]
        assert np.all(got[:, 2] == got[:, 1] * w + got[:, 0])
        gx, gy = got[:, 0].astype(np.int32), got[:, 1].astype(np.int32)
        fu, fv = _ref_uv(dirs.astype(np.float64), w, h)
        tie = _near_edge(fu, 5e-5) | _near_edge(fv, 5e-5)
        bad = ((gx != want[:, 0]) | (gy != want[:, 1])) & ~tie
        assert not bad.any(), (w, h, np.nonzero(bad)[0][:8], dirs[bad][:4], got[bad][:4], want[bad][:4])
        assert tie.mean() < 0.1
        # the mirrored half and the x axis are covered
        assert ((dirs[:, 2] < 0) & ~tie).sum() > 1000


def test_texture_sample_matches_reference(pkg, ctx):
    g = golden("texel_ref.npz")
    sd, _, _ = pkg.workloads.textured_scene()
    assert sd.digest() == str(g["digest"])
    sid = ctx.upload(sd)
    try:
        for t, tex in enumerate(sd.textures):
            uv = g["uv_%d" % t]
            got = ctx.texture_sample(sid, t, uv)
            h, w = tex.shape[:2]
            cu = np.clip(uv.astype(np.float64), 0.0, 1.0) * 0.99999
            # an edge inside the texture (a coordinate clamped to 0 reads texel 0 on both sides)
            tie = (_near_edge(cu[:, 0] * w, 2e-5) & (cu[:, 0] > 0)) | (_near_edge(cu[:, 1] * h, 2e-5) & (cu[:, 1] > 0))
            bad = np.any(got != g["rgb_%d" % t], axis=1) & ~tie
            assert not bad.any(), (t, np.nonzero(bad)[0][:8], uv[bad][:4])
            assert tie.mean() < 0.05
            # u or v = 1 (and beyond) read the last texel, not one past it
            one = (uv[:, 0] >= 1.0) & (uv[:, 1] >= 1.0)
            assert one.any() and np.all(got[one] == tex[-1, -1])
        with pytest.raises(pkg.Or3Error):
            ctx.texture_sample(sid, len(sd.textures), g["uv_0"][:4])
    finally:
        ctx.release(sid)


def test_textured_render_matches_reference(pkg, ctx):
    g = golden("render_textured.npz")
    sd, cam, st = pkg.workloads.textured_scene()
    assert sd.digest() == str(g["digest"])
    sid = ctx.upload(sd)
    try:
        ctx.render(sid, cam, seed=3, **st)
        s, _, n = ctx.moments(cam.width, cam.height)
    finally:
        ctx.release(sid)
    assert n == int(g["n"])
    m = s / n
    want = g["mean"].astype(np.float64)
    close = np.all(np.abs(m - want) <= 1e-5 * np.maximum(np.abs(want), 1e-3), axis=2)
    # the rest: a sub-pixel ray within FP32 rounding of a texel edge or of a silhouette
    assert close.mean() >= 0.98, close.mean()
    assert abs(m.mean() - want.mean()) <= 1e-3 * want.mean()
    textured = np.any(want != 1.0, axis=2)
    assert close[textured].mean() >= 0.97, close[textured].mean()


@pytest.mark.parametrize("fixture,aperture,focal", [("render_lens_main.npz", 1.3, 300.0),
                                                     ("render_lens_dof.npz", 20.0, 150.0)])
def test_thin_lens_render_matches_reference(pkg, ctx, fixture, aperture, focal):
    g = golden(fixture)
    sd, cam, _ = pkg.workloads.cornell_lens(int(g["width"]), int(g["height"]), aperture, focal)
    assert sd.digest() == str(g["digest"])
    assert float(g["aperture"]) == aperture and float(g["focal"]) == focal
    ss = int(g["supersamples"])
    sid = ctx.upload(sd)
    try:
        # the fixture's schedule: one sample per pass, so every path has its own lens sample
        ctx.render(sid, cam, supersamples=ss, min_samples=1, max_samples=int(g["max_samples"]), step_samples=1,
                   seed=91, rr_min_depth=5, max_depth=0)
        s, q, n = ctx.moments(cam.width, cam.height)
    finally:
        ctx.release(sid)
    assert n == int(g["n"])
    m, se = moments_to_mean_se(s, q, n)
    z = zscores(m, se, n, g["mean"], g["se"], int(g["n"]))
    assert np.mean(np.abs(z) > 3) < 0.01, np.mean(np.abs(z) > 3)
    assert abs(z.mean()) < 0.05, z.mean()
    assert 0.8 < z.var() < 1.25, z.var()


def test_lens_changes_the_image(pkg, ctx):
    # the depth of field is visible: a pinhole render of the same box differs
    # from the strong-lens fixture by far more than the noise
    g = golden("render_lens_dof.npz")
    sd, cam, _ = pkg.workloads.cornell_box(int(g["width"]), int(g["height"]))
    sid = ctx.upload(sd)
    try:
        ctx.render(sid, cam, supersamples=int(g["supersamples"]), min_samples=1, max_samples=64, step_samples=1,
                   seed=92, rr_min_depth=5, max_depth=0)
        s, q, n = ctx.moments(cam.width, cam.height)
    finally:
        ctx.release(sid)
    m, se = moments_to_mean_se(s, q, n)
    z = zscores(m, se, n, g["mean"], g["se"], int(g["n"]))
    # the reference-render test allows 1% of pixels beyond 3 SE, so a pinhole would fail it
    assert np.mean(np.abs(z) > 3) > 0.02, np.mean(np.abs(z) > 3)
