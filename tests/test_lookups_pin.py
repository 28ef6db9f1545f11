"""The oracle's IBL lookup, texel lookup and textured shading against the
reference's own functions (golden vectors made by tests/golden/make_golden.py
from the compiled reference): IBL::Sample(dir) (src/renderer/IBL.h:30-45),
Image::GetPixelByUV (src/tools/Image.h:20-31), GetTexturedColor
(src/renderer/PathTracer.cpp:327-346) with polygon and sphere uv
(Polygon.h:63-106, Sphere.h:61-75).  Both sides compute in FP64 on the same
inputs, so the answers must be identical."""
import os
import sys

import numpy as np

from conftest import GOLDEN, golden

sys.path.insert(0, GOLDEN)
import make_golden as MG  # noqa: E402


def test_oracle_env_lookup_matches_reference(pkg, orc):
    g = golden("ibl_ref.npz")
    dirs = g["dirs"].astype(np.float64)
    assert (dirs[:, 2] < 0).sum() > 1000 and np.signbit(dirs[:, 2]).sum() > (dirs[:, 2] < 0).sum()
    for w, h in g["sizes"]:
        c = orc.scene(MG.ibl_scene(int(w), int(h)), use_bvh=False).env_sample(dirs)
        np.testing.assert_array_equal(c[:, :2].astype(np.int32), g["texel_%dx%d" % (w, h)])


def test_oracle_texel_matches_reference(pkg, orc):
    g = golden("texel_ref.npz")
    sd, _, _ = pkg.workloads.textured_scene()
    assert sd.digest() == str(g["digest"])
    s = orc.scene(sd, use_bvh=False)
    for t in range(len(sd.textures)):
        got = s.texel(t, g["uv_%d" % t].astype(np.float64)).astype(np.float32)
        np.testing.assert_array_equal(got, g["rgb_%d" % t])


def test_oracle_textured_render_matches_reference(pkg, orc):
    g = golden("render_textured.npz")
    sd, cam, st = pkg.workloads.textured_scene()
    assert sd.digest() == str(g["digest"])
    s, _, _ = orc.scene(sd, use_bvh=False).render(cam, nthreads=os.cpu_count(), **st)
    m = (s / int(g["n"])).astype(np.float32)
    np.testing.assert_allclose(m, g["mean"], rtol=1e-6, atol=1e-7)
    # the fixture covers both textured objects and the clamped uv border
    assert 0.2 < np.mean(g["mean"] != 1.0) < 0.9


def test_lens_fixtures_carry_their_camera(pkg):
    for name, ap, foc in (("render_lens_main.npz", 1.3, 300.0), ("render_lens_dof.npz", 20.0, 150.0)):
        g = golden(name)
        sd, cam, _ = pkg.workloads.cornell_lens(int(g["width"]), int(g["height"]), ap, foc)
        assert sd.digest() == str(g["digest"])
        assert float(g["aperture"]) == cam.aperture_radius and float(g["focal"]) == cam.focal_distance
        assert int(g["max_samples"]) == 64 and int(g["step_samples"]) == 1  # one lens sample per path


def test_oracle_thin_lens_matches_reference(pkg, orc):
    # the oracle's lens (the GPU's counters, FP64) against the reference's own
    # thin-lens render: per-pixel 3-SE agreement
    from conftest import moments_to_mean_se, zscores
    g = golden("render_lens_dof.npz")
    sd, cam, _ = pkg.workloads.cornell_lens(int(g["width"]), int(g["height"]), 20.0, 150.0)
    s, q, _ = orc.scene(sd, use_bvh=False).render(cam, nthreads=os.cpu_count(), supersamples=int(g["supersamples"]),
                                                   min_samples=1, max_samples=int(g["max_samples"]), step_samples=1,
                                                   seed=17, rr_min_depth=5, max_depth=0)
    n = int(g["n"])
    m, se = moments_to_mean_se(s, q, n)
    z = zscores(m, se, n, g["mean"], g["se"], n)
    assert np.mean(np.abs(z) > 3) < 0.01, np.mean(np.abs(z) > 3)
    assert abs(z.mean()) < 0.05 and 0.8 < z.var() < 1.25, (z.mean(), z.var())
