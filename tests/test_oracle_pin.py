"""Pins the C oracle (oracle/or3_oracle.c) to the reference.

Against the committed golden vectors (made from the reference's compiled code
by tests/golden/make_golden.py) everywhere, and against the reference itself
where its sources are present (marker `reference`).  CPU only.
"""
import numpy as np
import pytest

from conftest import golden, moments_to_mean_se, zscores

CLOSEST = ["cornell", "refcornell", "tris3000", "ico3", "ico6"]


def _closest_scene(pkg, name):
    W = pkg.workloads
    return {
        "cornell": lambda: W.cornell_box()[0],
        "refcornell": lambda: W.reference_cornell()[0],
        "tris3000": lambda: W.random_triangles(3000, 7),
        "ico3": lambda: W.icosphere_in_box(64, 48, level=3)[0],
        "ico6": lambda: W.icosphere_in_box(64, 48, level=6)[0],
    }[name]().quantized_f32()


def test_philox_known_answers(orc):
    # Random123 known-answer vectors for philox4x32 with 10 rounds
    assert orc.philox([0, 0, 0, 0], 0, 0) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert orc.philox([0xFFFFFFFF] * 4, 0xFFFFFFFF, 0xFFFFFFFF) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert orc.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], 0xA4093822, 0x299F31D0) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


@pytest.mark.parametrize("name", CLOSEST)
@pytest.mark.parametrize("use_bvh", [True, False])
def test_oracle_closest_matches_golden(pkg, orc, name, use_bvh):
    g = golden("closest_%s.npz" % name)
    sd = _closest_scene(pkg, name)
    assert sd.digest() == str(g["digest"]), "scene generator changed since the fixture was made"
    ids, t, nrm = orc.scene(sd, use_bvh=use_bvh).closest(g["orig"], g["dir"])
    want_ids = g["ids"] if use_bvh else g["ids_bruteforce"]
    want_t = g["t"] if use_bvh else g["t_bruteforce"]
    np.testing.assert_array_equal(ids, want_ids)
    np.testing.assert_array_equal(t, want_t)  # same FP64 arithmetic: bit-identical
    if use_bvh:
        np.testing.assert_allclose(nrm.astype(np.float32), g["normal"], atol=1e-6)


def test_oracle_empty_and_miss_rays(pkg, orc):
    sd = pkg.workloads.cornell_box()[0]
    s = orc.scene(sd, use_bvh=True)
    ids, t, _ = s.closest(np.zeros((0, 3)), np.zeros((0, 3)))
    assert ids.shape == (0,)
    # rays pointing away from everything miss
    o = np.array([[50.0, 50.0, 300.0]])
    d = np.array([[0.0, 0.0, 1.0]])
    ids, t, _ = s.closest(o, d)
    assert ids[0] == -1 and t[0] > 1e37


RENDERS = [
    # fixture, workload builder, oracle samples (fewer than the fixture: the z test uses both SEs)
    ("render_cornell_ref.npz", lambda W: W.cornell_box(256, 256), 4, dict(rr_min_depth=5, max_depth=0)),
    ("render_cornell_cfg.npz", lambda W: W.cornell_box(128, 128), 8, dict(rr_min_depth=3, max_depth=8)),
    ("render_refcornell.npz", lambda W: W.reference_cornell(160, 120), 8, dict(rr_min_depth=5, max_depth=0)),
]


@pytest.mark.parametrize("fixture,build,samples,depth", RENDERS)
def test_oracle_render_statistically_matches_reference(pkg, orc, fixture, build, samples, depth):
    g = golden(fixture)
    sd, cam, _ = build(pkg.workloads)
    assert sd.digest() == str(g["digest"])
    ss = int(g["supersamples"])
    s, q, _ = orc.scene(sd, use_bvh=False).render(cam, supersamples=ss, min_samples=1, max_samples=samples,
                                                  step_samples=1, seed=123, **depth)
    n = samples * ss * ss
    m, se = moments_to_mean_se(s, q, n)
    z = zscores(m, se, n, g["mean"], g["se"], int(g["n"]))
    # per-pixel agreement within 3 standard errors (the tail beyond 3 SE of a
    # normal is 0.27%; heavy-tailed path radiance makes it a little larger)
    assert np.mean(np.abs(z) > 3) < 0.01, np.mean(np.abs(z) > 3)
    assert abs(z.mean()) < 0.05
    assert 0.8 < z.var() < 1.25
    rel = abs(m.mean() - g["mean"].astype(np.float64).mean()) / g["mean"].astype(np.float64).mean()
    assert rel < 0.01


@pytest.mark.reference
def test_oracle_closest_matches_reference_live(pkg, orc, ref):
    sd = pkg.workloads.random_triangles(800, 99)
    o, d = pkg.workloads.random_rays(3000, 17)
    for use_bvh in (True, False):
        a = orc.scene(sd, use_bvh=use_bvh).closest(o, d)
        b = ref.scene(sd, use_bvh=use_bvh).closest(o, d)
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])


@pytest.mark.reference
def test_reference_render_scene_layout(pkg, ref):
    """The reference's own RenderScene: 2W x H buffer, image in the left viewport."""
    sd, cam, _ = pkg.workloads.cornell_box(24, 16)
    out, _ = ref.scene(sd, use_bvh=False).render_scene(cam, supersamples=1, min_samples=1, max_samples=2,
                                                       nthreads=1)
    assert out.shape == (16, 48, 3)
    assert np.all(out[:, 24:] == 0)
    assert out[:, :24].sum() > 0
