"""Every kernel variant behind or3_render_params.tuning renders the same paths.

The closest hit of a ray does not depend on the tree's box format (FP32
child boxes by default, 8-bit quantised ones for variants 1, 3 and 6), on
the order children are visited, on shared-memory node staging or on the
lane refill threshold; only ties (two primitives at one distance) may
resolve differently.  So each variant's per-path radiance must equal the
default's for all but a handful of paths, shadow rays included (NEE on).
The material-sorted shade (0x800) files hits by material class and shades
each class with its own kernel instance; the paths are the same too.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

VARIANTS = {
    "step1_quantised": 1,
    "gridstride_quantised": 3,
    "refill8": 4,
    "refill24": 5,
    "step2_quantised": 6,
    "nearest_first": 7,
    "step2_quantised_smem": 6 | 0x10,
    "shadow_unsorted": 0x20,
    "l2_window": 0x40,
    "shade_nee_4_blocks": 0x80,
    "sorted_shade": 0x800,
    "unsorted_shade": 0x2000,
    "block_append": 0x1000,
    "wide8": 0x4000,
    "shadow_refill8": 0x8000,
}


def _scenes(W):
    return {
        "ico_phong": (W.icosphere_in_box(64, 48, level=4)[:2], dict(rr_min_depth=5, max_depth=10)),
        "terrain_nee": (W.terrain_ibl(64, 36, cells_x=128, cells_z=64, spheres=16)[:2],
                        dict(rr_min_depth=5, max_depth=12, next_event_estimation=True)),
        # mirror and glass (split paths), NEE off
        "cornell": (W.cornell_box(48, 48)[:2], dict(rr_min_depth=3, max_depth=8)),
        # a sphere light, a two-layer sphere and floors (planes) with NEE on
        "refcornell_nee": (W.reference_cornell(48, 36)[:2], dict(rr_min_depth=5, max_depth=0,
                                                                  next_event_estimation=True)),
        # a constant background sampled as a light
        "sky_constant": (W.sky_floor(48, 48, constant=(0.6, 0.7, 0.9)),
                         dict(rr_min_depth=5, max_depth=8, next_event_estimation=True)),
    }


@pytest.mark.parametrize("scene", ["ico_phong", "terrain_nee", "cornell", "refcornell_nee", "sky_constant"])
def test_variants_render_the_same_paths(pkg, ctx, scene):
    (sd, cam), st = _scenes(pkg.workloads)[scene]
    sid = ctx.upload(sd)
    try:
        def paths(tuning):
            ctx.render(sid, cam, supersamples=2, seed=77, tuning=tuning, flags=pkg.abi.OR3_FLAG_KEEP_PATHS, **st)
            return ctx.path_radiance().astype(np.float64)

        base = paths(0)
        assert np.isfinite(base).all() and base.sum() > 0
        for name, tuning in VARIANTS.items():
            p = paths(tuning)
            same = (np.abs(p - base) <= 1e-5 * (1.0 + np.abs(base))).all(axis=1)
            assert same.mean() >= 0.999, (name, same.mean())
    finally:
        ctx.release(sid)
