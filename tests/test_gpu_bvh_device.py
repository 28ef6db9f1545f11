"""The device BVH build against the host build, through the C ABI.

Both builds follow the same rules (binned SAH, 16 bins, leaves <= 4, greedy
4-wide collapse, 8-bit child boxes); the trees differ only in the order in
which primitives with equal cost were partitioned.  So on the same rays:
  * hit distances are bit-identical (same FP32 geometry, same intersection
    code; the closest hit does not depend on the tree);
  * primitive ids are identical except ties (two primitives at the same
    distance, e.g. a ray through a shared edge);
  * the tree is as good: wide-node count and the nodes + primitives a
    render visits within a few percent of the host tree's;
  * a second device build of the same scene renders bit-identical paths
    (the build is deterministic).
"""
import copy

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _degenerate(pkg):
    """2000 copies of one triangle plus a few others: centroids coincide, so
    every split of the big cluster is a median split."""
    sd = pkg.scene.SceneDesc()
    m = sd.material(pkg.abi.OR3_LAMBERT, (0.5, 0.5, 0.5))
    tri = np.array([[10.0, 10.0, 50.0], [30.0, 10.0, 50.0], [10.0, 30.0, 50.0]])
    sd.add_triangles(np.repeat(tri[None], 2000, axis=0), sd.layers(m))
    sd.add_triangles(pkg.workloads.random_triangles(300, 3).tris[0][0], sd.layers(m))
    return sd


def _scenes(pkg):
    W = pkg.workloads
    return {
        "ico6_mesh": lambda: W.icosphere_in_box(64, 48, level=6)[0],
        "tris_and_spheres": lambda: W.random_triangles(40000, 11),
        "terrain": lambda: W.terrain_ibl(64, 36, cells_x=256, cells_z=128, spheres=16)[0],
        "tiny": lambda: W.cornell_box(16, 16)[0],
        "degenerate": lambda: _degenerate(pkg),
    }


def _with_build(sd, build):
    s = copy.copy(sd)
    s.build = build
    return s


@pytest.mark.parametrize("name", ["ico6_mesh", "tris_and_spheres", "terrain", "tiny", "degenerate"])
def test_device_build_matches_host_build(pkg, ctx, name):
    A = pkg.abi
    sd = _scenes(pkg)[name]()
    host = ctx.upload(_with_build(sd, A.OR3_BUILD_HOST))
    dev = ctx.upload(_with_build(sd, A.OR3_BUILD_DEVICE))
    try:
        ih, idv = ctx.scene_info(host), ctx.scene_info(dev)
        assert ih["num_primitives"] == idv["num_primitives"]
        assert 1 <= idv["tree_depth"] <= 20
        assert 0.8 * ih["num_nodes"] <= idv["num_nodes"] <= 1.25 * ih["num_nodes"] + 2
        o, d = pkg.workloads.random_rays(200000, seed=5)
        if name == "terrain":
            o, d = pkg.workloads.random_rays(200000, seed=5, lo=-1000.0, hi=1000.0, target_lo=-500.0,
                                             target_hi=500.0)
        a_ids, a_t, _ = ctx.trace_closest(host, o, d)
        b_ids, b_t, _ = ctx.trace_closest(dev, o, d)
        np.testing.assert_array_equal(a_t, b_t)
        diff = a_ids != b_ids
        # every id difference is a tie: both primitives hit at the same distance
        assert (a_t[diff] < 1e30).all()
        assert diff.mean() <= (1.0 if name == "degenerate" else 1e-3), diff.mean()
        # any-hit agrees exactly
        tmax = np.where(a_t < 1e30, a_t * 0.5, 1e3).astype(np.float32)
        np.testing.assert_array_equal(ctx.trace_occluded(host, o, d, tmax), ctx.trace_occluded(dev, o, d, tmax))
    finally:
        ctx.release(host)
        ctx.release(dev)


def test_device_tree_quality_and_determinism(pkg, ctx):
    A = pkg.abi
    sd, cam, st = pkg.workloads.icosphere_in_box(96, 72, level=6)
    st = dict(st, supersamples=4)
    counts, paths = {}, []
    for key, build in (("host", A.OR3_BUILD_HOST), ("dev", A.OR3_BUILD_DEVICE), ("dev2", A.OR3_BUILD_DEVICE)):
        sid = ctx.upload(_with_build(sd, build))
        try:
            s = ctx.render(sid, cam, seed=3, flags=A.OR3_FLAG_COUNT_TRAVERSAL | A.OR3_FLAG_KEEP_PATHS, **st)
            counts[key] = (64.0 * s["nodes_visited"] + 48.0 * s["tris_tested"] + 16.0 * s["spheres_tested"]) / \
                s["extension_rays"]
            paths.append(ctx.path_radiance())
        finally:
            ctx.release(sid)
    # algorithmic bytes per ray within 5% of the host tree's
    assert counts["dev"] <= 1.05 * counts["host"], counts
    assert counts["dev"] == counts["dev2"]
    np.testing.assert_array_equal(paths[1], paths[2])
    # host and device trees render the same paths (ties aside)
    same = (np.abs(paths[0] - paths[1]) <= 1e-4 * (1 + np.abs(paths[0]))).all(axis=1)
    assert same.mean() >= 0.999, same.mean()


def test_auto_build_location(pkg, ctx):
    # below OR3_BUILD_DEVICE_MIN_PRIMS the host builds; above, the device (same results either way)
    A = pkg.abi
    small = pkg.workloads.random_triangles(1000, 2)
    big = pkg.workloads.random_triangles(A.OR3_BUILD_DEVICE_MIN_PRIMS + 10, 2)
    for sd in (small, big):
        sid = ctx.upload(sd)
        ctx.release(sid)
    bad = _with_build(small, 7)
    with pytest.raises(pkg.Or3Error):
        ctx.upload(bad)


def test_upload_names_the_first_invalid_primitive(pkg, ctx):
    """The primitives are flattened on all host threads; the error is still the
    one a sequential check meets first (lowest triangle index, then spheres)."""
    def scene(bad_tris=(), inf_tri=None, bad_sphere=False):
        sd = pkg.SceneDesc()
        m = sd.material(pkg.abi.OR3_LAMBERT, (0.5, 0.5, 0.5))
        rng = np.random.default_rng(5)
        v = rng.uniform(0, 100, (40000, 1, 3)) + rng.uniform(-2, 2, (40000, 3, 3))
        if inf_tri is not None:
            v[inf_tri, 1, 0] = np.inf
        lay = np.tile(np.asarray(sd.layers(m), np.uint32), (40000, 1))
        for i in bad_tris:
            lay[i] = (0, 0)
        sd.add_triangles(v, lay)
        sd.add_sphere((50, 50, 50), -1.0 if bad_sphere else 3.0, sd.layers(m))
        return sd

    for kw, text in ((dict(bad_tris=(31000, 20001, 39999)), "triangle 20001"),
                     (dict(bad_sphere=True), "sphere 0"),
                     (dict(bad_tris=(7,), bad_sphere=True), "triangle 7")):
        with pytest.raises(pkg.Or3Error) as e:
            ctx.upload(scene(**kw))
        assert e.value.code == pkg.abi.OR3_ERR_INVALID_ARGUMENT
        assert text in str(e.value), str(e.value)
    with pytest.raises(pkg.Or3Error) as e:
        ctx.upload(scene(inf_tri=12345))
    assert "non-finite" in str(e.value)
    # the context stays usable
    sid = ctx.upload(scene())
    assert ctx.scene_info(sid)["flatten_ms"] > 0
    ctx.release(sid)
