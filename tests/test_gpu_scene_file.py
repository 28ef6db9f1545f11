"""A scene read from the reference's text format, rendered on the GPU.

tests/golden/scene/full.scene.in (a transformed .obj mesh, layered spheres, a
sphere light, six floors, an infinite floor, an IBL) goes through
or3_scene_load_file twice: straight into or3_scene_upload (Context.upload_file)
and through the Python copy (load_scene_file + Context.upload).  Both must
render the same image (up to the order of the per-pixel atomic sums), and paths traced on the GPU must match the oracle's
FP64 replay of the same random numbers (the 1% allowance of the other path
tests for paths whose discrete decisions FP32 rounding flips).
"""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN

sys.path.insert(0, os.path.join(GOLDEN, "scene"))
from cases import stage_scene_dir  # noqa: E402

pytestmark = pytest.mark.gpu


def _camera(pkg):
    return pkg.Camera.from_fov(64, 48, (0.0, 3.0, 24.0), (0.0, 1.0, 0.0), 50.0)


@pytest.mark.parametrize("nee", [False, True])
def test_scene_file_upload_paths_equal_and_match_the_oracle(pkg, ctx, orc, tmp_path, nee):
    torch = pytest.importorskip("torch")
    path = stage_scene_dir(str(tmp_path))
    sd, _ = pkg.load_scene_file(path)
    cam = _camera(pkg)
    settings = dict(supersamples=2, min_samples=1, max_samples=1, step_samples=1, seed=11,
                    next_event_estimation=nee, rr_min_depth=5)
    s_file = ctx.upload_file(path)
    s_copy = ctx.upload(sd)
    try:
        keys = ("num_primitives", "num_nodes", "device_bytes", "tree_depth", "num_lights")
        i_file, i_copy = ctx.scene_info(s_file), ctx.scene_info(s_copy)
        assert {k: i_file[k] for k in keys} == {k: i_copy[k] for k in keys}
        assert i_file["num_lights"] == 3  # the sphere light and the emissive floor's two triangles
        ctx.render(s_file, cam, **settings)
        f_file = ctx.frame(cam.width, cam.height)[0]
        ctx.render(s_copy, cam, **settings)
        f_copy = ctx.frame(cam.width, cam.height)[0]
        n = pkg.abi.OR3_NOALLOC_MAX_PATHS
        out = torch.zeros(3 * n, dtype=torch.float32, device="cuda:0")
        ctx.render_paths_noalloc(s_file, cam, 0, n, out.data_ptr(), **settings)
        torch.cuda.synchronize()
        got = out.cpu().numpy().reshape(n, 3).astype(np.float64)
    finally:
        ctx.release(s_file)
        ctx.release(s_copy)
    assert np.isfinite(f_file).all() and f_file.sum() > 0
    np.testing.assert_allclose(f_file, f_copy, rtol=1e-5, atol=1e-7)  # sub-pixel sums are atomic adds
    ref = orc.scene(sd, use_bvh=True).path_radiance(cam, 0, n, **settings)
    close = (np.abs(got - ref) <= 1e-3 * (1.0 + np.abs(ref))).all(axis=1)
    assert close.mean() >= 0.99, close.mean()
    assert abs(got.mean() - ref.mean()) <= 0.02 * max(ref.mean(), 1e-3) + 4 * got.std() / np.sqrt(n)
