"""or3_render_paths_noalloc -- rendering camera paths with no device allocation.

The entry point is for callers that cannot allocate device memory while they
render (an engine that owns the whole device through its own pool, a frame
loop that cannot let cudaMalloc stall the device).  It keeps its ray queues
in a fixed array compiled into the library, so it must give the same
radiance, path for path, as the allocating or3_render, and keep doing so call
after call on the shared array.  It also puts the caller's current device
back before it returns.

This file is collected last so that a failure here leaves every other test
already run.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SETTINGS = dict(supersamples=4, min_samples=2, max_samples=2, step_samples=1, rr_min_depth=3, max_depth=8,
                seed=42)


def _close(a, b):
    # the per-path tolerance of the render parity tests
    return np.abs(a - b) <= 1e-3 * (1.0 + np.abs(b))


def test_noalloc_matches_render_on_consecutive_calls(pkg):
    torch = pytest.importorskip("torch")
    ctx = pkg.Context(0)
    try:
        # the Cornell box has a glass sphere, so paths split: the scratch's
        # eight-rays-per-path queue bound is exercised
        sd, cam, _ = pkg.workloads.cornell_box(48, 32)
        sid = ctx.upload(sd)
        ctx.render(sid, cam, flags=pkg.abi.OR3_FLAG_KEEP_PATHS, **SETTINGS)
        ref = ctx.path_radiance()
        assert ref.shape[0] == 48 * 32 * 16 * 2
        n = pkg.abi.OR3_NOALLOC_MAX_PATHS
        out = torch.zeros(3 * n, dtype=torch.float32, device="cuda:0")
        firsts = [0, 20000, 0]  # two different calls in a row, then the first again
        got = []
        for first in firsts:
            out.fill_(-1.0)
            dev_before = torch.cuda.current_device()
            ctx.render_paths_noalloc(sid, cam, first, n, out.data_ptr(), **SETTINGS)
            assert torch.cuda.current_device() == dev_before
            torch.cuda.synchronize()
            got.append(out.cpu().numpy().reshape(n, 3).astype(np.float64))
        for first, g in zip(firsts, got):
            want = ref[first:first + n].astype(np.float64)
            ok = _close(g, want).all(axis=1)
            assert ok.all(), (first, np.nonzero(~ok)[0][:5])
        np.testing.assert_allclose(got[0], got[2], rtol=1e-6, atol=1e-7)
        ctx.release(sid)
    finally:
        ctx.close()


def test_noalloc_rejects_more_paths_than_its_scratch(pkg):
    torch = pytest.importorskip("torch")
    ctx = pkg.Context(0)
    try:
        sd, cam, _ = pkg.workloads.cornell_box(48, 32)
        sid = ctx.upload(sd)
        n = pkg.abi.OR3_NOALLOC_MAX_PATHS + 1
        out = torch.zeros(3 * n, dtype=torch.float32, device="cuda:0")
        with pytest.raises(pkg.Or3Error) as e:
            ctx.render_paths_noalloc(sid, cam, 0, n, out.data_ptr(), **SETTINGS)
        assert e.value.code == pkg.abi.OR3_ERR_INVALID_ARGUMENT
        assert "limit" in str(e.value)
        ctx.release(sid)
    finally:
        ctx.close()


def test_noalloc_with_light_sampling_matches_render(pkg):
    # next-event estimation: the scratch's shadow queue is exercised too
    torch = pytest.importorskip("torch")
    ctx = pkg.Context(0)
    try:
        sd, cam = pkg.workloads.sphere_light_box(40, 32)
        sid = ctx.upload(sd)
        st = dict(SETTINGS, next_event_estimation=True)
        ctx.render(sid, cam, flags=pkg.abi.OR3_FLAG_KEEP_PATHS, **st)
        ref = ctx.path_radiance().astype(np.float64)
        n = pkg.abi.OR3_NOALLOC_MAX_PATHS
        out = torch.zeros(3 * n, dtype=torch.float32, device="cuda:0")
        ctx.render_paths_noalloc(sid, cam, 4096, n, out.data_ptr(), **st)
        torch.cuda.synchronize()
        got = out.cpu().numpy().reshape(n, 3).astype(np.float64)
        ok = _close(got, ref[4096:4096 + n]).all(axis=1)
        assert ok.all(), np.nonzero(~ok)[0][:5]
        ctx.release(sid)
    finally:
        ctx.close()
