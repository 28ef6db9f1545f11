"""Batched and served forms through the C ABI.

The property both must keep: a job's image is the same alone and in a mix.
Each job's camera paths keep or3_render's numbering and Philox keys, so its
per-pixel sums must equal a plain or3_render of the same job to float
rounding (the only order-dependent step is the float atomics that add the two
branches of a glass split): rtol 1e-5.
"""
import threading
import time
from collections import defaultdict

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _jobs(pkg, ctx, nee=False):
    """Three jobs; nee: with next-event estimation (the Cornell box's area
    light, the reference Cornell's SphereLight, the icosphere box's light quad)."""
    W = pkg.workloads
    a = W.cornell_box(40, 32)
    b = W.icosphere_in_box(48, 32, level=3)
    c = W.reference_cornell(32, 24)
    sids = [ctx.upload(x[0]) for x in (a, b, c)]
    jobs = [
        (sids[0], a[1], dict(supersamples=2, min_samples=1, max_samples=3, step_samples=1, rr_min_depth=3,
                             max_depth=8, seed=5)),
        (sids[1], b[1], dict(supersamples=4, min_samples=2, max_samples=2, step_samples=1, rr_min_depth=5,
                             max_depth=10, seed=6)),
        (sids[2], c[1], dict(supersamples=1, min_samples=4, max_samples=8, step_samples=4, rr_min_depth=5,
                             max_depth=0, seed=7)),
    ]
    if nee:
        for _, _, st in jobs:
            st["next_event_estimation"] = True
    return sids, jobs


def _plain(ctx, sid, cam, st):
    ctx.render(sid, cam, **st)
    s, q, n = ctx.moments(cam.width, cam.height)
    img, _ = ctx.frame(cam.width, cam.height)
    return s, q, n, img


@pytest.mark.parametrize("wave_paths,flags,nee", [(0, 0, False), (3000, 0, False), (3000, 64, False),
                                                (3000, 256, False), (0, 0, True), (3000, 0, True),
                                                (3000, 512, True), (0, 1024, False), (3000, 1024, False),
                                                (3000, 1024 | 64, False), (0, 1024, True), (3000, 1024, True)])
def test_batch_jobs_equal_their_plain_renders(pkg, ctx, wave_paths, flags, nee):
    """flags 64 = OR3_FLAG_ONE_LANE (every wave on one stream; the default
    deals waves to three lanes); 256 = OR3_FLAG_HOIST_NODES (the node array
    copied to registers per ray instead of read through the scene descriptor
    every step: the same traversal); nee:
    light sampling on, where the material-sorted shade is the default and 512
    (OR3_FLAG_UNSORTED_SHADE) selects the single shade kernel.  By default each
    lane is one graph launch that takes waves from a device queue until none
    is left; 1024 = OR3_FLAG_HOST_LOOP hands the waves out from the host and
    replays each wave's bounce graph."""
    sids, jobs = _jobs(pkg, ctx, nee)
    try:
        alone = [_plain(ctx, *j) for j in jobs]
        stats, frames = ctx.render_batch(jobs, frames=True, wave_paths=wave_paths, flags=flags)
        if wave_paths:
            assert stats["waves"] > 3  # jobs really were cut and mixed across waves
        for k, (sid, cam, st) in enumerate(jobs):
            s, q, n = ctx.batch_moments(k, cam.width, cam.height)
            s0, q0, n0, img0 = alone[k]
            assert n == n0
            np.testing.assert_allclose(s, s0, rtol=1e-5, atol=1e-6)
            np.testing.assert_allclose(q, q0, rtol=1e-5, atol=1e-6)
            np.testing.assert_allclose(frames[k], img0, rtol=1e-5, atol=1e-7)
        assert stats["camera_paths"] == sum(c.width * c.height * st["supersamples"] ** 2 *
                                            (st["min_samples"] + (st["max_samples"] - st["min_samples"]) //
                                             st["step_samples"] * st["step_samples"]) for _, c, st in jobs)
    finally:
        for s in sids:
            ctx.release(s)


@pytest.mark.parametrize("flags", [0, 64])
def test_batch_split_overflow_renders_waves_again(pkg, ctx, flags):
    """Glass: the device loop's queues hold two rays per camera path.  A job
    whose camera sees only a glass sphere makes three rays per path at depth
    3, so its waves overflow; they are not accumulated and are rendered again
    after the loop in waves that cannot overflow.  Every job still equals its
    plain render (64 = one lane)."""
    A = pkg.abi
    sids, jobs = _jobs(pkg, ctx)
    sd, cam, _ = pkg.workloads.cornell_box(40, 30)
    glass = sd.material(A.OR3_REFRACTION, (0.99, 0.99, 0.99), ior=1.5)
    sd.add_sphere((50.0, 50.0, 150.0), 60.0, sd.layers(glass))  # fills the view of the camera at z = 250
    sids.append(ctx.upload(sd))
    jobs.append((sids[-1], cam, dict(supersamples=2, min_samples=1, max_samples=2, step_samples=1,
                                     rr_min_depth=3, max_depth=8, seed=11)))
    try:
        alone = [_plain(ctx, *j) for j in jobs]
        stats, frames = ctx.render_batch(jobs, frames=True, wave_paths=3000, flags=flags)
        assert stats["waves_rerun"] > 0
        for k, (sid, cam_k, st) in enumerate(jobs):
            s, q, n = ctx.batch_moments(k, cam_k.width, cam_k.height)
            s0, q0, n0, img0 = alone[k]
            assert n == n0
            np.testing.assert_allclose(s, s0, rtol=1e-5, atol=1e-6)
            np.testing.assert_allclose(q, q0, rtol=1e-5, atol=1e-6)
            np.testing.assert_allclose(frames[k], img0, rtol=1e-5, atol=1e-7)
        assert stats["camera_paths"] == sum(c.width * c.height * st["supersamples"] ** 2 *
                                            (st["min_samples"] + (st["max_samples"] - st["min_samples"]) //
                                             st["step_samples"] * st["step_samples"]) for _, c, st in jobs)
    finally:
        for s_ in sids:
            ctx.release(s_)


@pytest.mark.parametrize("flags", [128, 128 | 256])
def test_batch_over_quantised_nodes(pkg, ctx, flags):
    """OR3_FLAG_QUANTISED_NODES: the 64-byte nodes bound the same leaves more
    loosely, so the same closest hits are found in another order; only hits at
    exactly equal distance (shared edges) can resolve to the other primitive."""
    sids, jobs = _jobs(pkg, ctx)
    try:
        ctx.render_batch(jobs, wave_paths=3000)
        ref = [ctx.batch_moments(k, c.width, c.height) for k, (_, c, _) in enumerate(jobs)]
        ctx.render_batch(jobs, wave_paths=3000, flags=flags)
        for k, (sid, cam, st) in enumerate(jobs):
            s, q, n = ctx.batch_moments(k, cam.width, cam.height)
            s0, _, n0 = ref[k]
            assert n == n0
            off = np.abs(s - s0) > 1e-5 * np.abs(s0) + 1e-6
            assert off.mean() < 0.005, (k, off.mean())
            assert abs(s.sum() - s0.sum()) <= 2e-3 * abs(s0.sum())
    finally:
        for s_ in sids:
            ctx.release(s_)


def test_batch_without_graph_and_autotune(pkg, ctx):
    sids, jobs = _jobs(pkg, ctx)
    try:
        ctx.render_batch(jobs, graph_bounces=4)
        s1 = [ctx.batch_moments(k, c.width, c.height)[0] for k, (_, c, _) in enumerate(jobs)]
        ctx.render_batch(jobs, flags=pkg.abi.OR3_FLAG_NO_GRAPH)
        s2 = [ctx.batch_moments(k, c.width, c.height)[0] for k, (_, c, _) in enumerate(jobs)]
        for a, b in zip(s1, s2):
            np.testing.assert_allclose(a, b, rtol=1e-5, atol=1e-6)
        best, rate = ctx.autotune_batch(jobs, sample_paths=100000)
        assert best["wave_paths"] in (1 << 21, 1 << 22, 1 << 23, 1 << 24, 1 << 25)
        assert best["graph_bounces"] in (4, 8, 16)
        assert rate > 0
    finally:
        for s in sids:
            ctx.release(s)


def test_batch_rejects_bad_jobs(pkg, ctx):
    sd, cam, _ = pkg.workloads.cornell_box(8, 8)
    sid = ctx.upload(sd)
    with pytest.raises(pkg.Or3Error):
        ctx.render_batch([(sid + 1000, cam, dict(supersamples=1))])
    with pytest.raises(pkg.Or3Error):
        ctx.render_batch([(sid, cam, dict(supersamples=0))])
    ctx.release(sid)


@pytest.mark.parametrize("one_lane,nee", [(False, False), (True, False), (False, True)])
def test_server_continuous_batching_same_alone_and_in_mix(pkg, ctx, one_lane, nee):
    sids, jobs = _jobs(pkg, ctx, nee)
    alone = [_plain(ctx, *j) for j in jobs]
    frames = defaultdict(list)
    lock = threading.Lock()

    def on_frame(jid, samples, img, final):
        with lock:
            frames[jid].append((samples, final, img))

    ctx.server_start(keep_moments=True, frame_every_samples=1, wave_paths=1 << 16, on_frame=on_frame,
                     one_lane=one_lane)
    try:
        # later arrivals join while the first job runs: submitted right behind it
        # (microseconds), while the first job takes many waves and frame callbacks
        ids = [ctx.server_submit(*jobs[0][:2], **jobs[0][2])]
        ids += [ctx.server_submit(j[0], j[1], **j[2]) for j in jobs[1:]]
        ctx.server_drain(120.0)
        stats = ctx.server_stats()
        for k, jid in enumerate(ids):
            cam = jobs[k][1]
            st = ctx.server_poll(jid)
            assert st["state"] == pkg.abi.OR3_JOB_DONE
            s, q, n = ctx.server_moments(jid, cam.width, cam.height)
            s0, q0, n0, img0 = alone[k]
            assert n == n0
            np.testing.assert_allclose(s, s0, rtol=1e-5, atol=1e-6)
            fs = frames[jid]
            assert fs[-1][1] and not any(f[1] for f in fs[:-1])
            assert [f[0] for f in fs] == sorted(f[0] for f in fs)
            np.testing.assert_allclose(fs[-1][2], img0, rtol=1e-5, atol=1e-7)
        assert stats["jobs_done"] == 3
        assert stats["latency_p99_s"] >= stats["latency_p50_s"] > 0
        assert stats["peak_active_jobs"] >= 2  # the jobs overlapped on the device
    finally:
        ctx.server_stop()
        for s in sids:
            ctx.release(s)


def test_server_split_overflow_renders_pieces_again(pkg, ctx):
    """Glass: the server's queues hold two rays per camera path.  A job whose
    camera sees only a glass sphere overflows its lanes' queues (three rays
    per path at depth 3); those lanes are not accumulated and their segments
    are rendered again in pieces that cannot overflow: every job still
    equals its plain render."""
    A = pkg.abi
    sids, jobs = _jobs(pkg, ctx)
    # 153,600 paths: once the small jobs are done it fills whole lanes
    # (65,536 paths each, queues of 131,072 rays)
    sd, cam, _ = pkg.workloads.cornell_box(160, 120)
    glass = sd.material(A.OR3_REFRACTION, (0.99, 0.99, 0.99), ior=1.5)
    sd.add_sphere((50.0, 50.0, 150.0), 60.0, sd.layers(glass))  # fills the view of the camera at z = 250
    sids.append(ctx.upload(sd))
    jobs.append((sids[-1], cam, dict(supersamples=2, min_samples=1, max_samples=2, step_samples=1,
                                     rr_min_depth=3, max_depth=8, seed=11)))
    alone = [_plain(ctx, *j) for j in jobs]
    ctx.server_start(keep_moments=True, frame_every_samples=1, wave_paths=1 << 16)
    try:
        ids = [ctx.server_submit(j[0], j[1], **j[2]) for j in jobs]
        ctx.server_drain(120.0)
        stats = ctx.server_stats()
        assert stats["waves_rerun"] > 0
        for k, jid in enumerate(ids):
            cam_k = jobs[k][1]
            assert ctx.server_poll(jid)["state"] == A.OR3_JOB_DONE
            s, q, n = ctx.server_moments(jid, cam_k.width, cam_k.height)
            s0, q0, n0, _ = alone[k]
            assert n == n0
            np.testing.assert_allclose(s, s0, rtol=1e-5, atol=1e-6)
            np.testing.assert_allclose(q, q0, rtol=1e-5, atol=1e-6)
        assert stats["jobs_done"] == len(jobs)
    finally:
        ctx.server_stop()
        for s_ in sids:
            ctx.release(s_)


def test_server_budget_admission_and_cancel(pkg, ctx):
    sids, jobs = _jobs(pkg, ctx)
    big = pkg.workloads.cornell_box(64, 64)
    bsid = ctx.upload(big[0])
    # budget (80 kB) above any one small job's buffers (<= 48x32 px x 48 B = 73.7 kB)
    # and below any two: admission serialises them; the big job (196 kB) only
    # gets in because nothing else is running
    ctx.server_start(hbm_budget_bytes=80000, wave_paths=1 << 16)
    try:
        # long enough (4000 passes) to be running still when it is cancelled
        long_id = ctx.server_submit(bsid, big[1], supersamples=2, min_samples=4000, max_samples=4000, seed=1)
        ids = [ctx.server_submit(j[0], j[1], **j[2]) for j in jobs]
        time.sleep(0.05)
        ctx.server_cancel(long_id)
        ctx.server_drain(120.0)
        assert ctx.server_poll(long_id)["state"] == pkg.abi.OR3_JOB_CANCELLED
        for jid in ids:
            assert ctx.server_poll(jid)["state"] == pkg.abi.OR3_JOB_DONE
        st = ctx.server_stats()
        assert st["peak_active_jobs"] == 1
        assert st["jobs_cancelled"] == 1
    finally:
        ctx.server_stop()
        for s in sids + [bsid]:
            ctx.release(s)
