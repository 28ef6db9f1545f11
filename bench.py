#!/usr/bin/env python
"""Mpaths/s of the GB300 path-tracing hot path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload mesh|cornell|terrain]

A step is one full render (or3_render) of the workload: by default the
largest single-GPU scene, the IBL terrain (1,048,576-triangle height field,
64 glass spheres, 2048x1024 float sky with a 1e4 sun importance-sampled
through its marginal/conditional CDF, next-event estimation), 1920x1080 with
a 32x32 sub-pixel grid = 1024 samples per pixel, max depth 12 --
2,123,366,400 camera paths per step.  `--workload mesh` is the displaced
level-6 icosphere (81,920 triangles, Lambert + Phong layers) in the Cornell
box, 1024x768, 256 spp, max depth 10; `--workload cornell` the reference's
CPU-runnable Cornell box.  Synthetic, seeded scenes.

value      camera paths / device time of the passes (CUDA events on the
           library's stream, scene resident in HBM), Mpaths/s
e2e        the same through the C ABI from host buffers: scene upload
           (flatten + BVH build + H2D), render, frame D2H, per step
roofline   extend (closest-hit) kernel: algorithmic bytes (64 B per wide node
           visited, 48 B per triangle record, 16 B per sphere record, counted
           by an instrumented run of the same render) / its event-timed
           duration, against the measured HBM copy bandwidth
cpu_baseline  the C oracle (FP64 restatement of the reference path, its BVH)
           on all host cores over a bounded, evenly spread sample of paths
With --gpus N > 1 (torchrun), every rank renders a replica of the workload
(the path does not exchange data between GPUs): scaling "weak".
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
import __graft_entry__ as ge  # noqa: E402

METRIC = "Mpaths/s on 1 GB300 at fixed RMSE vs host-CPU ref; p50/p99 latency when served"

# Figures that come from an ncu capture, not from this run (ncu cannot run
# inside the timed bench).  Per workload: DRAM bytes (read + write) per ray of
# the extend kernel, from dram__bytes_read.sum + dram__bytes_write.sum of one
# `ncu --set full` capture of its first two launches on a smaller image of the
# same scene (queue bytes grow with the rays, the scene stays in L2), and the
# share of issue slots the kernel used on its active cycles
# (smsp__issue_active) in the same launches.  roofline.traffic is the bytes
# per ray times the rays of an average launch of this run.
NCU_EXTEND = {
    "mesh": {"dram_bytes_per_ray": 48.3, "issue_active": (0.755, 0.646),
             "source": "ncu --set full, k_extend launches 1-2, mesh scene at 512x384, 8x8 sub-pixel grid"},
    "terrain": {"dram_bytes_per_ray": 49.7, "issue_active": (0.747, 0.748),
                "source": "ncu --set full, k_extend launches 1-2, terrain scene at 480x270, 8x8 sub-pixel grid"},
}


def workload(pkg, name):
    W = pkg.workloads
    if name == "cornell":
        sd, cam, st = W.cornell_box(256, 256)
        desc = "cornell_box_10tri_2spheres_256x256_ss8_64spp_rr3_maxdepth8"
    elif name == "terrain":
        sd, cam, st = W.terrain_ibl()
        desc = "terrain_1048576tri_64glass_ibl2048x1024_envcdf_nee_1920x1080_ss32_1024spp_maxdepth12"
    else:
        sd, cam, st = W.icosphere_in_box()
        desc = "displaced_icosphere_81920tri_phong_in_cornell_1024x768_ss16_256spp_maxdepth10"
    return sd, cam, st, desc


def tile_rmse(s, q, n, fixture):
    """RMSE of a render's pixel moments (sums s, sums of squares q over n
    samples, rows top-down) against a 16384-spp reference fixture: tiles (rows
    counted from the bottom, as camera rows) or a whole image; with the RMSE
    the noise of both renders predicts."""
    g = np.load(fixture)
    m = s / n
    se2 = np.maximum(q / n - m * m, 0.0) / n
    if "tiles" in g.files:
        H = m.shape[0]
        d2, v, ref = [], [], []
        for k, (x0, y0, w, h) in enumerate(g["tiles"].tolist()):
            rows = H - 1 - (y0 + np.arange(h))
            d2.append((m[rows, x0:x0 + w] - g["mean"][k]) ** 2)
            v.append(se2[rows, x0:x0 + w] + g["se"][k].astype(np.float64) ** 2)
            ref.append(g["mean"][k])
        what = "16384-spp FP64 oracle render of five 32x32 tiles, same sub-pixel grid"
    else:
        d2, v, ref = [(m - g["mean"]) ** 2], [se2 * (1.0 + n / float(g["n"]))], [g["mean"]]
        what = "the reference's own 16384-spp render of the whole image, same sub-pixel grid"
    rmse = float(np.sqrt(np.mean(d2)))
    return {"value": rmse, "expected_from_noise": float(np.sqrt(np.mean(v))),
            "relative": rmse / float(np.mean(ref)), "spp": int(n), "reference": what}


def rmse_vs_16k(ctx, cam, name):
    """Image RMSE of the last render against the workload's 16384-spp
    reference (tests/golden/rmse_*.npz: tiles of an FP64 oracle render for the
    mesh and terrain, the reference's own full image for the Cornell box).
    None without one."""
    fname = {"cornell": "rmse_cornell_cfg.npz", "mesh": "rmse_mesh.npz", "terrain": "rmse_terrain.npz"}[name]
    path = os.path.join(ROOT, "tests", "golden", fname)
    if not os.path.exists(path):
        return None
    s, q, n = ctx.moments(cam.width, cam.height)
    return tile_rmse(s, q, n, path)


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": len(self.rows)}
        if not self.rows:
            return out
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        out["sm_mhz"] = float(np.median(sm)) if sm else None
        out["sm_max_mhz"] = max(mx) if mx else None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for k, nm in enumerate(names):
            if any(len(r) > 5 + k and r[5 + k] == "Active" for r in self.rows):
                out["reasons"].append(nm)
        return out


def desc_bytes(sd):
    a = sd.arrays()
    n = sum(v.nbytes for k, v in a.items() if isinstance(v, np.ndarray))
    n += len(a["mat"]) * 80
    if sd.env is not None:
        n += sd.env.nbytes
    return int(n)


def cpu_baseline(pkg, sd, cam, st, target_s=15.0, nthreads=None):
    """The oracle port on all host cores over an evenly spread sample of paths."""
    orc = ge.load_oracle().CRestatement()
    nthreads = nthreads or os.cpu_count()
    scene = orc.scene(sd, use_bvh=True)
    ss2 = st["supersamples"] ** 2
    total = cam.width * cam.height * ss2 * st["max_samples"]
    kw = dict(supersamples=st["supersamples"], min_samples=st["min_samples"], max_samples=st["max_samples"],
              step_samples=st["step_samples"], rr_min_depth=st["rr_min_depth"], max_depth=st["max_depth"], seed=1,
              next_event_estimation=st.get("next_event_estimation", False))
    chunks = 64
    stride = max(total // chunks, 1)
    # calibrate on a sample spread over the workload
    probe = 512
    t0 = time.perf_counter()
    for c in range(chunks):
        scene.path_radiance(cam, stride * c, probe, nthreads=nthreads, **kw)
    rate = probe * chunks / max(time.perf_counter() - t0, 1e-6)
    # rounds of `chunks` evenly spaced runs, each round about an eighth of the
    # target, until the target time is used (or the workload is exhausted)
    per = int(min(max(rate * target_s / 8 / chunks, 256), stride))
    done = rounds = 0
    t0 = time.perf_counter()
    while True:
        for c in range(chunks):
            scene.path_radiance(cam, stride * c + rounds * per, per, nthreads=nthreads, **kw)
        done += per * chunks
        rounds += 1
        sec = time.perf_counter() - t0
        if sec >= target_s or (rounds + 1) * per > stride:
            break
    return {"value": done / sec / 1e6, "unit": "Mpaths/s", "cores": nthreads, "kind": "port",
            "sample": "%d camera paths in %d rounds of %d evenly spaced runs of the %d-path workload, FP64 C "
                      "oracle, reference BVH, %.1f s" % (done, rounds, chunks, total, sec),
            "port_vs_reference": "the port renders 1.2-1.4x (1 thread) and 1.4-2.3x (8 threads) the Mpaths/s "
                                 "of the reference's own integrator on the same scenes and estimator "
                                 "(oracle/port_vs_reference.py where the reference compiles), so this "
                                 "overstates the reference's speed"}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def run_reference(args, pkg, world, rank):
    if rank != 0:
        return
    sd, cam, st, desc = workload(pkg, args.workload)
    vals = []
    for _ in range(args.warmup):
        cpu_baseline(pkg, sd, cam, st, target_s=2.0)
    for _ in range(args.steps):
        vals.append(cpu_baseline(pkg, sd, cam, st, target_s=args.cpu_seconds / max(args.steps, 1)))
    v = float(np.mean([x["value"] for x in vals]))
    cb = dict(vals[-1])
    cb["value"] = v
    line = {"metric": METRIC, "impl": "reference", "value": v, "unit": "Mpaths/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": desc, "paths_per_step": cam.width * cam.height * st["supersamples"] ** 2
                       * st["max_samples"]},
            "cpu_baseline": cb, "e2e": {"value": v, "unit": "Mpaths/s", "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0},
            "note": "the reference's own C++ cannot be built on this host (its sources are not shipped); "
                    "this arm times the FP64 C restatement of the same path (oracle port) on all host cores"}
    print(json.dumps(line), flush=True)


def run_batched(args, pkg):
    """Batched workload: 64 seeded scenes rendered one by one (plain form) and as one batch."""
    W = pkg.workloads
    ctx = pkg.Context(0)
    t0 = time.perf_counter()
    jobs_sd = W.batched_jobs(n=args.jobs, scale=args.scale, small=args.mix == "small")
    gen_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    sids = [ctx.upload(sd) for sd, _, _ in jobs_sd]
    upload_s = time.perf_counter() - t0
    jobs = [(sid, cam, st) for sid, (_, cam, st) in zip(sids, jobs_sd)]
    tris = sum(ctx.scene_info(s)["num_primitives"] for s in sids)
    paths = sum(c.width * c.height * st["supersamples"] ** 2 * st["max_samples"] for _, c, st in jobs)
    best = {}
    if args.autotune:
        best, _ = ctx.autotune_batch(jobs, sample_paths=1 << 25)
    if args.wave_paths:
        best["wave_paths"] = args.wave_paths
    if args.one_lane:
        best["flags"] = best.get("flags", 0) | pkg.abi.OR3_FLAG_ONE_LANE
    if args.batch_flags:
        best["flags"] = best.get("flags", 0) | args.batch_flags
    if args.batch_only:
        # the batched form alone (a small-footprint run for profiling): no plain renders
        for _ in range(max(args.warmup, 1)):
            ctx.render_batch(jobs[:4], **best)
        ms = [ctx.render_batch(jobs, **best)[0]["render_ms"] for _ in range(args.steps)]
        print(json.dumps({"form": "batched", "batch_only": True, "value": paths / float(np.median(ms)) / 1e3,
                          "unit": "Mpaths/s", "ms": float(np.median(ms)), "jobs": len(jobs),
                          "camera_paths": int(paths), "triangles_total": int(tris), "tuning": best}), flush=True)
        ctx.close()
        return
    for _ in range(max(args.warmup, 1)):
        ctx.render_batch(jobs[:4], **best)
        for sid, cam, st in jobs[:4]:
            ctx.render(sid, cam, **st)
    plain_ms = 0.0
    plain_wall = time.perf_counter()
    for sid, cam, st in jobs:
        plain_ms += ctx.render(sid, cam, **st)["render_ms"]
    plain_wall = time.perf_counter() - plain_wall
    batch_ms, batch_wall = [], []
    for _ in range(args.steps):
        w0 = time.perf_counter()
        s, _ = ctx.render_batch(jobs, **best)
        batch_wall.append(time.perf_counter() - w0)
        batch_ms.append(s["render_ms"])
    # image error of the first job in the last timed batch (the same paths as its plain render)
    rmse = None
    fix = os.path.join(ROOT, "tests", "golden", "rmse_batched_job0.npz")
    if (args.mix == "config" and args.scale == 1.0 and os.path.exists(fix) and
            jobs_sd[0][0].digest() == str(np.load(fix)["digest"])):
        cam0 = jobs[0][1]
        s0, q0, n0 = ctx.batch_moments(0, cam0.width, cam0.height)
        rmse = dict(tile_rmse(s0, q0, n0, fix), job=0)
    # equal images: a batched job equals its plain render (same paths), checked on a few jobs
    maxdiff = 0.0
    for k in (0, 1, len(jobs) - 1):
        sid, cam, st = jobs[k]
        ctx.render(sid, cam, **st)
        sp, _, _ = ctx.moments(cam.width, cam.height)
        ctx.render_batch([jobs[k]], **best)
        sb, _, _ = ctx.batch_moments(0, cam.width, cam.height)
        maxdiff = max(maxdiff, float(np.max(np.abs(sb - sp) / (np.abs(sp) + 1e-3))))
    bms = float(np.median(batch_ms))
    line = {"metric": METRIC, "form": "batched", "value": paths / bms / 1e3, "unit": "Mpaths/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": bms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generators)",
            "config": {"workload": ("batched_%d_scenes_1k-2M_tris_log_uniform_x%g_128-1024px_16-512spp" %
                                    (len(jobs), args.scale)) if args.mix == "config" else
                                   ("batched_%d_small_jobs_1k-2M_tris_x%g_64-256px_16-64spp" % (len(jobs), args.scale)),
                       "triangles_total": int(tris), "camera_paths": int(paths), "scene_gen_s": gen_s,
                       "scene_upload_s": upload_s, "tuning": best},
            "plain_form": {"value": paths / plain_ms / 1e3, "ms": plain_ms, "wall_s": plain_wall,
                           "what": "the same 64 renders, one or3_render call each, scenes resident"},
            "speedup_vs_plain": plain_ms / bms, "batch_wall_s": float(np.median(batch_wall)),
            "speedup_vs_plain_wall": plain_wall / float(np.median(batch_wall)),
            "equal_images_max_rel_diff": maxdiff, "rmse_vs_16k": rmse}
    print(json.dumps(line), flush=True)
    ctx.close()


def _plain_fifo(ctx, sids, reqs):
    """The same requests through the plain form, one or3_render after another
    (progressive frames every 16 spp through the frame callback, as the server
    delivers them).  Returns per-request device ms and paths."""
    durs, paths = [], []
    for t_arr, s, cam, st in reqs:
        st = dict(st, min_samples=1, step_samples=1)  # one pass (16 spp) per frame
        frames = []
        w0 = time.perf_counter()
        ctx.render(sids[s], cam, callback=lambda *a: frames.append(a[0]), **st)
        durs.append(time.perf_counter() - w0)
        paths.append(cam.width * cam.height * st["supersamples"] ** 2 * st["max_samples"])
    return np.array(durs), np.array(paths, np.float64)


def _fifo_latency(arrivals, durs):
    """Latency of a single FIFO renderer that starts each request when it
    arrives or when the previous one finishes."""
    finish, lat = 0.0, []
    for a, d in zip(arrivals, durs):
        start = max(a, finish)
        finish = start + d
        lat.append(finish - a)
    return np.array(lat)


def run_served(args, pkg):
    """Served workload: Poisson requests over a resident scene pool, continuous
    batching, against the plain form replaying the same request stream."""
    W = pkg.workloads
    ctx = pkg.Context(0)
    t0 = time.perf_counter()
    pool = W.served_pool(n=args.scenes, scale=args.scale, env=(args.env_w, args.env_h))
    gen_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    sids = [ctx.upload(sd) for sd, _ in pool]
    upload_s = time.perf_counter() - t0
    eyes = [e for _, e in pool]
    results = {}
    rng = np.random.default_rng(11)
    mean_paths = np.mean([w * h for w, h in W.SERVED_RES]) * np.mean(W.SERVED_SPP) * 1.0
    # warm both forms (context queues, graph capture, first-touch of every scene)
    for k in range(len(sids)):
        s, cam, st = W.served_request(np.random.default_rng(k), len(sids), lambda i: eyes[i])
        ctx.render(sids[k], cam, **dict(st, max_samples=1, min_samples=1))
    for label, rate, secs in (("stated_rate", args.rate, args.seconds),
                              ("sustainable_rate", None, args.sustain_seconds)):
        if rate is None:
            cap = results["stated_rate"]["mpaths_per_s"] * 1e6
            rate = 0.6 * cap / mean_paths
        reqs, t = [], 0.0
        while True:
            t += rng.exponential(1.0 / rate)
            if t > secs:
                break
            reqs.append((t,) + tuple(W.served_request(rng, len(sids), lambda k: eyes[k])))
        ctx.server_start(frame_every_samples=1, wave_paths=args.wave_paths)
        tstart = time.perf_counter()
        for t_arr, s, cam, st in reqs:
            time.sleep(max(0.0, tstart + t_arr - time.perf_counter()))
            ctx.server_submit(sids[s], cam, **st)
        ctx.server_drain(args.drain_timeout)
        wall = time.perf_counter() - tstart
        stt = ctx.server_stats()
        ctx.server_stop()
        durs, paths = _plain_fifo(ctx, sids, reqs)
        lat = _fifo_latency([r[0] for r in reqs], durs)
        served_rate = stt["camera_paths"] / max(stt["busy_s"], 1e-9) / 1e6
        plain_rate = paths.sum() / durs.sum() / 1e6
        results[label] = {"rate_req_per_s": rate, "arrival_window_s": secs, "requests": len(reqs),
                          "latency_p50_s": stt["latency_p50_s"], "latency_p99_s": stt["latency_p99_s"],
                          "queue_p50_s": stt["queue_p50_s"], "queue_p99_s": stt["queue_p99_s"],
                          "first_frame_p50_s": stt["first_frame_p50_s"],
                          "mpaths_per_s": stt["camera_paths"] / (stt["device_ms"] / 1e3) / 1e6,
                          "mpaths_per_s_wall": served_rate,
                          "camera_paths": stt["camera_paths"], "wall_s": wall,
                          "peak_active_jobs": stt["peak_active_jobs"],
                          "plain_form": {"mpaths_per_s_wall": plain_rate,
                                         "fifo_latency_p50_s": float(np.percentile(lat, 50)),
                                         "fifo_latency_p99_s": float(np.percentile(lat, 99)),
                                         "busy_s": float(durs.sum()),
                                         "what": "same requests, one blocking or3_render each (frame per 16 spp), "
                                                 "FIFO from the same arrival times"},
                          "served_over_plain_wall": served_rate / plain_rate}
    sr = results["stated_rate"]
    line = {"metric": METRIC, "form": "served", "value": sr["mpaths_per_s_wall"], "unit": "Mpaths/s", "n_gpus": 1,
            "steps": 1, "warmup": 1, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scenes, Poisson arrivals)",
            "config": {"workload": "served_%d_scenes_10k-4M_tris_x%g_env%dx%d" % (args.scenes, args.scale,
                                                                                args.env_w, args.env_h),
                       "scene_gen_s": gen_s, "scene_upload_s": upload_s,
                       "requests": "res {256^2,512^2,1280x720,1920x1080} x spp {16,64,256,1024}, frames every 16 spp",
                       "value": "camera paths / server busy wall time at the stated rate"},
            "served": results}
    print(json.dumps(line), flush=True)
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="terrain", choices=["mesh", "cornell", "terrain"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--res", default="", help="WxH override (smaller case for profiling)")
    ap.add_argument("--ss", type=int, default=0, help="sub-pixel grid override")
    ap.add_argument("--form", default="plain", choices=["plain", "batched", "served"])
    ap.add_argument("--tuning", type=int, default=0, help="or3_render_params.tuning (kernel variant A/B)")
    ap.add_argument("--leaf-max", type=int, default=0, help="BVH leaf size bound (0 = library default)")
    ap.add_argument("--trav-cost", type=float, default=0.0, help="BVH SAH node cost (0 = library default)")
    ap.add_argument("--scale", type=float, default=1.0, help="triangle-count scale of batched/served scenes")
    ap.add_argument("--jobs", type=int, default=64)
    ap.add_argument("--autotune", action="store_true")
    ap.add_argument("--wave-paths", type=int, default=0,
                    help="camera paths per wave, plain and batched forms (0 = library default)")
    ap.add_argument("--one-lane", action="store_true", help="batched form: every wave on one stream")
    ap.add_argument("--batch-flags", type=int, default=0,
                    help="batched form: extra or3_batch_params.flags (OR3_FLAG_QUANTISED_NODES 128, "
                         "OR3_FLAG_HOIST_NODES 256)")
    ap.add_argument("--batch-only", action="store_true", help="batched form only, no plain renders (profiling)")
    ap.add_argument("--mix", default="config", choices=["config", "small"],
                    help="batched jobs: the stated mix, or small jobs (64-256 px, 16-64 spp)")
    ap.add_argument("--scenes", type=int, default=32)
    ap.add_argument("--rate", type=float, default=50.0)
    ap.add_argument("--seconds", type=float, default=2.0)
    ap.add_argument("--sustain-seconds", type=float, default=20.0)
    ap.add_argument("--drain-timeout", type=float, default=600.0)
    ap.add_argument("--env-w", type=int, default=2048)
    ap.add_argument("--env-h", type=int, default=1024)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    pkg = ge.load_package()
    if args.form == "batched":
        run_batched(args, pkg)
        return
    if args.form == "served":
        run_served(args, pkg)
        return
    world, rank, local, dist = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, pkg, world, rank)
        return

    import torch
    ctx = pkg.Context(local)
    sd, cam, st, desc = workload(pkg, args.workload)
    if args.res:
        cam.width, cam.height = (int(x) for x in args.res.lower().split("x"))
        desc += "_resized_%dx%d" % (cam.width, cam.height)
    if args.ss:
        st["supersamples"] = args.ss
        desc += "_ss%d" % args.ss
    A = pkg.abi
    kw = dict(supersamples=st["supersamples"], min_samples=st["min_samples"], max_samples=st["max_samples"],
              step_samples=st["step_samples"], rr_min_depth=st["rr_min_depth"], max_depth=st["max_depth"],
              next_event_estimation=st.get("next_event_estimation", False), tuning=args.tuning)
    if args.tuning:
        desc += "_tuning%d" % args.tuning
    if args.wave_paths:  # smaller waves hold smaller ray queues (profiling captures)
        kw["wave_paths"] = args.wave_paths
        desc += "_wave%d" % args.wave_paths
    if args.leaf_max or args.trav_cost:
        sd.leaf_max, sd.traversal_cost = args.leaf_max, args.trav_cost
        desc += "_leaf%d_ct%g" % (args.leaf_max, args.trav_cost)
    t0 = time.perf_counter()
    sid = ctx.upload(sd)
    upload_s = time.perf_counter() - t0
    info = ctx.scene_info(sid)

    # algorithmic bytes per extension ray (instrumented run, untimed)
    c = ctx.render(sid, cam, seed=99, flags=A.OR3_FLAG_COUNT_TRAVERSAL, **kw)
    # the per-unit figure of a node visit is 64 B whatever the node layout (the
    # default FP32-box nodes load 128 B, from L1/L2 on these scenes)
    alg_bytes_per_ray = (64.0 * c["nodes_visited"] + 48.0 * c["tris_tested"] + 16.0 * c["spheres_tested"]) / \
        max(c["extension_rays"], 1)

    for i in range(args.warmup):
        ctx.render(sid, cam, seed=1000 + i, **kw)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda:%d" % local)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    barrier(dist)
    torch.cuda.synchronize()
    render_ms = 0.0
    shadow_rays = 0
    launches = paths = ext_rays = bounces = waves = passes = 0
    w0 = time.perf_counter()
    for i in range(args.steps):
        flush.zero_()  # L2 (129 MB) flushed between steps
        s = ctx.render(sid, cam, seed=i, **kw)
        render_ms += s["render_ms"]
        shadow_rays += s["shadow_rays"]
        launches += s["kernel_launches"]
        paths += s["camera_paths"]
        ext_rays += s["extension_rays"]
        bounces += s["bounces"]
        waves += s["waves"]
        passes += s["passes"]
    torch.cuda.synchronize()
    barrier(dist)
    wall_s = time.perf_counter() - w0
    clk = clocks.stop()
    # image error of the last timed render (untimed read of its pixel moments)
    rmse = rmse_vs_16k(ctx, cam, args.workload) if not (args.res or args.ss) else None
    # the kernel split: one more render of the same step with per-kernel CUDA
    # events (that flag keeps every wave on one stream), untimed
    flush.zero_()
    t = ctx.render(sid, cam, seed=args.steps, flags=A.OR3_FLAG_TIME_KERNELS, **kw)
    ext_ms, shade_ms, shadow_ms = t["extend_ms"], t["shade_ms"], t["shadow_ms"]
    ext_launches, t_ext_rays = t["extend_launches"], t["extension_rays"]
    dev_s = max_over_ranks(dist, render_ms / 1000.0)
    total_paths = sum_over_ranks(dist, float(paths))
    value = total_paths / dev_s / 1e6

    # end to end through the C ABI from host buffers
    e2e_steps = max(args.e2e_steps, 1)
    frame_bytes = 2 * cam.width * cam.height * 3 * 8
    h2d = desc_bytes(sd) + 2 * 200
    img = np.zeros((cam.height, 2 * cam.width, 3), np.float64)  # the caller's frame buffer, reused per step
    img[:] = 1.0
    barrier(dist)
    parts = np.zeros(4)  # wall seconds: upload, render, frame read-back, release
    render_dev_ms = 0.0  # the renders' own device time (CUDA events)
    e0 = time.perf_counter()
    for i in range(e2e_steps):
        t0 = time.perf_counter()
        sid2 = ctx.upload(sd)
        t1 = time.perf_counter()
        info2 = ctx.scene_info(sid2)  # the upload's own split (a few microseconds, outside the parts)
        e0 += time.perf_counter() - t1
        t1 = time.perf_counter()
        r2 = ctx.render(sid2, cam, seed=50 + i, **kw)
        t2 = time.perf_counter()
        render_dev_ms += r2["render_ms"]
        ctx.frame(cam.width, cam.height, out=img)
        t3 = time.perf_counter()
        ctx.release(sid2)
        parts += (t1 - t0, t2 - t1, t3 - t2, time.perf_counter() - t3)
    e2e_s = max_over_ranks(dist, time.perf_counter() - e0)
    e2e_paths = sum_over_ranks(dist, float(paths / args.steps * e2e_steps))

    avg_ext_ms = ext_ms / max(ext_launches, 1)
    achieved = alg_bytes_per_ray * t_ext_rays / (ext_ms / 1000.0) / 1e9 if ext_ms > 0 else None
    peak, peak_kind = load_peaks()
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(pkg, sd, cam, st, target_s=args.cpu_seconds)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "Mpaths/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": render_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "dtype_note": "FP32 arithmetic and hit distances, as the target path specifies; the reference "
                          "computes in FP64 (its Vector3 is double), so parity with it is statistical",
            "data": "synthetic (seeded scene generators)",
            "config": {"workload": desc, "paths_per_step": paths // args.steps,
                       "extension_rays_per_step": ext_rays // args.steps, "triangles": int(info["num_primitives"]),
                       "wide_nodes": int(info["num_nodes"]), "scene_upload_ms": upload_s * 1000.0,
                       "bvh_build_ms": info["build_ms"], "flatten_ms": info["flatten_ms"],
                       "records_env_upload_ms": info["upload_ms"], "l2": "flushed between steps (256 MB write)",
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "wall_s_timed": wall_s, "shadow_rays_per_step": shadow_rays // args.steps,
                       "mrays_per_s": (ext_rays + shadow_rays) / (render_ms / 1000.0) / 1e6,
                       "kernel_split": "extend / shade / shadow device time of one more step with per-kernel "
                                       "CUDA events, all waves on one stream",
                       "extend_ms_per_step": ext_ms, "shade_ms_per_step": shade_ms, "shadow_ms_per_step": shadow_ms,
                       "per_extension_ray": {k: c[k] / max(c["extension_rays"], 1)
                                             for k in ("nodes_visited", "tris_tested", "spheres_tested")}},
            "e2e": {"value": e2e_paths / e2e_s / 1e6, "unit": "Mpaths/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": frame_bytes,
                    "what": "or3_scene_upload (flatten, BVH build, H2D) + or3_render + or3_get_frame per step",
                    "ms_per_step": {k: float(v) * 1000.0 / e2e_steps
                                    for k, v in zip(("upload", "render", "frame", "release"), parts)},
                    "render_device_ms_per_step": render_dev_ms / e2e_steps,
                    "last_upload_ms": {"flatten": info2["flatten_ms"], "flatten_and_bvh": info2["build_ms"],
                                       "records_env": info2["upload_ms"]}},
            "roofline": {"bound": "hbm", "kernel": "k_extend", "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s",
                         "frac": achieved / peak if achieved else None,
                         "traffic": (NCU_EXTEND[args.workload]["dram_bytes_per_ray"] * t_ext_rays /
                                     max(ext_launches, 1) if args.workload in NCU_EXTEND else None),
                         "traffic_unit": "bytes per launch",
                         "traffic_source": (NCU_EXTEND[args.workload]["source"] + ", DRAM bytes per ray scaled "
                                            "to this run's rays per launch" if args.workload in NCU_EXTEND
                                            else None),
                         "alg_bytes_per_launch": alg_bytes_per_ray * t_ext_rays / max(ext_launches, 1),
                         "alg_bytes_per_ray": alg_bytes_per_ray, "avg_launch_ms": avg_ext_ms,
                         "launches": ext_launches,
                         "sm_issue_active_ncu": (NCU_EXTEND[args.workload]["issue_active"]
                                                 if args.workload in NCU_EXTEND else None),
                         "sm_issue_active_source": (NCU_EXTEND[args.workload]["source"]
                                                    if args.workload in NCU_EXTEND else None)},
            "rmse_vs_16k": rmse,
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": launches,
            "gpu_launches_how": "sum of or3_render_stats.kernel_launches over the timed steps (the library "
                                "counts every kernel it launches)",
        }
        print(json.dumps(line), flush=True)
    ctx.release(sid)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
