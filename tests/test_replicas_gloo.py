"""The multi-rank path of bench.py on CPU (gloo, world size 2).

The path has no exchange step: with N GPUs every rank renders a replica and
the bench reports whole-job throughput = paths over all ranks / the slowest
rank's time.  These tests run the rank plumbing and that aggregation as two
gloo processes on 127.0.0.1, and the reference arm under the launcher (rank 0
alone prints; the other rank exits without work).
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


RANK_SCRIPT = r"""
import json, os, sys
sys.path.insert(0, %(root)r)
import bench
class A: pass
world, rank, local, dist = bench.dist_setup(A())
assert world == 2 and dist is not None and dist.get_backend() == "gloo"
bench.barrier(dist)
seconds = [1.5, 2.0][rank]     # per-rank device time of the timed steps
paths = [3e9, 5e9][rank]       # per-rank camera paths
t = bench.max_over_ranks(dist, seconds)
p = bench.sum_over_ranks(dist, paths)
print(json.dumps({"rank": rank, "max_s": t, "sum_paths": p, "value": p / t / 1e6}))
dist.destroy_process_group()
"""


def test_rank_aggregation_over_gloo(tmp_path):
    script = tmp_path / "rank.py"
    script.write_text(RANK_SCRIPT % {"root": ROOT})
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, WORLD_SIZE="2", RANK=str(r), LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, str(script)], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    for p, (o, e) in zip(procs, outs):
        assert p.returncode == 0, e
    res = [json.loads(o.strip().splitlines()[-1]) for o, _ in outs]
    for r in res:
        assert r["max_s"] == 2.0 and r["sum_paths"] == 8e9
        assert r["value"] == pytest.approx(8e9 / 2.0 / 1e6)


def test_reference_arm_prints_once_under_the_launcher():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "1", "--cpu-seconds", "1", "--workload", "cornell"]
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="", OMP_NUM_THREADS="2")
    r = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["value"] > 0 and line["n_gpus"] == 2
    assert line["e2e"]["h2d_bytes_per_step"] == 0
