"""The multi-rank path of bench.py on CPU: two gloo ranks (replicas).

bench.py under torchrun runs one replica per GPU; the job's time is the slowest
rank's (all-reduce MAX) and its value counts every rank's work.  The reference
arm runs on rank 0 alone; the other ranks exit without work.  Host logic only.
"""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


RANK_SCRIPT = r"""
import os, sys, json
sys.path.insert(0, {root!r})
import torch.distributed as dist
import bench
dist.init_process_group("gloo", init_method="env://")
ws, rank, _ = bench.dist_env()
t = bench.max_over_ranks(0.5 + rank, ws)            # rank 1 is the slow one
v = bench.job_gteps(ws, 2.0e9, 10, t)
print(json.dumps({{"rank": rank, "ws": ws, "t": t, "v": v}}), flush=True)
dist.barrier()
dist.destroy_process_group()
"""


def _run_ranks(script, ws=2):
    port = _free_port()
    procs = []
    for r in range(ws):
        env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(ws), RANK=str(r),
                   LOCAL_RANK=str(r))
        procs.append(subprocess.Popen([sys.executable, "-c", script], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=120)
        assert p.returncode == 0, e
        outs.append(o)
    return outs


def test_max_over_ranks_and_job_value():
    import json
    outs = _run_ranks(RANK_SCRIPT.format(root=ROOT))
    rows = [json.loads(o.strip().splitlines()[-1]) for o in outs]
    for r in rows:
        assert r["ws"] == 2
        assert r["t"] == 1.5                            # the slowest rank's time on every rank
        assert abs(r["v"] - 2 * 2.0e9 * 10 / 1.5 / 1e9) < 1e-9  # both replicas' work


def test_single_rank_is_unchanged():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(0.25, 1) == 0.25
    assert bench.job_gteps(1, 1.0e9, 4, 2.0) == 2.0


def test_reference_arm_only_on_rank_zero():
    """Rank 1 of the reference arm returns at once and prints nothing."""
    script = (f"import sys; sys.path.insert(0, {ROOT!r}); import bench, types; "
              "bench.run_reference(types.SimpleNamespace(scale=20, sources=512, steps=1, warmup=1))")
    env = dict(os.environ, WORLD_SIZE="2", RANK="1", LOCAL_RANK="1")
    p = subprocess.run([sys.executable, "-c", script], env=env, capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stderr
    assert p.stdout.strip() == ""
