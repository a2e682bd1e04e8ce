"""The N > 1 host path of bench.py on CPU with the gloo backend (two ranks):
process-group setup from the torchrun environment, the barrier, the maximum
over ranks of the timed region, and the reference arm's rank-0-only output.
The GPU arm's replicas have no data-path collective (one independent solve
per GPU), so these are the only multi-rank parts."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, q):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(ws),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "AXG_BENCH_BACKEND": "gloo"})
    sys.path.insert(0, str(ROOT))
    import bench
    got_ws, got_rank, _ = bench.dist_init()
    bench.barrier(got_ws)
    m = bench.max_over_ranks(1.5 + rank, got_ws)
    import torch.distributed as dist
    dist.destroy_process_group()
    q.put((got_rank, got_ws, m))


def test_two_ranks_reduce_the_maximum():
    torch = pytest.importorskip("torch")
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 2, 2.5), (1, 2, 2.5)]


def test_reference_arm_under_torchrun_prints_once():
    pytest.importorskip("torch")
    env = dict(os.environ, AXG_BENCH_BACKEND="gloo")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_port()), str(ROOT / "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1", "--size", "64"]
    r = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
