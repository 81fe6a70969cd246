"""Multi-process paths on CPU (gloo, world size 2).

The plain path runs as independent replicas, one per GPU (no collective on the data path);
bench.py combines the ranks with two host reductions: the max over ranks of the timed
duration and the sum of ion-steps. These tests run those reductions over gloo, and run the
reference arm of bench.py under torchrun with two ranks (rank 0 alone measures and prints).
"""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": "2", "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench

    d = bench.Dist("gloo")
    t = [3.0, 5.0][rank]
    ions = [100.0, 200.0][rank]
    out.put((rank, d.reduce(t, "max"), d.reduce(ions, "sum")))
    d.barrier()
    d.close()


def test_rank_reductions_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29511
    procs = [ctx.Process(target=_worker, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, tmax, ions in res:
        assert tmax == 5.0 and ions == 300.0


def test_reference_arm_two_ranks():
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", "29512", "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0", "--workload", "small_plain",
           "--cpu-sample-targets", "16"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["n_gpus"] == 2
