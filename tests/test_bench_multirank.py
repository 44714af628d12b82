"""The N>1 path of bench.py on CPU: two gloo ranks on 127.0.0.1.

bench.py runs one process per GPU under torchrun; with GPUs NCCL carries
the max-over-ranks reduction.  Here the same code runs with the gloo
backend (FC_BENCH_BACKEND=gloo): the rank helpers reduce to the maximum and
the reference arm prints exactly one JSON line, from rank 0, with the world
size as n_gpus, while rank 1 exits 0 without work.
"""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank), FC_BENCH_BACKEND="gloo")
    sys.path.insert(0, str(ROOT))
    import bench

    w, r, _ = bench.dist_setup()
    bench.barrier(w)
    q.put((r, bench.reduce_max(10.0 + r, w)))
    import torch.distributed as dist

    dist.destroy_process_group()


def test_rank_helpers_reduce_to_max():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 11.0), (1, 11.0)]


def test_reference_arm_two_ranks_one_line(tmp_path):
    pytest.importorskip("scipy")
    env = dict(os.environ, FC_BENCH_BACKEND="gloo", FC_BENCH_REF_BUDGET_S="5")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", f"--master-port={_free_port()}", str(ROOT / "bench.py"),
           "--impl", "reference", "--config", "c1", "--gpus", "2", "--steps", "2", "--warmup", "3"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2
    assert d["value"] > 0 and d["e2e"]["value"] == d["value"]
    assert d["cpu_baseline"]["kind"] in ("port", "reference")
