"""The multi-rank host logic of bench.py on CPU (gloo, world size 2).

With N GPUs each rank solves its own independent N = 2^20 system (replicas:
the reference's SPMD subtree split is not built), so the only cross-rank step
is the report: the per-step time is the maximum over ranks and only rank 0
prints.  The reference arm under torchrun runs on rank 0 alone; the other
ranks exit 0 without work."""
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


def _rank_main(rank, world, port, values, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        got = bench.max_over_ranks(values[rank], "cpu")
        e2e = bench.max_over_ranks(values[rank] * 2.0, "cpu")
        out.put((rank, got, e2e))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    values = [3.25, 7.5]
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, values, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 7.5, 15.0), (1, 7.5, 15.0)]


def test_max_over_ranks_without_group_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(4.0, "cpu") == 4.0
    assert bench.max_over_ranks(None, "cpu") is None


def test_reference_arm_under_torchrun_prints_once():
    """`--impl reference` launched like the driver's N = 2 run: one JSON line
    from rank 0, exit status 0 on every rank."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--small",
           "--steps", "1", "--warmup", "0"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    p = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, p.stdout
    rec = json.loads(lines[0])
    assert rec["impl"] == "reference" and rec["n_gpus"] == 2
    assert rec["value"] > 0 and rec["e2e"]["value"] == rec["value"]
    assert rec["cpu_baseline"]["kind"] == "port"
