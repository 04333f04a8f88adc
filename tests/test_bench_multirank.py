"""The bench's N > 1 path on CPU: replicas with no data-path collective,
timed as the slowest rank (max over ranks), the reference arm printing one
line from rank 0 -- exercised with gloo ranks on this host."""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    t = bench.max_over_ranks(0.010 * (rank + 1), ws)   # rank 1 is slower
    r = bench.replica_rate(1_000_000, t, ws)
    out.put((rank, t, r))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # both ranks see the slowest rank's time; the job rate counts both replicas
    assert [t for _, t, _ in res] == [pytest.approx(0.020)] * 2
    assert [r for _, _, r in res] == [pytest.approx(2 * 1_000_000 / 0.020 / 1e6)] * 2


def test_reference_arm_two_ranks():
    """torchrun with two ranks: rank 0 times the CPU implementation and
    prints the one JSON line, rank 1 exits 0 without work"""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "Mpx/s" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] in ("port", "reference")
