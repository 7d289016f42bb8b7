"""bench.py's N>1 path on CPU: two gloo ranks stand in for two GPUs.

The path does not shard (replicas only): every rank runs its own copy of the
workload, and the reported value is all ranks' cell-updates over the slowest
rank's time.  The reference arm runs on rank 0 only; other ranks exit 0."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, ws: int, port: int, out) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        bench.dist_barrier(ws)
        # rank r took (r+1)*10 ms for 3 steps of a 64x64 replica
        v = bench.replica_value(64 * 64, 3, 10.0 * (rank + 1), ws)
        m = bench.dist_max(float(rank), ws)

        class A:
            n, steps, warmup = 64, 1, 0
        rc = bench.run_reference(A, ws, rank) if rank == 1 else 0
        out.put((rank, v, m, rc))
    finally:
        dist.destroy_process_group()


def test_replica_aggregation_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    expect = 2 * 64 * 64 * 3 / 0.020  # both ranks' work over the slower rank's 20 ms
    for rank, v, m, rc in res:
        assert v == pytest.approx(expect)
        assert m == 1.0
        assert rc == 0
