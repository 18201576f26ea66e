"""bench.py's multi-rank plumbing on a world of two gloo ranks on the CPU: each
rank's time becomes the maximum over ranks, the barrier releases every rank,
and the reference arm does its work and reports on rank 0 only (the other
ranks return without output)."""

from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, q) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench

    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ws, r, local = bench.dist_info()
        worst = bench.max_over_ranks(torch, 10.0 + 5.0 * rank)
        bench.barrier(torch)
        ref = "rank 0 not run here" if rank == 0 else bench.run_reference(None)
        q.put((rank, ws, r, local, worst, ref))
    finally:
        torch.distributed.destroy_process_group()


def test_two_gloo_ranks_take_the_max_and_only_rank0_reports():
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    codes = [p.exitcode for p in procs]
    for p in procs:
        if p.is_alive():
            p.kill()
    assert codes == [0, 0], codes
    got = sorted(q.get(timeout=5) for _ in range(2))
    assert [g[:4] for g in got] == [(0, 2, 0, 0), (1, 2, 1, 1)]
    assert [g[4] for g in got] == [15.0, 15.0]  # both ranks report the slower rank's time
    assert got[1][5] is None  # rank 1 of the reference arm prints nothing
