"""The N-replica bench path on CPU: two gloo ranks on 127.0.0.1.

bench.py --gpus N runs one replica of the workload per GPU with no data-path
collective; the only collectives are the barrier and the whole-job figures:
the slowest rank's step and end-to-end times (max) and all ranks' converged
solves (sum).  The reference arm runs on rank 0 alone; other ranks return
without work.
"""
import multiprocessing as mp
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, port: int, q) -> None:
    sys.path.insert(0, str(ROOT))
    os.environ.update(RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=2)
    try:
        ws, r, local = bench.dist_env()
        ms, e2e_s, n = bench.reduce_over_ranks(100.0 + 50.0 * rank, 1.0 + rank, 500 + rank, device="cpu")
        # the reference arm: rank 1 returns at once (no build, no work)
        ref = bench.run_reference(None) if rank == 1 else None
        dist.barrier()
        q.put((rank, ws, r, local, ms, e2e_s, n, ref))
    finally:
        dist.destroy_process_group()


def test_two_replicas_reduce_to_whole_job_figures():
    pytest.importorskip("torch")
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
    assert all(p.exitcode == 0 for p in ps), [p.exitcode for p in ps]
    out = sorted(q.get(timeout=10) for _ in range(2))
    for rank, ws, r, local, ms, e2e_s, n, ref in out:
        assert (ws, r, local) == (2, rank, rank)
        assert (ms, e2e_s, n) == (150.0, 2.0, 1001)
        assert ref is None


def test_one_rank_figures_unchanged():
    pytest.importorskip("torch")
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.reduce_over_ranks(12.5, 0.5, 7, device="cpu") == (12.5, 0.5, 7)
