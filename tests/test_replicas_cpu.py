"""Host logic of the multi-GPU bench path on CPU: world_size-2 gloo ranks.

Rays and frames are independent, so N GPUs run N replicas with no collective
on the data path; the only cross-rank steps are the barriers around the timed
region and the max of the ranks' times."""

import os
import socket
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        got_ws, got_rank, _ = bench.dist_env()
        dist.barrier()
        slowest = bench.max_over_ranks(0.5 + rank, got_ws, "cpu")
        dist.barrier()
        q.put((got_rank, got_ws, slowest, bench.replicas_value(1000, 10, got_ws, slowest)))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1]
    assert all(r[1] == 2 for r in res)
    assert all(r[2] == pytest.approx(1.5) for r in res)  # max of 0.5 and 1.5 s
    assert all(r[3] == pytest.approx(1000 * 10 * 2 / 1.5 / 1e6) for r in res)


def test_reference_arm_runs_on_rank0_only():
    class A:
        pass

    assert bench.run_reference(A(), 2, 1) is None
