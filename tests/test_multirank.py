"""The replicas-only multi-GPU path of bench.py, on CPU: world_size 2 over
gloo.  Each rank assembles its own problem, the job's step time is the
largest rank's, the job's throughput counts every rank's units, and the
reference arm runs on rank 0 alone."""
import io
import os
import socket
import contextlib

import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 1.0 + 2.0 * rank  # rank 1 is the slow one
        job_ms = bench.max_over_ranks(ms, dist, "cpu")
        out[rank] = (job_ms, bench.job_rate(1000, world, job_ms))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_job_rate_gloo():
    world = 2
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1] == (3.0, 2 * 1000 / 3.0e-3)


def test_single_rank_is_identity():
    assert bench.max_over_ranks(2.5) == 2.5
    assert bench.job_rate(10, 1, 1.0) == 10 / 1e-3


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("LOCAL_RANK", "1")

    class Args:
        steps, warmup = 1, 3

    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.run_reference(Args())
    assert buf.getvalue() == ""
