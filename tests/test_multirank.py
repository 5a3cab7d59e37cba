"""The N-GPU bench path on CPU with gloo (world size 2): frames are independent replicas, the job time
is the slowest rank's total over all ranks' frames, each rank draws its own inputs, and the reference
arm runs on rank 0 only."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, local_sums, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dist.barrier()
        res = bench.job_ms_over_ranks(local_sums[rank], 10, world, "cpu")
        out.put((rank, res))
    finally:
        dist.destroy_process_group()


def test_job_time_is_slowest_rank_over_all_frames():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    sums = [120.0, 200.0]  # ms over 10 timed frames on each rank
    procs = [ctx.Process(target=_rank, args=(r, world, port, sums, q)) for r in range(world)]
    for p in procs:
        p.start()
    results = dict(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert results == {0: pytest.approx(10.0), 1: pytest.approx(10.0)}  # max 200 ms / (10 x 2) frames


def test_single_rank_job_time():
    assert bench.job_ms_over_ranks(50.0, 10, 1, "cpu") == pytest.approx(5.0)


def test_replicas_draw_their_own_inputs(native):
    a = bench.make_inputs(0)
    b = bench.make_inputs(1)
    assert not np.array_equal(a[0], b[0]) and not np.array_equal(a[3], b[3])
    assert np.array_equal(a[5], b[5])  # the radix keys are shared


def test_reference_arm_runs_on_rank_zero_only(capsys):
    class Args:
        steps, warmup = 1, 0
    assert bench.run_reference(Args, 1, 2) is None
    assert capsys.readouterr().out == ""
