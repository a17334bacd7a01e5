"""The bench's multi-rank path on CPU: two gloo ranks on 127.0.0.1.

With N GPUs the bench runs N independent replicas of the workload (the
blocks shard with no data exchanged), times each rank on its own device,
takes the largest time over the ranks and reports the whole job's bytes in
that time; the reference arm runs on rank 0 alone. These tests run the same
functions with a gloo process group instead of NCCL, so no GPU is needed."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, q):
    try:
        sys.path.insert(0, ROOT)
        os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                          WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
        import argparse

        import torch.distributed as dist
        dist.init_process_group("gloo", rank=rank, world_size=world)
        import bench
        # each rank's own step time; the job is as slow as its slowest rank
        slowest = bench.max_over_ranks(0.010 + 0.005 * rank, world, device="cpu")
        value = bench.job_gbs(world, slowest)
        # the reference arm: ranks other than 0 leave without work
        ref = bench.run_reference(argparse.Namespace(steps=1, warmup=0)) if rank else None
        dist.barrier()
        dist.destroy_process_group()
        q.put((rank, slowest, value, ref))
    except Exception as e:  # reported to the parent, which fails the test
        q.put((rank, "error", repr(e), None))


@pytest.mark.timeout(180)
def test_two_gloo_ranks_take_the_slowest_rank_and_whole_job_bytes():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    world = 2
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=150) for _ in range(world))
    for p in procs:
        p.join(timeout=30)
    assert all(p.exitcode == 0 for p in procs)
    sys.path.insert(0, ROOT)
    import bench
    for rank, slowest, value, ref in results:
        assert slowest != "error", value
        assert slowest == pytest.approx(0.015)
        assert value == pytest.approx(world * bench.BYTES_PER_STEP / 0.015 / 1e9)
        assert ref is None


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(0.25, 1) == 0.25
    assert bench.job_gbs(1, 1e-3) == pytest.approx(bench.BYTES_PER_STEP / 1e-3 / 1e9)
