"""Multi-GPU logic on CPU: two gloo ranks as bench.py runs them under
torchrun. The path shards by planes and frames with no exchange, so N GPUs
are N replicas: each rank draws its own seeded batch, and only the timing is
reduced (the slowest rank's time, the sum of all ranks' output samples)."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        jobs, cfg = bench.rank_workload("yuv420_batch", 8, rank)
        px = sum(j["dw"] * j["dh"] for j in jobs)
        ms = bench.max_over_ranks(1.0 + rank)
        total_px = bench.sum_over_ranks(px)
        q.put((rank, [(j["sw"], j["sh"]) for j in jobs], ms, px, total_px))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_replicas_over_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        results = sorted(q.get(timeout=180) for _ in range(2))
    finally:
        for p in procs:
            p.join(timeout=60)
    assert all(p.exitcode == 0 for p in procs)
    (r0, sizes0, ms0, px0, tot0), (r1, sizes1, ms1, px1, tot1) = results
    assert (r0, r1) == (0, 1)
    assert ms0 == ms1 == 2.0                 # the slowest rank's time on every rank
    assert tot0 == tot1 == px0 + px1         # whole-job output samples
    assert sizes0 != sizes1                  # each replica processes its own frames


def test_single_process_reductions_are_identity():
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.sum_over_ranks(7.0) == 7.0
