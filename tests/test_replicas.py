"""Replicas on several GPUs (cusna_gb300.replicas): the chain ranges of the
ranks tile one run without overlap, and the timing report is the slowest
rank's time with the ministeps summed, over torch.distributed (gloo, two
processes on the CPU; the GPU runs use the same calls over NCCL)."""
import os
import socket

import pytest

from cusna_gb300.replicas import chain_range, reduce_timing


def test_chain_ranges_tile_the_run():
    world, per = 4, 1024
    seen = []
    for r in range(world):
        off, cnt = chain_range(r, world, per)
        seen.extend(range(off, off + cnt))
    assert seen == list(range(world * per))
    with pytest.raises(ValueError):
        chain_range(4, 4, 10)


def test_reduce_timing_single_process_is_identity():
    assert reduce_timing(12.5, 1000) == (12.5, 1000.0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = [100.0, 130.0][rank]
        steps = [6_500_000, 6_400_000][rank]
        out[rank] = reduce_timing(ms, steps)
    finally:
        dist.destroy_process_group()


def test_reduce_timing_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    assert out[0] == out[1] == (130.0, 12_900_000.0)
