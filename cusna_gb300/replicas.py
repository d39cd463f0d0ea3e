"""Replicas of the simulator on several GPUs, one process per GPU.

The path shards by chains with no data exchange: rank r simulates the
contiguous chain range [r * M, (r + 1) * M) of one run through
cusna_gpu_options.chain_offset. The Philox counters are keyed by the global
chain index (src/libcusna_saom_cpu.cpp:167, :266), so the split changes no
chain. The only cross-rank step is the timing report: the slowest rank's time
and the sum of the ranks' ministeps (torch.distributed, any backend).
"""
from __future__ import annotations


def chain_range(rank: int, world: int, per_rank: int) -> tuple[int, int]:
    """(chain offset, chain count) of `rank` when every rank runs `per_rank`
    chains (weak scaling)."""
    if not (0 <= rank < world) or per_rank < 1:
        raise ValueError(f"rank {rank} of {world}, {per_rank} chains per rank")
    return rank * per_rank, per_rank


def reduce_timing(total_ms: float, ministeps: float, device=None) -> tuple[float, float]:
    """(slowest rank's time, sum of the ranks' ministeps); the local values when
    torch.distributed is not initialised or has one rank."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(total_ms), float(ministeps)
    t = torch.tensor([float(total_ms)], dtype=torch.float64, device=device)
    m = torch.tensor([float(ministeps)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(m, op=dist.ReduceOp.SUM)
    return float(t.item()), float(m.item())
