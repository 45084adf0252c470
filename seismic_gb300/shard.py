"""Multi-process (one process per GPU) helpers.

Pairs are independent, so a catalog shards with no data exchange: rank r of
`world` ranks runs the pair kernel on its own contiguous range of work items
(seismic_pairs_device_range), writing only its pairs of the packed output;
a host-side gather of the slices (or of per-rank catalogs: weak scaling)
completes the job.  The only collective is the timing reduction of
benchmarks (max over ranks).  This replaces the row split of the reference's
multi-GPU variant (Correlation_in_MultiCUDA/correlation_multicuda.cu:157-203)
with an item split that balances work exactly.
"""
from __future__ import annotations


def couple_range(total: int, world: int, rank: int) -> tuple[int, int]:
    """Contiguous, balanced [begin, end) of `total` work items for `rank`."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad world / rank")
    base, extra = divmod(total, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def max_over_ranks(value: float, device=None) -> float:
    """Maximum of `value` over the ranks of the default process group (the
    value itself when torch.distributed is not initialised)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
