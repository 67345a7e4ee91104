"""Phase sharding across independent replicas (one process per GPU).

The per-phase stages have no data dependency between phases (SOAP_integration.cu's
phase loop at :661-845 and SOAP_resolution.cu's at :379-428 only share read-only
inputs), so a job over many phases splits into contiguous phase blocks, one per
rank, with no collective on the data path; results are gathered once at the end.
"""
from __future__ import annotations

from typing import Callable, List, Sequence, Tuple


def phase_shard(n_phase: int, world: int, rank: int) -> Tuple[int, int]:
    """Contiguous block [start, stop) of phases for `rank` (sizes differ by at most one)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad world/rank %d/%d" % (world, rank))
    base, extra = divmod(n_phase, world)
    start = rank * base + min(rank, extra)
    stop = start + base + (1 if rank < extra else 0)
    return start, stop


def run_sharded(n_phase: int, work: Callable[[int, int], list], group=None) -> list:
    """Run `work(start, stop)` on this rank's block and gather every rank's list in
    phase order (torch.distributed, any backend; single process without a group)."""
    try:
        import torch.distributed as dist
        ready = dist.is_available() and dist.is_initialized()
    except Exception:  # pragma: no cover
        ready = False
    if not ready:
        return list(work(0, n_phase))
    world, rank = dist.get_world_size(group), dist.get_rank(group)
    start, stop = phase_shard(n_phase, world, rank)
    mine = list(work(start, stop))
    gathered: List[object] = [None] * world
    dist.all_gather_object(gathered, mine, group=group)
    out: list = []
    for part in gathered:
        out.extend(part)
    return out
