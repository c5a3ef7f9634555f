"""Multi-process helpers for running the path as independent replicas.

Specimens are independent, so several GPUs (one process each) split a list of
specimens with no data exchange; the only collective steps are a barrier,
the maximum of the per-rank step times and the gather of per-specimen results
on rank 0 -- host-side bookkeeping, not part of the data path.
"""

from __future__ import annotations

from typing import List, Sequence


def shard(sizes: Sequence[int], world: int, rank: int) -> List[int]:
    """Indices of the specimens this rank processes: largest first, each to the
    rank with the least voxels so far (ties to the lower rank).  Every index is
    assigned to exactly one rank, identically on every rank."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("bad world / rank")
    load = [0] * world
    owner = [0] * len(sizes)
    for i in sorted(range(len(sizes)), key=lambda k: (-int(sizes[k]), k)):
        r = min(range(world), key=lambda q: (load[q], q))
        owner[i] = r
        load[r] += int(sizes[i])
    return [i for i in range(len(sizes)) if owner[i] == rank]


def max_over_ranks(value: float) -> float:
    """Maximum of a float over all ranks of the default process group (identity
    without an initialised group)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_to_rank0(obj):
    """List of every rank's obj on rank 0 (None elsewhere)."""
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return [obj]
    out = [None] * dist.get_world_size() if dist.get_rank() == 0 else None
    dist.gather_object(obj, out, dst=0)
    return out
