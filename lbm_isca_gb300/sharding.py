"""Member sharding across processes (one GPU each).

Members are independent: they share only the basic state and the operators,
so an ensemble splits across ranks with no exchange inside a step.  Each
rank integrates a contiguous block of members; results are gathered on the
host at the end.  The same split is used for weak scaling (fixed members per
rank) and strong scaling (a fixed ensemble divided among ranks).
"""

from __future__ import annotations


def member_block(nmem_total, world, rank):
    """(first, count) of the members rank `rank` integrates."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad world/rank")
    base, extra = divmod(int(nmem_total), int(world))
    first = rank * base + min(rank, extra)
    return first, base + (1 if rank < extra else 0)


def gather_members(local, world, group=None):
    """All-gather per-rank member blocks (torch tensors, member axis first)
    into the full ensemble on every rank; blocks may differ in size."""
    import torch
    import torch.distributed as dist
    if world == 1:
        return local
    n = torch.tensor([local.shape[0]], dtype=torch.int64, device=local.device)
    sizes = [torch.zeros_like(n) for _ in range(world)]
    dist.all_gather(sizes, n, group=group)
    mx = int(max(int(s) for s in sizes))
    pad = torch.zeros((mx,) + tuple(local.shape[1:]), dtype=local.dtype, device=local.device)
    pad[:local.shape[0]] = local
    bufs = [torch.zeros_like(pad) for _ in range(world)]
    dist.all_gather(bufs, pad, group=group)
    return torch.cat([b[:int(s)] for b, s in zip(bufs, sizes)], dim=0)
