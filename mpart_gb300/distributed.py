"""Host-side pieces of the N-GPU layout (one process per GPU).

The monotone-component path shards by points: Evaluate, LogDeterminant,
Inverse and the coefficient adjoint of a point set need no exchange, so the
benchmark runs one replica per GPU.  The standard-normal KL objective over a
sharded sample set needs one all-reduce: every rank holds the mean loss and
gradient of its own points, and the global means are the point-count weighted
sums.  These helpers run on any torch.distributed backend (NCCL between GPUs,
gloo on CPU for tests)."""
from __future__ import annotations

import numpy as np


def shard_range(n: int, rank: int, world: int):
    """Contiguous share [start, stop) of n points for a rank (sizes differ by at most one)."""
    base, extra = divmod(int(n), int(world))
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def max_over_ranks(value: float, group=None, device="cpu") -> float:
    """Largest value over the ranks (the bench's wall-clock rule)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def sharded_kl_objective(local_loss, local_grad, n_local: int, group=None, device="cpu"):
    """Global per-component KL loss and coefficient gradient from per-rank means
    over n_local points each: one all-reduce of [n_local * loss, n_local * grad, n_local]."""
    import torch
    import torch.distributed as dist
    loss = np.asarray(local_loss, dtype=np.float64).reshape(-1)
    grad = np.asarray(local_grad, dtype=np.float64).reshape(-1)
    buf = torch.as_tensor(np.concatenate([n_local * loss, n_local * grad, [float(n_local)]]), device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=group)
    buf = buf.cpu().numpy()
    n = buf[-1]
    return buf[:loss.size] / n, buf[loss.size:loss.size + grad.size] / n
