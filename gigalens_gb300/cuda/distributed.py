"""Data parallelism over GPUs, one process per GPU (``torch.distributed``).

The reference's JAX substrate spreads the modelling sequence over devices with
``pmap`` (``gigalens/jax/inference.py:52-62`` MAP, ``:112-117`` SVI,
``:163-190`` HMC).  Chains are independent units, so:

* MAP and HMC shard the chains over ranks and exchange nothing while they run;
  the best MAP chain and the HMC samples are gathered once at the end;
* SVI averages the ELBO and its gradient over ranks every step (the one real
  exchange: ``d + d(d+1)/2`` floats plus the loss), each rank drawing its own
  ``n_vi / world`` samples.

Every helper is a no-op in a single process, so the drivers call them
unconditionally.  The process group is the caller's (NCCL on GPUs; the tests
use gloo on the CPU).
"""
from typing import Tuple

import torch


def rank_world() -> Tuple[int, int]:
    """(rank, world size) of the default process group, (0, 1) without one."""
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized():
        return dist.get_rank(), dist.get_world_size()
    return 0, 1


def shard_range(n: int, rank: int = None, world: int = None) -> Tuple[int, int]:
    """Contiguous ``[start, stop)`` of ``n`` units owned by ``rank``; the first
    ``n % world`` ranks take one extra unit."""
    if rank is None or world is None:
        rank, world = rank_world()
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def allreduce_mean_(t: torch.Tensor) -> torch.Tensor:
    """In-place mean over ranks."""
    import torch.distributed as dist

    _, world = rank_world()
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        t.div_(world)
    return t


def gather_chains(x: torch.Tensor, dim: int = 0) -> torch.Tensor:
    """Concatenate every rank's chains along ``dim`` in rank order (shards may
    differ in size by one, as ``shard_range`` makes them)."""
    import torch.distributed as dist

    _, world = rank_world()
    if world == 1:
        return x
    n = torch.tensor([x.shape[dim]], dtype=torch.int64, device=x.device)
    sizes = [torch.zeros_like(n) for _ in range(world)]
    dist.all_gather(sizes, n)
    sizes = [int(s) for s in sizes]
    m = max(sizes)
    pad_shape = list(x.shape)
    pad_shape[dim] = m - x.shape[dim]
    xp = torch.cat([x, x.new_zeros(pad_shape)], dim=dim) if pad_shape[dim] else x.contiguous()
    parts = [torch.empty_like(xp) for _ in range(world)]
    dist.all_gather(parts, xp.contiguous())
    return torch.cat([p.narrow(dim, 0, s) for p, s in zip(parts, sizes)], dim=dim)


def global_best(z: torch.Tensor, logp: torch.Tensor) -> torch.Tensor:
    """The chain with the highest finite log posterior over all ranks (the
    reference picks ``argmax`` of the MAP log posterior before SVI); every rank
    receives it."""
    import torch.distributed as dist

    lp = torch.nan_to_num(logp.detach().reshape(-1), nan=-float("inf"))
    _, world = rank_world()
    if lp.numel() == 0:
        # an empty shard (fewer chains than ranks) still takes part in the
        # exchange, with -inf so that it never wins
        if world == 1:
            raise ValueError("global_best: no chains")
        best = z.new_zeros(z.shape[1:])
        val = torch.full((1,), -float("inf"), dtype=lp.dtype, device=lp.device)
    else:
        i = int(torch.argmax(lp))
        best = z[i].detach().clone()
        if world == 1:
            return best
        val = lp[i].reshape(1).clone()
    vals = [torch.empty_like(val) for _ in range(world)]
    dist.all_gather(vals, val)
    winner = int(torch.argmax(torch.cat(vals)))
    dist.broadcast(best, src=winner)
    return best
