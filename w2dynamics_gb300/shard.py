"""Chains over several GPUs: partition and host-side reduction.

Markov chains never interact, so a job of many chains shards by chains with
no collective on the data path (the reference runs one chain per MPI rank,
``w2dyn/dmft/cthyb_solver.py:104-108``, and combines the ranks' results
afterwards).  The one exchange is the final reduction of the per-rank
accumulators: G(tau) sums, sign sums and measurement counts, a few hundred
kB, reduced on the host over a CPU process group.
"""
import numpy as np


def chain_range(nchains, rank, world):
    """(first, count) of the chains of `rank` when `nchains` chains are split
    over `world` ranks as evenly as possible (the first nchains % world
    ranks take one more)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(int(nchains), int(world))
    first = rank * base + min(rank, extra)
    return first, base + (1 if rank < extra else 0)


def shard_groups(groups, rank, world):
    """Per group, the (seed0, nchains) of this rank's share; chain c of a
    group keeps seed seed0 + c, so the union over ranks is the unsharded
    job."""
    out = []
    for g in groups:
        first, count = chain_range(g["nchains"], rank, world)
        out.append(dict(g, seed0=g["seed0"] + first, nchains=count))
    return out


def reduce_group_sums(gsum, sign_sum, count, pg=None):
    """Sum G(tau) sums, sign sums and measurement counts over the ranks of
    the CPU process group `pg` (torch.distributed, gloo) and normalise as
    the reference does: G = -Gsum/(-mean_sign)/count * Ntau/beta^2 is left to
    the caller; returned are the global sums."""
    import torch
    import torch.distributed as dist
    g = torch.as_tensor(np.ascontiguousarray(gsum, np.float64)).reshape(-1).clone()
    s = torch.tensor([float(sign_sum), float(count)], dtype=torch.float64)
    if dist.is_available() and dist.is_initialized():
        dist.all_reduce(g, op=dist.ReduceOp.SUM, group=pg)
        dist.all_reduce(s, op=dist.ReduceOp.SUM, group=pg)
    return g.numpy().reshape(np.shape(gsum)), float(s[0]), int(round(float(s[1])))


def max_over_ranks(value, pg=None):
    """Largest `value` over the ranks (step time of the slowest rank)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64)
    if dist.is_available() and dist.is_initialized():
        dist.all_reduce(t, op=dist.ReduceOp.MAX, group=pg)
    return float(t[0])
