"""Shot-parallel runs over several processes (one GPU each).

Independent shots shard with no exchange during the time loop: each rank
takes a contiguous block of the shot list, runs it as one batch on its GPU,
and the seismograms are gathered on rank 0 at the end -- the only
collective of the run.
"""

import numpy as np


def shard(nshot, rank, world):
    """Shot indices of `rank` among `world` ranks: contiguous blocks, sizes
    differing by at most one, every shot in exactly one block."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d of world %d" % (rank, world))
    base, extra = divmod(int(nshot), int(world))
    start = rank * base + min(rank, extra)
    return list(range(start, start + base + (1 if rank < extra else 0)))


def gather_to_root(local, rank, world, group=None):
    """Gather a picklable object from every rank on rank 0 (torch.distributed
    gather_object over the initialised process group, any backend).  Returns
    the list of the ranks' objects on rank 0, None elsewhere; with one rank,
    [local]."""
    if world == 1:
        return [local]
    import torch.distributed as dist
    out = [None] * world if rank == 0 else None
    dist.gather_object(local, out, dst=0, group=group)
    return out


def traces(problem):
    """The station seismograms of a problem as (nrecv, ncmp, max_nt)."""
    r = problem.recv
    return np.asarray(r["seismo"]).reshape(r["n"], r["ncmp"], r["max_nt"])
