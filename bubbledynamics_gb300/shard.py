"""Work split across ranks (one process per GPU, torch.distributed).

The solvers themselves run on one GPU each; what shards is the work:

* Gilmore bubbles are independent (the launch of G:573 is one thread per
  item), so rank r integrates a contiguous index range and the result rows are
  gathered in index order — no collective on the data path beyond the final
  gather.
* Phased-array gradients are sums over source cells, so ranks that each
  handle part of an ensemble (several foci, several media) add their
  per-element gradients with one all-reduce of 2 x n_elements doubles.

Everything here is host logic; `run` is the per-rank integrator (for example
`lambda b: ctx.gilmore(medium, b, ode)[0]`).
"""
import numpy as np


def shard_range(n, rank, world):
    """Contiguous [lo, hi) of n items for `rank` of `world`; the first n % world
    ranks take one item more."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("bad rank %r of world %r" % (rank, world))
    base, extra = divmod(int(n), int(world))
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def gilmore_sharded(bubbles, run, group=None):
    """Runs this rank's range of `bubbles` through `run` and gathers every
    rank's result rows (a numpy structured array, in index order) on all
    ranks.  Without an initialised process group it is a plain call."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return run(bubbles)
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    lo, hi = shard_range(len(bubbles), rank, world)
    mine = run(bubbles[lo:hi])
    parts = [None] * world
    dist.all_gather_object(parts, (lo, mine.tobytes(), mine.dtype.descr), group=group)
    out = None
    for lo_r, raw, descr in sorted(parts, key=lambda p: p[0]):
        arr = np.frombuffer(raw, dtype=np.dtype(descr))
        out = arr.copy() if out is None else np.concatenate([out, arr])
    return out


def allreduce_gradients(grad_phase, grad_amp, group=None):
    """Sum of per-element gradients over ranks (in place on float64 arrays)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return grad_phase, grad_amp
    t = torch.from_numpy(np.concatenate([grad_phase, grad_amp]).astype(np.float64))
    if dist.get_backend(group) == "nccl":     # NCCL reduces device tensors only
        t = t.to(torch.device("cuda", torch.cuda.current_device()))
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    t = t.cpu()
    n = len(grad_phase)
    grad_phase[:] = t[:n].numpy()
    grad_amp[:] = t[n:].numpy()
    return grad_phase, grad_amp
