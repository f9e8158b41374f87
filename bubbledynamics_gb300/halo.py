"""z-slab decomposition of the Westervelt and heat solves across ranks.

The reference runs one grid on one device (W:353).  Here a grid of nz planes
is split into contiguous slabs of whole planes, one per rank; each rank keeps 3
ghost planes beyond each internal face (the 6th-order stencil reads p^n at
iz +- 3, W:169-174) and refreshes them after every step with one message to
and one from each neighbour.  Everything else a step reads is cell-local, and
the peak, energy and DFT maps are per cell, so nothing else is exchanged.

* `slab_bounds(nz, n)` — the [z_begin, z_end) of each slab.
* `exchange_halos(...)` — the per-step message pattern over torch.distributed
  (NCCL for device tensors, gloo for host tensors): send the owned boundary
  planes down and up, receive the ghost planes from below and above.
* `run_slab_rank(ctx, prob)` — one rank's solve: slab session, one step at a
  time, pack / exchange / unpack through the library's halo copies.
* `run_slabs_local(ctx, prob, n)` — the same data path for n slabs held by one
  process on one device (the buffers are handed over in place of messages).
* `run_heat_slab_rank(...)`, `run_heat_slabs_local(...)` — the same for the
  heat run, whose 7-point stencil reaches one plane (T:72-73): one ghost plane
  per internal face, slabs of at least 2 planes.
"""
import numpy as np

HALO = 3


def slab_bounds(nz, n):
    """[z_begin, z_end) of n slabs of nz planes, as equal as whole planes allow
    (the split bd_westervelt_run_slabs uses)."""
    if n < 1 or nz < 8 * n:
        raise ValueError("%d planes cannot make %d slabs of at least 8 planes" % (nz, n))
    return [(nz * k // n, nz * (k + 1) // n) for k in range(n)]


def exchange_halos(send_lo, send_hi, recv_lo, recv_hi, rank, world, group=None):
    """One halo refresh: send_lo goes to rank - 1 and send_hi to rank + 1,
    recv_lo comes from rank - 1 and recv_hi from rank + 1 (the end ranks skip
    their missing neighbour).  All four are tensors of the same size, on the
    device for NCCL or on the host for gloo."""
    import torch.distributed as dist
    ops = []
    if rank > 0:
        ops.append(dist.P2POp(dist.isend, send_lo, rank - 1, group))
        ops.append(dist.P2POp(dist.irecv, recv_lo, rank - 1, group))
    if rank + 1 < world:
        ops.append(dist.P2POp(dist.isend, send_hi, rank + 1, group))
        ops.append(dist.P2POp(dist.irecv, recv_hi, rank + 1, group))
    if ops:
        for r in dist.batch_isend_irecv(ops):
            r.wait()


def _halo_buffers(session, n):
    import torch
    nbytes = session.halo_bytes()
    return [torch.empty(nbytes, dtype=torch.uint8, device="cuda") for _ in range(n)]


def run_slab_rank(ctx, prob, group=None, want=("p_final", "peak", "energy", "Q", "dft")):
    """This rank's slab of prob, stepped with a halo refresh after every step
    over torch.distributed; returns its owned planes (see
    WesterveltSession.finish).  The halo copies run on torch's current stream,
    after the step (advance() returns once the step is done) and before the
    messages."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    zb, ze = slab_bounds(prob.grid.nz, world)[rank]
    s = ctx.westervelt_slab(prob, zb, ze)
    send_lo, send_hi, recv_lo, recv_hi = _halo_buffers(s, 4)
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(prob.params.n_steps):
        s.advance(1)
        if rank > 0:
            s.halo_copy(0, 0, send_lo.data_ptr(), stream)
        if rank + 1 < world:
            s.halo_copy(1, 0, send_hi.data_ptr(), stream)
        exchange_halos(send_lo, send_hi, recv_lo, recv_hi, rank, world, group)
        if rank > 0:
            s.halo_copy(0, 1, recv_lo.data_ptr(), stream)
        if rank + 1 < world:
            s.halo_copy(1, 1, recv_hi.data_ptr(), stream)
        torch.cuda.current_stream().synchronize()
    out = s.finish(want)
    s.close()
    return out


def run_slabs_local(ctx, prob, n_slabs, want=("p_final", "peak", "energy", "Q")):
    """n_slabs slab sessions of prob in this process, stepped in lockstep; the
    halo planes travel through device buffers exactly as run_slab_rank's
    messages do (pack, hand over, unpack).  Returns the whole grid's maps."""
    import torch
    bounds = slab_bounds(prob.grid.nz, n_slabs)
    slabs = [ctx.westervelt_slab(prob, zb, ze) for zb, ze in bounds]
    bufs = [_halo_buffers(s, 2) for s in slabs]      # [k][0]: going down, [k][1]: going up
    stream = torch.cuda.current_stream().cuda_stream
    try:
        for _ in range(prob.params.n_steps):
            for s in slabs:
                s.advance(1)
            for k, s in enumerate(slabs):
                if k > 0:
                    s.halo_copy(0, 0, bufs[k][0].data_ptr(), stream)
                if k + 1 < n_slabs:
                    s.halo_copy(1, 0, bufs[k][1].data_ptr(), stream)
            for k, s in enumerate(slabs):
                if k > 0:
                    s.halo_copy(0, 1, bufs[k - 1][1].data_ptr(), stream)     # from the slab below
                if k + 1 < n_slabs:
                    s.halo_copy(1, 1, bufs[k + 1][0].data_ptr(), stream)     # from the slab above
            torch.cuda.current_stream().synchronize()
        parts = [s.finish(want) for s in slabs]
    finally:
        for s in slabs:
            s.close()
    return {k: np.concatenate([p[k] for p in parts], axis=0) for k in parts[0] if k != "steps_done"}


def heat_slab_bounds(nz, n):
    """[z_begin, z_end) of n heat slabs of nz planes (the split
    bd_spiral_heat_run_slabs uses; at least 2 planes each)."""
    if n < 1 or nz < 2 * n:
        raise ValueError("%d planes cannot make %d slabs of at least 2 planes" % (nz, n))
    return [(nz * k // n, nz * (k + 1) // n) for k in range(n)]


def _heat_refresh(slabs, bufs, stream):
    """Ghost planes of neighbouring heat slabs of one process through device
    buffers: pack every slab's boundary planes, then unpack the neighbours'."""
    n = len(slabs)
    for k, s in enumerate(slabs):
        if k > 0:
            s.halo_copy(0, 0, bufs[k][0].data_ptr(), stream)
        if k + 1 < n:
            s.halo_copy(1, 0, bufs[k][1].data_ptr(), stream)
    for k, s in enumerate(slabs):
        if k > 0:
            s.halo_copy(0, 1, bufs[k - 1][1].data_ptr(), stream)     # from the slab below
        if k + 1 < n:
            s.halo_copy(1, 1, bufs[k + 1][0].data_ptr(), stream)     # from the slab above


def run_heat_slab_rank(ctx, thermal, Q, traj, max_steps=0, group=None):
    """This rank's slab of the heat run, stepped with a ghost-plane refresh
    after every step over torch.distributed; returns its owned planes of T and
    the dose (see HeatSlab.finish)."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    zb, ze = heat_slab_bounds(thermal.nz, world)[rank]
    s = ctx.heat_slab(thermal, Q, traj, zb, ze, max_steps)
    send_lo, send_hi, recv_lo, recv_hi = _halo_buffers(s, 4)
    stream = torch.cuda.current_stream().cuda_stream
    total, _ = s.steps()
    for _ in range(total):
        s.advance(1)
        if rank > 0:
            s.halo_copy(0, 0, send_lo.data_ptr(), stream)
        if rank + 1 < world:
            s.halo_copy(1, 0, send_hi.data_ptr(), stream)
        exchange_halos(send_lo, send_hi, recv_lo, recv_hi, rank, world, group)
        if rank > 0:
            s.halo_copy(0, 1, recv_lo.data_ptr(), stream)
        if rank + 1 < world:
            s.halo_copy(1, 1, recv_hi.data_ptr(), stream)
        torch.cuda.current_stream().synchronize()
    out = s.finish()
    s.close()
    return out


def run_heat_slabs_local(ctx, thermal, Q, traj, n_slabs, max_steps=0):
    """n_slabs heat slabs in this process, stepped in lockstep, the ghost planes
    travelling through device buffers as run_heat_slab_rank's messages do.
    Returns the whole grid's T and dose."""
    import torch
    bounds = heat_slab_bounds(thermal.nz, n_slabs)
    slabs = [ctx.heat_slab(thermal, Q, traj, zb, ze, max_steps) for zb, ze in bounds]
    bufs = [_halo_buffers(s, 2) for s in slabs]      # [k][0]: going down, [k][1]: going up
    stream = torch.cuda.current_stream().cuda_stream
    try:
        total, _ = slabs[0].steps()
        for _ in range(total):
            for s in slabs:
                s.advance(1)
            _heat_refresh(slabs, bufs, stream)
            torch.cuda.current_stream().synchronize()
        parts = [s.finish() for s in slabs]
    finally:
        for s in slabs:
            s.close()
    return {k: np.concatenate([p[k] for p in parts], axis=0) for k in ("T", "dose")}
