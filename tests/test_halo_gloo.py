"""z-slab decomposition on CPU ranks (gloo, world size 2 and 3): every rank
keeps its slab of a field plus 3 ghost planes per internal face and refreshes
them with halo.exchange_halos after every step of a leapfrog with the 6th-order
z stencil of W:169-174 (or 1 ghost plane and the 3-point z stencil of the heat
step, T:72-73); the owned planes equal, bit for bit, the same update on the
whole field.  The message pattern and plane bookkeeping are the ones
halo.run_slab_rank drives between GPUs."""
import os
import socket
import tempfile

import numpy as np
import pytest

torch = pytest.importorskip("torch")

NZ, NY, NX, STEPS = 27, 5, 4, 12


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _d2z(p, width=3):
    """Along axis 0, zero outside: (-490 p + 270 (p[+-1]) - 27 (p[+-2]) + 2 (p[+-3])) / 180
    for width 3, p[+1] - 2 p + p[-1] for width 1."""
    q = np.zeros((p.shape[0] + 6,) + p.shape[1:], p.dtype)
    q[3:-3] = p
    s = lambda k: q[3 + k: q.shape[0] - 3 + k]
    if width == 1:
        return s(1) - 2.0 * p + s(-1)
    return (-490.0 * p + 270.0 * (s(1) + s(-1)) - 27.0 * (s(2) + s(-2)) + 2.0 * (s(3) + s(-3))) / 180.0


def _step(p, pm, width):
    """Leapfrog (width 3) or explicit diffusion (width 1) on whole arrays."""
    if width == 1:
        return p + 0.2 * _d2z(p, 1), p
    return 2.0 * p - pm + 0.1 * _d2z(p, 3), p


def _initial():
    rng = np.random.default_rng(3)
    return rng.standard_normal((NZ, NY, NX)), rng.standard_normal((NZ, NY, NX))


def _whole(width=3):
    p, pm = _initial()
    for _ in range(STEPS):
        p, pm = _step(p, pm, width)
    return p


def _worker(rank, world, port, out_dir, width=3):
    import torch.distributed as dist
    from bubbledynamics_gb300 import halo
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        zb, ze = halo.slab_bounds(NZ, world)[rank]
        lo = zb - width if rank > 0 else 0
        hi = ze + width if rank + 1 < world else NZ
        p0, pm0 = _initial()
        p = np.full((hi - lo, NY, NX), np.nan)
        pm = np.full((hi - lo, NY, NX), np.nan)
        p[zb - lo: ze - lo], pm[zb - lo: ze - lo] = p0[zb:ze], pm0[zb:ze]    # ghosts start unknown
        own = slice(zb - lo, ze - lo)
        nb = width * NY * NX

        def refresh(f):
            send_lo = torch.from_numpy(np.ascontiguousarray(f[own][:width]).reshape(-1))
            send_hi = torch.from_numpy(np.ascontiguousarray(f[own][-width:]).reshape(-1))
            recv_lo, recv_hi = torch.zeros(nb, dtype=torch.float64), torch.zeros(nb, dtype=torch.float64)
            halo.exchange_halos(send_lo, send_hi, recv_lo, recv_hi, rank, world)
            if rank > 0:
                f[:zb - lo] = recv_lo.numpy().reshape(width, NY, NX)
            if rank + 1 < world:
                f[ze - lo:] = recv_hi.numpy().reshape(width, NY, NX)

        refresh(p)
        refresh(pm)
        for _ in range(STEPS):
            new = np.array(p)
            new[own] = _step(p, pm, width)[0][own]
            p, pm = new, p
            refresh(p)
        np.save(os.path.join(out_dir, "slab%d.npy" % rank), p[own])
    finally:
        dist.destroy_process_group()


def test_slab_bounds_cover_the_grid():
    from bubbledynamics_gb300 import halo
    for nz in (16, 27, 256):
        for n in (1, 2, 3):
            if nz < 8 * n:
                continue
            b = halo.slab_bounds(nz, n)
            assert b[0][0] == 0 and b[-1][1] == nz
            assert all(b[i][1] == b[i + 1][0] for i in range(n - 1))
            assert all(ze - zb >= 8 for zb, ze in b)
    with pytest.raises(ValueError):
        halo.slab_bounds(20, 3)


@pytest.mark.parametrize("world,width", [(2, 3), (3, 3), (3, 1)])
def test_halo_exchange_over_gloo_ranks_matches_whole_grid(world, width):
    import torch.multiprocessing as mp
    whole = _whole(width)
    with tempfile.TemporaryDirectory() as d:
        mp.start_processes(_worker, args=(world, _free_port(), d, width), nprocs=world, start_method="spawn",
                           join=True)
        parts = [np.load(os.path.join(d, "slab%d.npy" % r)) for r in range(world)]
    got = np.concatenate(parts, axis=0)
    assert np.isfinite(got).all()
    np.testing.assert_array_equal(got, whole)
