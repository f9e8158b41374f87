"""Multi-rank work split on CPU ranks (gloo, world size 2): Gilmore bubbles
sharded by index range and gathered in order give the same rows as one rank;
per-element gradients are summed across ranks.  The per-rank integrator here
is the CPU oracle (no GPU needed)."""
import os
import socket
import tempfile

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _oracle_run(orc, medium, ode):
    from bubbledynamics_gb300 import abi, api

    def run(b):
        if len(b) == 0:
            return np.zeros(0, api.RESULT_DTYPE)
        res = orc.gilmore(medium, (abi.Bubble * len(b)).from_buffer_copy(np.ascontiguousarray(b).tobytes()), ode)
        return np.frombuffer(bytes(res), dtype=api.RESULT_DTYPE).copy()
    return run


def _case():
    from bubbledynamics_gb300 import presets
    med = presets.cfg2_medium()
    b = presets.cfg2_bubbles(37, seed=11)
    b["a"] *= 0.2
    ode = presets.cfg2_ode(t_end=0.2e-6)
    return med, b, ode


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist
    from oracle.oracle import Oracle
    from bubbledynamics_gb300 import shard
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        med, b, ode = _case()
        res = shard.gilmore_sharded(b, _oracle_run(Oracle(), med, ode))
        gp = np.full(5, float(rank + 1))
        ga = np.arange(5, dtype=np.float64) * (rank + 1)
        shard.allreduce_gradients(gp, ga)
        np.save(os.path.join(out_dir, "res%d.npy" % rank), res)
        np.save(os.path.join(out_dir, "grad%d.npy" % rank), np.concatenate([gp, ga]))
    finally:
        dist.destroy_process_group()


def test_shard_range_covers_every_item_once():
    from bubbledynamics_gb300.shard import shard_range
    for n in (0, 1, 5, 37, 1 << 20):
        for world in (1, 2, 3, 8):
            got = [shard_range(n, r, world) for r in range(world)]
            assert got[0][0] == 0 and got[-1][1] == n
            assert all(got[i][1] == got[i + 1][0] for i in range(world - 1))
            sizes = [hi - lo for lo, hi in got]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def test_gilmore_sharded_over_two_gloo_ranks_matches_one_rank():
    import torch.multiprocessing as mp
    from oracle.oracle import Oracle
    med, b, ode = _case()
    single = _oracle_run(Oracle(), med, ode)(b)
    with tempfile.TemporaryDirectory() as d:
        mp.start_processes(_worker, args=(2, _free_port(), d), nprocs=2, start_method="spawn", join=True)
        for r in range(2):
            res = np.load(os.path.join(d, "res%d.npy" % r))
            assert res.dtype == single.dtype and len(res) == len(b)
            for k in ("R", "Rdot", "t", "n_accept", "status"):
                np.testing.assert_array_equal(res[k], single[k])
            g = np.load(os.path.join(d, "grad%d.npy" % r))
            np.testing.assert_array_equal(g[:5], np.full(5, 3.0))
            np.testing.assert_array_equal(g[5:], np.arange(5) * 3.0)
