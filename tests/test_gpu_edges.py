"""Edge cases on the GPU: empty inputs (a solve of zero time steps, no
bubbles, no threshold items, a trajectory of zero steps), rows whose pitch is
not a multiple of 16 bytes (the plain step kernel), odd grid sizes that leave
partial tiles at every edge, and the per-cell-condition-free planes next to
tiles that straddle the grid's edge."""
import numpy as np
import pytest

from bubbledynamics_gb300 import abi, api, presets

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_westervelt_zero_steps(ctx):
    """No time step: every output is the initial (zero) state, one domain and slabs."""
    p = presets.cfg1(40, 40, 72, 0, precision=abi.BD_F32)
    r = ctx.westervelt(p, want=("p_final", "peak", "energy"))
    assert r["steps_done"] == 0
    for k in ("p_final", "peak", "energy"):
        assert r[k].shape == (72, 40, 40) and not np.any(r[k]), k
    r3 = ctx.westervelt_slabs(p, 3, want=("p_final", "peak", "energy"))
    for k in ("p_final", "peak", "energy"):
        assert not np.any(r3[k]), k


def test_gilmore_and_threshold_search_without_items(ctx):
    res, ms = ctx.gilmore(presets.cfg2_medium(), np.zeros(0, api.BUBBLE_DTYPE), presets.cfg2_ode(t_end=1e-9))
    assert res.size == 0 and ms == 0.0
    A, ms = ctx.gilmore_threshold(presets.ref_G_medium(), np.zeros((0, 3)), presets.ref_G_R0s()[:4])
    assert A.shape == (0, 4)
    A, ms = ctx.gilmore_threshold(presets.ref_G_medium(), api.gilmore_combos()[:2], np.zeros(0))
    assert A.shape == (2, 0)


@pytest.mark.parametrize("n_slabs", [1, 2])
def test_heat_zero_steps(ctx, n_slabs):
    """Spots of zero duration: no step runs, T and the dose stay at their
    initial values (T:232-257), and a snapshot after the first leg is that state."""
    k = presets.ref_T_mini_constants(Nxy=24, Nz=20, legs=2)
    prob = presets.make_ref_T(k, precision=abi.BD_F64)
    prob.set_spots([0, 3], [0, 1], [0, 0])
    Q = np.full(prob.shape, 1e7)
    r = ctx.heat(prob.thermal, Q, prob.traj, snapshot_legs=[1], n_slabs=n_slabs)
    T0, TD0 = prob.initial_fields()
    assert r["steps_done"] == 0
    np.testing.assert_array_equal(r["T"], T0)
    np.testing.assert_array_equal(r["dose"], TD0)
    np.testing.assert_array_equal(r["snapshots"][0], T0)


@pytest.mark.parametrize("nxy", [21, 23])
def test_odd_row_pitch_takes_the_plain_kernel(ctx, oracle, nxy):
    """Rows of 21 or 23 cells (84 / 92 bytes in FP32, 168 / 184 in FP64: not
    16-byte multiples, like the reference's 426) run the plain step kernel;
    the reference physics against the FP64 oracle, and the TMA variants are
    refused for them."""
    prob = presets.ref_W_mini(abi.BD_F64, Nxy=nxy, Nz=40, loop1_periods=1, periods=1)
    exp = oracle.westervelt(prob)
    got = ctx.westervelt(prob)
    assert got["tile_variant"] == 0
    for k in ("p_final", "peak", "Q"):
        assert rel_l2(got[k], exp[k]) < 1e-9, k
    p32 = presets.ref_W_mini(abi.BD_F32, Nxy=nxy, Nz=40, loop1_periods=1, periods=1)
    p32.params.tile_variant = 21
    with pytest.raises(api.BDError):
        ctx.westervelt(p32)


def test_partial_tiles_at_every_edge(ctx):
    """A 68 x 44 x 50 grid (64 x 8 tiles leave 4 columns and 4 rows over; the
    last z-chunk is short): tiles inside the grid take the per-cell-condition-
    free planes and the tiles that straddle an edge the guarded code; every
    two-cell variant equals the one-cell and the plain kernels bit for bit."""
    base = None
    for v in (0, 17, 19, 20, 21, 22, 23):
        p = presets.cfg1(68, 44, 50, 80, precision=abi.BD_F32)
        p.params.tile_variant = v
        r = ctx.westervelt(p, want=("p_final", "peak", "energy"))
        if base is None:
            base = r
            assert np.abs(base["p_final"]).max() > 0
            continue
        for k in ("p_final", "peak", "energy"):
            np.testing.assert_array_equal(r[k], base[k], err_msg="variant %d, %s" % (v, k))
