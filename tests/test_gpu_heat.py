"""Bioheat + CEM43 dose on the GPU against the reference's own kernel
(fixture) and the CPU oracle."""
import numpy as np
import pytest

from bubbledynamics_gb300 import abi, api, presets
from tests.conftest import golden_path

pytestmark = pytest.mark.gpu


def mini():
    from tests.golden.make_golden import t_mini_inputs
    return t_mini_inputs()


def test_heat_f64_matches_reference_fixture(ctx):
    g = np.load(golden_path("T_mini.npz"))
    k, prob, sx, sy, Q = mini()
    r = ctx.heat(prob.thermal, Q, prob.traj)
    assert r["steps_done"] == int(g["n_steps"])
    np.testing.assert_allclose(r["T"], g["T"], rtol=1e-13, atol=0)
    np.testing.assert_allclose(r["dose"], g["TD"], rtol=1e-11, atol=0)


def test_heat_f32_close_to_oracle(ctx, oracle):
    k, prob, sx, sy, Q = mini()
    T0, TD0 = prob.initial_fields()
    To, TDo, _ = oracle.heat(prob.thermal, Q, sx, sy, T0, TD0)
    p32 = presets.make_ref_T(k, precision=abi.BD_F32)
    r = ctx.heat(p32.thermal, Q, p32.traj)
    rise = To.reshape(prob.shape) - T0
    err_T = np.abs(r["T"] - To.reshape(prob.shape)).max() / np.abs(rise).max()
    err_D = np.abs(r["dose"] - TDo.reshape(prob.shape)).max() / np.abs(TDo).max()
    print("heat f32: max |dT| error / max rise %.3g, dose %.3g" % (err_T, err_D))
    assert err_T < 1e-5
    assert err_D < 1e-5


def test_heat_snapshots_and_spots(ctx, oracle):
    k, prob, sx, sy, Q = mini()
    prob.set_spots([0, 4, -3], [0, 2, 5], [40, 30, 25])
    ssx, ssy, legs = api.trajectory_shifts(prob.traj)
    T0, TD0 = prob.initial_fields()
    To, TDo, snaps = oracle.heat(prob.thermal, Q, ssx, ssy, T0, TD0, snap_steps=[40, 70])
    r = ctx.heat(prob.thermal, Q, prob.traj, snapshot_legs=[1, 2])
    np.testing.assert_allclose(r["snapshots"][0].reshape(-1), snaps[0], rtol=1e-13)
    np.testing.assert_allclose(r["snapshots"][1].reshape(-1), snaps[1], rtol=1e-13)
    np.testing.assert_allclose(r["T"].reshape(-1), np.asarray(To).reshape(-1), rtol=1e-13)


def test_pennes_perfusion_decay(ctx):
    """No source, uniform excess temperature: T - T_art decays as (1 - w dt)^n."""
    k, prob, sx, sy, Q = mini()
    for m in range(prob.thermal.n_materials):
        prob.thermal.mat[m].perfusion = 0.5
        prob.thermal.mat[m].T_art = 310.0
        prob.thermal.mat[m].T_init = 315.0
        prob.thermal.mat[m].k_t = 0.0
    prob.set_spots([0], [0], [200])
    r = ctx.heat(prob.thermal, np.zeros(prob.shape), prob.traj, want_dose=False)
    expect = 310.0 + 5.0 * (1.0 - 0.5 * prob.thermal.dt) ** 200
    inner = r["T"][1:-1, 1:-1, 1:-1]
    np.testing.assert_allclose(inner, expect, rtol=1e-12)


def test_cem43_constant_temperatures(ctx):
    """Constant 44 C for 1 s adds 2 s of dose per second, 42 C adds 0.25 s/s."""
    k, prob, sx, sy, Q = mini()
    for T_c, rate in ((44.0, 2.0), (42.0, 0.25)):
        for m in range(prob.thermal.n_materials):
            prob.thermal.mat[m].T_init = 273.15 + T_c
            prob.thermal.mat[m].k_t = 0.0
        prob.thermal.dose_init = 0
        prob.set_spots([0], [0], [1000])
        r = ctx.heat(prob.thermal, np.zeros(prob.shape), prob.traj)
        inner = r["dose"][1:-1, 1:-1, 1:-1]
        np.testing.assert_allclose(inner, rate * 1.0, rtol=1e-9)


@pytest.mark.parametrize("precision", [abi.BD_F32, abi.BD_F64])
def test_heat_graph_and_plain_launches_identical(ctx, precision):
    """The step loop replayed as captured CUDA graphs (one per chunk parity)
    and launched kernel by kernel give the same bits, with snapshots that
    split the run at odd steps and chunks that end part-way."""
    k, _, _, _, Q = mini()
    res = []
    for plain in (0, 1):
        prob = presets.make_ref_T(k, precision=precision)
        prob.set_spots([0, 4, -3], [0, 2, 5], [101, 70, 200])
        prob.thermal.plain_launches = plain
        r = ctx.heat(prob.thermal, Q, prob.traj, snapshot_legs=[1, 2])
        assert r["steps_done"] == 371
        res.append(r)
    for key in ("T", "dose", "snapshots"):
        np.testing.assert_array_equal(res[0][key], res[1][key], err_msg=key)


@pytest.mark.parametrize("precision,nxy,plain", [(abi.BD_F32, 44, 0), (abi.BD_F32, 41, 1), (abi.BD_F64, 41, 0)])
def test_heat_slabs_equal_single_domain(ctx, precision, nxy, plain):
    """The z-slab split of the heat run: 2, 3 and 7 slabs, each with its own
    buffers and one ghost plane per internal face refreshed after every step,
    give the one-domain temperature, dose and snapshots bit for bit.  Covers
    the four-cell FP32 kernel (nx % 4 == 0), the scalar FP32 and FP64 kernels,
    graphs and plain launches, snapshots at odd steps, the water/tissue plane
    materials and a per-cell material map."""
    k = presets.ref_T_mini_constants(Nxy=nxy, Nz=40, legs=2)
    Q = presets.gaussian_focus_Q((40, nxy, nxy), (22, 20, 20), (3.0, 2.0, 2.0), 4.0e7)
    rng = np.random.default_rng(5)
    mm = (rng.random((40, nxy, nxy)) < 0.5).astype(np.uint8)
    for with_map in (False, True):
        res = {}
        for n_slabs in (1, 2, 3, 7):
            prob = presets.make_ref_T(k, precision=precision)
            prob.set_spots([0, 4, -3], [0, 2, 5], [101, 70, 60])
            prob.thermal.plain_launches = plain
            if with_map:
                prob.set_material_map(mm)
            res[n_slabs] = ctx.heat(prob.thermal, Q, prob.traj, snapshot_legs=[1, 2], n_slabs=n_slabs)
        assert res[1]["steps_done"] == 231
        assert np.abs(res[1]["snapshots"][1] - res[1]["snapshots"][0]).max() > 0   # the source heats
        for n_slabs in (2, 3, 7):
            for key in ("T", "dose", "snapshots"):
                np.testing.assert_array_equal(res[n_slabs][key], res[1][key],
                                              err_msg="%d slabs, %s, map %s" % (n_slabs, key, with_map))


def test_heat_slab_count_checked(ctx):
    k, prob, sx, sy, Q = mini()
    with pytest.raises(api.BDError):
        ctx.heat(prob.thermal, Q, prob.traj, n_slabs=prob.thermal.nz)   # fewer than 2 planes per slab


@pytest.mark.parametrize("precision,nxy", [(abi.BD_F32, 44), (abi.BD_F64, 41)])
def test_heat_slab_sessions_through_halo_buffers(ctx, precision, nxy):
    """The data path of a multi-rank heat run (each slab its own session,
    stepped one step at a time; pack the owned boundary plane into a device
    buffer, hand it over, unpack into the neighbour's ghost plane) for 2 and 3
    slab sessions in this process: the one-domain T and dose bit for bit."""
    torch = pytest.importorskip("torch")
    from bubbledynamics_gb300 import halo
    k = presets.ref_T_mini_constants(Nxy=nxy, Nz=30, legs=2)
    Q = presets.gaussian_focus_Q((30, nxy, nxy), (16, 20, 20), (3.0, 2.0, 2.0), 4.0e7)

    def problem():
        prob = presets.make_ref_T(k, precision=precision)
        prob.set_spots([0, 4, -3], [0, 2, 5], [41, 30, 29])
        return prob
    p = problem()
    one = ctx.heat(p.thermal, Q, p.traj)
    assert one["steps_done"] == 100
    for n_slabs in (2, 3):
        p = problem()
        got = halo.run_heat_slabs_local(ctx, p.thermal, Q, p.traj, n_slabs)
        np.testing.assert_array_equal(got["T"], one["T"], err_msg="T, %d slabs" % n_slabs)
        np.testing.assert_array_equal(got["dose"], one["dose"], err_msg="dose, %d slabs" % n_slabs)
    p = problem()
    s = ctx.heat_slab(p.thermal, Q, p.traj, 0, 15)
    buf = torch.empty(s.halo_bytes(), dtype=torch.uint8, device="cuda")
    with pytest.raises(api.BDError):
        s.halo_copy(0, 0, buf.data_ptr())     # side 0 of the first slab is the grid's face
    with pytest.raises(api.BDError):
        s.advance(101)                        # past the end of the run
    s.close()
    with pytest.raises(api.BDError):
        ctx.heat_slab(p.thermal, Q, p.traj, 10, 11)   # fewer than 2 planes
