"""The CPU oracle against the reference itself: golden fixtures produced by
the reference's own kernel code (tests/golden/make_golden.py), and the live
host build of that code when it is available."""
import numpy as np
import pytest

from bubbledynamics_gb300 import abi, presets
from tests.conftest import golden_path


def test_westervelt_mini_matches_reference_fixture(oracle):
    g = np.load(golden_path("W_mini.npz"))
    prob = presets.ref_W_mini()
    assert prob.meta["n_loop1"] == int(g["steps"][0])
    assert prob.meta["n_water"] == int(g["steps"][1])
    p1 = prob.copy()
    p1.params.n_steps = prob.meta["n_loop1"]
    P = oracle.westervelt(p1, want=("p_final",))["p_final"]
    # pressure after the first loop: bit-identical (same operation order, Mur in serial order)
    np.testing.assert_array_equal(P[g["planes"]], g["P"])
    assert np.abs(P).sum() == pytest.approx(float(g["P_sum"]), rel=1e-12)
    Q = oracle.westervelt(prob, want=("Q",))["Q"]
    split = prob.params.q_iz_split
    planes = g["planes"]
    water = planes < split
    # water power is the same arithmetic; tissue power differs by the reference's FP32 FFT
    np.testing.assert_array_equal(Q[planes[water]], g["Q"][water])
    qt, gt = Q[planes[~water]], g["Q"][~water]
    rel = np.abs(qt - gt) / np.maximum(np.abs(gt), 1e-6 * np.abs(gt).max())
    assert rel.max() < 2e-6


@pytest.mark.slow
def test_westervelt_mini_matches_live_reference(oracle, ref):
    k = presets.ref_W_mini_constants(Nxy=16, Nz=48, loop1_periods=1, periods=1)
    k["nx_slab"] = 8
    P_ref, Q_ref, steps = ref.w_run(k)
    prob = presets.make_ref_W(k)
    p1 = prob.copy()
    p1.params.n_steps = int(steps[0])
    P = oracle.westervelt(p1, want=("p_final",))["p_final"]
    np.testing.assert_array_equal(P, P_ref)


def test_heat_mini_matches_reference_fixture(oracle):
    from tests.golden.make_golden import t_mini_inputs
    g = np.load(golden_path("T_mini.npz"))
    k, prob, sx, sy, Q = t_mini_inputs()
    assert len(sx) == int(g["n_steps"])
    T0, TD0 = prob.initial_fields()
    T, TD, _ = oracle.heat(prob.thermal, Q, sx, sy, T0, TD0)
    np.testing.assert_array_equal(T.reshape(prob.shape), g["T"])
    np.testing.assert_array_equal(TD.reshape(prob.shape), g["TD"])


def test_spiral_matches_reference_loop(oracle, lib):
    g = np.load(golden_path("T_spiral.npz"))
    prob = presets.ref_T()
    sx, sy, legs, n = oracle.spiral_shifts(prob.traj)
    assert n == len(g["sx"]) == 77474
    np.testing.assert_array_equal(sx, g["sx"])
    np.testing.assert_array_equal(sy, g["sy"])
    # leg ends: the reference increments `lines` after each leg
    ends = np.flatnonzero(np.diff(g["leg"])) + 1
    np.testing.assert_array_equal(legs[:-1], ends)
    # the product's host implementation of the same loop (C ABI, no GPU needed)
    from bubbledynamics_gb300 import api
    psx, psy, plegs = api.trajectory_shifts(prob.traj)
    np.testing.assert_array_equal(psx, g["sx"])
    np.testing.assert_array_equal(psy, g["sy"])
    np.testing.assert_array_equal(plegs, legs)


def test_gilmore_threshold_matches_reference_fixture(oracle):
    g = np.load(golden_path("G_threshold.npz"))
    A = oracle.gilmore_threshold(presets.ref_G_medium(), g["combos"], g["R0"])
    np.testing.assert_array_equal(A, g["A"])


def test_gilmore_threshold_bisection_matches_reference_fixture(oracle):
    """The opt-in bisection search (stages 2-3 of G:391-426 replaced by
    bisection on the 1 kPa grid inside the last 0.1 MPa bracket) lands on the
    amplitudes of the reference's linear scan for a combination whose
    threshold response is monotone."""
    g = np.load(golden_path("G_threshold.npz"))
    A = oracle.gilmore_threshold(presets.ref_G_medium(), g["combos"][3:], g["R0"], bisect=True)
    np.testing.assert_array_equal(A, g["A"][3:])


def test_gilmore_forward_matches_reference_fixture(oracle):
    """G's DPRK_step loop (G:212-318, G:378) for moderate drives to endT and one
    strong drive stopped at R' <= -C_inf: bit-identical."""
    g = np.load(golden_path("G_forward.npz"))
    med = presets.ref_G_medium()
    endT = g["endT"]
    s1, c1, t1 = oracle.gilmore_forward_combo(med, g["R0"][:4], g["A"][:4], g["f3"][:4], float(endT[0]),
                                              max_steps=200000)
    s2, c2, t2 = oracle.gilmore_forward_combo(med, g["R0"][4:], g["A"][4:], g["f3"][4:], float(endT[4]),
                                              max_steps=200000, stop_at_threshold=True)
    np.testing.assert_array_equal(np.vstack([s1, s2]), g["state"])
    np.testing.assert_array_equal(np.concatenate([c1, c2]), g["counts"])
    np.testing.assert_array_equal(np.concatenate([t1, t2]), g["thr"])
