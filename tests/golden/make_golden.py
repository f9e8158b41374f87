"""Generate the golden fixtures of tests/golden/ by running the reference's own
kernel code compiled for the host (oracle/_ref, built by oracle/build.py from
the reference sources).  Run from the repository root:

    python tests/golden/make_golden.py

Fixtures (numpy .npz):
  W_mini.npz     the W program on a 32x32x64 box: pressure after the first loop
                 (planes listed in `planes`) and the acoustic power Q
  T_mini.npz     the T kernel on a 41x41x48 box for a short spiral: T and dose
  T_spiral.npz   the reference's own spiral loop: per-step shifts and leg index
  G_threshold.npz  threshold amplitudes of G's search kernel for a set of
                 high-frequency combos and R0 values
  G_forward.npz  states of G's DPRK_step integration for a few bubbles
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from bubbledynamics_gb300 import presets  # noqa: E402
from oracle.oracle import RefLib, RefTCfg, RefGCfg  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
W_PLANES = [0, 1, 2, 3, 10, 31, 32, 33, 45, 60, 61, 62, 63]


def w_mini(r):
    k = presets.ref_W_mini_constants()
    P, Q, steps = r.w_run(k)
    np.savez_compressed(os.path.join(OUT, "W_mini.npz"), planes=np.array(W_PLANES), P=P[W_PLANES], Q=Q[W_PLANES],
                        P_sum=np.abs(P).sum(), Q_sum=Q.sum(), steps=steps)


def t_cfg(k):
    c = RefTCfg()
    c.Nxy, c.Nz = k["Nxy"], k["Nz"]
    c.dz, c.water_tissue, c.dt_T = k["dz"], k["water_tissue"], k["dt_T"]
    for name, v in presets.thermal_cfg_constants(k).items():
        setattr(c, name, v)
    return c


def t_mini_inputs():
    """Mini heat problem: constants, shifts of a short spiral, Gaussian source."""
    from oracle.oracle import Oracle
    k = presets.ref_T_mini_constants()
    prob = presets.make_ref_T(k)
    sx, sy, legs, n = Oracle().spiral_shifts(prob.traj)
    Q = presets.gaussian_focus_Q(prob.shape, (30, 20, 20), (3.0, 2.0, 2.0), 4.0e7)
    return k, prob, sx, sy, Q


def t_mini(r):
    k, prob, sx, sy, Q = t_mini_inputs()
    T0, TD0 = prob.initial_fields()
    T, TD = r.t_run(t_cfg(k), Q, T0, TD0, sx, sy)
    np.savez_compressed(os.path.join(OUT, "T_mini.npz"), T=T, TD=TD, n_steps=len(sx))


def t_spiral(r):
    import ctypes as C
    cap = 200000
    rec = np.zeros(3 * cap, np.int32)
    n = r.lib.bdref_t_trajectory
    n.restype = C.c_int64
    n.argtypes = [C.c_void_p, C.c_int64]
    k = n(rec.ctypes.data, cap)
    rec = rec[:3 * k].reshape(k, 3)
    np.savez_compressed(os.path.join(OUT, "T_spiral.npz"), sx=rec[:, 0], sy=rec[:, 1], leg=rec[:, 2])


def g_cfg():
    m = presets.ref_G_medium()
    c = RefGCfg()
    c.rho, c.P0, c.S2, c.mu4, c.G4_3 = m.rho, m.P0, m.S2, m.mu4, m.G4_3
    c.C_inf, c.lambda_, c.n, c.B, c.gamma = m.C_inf, m.lambda_, m.n, m.B, m.gamma
    c.gamma3 = 3.0 * m.gamma
    c.minA, c.stepA = 1e4, 1000.0
    c.minR0, c.stepR0 = 1e-7, 1e-7
    c.triple_fr = 1
    return c


def g_threshold_inputs():
    """Four high-frequency combos (short end times) and R0 = 2.0, 2.1 um, where
    the threshold lies near 3 MPa (about 30 + 10 + 10 integrations per item)."""
    from oracle.oracle import Oracle
    combos = Oracle().gilmore_combos()
    sel = [27700, 27690, 27680, 27670]
    minR0, stepR0, nR0 = 2.0e-6, 1e-7, 2
    R0 = np.array([minR0 + i * stepR0 for i in range(nR0)])   # G:332
    return combos[sel], np.array(sel), minR0, stepR0, R0


def g_threshold(r):
    fr, sel, minR0, stepR0, R0 = g_threshold_inputs()
    c = g_cfg()
    c.minR0, c.stepR0 = minR0, stepR0
    res = r.g_threshold(c, fr, len(R0))
    np.savez_compressed(os.path.join(OUT, "G_threshold.npz"), combos=fr, sel=sel, R0=R0, A=res)


def g_forward(r):
    # moderate drives (no inertial collapse) integrated over 0.1 us, and one strong
    # 5 MHz drive stopped at the threshold R' <= -C_inf (G:313, G:378)
    R0 = np.array([1e-6, 2e-6, 3e-6, 5e-6, 0.5e-6])
    A = np.array([0.1e6, 0.2e6, 0.15e6, 0.1e6, 4.0e6])
    f3 = np.array([[1e6, 1e6, 1e6], [1e6, 1e6, 1.2e6], [1e6, 1.1e6, 1.2e6], [2e6, 2e6, 2e6], [5e6, 5e6, 5e6]])
    endT = np.array([0.1e-6] * 4 + [0.4e-6])
    state, counts, thr = r.g_forward(g_cfg(), R0[:4], A[:4], f3[:4], float(endT[0]), max_steps=200000)
    s2, c2, t2 = r.g_forward(g_cfg(), R0[4:], A[4:], f3[4:], float(endT[4]), max_steps=200000, stop_at_threshold=True)
    state, counts, thr = np.vstack([state, s2]), np.concatenate([counts, c2]), np.concatenate([thr, t2])
    np.savez_compressed(os.path.join(OUT, "G_forward.npz"), R0=R0, A=A, f3=f3, endT=endT, state=state,
                        counts=counts, thr=thr)


if __name__ == "__main__":
    import time
    r = RefLib()
    todo = sys.argv[1:] or ["t_spiral", "t_mini", "g_forward", "g_threshold", "w_mini"]
    for name in todo:
        t = time.time()
        globals()[name](r)
        print("wrote", name, "%.1fs" % (time.time() - t), flush=True)
