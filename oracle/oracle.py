"""Python access to the CPU oracle.  TEST INFRASTRUCTURE ONLY.

`Oracle` wraps oracle/_build/libbdoracle.so (the FP64 restatement); `RefLib`
wraps oracle/_ref/libbdref.so (the reference's own kernel code compiled for
the host).  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg import this module.
"""
import ctypes as C
import os

import numpy as np

from bubbledynamics_gb300 import abi
from bubbledynamics_gb300.presets import WesterveltProblem

from . import build as _build

P = C.c_void_p


def _ptr(a):
    return None if a is None else a.ctypes.data


class Oracle:
    def __init__(self, path=None):
        path = path or _build.build_oracle()
        self.lib = C.CDLL(path)
        L = self.lib
        L.bdo_westervelt_run.argtypes = [P, P, P, P, P]
        L.bdo_westervelt_run.restype = C.c_int
        L.bdo_westervelt_adjoint.argtypes = [P, P, P, P, P, P, P, P]
        L.bdo_westervelt_adjoint.restype = C.c_int
        L.bdo_heat_run.argtypes = [P, P, P, P, C.c_int64, P, P, P, C.c_int32, P]
        L.bdo_heat_run.restype = C.c_int
        L.bdo_spiral_shifts.argtypes = [P, P, P, C.c_int64, P, P, C.c_int32]
        L.bdo_spiral_shifts.restype = C.c_int
        L.bdo_gilmore_run.argtypes = [P, C.c_int64, P, P, P]
        L.bdo_gilmore_run.restype = C.c_int
        L.bdo_gilmore_threshold.argtypes = [P, P, C.c_int64, P, C.c_int64, C.c_int64, P]
        L.bdo_gilmore_threshold.restype = C.c_int
        L.bdo_gilmore_threshold_bisect.argtypes = [P, P, C.c_int64, P, C.c_int64, C.c_int64, P]
        L.bdo_gilmore_threshold_bisect.restype = C.c_int
        L.bdo_gilmore_forward_combo.argtypes = [P, C.c_int64, P, P, P, C.c_double, C.c_double, C.c_int64,
                                                 C.c_int32, P, P, P]
        L.bdo_gilmore_forward_combo.restype = C.c_int
        L.bdo_gilmore_combos.argtypes = [C.c_int32, C.c_double, C.c_double, P, C.c_int64]
        L.bdo_gilmore_combos.restype = C.c_int64
        L.bdo_omp_threads.restype = C.c_int
        L.bdo_set_threads.argtypes = [C.c_int]

    def threads(self):
        return self.lib.bdo_omp_threads()

    def set_threads(self, n):
        self.lib.bdo_set_threads(int(n))

    # ---------------------------------------------------------------- W
    def westervelt(self, prob: WesterveltProblem, want=("p_final", "peak", "energy", "Q", "dft")):
        dt = prob.dtype
        n = prob.ncell
        out = abi.WesterveltOutputs()
        res = {}
        if "p_final" in want:
            res["p_final"] = np.zeros(n, dt)
            out.p_final = _ptr(res["p_final"])
        if "peak" in want:
            res["peak"] = np.zeros(n, dt)
            out.peak = _ptr(res["peak"])
        if "energy" in want:
            res["energy"] = np.zeros(n, dt)
            out.energy = _ptr(res["energy"])
        p = prob.params
        if "dft" in want and p.n_dft > 0:
            nz = max(0, min(prob.grid.nz, p.dft_z_hi) - max(0, p.dft_z_lo))
            m = p.n_dft * prob.grid.nx * prob.grid.ny * nz
            res["dft_re"] = np.zeros(m, dt)
            res["dft_im"] = np.zeros(m, dt)
            out.dft_re = _ptr(res["dft_re"])
            out.dft_im = _ptr(res["dft_im"])
        if "Q" in want and p.q_mode == abi.BD_Q_REFERENCE:
            res["Q"] = np.zeros(n, np.float64)
            out.Q = _ptr(res["Q"])
        st = self.lib.bdo_westervelt_run(C.byref(prob.grid), C.byref(prob.medium), C.byref(prob.source),
                                         C.byref(prob.params), C.byref(out))
        if st != 0:
            raise RuntimeError("oracle westervelt failed: %s" % abi.STATUS_NAMES.get(st, st))
        shp = prob.shape
        for k in ("p_final", "peak", "energy", "Q"):
            if k in res:
                res[k] = res[k].reshape(shp)
        return res

    def westervelt_adjoint(self, prob: WesterveltProblem, loss):
        """FP64 loss and its gradient w.r.t. element phases and amplitudes."""
        ne = prob.source.n_elements
        gp = np.zeros(ne, np.float64)
        ga = np.zeros(ne, np.float64)
        L = C.c_double(0.0)
        st = self.lib.bdo_westervelt_adjoint(C.byref(prob.grid), C.byref(prob.medium), C.byref(prob.source),
                                             C.byref(prob.params), C.byref(loss), C.addressof(L), _ptr(gp), _ptr(ga))
        if st != 0:
            raise RuntimeError("oracle adjoint failed: %s" % abi.STATUS_NAMES.get(st, st))
        return L.value, gp, ga

    # ---------------------------------------------------------------- T
    def heat(self, thermal, Q, sx, sy, T0, TD0, snap_steps=None):
        T = np.ascontiguousarray(T0, dtype=np.float64).copy()
        TD = np.ascontiguousarray(TD0, dtype=np.float64).copy()
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        sx = np.ascontiguousarray(sx, dtype=np.int32)
        sy = np.ascontiguousarray(sy, dtype=np.int32)
        n = T.size
        snap = None
        ss = None
        ns = 0
        if snap_steps is not None and len(snap_steps):
            ss = np.ascontiguousarray(snap_steps, dtype=np.int64)
            ns = len(ss)
            snap = np.zeros((ns, n), np.float64)
        st = self.lib.bdo_heat_run(C.byref(thermal), _ptr(Q), _ptr(sx), _ptr(sy), len(sx), _ptr(T), _ptr(TD),
                                   _ptr(ss), ns, _ptr(snap))
        if st != 0:
            raise RuntimeError("oracle heat failed")
        return T, TD, snap

    def spiral_shifts(self, traj, cap=1 << 22, leg_cap=64):
        sx = np.zeros(cap, np.int32)
        sy = np.zeros(cap, np.int32)
        legs = np.zeros(leg_cap, np.int64)
        n = C.c_int64(0)
        self.lib.bdo_spiral_shifts(C.byref(traj), _ptr(sx), _ptr(sy), cap, C.byref(n), _ptr(legs), leg_cap)
        k = n.value
        return sx[:min(k, cap)], sy[:min(k, cap)], legs[:traj.n_legs], k

    # ---------------------------------------------------------------- G
    def gilmore(self, medium, bubbles, ode):
        n = len(bubbles)
        res = (abi.BubbleResult * n)()
        st = self.lib.bdo_gilmore_run(C.byref(medium), n, C.cast(bubbles, P), C.byref(ode), C.cast(res, P))
        if st != 0:
            raise RuntimeError("oracle gilmore failed")
        return res

    def gilmore_forward_combo(self, medium, R0, A, f3, endT, h0=1e-13, max_steps=10 ** 7, stop_at_threshold=False):
        R0 = np.ascontiguousarray(R0, dtype=np.float64)
        A = np.ascontiguousarray(A, dtype=np.float64)
        f3 = np.ascontiguousarray(f3, dtype=np.float64).reshape(-1)
        n = R0.size
        state = np.zeros((n, 5))
        counts = np.zeros(n, np.int64)
        thr = np.zeros(n)
        self.lib.bdo_gilmore_forward_combo(C.byref(medium), n, _ptr(R0), _ptr(A), _ptr(f3), endT, h0, max_steps,
                                           1 if stop_at_threshold else 0, _ptr(state), _ptr(counts), _ptr(thr))
        return state, counts, thr

    def gilmore_threshold(self, medium, fr_combo, R0, max_steps=0, bisect=False):
        fr = np.ascontiguousarray(fr_combo, dtype=np.float64).reshape(-1)
        R0 = np.ascontiguousarray(R0, dtype=np.float64)
        nc = fr.size // 3
        out = np.zeros(nc * R0.size, np.float64)
        fn = self.lib.bdo_gilmore_threshold_bisect if bisect else self.lib.bdo_gilmore_threshold
        fn(C.byref(medium), _ptr(fr), nc, _ptr(R0), R0.size, max_steps, _ptr(out))
        return out.reshape(nc, R0.size)

    def gilmore_combos(self, n_fr=55, f_min=0.02e6, f_max=5.0e6):
        k = self.lib.bdo_gilmore_combos(n_fr, f_min, f_max, None, 0)
        out = np.zeros(3 * k, np.float64)
        self.lib.bdo_gilmore_combos(n_fr, f_min, f_max, _ptr(out), k)
        return out.reshape(k, 3)


# ---------------------------------------------------------------------------
# the reference's own kernels, host build
# ---------------------------------------------------------------------------
class RefWCfg(C.Structure):
    _fields_ = [("Nxy", C.c_int32), ("Nz", C.c_int32)] + [
        (k, C.c_double) for k in (
            "rho", "c_inf", "delta", "beta", "abs_water",
            "rho_tissue", "c_inf_tissue", "beta_tissue", "abs_tissue",
            "delta_tissue", "c1", "c2", "tau1", "tau2",
            "fr", "d", "alpha", "alpha_hole", "p0", "water_tissue",
            "xy_min", "dxy", "z_min", "dz", "dt", "t_max")
    ] + [("periods", C.c_int32), ("iz_tissue", C.c_int32), ("nx_slab", C.c_int32), ("N_harm", C.c_int32),
         ("do_power", C.c_int32), ("pad0", C.c_int32)]


class RefTCfg(C.Structure):
    _fields_ = [("Nxy", C.c_int32), ("Nz", C.c_int32)] + [
        (k, C.c_double) for k in ("dz", "water_tissue", "dt_T", "kdt_dxy", "kdt_dz", "kdt_dxy_water",
                                  "kdt_dz_water", "dt_rho_ct", "dt_rho_ct_water")]


class RefGCfg(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("rho", "P0", "S2", "mu4", "G4_3", "C_inf", "lambda_", "n", "B",
                                          "gamma", "gamma3", "minA", "stepA", "minR0", "stepR0")] + [
        ("triple_fr", C.c_int32), ("pad0", C.c_int32)]


def ref_w_cfg(k, do_power=True):
    c = RefWCfg()
    c.Nxy, c.Nz = k["Nxy"], k["Nz"]
    c.rho, c.c_inf, c.delta, c.beta, c.abs_water = (k["rho_water"], k["c_water"], k["delta_water"],
                                                    k["beta_water"], k["abs_water"])
    c.rho_tissue, c.c_inf_tissue, c.beta_tissue, c.abs_tissue = (k["rho_tissue"], k["c_tissue"],
                                                                 k["beta_tissue"], k["abs_tissue"])
    c.delta_tissue, c.c1, c.c2, c.tau1, c.tau2 = k["delta_tissue"], k["c1"], k["c2"], k["tau1"], k["tau2"]
    c.fr, c.d, c.alpha, c.alpha_hole, c.p0, c.water_tissue = (k["fr"], k["d"], k["alpha"], k["alpha_hole"],
                                                              k["p0"], k["water_tissue"])
    c.xy_min, c.dxy, c.z_min, c.dz, c.dt = k["xy_min"], k["dxy"], k["z_min"], k["dz"], k["dt"]
    c.t_max = k["t_max"]
    c.periods, c.iz_tissue, c.nx_slab, c.N_harm = k["periods"], k["iz_tissue"], k["nx_slab"], k["N_harm"]
    c.do_power = 1 if do_power else 0
    return c


class RefLib:
    """The reference's kernel code compiled for the host (oracle/_ref)."""

    def __init__(self, path=None):
        path = path or _build.build_ref()
        if path is None or not os.path.exists(path):
            raise FileNotFoundError("oracle/_ref/libbdref.so is not available")
        self.lib = C.CDLL(path)
        L = self.lib
        L.bdref_w_run.argtypes = [P, P, P, P]
        L.bdref_w_steps.argtypes = [P, C.c_int64, P]
        L.bdref_t_run.argtypes = [P, P, P, P, P, P, P, C.c_int64, P]
        L.bdref_g_threshold.argtypes = [P, P, C.c_int32, C.c_int32, P]
        L.bdref_g_forward.argtypes = [P, C.c_int64, P, P, P, C.c_double, C.c_double, C.c_int64, C.c_int32,
                                      P, P, P]

    def w_run(self, k, do_power=True):
        c = ref_w_cfg(k, do_power)
        n = k["Nxy"] * k["Nxy"] * k["Nz"]
        Psnap = np.zeros(n, np.float64)
        Q = np.zeros(n, np.float64)
        steps = np.zeros(3, np.int64)
        self.lib.bdref_w_run(C.byref(c), _ptr(Psnap), _ptr(Q), _ptr(steps))
        shp = (k["Nz"], k["Nxy"], k["Nxy"])
        return Psnap.reshape(shp), Q.reshape(shp), steps

    def w_steps(self, k, n_steps, init=None):
        c = ref_w_cfg(k, False)
        n = k["Nxy"] * k["Nxy"] * k["Nz"]
        state = (np.zeros((12, n), np.float64) if init is None
                 else np.ascontiguousarray(init, dtype=np.float64).reshape(12, n).copy())
        self.lib.bdref_w_steps(C.byref(c), n_steps, _ptr(state))
        return state.reshape(12, k["Nz"], k["Nxy"], k["Nxy"])

    def t_run(self, cfg, Q, T0, TD0, sx, sy):
        Tp = np.ascontiguousarray(T0, dtype=np.float64).copy()
        Tn = Tp.copy()
        TD = np.ascontiguousarray(TD0, dtype=np.float64).copy()
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        sx = np.ascontiguousarray(sx, dtype=np.int32)
        sy = np.ascontiguousarray(sy, dtype=np.int32)
        up = C.c_int32(0)
        self.lib.bdref_t_run(C.byref(cfg), _ptr(Q), _ptr(Tp), _ptr(Tn), _ptr(TD), _ptr(sx), _ptr(sy), len(sx),
                             C.byref(up))
        latest = Tp if up.value else Tn   # T:568-571
        return latest, TD

    def g_threshold(self, cfg, fr_combo, n_R0):
        fr = np.ascontiguousarray(fr_combo, dtype=np.float64).reshape(-1)
        nc = fr.size // 3
        out = np.zeros(nc * n_R0, np.float64)
        self.lib.bdref_g_threshold(C.byref(cfg), _ptr(fr), nc, n_R0, _ptr(out))
        return out.reshape(nc, n_R0)

    def g_forward(self, cfg, R0, A, f3, endT, h0=1e-13, max_steps=10 ** 7, stop_at_threshold=False):
        R0 = np.ascontiguousarray(R0, dtype=np.float64)
        A = np.ascontiguousarray(A, dtype=np.float64)
        f3 = np.ascontiguousarray(f3, dtype=np.float64).reshape(-1)
        n = R0.size
        state = np.zeros((n, 5), np.float64)
        counts = np.zeros(n, np.int64)
        thr = np.zeros(n, np.float64)
        self.lib.bdref_g_forward(C.byref(cfg), n, _ptr(R0), _ptr(A), _ptr(f3), endT, h0, max_steps,
                                 1 if stop_at_threshold else 0, _ptr(state), _ptr(counts), _ptr(thr))
        return state, counts, thr


def ref_g_cfg(medium, triple_fr=True):
    """G's __device__ constants (G:13-33) from a bd_gilmore_medium."""
    c = RefGCfg()
    m = medium
    c.rho, c.P0, c.S2, c.mu4, c.G4_3 = m.rho, m.P0, m.S2, m.mu4, m.G4_3
    c.C_inf, c.lambda_, c.n, c.B, c.gamma = m.C_inf, m.lambda_, m.n, m.B, m.gamma
    c.gamma3 = 3.0 * m.gamma
    c.minA, c.stepA = 1e4, 1000.0
    c.minR0, c.stepR0 = 1e-7, 1e-7
    c.triple_fr = 1 if triple_fr else 0
    return c


class RefGpuLib:
    """The reference's own CUDA kernels on the GPU (oracle/_ref/libbdref_gpu.so)."""

    def __init__(self, path=None):
        path = path or _build.build_ref_gpu()
        if path is None or not os.path.exists(path):
            raise FileNotFoundError("oracle/_ref/libbdref_gpu.so is not available")
        self.lib = C.CDLL(path)
        L = self.lib
        L.bdref_gpu_w_steps.argtypes = [P, C.c_int64, C.c_int64, P, P, C.c_int32]
        L.bdref_gpu_w_steps.restype = C.c_int
        L.bdref_gpu_g_forward.argtypes = [P, C.c_int64, P, P, P, C.c_double, C.c_double, C.c_int64, P, P, P]
        L.bdref_gpu_g_forward.restype = C.c_int

    def w_steps(self, k, n_steps, warm=0, want_state=False, init=None):
        """Runs W's loop from zero (or from `init`, 12 fields); returns (ms of
        the timed steps, final state or None)."""
        c = ref_w_cfg(k, False)
        n = k["Nxy"] * k["Nxy"] * k["Nz"]
        if init is not None:
            state = np.ascontiguousarray(init, dtype=np.float64).reshape(12, n).copy()
        else:
            state = np.zeros((12, n), np.float64) if want_state else None
        ms = C.c_double(0.0)
        st = self.lib.bdref_gpu_w_steps(C.byref(c), warm, n_steps, C.addressof(ms), _ptr(state),
                                        1 if init is not None else 0)
        if st != 0:
            raise RuntimeError("reference GPU Westervelt loop failed (%d)" % st)
        if state is not None:
            state = state.reshape(12, k["Nz"], k["Nxy"], k["Nxy"])
        return ms.value, state

    def g_forward(self, cfg, R0, A, f3, endT, h0=1e-13, max_steps=10 ** 7):
        R0 = np.ascontiguousarray(R0, dtype=np.float64)
        A = np.ascontiguousarray(A, dtype=np.float64)
        f3 = np.ascontiguousarray(f3, dtype=np.float64).reshape(-1)
        n = R0.size
        state = np.zeros((n, 5), np.float64)
        counts = np.zeros(n, np.int64)
        ms = C.c_double(0.0)
        st = self.lib.bdref_gpu_g_forward(C.byref(cfg), n, _ptr(R0), _ptr(A), _ptr(f3), endT, h0, max_steps,
                                          _ptr(state), _ptr(counts), C.addressof(ms))
        if st != 0:
            raise RuntimeError("reference GPU Gilmore loop failed (%d)" % st)
        return state, counts, ms.value
