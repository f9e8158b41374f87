"""Python host layer over libbubbledyn (include/bubbledyn.h).

Each method maps one-to-one onto a C entry point.  There is no CPU fallback:
if the compiled library is missing, `load()` raises.
"""
import ctypes as C
import os

import numpy as np

from . import abi
from .presets import WesterveltProblem

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libbubbledyn.so")

P = C.c_void_p
_lib = None

# numpy mirrors of the bulk structs (same layout as the C structs)
BUBBLE_DTYPE = np.dtype([("R0", "f8"), ("n_tones", "i4"), ("pad0", "i4"),
                         ("f", "f8", (abi.BD_MAX_BUBBLE_TONES,)), ("a", "f8", (abi.BD_MAX_BUBBLE_TONES,)),
                         ("phi", "f8", (abi.BD_MAX_BUBBLE_TONES,))])
RESULT_DTYPE = np.dtype([("R", "f8"), ("Rdot", "f8"), ("tau", "f8"), ("q", "f8"), ("t", "f8"),
                         ("R_max", "f8"), ("R_min", "f8"), ("t_threshold", "f8"),
                         ("n_accept", "i8"), ("n_reject", "i8"), ("status", "i4"), ("threshold", "i4")])
assert BUBBLE_DTYPE.itemsize == C.sizeof(abi.Bubble)
assert RESULT_DTYPE.itemsize == C.sizeof(abi.BubbleResult)


class BDError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (abi.STATUS_NAMES.get(status, status), msg))
        self.status = status


def _sig(L, name, args, res=C.c_int):
    f = getattr(L, name)
    f.argtypes = args
    f.restype = res


def load(path=None):
    """Load the compiled library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError("libbubbledyn.so not found at %s: run __graft_entry__.build() "
                           "(there is no CPU fallback)" % path)
    L = C.CDLL(path)
    _sig(L, "bd_context_create", [C.c_int, C.POINTER(P)])
    _sig(L, "bd_context_destroy", [P])
    _sig(L, "bd_last_error_string", [], C.c_char_p)
    _sig(L, "bd_abi_version", [])
    _sig(L, "bd_context_kernel_launches", [P, C.POINTER(C.c_int64)])
    _sig(L, "bd_selftest_bounded_wait", [P, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_double)])
    _sig(L, "bd_westervelt_run", [P, P, P, P, P, P])
    _sig(L, "bd_westervelt_begin", [P, P, P, P, P, C.POINTER(P)])
    _sig(L, "bd_westervelt_advance", [P, C.c_int64])
    _sig(L, "bd_westervelt_step_index", [P, C.POINTER(C.c_int64)])
    _sig(L, "bd_westervelt_finish", [P, P])
    _sig(L, "bd_westervelt_end", [P])
    _sig(L, "bd_westervelt_last_ms", [P, C.POINTER(C.c_double)])
    _sig(L, "bd_westervelt_slab_begin", [P, P, P, P, P, C.c_int32, C.c_int32, C.POINTER(P)])
    _sig(L, "bd_westervelt_halo_bytes", [P, C.POINTER(C.c_size_t)])
    _sig(L, "bd_westervelt_halo_copy", [P, C.c_int32, C.c_int32, P, P])
    _sig(L, "bd_halo_exchange", [P, P])
    _sig(L, "bd_westervelt_run_slabs", [P, P, P, P, P, C.c_int32, P])
    _sig(L, "bd_checkpoint_size", [P, C.POINTER(C.c_size_t)])
    _sig(L, "bd_checkpoint_save", [P, P, C.c_size_t])
    _sig(L, "bd_checkpoint_load", [P, P, C.c_size_t])
    _sig(L, "bd_trajectory_shifts", [P, P, P, C.c_int64, C.POINTER(C.c_int64), P, C.c_int32])
    _sig(L, "bd_unfold_quarter", [P, C.c_int32, C.c_int32, P])
    _sig(L, "bd_spiral_heat_run", [P, P, P, P, C.c_int64, P])
    _sig(L, "bd_spiral_heat_run_slabs", [P, P, P, P, C.c_int64, C.c_int32, P])
    _sig(L, "bd_heat_slab_begin", [P, P, P, P, C.c_int64, C.c_int32, C.c_int32, C.POINTER(P)])
    _sig(L, "bd_heat_slab_steps", [P, C.POINTER(C.c_int64), C.POINTER(C.c_int64)])
    _sig(L, "bd_heat_slab_advance", [P, C.c_int64])
    _sig(L, "bd_heat_slab_halo_bytes", [P, C.POINTER(C.c_size_t)])
    _sig(L, "bd_heat_slab_halo_copy", [P, C.c_int32, C.c_int32, P, P])
    _sig(L, "bd_heat_slab_finish", [P, P])
    _sig(L, "bd_heat_slab_end", [P])
    _sig(L, "bd_gilmore_combo_tones", [C.c_double, P, P, P])
    _sig(L, "bd_gilmore_combos", [C.c_int32, C.c_double, C.c_double, P, C.c_int64, C.POINTER(C.c_int64)])
    _sig(L, "bd_gilmore_run", [P, P, C.c_int64, P, P, P, C.POINTER(C.c_double)])
    _sig(L, "bd_gilmore_run_device", [P, P, C.c_int64, P, P, P, P])
    _sig(L, "bd_gilmore_threshold", [P, P, P, C.c_int64, P, C.c_int64, C.c_int32, C.c_int64, P,
                                     C.POINTER(C.c_double)])
    _sig(L, "bd_gilmore_threshold_search", [P, P, P, C.c_int64, P, C.c_int64, C.c_int32, C.c_int64, C.c_int32, P,
                                            C.POINTER(C.c_double)])
    _sig(L, "bd_heat_run_device_noalloc", [P, P, P, P, P, P, C.c_int64, P])
    _sig(L, "bd_westervelt_adjoint", [P, P, P, P, P, P, C.POINTER(C.c_double), P, P, P])
    _sig(L, "bd_westervelt_adjoint_slabs", [P, P, P, P, P, P, C.c_int32, C.POINTER(C.c_double), P, P, P])
    _sig(L, "bd_write_q_bin", [C.c_char_p, P, C.c_int32, C.c_int32, C.c_int32, C.c_int32])
    _sig(L, "bd_read_q_bin", [C.c_char_p, P, C.c_int64, C.POINTER(C.c_int64)])
    _sig(L, "bd_write_q_axis_dat", [C.c_char_p, P, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_double,
                                    C.c_int32])
    _sig(L, "bd_write_slice_dat", [C.c_char_p, P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                   C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_char_p])
    _sig(L, "bd_write_threshold_table", [C.c_char_p, P, C.c_int64, P, C.c_int64, P, C.c_double])
    _lib = L
    return L


def check(st):
    if st != abi.BD_OK:
        raise BDError(st, load().bd_last_error_string().decode(errors="replace"))


def _ptr(a):
    return None if a is None else a.ctypes.data


def trajectory_shifts(traj, leg_cap=4096):
    """Per-step (sx, sy) shifts and the step count after each leg/spot."""
    L = load()
    n = C.c_int64(0)
    check(L.bd_trajectory_shifts(C.byref(traj), None, None, 0, C.byref(n), None, 0))
    sx = np.zeros(max(n.value, 1), np.int32)
    sy = np.zeros(max(n.value, 1), np.int32)
    legs = np.zeros(leg_cap, np.int64)
    check(L.bd_trajectory_shifts(C.byref(traj), _ptr(sx), _ptr(sy), n.value, C.byref(n), _ptr(legs), leg_cap))
    nl = traj.n_spots if traj.kind == abi.BD_TRAJ_SPOTS else traj.n_legs
    return sx[:n.value], sy[:n.value], legs[:nl]


def unfold_quarter(small, n_half, nz):
    L = load()
    small = np.ascontiguousarray(small, dtype=np.float64)
    nf = 2 * n_half + 1
    full = np.zeros(nz * nf * nf, np.float64)
    check(L.bd_unfold_quarter(_ptr(small), n_half, nz, _ptr(full)))
    return full.reshape(nz, nf, nf)


def gilmore_combos(n_fr=55, f_min=0.02e6, f_max=5.0e6):
    L = load()
    n = C.c_int64(0)
    check(L.bd_gilmore_combos(n_fr, f_min, f_max, None, 0, C.byref(n)))
    out = np.zeros(3 * n.value, np.float64)
    check(L.bd_gilmore_combos(n_fr, f_min, f_max, _ptr(out), n.value, C.byref(n)))
    return out.reshape(n.value, 3)


# --------------------------------------------------------------------------
# the reference programs' files
# --------------------------------------------------------------------------
def write_q_bin(path, Q, iz_first=2):
    """W's Q3D_*.bin layout (W:778-790) of a (nz, ny, nx) field."""
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    nz, ny, nx = Q.shape
    check(load().bd_write_q_bin(str(path).encode(), _ptr(Q), nx, ny, nz, iz_first))


def read_q_bin(path, n_half, nz):
    """The quarter-domain volume T reads (T:276-279): (nz, n_half+1, n_half+1)."""
    m = (n_half + 1) ** 2 * nz
    out = np.zeros(m, np.float64)
    got = C.c_int64(0)
    check(load().bd_read_q_bin(str(path).encode(), _ptr(out), m, C.byref(got)))
    return out.reshape(nz, n_half + 1, n_half + 1)


def write_q_axis_dat(path, Q, z_min, dz, iz_first=2):
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    nz, ny, nx = Q.shape
    check(load().bd_write_q_axis_dat(str(path).encode(), _ptr(Q), nx, ny, nz, z_min, dz, iz_first))


def write_slice_dat(path, field, orientation, fixed, rows, cols, header=None):
    """T's slice files (T:419-448, T:576-640); rows / cols are (start, stop)."""
    f = np.ascontiguousarray(field, dtype=np.float64)
    nz, ny, nx = f.shape
    check(load().bd_write_slice_dat(str(path).encode(), _ptr(f), nx, ny, nz, orientation, fixed, rows[0], rows[1],
                                    cols[0], cols[1], header.encode() if header else None))


def write_threshold_table(path, fr_combo, R0, results, elapsed_s):
    """G's dR_Cinf_*.dat table (G:582-613)."""
    fr = np.ascontiguousarray(fr_combo, dtype=np.float64).reshape(-1)
    R0 = np.ascontiguousarray(R0, dtype=np.float64)
    res = np.ascontiguousarray(results, dtype=np.float64).reshape(-1)
    check(load().bd_write_threshold_table(str(path).encode(), _ptr(fr), fr.size // 3, _ptr(R0), R0.size, _ptr(res),
                                          float(elapsed_s)))


class Context:
    """A device context (stream, events, device memory pool)."""

    def __init__(self, device=0):
        self.L = load()
        h = P()
        check(self.L.bd_context_create(device, C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.L.bd_context_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def kernel_launches(self):
        n = C.c_int64(0)
        check(self.L.bd_context_kernel_launches(self.h, C.byref(n)))
        return n.value

    def selftest_bounded_wait(self, limit_ms=100):
        """(timed_out, device ms) of a kernel whose pipeline wait nothing completes."""
        t = C.c_int32(0)
        ms = C.c_double(0)
        check(self.L.bd_selftest_bounded_wait(self.h, int(limit_ms), C.byref(t), C.byref(ms)))
        return bool(t.value), ms.value

    # ------------------------------------------------------------ Westervelt
    @staticmethod
    def _outputs(prob, want):
        dt = prob.dtype
        n = prob.ncell
        out = abi.WesterveltOutputs()
        res = {}
        for k in ("p_final", "peak", "energy"):
            if k in want:
                res[k] = np.zeros(n, dt)
                setattr(out, k, _ptr(res[k]))
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
        return out, res

    @staticmethod
    def _shape(prob, res, out):
        for k in ("p_final", "peak", "energy", "Q"):
            if k in res:
                res[k] = res[k].reshape(prob.shape)
        res["elapsed_ms"] = out.elapsed_ms
        res["steps_done"] = out.steps_done
        res["tile_variant"] = out.tile_variant
        return res

    def westervelt(self, prob: WesterveltProblem, want=("p_final", "peak", "energy", "Q", "dft")):
        """Full solve (bd_westervelt_run); returns the requested host arrays."""
        out, res = self._outputs(prob, want)
        check(self.L.bd_westervelt_run(self.h, C.byref(prob.grid), C.byref(prob.medium), C.byref(prob.source),
                                       C.byref(prob.params), C.byref(out)))
        return self._shape(prob, res, out)

    def westervelt_session(self, prob: WesterveltProblem):
        return WesterveltSession(self, prob)

    def westervelt_slabs(self, prob: WesterveltProblem, n_slabs, want=("p_final", "peak", "energy", "Q", "dft")):
        """The solve as n_slabs z slabs on this device with the ghost planes
        exchanged after every step (bd_westervelt_run_slabs): the same outputs
        as westervelt(), bit for bit."""
        out, res = self._outputs(prob, want)
        check(self.L.bd_westervelt_run_slabs(self.h, C.byref(prob.grid), C.byref(prob.medium), C.byref(prob.source),
                                             C.byref(prob.params), int(n_slabs), C.byref(out)))
        return self._shape(prob, res, out)

    def westervelt_slab(self, prob: WesterveltProblem, z_begin, z_end):
        """Session over the planes [z_begin, z_end) of prob (bd_westervelt_slab_begin)."""
        return WesterveltSession(self, prob, slab=(int(z_begin), int(z_end)))

    def westervelt_adjoint(self, prob: WesterveltProblem, loss, n_slabs=1):
        """Loss of `loss` (abi.FocalLoss) and its gradient w.r.t. the element
        phases and amplitudes of prob's BD_SRC_ARRAY source
        (bd_westervelt_adjoint; n_slabs > 1: bd_westervelt_adjoint_slabs, the
        same bits from that many z slabs).  Returns (loss, grad_phase,
        grad_amp, timings) with timings = {"forward_ms", "recompute_ms",
        "backward_ms"}."""
        ne = prob.source.n_elements
        gp = np.zeros(ne, np.float64)
        ga = np.zeros(ne, np.float64)
        tm = np.zeros(3, np.float64)
        L = C.c_double(0.0)
        if n_slabs == 1:
            check(self.L.bd_westervelt_adjoint(self.h, C.byref(prob.grid), C.byref(prob.medium),
                                               C.byref(prob.source), C.byref(prob.params), C.byref(loss), C.byref(L),
                                               _ptr(gp), _ptr(ga), _ptr(tm)))
        else:
            check(self.L.bd_westervelt_adjoint_slabs(self.h, C.byref(prob.grid), C.byref(prob.medium),
                                                     C.byref(prob.source), C.byref(prob.params), C.byref(loss),
                                                     int(n_slabs), C.byref(L), _ptr(gp), _ptr(ga), _ptr(tm)))
        return L.value, gp, ga, {"forward_ms": tm[0], "recompute_ms": tm[1], "backward_ms": tm[2]}

    # ------------------------------------------------------------ heat
    def heat(self, thermal, Q, traj, max_steps=0, snapshot_legs=(), want_T=True, want_dose=True, n_slabs=1):
        """Heat + dose run over the trajectory (bd_spiral_heat_run); n_slabs > 1
        runs it as that many z slabs with ghost-plane exchange
        (bd_spiral_heat_run_slabs), which gives the same bits."""
        n = thermal.nx * thermal.ny * thermal.nz
        Q = np.ascontiguousarray(Q, dtype=np.float64).reshape(-1)
        assert Q.size == n
        out = abi.HeatOutputs()
        res = {}
        if want_T:
            res["T"] = np.zeros(n, np.float64)
            out.T_final = _ptr(res["T"])
        if want_dose:
            res["dose"] = np.zeros(n, np.float64)
            out.dose = _ptr(res["dose"])
        legs = np.ascontiguousarray(snapshot_legs, dtype=np.int32)
        if legs.size:
            res["snapshots"] = np.zeros((legs.size, n), np.float64)
            out.snapshots = _ptr(res["snapshots"])
            out.snapshot_legs = _ptr(legs)
            out.n_snap = legs.size
        if n_slabs == 1:
            check(self.L.bd_spiral_heat_run(self.h, C.byref(thermal), _ptr(Q), C.byref(traj), max_steps,
                                            C.byref(out)))
        else:
            check(self.L.bd_spiral_heat_run_slabs(self.h, C.byref(thermal), _ptr(Q), C.byref(traj), max_steps,
                                                  int(n_slabs), C.byref(out)))
        shp = (thermal.nz, thermal.ny, thermal.nx)
        for k in ("T", "dose"):
            if k in res:
                res[k] = res[k].reshape(shp)
        if "snapshots" in res:
            res["snapshots"] = res["snapshots"].reshape((legs.size,) + shp)
        res["elapsed_ms"] = out.elapsed_ms
        res["steps_done"] = out.steps_done
        return res

    def heat_slab(self, thermal, Q, traj, z_begin, z_end, max_steps=0):
        """One rank's z slab of the heat run over the planes [z_begin, z_end)
        (bd_heat_slab_begin)."""
        return HeatSlab(self, thermal, Q, traj, z_begin, z_end, max_steps)

    # ------------------------------------------------------------ Gilmore
    def gilmore(self, medium, bubbles, ode):
        """bubbles: numpy array of BUBBLE_DTYPE; returns (results RESULT_DTYPE, device ms)."""
        bubbles = np.ascontiguousarray(bubbles, dtype=BUBBLE_DTYPE)
        res = np.zeros(bubbles.size, RESULT_DTYPE)
        ms = C.c_double(0)
        check(self.L.bd_gilmore_run(self.h, C.byref(medium), bubbles.size, _ptr(bubbles), C.byref(ode),
                                    _ptr(res), C.byref(ms)))
        return res, ms.value

    def gilmore_threshold(self, medium, fr_combo, R0, ref_arith=1, max_steps=0, search=abi.BD_SEARCH_LINEAR):
        """G's threshold search per (combination, R0); search=BD_SEARCH_BISECT
        bisects the last 0.1 MPa bracket instead of G's 10 kPa / 1 kPa scan."""
        fr = np.ascontiguousarray(fr_combo, dtype=np.float64).reshape(-1)
        R0 = np.ascontiguousarray(R0, dtype=np.float64)
        nc = fr.size // 3
        out = np.zeros(nc * R0.size, np.float64)
        ms = C.c_double(0)
        check(self.L.bd_gilmore_threshold_search(self.h, C.byref(medium), _ptr(fr), nc, _ptr(R0), R0.size, ref_arith,
                                                 max_steps, search, _ptr(out), C.byref(ms)))
        return out.reshape(nc, R0.size), ms.value


class HeatSlab:
    """bd_heat_slab_begin / advance / halo_copy / finish / end: one z slab of a
    heat run, stepped by its caller, who refreshes the ghost plane beyond
    each internal face between steps."""

    def __init__(self, ctx, thermal, Q, traj, z_begin, z_end, max_steps=0):
        self.L = ctx.L
        self.shape = (thermal.nz, thermal.ny, thermal.nx)
        self.z = (int(z_begin), int(z_end))
        Q = np.ascontiguousarray(Q, dtype=np.float64).reshape(-1)
        assert Q.size == thermal.nx * thermal.ny * thermal.nz
        h = P()
        check(self.L.bd_heat_slab_begin(ctx.h, C.byref(thermal), _ptr(Q), C.byref(traj), int(max_steps), self.z[0],
                                        self.z[1], C.byref(h)))
        self.h = h

    def steps(self):
        """(steps of the whole run, steps done)"""
        t, d = C.c_int64(0), C.c_int64(0)
        check(self.L.bd_heat_slab_steps(self.h, C.byref(t), C.byref(d)))
        return t.value, d.value

    def advance(self, n):
        check(self.L.bd_heat_slab_advance(self.h, int(n)))

    def halo_bytes(self):
        n = C.c_size_t(0)
        check(self.L.bd_heat_slab_halo_bytes(self.h, C.byref(n)))
        return n.value

    def halo_copy(self, side, to_ghost, d_ptr, stream=None):
        check(self.L.bd_heat_slab_halo_copy(self.h, int(side), int(to_ghost), d_ptr, stream))

    def finish(self):
        """The owned planes of T and the dose, as (z_end - z_begin, ny, nx) arrays."""
        n = self.shape[0] * self.shape[1] * self.shape[2]
        T = np.zeros(n, np.float64)
        D = np.zeros(n, np.float64)
        out = abi.HeatOutputs()
        out.T_final = _ptr(T)
        out.dose = _ptr(D)
        check(self.L.bd_heat_slab_finish(self.h, C.byref(out)))
        zb, ze = self.z
        return {"T": T.reshape(self.shape)[zb:ze].copy(), "dose": D.reshape(self.shape)[zb:ze].copy(),
                "steps_done": out.steps_done}

    def close(self):
        if self.h:
            self.L.bd_heat_slab_end(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class WesterveltSession:
    """bd_westervelt_begin / advance / checkpoint / finish / end."""

    def __init__(self, ctx: Context, prob: WesterveltProblem, slab=None):
        self.ctx = ctx
        self.prob = prob
        self.L = ctx.L
        self.slab = slab
        h = P()
        if slab is None:
            check(self.L.bd_westervelt_begin(ctx.h, C.byref(prob.grid), C.byref(prob.medium), C.byref(prob.source),
                                             C.byref(prob.params), C.byref(h)))
        else:
            check(self.L.bd_westervelt_slab_begin(ctx.h, C.byref(prob.grid), C.byref(prob.medium),
                                                  C.byref(prob.source), C.byref(prob.params), slab[0], slab[1],
                                                  C.byref(h)))
        self.h = h

    # -- z slabs: halo messages of the newest pressure level
    def halo_bytes(self):
        n = C.c_size_t(0)
        check(self.L.bd_westervelt_halo_bytes(self.h, C.byref(n)))
        return n.value

    def halo_copy(self, side, to_ghost, d_ptr, stream=None):
        """side 0 / 1 = low / high z face; to_ghost 0 packs the owned planes into
        the device buffer at d_ptr, 1 unpacks it into the ghost planes."""
        check(self.L.bd_westervelt_halo_copy(self.h, int(side), int(to_ghost), d_ptr, stream))

    def exchange_with(self, upper):
        """Same-device halo exchange with the neighbouring slab above (bd_halo_exchange)."""
        check(self.L.bd_halo_exchange(self.h, upper.h))

    def advance(self, n):
        check(self.L.bd_westervelt_advance(self.h, int(n)))

    def step(self):
        s = C.c_int64(0)
        check(self.L.bd_westervelt_step_index(self.h, C.byref(s)))
        return s.value

    def last_ms(self):
        v = C.c_double(0)
        check(self.L.bd_westervelt_last_ms(self.h, C.byref(v)))
        return v.value

    def checkpoint(self):
        n = C.c_size_t(0)
        check(self.L.bd_checkpoint_size(self.h, C.byref(n)))
        blob = np.zeros(n.value, np.uint8)
        check(self.L.bd_checkpoint_save(self.h, _ptr(blob), n.value))
        return blob

    def restore(self, blob):
        blob = np.ascontiguousarray(blob, dtype=np.uint8)
        check(self.L.bd_checkpoint_load(self.h, _ptr(blob), blob.size))

    def finish(self, want=("p_final", "peak", "energy", "Q", "dft")):
        if self.slab is not None:
            return self._finish_slab(want)
        out, res = Context._outputs(self.prob, want)
        check(self.L.bd_westervelt_finish(self.h, C.byref(out)))
        return Context._shape(self.prob, res, out)

    def _finish_slab(self, want):
        """The owned planes of a slab session, shaped (z_end - z_begin, ny, nx)."""
        zb, ze = self.slab
        g, p = self.prob.grid, self.prob.params
        dt = self.prob.dtype
        plane = g.nx * g.ny
        out = abi.WesterveltOutputs()
        res = {}
        for k in ("p_final", "peak", "energy"):
            if k in want:
                res[k] = np.zeros((ze - zb) * plane, dt)
                setattr(out, k, _ptr(res[k]))
        if "dft" in want and p.n_dft > 0:
            nz = max(0, min(ze, p.dft_z_hi) - max(zb, p.dft_z_lo))
            res["dft_re"] = np.zeros(p.n_dft * plane * nz, dt)
            res["dft_im"] = np.zeros(p.n_dft * plane * nz, dt)
            out.dft_re, out.dft_im = _ptr(res["dft_re"]), _ptr(res["dft_im"])
        if "Q" in want and p.q_mode == abi.BD_Q_REFERENCE:
            res["Q"] = np.zeros((ze - zb) * plane, np.float64)
            out.Q = _ptr(res["Q"])
        check(self.L.bd_westervelt_finish(self.h, C.byref(out)))
        for k in ("p_final", "peak", "energy", "Q"):
            if k in res:
                res[k] = res[k].reshape(ze - zb, g.ny, g.nx)
        res["steps_done"] = out.steps_done
        return res

    def close(self):
        if self.h:
            self.L.bd_westervelt_end(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
