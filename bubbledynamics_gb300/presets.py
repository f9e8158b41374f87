"""Parameter sets: the reference's own (ref_W, ref_T, ref_G), scaled-down
variants of them for tests, and the five benchmark configurations.

Every preset returns plain objects holding the ctypes structs of
``abi`` plus the numpy arrays their pointers refer to (kept alive by the
object).  Physical constants of the reference presets are evaluated with the
same double-precision expressions as the reference's host code, so derived
quantities (layer split, step counts, p0) come out bit-identical.
"""
import math

import numpy as np

from . import abi


# --------------------------------------------------------------------------
# containers
# --------------------------------------------------------------------------
class WesterveltProblem:
    """grid / medium / source / params structs plus the arrays they point to."""

    def __init__(self, name, grid, medium, source, params, keep=None, meta=None):
        self.name = name
        self.grid = grid
        self.medium = medium
        self.source = source
        self.params = params
        self._keep = dict(keep or {})
        self.meta = dict(meta or {})

    @property
    def shape(self):
        g = self.grid
        return (g.nz, g.ny, g.nx)

    @property
    def ncell(self):
        g = self.grid
        return g.nx * g.ny * g.nz

    def keep(self, name, arr):
        self._keep[name] = arr
        return arr

    def array(self, name):
        return self._keep.get(name)

    def set_t_src(self, t):
        t = np.ascontiguousarray(t, dtype=np.float64)
        self.keep("t_src", t)
        self.params.t_src = abi.ptr(t)

    def set_c_map(self, c):
        c = np.ascontiguousarray(c, dtype=np.float32)
        assert c.size == self.ncell
        self.keep("c_map", c)
        self.medium.c_map = abi.ptr(c)

    def set_material_map(self, m):
        m = np.ascontiguousarray(m, dtype=np.uint8)
        assert m.size == self.ncell
        self.keep("material_map", m)
        self.medium.material_map = abi.ptr(m)

    def set_plane_material(self, pm):
        pm = np.ascontiguousarray(pm, dtype=np.int32)
        assert pm.size == self.grid.nz
        self.keep("plane_material", pm)
        self.medium.plane_material = abi.ptr(pm)

    def set_elements(self, element_of_cell, phase, amp):
        e = np.ascontiguousarray(element_of_cell, dtype=np.int32)
        ph = np.ascontiguousarray(phase, dtype=np.float64)
        am = np.ascontiguousarray(amp, dtype=np.float64)
        assert e.size == self.grid.nx * self.grid.ny
        self.keep("element_of_cell", e)
        self.keep("element_phase", ph)
        self.keep("element_amp", am)
        self.source.element_of_cell = abi.ptr(e)
        self.source.element_phase = abi.ptr(ph)
        self.source.element_amp = abi.ptr(am)
        self.source.n_elements = int(ph.size)

    def copy(self):
        """Shallow copy: new structs, same arrays."""
        return WesterveltProblem(self.name, _clone(self.grid), _clone(self.medium), _clone(self.source),
                                 _clone(self.params), dict(self._keep), dict(self.meta))

    @property
    def dtype(self):
        return np.float32 if self.params.precision == abi.BD_F32 else np.float64


def _clone(st):
    import ctypes
    out = type(st)()
    ctypes.memmove(ctypes.byref(out), ctypes.byref(st), ctypes.sizeof(st))
    return out


def accumulate_times(dt, t_end, t_start=0.0):
    """Replicate `while (t < t_end) { ...; t = t + dt; }` (W:558-564) in double:
    returns the times after each increment."""
    out = []
    t = t_start
    while t < t_end:
        t = t + dt
        out.append(t)
    return out


def _material(c0, rho, beta, delta, relax=(), absorption=0.0, harm_absorption=0.0):
    m = abi.Material()
    m.c0, m.rho, m.beta, m.delta = c0, rho, beta, delta
    m.n_relax = len(relax)
    for k, (cv, tau) in enumerate(relax):
        m.relax_c[k] = cv
        m.relax_tau[k] = tau
    m.absorption = absorption
    m.harm_absorption = harm_absorption
    return m


def _params_default(n_steps, precision):
    p = abi.WesterveltParams()
    p.precision = precision
    p.energy_mode = abi.BD_ENERGY_P2
    p.n_steps = n_steps
    p.t0 = 0.0
    p.t_src = None
    p.peak_start, p.peak_end = 0, n_steps
    p.energy_start, p.energy_end = 0, n_steps
    p.dft_start, p.dft_len = 0, 0
    p.n_dft = 0
    p.dft_z_lo, p.dft_z_hi = 0, 0
    p.q_mode = abi.BD_Q_NONE
    p.q_iz_split = 0
    p.q_n_harm = 0
    p.q_freq = 0.0
    p.check_every = 0
    p.fault_at_step = -1
    p.blowup_limit = 0.0
    p.graph_chunk = 0
    p.tile_variant = -1
    p.relax_scheme = abi.BD_RELAX_REFERENCE
    return p


# --------------------------------------------------------------------------
# reference Westervelt program (W:355-416)
# --------------------------------------------------------------------------
def ref_W_constants():
    """Host constants of W:355-416 evaluated in double like the reference."""
    k = {}
    k["fr"] = 1.253 * 10.0 ** 6
    k["d"] = 0.15
    a = 0.151 / 2.0
    k["h"] = k["d"] - math.sqrt((k["d"] * k["d"]) - (a * a))
    a_hole = 0.041 / 2.0
    k["alpha"] = math.asin(a / k["d"])
    k["alpha_hole"] = math.asin(a_hole / k["d"])
    k["rho_water"] = 1000.0
    k["c_water"] = 1500.0
    k["abs_water"] = 0.026 * math.pow(k["fr"] / 10.0 ** 6, 2)
    k["delta_water"] = (2.0 * k["abs_water"] * math.pow(k["c_water"], 3)) / math.pow(2.0 * math.pi * k["fr"], 2)
    k["beta_water"] = 3.5
    k["rho_tissue"] = 1055.0
    k["c_tissue"] = 1600.0
    k["beta_tissue"] = 4.5
    k["abs_tissue"] = 7.2 * k["fr"] / 10.0 ** 6
    k["delta_tissue"] = 4.2318 * math.pow(10.0, -5)
    k["c1"] = 4.03536
    k["c2"] = 6.14150
    k["tau1"] = 1.6178 * math.pow(10.0, -8)
    k["tau2"] = 1.1494 * math.pow(10.0, -7)
    eps, E = 0.89, 100.0
    u0 = math.sqrt(2.0 * E * eps / (k["rho_water"] * k["c_water"] * 2.0 * math.pi * k["d"] * k["h"]))
    k["p0"] = k["rho_water"] * k["c_water"] * u0
    k["water_tissue"] = 0.12
    k["xy_min"], xy_max, k["dxy"] = 0.0, 0.085, 0.0002
    k["Nxy"] = 1 + int(round((xy_max - k["xy_min"]) / k["dxy"]))
    z_max, k["z_min"], k["dz"] = 0.2, -0.0002, 0.0001
    k["Nz"] = 1 + int(round((z_max - k["z_min"]) / k["dz"]))
    k["dt"] = 0.01 / k["fr"]
    k["t_max"] = 165.0 / k["fr"]
    k["periods"] = 4
    k["N_harm"] = 10
    k["iz_tissue"] = 1202
    k["nx_slab"] = 6
    return k


def make_ref_W(k, precision=abi.BD_F64):
    """Westervelt problem equal to the reference program W for constants k
    (full size from ref_W_constants(), or a scaled variant)."""
    Nxy, Nz = k["Nxy"], k["Nz"]
    dt = k["dt"]
    t1 = accumulate_times(dt, k["t_max"])
    n1 = len(t1)
    n_time = k["periods"] * 100                      # W:668
    # the FFT loop restarts from time_165p and accumulates again (W:690-714)
    t = t1[-1]
    t2 = []
    for _ in range(n_time):
        t = t + dt
        t2.append(t)
    n_water = len(accumulate_times(dt, k["t_max"] + 1 / k["fr"], t1[-1]))   # W:627
    n_steps = n1 + n_time
    g = abi.Grid()
    g.nx = g.ny = Nxy
    g.nz = Nz
    g.x0 = g.y0 = k["xy_min"]
    g.z0 = k["z_min"]
    g.dx, g.dz, g.dt = k["dxy"], k["dz"], dt
    g.face[:] = [abi.BD_FACE_MIRROR, abi.BD_FACE_MUR, abi.BD_FACE_MIRROR, abi.BD_FACE_MUR,
                 abi.BD_FACE_MUR, abi.BD_FACE_MUR]
    g.mur_layers = 3
    g.sponge_cells = 0
    g.sponge_strength = 0.0
    med = abi.Medium()
    med.n_materials = 2
    med.mat[0] = _material(k["c_water"], k["rho_water"], k["beta_water"], k["delta_water"],
                           absorption=k["abs_water"])
    med.mat[1] = _material(k["c_tissue"], k["rho_tissue"], k["beta_tissue"], k["delta_tissue"],
                           relax=((k["c1"], k["tau1"]), (k["c2"], k["tau2"])),
                           absorption=k["abs_tissue"], harm_absorption=7.2)
    src = abi.Source()
    src.kind = abi.BD_SRC_BOWL
    src.plane_iz = 2
    src.focal_length = k["d"]
    src.alpha = k["alpha"]
    src.alpha_hole = k["alpha_hole"]
    src.p0 = k["p0"]
    src.c_delay = k["c_water"]
    src.cx = src.cy = 0.0
    src.n_tones = 1
    src.freq[0] = k["fr"]
    src.amp[0] = 1.0
    src.phase[0] = 0.0
    src.burst_cycles = 0.0
    p = _params_default(n_steps, precision)
    p.energy_mode = abi.BD_ENERGY_DPDT2
    p.peak_start, p.peak_end = 0, n_steps
    p.energy_start, p.energy_end = n1, n1 + n_water
    p.dft_start, p.dft_len = n1, n_time
    p.n_dft = k["N_harm"]
    for j in range(k["N_harm"]):
        p.dft_freq[j] = (j + 1) * k["fr"]    # bin 4n of the 400-sample window (W:341)
    p.dft_z_lo, p.dft_z_hi = k["iz_tissue"], Nz
    p.q_mode = abi.BD_Q_REFERENCE
    p.q_iz_split = k["iz_tissue"]
    p.q_n_harm = k["N_harm"]
    p.q_freq = k["fr"]
    prob = WesterveltProblem("ref_W", g, med, src, p, meta={"n_loop1": n1, "n_water": n_water,
                                                             "n_time": n_time, "constants": k})
    # layer of each plane: `z_min + iz*dz < water_tissue` (W:212)
    planes = np.array([0 if (k["z_min"] + iz * k["dz"]) < k["water_tissue"] else 1 for iz in range(Nz)],
                      dtype=np.int32)
    prob.set_plane_material(planes)
    prob.set_t_src(np.array(t1 + t2, dtype=np.float64))
    return prob


def ref_W(precision=abi.BD_F64):
    return make_ref_W(ref_W_constants(), precision)


def ref_W_mini_constants(Nxy=32, Nz=64, loop1_periods=3, periods=4):
    """The reference physics on a small box: same constants and discretisation,
    a bowl scaled so that its ring and focus fall inside the box."""
    k = ref_W_constants()
    k["Nxy"], k["Nz"] = Nxy, Nz
    k["d"] = 0.005
    a, a_hole = 0.004, 0.0008
    k["alpha"] = math.asin(a / k["d"])
    k["alpha_hole"] = math.asin(a_hole / k["d"])
    k["p0"] = 2.0e5
    k["water_tissue"] = 0.003
    k["t_max"] = loop1_periods / k["fr"]
    k["periods"] = periods
    split = [iz for iz in range(Nz) if not (k["z_min"] + iz * k["dz"]) < k["water_tissue"]]
    k["iz_tissue"] = split[0]
    k["nx_slab"] = 8 if Nxy % 8 == 0 else 1
    return k


def ref_W_mini(precision=abi.BD_F64, **kw):
    p = make_ref_W(ref_W_mini_constants(**kw), precision)
    p.name = "ref_W_mini"
    return p


# --------------------------------------------------------------------------
# benchmark configurations
# --------------------------------------------------------------------------
def water_delta(f, c=1500.0):
    """Diffusivity of W:371-372: alpha = 0.026 f_MHz^2 Np/m, delta = 2 alpha c^3 / omega^2."""
    a = 0.026 * (f / 1e6) ** 2
    return (2.0 * a * c ** 3) / (2.0 * math.pi * f) ** 2


def gaussian_heterogeneity(shape, sigma_cells, seed):
    """White noise filtered by a Gaussian of sigma_cells (FFT, periodic), scaled
    to max |g| = 1.  Deterministic for a given seed."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal(shape).astype(np.float64)
    F = np.fft.rfftn(w)
    ks = [np.fft.fftfreq(n) for n in shape[:-1]] + [np.fft.rfftfreq(shape[-1])]
    kk = np.zeros(F.shape)
    for ax, k in enumerate(ks):
        sh = [1] * len(shape)
        sh[ax] = -1
        kk = kk + (k.reshape(sh) ** 2)
    F *= np.exp(-2.0 * (math.pi ** 2) * (sigma_cells ** 2) * kk)
    g = np.fft.irfftn(F, s=shape, axes=tuple(range(len(shape))))
    g /= np.max(np.abs(g))
    return g


def cfg1(nx=128, ny=128, nz=256, n_steps=3000, precision=abi.BD_F32, seed=1, heterogeneity=True):
    """Plain Westervelt FP32, 128x128x256, dx = 0.1875 mm, c = 1500(1 + 0.02 g),
    rho 1000, beta 3.5, one relaxation (tau 1e-7 s, dc 5 m/s), 20 mm bowl with
    16 mm aperture, 1 MHz 10-cycle burst at 0.5 MPa, CFL 0.3, 20-cell sponge.
    Smaller nx/ny/nz/n_steps give the same physics on a smaller box (tests)."""
    dx = 0.1875e-3
    f = 1.0e6
    c0 = 1500.0
    cmax = c0 * 1.02
    dt = 0.3 * dx / cmax
    sponge = 20 if min(nx, ny, nz) >= 96 else max(4, min(nx, ny, nz) // 8)
    g = abi.Grid()
    g.nx, g.ny, g.nz = nx, ny, nz
    g.x0 = -0.5 * (nx - 1) * dx
    g.y0 = -0.5 * (ny - 1) * dx
    g.z0 = -sponge * dx
    g.dx = g.dz = dx
    g.dt = dt
    g.face[:] = [abi.BD_FACE_OPEN] * 6
    g.mur_layers = 0
    g.sponge_cells = sponge
    g.sponge_strength = 0.35
    med = abi.Medium()
    med.n_materials = 1
    med.mat[0] = _material(c0, 1000.0, 3.5, water_delta(f, c0), relax=((5.0, 1e-7),))
    src = abi.Source()
    src.kind = abi.BD_SRC_BOWL
    src.plane_iz = sponge
    scale = nx / 128.0
    F = 20e-3 * scale
    a = 8e-3 * scale
    src.focal_length = F
    src.alpha = math.asin(a / F)
    src.alpha_hole = 0.0
    src.p0 = 0.5e6
    src.c_delay = c0
    src.n_tones = 1
    src.freq[0] = f
    src.amp[0] = 1.0
    src.burst_cycles = 10.0
    p = _params_default(n_steps, precision)
    # CFL 0.3 puts grid-scale modes where the reference's relaxation coupling
    # amplifies them (0.76 % per step); the semi-implicit coupling damps them.
    p.relax_scheme = abi.BD_RELAX_SEMI_IMPLICIT
    prob = WesterveltProblem("cfg1", g, med, src, p, meta={"f": f})
    if heterogeneity:
        sig = 1.0e-3 / dx
        gfield = gaussian_heterogeneity((nz, ny, nx), sig, seed)
        prob.set_c_map((c0 * (1.0 + 0.02 * gfield)).astype(np.float32))
    return prob


# --------------------------------------------------------------------------
# phased-array focusing problem of the adjoint (3 z-slabs, cap-shaped array)
# --------------------------------------------------------------------------
def fibonacci_cap(n, alpha):
    """n points spread evenly over the spherical cap of half-angle alpha
    (Fibonacci lattice): polar angles theta_k and azimuths phi_k."""
    k = np.arange(n, dtype=np.float64) + 0.5
    cos_t = 1.0 - (1.0 - math.cos(alpha)) * k / n
    theta = np.arccos(cos_t)
    phi = np.mod(k * math.pi * (3.0 - math.sqrt(5.0)), 2.0 * math.pi)
    return theta, phi


def assign_cap_elements(prob, n_elements, F, aperture):
    """Make prob's source a cap-shaped array of n_elements (Fibonacci points of
    the cap of focal length F and planar aperture radius `aperture`): every
    source-plane cell inside the aperture belongs to the element whose
    projected centre F tan(theta) (cos phi, sin phi) is nearest.  Phases 0,
    amplitudes 1.  Returns the element angles (theta, phi)."""
    g = prob.grid
    theta, phi = fibonacci_cap(n_elements, math.atan(aperture / F))
    ex = F * np.tan(theta) * np.cos(phi)
    ey = F * np.tan(theta) * np.sin(phi)
    xs = g.x0 + g.dx * np.arange(g.nx)
    ys = g.y0 + g.dx * np.arange(g.ny)
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    d2 = (X[..., None] - ex) ** 2 + (Y[..., None] - ey) ** 2
    elem = np.argmin(d2, axis=-1).astype(np.int32)
    elem[np.hypot(X, Y) > aperture] = -1
    prob.source.kind = abi.BD_SRC_ARRAY
    prob.set_elements(elem.reshape(-1), np.zeros(n_elements), np.ones(n_elements))
    prob.meta["elements"] = (theta, phi)
    return theta, phi


def steering_phases(theta, phi, F, offset, f, c0):
    """Element phases that move the focus of a cap array (focal length F,
    element angles theta / phi) by `offset` = (dx, dy, dz) [m] from its
    geometric focus: each element fires earlier by its extra path to the new
    point, (|r_e - r_spot| - F) / c0, i.e. phase 2 pi f times that."""
    ex = F * np.sin(theta) * np.cos(phi)
    ey = F * np.sin(theta) * np.sin(phi)
    ez = -F * np.cos(theta)                     # the cap lies below the focus
    dxs, dys, dzs = offset
    dist = np.sqrt((ex - dxs) ** 2 + (ey - dys) ** 2 + (ez - dzs) ** 2)
    return 2.0 * math.pi * f * (dist - F) / c0


def slab_materials(f):
    """Water / fat / liver (c, rho, beta, delta, relaxation)."""
    water = _material(1500.0, 1000.0, 3.5, water_delta(f, 1500.0))
    fat = _material(1450.0, 950.0, 6.0, 4.0 * water_delta(f, 1450.0), relax=((3.0, 2.0e-7),))
    liver = _material(1590.0, 1060.0, 4.25, 3.0 * water_delta(f, 1590.0), relax=((5.0, 1.0e-7),))
    return [water, fat, liver]


def focal_array_problem(nx, ny, nz, dx, n_elements, n_steps, window, F, aperture, precision=abi.BD_F32,
                        seed=4, f=1.0e6, p0=0.3e6, sponge=None, slabs=(0.35, 0.55), jitter_cells=1.5,
                        focal_radius=2, side_radius=None, side_weight=0.1, name="focal_array"):
    """A cap-shaped phased array focusing through water / fat / liver slabs.

    The source plane (iz = sponge) carries the bowl delay law of focal length F
    and planar aperture radius `aperture`; element k covers the plane cells
    nearest to the projection F tan(theta_k) (cos phi_k, sin phi_k) of its
    Fibonacci cap point.  Initial element phases are U[0, 2 pi) from `seed`,
    amplitudes 1.  Slab interfaces sit at the fractions `slabs` of the depth
    between the source plane and the far sponge, each displaced per (x, y) by a
    seeded Gaussian-correlated jitter of up to `jitter_cells`.  Continuous wave
    at f; the loss window is the last part of the run.  Returns (problem, loss)."""
    sponge = sponge if sponge is not None else max(4, min(nx, ny, nz) // 10)
    c_max = 1590.0
    dt = 0.3 * dx / c_max
    g = abi.Grid()
    g.nx, g.ny, g.nz = nx, ny, nz
    g.x0 = -0.5 * (nx - 1) * dx
    g.y0 = -0.5 * (ny - 1) * dx
    g.z0 = -sponge * dx
    g.dx = g.dz = dx
    g.dt = dt
    g.face[:] = [abi.BD_FACE_OPEN] * 6
    g.mur_layers = 0
    g.sponge_cells = sponge
    g.sponge_strength = 0.35
    med = abi.Medium()
    mats = slab_materials(f)
    med.n_materials = len(mats)
    for k, m in enumerate(mats):
        med.mat[k] = m
    src = abi.Source()
    src.kind = abi.BD_SRC_ARRAY
    src.plane_iz = sponge
    src.focal_length = F
    src.alpha = math.atan(aperture / F)
    src.alpha_hole = 0.0
    src.p0 = p0
    src.c_delay = 1500.0
    src.n_tones = 1
    src.freq[0] = f
    src.amp[0] = 1.0
    src.burst_cycles = 0.0
    p = _params_default(n_steps, precision)
    p.relax_scheme = abi.BD_RELAX_SEMI_IMPLICIT
    p.peak_start = p.peak_end = 0
    p.energy_start, p.energy_end = window
    prob = WesterveltProblem(name, g, med, src, p, meta={"f": f})
    rng = np.random.default_rng(seed)
    # slabs with jittered interfaces
    depth = nz - 2 * sponge
    z = np.arange(nz).reshape(nz, 1, 1)
    mm = np.zeros((nz, ny, nx), np.uint8)
    for k, frac in enumerate(slabs):
        jit = gaussian_heterogeneity((ny, nx), max(1.0, 1.0e-3 / dx), seed + 10 + k) * jitter_cells
        zi = sponge + frac * depth + jit.reshape(1, ny, nx)
        mm[z >= zi] = k + 1
    prob.set_material_map(mm)
    theta, phi = assign_cap_elements(prob, n_elements, F, aperture)
    phase = rng.uniform(0.0, 2.0 * math.pi, n_elements)
    prob.set_elements(prob.array("element_of_cell"), phase, np.ones(n_elements))
    loss = abi.FocalLoss()
    loss.focus_ix, loss.focus_iy = nx // 2, ny // 2
    loss.focus_iz = min(nz - sponge - 1, sponge + int(round(F / dx)))
    loss.focal_radius = focal_radius
    loss.side_radius = side_radius if side_radius is not None else 3 * focal_radius
    loss.checkpoint_every = 0
    loss.side_weight = side_weight
    loss.window_start, loss.window_end = window
    return prob, loss


def cfg4(n_steps=4000, precision=abi.BD_F32, seed=4):
    """Adjoint configuration: 192^3 at dx = 0.2 mm, water / fat / liver slabs
    with jittered interfaces, 256-element cap array (F = 25 mm, aperture
    radius 14 mm) at 1 MHz CW with seeded random phases, 20-cell sponge;
    loss = -(focal energy) + 0.1 (focal-plane side-lobe energy) over the
    last quarter of the run."""
    w = (3 * n_steps // 4, n_steps)
    return focal_array_problem(192, 192, 192, 0.2e-3, 256, n_steps, w, 25e-3, 14e-3, precision=precision,
                               seed=seed, sponge=20, focal_radius=4, side_radius=12, name="cfg4")


def adjoint_mini(precision=abi.BD_F64, n_elements=16, n_steps=200, seed=4):
    """The cfg4 physics on a 24 x 24 x 36 box (dx = 0.2 mm, 16 elements) for
    gradient checks."""
    w = (n_steps - 60, n_steps)
    return focal_array_problem(24, 24, 36, 0.2e-3, n_elements, n_steps, w, 3.6e-3, 1.5e-3, precision=precision,
                               seed=seed, sponge=4, focal_radius=2, side_radius=5, name="adjoint_mini")


# --------------------------------------------------------------------------
# bioheat program (T:114-224)
# --------------------------------------------------------------------------
class ThermalProblem:
    """bd_thermal + bd_trajectory structs plus the arrays they point to."""

    def __init__(self, name, thermal, traj, keep=None, meta=None):
        self.name = name
        self.thermal = thermal
        self.traj = traj
        self._keep = dict(keep or {})
        self.meta = dict(meta or {})

    @property
    def shape(self):
        t = self.thermal
        return (t.nz, t.ny, t.nx)

    def set_plane_material(self, pm):
        pm = np.ascontiguousarray(pm, dtype=np.int32)
        self._keep["plane_material"] = pm
        self.thermal.plane_material = abi.ptr(pm)

    def set_material_map(self, m):
        """Per-cell material indices (uint8, nz x ny x nx); overrides the plane materials."""
        m = np.ascontiguousarray(m, dtype=np.uint8)
        self._keep["material_map"] = m
        self.thermal.material_map = abi.ptr(m)

    def set_spots(self, sx, sy, steps):
        sx = np.ascontiguousarray(sx, dtype=np.int32)
        sy = np.ascontiguousarray(sy, dtype=np.int32)
        st = np.ascontiguousarray(steps, dtype=np.int64)
        self._keep.update(spot_sx=sx, spot_sy=sy, spot_steps=st)
        self.traj.kind = abi.BD_TRAJ_SPOTS
        self.traj.n_spots = sx.size
        self.traj.spot_sx, self.traj.spot_sy, self.traj.spot_steps = abi.ptr(sx), abi.ptr(sy), abi.ptr(st)

    def set_start(self, T, dose):
        """Start the next run from these fields (a run continuing an earlier one)."""
        T = np.ascontiguousarray(T, dtype=np.float64)
        dose = np.ascontiguousarray(dose, dtype=np.float64)
        self._keep.update(T_start=T, dose_start=dose)
        self.thermal.T_start, self.thermal.dose_start = abi.ptr(T), abi.ptr(dose)

    def initial_fields(self):
        """Initial T and dose as T:232-257 sets them (dose_init = 1), or the
        start fields of set_start."""
        if self._keep.get("T_start") is not None:
            return (self._keep["T_start"].reshape(self.shape).copy(),
                    self._keep["dose_start"].reshape(self.shape).copy())
        t = self.thermal
        pm = self._keep.get("plane_material")
        T = np.zeros(self.shape)
        TD = np.zeros(self.shape)
        for iz in range(t.nz):
            m = t.mat[int(pm[iz]) if pm is not None else 0]
            T[iz] = m.T_init
            TD[iz] = math.pow(4.0, m.T_init - 273.15 - 43.0) * t.dt if t.dose_init else 0.0
        return T, TD


def _thermal_material(rho, c_t, k_t, T_init, perfusion=0.0, T_art=None):
    m = abi.ThermalMaterial()
    m.rho, m.c_t, m.k_t, m.T_init = rho, c_t, k_t, T_init
    m.perfusion = perfusion
    m.T_art = T_init if T_art is None else T_art
    return m


def ref_T_constants():
    k = {}
    k["xy_min"], xy_max, k["dxy"] = -0.085, 0.085, 0.0002
    k["Nxy"] = 1 + int(round((xy_max - k["xy_min"]) / k["dxy"]))
    k["Nxy_half"] = k["Nxy"] // 2
    z_max, k["dz"] = 0.2, 0.0001
    k["Nz"] = 1 + int(round(z_max / k["dz"]))
    k["dt_T"] = 0.001
    k["rho_water"], k["c_t_water"], k["K_water"] = 1000.0, 4200.0, 0.6
    k["rho_tissue"], k["c_t_tissue"], k["K_tissue"] = 1055.0, 3700.0, 0.51
    k["water_tissue"] = 0.12
    k["T0"] = 23.6 + 273.15
    k["T0_water"] = 22.7 + 273.15
    k["speed"] = 2.0 * math.pow(10.0, -3)
    k["scale"] = 3.0 * math.pow(10.0, -3)
    k["speed_init"] = 0.05 * math.pow(10.0, -3)
    k["t_acc"] = 0.15
    k["spiral_lines"] = 13
    return k


def make_ref_T(k, precision=abi.BD_F64, name="ref_T"):
    t = abi.Thermal()
    t.nx = t.ny = k["Nxy"]
    t.nz = k["Nz"]
    t.precision = precision
    t.dx, t.dz, t.dt = k["dxy"], k["dz"], k["dt_T"]
    t.T_ref = k["T0"]
    t.n_materials = 2
    t.dose_init = 1
    t.mat[0] = _thermal_material(k["rho_water"], k["c_t_water"], k["K_water"], k["T0_water"])
    t.mat[1] = _thermal_material(k["rho_tissue"], k["c_t_tissue"], k["K_tissue"], k["T0"])
    tr = abi.Trajectory()
    tr.kind = abi.BD_TRAJ_SQUARE_SPIRAL
    tr.n_legs = k["spiral_lines"]
    tr.speed, tr.scale, tr.speed_init, tr.t_acc = k["speed"], k["scale"], k["speed_init"], k["t_acc"]
    tr.dxy, tr.dt = k["dxy"], k["dt_T"]
    prob = ThermalProblem(name, t, tr, meta={"constants": k})
    # `Z = iz*dz; Z < water_tissue` (T:79, T:84)
    prob.set_plane_material([0 if iz * k["dz"] < k["water_tissue"] else 1 for iz in range(k["Nz"])])
    return prob


def ref_T(precision=abi.BD_F64):
    return make_ref_T(ref_T_constants(), precision)


def ref_T_mini_constants(Nxy=41, Nz=48, legs=3):
    k = ref_T_constants()
    k["Nxy"], k["Nz"] = Nxy, Nz
    k["Nxy_half"] = Nxy // 2
    k["water_tissue"] = 0.0024
    k["speed"] = 0.02
    k["scale"] = 0.0006
    k["t_acc"] = 0.02
    k["spiral_lines"] = legs
    return k


def thermal_cfg_constants(k):
    """kdt / dt_rho_ct constants of T:212-217 for a constants dict."""
    kt = k["K_tissue"] / (k["rho_tissue"] * k["c_t_tissue"])
    kw = k["K_water"] / (k["rho_water"] * k["c_t_water"])
    return {
        "kdt_dxy": k["dt_T"] * kt / (k["dxy"] * k["dxy"]),
        "kdt_dz": k["dt_T"] * kt / (k["dz"] * k["dz"]),
        "kdt_dxy_water": k["dt_T"] * kw / (k["dxy"] * k["dxy"]),
        "kdt_dz_water": k["dt_T"] * kw / (k["dz"] * k["dz"]),
        "dt_rho_ct": k["dt_T"] / (k["rho_tissue"] * k["c_t_tissue"]),
        "dt_rho_ct_water": k["dt_T"] / (k["rho_water"] * k["c_t_water"]),
    }


def gaussian_focus_Q(shape, center, sigma_cells, q_max):
    """Synthetic heat source: a Gaussian focal spot [W/m^3]."""
    nz, ny, nx = shape
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    sz, sy, sx = sigma_cells
    cz, cy, cx = center
    return q_max * np.exp(-0.5 * (((z - cz) / sz) ** 2 + ((y - cy) / sy) ** 2 + ((x - cx) / sx) ** 2))


# --------------------------------------------------------------------------
# cfg3: liver heating along a 49-spot square spiral
# --------------------------------------------------------------------------
CFG3 = dict(nx=256, ny=256, nz=384, dx=0.15e-3, f=1.2e6, p0=0.11e6, F=40e-3, aperture=15e-3,
            water_mm=10.0, sponge=20, n_spots_side=7, pitch=1.667e-3, spot_s=2.0, dt_T=1e-3)


def liver_acoustic(f=1.2e6, c=1590.0):
    """Liver for the acoustic solver: c 1590, rho 1060, beta 4.25, 0.5 dB/cm/MHz
    through two fitted relaxation processes (relax_fit) on top of a water-like
    thermoviscous term.  Returns (bd_material, alpha0 [Np/m/MHz], fit error)."""
    from . import relax_fit as rf
    a0 = rf.db_cm_mhz_to_np_m_mhz(0.5)
    delta = water_delta(f, c)
    relax, err = rf.fit_relaxation(a0, 1.0, c, delta)
    return _material(c, 1060.0, 4.25, delta, relax=relax, absorption=a0 * f / 1e6), a0, err


def cfg3_acoustic(nx=None, ny=None, nz=None, n_steps=None, precision=abi.BD_F32):
    """The acoustic half of cfg3: FP32 Westervelt on 256x256x384 at dx = 0.15 mm,
    a 10 mm water path then liver, a 1.2 MHz bowl (F = 40 mm, aperture radius
    15 mm) continuous wave, 20-cell sponges.  The bowl's surface pressure of
    0.11 MPa gives about 1.5 MPa at the focus (focusing gain ~14).  The energy window is
    the last ten periods, after the wave front has crossed the box.  Smaller
    sizes scale the geometry (tests)."""
    k = CFG3
    nx = nx or k["nx"]; ny = ny or k["ny"]; nz = nz or k["nz"]
    scale = nz / k["nz"]
    dx = k["dx"]
    sponge = k["sponge"] if min(nx, ny, nz) >= 96 else max(4, min(nx, ny, nz) // 10)
    g = abi.Grid()
    g.nx, g.ny, g.nz = nx, ny, nz
    g.x0 = -0.5 * (nx - 1) * dx
    g.y0 = -0.5 * (ny - 1) * dx
    g.z0 = -sponge * dx
    g.dx = g.dz = dx
    g.dt = 0.3 * dx / 1590.0
    g.face[:] = [abi.BD_FACE_OPEN] * 6
    g.sponge_cells = sponge
    g.sponge_strength = 0.35
    liver, a0, err = liver_acoustic(k["f"])
    med = abi.Medium()
    med.n_materials = 2
    med.mat[0] = _material(1500.0, 1000.0, 3.5, water_delta(k["f"]), absorption=0.026 * (k["f"] / 1e6) ** 2)
    med.mat[1] = liver
    src = abi.Source()
    src.kind = abi.BD_SRC_BOWL
    src.plane_iz = sponge
    F = k["F"] * scale
    src.focal_length = F
    src.alpha = math.atan(min(k["aperture"] * scale, 0.5 * min(nx, ny) * dx - (sponge + 2) * dx) / F)
    src.p0 = k["p0"]
    src.c_delay = 1500.0
    src.n_tones = 1
    src.freq[0] = k["f"]
    src.amp[0] = 1.0
    period = 1.0 / k["f"]
    if n_steps is None:
        t_cross = (nz * dx) / 1500.0 + 5 * period
        n_steps = int(math.ceil(t_cross / g.dt)) + int(math.ceil(10 * period / g.dt))
    p = _params_default(n_steps, precision)
    p.relax_scheme = abi.BD_RELAX_SEMI_IMPLICIT
    p.peak_start, p.peak_end = 0, n_steps
    n_win = int(round(10 * period / g.dt))
    p.energy_start, p.energy_end = n_steps - n_win, n_steps
    prob = WesterveltProblem("cfg3_acoustic", g, med, src, p,
                             meta={"f": k["f"], "alpha0": a0, "fit_error": err, "window_s": n_win * g.dt})
    iz_liver = sponge + int(round(k["water_mm"] * 1e-3 * scale / dx))
    prob.set_plane_material([0 if iz < iz_liver else 1 for iz in range(nz)])
    return prob


def cfg3_array(n_elements=256, **kw):
    """cfg3's acoustic problem with the bowl split into a cap-shaped array of
    n_elements, for electronic steering of the focus (steering_phases)."""
    prob = cfg3_acoustic(**kw)
    F = prob.source.focal_length
    aperture = F * math.tan(prob.source.alpha)
    assign_cap_elements(prob, n_elements, F, aperture)
    prob.name = "cfg3_array"
    return prob


def square_spiral_spots(n_side, pitch_cells):
    """Offsets (sx, sy) in cells of n_side^2 spots on a square spiral starting
    at the centre (right, down, left, left, up, up, right x3, ...)."""
    xs, ys = [0], [0]
    x = y = 0
    leg, d = 1, 0
    dirs = [(1, 0), (0, 1), (-1, 0), (0, -1)]
    while len(xs) < n_side * n_side:
        for _ in range(2):
            for _ in range(leg):
                x += dirs[d][0]
                y += dirs[d][1]
                if len(xs) < n_side * n_side:
                    xs.append(x)
                    ys.append(y)
            d = (d + 1) % 4
        leg += 1
    sx = np.round(np.array(xs) * pitch_cells).astype(np.int32)
    sy = np.round(np.array(ys) * pitch_cells).astype(np.int32)
    return sx, sy


def cfg3_thermal(prob_acoustic, n_spots=None, steps_per_spot=None, precision=abi.BD_F32):
    """The thermal half of cfg3 on the acoustic grid: water (k 0.6, rho 1000,
    c_p 4180) then liver (k 0.52, rho 1060, c_p 3600, perfusion 0.0167 1/s),
    37 C everywhere, dt = 1 ms, 49 spots of 2 s on a 10 mm square spiral
    (7 x 7, 1.667 mm pitch), CEM43 dose from zero."""
    k = CFG3
    g = prob_acoustic.grid
    t = abi.Thermal()
    t.nx, t.ny, t.nz = g.nx, g.ny, g.nz
    t.precision = precision
    t.dx, t.dz, t.dt = g.dx, g.dz, k["dt_T"]
    t.T_ref = 310.15
    t.n_materials = 2
    t.dose_init = 0
    t.mat[0] = _thermal_material(1000.0, 4180.0, 0.6, 310.15)
    t.mat[1] = _thermal_material(1060.0, 3600.0, 0.52, 310.15, perfusion=0.0167, T_art=310.15)
    tr = abi.Trajectory()
    tr.dxy, tr.dt = g.dx, k["dt_T"]
    prob = ThermalProblem("cfg3_thermal", t, tr)
    prob.set_plane_material(prob_acoustic.array("plane_material"))
    sx, sy = square_spiral_spots(k["n_spots_side"], k["pitch"] / g.dx)
    n = len(sx) if n_spots is None else n_spots
    steps = int(round(k["spot_s"] / k["dt_T"])) if steps_per_spot is None else steps_per_spot
    prob.set_spots(sx[:n], sy[:n], np.full(n, steps, np.int64))
    return prob


# --------------------------------------------------------------------------
# cfg5: large nonlinear field, 9-frequency DFT, bubbles driven by the field
# --------------------------------------------------------------------------
CFG5 = dict(nx=512, ny=512, nz=768, dx=0.1e-3, tones=(1.0e6, 1.1e6, 1.2e6), p_tone=2.0e6, F=64e-3,
            aperture=22e-3, sponge=20, n_steps=12000, window_s=10e-6, focal_mm=(2.0, 5.0))


def cfg5(nx=None, ny=None, nz=None, n_steps=None, window_steps=None, precision=abi.BD_F32):
    """Large nonlinear Westervelt: 512x512x768 at dx = 0.1 mm in liver (two
    fitted relaxation processes), a 64 mm bowl (aperture radius 22 mm) driven
    by 1.0 / 1.1 / 1.2 MHz, each tone about 2 MPa at the focus (bowl surface
    2/17.5 MPa per tone, focusing gain ~17.5), 12,000 steps with dt chosen so
    that 10 us is exactly 530 steps (CFL 0.30), and the on-the-fly DFT at the
    three fundamentals and their 2nd and 3rd harmonics over the last 10 us, kept
    on the planes within 10 mm of the focus.  Smaller sizes scale the geometry."""
    k = CFG5
    nx = nx or k["nx"]; ny = ny or k["ny"]; nz = nz or k["nz"]
    scale = nz / k["nz"]
    dx = k["dx"]
    sponge = k["sponge"] if min(nx, ny, nz) >= 96 else max(4, min(nx, ny, nz) // 10)
    spw = 530                                   # steps per 10 us
    g = abi.Grid()
    g.nx, g.ny, g.nz = nx, ny, nz
    g.x0 = -0.5 * (nx - 1) * dx
    g.y0 = -0.5 * (ny - 1) * dx
    g.z0 = -sponge * dx
    g.dx = g.dz = dx
    g.dt = k["window_s"] / spw
    g.face[:] = [abi.BD_FACE_OPEN] * 6
    g.sponge_cells = sponge
    g.sponge_strength = 0.35
    liver, a0, err = liver_acoustic(1.1e6)
    med = abi.Medium()
    med.n_materials = 1
    med.mat[0] = liver
    src = abi.Source()
    src.kind = abi.BD_SRC_BOWL
    src.plane_iz = sponge
    F = k["F"] * scale
    src.focal_length = F
    src.alpha = math.atan(min(k["aperture"] * scale, 0.5 * min(nx, ny) * dx - (sponge + 2) * dx) / F)
    src.p0 = k["p_tone"] / 17.5
    src.c_delay = 1590.0
    src.n_tones = len(k["tones"])
    for j, f in enumerate(k["tones"]):
        src.freq[j] = f
        src.amp[j] = 1.0
    n_steps = n_steps or (k["n_steps"] if scale == 1.0 else int(round(k["n_steps"] * scale)))
    n_win = window_steps or spw
    p = _params_default(n_steps, precision)
    p.relax_scheme = abi.BD_RELAX_SEMI_IMPLICIT
    p.peak_start, p.peak_end = 0, n_steps
    p.energy_start, p.energy_end = n_steps - n_win, n_steps
    freqs = [f * h for h in (1, 2, 3) for f in k["tones"]]
    p.n_dft = len(freqs)
    for j, f in enumerate(freqs):
        p.dft_freq[j] = f
    p.dft_start, p.dft_len = n_steps - n_win, n_win
    iz_f = sponge + int(round(F / dx))
    half = int(round(10e-3 * scale / dx))
    p.dft_z_lo, p.dft_z_hi = max(0, iz_f - half), min(nz, iz_f + half)
    return WesterveltProblem("cfg5", g, med, src, p, meta={"f": 1.1e6, "iz_focus": iz_f, "fit_error": err,
                                                            "dft_freqs": freqs})


# --------------------------------------------------------------------------
# Gilmore program (G:440-470) and the batched forward configuration
# --------------------------------------------------------------------------
def ref_G_medium():
    m = abi.GilmoreMedium()
    m.rho = 1100.0
    m.P0 = 1.013 * math.pow(10.0, 5)
    m.S2 = 2.0 * 0.056
    m.mu4 = 4.0 * 0.009
    m.G4_3 = 0.04 * math.pow(10.0, 6) * 4.0 / 3.0
    m.C_inf = 1549.0
    m.lambda_ = 3.0 * math.pow(10.0, -9)
    m.n = 7.0
    m.B = (m.C_inf * m.C_inf * m.rho / m.n) - m.P0
    m.gamma = 1.4
    return m


def ref_G_R0s():
    """R0 = minR0 + i*stepR0 (G:332, G:457-460)."""
    stepR0 = math.pow(10.0, -7)
    minR0 = math.pow(10.0, -7)
    maxR0 = math.pow(10.0, -5)
    N_R0 = 1 + int((maxR0 - minR0) / stepR0)
    return np.array([minR0 + i * stepR0 for i in range(N_R0)])


def cfg2_medium():
    """Liver-like medium of the batched Gilmore configuration; G and lambda
    keep the reference values (G:444, G:446)."""
    m = abi.GilmoreMedium()
    m.rho = 1060.0
    m.P0 = 1.013e5
    m.S2 = 2.0 * 0.056
    m.mu4 = 4.0 * 0.005
    m.G4_3 = 0.04e6 * 4.0 / 3.0
    m.C_inf = 1590.0
    m.lambda_ = 3.0e-9
    m.n = 7.15
    m.B = 3.049e8
    m.gamma = 1.4
    return m


def cfg2_bubbles(n=1 << 20, seed=2, freqs=(1.0e6, 1.1e6, 1.2e6)):
    """R0 log-uniform in [0.5, 5] um, A ~ U[0.5, 3] MPa split equally over the
    three tones (A/sqrt(3) each, the triple combo of G:55), phases U[0, 2 pi)."""
    from .api import BUBBLE_DTYPE
    rng = np.random.default_rng(seed)
    b = np.zeros(n, BUBBLE_DTYPE)
    b["R0"] = np.exp(rng.uniform(np.log(0.5e-6), np.log(5e-6), n))
    A = rng.uniform(0.5e6, 3.0e6, n)
    b["n_tones"] = len(freqs)
    for k, f in enumerate(freqs):
        b["f"][:, k] = f
        b["a"][:, k] = A / math.sqrt(len(freqs))
    b["phi"][:, :len(freqs)] = rng.uniform(0.0, 2.0 * math.pi, (n, len(freqs)))
    return b


def cfg2_ode(t_end=200e-6, rtol=1e-8, atol=1e-14, max_steps=10 ** 7):
    o = abi.OdeParams()
    o.t_end, o.h0, o.atol, o.rtol, o.fac_max = t_end, 1e-13, atol, rtol, 5.0
    o.max_steps = max_steps
    o.stop_at_threshold = 0
    o.ref_arith = 0
    return o
