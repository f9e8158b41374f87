"""Acoustic -> thermal hand-off (the reference's W -> T file hand-off, W:757-790
-> T:269-306, done in memory) and the cfg3 heating run.

W writes the absorbed power Q [W/m^3] to a file and T reads it back; here the
energy map of a Westervelt solve becomes Q directly:

    Q(x) = 2 alpha(x) <p^2>(x) / (rho(x) c(x)),   <p^2> = E(x) / T_window

with E the p^2 dt energy accumulated over a whole number of periods and
alpha the absorption of the cell's material at the drive frequency (the
plane-wave intensity form of W:261's water power).
"""
import numpy as np

from . import abi, presets


def heat_source_from_energy(prob, energy, window_s):
    """Q [W/m^3] on the acoustic grid from a P2 energy map (float64 array)."""
    med = prob.medium
    nz = prob.grid.nz
    pm = prob.array("plane_material")
    mm = prob.array("material_map")
    cmap = prob.array("c_map")
    E = np.asarray(energy, dtype=np.float64).reshape(prob.shape)
    if mm is not None:
        mat = mm.reshape(prob.shape).astype(np.int64)
    elif pm is not None:
        mat = np.broadcast_to(np.asarray(pm, np.int64).reshape(nz, 1, 1), prob.shape)
    else:
        mat = np.zeros(prob.shape, np.int64)
    alpha = np.array([med.mat[k].absorption for k in range(med.n_materials)])[mat]
    rho = np.array([med.mat[k].rho for k in range(med.n_materials)])[mat]
    c = (cmap.reshape(prob.shape).astype(np.float64) if cmap is not None
         else np.array([med.mat[k].c0 for k in range(med.n_materials)])[mat])
    return 2.0 * alpha * (E / window_s) / (rho * c)


def cfg3_run(ctx, acoustic=None, n_spots=None, steps_per_spot=None, thermal_precision=abi.BD_F32):
    """cfg3 end to end on the device: Westervelt (energy over ten periods) ->
    Q -> bioheat + CEM43 dose along the spiral.  Returns a dict with the
    acoustic and thermal results and their device times."""
    ac = acoustic or presets.cfg3_acoustic()
    r = ctx.westervelt(ac, want=("energy", "peak"))
    Q = heat_source_from_energy(ac, r["energy"], ac.meta["window_s"])
    th = presets.cfg3_thermal(ac, n_spots=n_spots, steps_per_spot=steps_per_spot, precision=thermal_precision)
    h = ctx.heat(th.thermal, Q, th.traj)
    return {"acoustic": ac, "thermal": th, "Q": Q, "peak": r["peak"], "acoustic_ms": r["elapsed_ms"],
            "T": h["T"], "dose": h["dose"], "heat_ms": h["elapsed_ms"], "heat_steps": h["steps_done"]}


def steered_spots_run(ctx, acoustic, n_spots=None, steps_per_spot=None, thermal_precision=abi.BD_F32,
                      keep_q=False):
    """The spiral of cfg3 with the field re-solved for every spot (instead of
    translating one Q, T:61-77): the array source of `acoustic` (cfg3_array) is
    steered electronically to each spot, the Westervelt solve gives that
    spot's Q, and the heat run continues from the previous spot's temperature
    and dose with the source in place.  Returns the final T and dose, the
    focal peak position per spot and the device times."""
    from . import presets as P
    g = acoustic.grid
    theta, phi = acoustic.meta["elements"]
    F = acoustic.source.focal_length
    f = acoustic.source.freq[0]
    th0 = P.cfg3_thermal(acoustic, n_spots=n_spots, steps_per_spot=steps_per_spot, precision=thermal_precision)
    sx, sy, steps = th0._keep["spot_sx"], th0._keep["spot_sy"], th0._keep["spot_steps"]
    T, dose = th0.initial_fields()
    amps = acoustic.array("element_amp")
    elem = acoustic.array("element_of_cell")
    peaks, qs, ac_ms, heat_ms = [], [], 0.0, 0.0
    izf = acoustic.source.plane_iz + int(round(F / g.dz))
    for k in range(len(sx)):
        q = acoustic.copy()
        q.set_elements(elem, P.steering_phases(theta, phi, F, (sx[k] * g.dx, sy[k] * g.dx, 0.0), f, 1500.0), amps)
        r = ctx.westervelt(q, want=("energy", "peak"))
        ac_ms += r["elapsed_ms"]
        pk = r["peak"][izf]
        peaks.append(np.unravel_index(int(np.argmax(pk)), pk.shape))
        Q = heat_source_from_energy(q, r["energy"], q.meta["window_s"])
        if keep_q:
            qs.append(Q)
        th = P.cfg3_thermal(acoustic, n_spots=1, steps_per_spot=int(steps[k]), precision=thermal_precision)
        th.set_spots([0], [0], [int(steps[k])])
        th.set_start(T, dose)
        h = ctx.heat(th.thermal, Q, th.traj)
        heat_ms += h["elapsed_ms"]
        T, dose = h["T"], h["dose"]
    return {"T": T, "dose": dose, "focal_peaks": peaks, "spots": list(zip(sx.tolist(), sy.tolist())),
            "steps": steps.tolist(), "Q": qs, "acoustic_ms": ac_ms, "heat_ms": heat_ms}


def bubbles_from_dft(prob, dft_re, dft_im, n, seed=5, radius=2e-3, length=5e-3, R0_range=(0.5e-6, 5e-6)):
    """n bubbles at seeded random points of the focal region (a cylinder of
    `radius` and +-`length` around the focus), each driven by the field at its
    cell as reconstructed from the DFT: tone j has frequency f_j, amplitude
    2 |X_j| / N and phase arg X_j + pi/2, so that sum_j a_j sin(2 pi f_j t + phi_j)
    is the pressure there with t = 0 at the start of the DFT window (the sample
    phase of the accumulators is 2 pi f (s - dft_start) dt).  R0 log-uniform in
    R0_range (the cfg2 distribution).  Returns (bubbles, cell indices)."""
    from .api import BUBBLE_DTYPE
    p = prob.params
    g = prob.grid
    rng = np.random.default_rng(seed)
    izf = prob.meta["iz_focus"]
    r = radius * np.sqrt(rng.uniform(0.0, 1.0, n))
    th = rng.uniform(0.0, 2.0 * np.pi, n)
    zz = rng.uniform(-length, length, n)
    ix = np.clip(np.round((r * np.cos(th) - g.x0) / g.dx).astype(np.int64), 0, g.nx - 1)
    iy = np.clip(np.round((r * np.sin(th) - g.y0) / g.dx).astype(np.int64), 0, g.ny - 1)
    iz = np.clip(izf + np.round(zz / g.dz).astype(np.int64), p.dft_z_lo, p.dft_z_hi - 1)
    nd = p.n_dft
    plane = g.nx * g.ny
    nzd = p.dft_z_hi - p.dft_z_lo
    re = np.asarray(dft_re, dtype=np.float64).reshape(nd, nzd * plane)
    im = np.asarray(dft_im, dtype=np.float64).reshape(nd, nzd * plane)
    cell = (iz - p.dft_z_lo) * plane + iy * g.nx + ix
    X = re[:, cell] + 1j * im[:, cell]                      # (nd, n)
    b = np.zeros(n, BUBBLE_DTYPE)
    b["R0"] = np.exp(rng.uniform(np.log(R0_range[0]), np.log(R0_range[1]), n))
    b["n_tones"] = nd
    for j in range(nd):
        b["f"][:, j] = p.dft_freq[j]
        b["a"][:, j] = 2.0 * np.abs(X[j]) / p.dft_len
        b["phi"][:, j] = np.angle(X[j]) + 0.5 * np.pi
    return b, (iz * plane + iy * g.nx + ix)
