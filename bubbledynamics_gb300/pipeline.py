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
