"""cfg3 (liver heating along a spiral of focal spots) on a reduced box: the
acoustic solve against the FP64 oracle, the W -> T hand-off, and the heat +
dose run against the oracle.  Tolerances: FP32 energy map 1e-5 relative L2
(the field tolerance); heat FP32 within 1e-5 of the largest temperature
rise, dose within 2 ln(4) x that temperature tolerance relative (the dose is
exponential in T)."""
import numpy as np
import pytest

from bubbledynamics_gb300 import abi, api, pipeline, presets

pytestmark = pytest.mark.gpu


def _small():
    return presets.cfg3_acoustic(nx=48, ny=48, nz=72)


def test_cfg3_acoustic_matches_oracle(ctx, oracle):
    p32 = _small()
    r = ctx.westervelt(p32, want=("energy", "peak"))
    p64 = _small()
    p64.params.precision = abi.BD_F64
    e = oracle.westervelt(p64, want=("energy", "peak"))
    for k in ("energy", "peak"):
        rel = np.linalg.norm(r[k].astype(np.float64) - e[k]) / np.linalg.norm(e[k])
        assert rel <= 1e-5, (k, rel)
    assert r["peak"].max() > 1e5


def test_cfg3_heat_along_spots_matches_oracle(ctx, oracle):
    ac = _small()
    res = pipeline.cfg3_run(ctx, acoustic=ac, n_spots=3, steps_per_spot=150)
    Q = res["Q"]
    assert Q.max() > 0
    th = res["thermal"]
    sx, sy, _ = api.trajectory_shifts(th.traj)
    assert len(sx) == 450
    T0, TD0 = th.initial_fields()
    T, TD, _ = oracle.heat(th.thermal, Q, sx, sy, T0, TD0)
    rise = np.abs(T - T0).max()
    assert rise > 1e-3
    assert np.abs(res["T"] - T).max() <= 1e-5 * rise
    # the dose increment is 4^(T - 43) dt below 43 C, so a temperature error e
    # moves it by ln(4) e relative: the dose tolerance follows the temperature one
    rtol = max(1e-5, 2.0 * np.log(4.0) * 1e-5 * rise)
    np.testing.assert_allclose(res["dose"], TD, rtol=rtol, atol=1e-300)
