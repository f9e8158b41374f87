"""Electronic steering of a cap-shaped array and the spiral with the field
re-solved per spot (cfg3 physics on a reduced box).  Tolerances: the focal
maximum lands within one cell of the steered offset; heat FP32 within 1e-5
of the largest temperature rise and dose within 2 ln(4) x that, as in the
cfg3 tests."""
import numpy as np
import pytest

from bubbledynamics_gb300 import abi, pipeline, presets

pytestmark = pytest.mark.gpu


def _small():
    return presets.cfg3_array(n_elements=64, nx=48, ny=48, nz=72)


def _peak(ctx, prob, offset):
    g = prob.grid
    th, ph = prob.meta["elements"]
    q = prob.copy()
    phases = presets.steering_phases(th, ph, prob.source.focal_length, offset, prob.source.freq[0], 1500.0)
    q.set_elements(prob.array("element_of_cell"), phases, prob.array("element_amp"))
    return ctx.westervelt(q, want=("peak",))["peak"]


def test_steering_moves_the_focus(ctx):
    """The unsteered pressure maximum sits short of the geometric focus (a
    small box has a low Fresnel number); steering to lateral offsets in the
    plane of that maximum moves it there."""
    prob = _small()
    g = prob.grid
    izf = prob.source.plane_iz + int(round(prob.source.focal_length / g.dz))
    pk = _peak(ctx, prob, (0.0, 0.0, 0.0))
    first = prob.source.plane_iz + 5
    izm = first + int(np.argmax(pk[first:].max(axis=(1, 2))))
    y0, x0 = np.unravel_index(int(np.argmax(pk[izm])), pk[izm].shape)
    for off in ((3, 0), (0, -3), (2, 2)):
        pk = _peak(ctx, prob, (off[0] * g.dx, off[1] * g.dx, (izm - izf) * g.dz))
        y1, x1 = np.unravel_index(int(np.argmax(pk[izm])), pk[izm].shape)
        assert abs((x1 - x0) - off[0]) <= 1 and abs((y1 - y0) - off[1]) <= 1, (off, x1 - x0, y1 - y0)


def test_per_spot_resolve_continues_heat_like_the_oracle(ctx, oracle):
    prob = _small()
    res = pipeline.steered_spots_run(ctx, prob, n_spots=2, steps_per_spot=120, keep_q=True)
    th = presets.cfg3_thermal(prob, n_spots=1, steps_per_spot=120)
    T, TD = th.initial_fields()
    T0 = T.copy()
    for Q in res["Q"]:
        z = np.zeros(120, np.int32)
        T, TD, _ = oracle.heat(th.thermal, Q, z, z, T, TD)
    rise = np.abs(T - T0).max()
    assert rise > 1e-3
    assert np.abs(res["T"] - T).max() <= 1e-5 * rise
    rtol = max(1e-5, 2.0 * np.log(4.0) * 1e-5 * rise)
    np.testing.assert_allclose(res["dose"], TD, rtol=rtol, atol=1e-300)
