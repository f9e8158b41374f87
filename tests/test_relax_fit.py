"""Relaxation fit (no GPU): the dispersion relation of the solver's medium
model and the two-process fit of 0.5 dB/cm/MHz used by cfg3."""
import math

import numpy as np

from bubbledynamics_gb300 import presets
from bubbledynamics_gb300 import relax_fit as rf


def test_single_process_and_thermoviscous_limits():
    f = np.geomspace(0.2e6, 8e6, 9)
    w = 2 * math.pi * f
    c, delta = 1540.0, 4e-6
    a, cp = rf.attenuation(f, c, delta, [])
    # water definition of W:371-372: alpha = delta w^2 / (2 c^3) (small-loss limit)
    np.testing.assert_allclose(a, delta * w ** 2 / (2 * c ** 3), rtol=1e-4)
    cv, tv = 5.0, 1e-7
    a1, cp1 = rf.attenuation(f, c, 0.0, [(cv, tv)])
    np.testing.assert_allclose(a1, (cv / c ** 2) * w ** 2 * tv / (1 + (w * tv) ** 2), rtol=1e-2)
    assert np.all(np.diff(cp1) > 0)                  # relaxation: phase speed rises with frequency


def test_liver_fit_follows_the_power_law():
    a0 = rf.db_cm_mhz_to_np_m_mhz(0.5)
    assert abs(a0 - 5.7565) < 1e-3
    delta = presets.water_delta(1.2e6, 1590.0)
    relax, err = rf.fit_relaxation(a0, 1.0, 1590.0, delta)
    assert len(relax) == 2 and err < 0.07
    assert all(cv > 0 and tv > 0 for cv, tv in relax)
    f = np.array([1.2e6, 2.4e6, 3.6e6])              # fundamental and harmonics of cfg3
    a, _ = rf.attenuation(f, 1590.0, delta, relax)
    np.testing.assert_allclose(a, a0 * f / 1e6, rtol=0.05)


def test_reference_muscle_values_are_a_near_linear_law():
    """W:389-393's hard-coded fit under this model: close to linear in f above
    1 MHz (the reference's nominal tissue absorption is 7.2 f_MHz Np/m)."""
    k = presets.ref_W_constants()
    f = np.array([1e6, 2e6, 3e6, 5e6])
    a, _ = rf.attenuation(f, k["c_tissue"], k["delta_tissue"], [(k["c1"], k["tau1"]), (k["c2"], k["tau2"])])
    slope = a / (f / 1e6)
    assert slope.max() / slope.min() < 1.15
    assert 7.0 < slope.mean() < 10.0
