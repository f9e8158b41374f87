"""Relaxation-process fit: absorption power law -> (c_nu, tau_nu).

The reference hard-codes the result of such a fit (W:389-393, muscle) and has
no fitting code.  The medium model is the one the solver integrates
(W:203-234): with the thermoviscous term (delta / c^2) p_ttt and memory
variables tau_nu R_nu' + R_nu = (2 c_nu tau_nu / c^3) p_ttt entering as
c^2 sum_nu R_nu, a plane wave exp(i(w t - k x)) has

    c^2 k^2 = w^2 [1 - i w delta / c^2 - i w sum_nu (2 c_nu tau_nu / c) / (1 + i w tau_nu)]

so process nu alone absorbs (c_nu / c^2) w^2 tau_nu / (1 + w^2 tau_nu^2) and
the thermoviscous term w^2 delta / (2 c^3) (the water definition of W:371-372).
`fit_relaxation` chooses c_nu, tau_nu so that the exact attenuation -Im k
follows alpha0 * f_MHz^y over a band, in the least-squares sense of the
relative error at log-spaced frequencies.
"""
import math

import numpy as np


def attenuation(f, c, delta, relax):
    """-Im k [Np/m] and the phase speed w / Re k [m/s] at frequencies f [Hz]
    for relaxation processes relax = [(c_nu, tau_nu), ...]."""
    w = 2.0 * np.pi * np.asarray(f, dtype=np.float64)
    s = 1.0 - 1j * w * delta / c ** 2
    for cv, tv in relax:
        s = s - 1j * w * (2.0 * cv * tv / c) / (1.0 + 1j * w * tv)
    k = (w / c) * np.sqrt(s)
    return -k.imag, w / k.real


def fit_relaxation(alpha0, y, c, delta=0.0, n_proc=2, f_band=(0.3e6, 6.0e6), n_freq=40):
    """Fit n_proc relaxation processes to alpha(f) = alpha0 [Np/m/MHz^y] * f_MHz^y
    over f_band.  Returns (relax, max relative error over the band)."""
    from scipy.optimize import least_squares
    f = np.geomspace(f_band[0], f_band[1], n_freq)
    target = alpha0 * (f / 1e6) ** y

    def resid(x):
        relax = [(math.exp(x[2 * i]), math.exp(x[2 * i + 1])) for i in range(n_proc)]
        a, _ = attenuation(f, c, delta, relax)
        return a / target - 1.0

    # relaxation times spread over the band, strengths from the single-process peak
    taus = np.geomspace(1.0 / (2 * np.pi * f_band[1]), 1.0 / (2 * np.pi * f_band[0]), n_proc)
    x0 = []
    for t in taus:
        w0 = 1.0 / t
        cv = 2.0 * alpha0 * (w0 / 2.0 / np.pi / 1e6) ** y * c * c / w0 / n_proc
        x0 += [math.log(max(cv, 1e-6)), math.log(t)]
    sol = least_squares(resid, np.array(x0), method="lm", xtol=1e-14, ftol=1e-14, max_nfev=20000)
    relax = [(math.exp(sol.x[2 * i]), math.exp(sol.x[2 * i + 1])) for i in range(n_proc)]
    relax.sort(key=lambda p: p[1])
    return relax, float(np.max(np.abs(resid(sol.x))))


def db_cm_mhz_to_np_m_mhz(a_db):
    """dB/cm/MHz -> Np/m/MHz."""
    return a_db * 100.0 / (20.0 / math.log(10.0))
