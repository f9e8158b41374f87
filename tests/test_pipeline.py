"""Host-side glue (no GPU): tone reconstruction from DFT accumulators and the
energy -> heat-source conversion."""
import numpy as np

from bubbledynamics_gb300 import pipeline, presets


def test_bubbles_from_dft_recovers_tones():
    prob = presets.cfg5(nx=48, ny=48, nz=72)
    p = prob.params
    g = prob.grid
    nd, n = p.n_dft, p.dft_len
    nzd = p.dft_z_hi - p.dft_z_lo
    plane = g.nx * g.ny
    rng = np.random.default_rng(0)
    A = rng.uniform(1e5, 1e6, nd)
    psi = rng.uniform(0, 2 * np.pi, nd)
    # the accumulators of p(s) = sum_j A_j sin(2 pi f_j (s - dft_start) dt + psi_j) over the window
    s = np.arange(n)
    re = np.zeros((nd, nzd * plane))
    im = np.zeros((nd, nzd * plane))
    sig = sum(A[j] * np.sin(2 * np.pi * p.dft_freq[j] * s * g.dt + psi[j]) for j in range(nd))
    for j in range(nd):
        th = 2 * np.pi * p.dft_freq[j] * s * g.dt
        re[j, :] = np.sum(sig * np.cos(th))
        im[j, :] = -np.sum(sig * np.sin(th))
    b, cells = pipeline.bubbles_from_dft(prob, re, im, 5)
    for j in range(nd):
        np.testing.assert_allclose(b["a"][:, j], A[j], rtol=1e-6)
        d = np.angle(np.exp(1j * (b["phi"][:, j] - psi[j])))
        assert np.abs(d).max() < 1e-6


def test_heat_source_from_energy_is_2_alpha_intensity():
    prob = presets.cfg3_acoustic(nx=48, ny=48, nz=72)
    E = np.full(prob.shape, 2.0)
    Q = pipeline.heat_source_from_energy(prob, E, 0.5)
    liver = prob.medium.mat[1]
    iz = prob.shape[0] - 1                      # a liver plane
    np.testing.assert_allclose(Q[iz], 2 * liver.absorption * (2.0 / 0.5) / (liver.rho * liver.c0))
