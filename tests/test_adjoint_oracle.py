"""The FP64 CPU adjoint of the oracle against central finite differences of
the oracle's own forward solve (no GPU).  The adjoint has no reference
counterpart; its forward model is W:139-236 with the source of W:62-85.

Tolerance: central differences with h = 1e-4 rad (phase) / 1e-4 (amplitude)
in FP64 have a truncation error near 1e-9 of the gradient; the check is
|adjoint - FD| <= 1e-6 * max|gradient|."""
import numpy as np
import pytest

from bubbledynamics_gb300 import abi, presets
from bubbledynamics_gb300.adjoint import loss_weights, with_elements


def _fd_loss(oracle, prob, loss):
    q = prob.copy()
    q.params.energy_mode = abi.BD_ENERGY_P2
    q.params.energy_start, q.params.energy_end = loss.window_start, loss.window_end
    E = oracle.westervelt(q, want=("energy",))["energy"]
    return float(np.sum(loss_weights(q.shape, loss) * E))


def _fd(oracle, prob, loss, which, elems, h=1e-4):
    ph = prob.array("element_phase").copy()
    am = prob.array("element_amp").copy()
    out = []
    for e in elems:
        vals = []
        for s in (1.0, -1.0):
            p2, a2 = ph.copy(), am.copy()
            (p2 if which == "phase" else a2)[e] += s * h
            vals.append(_fd_loss(oracle, with_elements(prob, p2, a2), loss))
        out.append((vals[0] - vals[1]) / (2 * h))
    return np.array(out)


def test_oracle_loss_matches_weights_times_energy(oracle):
    prob, loss = presets.adjoint_mini()
    L, _, _ = oracle.westervelt_adjoint(prob, loss)
    assert L == pytest.approx(_fd_loss(oracle, prob, loss), rel=1e-12)


@pytest.mark.slow
def test_oracle_adjoint_phase_gradient_vs_central_fd_16_elements(oracle):
    prob, loss = presets.adjoint_mini()
    _, gp, _ = oracle.westervelt_adjoint(prob, loss)
    fd = _fd(oracle, prob, loss, "phase", range(16))
    assert np.abs(gp).max() > 0
    assert np.abs(fd - gp).max() <= 1e-6 * np.abs(gp).max()


def test_oracle_adjoint_amplitude_gradient_vs_central_fd(oracle):
    prob, loss = presets.adjoint_mini()
    _, _, ga = oracle.westervelt_adjoint(prob, loss)
    elems = [0, 7, 15]
    fd = _fd(oracle, prob, loss, "amp", elems)
    assert np.abs(fd - ga[elems]).max() <= 1e-6 * np.abs(ga).max()


def test_oracle_adjoint_reference_relaxation_scheme(oracle):
    prob, loss = presets.adjoint_mini(n_steps=120)
    prob.params.relax_scheme = abi.BD_RELAX_REFERENCE
    _, gp, _ = oracle.westervelt_adjoint(prob, loss)
    elems = [1, 9]
    fd = _fd(oracle, prob, loss, "phase", elems)
    assert np.abs(fd - gp[elems]).max() <= 1e-6 * np.abs(gp).max()


def test_oracle_adjoint_rejects_closed_faces(oracle):
    prob, loss = presets.adjoint_mini()
    prob.grid.face[4] = abi.BD_FACE_MUR
    with pytest.raises(RuntimeError):
        oracle.westervelt_adjoint(prob, loss)
