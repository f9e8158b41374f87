"""cfg5 on a reduced box: the 9-frequency on-the-fly DFT of a three-tone
nonlinear field against the FP64 oracle, and bubbles driven by the
DFT-reconstructed local pressure against the oracle's integrator.
Tolerances: FP32 DFT maps 1e-5 relative L2 (the field tolerance); Gilmore
fast path vs the oracle 1e-6 relative on R (as in test_gpu_gilmore)."""
import numpy as np
import pytest

from bubbledynamics_gb300 import abi, pipeline, presets

pytestmark = pytest.mark.gpu


def _small(prec=abi.BD_F32):
    return presets.cfg5(nx=48, ny=48, nz=72, precision=prec)


def test_cfg5_dft_matches_oracle(ctx, oracle):
    r = ctx.westervelt(_small(), want=("dft", "peak"))
    e = oracle.westervelt(_small(abi.BD_F64), want=("dft", "peak"))
    X = r["dft_re"].astype(np.float64) + 1j * r["dft_im"].astype(np.float64)
    Xe = e["dft_re"] + 1j * e["dft_im"]
    rel = np.linalg.norm(X - Xe) / np.linalg.norm(Xe)
    assert rel <= 1e-5, rel
    # every one of the nine bins carries signal (fundamentals and harmonics)
    per = np.abs(Xe.reshape(9, -1)).max(axis=1)
    assert np.all(per > 0)
    relp = np.linalg.norm(r["peak"] - e["peak"]) / np.linalg.norm(e["peak"])
    assert relp <= 1e-5, relp


def test_cfg5_bubbles_driven_by_local_field(ctx, oracle):
    prob = _small()
    r = ctx.westervelt(prob, want=("dft",))
    b, cells = pipeline.bubbles_from_dft(prob, r["dft_re"], r["dft_im"], 48, radius=0.3e-3, length=0.6e-3)
    assert np.all(b["n_tones"] == 9) and np.all(b["a"][:, :3].max(axis=1) > 0)
    med = presets.cfg2_medium()
    ode = presets.cfg2_ode(t_end=0.05e-6)
    res, _ = ctx.gilmore(med, b, ode)
    ro = oracle.gilmore(med, (abi.Bubble * len(b)).from_buffer_copy(b.tobytes()), ode)
    assert np.all(res["status"] == abi.BD_BUBBLE_DONE)
    np.testing.assert_allclose(res["R"], [x.R for x in ro], rtol=1e-6)


def test_cfg5_dft_same_bits_in_every_tile_variant(ctx):
    """The DFT accumulators through the one-cell kernel and the two-cell
    kernels (pair read-modify-writes of the accumulator planes), with two
    relaxation processes and three tones: the same bits."""
    res = {}
    for v in (17, 21, 23):
        p = _small()
        p.params.tile_variant = v
        res[v] = ctx.westervelt(p, want=("p_final", "peak", "energy", "dft"))
        assert res[v]["tile_variant"] == v
    assert np.abs(res[17]["dft_re"]).max() > 0
    for v in (21, 23):
        for k in ("p_final", "peak", "energy", "dft_re", "dft_im"):
            np.testing.assert_array_equal(res[v][k], res[17][k], err_msg="variant %d, %s" % (v, k))
