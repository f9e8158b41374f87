"""The device adjoint (bd_westervelt_adjoint) through the C ABI: against the
FP64 CPU adjoint of the oracle, against central finite differences of the
device forward solve on 16 elements, across checkpoint intervals, in FP32,
and through the torch autograd wrapper.

Tolerances (relative to max |gradient|): FP64 device vs FP64 oracle 1e-9
(same arithmetic, different summation order); FP64 central differences
(h = 1e-4) 1e-6; FP32 device vs FP64 oracle 1e-3 (single-precision forward
levels and adjoint accumulation over 200 steps)."""
import numpy as np
import pytest

from bubbledynamics_gb300 import abi, api, presets
from bubbledynamics_gb300.adjoint import forward_loss, with_elements

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max()


def test_adjoint_f64_matches_oracle_adjoint(ctx, oracle):
    prob, loss = presets.adjoint_mini(precision=abi.BD_F64)
    Lo, gpo, gao = oracle.westervelt_adjoint(prob, loss)
    L, gp, ga, tm = ctx.westervelt_adjoint(prob, loss)
    assert L == pytest.approx(Lo, rel=1e-11)
    assert _rel(gp, gpo) <= 1e-9
    assert _rel(ga, gao) <= 1e-9
    assert tm["forward_ms"] > 0 and tm["backward_ms"] > 0


def test_adjoint_f64_reference_relaxation_scheme_matches_oracle(ctx, oracle):
    prob, loss = presets.adjoint_mini(precision=abi.BD_F64, n_steps=120)
    prob.params.relax_scheme = abi.BD_RELAX_REFERENCE
    Lo, gpo, gao = oracle.westervelt_adjoint(prob, loss)
    L, gp, ga, _ = ctx.westervelt_adjoint(prob, loss)
    assert L == pytest.approx(Lo, rel=1e-11)
    assert _rel(gp, gpo) <= 1e-9
    assert _rel(ga, gao) <= 1e-9


def test_adjoint_f64_vs_central_fd_16_elements(ctx):
    prob, loss = presets.adjoint_mini(precision=abi.BD_F64)
    L, gp, ga, _ = ctx.westervelt_adjoint(prob, loss)
    assert forward_loss(ctx, prob, loss) == pytest.approx(L, rel=1e-12)
    ph = prob.array("element_phase")
    am = prob.array("element_amp")
    h = 1e-4
    fd = np.zeros(16)
    for e in range(16):
        v = []
        for s in (1.0, -1.0):
            p2 = ph.copy()
            p2[e] += s * h
            v.append(forward_loss(ctx, with_elements(prob, p2, am), loss))
        fd[e] = (v[0] - v[1]) / (2 * h)
    assert _rel(gp, fd) <= 1e-6


@pytest.mark.parametrize("prec", [abi.BD_F64, abi.BD_F32])
def test_adjoint_gradient_independent_of_checkpoint_interval(ctx, prec):
    prob, loss = presets.adjoint_mini(precision=prec)
    ref = None
    for k in (0, 1, 7, prob.params.n_steps, -1):
        loss.checkpoint_every = k
        L, gp, ga, _ = ctx.westervelt_adjoint(prob, loss)
        if ref is None:
            ref = (L, gp, ga)
        else:
            assert L == ref[0]
            np.testing.assert_array_equal(gp, ref[1])
            np.testing.assert_array_equal(ga, ref[2])


@pytest.mark.parametrize("prec", [abi.BD_F64, abi.BD_F32])
def test_adjoint_slabs_equal_single_domain(ctx, prec):
    """The z-slab split of the gradient: 2, 3 and 4 slabs (each its own fields,
    checkpoints and adjoint rings; ghost planes of p^n after every forward and
    recompute step, of H after every backward step) give the one-domain loss
    and gradients bit for bit, with sqrt(N) checkpoints and with an interval of
    7.  FP32 runs the fused backward pass, FP64 the pointwise and stencil
    passes with the exchange between them."""
    for k in (0, 7):
        prob, loss = presets.adjoint_mini(precision=prec)
        loss.checkpoint_every = k
        ref = ctx.westervelt_adjoint(prob, loss)
        assert np.abs(ref[1]).max() > 0
        for n_slabs in (2, 3, 4):
            prob, loss = presets.adjoint_mini(precision=prec)
            loss.checkpoint_every = k
            got = ctx.westervelt_adjoint(prob, loss, n_slabs=n_slabs)
            assert got[0] == ref[0], (k, n_slabs)
            np.testing.assert_array_equal(got[1], ref[1], err_msg="phase, K = %d, %d slabs" % (k, n_slabs))
            np.testing.assert_array_equal(got[2], ref[2], err_msg="amplitude, K = %d, %d slabs" % (k, n_slabs))
    prob, loss = presets.adjoint_mini(precision=prec)
    with pytest.raises(api.BDError):
        ctx.westervelt_adjoint(prob, loss, n_slabs=5)        # fewer than 8 planes per slab


@pytest.mark.parametrize("prec", [abi.BD_F64, abi.BD_F32])
def test_adjoint_graphs_and_plain_launches_identical(ctx, prec):
    """The recompute and backward sweeps replayed as captured CUDA graphs (one
    per segment parity and adjoint-ring rotation) give the bits of plain
    launches, for segment lengths that are odd, even and longer than 6."""
    for k in (7, 8, 15, 0):
        res = []
        for chunk in (0, -1):
            prob, loss = presets.adjoint_mini(precision=prec)
            prob.params.graph_chunk = chunk
            loss.checkpoint_every = k
            res.append(ctx.westervelt_adjoint(prob, loss))
        assert res[0][0] == res[1][0], k
        np.testing.assert_array_equal(res[0][1], res[1][1], err_msg="phase, K = %d" % k)
        np.testing.assert_array_equal(res[0][2], res[1][2], err_msg="amplitude, K = %d" % k)


def test_adjoint_f32_close_to_f64_oracle(ctx, oracle):
    p64, loss = presets.adjoint_mini(precision=abi.BD_F64)
    _, gpo, gao = oracle.westervelt_adjoint(p64, loss)
    p32, loss = presets.adjoint_mini(precision=abi.BD_F32)
    _, gp, ga, _ = ctx.westervelt_adjoint(p32, loss)
    assert _rel(gp, gpo) <= 1e-3
    assert _rel(ga, gao) <= 1e-3


def test_adjoint_rejects_closed_faces_and_bowls(ctx):
    prob, loss = presets.adjoint_mini(precision=abi.BD_F64)
    q = prob.copy()
    q.grid.face[5] = abi.BD_FACE_MUR
    q.grid.mur_layers = 2
    with pytest.raises(api.BDError) as e:
        ctx.westervelt_adjoint(q, loss)
    assert e.value.status == abi.BD_ERR_UNSUPPORTED
    bad = abi.FocalLoss()
    bad.window_start, bad.window_end = 10, prob.params.n_steps + 1
    with pytest.raises(api.BDError):
        ctx.westervelt_adjoint(prob, bad)


def test_autograd_function(ctx):
    torch = pytest.importorskip("torch")
    from bubbledynamics_gb300.adjoint import AdjointWestervelt
    prob, loss = presets.adjoint_mini(precision=abi.BD_F64)
    L, gp, ga, _ = ctx.westervelt_adjoint(prob, loss)
    phases = torch.tensor(prob.array("element_phase"), dtype=torch.float64, requires_grad=True)
    amps = torch.tensor(prob.array("element_amp"), dtype=torch.float64, requires_grad=True)
    out = AdjointWestervelt.apply(phases, amps, prob, loss, ctx)
    (2.0 * out).backward()
    assert out.item() == pytest.approx(L, rel=1e-12)
    np.testing.assert_allclose(phases.grad.numpy(), 2.0 * gp, rtol=1e-12)
    np.testing.assert_allclose(amps.grad.numpy(), 2.0 * ga, rtol=1e-12)
    with torch.no_grad():
        out2 = AdjointWestervelt.apply(phases, amps, prob, loss, ctx)
    assert out2.item() == pytest.approx(L, rel=1e-12)


@pytest.mark.slow
def test_cfg4_fp32_gradient_vs_fp64_central_fd_on_16_elements(ctx):
    """The cfg4 geometry at full size (192^3, 256-element cap array, water /
    fat / liver), shortened to 1000 steps: the FP32 adjoint gradient of 16
    element phases against central differences of the FP64 forward solve
    (h = 1e-3 rad).  Tolerance 1e-2 of the largest of the 16 gradients: FP32
    forward levels and adjoint accumulation over 1000 steps."""
    p32, loss = presets.cfg4(n_steps=1000)
    _, gp, _, _ = ctx.westervelt_adjoint(p32, loss)
    p64, _ = presets.cfg4(n_steps=1000, precision=abi.BD_F64)
    ph = p64.array("element_phase")
    am = p64.array("element_amp")
    elems = np.argsort(-np.abs(gp))[:16]
    h = 1e-3
    fd = np.zeros(16)
    for k, e in enumerate(elems):
        v = []
        for s in (1.0, -1.0):
            p2 = ph.copy()
            p2[e] += s * h
            v.append(forward_loss(ctx, with_elements(p64, p2, am), loss))
        fd[k] = (v[0] - v[1]) / (2 * h)
    assert np.abs(fd).max() > 0
    assert np.abs(gp[elems] - fd).max() <= 1e-2 * np.abs(fd).max()
