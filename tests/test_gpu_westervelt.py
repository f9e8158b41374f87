"""Westervelt solver on the GPU (through the C ABI) against the CPU oracle and
against fixtures of the reference's own code.

Tolerances: FP64 fields agree with the FP64 oracle to 1e-9 relative L2 (the
GPU contracts a*b+c into FMAs and uses its own sin); FP32 fields are held to
the 1e-5 relative L2 field accuracy of the FP32 design (peak and energy
maps), measured against the FP64 oracle."""
import numpy as np
import pytest

from bubbledynamics_gb300 import abi, api, presets
from tests.conftest import golden_path

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def ref_mini_oracle(oracle):
    prob = presets.ref_W_mini(abi.BD_F64)
    return prob, oracle.westervelt(prob)


def test_ref_mini_f64_matches_oracle(ctx, ref_mini_oracle):
    prob, exp = ref_mini_oracle
    got = ctx.westervelt(prob)
    assert got["steps_done"] == prob.params.n_steps
    assert rel_l2(got["p_final"], exp["p_final"]) < 1e-9
    assert rel_l2(got["peak"], exp["peak"]) < 1e-9
    assert rel_l2(got["Q"], exp["Q"]) < 1e-9


def test_ref_mini_f64_matches_reference_fixture(ctx):
    """The full W program on a small box: pressure snapshot after the first
    loop and the acoustic power Q of the reference's own kernels."""
    g = np.load(golden_path("W_mini.npz"))
    prob = presets.ref_W_mini(abi.BD_F64)
    p1 = prob.copy()
    p1.params.n_steps = prob.meta["n_loop1"]
    P = ctx.westervelt(p1, want=("p_final",))["p_final"]
    assert rel_l2(P[g["planes"]], g["P"]) < 1e-9
    Q = ctx.westervelt(prob, want=("Q",))["Q"]
    assert rel_l2(Q[g["planes"]], g["Q"]) < 2e-6      # the reference transforms in FP32 (cuFFT C2C)


def test_ref_mini_f32_close_to_oracle(ctx, ref_mini_oracle):
    """FP32 on the reference physics (two layers, two relaxation processes,
    Mur faces, the harmonic DFT): the final field and Q within the 1e-5 field
    tolerance of the FP32 design (measured 2.0e-6 and 7.2e-7)."""
    prob, exp = ref_mini_oracle
    p32 = presets.ref_W_mini(abi.BD_F32)
    got = ctx.westervelt(p32)
    e_p = rel_l2(got["p_final"], exp["p_final"])
    e_q = rel_l2(got["Q"], exp["Q"])
    print("ref_mini f32: p_final %.3g  Q %.3g" % (e_p, e_q))
    assert e_p < 1e-5
    assert e_q < 1e-5


@pytest.fixture(scope="module")
def cfg1_small_oracle(oracle):
    prob = presets.cfg1(48, 48, 96, 600, precision=abi.BD_F64)
    return prob, oracle.westervelt(prob)


def test_cfg1_small_f32_field_accuracy(ctx, cfg1_small_oracle):
    """FP32 kernel vs FP64 oracle on the benchmark physics (heterogeneous c,
    relaxation, sponge, burst): output maps and final field within 1e-5
    relative L2."""
    prob64, exp = cfg1_small_oracle
    prob = presets.cfg1(48, 48, 96, 600, precision=abi.BD_F32)
    got = ctx.westervelt(prob)
    e = {k: rel_l2(got[k], exp[k]) for k in ("peak", "energy", "p_final")}
    print("cfg1 small f32 errors:", e)
    for k, v in e.items():
        assert v < 1e-5, (k, v)


def test_cfg1_small_f64_matches_oracle(ctx, cfg1_small_oracle):
    prob64, exp = cfg1_small_oracle
    got = ctx.westervelt(prob64)
    for k in ("p_final", "peak", "energy"):
        assert rel_l2(got[k], exp[k]) < 1e-9, k


def test_graph_and_plain_launches_identical(ctx):
    a = presets.cfg1(40, 40, 64, 230, precision=abi.BD_F32)
    b = presets.cfg1(40, 40, 64, 230, precision=abi.BD_F32)
    a.params.graph_chunk = 20
    b.params.graph_chunk = -1
    ra = ctx.westervelt(a)
    rb = ctx.westervelt(b)
    for k in ("p_final", "peak", "energy"):
        np.testing.assert_array_equal(ra[k], rb[k])


def test_all_tile_variants_identical(ctx):
    """Plain and TMA-pipelined kernels, every tile shape: bitwise-identical fields."""
    base = None
    for v in range(24):
        p = presets.cfg1(40, 40, 72, 60, precision=abi.BD_F32)
        p.params.tile_variant = v
        r = ctx.westervelt(p, want=("p_final", "peak"))
        if base is None:
            base = r
        else:
            np.testing.assert_array_equal(r["p_final"], base["p_final"])
            np.testing.assert_array_equal(r["peak"], base["peak"])


def test_two_cell_variants_on_reference_physics(ctx):
    """The two-x-cells-per-thread variants on the reference's setup (mirror
    planes, Mur faces, source plane, water/tissue planes with two relaxation
    processes, the harmonic DFT): every output equal to the plain kernel's.
    nx = 28 is not a multiple of the 32- or 64-cell tiles, so the last tile column is
    partly outside the grid; FP64 fields are refused by these variants."""
    base = None
    for v in (0, 16, 19, 20, 21, 22, 23):
        p = presets.ref_W_mini(abi.BD_F32, Nxy=28, Nz=40, loop1_periods=1, periods=1)
        p.params.tile_variant = v
        r = ctx.westervelt(p)
        if base is None:
            base = r
            continue
        for k in ("p_final", "peak", "energy", "Q", "dft_re", "dft_im"):
            np.testing.assert_array_equal(r[k], base[k], err_msg="variant %d, %s" % (v, k))
    p64 = presets.ref_W_mini(abi.BD_F64, Nxy=28, Nz=40, loop1_periods=1, periods=1)
    p64.params.tile_variant = 19
    with pytest.raises(api.BDError):
        ctx.westervelt(p64)


def test_two_cell_variants_with_per_cell_materials(ctx):
    """A per-cell material map mixing water (no relaxation) and tissue (two
    processes) cell by cell, so the two cells of a thread often differ in
    material and relaxation count: every tile variant, including the paired
    ones, gives the plain kernel's bits."""
    base = None
    rng = np.random.default_rng(11)
    for v in (0, 16, 17, 19, 20, 21, 22, 23):
        p = presets.ref_W_mini(abi.BD_F32, Nxy=32, Nz=40, loop1_periods=1, periods=1)
        if base is None:
            mm = (rng.random(p.shape) < 0.5).astype(np.uint8)
        p.set_material_map(mm)
        p.params.tile_variant = v
        r = ctx.westervelt(p, want=("p_final", "peak", "energy"))
        assert r["tile_variant"] == v
        if base is None:
            base = r
            assert np.isfinite(base["p_final"]).all() and np.abs(base["p_final"]).max() > 0
            continue
        for k in ("p_final", "peak", "energy"):
            np.testing.assert_array_equal(r[k], base[k], err_msg="variant %d, %s" % (v, k))


@pytest.mark.parametrize("layout", ["no_relaxation", "plane_materials"])
def test_two_cell_variants_material_layouts(ctx, layout):
    """The paired kernel's other compile-time layouts on a cfg1 box: no
    relaxation process at all, and one process with a second material by
    planes (read per plane, no c-map shortcut).  Every variant gives the
    plain kernel's bits."""
    base = None
    for v in (0, 17, 19, 20, 21, 22, 23):
        p = presets.cfg1(40, 40, 72, 60, precision=abi.BD_F32)
        if layout == "no_relaxation":
            p.medium.mat[0].n_relax = 0
        else:
            m = p.medium.mat[0]
            p.medium.n_materials = 2
            p.medium.mat[1] = m
            p.medium.mat[1].c0 = 1560.0
            p.medium.mat[1].relax_c[0] = 8.0
            p.set_plane_material([0 if iz < 36 else 1 for iz in range(72)])
        p.params.tile_variant = v
        r = ctx.westervelt(p, want=("p_final", "peak", "energy"))
        if base is None:
            base = r
            assert np.abs(base["p_final"]).max() > 0
            continue
        for k in ("p_final", "peak", "energy"):
            np.testing.assert_array_equal(r[k], base[k], err_msg="%s, variant %d, %s" % (layout, v, k))


def test_bounded_wait_gives_up_and_context_survives(ctx):
    """The wait that guards every TMA pipeline slot, on a barrier nothing
    completes: it gives up after its limit and records the timeout instead of
    hanging, and the context then runs a solve with the same bits as before."""
    p = presets.ref_W_mini(abi.BD_F32, Nxy=24, Nz=40, loop1_periods=1, periods=1)
    before = ctx.westervelt(p)
    timed_out, ms = ctx.selftest_bounded_wait(100)
    assert timed_out
    assert 90.0 <= ms < 2000.0
    after = ctx.westervelt(p)
    for k in ("p_final", "Q"):
        np.testing.assert_array_equal(after[k], before[k])
    with pytest.raises(api.BDError):
        ctx.selftest_bounded_wait(0)


def test_run_twice_bitwise(ctx):
    p = presets.ref_W_mini(abi.BD_F32, Nxy=24, Nz=40, loop1_periods=1, periods=1)
    a = ctx.westervelt(p)
    b = ctx.westervelt(p)
    for k in ("p_final", "Q", "dft_re"):
        np.testing.assert_array_equal(a[k], b[k])


def test_checkpoint_resume_bitwise(ctx):
    p = presets.ref_W_mini(abi.BD_F32, Nxy=24, Nz=40, loop1_periods=1, periods=1)
    full = ctx.westervelt(p)
    n = p.params.n_steps
    with ctx.westervelt_session(p) as s:
        s.advance(137)
        assert s.step() == 137
        blob = s.checkpoint()
    with ctx.westervelt_session(p) as s2:
        s2.restore(blob)
        assert s2.step() == 137
        s2.advance(n - 137)
        res = s2.finish()
    for k in ("p_final", "peak", "energy", "Q", "dft_re", "dft_im"):
        np.testing.assert_array_equal(res[k], full[k])


def test_fault_injection_then_resume(ctx):
    """A host-side fault at step k stops the solve there; resuming from a
    checkpoint taken at the fault reproduces the uninterrupted result."""
    p = presets.ref_W_mini(abi.BD_F32, Nxy=24, Nz=40, loop1_periods=1, periods=1)
    full = ctx.westervelt(p)
    pf = p.copy()
    pf.params.fault_at_step = 75
    with ctx.westervelt_session(pf) as s:
        with pytest.raises(api.BDError) as ei:
            s.advance(pf.params.n_steps)
        assert ei.value.status == abi.BD_ERR_FAULT_INJECTED
        assert s.step() == 75
        blob = s.checkpoint()
    with ctx.westervelt_session(p) as s2:
        s2.restore(blob)
        s2.advance(p.params.n_steps - 75)
        res = s2.finish()
    np.testing.assert_array_equal(res["p_final"], full["p_final"])
    np.testing.assert_array_equal(res["Q"], full["Q"])


def test_blowup_probe_reports_unstable(ctx):
    p = presets.cfg1(32, 32, 48, 100, precision=abi.BD_F32)
    p.params.check_every = 10
    p.params.blowup_limit = 1.0          # any pressure above 1 Pa counts as a blow-up
    with pytest.raises(api.BDError) as ei:
        ctx.westervelt(p, want=("peak",))
    assert ei.value.status == abi.BD_ERR_UNSTABLE


def test_checkpoint_of_other_geometry_rejected(ctx):
    a = presets.cfg1(32, 32, 48, 20, precision=abi.BD_F32)
    b = presets.cfg1(32, 32, 56, 20, precision=abi.BD_F32)
    with ctx.westervelt_session(a) as s:
        s.advance(10)
        blob = s.checkpoint()
    with ctx.westervelt_session(b) as s2:
        with pytest.raises(api.BDError) as ei:
            s2.restore(blob)
        assert ei.value.status == abi.BD_ERR_STATE


def test_invalid_arguments(ctx):
    p = presets.cfg1(32, 32, 48, 20, precision=abi.BD_F32)
    p.params.precision = 7
    with pytest.raises(api.BDError) as ei:
        ctx.westervelt(p)
    assert ei.value.status == abi.BD_ERR_INVALID_ARG
    q = presets.cfg1(32, 32, 48, 20, precision=abi.BD_F32)
    q.source.plane_iz = 999
    with pytest.raises(api.BDError):
        ctx.westervelt(q)


def test_kernel_launches_counted(ctx):
    before = ctx.kernel_launches()
    p = presets.cfg1(32, 32, 48, 30, precision=abi.BD_F32)
    ctx.westervelt(p, want=("peak",))
    assert ctx.kernel_launches() - before >= 30


def test_autotuned_short_run_matches_explicit_variant(ctx):
    """A run large enough to be tuned (2^21 cells, 300 steps) whose step count
    is below the tuner's total trial steps (10 per variant per round): every
    trial restarts at step 0, so the trials stay inside the per-step source
    tables, and the tuned solve equals the same problem run at the variant
    the tuner chose."""
    a = presets.cfg1(128, 128, 128, 300, precision=abi.BD_F32)
    assert a.ncell >= 1 << 21
    ra = ctx.westervelt(a, want=("p_final", "peak", "energy"))
    b = presets.cfg1(128, 128, 128, 300, precision=abi.BD_F32)
    b.params.tile_variant = int(ra["tile_variant"])
    rb = ctx.westervelt(b, want=("p_final", "peak", "energy"))
    assert np.abs(ra["peak"]).max() > 0
    for k in ("p_final", "peak", "energy"):
        np.testing.assert_array_equal(ra[k], rb[k], err_msg=k)


@pytest.fixture(scope="module")
def cfg1_full_oracle(oracle):
    prob = presets.cfg1(precision=abi.BD_F64)
    return oracle.westervelt(prob, want=("p_final", "peak", "energy"))


def test_cfg1_full_size_f32_accuracy(ctx, cfg1_full_oracle):
    """The benchmark configuration itself (128x128x256 cells, 3000 steps, FP32,
    the autotuned kernel) against the FP64 oracle: peak map, energy map and the
    final pressure field each within 1e-5 relative L2.  The final field is the
    hardest of the three: after 3000 steps the burst has left the box and the
    field is the residue of the sponge, so the error is relative to a field ten
    times weaker than the pulse."""
    got = ctx.westervelt(presets.cfg1(precision=abi.BD_F32), want=("p_final", "peak", "energy"))
    e = {k: rel_l2(got[k], cfg1_full_oracle[k]) for k in ("peak", "energy", "p_final")}
    print("cfg1 full-size f32 errors:", e, "variant", got["tile_variant"])
    for k, v in e.items():
        assert v < 1e-5, (k, v)


@pytest.mark.parametrize("chunk", [20, -1])
def test_partial_windows_take_the_accumulator_free_kernel(ctx, chunk):
    """Peak and energy windows that cover only part of the run: steps outside
    both windows run the paired kernel without accumulators, steps inside the
    peak window only run its peak-only mode (whole captured chunks or single
    steps), and every output equals the one-cell kernel's, which always
    carries the accumulators."""
    res = {}
    for v in (21, 17):
        p = presets.cfg1(40, 40, 64, 230, precision=abi.BD_F32)
        p.params.peak_start, p.params.peak_end = 50, 120
        p.params.energy_start, p.params.energy_end = 100, 185
        p.params.graph_chunk = chunk
        p.params.tile_variant = v
        res[v] = ctx.westervelt(p, want=("p_final", "peak", "energy"))
    assert np.abs(res[21]["energy"]).max() > 0
    for k in ("p_final", "peak", "energy"):
        np.testing.assert_array_equal(res[21][k], res[17][k], err_msg=k)
