"""z-slab decomposition of the Westervelt solve on one GPU: K slabs, each with
its own buffers and 3 ghost planes per internal face refreshed after every
step, give the single-domain fields bit for bit (the virtual sub-domain test of
a multi-GPU split).  Covers the benchmark physics (sponge, c map, burst source,
paired and one-cell TMA kernels and the plain kernel) and the reference physics
(mirror planes, Mur faces, two materials by plane, the harmonic DFT and Q),
both through the library's own exchange and through the pack / unpack halo
copies a multi-rank run sends between devices."""
import numpy as np
import pytest

from bubbledynamics_gb300 import abi, api, halo, presets

pytestmark = pytest.mark.gpu


def _equal(a, b, keys):
    for k in keys:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


@pytest.mark.parametrize("variant", [21, 17, 0])
@pytest.mark.parametrize("n_slabs", [2, 3])
def test_slabs_equal_single_domain_cfg1_box(ctx, variant, n_slabs):
    p = presets.cfg1(40, 40, 72, 200, precision=abi.BD_F32)
    p.params.tile_variant = variant
    one = ctx.westervelt(p, want=("p_final", "peak", "energy"))
    many = ctx.westervelt_slabs(p, n_slabs, want=("p_final", "peak", "energy"))
    assert np.abs(one["p_final"]).max() > 0
    _equal(one, many, ("p_final", "peak", "energy"))


@pytest.mark.parametrize("precision", [abi.BD_F64, abi.BD_F32])
def test_slabs_equal_single_domain_reference_physics(ctx, precision):
    p = presets.ref_W_mini(precision, Nxy=24, Nz=40, loop1_periods=1, periods=1)
    one = ctx.westervelt(p)
    many = ctx.westervelt_slabs(p, 2)
    assert np.abs(one["Q"]).max() > 0
    _equal(one, many, ("p_final", "peak", "energy", "Q", "dft_re", "dft_im"))


def test_slab_sessions_through_halo_buffers(ctx):
    """The data path of a multi-rank run (pack the owned boundary planes into a
    device buffer, hand it over, unpack into the neighbour's ghost planes) for
    three slab sessions in this process."""
    pytest.importorskip("torch")
    p = presets.cfg1(40, 40, 72, 120, precision=abi.BD_F32)
    one = ctx.westervelt(p, want=("p_final", "peak", "energy"))
    got = halo.run_slabs_local(ctx, p, 3, want=("p_final", "peak", "energy"))
    _equal(one, got, ("p_final", "peak", "energy"))


def test_slab_arguments_checked(ctx):
    p = presets.ref_W_mini(abi.BD_F32, Nxy=24, Nz=40, loop1_periods=1, periods=1)
    with pytest.raises(api.BDError):
        ctx.westervelt_slab(p, 0, 5)          # fewer than 8 owned planes
    with pytest.raises(api.BDError):
        ctx.westervelt_slab(p, 4, 20)         # the ghost planes would reach the z- Mur layers
    with pytest.raises(api.BDError):
        ctx.westervelt_slabs(p, 6)            # more slabs than nz / 8
    torch = pytest.importorskip("torch")
    s = ctx.westervelt_slab(p, 0, 20)
    buf = torch.empty(s.halo_bytes(), dtype=torch.uint8, device="cuda")
    with pytest.raises(api.BDError) as ei:
        s.halo_copy(0, 0, buf.data_ptr())     # side 0 of the first slab is the grid's face
    assert ei.value.status == abi.BD_ERR_INVALID_ARG and "face of the grid" in str(ei.value)
    s.halo_copy(1, 0, buf.data_ptr())         # side 1 is an internal face
    s.close()


def test_slab_boundary_inside_the_dft_planes(ctx):
    """cfg5 physics on a 64x64x96 box (two relaxation processes, three tones,
    the 9-frequency DFT on planes 74..95) in five slabs, the last boundary at
    plane 76 inside the DFT planes: every slab keeps its own part of the DFT
    and the assembled maps equal the one-domain solve bit for bit."""
    p = presets.cfg5(nx=64, ny=64, nz=96, n_steps=150, window_steps=60)
    p.params.tile_variant = 21
    assert p.params.dft_z_lo < 76 < p.params.dft_z_hi
    one = ctx.westervelt(p, want=("p_final", "peak", "energy", "dft"))
    many = ctx.westervelt_slabs(p, 5, want=("p_final", "peak", "energy", "dft"))
    assert np.abs(one["dft_re"]).max() > 0
    _equal(one, many, ("p_final", "peak", "energy", "dft_re", "dft_im"))
