"""The C++ command-line drivers (bubbledynamics_gb300/cli): the programs that
stand in for the reference's three main() functions and write its files
through libbubbledyn.  On the CPU: they build and answer --help.  On the GPU:
their output files equal, byte for byte, the files the Python path writes
for the same problem through the same library."""
import os
import subprocess

import numpy as np
import pytest

from bubbledynamics_gb300 import abi, api, build, presets

W_BIN = "Q3D_E100_space6_att9_abs7_2_c1600_relax_fft_v3.bin"
W_DAT = "Q_Z_E100_space6_att9_abs7_2_c1600_relax_fft_v3.dat"


def _run(name, *args, cwd=None):
    exe = build.cli_path(name)
    r = subprocess.run([exe] + [str(a) for a in args], capture_output=True, text=True, cwd=cwd, timeout=600)
    assert r.returncode == 0, (name, r.stdout, r.stderr)
    return r.stdout


@pytest.fixture(scope="module")
def drivers(lib):
    return build.build_cli()


def test_drivers_build_and_answer_help(drivers):
    assert len(drivers) == 3
    for name in ("bd_westervelt", "bd_spiral", "bd_gilmore"):
        out = _run(name, "--help")
        assert name in out


def test_driver_rejects_unknown_arguments(drivers):
    r = subprocess.run([build.cli_path("bd_gilmore"), "positional"], capture_output=True, text=True)
    assert r.returncode == 2


def _same_bytes(a, b):
    with open(a, "rb") as fa, open(b, "rb") as fb:
        return fa.read() == fb.read()


@pytest.mark.gpu
def test_westervelt_driver_files_equal_python_path(ctx, drivers, tmp_path):
    d = tmp_path / "cli"
    d.mkdir()
    _run("bd_westervelt", "--mini", "--nxy", 24, "--nz", 40, "--loop1-periods", 1, "--periods", 1,
         "--precision", "f32", "--out-dir", d)
    prob = presets.ref_W_mini(abi.BD_F32, Nxy=24, Nz=40, loop1_periods=1, periods=1)
    Q = ctx.westervelt(prob, want=("Q",))["Q"]
    k = prob.meta["constants"]
    api.write_q_bin(tmp_path / W_BIN, Q, iz_first=2)
    api.write_q_axis_dat(tmp_path / W_DAT, Q, k["z_min"], k["dz"], iz_first=2)
    assert np.abs(Q).max() > 0
    assert _same_bytes(d / W_BIN, tmp_path / W_BIN)
    assert _same_bytes(d / W_DAT, tmp_path / W_DAT)


@pytest.mark.gpu
def test_spiral_driver_reads_the_westervelt_file(ctx, drivers, tmp_path):
    """W's output volume feeds T like in the reference workflow: the spiral
    driver mirrors the quarter domain, heats along the spiral and writes T's
    dose slice; the Python path does the same through the library."""
    _run("bd_westervelt", "--mini", "--nxy", 24, "--nz", 40, "--loop1-periods", 1, "--periods", 1,
         "--out-dir", tmp_path)
    _run("bd_spiral", "--mini", "--nxy-half", 23, "--nz", 38, "--legs", 2, "--out-dir", tmp_path)
    small = api.read_q_bin(tmp_path / W_BIN, 23, 38)
    Q = api.unfold_quarter(small, 23, 38)
    prob = presets.make_ref_T(presets.ref_T_mini_constants(Nxy=47, Nz=38, legs=2))
    r = ctx.heat(prob.thermal, Q, prob.traj)
    ref = tmp_path / "td_python.dat"
    api.write_slice_dat(ref, r["dose"], abi.BD_SLICE_XZ, 23, (0, 38), (0, 47),
                        header="Z=rows;X=columns;speed=;1600;c_t=;3700;K_t=;0.51")
    assert _same_bytes(tmp_path / "TD_XZ_E100_2mms_3mm_att9_abs7_2_c1600_relax_v2.dat", ref)
    assert (tmp_path / "T_XZ_E100_2mms_3mm_att9_abs7_2_c1600_relax_v2_loop0.dat").exists()


@pytest.mark.gpu
def test_gilmore_driver_table_equals_python_path(ctx, drivers, tmp_path):
    out = tmp_path / "table.dat"
    _run("bd_gilmore", "--combo-first", 27670, "--combo-count", 2, "--r0-first", 19, "--r0-count", 2,
         "--max-steps", 300, "--out", out)
    combos = api.gilmore_combos()[27670:27672]
    R0 = presets.ref_G_R0s()[19:21]
    A, ms = ctx.gilmore_threshold(presets.ref_G_medium(), combos, R0, ref_arith=1, max_steps=300)
    ref = tmp_path / "table_python.dat"
    api.write_threshold_table(ref, combos, R0, A, ms * 1e-3)
    got = open(out).read().splitlines()
    exp = open(ref).read().splitlines()
    assert got[:-1] == exp[:-1]          # the last row holds the run time
    assert got[-1].startswith("time (s);")
