"""Readers and writers of the reference programs' files (host code of the C
ABI, no GPU): W's Q3D .bin and on-axis .dat (W:767-790), the quarter-domain
read-back and unfold of T (T:269-306), T's slice .dat files (T:419-448,
T:576-640) and G's threshold table (G:582-613)."""
import numpy as np
import pytest

from bubbledynamics_gb300 import abi, api


def _g(v):
    return "%g" % v


def test_q_bin_round_trip_through_the_quarter_domain_reader(tmp_path):
    rng = np.random.default_rng(1)
    n_half, nz_t = 4, 6
    Q = rng.uniform(0, 1e6, (nz_t + 2, n_half + 1, n_half + 1))     # W's grid: 2 planes below z = 0
    path = tmp_path / "Q3D.bin"
    api.write_q_bin(path, Q)
    assert path.stat().st_size == nz_t * (n_half + 1) ** 2 * 8
    small = api.read_q_bin(path, n_half, nz_t)
    np.testing.assert_array_equal(small, Q[2:])
    full = api.unfold_quarter(small, n_half, nz_t)
    nf = 2 * n_half + 1
    idx = np.abs(np.arange(nf) - n_half)
    np.testing.assert_array_equal(full, small[:, idx][:, :, idx])
    with pytest.raises(api.BDError):
        api.read_q_bin(path, n_half + 1, nz_t)


def test_q_axis_dat(tmp_path):
    Q = np.arange(5 * 3 * 3, dtype=np.float64).reshape(5, 3, 3) * 1.5e3
    path = tmp_path / "Q_Z.dat"
    api.write_q_axis_dat(path, Q, -0.0002, 0.0001)
    lines = path.read_text().split("\n")
    assert lines[0] == "z(m);Q(W/m^3)"
    assert len(lines) == 1 + 3
    for k, iz in enumerate(range(2, 5)):
        assert lines[1 + k] == "%s;%s" % (_g(-0.0002 + iz * 0.0001), _g(Q[iz, 0, 0]))


def test_slice_dat_xz_and_xy(tmp_path):
    rng = np.random.default_rng(2)
    T = 300 + rng.uniform(0, 20, (7, 6, 5))
    p = tmp_path / "T_XZ.dat"
    api.write_slice_dat(p, T, abi.BD_SLICE_XZ, 3, (1, 6), (0, 4))
    lines = p.read_text().split("\n")
    assert lines[0] == "Z=rows;X=columns" and len(lines) == 6
    assert lines[1] == "".join(_g(T[1, 3, ix]) + ";" for ix in range(0, 4))
    p = tmp_path / "TD_XY.dat"
    hdr = "Y=rows;X=columns;z=15cm"
    api.write_slice_dat(p, T, abi.BD_SLICE_XY, 4, (2, 5), (1, 5), header=hdr)
    lines = p.read_text().split("\n")
    assert lines[0] == hdr and len(lines) == 4
    assert lines[3] == "".join(_g(T[4, 4, ix]) + ";" for ix in range(1, 5))
    with pytest.raises(api.BDError):
        api.write_slice_dat(p, T, abi.BD_SLICE_XY, 9, (0, 1), (0, 1))


def test_threshold_table(tmp_path):
    fr = np.array([[0.02e6, 0.02e6, 0.02e6], [0.02e6, 0.0222e6, 0.0222e6]])
    R0 = np.array([1e-7, 2e-7, 3e-7])
    res = np.array([[1e7, 2.5e6, 1.1e6], [1e7, 3e6, -1.0]])
    p = tmp_path / "dR.dat"
    api.write_threshold_table(p, fr, R0, res, 12.5)
    lines = p.read_text().split("\n")
    assert lines[0] == "fr1;fr2;fr3 --> R0;" + ";".join(_g(r) for r in R0)
    assert lines[2] == ";".join(_g(v) for v in list(fr[1]) + list(res[1]))
    assert lines[-1] == "time (s);12.5"
