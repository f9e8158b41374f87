"""The C ABI library loads without a GPU, exports every function declared in
include/bubbledyn.h, and its structs have the layout the Python mirror uses.
Host-only entry points (trajectory, quarter unfolding, combos) run here."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

from bubbledynamics_gb300 import abi, api, presets
from tests.conftest import ROOT

HEADER = os.path.join(ROOT, "include", "bubbledyn.h")


def declared_functions():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^(?:bd_status|const char\*|int)\s+(bd_[a-z0-9_]+)\(", txt, re.M)))


def test_library_exports_every_declared_function(lib):
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert missing == []
    assert lib.bd_abi_version() == 2


def test_struct_layout_matches_c():
    src = ['#include <stdio.h>', '#include <stddef.h>', '#include "bubbledyn.h"', "int main(void) {"]
    for cname in abi.ALL_STRUCTS:
        src.append('printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
    src.append("return 0; }")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(c, "w").write("\n".join(src))
        subprocess.run(["gcc", "-I", os.path.dirname(HEADER), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    sizes = dict(l.split() for l in out.strip().splitlines())
    for cname, py in abi.ALL_STRUCTS.items():
        assert int(sizes[cname]) == C.sizeof(py), cname


def test_status_codes_and_errors(lib):
    # a host-only call with a bad argument returns BD_ERR_INVALID_ARG and sets the error text
    n = C.c_int64(0)
    st = lib.bd_gilmore_combos(1, 1.0, 2.0, None, 0, C.byref(n))
    assert st == abi.BD_ERR_INVALID_ARG
    assert b"combo" in lib.bd_last_error_string()


def test_combos_match_reference_count(oracle):
    fr = api.gilmore_combos()
    assert fr.shape == (27775, 3)                           # G:468
    np.testing.assert_array_equal(fr, oracle.gilmore_combos())
    assert np.all(fr[:, 0] <= fr[:, 1]) and np.all(fr[:, 1] <= fr[:, 2])
    # no (i < ii == iii) triples (G:505-507)
    assert not np.any((fr[:, 0] < fr[:, 1]) & (fr[:, 1] == fr[:, 2]))


def test_combo_tones_normalisation(lib):
    for f, nt, amp in (([1e6, 1e6, 1e6], 1, 1.0), ([1e6, 1e6, 2e6], 2, 2 ** -0.5), ([1e6, 2e6, 2e6], 2, 2 ** -0.5),
                       ([1e6, 2e6, 3e6], 3, 3 ** -0.5)):
        b = abi.Bubble()
        b.R0 = 1e-6
        fa = np.array(f)
        api.check(lib.bd_gilmore_combo_tones(2.0e6, fa.ctypes.data, None, C.byref(b)))
        assert b.n_tones == nt and b.R0 == 1e-6
        assert b.a[0] == pytest.approx(2.0e6 * amp)
        if nt == 2:
            assert (b.f[0], b.f[1]) == (f[0], f[2])          # G:52 drives f1 and f3


def test_unfold_quarter_mirrors():
    h, nz = 4, 3
    small = np.arange(nz * (h + 1) * (h + 1), dtype=np.float64)
    full = api.unfold_quarter(small, h, nz)
    s = small.reshape(nz, h + 1, h + 1)
    for iz in range(nz):
        for iy in range(2 * h + 1):
            for ix in range(2 * h + 1):
                assert full[iz, iy, ix] == s[iz, abs(iy - h), abs(ix - h)]


def test_spot_trajectory():
    t = presets.make_ref_T(presets.ref_T_mini_constants())
    t.set_spots([0, 3, -2], [1, 1, 0], [5, 0, 7])
    sx, sy, legs = api.trajectory_shifts(t.traj)
    assert list(legs) == [5, 5, 12]
    assert list(sx) == [0] * 5 + [-2] * 7 and list(sy) == [1] * 5 + [0] * 7


def test_reference_presets():
    k = presets.ref_W_constants()
    assert (k["Nxy"], k["Nz"]) == (426, 2003)                          # W:410-414
    t1 = presets.accumulate_times(k["dt"], k["t_max"])
    assert len(t1) == 16500                                            # W:558 loop with float t
    assert len(presets.accumulate_times(k["dt"], k["t_max"] + 1 / k["fr"], t1[-1])) == 100   # W:627
    planes = [0 if (k["z_min"] + iz * k["dz"]) < k["water_tissue"] else 1 for iz in range(1198, 1206)]
    assert planes == [0, 0, 0, 0, 1, 1, 1, 1]                          # water ends before iz_tissue = 1202
    kt = presets.ref_T_constants()
    assert (kt["Nxy"], kt["Nz"]) == (851, 2001)                        # T:158, T:163
    assert len(presets.ref_G_R0s()) == 100                             # G:460
