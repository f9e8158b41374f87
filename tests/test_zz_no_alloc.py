"""The allocation-free heat entry point (bd_heat_run_device_noalloc), for
callers that cannot call cudaMalloc, checked through the C ABI against the
allocating entry point (bd_spiral_heat_run) on the same problem, twice in a
row so that leftovers of the first call in the shared scratch array cannot
hide.  Device buffers here are owned by the test (torch), as a caller's arena
would own them; the entry point itself allocates nothing.

Tolerance: the FP32 heat tolerance of the other tests (temperature within
1e-5 of the largest temperature rise, dose within 1e-5 relative)."""
import ctypes as C

import numpy as np
import pytest

from bubbledynamics_gb300 import abi, api, presets

pytestmark = pytest.mark.gpu


def _problem():
    k = presets.ref_T_mini_constants()
    prob = presets.make_ref_T(k, precision=abi.BD_F32)
    Q = presets.gaussian_focus_Q(prob.shape, (30, 20, 20), (3.0, 2.0, 2.0), 4.0e7)
    return prob, Q


def _even_spots(prob, n_steps):
    """A spot trajectory of prob's grid with an even step count, so that the
    last step writes the caller's own buffer (an odd count ends in the
    scratch buffer and a copy back)."""
    assert n_steps % 2 == 0
    prob.set_spots(np.array([0, 2], np.int32), np.array([0, -1], np.int32),
                   np.array([n_steps // 2, n_steps // 2], np.int64))
    return prob


@pytest.mark.parametrize("parity", ["odd", "even"])
def test_noalloc_matches_allocating_entry_point_twice(ctx, parity):
    torch = pytest.importorskip("torch")
    lib = api.load()
    prob, Q = _problem()
    if parity == "even":
        prob = _even_spots(prob, 180)
    th = prob.thermal
    expected = ctx.heat(th, Q, prob.traj)
    sx, sy, _ = api.trajectory_shifts(prob.traj)
    assert len(sx) % 2 == (1 if parity == "odd" else 0)
    shifts = np.ascontiguousarray(np.stack([sx, sy], axis=1).astype(np.int32).reshape(-1))
    T0, TD0 = prob.initial_fields()
    theta0 = (T0 - th.T_ref).astype(np.float32)
    hi = TD0.astype(np.float32)
    lo = (TD0 - hi.astype(np.float64)).astype(np.float32)
    dose0 = np.ascontiguousarray(np.stack([hi, lo], axis=-1))
    rise = np.abs(expected["T"] - T0).max()
    assert rise > 1e-3
    for call in range(2):
        d_theta = torch.from_numpy(theta0.copy()).cuda()
        d_Q = torch.from_numpy(Q.astype(np.float32)).cuda()
        d_dose = torch.from_numpy(dose0.copy()).cuda()
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        api.check(lib.bd_heat_run_device_noalloc(ctx.h, C.byref(th), d_theta.data_ptr(), d_Q.data_ptr(),
                                                 d_dose.data_ptr(), shifts.ctypes.data, len(sx), None))
        torch.cuda.synchronize()
        # the call allocated nothing on the device (the warm-up run above loaded the module)
        assert torch.cuda.mem_get_info()[0] == free_before, call
        T = th.T_ref + d_theta.cpu().numpy().astype(np.float64)
        dd = d_dose.cpu().numpy().astype(np.float64)
        dose = dd[..., 0] + dd[..., 1]
        assert np.abs(T - expected["T"]).max() <= 1e-5 * rise, call
        np.testing.assert_allclose(dose, expected["dose"], rtol=1e-5)


def test_noalloc_rejects_sizes_beyond_its_scratch(ctx):
    torch = pytest.importorskip("torch")
    lib = api.load()
    prob, Q = _problem()
    th = prob.thermal
    d = torch.zeros(8, device="cuda")
    shifts = np.zeros(2, np.int32)
    big = abi.Thermal()
    C.memmove(C.byref(big), C.byref(th), C.sizeof(th))
    big.nx = big.ny = 2048
    big.nz = 2048
    big.plane_material = None
    st = lib.bd_heat_run_device_noalloc(ctx.h, C.byref(big), d.data_ptr(), d.data_ptr(), d.data_ptr(),
                                        shifts.ctypes.data, 1, None)
    assert st == abi.BD_ERR_INVALID_ARG
    assert b"allocation-free limit" in lib.bd_last_error_string()
    st = lib.bd_heat_run_device_noalloc(ctx.h, C.byref(th), d.data_ptr(), d.data_ptr(), d.data_ptr(),
                                        shifts.ctypes.data, abi_max_steps() + 1, None)
    assert st == abi.BD_ERR_INVALID_ARG


def abi_max_steps():
    return 1 << 16
