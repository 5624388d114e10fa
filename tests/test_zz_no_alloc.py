"""pyrh_nlte_solve_static (the NLTE solve whose scratch is a fixed device
array, so that the call allocates nothing) against pyrh_nlte_solve with a
caller-allocated workspace, both through the C ABI, on two static calls in a
row (the second finds the first's contents in the array).

The two entry points run the same kernels in the same order, and every
rate and J sum of the solver has a fixed order; where the workspace solve
splits the rays of a small batch into groups whose partial sums would not
fit the static array, the static call keeps one group, which adds the same
terms in another order.  So the comparison uses the solver's parity
tolerances: FP64 populations and J within 1e-6 relative of the workspace
solve and of the reference's converged populations, with identical
iteration counts; FP32 within 1e-4 (the runs' convergence criterion).  The
file name sorts last so that the static array is first touched after every
other test's allocations."""
import ctypes as C

import numpy as np
import pytest

from pyrh_gb300 import _lib as L
from pyrh_gb300 import nlte

pytestmark = pytest.mark.gpu

STATIC_BYTES = 32 * 1024 * 1024
TOL = {L.PYRH_FP64: 1e-6, L.PYRH_FP32: 1e-4}


def _bind():
    lib = nlte._lib()
    lib.pyrh_nlte_solve_static.restype = C.c_int
    lib.pyrh_nlte_solve_static.argtypes = [C.POINTER(nlte.PyrhNlteBatch),
                                           C.POINTER(nlte.PyrhNlteConfig), C.c_int64,
                                           C.c_void_p, C.c_void_p, C.c_void_p]
    return lib


def _static(dev, cfg):
    import torch
    dev.reset()
    it = torch.full_like(dev.iterations, -1)
    dp = torch.full_like(dev.dpops, -1.0)
    st = _bind().pyrh_nlte_solve_static(C.byref(dev.batch), C.byref(cfg), dev.pk.phi_elems,
                                        it.data_ptr(), dp.data_ptr(), 0)
    torch.cuda.synchronize()
    return st, it.cpu().numpy(), dp.cpu().numpy(), dev.populations(), dev.mean_intensity()


def _rel(a, b):
    return float(np.abs(a / b - 1).max())


@pytest.mark.parametrize("names,precision", [
    (["nlte_c1"], L.PYRH_FP64),
    (["nlte_c1", "nlte_c4_50", "nlte_c4_120"], L.PYRH_FP64),
    (["nlte_c1", "nlte_c4_50", "nlte_c4_120"], L.PYRH_FP32),
])
def test_static_matches_workspace_solve(golden, names, precision):
    import torch
    fx = [golden(n) for n in names]
    cfg = nlte.make_config(fx[0], precision)
    dev = nlte.DeviceNlte(nlte.pack(fx, cfg.nrays), cfg)
    st0 = dev.solve(cfg)
    assert st0 in (L.PYRH_OK, L.PYRH_ERR_NONCONVERGED), L.lib().pyrh_last_error()
    if precision == L.PYRH_FP64:
        assert st0 == L.PYRH_OK
    torch.cuda.synchronize()
    it0 = dev.iterations.cpu().numpy().copy()
    dp0 = dev.dpops.cpu().numpy().copy()
    n0, J0 = dev.populations(), dev.mean_intensity()
    for call in range(2):
        st, it, dp, n, J = _static(dev, cfg)
        assert st == st0, (call, L.lib().pyrh_last_error())
        err_n = max(_rel(n[p], n0[p]) for p in range(len(fx)))
        err_J = max(np.abs(J[p] - J0[p]).max() / np.abs(J0[p]).max() for p in range(len(fx)))
        assert err_n < TOL[precision] and err_J < TOL[precision], (call, err_n, err_J)
        assert np.all(dp < cfg.iter_limit) == np.all(dp0 < cfg.iter_limit)
        if precision == L.PYRH_FP64:
            np.testing.assert_array_equal(it, it0)
            for p in range(len(fx)):
                assert _rel(n[p], fx[p]["n_final"]) < TOL[precision], (call, p)


def test_static_rejects_oversized_batch(golden):
    fx = golden("nlte_c1")
    cfg = nlte.make_config(fx, L.PYRH_FP64)
    dev = nlte.DeviceNlte(nlte.pack([fx], cfg.nrays), cfg)
    too_many = STATIC_BYTES // 8 + 1
    st = _bind().pyrh_nlte_solve_static(C.byref(dev.batch), C.byref(cfg), too_many,
                                        None, None, 0)
    assert st == L.PYRH_ERR_ARG
    assert b"static scratch" in L.lib().pyrh_last_error()
