"""GPU parity of the batched NLTE MALI solver (pyrh_nlte_solve /
pyrh_nlte_emergent through the C ABI) against the compiled reference's
golden populations and emergent intensities.

Tolerances (relative, element-wise):
  FP64: populations and emergent intensity vs reference   1e-6
  FP32 formal solution (FP64 rates, LU, Ng):               1e-3
The FP32 bound is measured, not designed: single-precision I and Psi change
the path of the iteration (a few more or fewer iterations, a different Ng
extrapolation), so the FP32 run stops at a different point inside the same
convergence limit of 1e-4; measured errors of the converged populations are
0.8e-4 to 3.5e-4 on these atmospheres.  The MALI effective intensity
I - Psi*eta of fillgamma.c:121-134 is formed without cancellation inside the
Bezier recurrence; formed as a difference it cost up to 2e-3 in optically
thick line cores.  FP64 is the parity mode.
"""
import numpy as np
import pytest

from oracle import oracle as O
from pyrh_gb300 import _lib as L
from pyrh_gb300 import nlte

pytestmark = pytest.mark.gpu

CASES = ["nlte_c1", "nlte_c4_50", "nlte_c4_120"]


def _solve(atms, precision, nmax_iter=None):
    cfg = nlte.make_config(atms[0], precision, nmax_iter=nmax_iter)
    pk = nlte.pack(atms, cfg.nrays)
    dev = nlte.DeviceNlte(pk, cfg)
    st = dev.solve(cfg)
    return dev, cfg, st


def _rel(a, b):
    return np.abs(a / b - 1).max()


@pytest.mark.parametrize("name", CASES)
def test_first_iteration_fp64(golden, name):
    """One iteration (Gamma from one formal pass, statEquil, no Ng) gives the
    reference's populations and J after its first iteration."""
    fx = golden(name)
    dev, cfg, st = _solve([fx], L.PYRH_FP64, nmax_iter=1)
    assert st in (L.PYRH_OK, L.PYRH_ERR_NONCONVERGED)
    assert _rel(dev.populations()[0], fx["n1"]) < 1e-7
    J = dev.mean_intensity()[0]
    assert np.abs(J - fx["J1"]).max() <= 1e-9 * np.abs(fx["J1"]).max()


@pytest.mark.parametrize("name", CASES)
def test_converged_fp64(golden, name):
    fx = golden(name)
    dev, cfg, st = _solve([fx], L.PYRH_FP64)
    assert st == L.PYRH_OK, L.lib().pyrh_last_error()
    n_or, J_or, it_or, dp_or, _ = O.nlte_solve(fx)
    assert int(dev.iterations.cpu()[0]) == it_or
    assert _rel(dev.populations()[0], fx["n_final"]) < 1e-6
    assert dev.emergent(cfg, float(fx["fmeta"][2])) == L.PYRH_OK
    I = dev.emergent_spectra()[0]
    m = O.output_mask(fx["lambda"], fx["fmeta"][1])
    assert _rel(I[m], fx["I_out"]) < 1e-6


def test_converged_fp32(golden):
    fx = golden("nlte_c1")
    dev, cfg, st = _solve([fx], L.PYRH_FP32)
    assert st == L.PYRH_OK, L.lib().pyrh_last_error()
    assert _rel(dev.populations()[0], fx["n_final"]) < 1e-3
    assert dev.emergent(cfg, float(fx["fmeta"][2])) == L.PYRH_OK
    m = O.output_mask(fx["lambda"], fx["fmeta"][1])
    assert _rel(dev.emergent_spectra()[0][m], fx["I_out"]) < 1e-3


def test_ragged_batch_fp64(golden):
    """Atmospheres with 82, 50 and 120 depths and 787, 629 and 989
    wavelengths converge in one batch, each after its own iteration count,
    to the same populations as alone."""
    atms = [golden(n) for n in CASES]
    dev, cfg, st = _solve(atms, L.PYRH_FP64)
    assert st == L.PYRH_OK, L.lib().pyrh_last_error()
    its = dev.iterations.cpu().numpy()
    for fx, n, it in zip(atms, dev.populations(), its):
        assert _rel(n, fx["n_final"]) < 1e-6
        assert it == O.nlte_solve(fx)[2]
