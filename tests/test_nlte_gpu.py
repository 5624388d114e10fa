"""GPU parity of the batched NLTE MALI solver (pyrh_nlte_solve /
pyrh_nlte_emergent through the C ABI) against the compiled reference's
golden populations and emergent intensities.

Tolerances (relative, element-wise):
  FP64: populations and emergent intensity vs reference   1e-6
  FP32 formal solution (FP64 rates, LU, Ng):               1e-4
The FP32 bound is the convergence criterion of the runs (ITER_LIMIT 1e-4);
measured 2-7e-6 with the reference's iteration counts.  Two reformulations
keep single precision from cancelling in optically thick line cores: the
MALI effective intensity I - Psi*eta (fillgamma.c:121-134) is built inside
the Bezier recurrence (and, for Feautrier wavelengths, as Psi times a sum of
positive terms of the two one-sided eliminations), and the preconditioned
downward rate
(2 h nu^3/c^2 + Ieff) g V W - chi_up Psi U_down (fillgamma.c:185-196) is
formed from the escape fraction 1 - X Psi / chi = X_other / chi +
(X / chi)(1 - Psi) with 1 - Psi from the positive Bezier weights.  Formed
as differences they cost up to 2e-3 and 9e-4.  Every rate and J sum has a
fixed order, so solves are bit-reproducible.
"""
import numpy as np
import pytest

from oracle import oracle as O
from pyrh_gb300 import _lib as L
from pyrh_gb300 import nlte

pytestmark = pytest.mark.gpu

CASES = ["nlte_c1", "nlte_c4_50", "nlte_c4_120"]
# nlte_static: the C1 atmosphere without velocities (below VMACRO_TRESH):
# Bezier3 where a polarized line is active, Feautrier elsewhere
PINNED = CASES + ["nlte_static"]


def _solve(atms, precision, nmax_iter=None):
    cfg = nlte.make_config(atms[0], precision, nmax_iter=nmax_iter)
    pk = nlte.pack(atms, cfg.nrays)
    dev = nlte.DeviceNlte(pk, cfg)
    st = dev.solve(cfg)
    return dev, cfg, st


def _rel(a, b):
    return np.abs(a / b - 1).max()


@pytest.mark.parametrize("name", PINNED)
def test_first_iteration_fp64(golden, name):
    """One iteration (Gamma from one formal pass, statEquil, no Ng) gives the
    reference's populations and J after its first iteration."""
    fx = golden(name)
    dev, cfg, st = _solve([fx], L.PYRH_FP64, nmax_iter=1)
    assert st in (L.PYRH_OK, L.PYRH_ERR_NONCONVERGED)
    assert _rel(dev.populations()[0], fx["n1"]) < 1e-7
    J = dev.mean_intensity()[0]
    assert np.abs(J - fx["J1"]).max() <= 1e-9 * np.abs(fx["J1"]).max()


@pytest.mark.parametrize("name", PINNED)
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


@pytest.mark.parametrize("name", PINNED)
def test_converged_fp32(golden, name):
    fx = golden(name)
    dev, cfg, st = _solve([fx], L.PYRH_FP32)
    assert st == L.PYRH_OK, L.lib().pyrh_last_error()
    assert int(dev.iterations.cpu()[0]) == O.nlte_solve(fx)[2]
    assert _rel(dev.populations()[0], fx["n_final"]) < 1e-4
    assert dev.emergent(cfg, float(fx["fmeta"][2])) == L.PYRH_OK
    m = O.output_mask(fx["lambda"], fx["fmeta"][1])
    assert _rel(dev.emergent_spectra()[0][m], fx["I_out"]) < 1e-4


@pytest.mark.parametrize("name", PINNED)
@pytest.mark.parametrize("precision", [L.PYRH_FP32, L.PYRH_FP64])
def test_radiative_rates(golden, name, precision):
    """R_ij and R_ji of every transition (addtoRates, fillgamma.c:375-461)
    after the first formal pass and after the last one of the converged
    solve, against the reference's; keeping them changes nothing else."""
    fx = golden(name)
    tol1, tol = (1e-9, 1e-6) if precision == L.PYRH_FP64 else (1e-5, 1e-4)
    for nmax, keys, bound in ((1, ("R1_line", "R1_cont"), tol1),
                              (None, ("R_final_line", "R_final_cont"), tol)):
        cfg = nlte.make_config(fx, precision, nmax_iter=nmax)
        dev = nlte.DeviceNlte(nlte.pack([fx], cfg.nrays), cfg, rates=True)
        st = dev.solve(cfg)
        assert st == L.PYRH_OK or (nmax == 1 and st == L.PYRH_ERR_NONCONVERGED)
        R = dev.radiative_rates()[0]
        assert _rel(R["lines"], fx[keys[0]]) < bound
        assert _rel(R["continua"], fx[keys[1]]) < bound
        ref = fx["n1"] if nmax == 1 else fx["n_final"]
        assert _rel(dev.populations()[0], ref) < (1e-7 if precision == L.PYRH_FP64 else 1e-4)


@pytest.mark.parametrize("precision", [L.PYRH_FP32, L.PYRH_FP64])
def test_bit_reproducible(golden, precision):
    """Three solves of the same ragged batch give identical populations and
    J, bit for bit (rate and J sums in a fixed order)."""
    atms = [golden(n) for n in CASES]
    cfg = nlte.make_config(atms[0], precision)
    dev = nlte.DeviceNlte(nlte.pack(atms, cfg.nrays), cfg)
    runs = []
    for _ in range(3):
        dev.reset()
        assert dev.solve(cfg) == L.PYRH_OK, L.lib().pyrh_last_error()
        runs.append((dev.t["n"].cpu().numpy().copy(), dev.t["J"].cpu().numpy().copy(),
                     dev.iterations.cpu().numpy().copy()))
    for n, J, it in runs[1:]:
        assert np.array_equal(n, runs[0][0]) and np.array_equal(J, runs[0][1])
        assert np.array_equal(it, runs[0][2])


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
