"""GPU background continuum (pyrh_background through the C ABI) against the
reference's Background() output in the `background` fixture and against the
oracle (oracle/background.py) on ragged batches, with the scattering added
to the opacity (the NLTE set-up) and with compute1d's fudge factors.

Tolerance: 1e-12 relative, element-wise (FP64; device exp / pow against the
host's)."""
import ctypes as C

import numpy as np
import pytest

from oracle import background as BG
from pyrh_gb300 import _lib as L
from pyrh_gb300 import background as B

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bgfx(golden):
    return golden("background")


def _rel(a, b):
    return np.abs(a / b - 1).max()


def test_matches_reference(bgfx):
    dev = B.DeviceBackground(B.model_from_setup(bgfx))
    atms = [B.setup_atmosphere(bgfx, a) for a in range(2)]
    chi, eta, sca = dev.compute(atms)
    for a in range(2):
        ref = bgfx["cont"][a]
        assert _rel(chi[a], ref[0]) < 1e-12
        assert _rel(eta[a], ref[1]) < 1e-12
        assert _rel(sca[a], ref[2]) < 1e-12


def _subset(fx, a, lam_idx, nd):
    """Atmosphere a of the fixture on some of its wavelengths and its first
    nd depths, in the oracle's form and in compute()'s."""
    sub = dict(fx)
    sub["lambda"] = fx["lambda"][lam_idx]
    for k in ("T", "ne", "nHmin", "nH2", "nOH", "nCH"):
        sub[k] = fx[k][a:a + 1, :nd]
    sub["atoms_n"] = fx["atoms_n"][a:a + 1, :, :nd]
    sub["atoms_nstar"] = fx["atoms_nstar"][a:a + 1, :, :nd]
    return sub, B.setup_atmosphere(sub, 0)


def test_ragged_batch_against_oracle(bgfx):
    """Three atmospheres with 71, 40 and 55 depths and 241, 97 and 13
    wavelengths in one call."""
    rng = np.random.default_rng(7)
    ns = len(bgfx["lambda"])
    cases = [(0, np.arange(ns), 71),
             (1, np.sort(rng.choice(ns, 97, replace=False)), 40),
             (0, np.sort(rng.choice(ns, 13, replace=False)), 55)]
    subs = [_subset(bgfx, a, idx, nd) for a, idx, nd in cases]
    dev = B.DeviceBackground(B.model_from_setup(bgfx))
    chi, eta, sca = dev.compute([s[1] for s in subs])
    for p, (sub, _) in enumerate(subs):
        c, e, s, _ = BG.background(sub, 0)
        assert _rel(chi[p], c) < 1e-12 and _rel(eta[p], e) < 1e-12 and _rel(sca[p], s) < 1e-12


def test_scatter_and_fudge(bgfx):
    fl = np.array([100.0, 400.0, 900.0, 3000.0, 30000.0])
    fv = np.array([[1.0, 1.3, 0.9, 1.1, 1.0],     # H-minus
                   [0.8, 1.0, 1.2, 1.0, 1.05],    # scattering
                   [1.5, 1.2, 1.0, 0.7, 1.0]])    # metals
    dev = B.DeviceBackground(B.model_from_setup(bgfx), add_scatter=True, fudge=(fl, fv))
    chi, eta, sca = dev.compute([B.setup_atmosphere(bgfx, 1)])
    c, e, s, _ = BG.background(bgfx, 1, add_scatter=True, fudge=(fl, fv))
    assert _rel(chi[0], c) < 1e-12 and _rel(eta[0], e) < 1e-12 and _rel(sca[0], s) < 1e-12
    # the fudge changes the result where it differs from one
    c0, _, _, _ = BG.background(bgfx, 1, add_scatter=True)
    assert _rel(c, c0) > 1e-3


def test_bad_rows_are_refused(bgfx):
    """A population row beyond npop is an argument error before any kernel
    runs."""
    m = B.model_from_setup(bgfx)
    m.npop = 10
    with pytest.raises(RuntimeError):
        B.DeviceBackground(m)
    assert "population row" in L.lib().pyrh_last_error().decode()


def test_population_rows_lte_or_not(bgfx):
    """LTE populations given once (n = n*, the passive atoms) or as separate
    n and n* rows: the same background."""
    atm = [B.setup_atmosphere(bgfx, 0)]
    a = B.DeviceBackground(B.model_from_setup(bgfx, lte=True)).compute(atm)
    b = B.DeviceBackground(B.model_from_setup(bgfx, lte=False)).compute(atm)
    for x, y in zip(a, b):
        assert _rel(x[0], y[0]) < 1e-14


def test_fp32_against_fp64(bgfx):
    """The FP32 depth loop (what the FP32 synthesis takes as chi_c, eta_c)
    within 2e-5 of FP64 wherever the FP64 value is inside FP32's normal
    range."""
    dev = B.DeviceBackground(B.model_from_setup(bgfx))
    atms = [B.setup_atmosphere(bgfx, a) for a in range(2)]
    r64 = dev.compute(atms)
    r32 = dev.compute(atms, precision=L.PYRH_FP32)
    for x64, x32 in zip(r64, r32):
        for a in range(2):
            assert x32[a].dtype == np.float32
            m = np.abs(x64[a]) > 1e-30
            assert np.abs(x32[a][m] / x64[a][m] - 1).max() < 2e-5
