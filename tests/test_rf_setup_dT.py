"""Temperature response functions that follow T through the set-up.

The reference's response functions are central differences of its whole
synthesis (rh/rhf1d/rf_ray.c:205-293).  For a perturbed temperature it
re-runs Background() (continuum opacity and emissivity, LTE stage densities,
proton density) and convertScales() (heights from tau_500), so its
temperature response includes how those inputs move with T.  The fixtures
<name>_dT.npz hold
  * the set-up's temperature derivatives, central differences of the
    reference's own set-up (tests/golden/make_golden.py, lte_dT_case): the
    set-up is local in depth, so perturbing every depth at once gives the
    derivative of each depth with respect to its own temperature;
  * the reference's temperature response functions themselves: central
    differences of rhf1d() (portable build) with T perturbed at one depth,
    at three steps.

Checked here, on the CPU:
  1. The oracle with the set-up moved to first order in T_k (the linearized
     set-up) reproduces the reference's response functions.  Both are
     compared at the same step, so both straddle the same non-smooth points:
     the centred-derivative limiter switches branch where S or chi has an
     extremum, e.g. at the temperature minimum, where neighbouring
     temperatures differ by 0.1 K and every usable reference step crosses
     the switch.  The bound is 1e-3 of the largest |dS/dT| (best of the three
     steps per element; measured 3.4e-4, the single-precision 4x4 inverse of
     the reference over the step).
  2. The adjoint (tests/native/rf_host.cu, FP64) with the set-up
     derivatives equals central differences of the oracle with the
     linearized set-up at the five steps of test_rf_host.py, within 1e-4 of
     the largest |dS/dT| (measured 5e-6), at every depth including the top
     and bottom two, where the interval-length terms end.
  3. The interval-length derivatives follow convertScales' tau_500 rule
     (pyrh_gb300.rf.tau500_interval_dT against the fixture).
Every wavelength is compared: DELO-Bezier3 where a line is inside its
window, Feautrier (as the reference) elsewhere.
"""
import numpy as np
import pytest

from conftest import delo_wavelengths, rf_eval
from oracle import oracle as O
from pyrh_gb300 import rf as RF

STEPS = (1e-3, 1e-4, 1e-5, 1e-6, 1e-7)


def setup_dT(d):
    return dict(dchi_c=d["dT_chi_c"], deta_c=d["dT_eta_c"], dline_pops=d["dT_line_pops"],
                dnp=d["dT_np"], dlen_up=d["dT_len_up"], dlen_dn=d["dT_len_dn"])


def linearized(fx, d, k, h):
    """The fixture with T_k + h and its set-up inputs moved by h times their
    temperature derivatives."""
    f = dict(fx)
    nd = len(fx["T"])
    f["T"] = fx["T"].copy()
    f["T"][k] += h
    for key in ("chi_c", "eta_c"):
        f[key] = fx[key].copy()
        f[key][:, k] += h * d["dT_" + key][:, k]
    f["line_pops"] = fx["line_pops"].copy()
    f["line_pops"][:, :, k] += h * d["dT_line_pops"][:, :, k]
    f["np"] = fx["np"].copy()
    f["np"][k] += h * d["dT_np"][k]
    length = np.abs(np.diff(fx["height"]))
    if k >= 1:
        length[k - 1] += h * d["dT_len_dn"][k]
    if k + 1 < nd:
        length[k] += h * d["dT_len_up"][k + 1]
    f["height"] = fx["height"][0] - np.concatenate([[0.0], np.cumsum(length)])
    return f


def fd_T(fx, d, k, h, sel):
    out = []
    for sgn in (1, -1):
        f = linearized(fx, d, k, sgn * h)
        out.append(O.lte_synth(f, md_float=False, lam=fx["lam"][sel], chi_c=f["chi_c"][sel],
                               eta_c=f["eta_c"][sel]))
    return (out[0] - out[1]) / (2 * h)


@pytest.mark.parametrize("name", ["lte_c0", "lte_edge"])
def test_linearized_setup_reproduces_reference_T_response(golden, name):
    fx, d = golden(name), golden(name + "_dT")
    out = O.output_mask(fx["lam"], float(fx["lambda_ref"]))
    assert np.array_equal(fx["lam"][out], fx["lam_out"])
    ref = d["fd_stokes"]                         # [depth][step][stokes][lam_out]
    scale = np.abs(ref).max()
    worst = 0.0
    for a, k in enumerate(d["fd_depths"]):
        errs = [np.abs(fd_T(fx, d, int(k), rel * fx["T"][k], out) - ref[a, b])
                for b, rel in enumerate(d["fd_steps"])]
        worst = max(worst, np.min(errs, axis=0).max() / scale)
    assert worst < 1e-3, worst


@pytest.mark.parametrize("name", ["lte_c0", "lte_edge"])
def test_adjoint_T_with_setup_matches_finite_differences(rf_harness, golden, name):
    fx, d = golden(name), golden(name + "_dT")
    win = delo_wavelengths(fx)
    far = np.setdiff1d(np.arange(len(fx["lam"])), win)      # Feautrier wavelengths
    sel = np.union1d(win[::7] if len(win) > 40 else win, far)
    _, rf = rf_eval(rf_harness, fx, sel, setup_dT=setup_dT(d))
    _, rf0 = rf_eval(rf_harness, fx, sel)
    nd = len(fx["T"])
    scale = np.abs(rf[:, :, 0, :]).max()
    depths = sorted({0, 1, 2, *(int(k) for k in d["fd_depths"]), nd - 3, nd - 2, nd - 1})
    worst, moved = 0.0, 0.0
    for k in depths:
        errs = [np.abs(fd_T(fx, d, k, rel * fx["T"][k], sel) - rf[:, :, 0, k].T) for rel in STEPS]
        worst = max(worst, np.min(errs, axis=0).max() / scale)
        moved = max(moved, np.abs(rf[:, :, 0, k] - rf0[:, :, 0, k]).max() / scale)
    assert worst < 1e-4, worst
    assert moved > 0.1          # the set-up terms are not a small correction
    # the other five parameters do not depend on the set-up
    assert np.array_equal(rf[:, :, 1:, :], rf0[:, :, 1:, :])


@pytest.mark.parametrize("name", ["lte_c0", "lte_edge"])
def test_forward_mode_agrees_with_setup_terms(rf_harness, golden, name):
    fx, d = golden(name), golden(name + "_dT")
    sel = delo_wavelengths(fx)[::11]
    _, rv = rf_eval(rf_harness, fx, sel, setup_dT=setup_dT(d))
    _, rj = rf_eval(rf_harness, fx, sel, jac=True, setup_dT=setup_dT(d))
    assert np.abs(rv - rj).max() <= 1e-12 * np.abs(rv).max()


@pytest.mark.parametrize("name", ["lte_c0", "lte_edge"])
def test_interval_length_derivatives_follow_tau500(golden, name):
    fx, d = golden(name), golden(name + "_dT")
    iref = int(np.argmin(np.abs(fx["lam"] - fx["lambda_ref"])))
    assert fx["lam"][iref] == fx["lambda_ref"]
    up, dn = RF.tau500_interval_dT(fx["height"], fx["chi_c"][iref], d["dT_chi_c"][iref])
    scale = max(np.abs(up).max(), np.abs(dn).max())
    assert np.abs(up - d["dT_len_up"]).max() <= 1e-12 * scale
    assert np.abs(dn - d["dT_len_dn"]).max() <= 1e-12 * scale
    # the height scale is the tau_500 one: h_{k-1} - h_k = 2 dtau / (chi_{k-1} + chi_k)
    tau = 10.0 ** fx["atm"][0]
    c = fx["chi_c"][iref]
    dh = fx["height"][:-1] - fx["height"][1:]
    assert np.allclose(dh, 2 * np.diff(tau) / (c[:-1] + c[1:]), rtol=1e-12, atol=0)
