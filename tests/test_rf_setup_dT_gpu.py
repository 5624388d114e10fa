"""GPU temperature response functions with the set-up's temperature
derivatives (pyrh_lte_setup_dT), through the C ABI.

Checked against
  * the same adjoint on the CPU in FP64 (tests/native/rf_host.cu), which
    tests/test_rf_setup_dT.py pins to central differences of the oracle with
    the linearized set-up, itself pinned there to the reference's own
    temperature response functions;
  * the reference's temperature response functions directly (central
    differences of rhf1d(), fixtures <name>_dT.npz), at the photospheric
    depths of the fixtures (index >= 40), at every wavelength (DELO-Bezier3
    or Feautrier, as the reference chooses).  Above them lies the temperature
    minimum, where the reference's finite-difference steps straddle a branch
    switch of the centred-derivative limiter (neighbouring temperatures
    differ by 0.1 K); the matched-step comparison of test_rf_setup_dT.py
    covers those depths.  Bound 5e-3 of the largest |dS/dT| there (best of
    the three reference steps per element; measured 2.6e-3 on the CPU
    adjoint: the reference's single-precision 4x4 inverse over the step);
  * each other: chi^2 gradient and VJP equal the contraction of the RFs.
Tolerances as in test_rf_gpu.py: FP64 kernel vs CPU adjoint 1e-8 of the
parameter's largest |RF|; FP32 2e-4 at the 99.9th percentile and 1e-3 at
most.
"""
import numpy as np
import pytest

from conftest import delo_wavelengths, rf_eval
from oracle import oracle as O
from pyrh_gb300 import _lib as L
from pyrh_gb300 import lte, rf as RF
from test_rf_gpu import contract_err, gpu_rf, rel_err
from test_rf_setup_dT import setup_dT

pytestmark = pytest.mark.gpu

FP64, FP32 = L.PYRH_FP64, L.PYRH_FP32


def with_dT(fx, d):
    out = dict(fx)
    out.update({k: v for k, v in d.items() if k.startswith("dT_")})
    return out


@pytest.mark.parametrize("name", ["lte_c0", "lte_edge"])
@pytest.mark.parametrize("precision", [FP64, FP32])
def test_rf_with_setup_matches_cpu_adjoint(rf_harness, golden, name, precision):
    fx, d = golden(name), golden(name + "_dT")
    dev, _, st, rfs = gpu_rf([with_dT(fx, d)], precision)
    assert dev.struct.setup_dT
    win = np.arange(len(fx["lam"]))       # DELO-Bezier3 and Feautrier wavelengths
    _, rf_h = rf_eval(rf_harness, fx, win, setup_dT=setup_dT(d))
    ref = rf_h.transpose(1, 2, 3, 0)                  # [4, 6, nd, nsel]
    mine = rfs[0][..., win]
    if precision == FP64:
        assert rel_err(mine, ref) < 1e-8
    else:
        for x in range(6):
            e = np.abs(mine[:, x] - ref[:, x]) / np.abs(ref[:, x]).max()
            assert np.percentile(e, 99.9) < 2e-4 and e.max() < 1e-3, (RF.PARAMS[x], e.max())
    # without the set-up derivatives only the temperature response changes
    _, _, _, rfs0 = gpu_rf([fx], precision)
    assert np.array_equal(rfs0[0][:, 1:], rfs[0][:, 1:])
    assert np.abs(rfs0[0][:, 0] - rfs[0][:, 0]).max() > 0.1 * np.abs(rfs[0][:, 0]).max()


@pytest.mark.parametrize("name", ["lte_c0", "lte_edge"])
def test_rf_T_matches_reference_response(golden, name):
    fx, d = golden(name), golden(name + "_dT")
    _, _, _, rfs = gpu_rf([with_dT(fx, d)], FP64)
    out = O.output_mask(fx["lam"], float(fx["lambda_ref"]))
    rows = [a for a, k in enumerate(d["fd_depths"]) if k >= 40]
    ref = d["fd_stokes"][rows]                        # [depth][step][stokes][lam]
    mine = np.stack([rfs[0][:, 0, int(d["fd_depths"][a])][:, out] for a in rows])
    err = np.min(np.abs(ref - mine[:, None]), axis=1)
    assert err.max() < 5e-3 * np.abs(ref).max(), err.max() / np.abs(ref).max()


def test_chi2_grad_and_vjp_with_setup_contract_rf(golden):
    """chi^2 gradient and VJP of a two-atmosphere ragged batch with set-up
    derivatives equal the contraction of its response functions (FP64)."""
    import torch
    a = with_dT(golden("lte_c0"), golden("lte_c0_dT"))
    c = with_dT(golden("lte_edge"), golden("lte_edge_dT"))
    c["mu"] = a["mu"]                                # one ray per batch
    dev, cfg, _, rfs = gpu_rf([a, c], FP64)
    rng = np.random.default_rng(11)
    S = dev.out.cpu().numpy().astype(np.float64)
    obs = S * (1 + 1e-2 * rng.standard_normal(S.shape))
    w = rng.uniform(0.5, 2.0, S.shape) / np.abs(S).max() ** 2
    chi2, grad = RF.chi2_grad(dev, cfg, torch.from_numpy(obs), torch.from_numpy(w))
    g = rng.standard_normal(S.shape) / np.abs(S).max()
    gv = RF.vjp(dev, cfg, torch.from_numpy(g))
    torch.cuda.synchronize()
    chi2, grad, gv = (x.cpu().numpy() for x in (chi2, grad, gv))
    pk = dev.pk
    for p in range(pk.natm):
        o, nl = int(pk.arrays["lam_off"][p]), int(pk.arrays["nlam"][p])
        d0, nd = int(pk.arrays["depth_off"][p]), int(pk.arrays["ndep"][p])
        sl = slice(4 * o, 4 * o + 4 * nl)
        Sp, Op, Wp, Gp = (x[sl].reshape(4, nl) for x in (S, obs, w, g))
        assert abs(chi2[p] - (Wp * (Sp - Op) ** 2).sum()) <= 1e-10 * chi2[p]
        assert np.all(contract_err(grad[:, d0:d0 + nd], 2 * Wp * (Sp - Op), rfs[p]) < 1e-9), p
        assert np.all(contract_err(gv[:, d0:d0 + nd], Gp, rfs[p]) < 1e-9), p
    # and each atmosphere's RFs equal those it gets alone
    for i, fx in enumerate((a, c)):
        _, _, _, one = gpu_rf([fx], FP64)
        assert np.abs(rfs[i] - one[0]).max() <= 1e-12 * np.abs(one[0]).max()
