"""GPU response functions, chi^2 gradients and vector-Jacobian products
(pyrh_lte_rf, pyrh_lte_chi2_grad, pyrh_lte_stokes_vjp through the C ABI).

Checked against
  * the same adjoint evaluated on the CPU in FP64 (tests/native/rf_host.cu),
    which tests/test_rf_host.py pins to central finite differences of the
    oracle's synthesis, the reference's definition of response functions
    (rh/rhf1d/rf_ray.c:205-293);
  * central finite differences of the GPU's own FP64 synthesis
    (pyrh_lte_stokes), at the five steps of tests/test_rf_host.py;
  * each other: chi^2 gradient and VJP equal the contraction of the RFs.
Tolerances are relative to the largest |RF| of each parameter:
  FP64 kernel vs CPU adjoint (FP64)   1e-8 (fused multiply-adds on the GPU)
  FP32 kernel vs CPU adjoint (FP64)   2e-4 at the 99.9th percentile, 1e-3 at
                                      most (polarized terms and isolated
                                      limiter-branch flips; see test_rf_host)
  GPU FD (FP64) vs FP64 kernel        1e-4, per element the closest of five
                                      steps (Humlicek region jumps, FP64
                                      noise of the synthesis)
  chi^2 gradient and VJP vs contracted RFs (FP64)   1e-9
  FP32 VJP vs FP64                                   1e-3 per parameter
  FP32 chi^2 gradient vs FP32 VJP of its seeds       1e-4 per parameter
"""
import numpy as np
import pytest

from conftest import batch_member, delo_wavelengths, rf_eval
from oracle import oracle as O
from pyrh_gb300 import _lib as L
from pyrh_gb300 import lte, rf as RF

pytestmark = pytest.mark.gpu

FP64, FP32 = L.PYRH_FP64, L.PYRH_FP32
PARAMS = RF.PARAMS


def device_batch(atms, precision):
    fx = atms[0]
    lines, n = lte.make_lines(fx["line_const"], fx["zeeman"], fx["zeeman_n"])
    pk = lte.pack(atms, n, precision)
    cfg = lte.make_config(precision=precision, mu=float(fx["mu"]),
                          vmicro_char=float(fx["vmicro_char"]), moving=bool(fx["moving"]))
    return lte.DeviceBatch(pk, lines, n), cfg


def gpu_rf(atms, precision):
    import torch
    dev, cfg = device_batch(atms, precision)
    rf = RF.response_functions(dev, cfg)
    torch.cuda.synchronize()
    assert L.lib().pyrh_last_launch_count() == 1
    rfs = [r.astype(np.float64) for r in RF.split_rf(dev.pk, rf.cpu().numpy())]
    st = [s.astype(np.float64) for s in lte.split_output(dev.pk, dev.out.cpu().numpy())]
    return dev, cfg, st, rfs


def rel_err(mine, ref):
    """max |mine - ref| per parameter over the largest |ref| of that
    parameter; arrays [4, 6, depth, lambda]."""
    scale = np.abs(ref).max(axis=(0, 2, 3))
    return (np.abs(mine - ref).max(axis=(0, 2, 3)) / np.where(scale > 0, scale, 1.0)).max()


def contract_err(got, seed, rf):
    """got [6, depth] against sum over (s, lambda) of seed * rf, per parameter,
    relative to the sum of the magnitudes of the terms (the rounding scale of
    the sum)."""
    want = np.einsum("sl,sxkl->xk", seed, rf)
    scale = np.einsum("sl,sxkl->xk", np.abs(seed), np.abs(rf)).max(axis=1)
    return np.abs(got - want).max(axis=1) / np.where(scale > 0, scale, 1.0)


@pytest.mark.parametrize("name", ["lte_c0", "lte_edge", "lte_mixed"])
@pytest.mark.parametrize("precision", [FP64, FP32])
def test_rf_matches_cpu_adjoint(rf_harness, golden, name, precision):
    fx = golden(name)
    _, _, st, rfs = gpu_rf([fx], precision)
    win = np.arange(len(fx["lam"]))       # DELO-Bezier3 and Feautrier wavelengths
    st_h, rf_h = rf_eval(rf_harness, fx, win)
    ref = rf_h.transpose(1, 2, 3, 0)                  # [4, 6, nd, nsel]
    mine = rfs[0][..., win]
    if precision == FP64:
        assert rel_err(mine, ref) < 1e-8
    else:
        for x in range(6):
            e = np.abs(mine[:, x] - ref[:, x]) / np.abs(ref[:, x]).max()
            assert np.percentile(e, 99.9) < 2e-4 and e.max() < 1e-3, (PARAMS[x], e.max())
    assert np.abs(st[0][:, win] - st_h.T).max() <= (1e-10 if precision == FP64 else 1e-5) * \
        st_h[:, 0].max()


@pytest.mark.parametrize("precision,tol", [(FP64, 1e-9), (FP32, 1e-5)])
def test_rf_stokes_equal_forward_kernel(golden, precision, tol):
    """The RF kernel's forward sweep gives the synthesis kernel's spectra at
    every wavelength: DELO-Bezier3 where a polarizable line is in its
    window, scalar Bezier3 where only unpolarizable lines are (lte_mixed),
    Feautrier where none is (lte_edge has four such wavelengths, every case
    LAMBDA_REF) and, in a static atmosphere, where only unpolarizable lines
    are (lte_static)."""
    b = golden("lte_batch")
    atms = [batch_member(b, i) for i in range(b["T"].shape[0])] + [golden("lte_edge")]
    atms[-1] = dict(atms[-1], mu=atms[0]["mu"])     # one ray per batch
    # lte_mixed has its own line list: a batch of its own, scalar Bezier3
    # near 629.60 nm
    for own in ("lte_mixed", "lte_static"):
        dm, cm, sm_, _ = gpu_rf([golden(own)], precision)
        dm.run(cm)
        fm = lte.split_output(dm.pk, dm.out.cpu().numpy())[0]
        assert np.abs(sm_[0] - fm).max() <= tol * fm[0].max(), own
    dev, cfg, st, _ = gpu_rf(atms, precision)
    dev.run(cfg)
    fwd = lte.split_output(dev.pk, dev.out.cpu().numpy())
    for p, fx in enumerate(atms):
        assert np.abs(st[p] - fwd[p]).max() <= tol * fwd[p][0].max()


def test_rf_ragged_batch_equals_single(golden):
    """Atmospheres of different depth and wavelength counts in one launch
    give the response functions each gives alone."""
    a, c = golden("lte_c0"), golden("lte_edge")
    c = dict(c)
    c["mu"] = a["mu"]                     # one ray per batch
    _, _, _, both = gpu_rf([a, c], FP64)
    for i, fx in enumerate((a, c)):
        _, _, _, one = gpu_rf([fx], FP64)
        assert np.abs(both[i] - one[0]).max() <= 1e-12 * np.abs(one[0]).max()


def test_fp32_ragged_batch_equals_single(golden):
    """FP32, where one block holds several work items (sub-blocks) that
    may belong to different atmospheres or be empty: a ragged batch of five
    atmospheres gives each atmosphere's response functions (no sums across
    threads: equal to rounding) and chi^2 gradient (shared-memory sums in a
    different order: 1e-5 of the largest entry) as it gives alone."""
    import torch
    a, c = golden("lte_c0"), dict(golden("lte_edge"))
    c["mu"] = a["mu"]
    atms = [a, c, a, c, a]
    dev, cfg, _, both = gpu_rf(atms, FP32)
    obs = torch.zeros_like(dev.out)
    w = torch.ones_like(dev.out)
    _, g_both = RF.chi2_grad(dev, cfg, obs, w)
    g_both = g_both.cpu().numpy().astype(np.float64)
    pk = dev.pk
    for i, fx in enumerate(atms):
        d1, _, _, one = gpu_rf([fx], FP32)
        assert np.abs(both[i] - one[0]).max() <= 1e-6 * np.abs(one[0]).max(), i
        _, g1 = RF.chi2_grad(d1, cfg, torch.zeros_like(d1.out), torch.ones_like(d1.out))
        g1 = g1.cpu().numpy().astype(np.float64)
        d0, nd = int(pk.arrays["depth_off"][i]), int(pk.arrays["ndep"][i])
        gb = g_both[:, d0:d0 + nd]
        scale = np.abs(g1).max(axis=1, keepdims=True)
        assert np.all(np.abs(gb - g1) <= 1e-5 * np.where(scale > 0, scale, 1.0)), i


def test_chi2_grad_and_vjp_contract_rf(golden):
    """FP64: chi^2, its gradient and a VJP equal the contraction of the
    response functions (the same linear map, evaluated three ways), to 1e-9
    of the sum of the magnitudes of the contracted terms: the Q and U of the
    15-50 G atmospheres are ~v_B^2 ~ 1e-5 of their profiles, so even FP64
    leaves them ~1e-11 relative rounding, independently in the three
    evaluations."""
    import torch
    b = golden("lte_batch")
    atms = [batch_member(b, i) for i in range(b["T"].shape[0])]
    dev, cfg, st, rfs = gpu_rf(atms, FP64)
    rng = np.random.default_rng(7)
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


def test_fp32_gradients_vs_fp64(golden):
    """FP32 adjoint against FP64.  The VJP (the same seeds for both) is
    compared per parameter relative to the largest |FP64 gradient| of that
    parameter and atmosphere, bound 1e-3.  The FP32 chi^2 gradient is checked
    against the FP32 VJP with the seeds 2 w (S32 - obs) of the FP32 spectra
    (bound 1e-4): against FP64 it also carries the FP32 spectra's absolute
    error (~1e-6 I_c), which adds coherently over wavelengths against
    noise-dominated residuals (1e-3 I_c) -- a property of the forward
    precision, not of the adjoint.  Targets as in the differentiation
    workload: spectra plus Gaussian noise of 1e-3 I_c, weights 1 / sigma^2.
    Below 100 G the VJP seeds only I and B, gamma and chi are not compared:
    there the polarized signals are small differences of the sigma and pi
    profiles (V ~ v_B, Q and U ~ v_B^2 of the profiles, v_B the Zeeman
    splitting in Doppler widths, ~0.007 at 46 G), so single-precision
    profiles (~1e-7) and their derivatives (~1e-6) leave Q, U and V and
    their response functions with relative errors of order 1e-6 / v_B^k:
    measured at 46 G, 6e-3 for Q and U themselves and up to 1e-1 for the
    v_los response of V, all below 1e-7 of I_c.  FP64 mode has no such
    limit and is the mode for weak-field polarimetry."""
    import torch
    b = golden("lte_batch")
    atms = [batch_member(b, i) for i in range(b["T"].shape[0])]
    d64, c64 = device_batch(atms, FP64)
    d32, c32 = device_batch(atms, FP32)
    d64.run(c64)
    torch.cuda.synchronize()
    rng = np.random.default_rng(7)
    S = d64.out.cpu().numpy()
    ic = np.concatenate([np.repeat(s[0].max(), s.size) for s in lte.split_output(d64.pk, S)])
    sigma = 1e-3 * ic
    obs = S + sigma * rng.standard_normal(S.shape)
    w = 1.0 / sigma ** 2
    g = rng.standard_normal(S.shape) / np.abs(S).max()
    for p, fx in enumerate(atms):   # weak fields: seeds on I only
        if np.abs(fx["B"]).min() < 0.01:
            o, nl = int(d64.pk.arrays["lam_off"][p]), int(d64.pk.arrays["nlam"][p])
            g[4 * o + nl:4 * o + 4 * nl] = 0.0
    vj = {}
    for tag, dev, cfg in (("64", d64, c64), ("32", d32, c32)):
        vj[tag] = RF.vjp(dev, cfg, torch.from_numpy(g)).cpu().numpy().astype(np.float64)
    _, grad32 = RF.chi2_grad(d32, c32, torch.from_numpy(obs), torch.from_numpy(w))
    S32 = d32.out.cpu().numpy().astype(np.float64)
    seed32 = 2 * w.astype(np.float32).astype(np.float64) * (S32 - obs.astype(np.float32))
    vj_chi2 = RF.vjp(d32, c32, torch.from_numpy(seed32)).cpu().numpy().astype(np.float64)
    grad32 = grad32.cpu().numpy().astype(np.float64)
    pk = d64.pk
    for p in range(pk.natm):
        d0, nd = int(pk.arrays["depth_off"][p]), int(pk.arrays["ndep"][p])
        params = 6 if np.abs(atms[p]["B"]).min() >= 0.01 else 3
        ref = vj["64"][:params, d0:d0 + nd]
        err = np.abs(vj["32"][:params, d0:d0 + nd] - ref).max(axis=1) / np.abs(ref).max(axis=1)
        assert np.all(err < 1e-3), (p, "vjp", err)
        ref = vj_chi2[:, d0:d0 + nd]
        err = np.abs(grad32[:, d0:d0 + nd] - ref).max(axis=1) / np.abs(ref).max(axis=1)
        assert np.all(err < 1e-4), (p, "chi2", err)


def test_autograd_function_uses_adjoint(golden):
    import torch
    b = golden("lte_batch")
    atms = [batch_member(b, i) for i in range(3)]
    dev, cfg = device_batch(atms, FP64)
    params = RF.get_params(dev).clone().requires_grad_(True)
    S = RF.synthesize(dev, cfg, params)
    g = torch.randn_like(S) / S.detach().abs().max()
    (S * g).sum().backward()
    want = RF.vjp(dev, cfg, g)
    torch.cuda.synchronize()
    assert torch.allclose(params.grad, want, rtol=1e-12, atol=1e-12 * want.abs().max().item())


def test_rf_matches_gpu_finite_differences(golden):
    """Central differences of pyrh_lte_stokes (FP64) at selected depths for
    all six parameters of two perturbed atmospheres at once."""
    import torch
    b = golden("lte_batch")
    atms = [batch_member(b, i) for i in range(2)]
    dev, cfg, _, rfs = gpu_rf(atms, FP64)
    base = RF.get_params(dev).clone()
    pk = dev.pk
    nd = int(pk.arrays["ndep"][0])
    worst = 0.0
    for x, key in enumerate(PARAMS):
        for k in (5, nd // 2, (2 * nd) // 3, nd - 2):
            errs = [[] for _ in range(pk.natm)]
            for rel in (1e-3, 1e-4, 1e-5, 1e-6, 1e-7):
                hs, outs = [], []
                for sgn in (1, -1):
                    pp = base.clone()
                    h = []
                    for p in range(pk.natm):
                        d = int(pk.arrays["depth_off"][p]) + k
                        v = base[x, d].item()
                        h.append(rel * 1e3 if key == "vel" else rel if key in ("gamma_B", "chi_B")
                                 else rel * max(abs(v), 0.1) if key == "B" else rel * abs(v))
                        pp[x, d] = v + sgn * h[-1]
                    hs = h
                    RF.set_params(dev, pp)
                    dev.run(cfg)
                    torch.cuda.synchronize()
                    outs.append(dev.out.cpu().numpy().copy())
                for p in range(pk.natm):
                    o, nl = int(pk.arrays["lam_off"][p]), int(pk.arrays["nlam"][p])
                    fd = (outs[0] - outs[1])[4 * o:4 * o + 4 * nl].reshape(4, nl) / (2 * hs[p])
                    win = delo_wavelengths(atms[p])
                    errs[p].append(np.abs(fd[:, win] - rfs[p][:, x, k][:, win]))
            for p in range(pk.natm):
                scale = np.abs(rfs[p][:, x]).max()
                worst = max(worst, np.min(errs[p], axis=0).max() / scale)
    RF.set_params(dev, base)
    assert worst < 1e-4, worst


@pytest.mark.parametrize("precision,tol", [(FP64, 1e-8), (FP32, 1e-3)])
def test_loggf_rf_matches_cpu_adjoint(rf_harness, golden, precision, tol):
    """dS/dlog10(gf) per line from pyrh_lte_rf against the CPU adjoint, and
    the chi^2 and VJP log gf gradients against their contraction."""
    import torch
    fx = golden("lte_c0")
    dev, cfg = device_batch([fx], precision)
    rf, gf = RF.response_functions(dev, cfg, loggf=True)
    torch.cuda.synchronize()
    nline = dev.nline
    gfs = RF.split_loggf_rf(dev.pk, nline, gf.cpu().numpy().astype(np.float64))[0]
    win = delo_wavelengths(fx)
    _, _, gf_h = rf_eval(rf_harness, fx, win, loggf=True)
    ref = gf_h.transpose(2, 1, 0)                       # [nline, 4, nsel]
    assert np.abs(gfs[..., win] - ref).max() <= tol * np.abs(ref).max()
    S = dev.out.cpu().numpy().astype(np.float64)
    rng = np.random.default_rng(3)
    g = rng.standard_normal(S.shape) / np.abs(S).max()
    _, gl = RF.vjp(dev, cfg, torch.from_numpy(g), loggf=True)
    want = np.einsum("sl,nsl->n", g.reshape(4, -1), gfs)
    scale = np.einsum("sl,nsl->n", np.abs(g.reshape(4, -1)), np.abs(gfs))
    assert np.all(np.abs(gl.cpu().numpy()[0] - want) <= (1e-10 if precision == FP64 else 1e-4) * scale)
    obs = S * (1 + 1e-2 * rng.standard_normal(S.shape))
    w = np.ones_like(S) / np.abs(S).max() ** 2
    _, _, gc = RF.chi2_grad(dev, cfg, torch.from_numpy(obs), torch.from_numpy(w), loggf=True)
    seed = (2 * w * (S - obs)).reshape(4, -1)
    want = np.einsum("sl,nsl->n", seed, gfs)
    scale = np.einsum("sl,nsl->n", np.abs(seed), np.abs(gfs))
    assert np.all(np.abs(gc.cpu().numpy()[0] - want) <= (1e-10 if precision == FP64 else 1e-3) * scale)


@pytest.mark.parametrize("precision", [FP64, FP32])
def test_no_stokes_rf_matches_cpu_adjoint(rf_harness, golden, precision):
    """STOKES_MODE = NO_STOKES through pyrh_lte_rf: Stokes I and its response
    functions (scalar solvers at every wavelength) and the log gf RFs,
    against the CPU adjoint, and the log gf RFs against central differences
    of the reference's own synthesis in log gf (lte_loggf, 1e-5 in FP64)."""
    import torch
    fx, g = golden("lte_nostokes"), golden("lte_loggf")
    lines, n = lte.make_lines(fx["line_const"], fx["zeeman"], fx["zeeman_n"])
    cfg = lte.make_config(precision=precision, mu=float(fx["mu"]),
                          vmicro_char=float(fx["vmicro_char"]), moving=bool(fx["moving"]),
                          stokes_mode=L.PYRH_NO_STOKES)
    dev = lte.DeviceBatch(lte.pack([fx], n, precision), lines, n)
    rf, gf = RF.response_functions(dev, cfg, loggf=True)
    torch.cuda.synchronize()
    mine = RF.split_rf(dev.pk, rf.cpu().numpy().astype(np.float64))[0]      # [4, 6, nd, nlam]
    mine_gf = RF.split_loggf_rf(dev.pk, n, gf.cpu().numpy().astype(np.float64))[0]
    sel = np.arange(len(fx["lam"]))
    st_h, rf_h, gf_h = rf_eval(rf_harness, fx, sel, loggf=True, no_stokes=True)
    ref = rf_h.transpose(1, 2, 3, 0)
    assert np.all(mine[1:] == 0.0)
    if precision == FP64:
        assert rel_err(mine, ref) < 1e-8
    else:
        for x in range(6):
            scale = np.abs(ref[0, x]).max()
            if scale == 0.0:          # the azimuth does not reach Stokes I
                assert np.all(mine[0, x] == 0.0)
                continue
            e = np.abs(mine[0, x] - ref[0, x]) / scale
            assert np.percentile(e, 99.9) < 2e-4 and e.max() < 1e-3, (PARAMS[x], e.max())
    ref_gf = gf_h.transpose(2, 1, 0)                 # [line, stokes, lambda]
    tol = 1e-8 if precision == FP64 else 1e-4
    assert np.abs(mine_gf - ref_gf).max() <= tol * np.abs(ref_gf).max()
    if precision == FP64:
        out = O.output_mask(fx["lam"], float(fx["lambda_ref"]))
        for l in range(n):
            fd = g["fd_loggf"][l]
            err = np.min(np.abs(fd - mine_gf[l, 0, out]), axis=0).max() / np.abs(fd).max()
            assert err < 1e-5, (l, err)
