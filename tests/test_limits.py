"""The size limits of include/pyrh_gb300.h, at and past their edges.

At the limits (GPU, marked `gpu`):
  * PYRH_MAX_DEPTH (512) depths in the synthesis, FP64 against the oracle to
    1e-8 of I_c and FP32 to 1e-4 (the tolerances of test_lte_gpu.py);
  * PYRH_RF_MAX_DEPTH (160) depths in the response functions, FP64 against
    the CPU adjoint to 1e-8 of each parameter's largest |RF|;
  * PYRH_NLTE_MAX_DEPTH (160) depths in the NLTE solve, against the NLTE
    oracle (the same iteration count; FP64 1e-6, FP32 1e-4);
  * PYRH_MAX_LINES (16) lines, one of them with PYRH_MAX_COMPONENTS (32)
    Zeeman components, all inside their windows at every wavelength, in the
    synthesis (against the oracle) and in the response functions at 71
    depths (against the CPU adjoint; the first two lines take the taped
    Zeeman sums, the other fourteen re-evaluate theirs in the reverse
    sweep).  The response-function kernel keeps 20 numbers per (line,
    depth) in shared memory, so lines x depths is bounded by the device's
    shared memory per block: 16 lines fit up to about 75 depths in FP64 and
    about 150 in FP32; beyond that the call returns PYRH_ERR_UNSUPPORTED.
The deep atmospheres are the C0 fixture interpolated in depth index (log of
the positive quantities), which keeps the heights monotonic; both sides
solve the same discrete problem, so its physical consistency does not
matter here.
Past the limits (CPU, no device work): empty batches, one depth more than
each limit, one line more and one component more are rejected with an
argument or unsupported status before anything is launched.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import delo_wavelengths, rf_eval
from oracle import oracle as O
from pyrh_gb300 import _lib as L
from pyrh_gb300 import lte, rf as RF

FP64, FP32 = L.PYRH_FP64, L.PYRH_FP32
DEPTH_KEYS = ("height", "T", "ne", "nHtot", "np", "vturb", "vel", "B", "gamma_B", "chi_B")
POSITIVE = ("T", "ne", "nHtot", "np")


def deepen(fx: dict, nd: int, sel=None) -> dict:
    """fx on nd depths (interpolated in depth index); wavelengths fx["lam"][sel]."""
    n0 = len(fx["T"])
    x0, x = np.arange(n0), np.linspace(0, n0 - 1, nd)
    out = dict(fx)
    for k in DEPTH_KEYS:
        v = fx[k]
        out[k] = np.exp(np.interp(x, x0, np.log(v))) if k in POSITIVE else np.interp(x, x0, v)
    lp = fx["line_pops"]
    out["line_pops"] = np.stack([np.stack([np.exp(np.interp(x, x0, np.log(lp[l, 0]))),
                                           np.interp(x, x0, lp[l, 1])])
                                 for l in range(lp.shape[0])])
    sel = np.arange(len(fx["lam"])) if sel is None else sel
    out["lam"] = fx["lam"][sel]
    for k in ("chi_c", "eta_c"):
        c = fx[k][sel]
        out[k] = np.stack([np.exp(np.interp(x, x0, np.log(row))) for row in c])
    return out


def many_lines(fx: dict, nline: int = 16) -> dict:
    """nline copies of the fixture's two lines, 0.01 nm apart (all inside
    each other's windows); line 0 gets a 32-component Zeeman pattern."""
    lc0, z0, zn0 = fx["line_const"], fx["zeeman"], fx["zeeman_n"]
    order = np.argsort(lc0[:, 0])
    lc = np.stack([lc0[order[i % 2]].copy() for i in range(nline)])
    base = lc[:, 0].min()
    for i in range(nline):
        lc[i, 0] = base + 0.01 * i
    maxc = L.PYRH_MAX_COMPONENTS
    z = np.zeros((nline, 3, maxc))
    zn = np.zeros(nline, np.int32)
    for i in range(nline):
        src = order[i % 2]
        n = int(zn0[src])
        z[i, :, :n] = z0[src, :, :n]
        zn[i] = n
    # 32 components: 11 sigma-, 10 pi, 11 sigma+, strengths normalised per q
    q = np.array([-1] * 11 + [0] * 10 + [1] * 11)
    shift = np.concatenate([np.linspace(-3.1, -0.6, 11), np.linspace(-0.9, 0.9, 10),
                            np.linspace(0.6, 3.1, 11)])
    w = 1.0 + 0.5 * np.cos(np.arange(32))
    for qq in (-1, 0, 1):
        w[q == qq] /= w[q == qq].sum()
    z[0, 0], z[0, 1], z[0, 2], zn[0] = q, shift, w, 32
    out = dict(fx)
    out["line_const"], out["zeeman"], out["zeeman_n"] = lc, z, zn
    lp = fx["line_pops"]
    out["line_pops"] = np.stack([lp[order[i % 2]] for i in range(nline)])
    lam = np.linspace(base - 0.04, base + 0.01 * (nline - 1) + 0.04, 48)
    out["lam"] = lam
    for k in ("chi_c", "eta_c"):
        c = fx[k]
        out[k] = np.stack([c[np.argmin(np.abs(fx["lam"] - l))] for l in lam])
    return out


def synth(atms, precision):
    import torch
    fx = atms[0]
    lines, n = lte.make_lines(fx["line_const"], fx["zeeman"], fx["zeeman_n"])
    assert L.lib().pyrh_check_lines(lines, n, L.PYRH_FULL_STOKES) == L.PYRH_OK
    cfg = lte.make_config(precision=precision, mu=float(fx["mu"]),
                          vmicro_char=float(fx["vmicro_char"]), moving=bool(fx["moving"]))
    db = lte.DeviceBatch(lte.pack(atms, n, precision), lines, n)
    db.run(cfg)
    torch.cuda.synchronize()
    return [o.astype(np.float64) for o in lte.split_output(db.pk, db.out.cpu().numpy())]


def gpu_rf(fx, precision=FP64):
    import torch
    lines, n = lte.make_lines(fx["line_const"], fx["zeeman"], fx["zeeman_n"])
    cfg = lte.make_config(precision=precision, mu=float(fx["mu"]),
                          vmicro_char=float(fx["vmicro_char"]), moving=bool(fx["moving"]))
    db = lte.DeviceBatch(lte.pack([fx], n, precision), lines, n)
    rf = RF.response_functions(db, cfg)
    torch.cuda.synchronize()
    return RF.split_rf(db.pk, rf.cpu().numpy().astype(np.float64))[0]   # [4, 6, nd, nlam]


def rel_err(mine, ref):
    scale = np.abs(ref).max(axis=(0, 2, 3))
    return (np.abs(mine - ref).max(axis=(0, 2, 3)) / np.where(scale > 0, scale, 1.0)).max()


# ----------------------------------------------------------------- GPU ---

@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [(FP64, 1e-8), (FP32, 1e-4)])
def test_synthesis_at_max_depth(golden, precision, tol):
    fx = deepen(golden("lte_c0"), L.PYRH_MAX_DEPTH, sel=np.arange(150, 260, 2))
    out = synth([fx], precision)[0]
    ref = O.lte_synth(fx, md_float=False)
    assert np.abs(out - ref).max() / ref[0].max() < tol


@pytest.mark.gpu
def test_response_functions_at_max_depth(rf_harness, golden):
    fx = deepen(golden("lte_c0"), L.PYRH_RF_MAX_DEPTH, sel=np.arange(180, 230, 2))
    mine = gpu_rf(fx)
    win = delo_wavelengths(fx)
    _, rf_h = rf_eval(rf_harness, fx, win)
    assert rel_err(mine[..., win], rf_h.transpose(1, 2, 3, 0)) < 1e-8


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [(FP64, 1e-8), (FP32, 1e-4)])
def test_synthesis_with_max_lines_and_components(golden, precision, tol):
    fx = many_lines(golden("lte_c0"))
    out = synth([fx], precision)[0]
    ref = O.lte_synth(fx, md_float=False)
    assert np.abs(out - ref).max() / ref[0].max() < tol
    # every line is inside its window at every wavelength
    assert len(delo_wavelengths(fx)) == len(fx["lam"])


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [FP64, FP32])
def test_response_functions_with_max_lines_and_components(rf_harness, golden, precision):
    fx = many_lines(golden("lte_c0"))
    mine = gpu_rf(fx, precision)
    _, rf_h = rf_eval(rf_harness, fx, np.arange(len(fx["lam"])))
    ref = rf_h.transpose(1, 2, 3, 0)
    if precision == FP64:
        assert rel_err(mine, ref) < 1e-8
    else:
        # sixteen overlapping lines add into the same opacity sums, so the
        # single-precision rounding of the small Zeeman differences behind
        # the B response grows with the line count: measured 3.8e-4 at the
        # 99.9th percentile and 1.1e-3 at most (two lines: 1e-4 / 4e-4)
        for x in range(6):
            e = np.abs(mine[:, x] - ref[:, x]) / np.abs(ref[:, x]).max()
            assert np.percentile(e, 99.9) < 1e-3 and e.max() < 3e-3, (RF.PARAMS[x], e.max())


NLTE_LOG = ("T", "ne", "nHtot", "ntotal", "vbroad", "background", "nstar", "n0", "adamp")
NLTE_LIN = ("vel", "vturb", "height", "C", "wphi", "atm")
NLTE_REF = ("Gamma1", "J1", "n1", "n_final", "J_final", "I_out", "phi_sample", "phi_sample_la")


def deepen_nlte(fx: dict, nd: int) -> dict:
    """An NLTE fixture on nd depths (interpolated in depth index, log of the
    positive quantities); the reference's results are dropped."""
    n0 = len(fx["T"])
    x0, x = np.arange(n0), np.linspace(0, n0 - 1, nd)
    out = {k: v for k, v in fx.items() if k not in NLTE_REF}
    for k in NLTE_LOG + NLTE_LIN:
        v = np.asarray(fx[k], np.float64)
        rows = v.reshape(-1, n0)
        if k in NLTE_LOG:
            r = np.stack([np.exp(np.interp(x, x0, np.log(row))) for row in rows])
        else:
            r = np.stack([np.interp(x, x0, row) for row in rows])
        out[k] = r.reshape(v.shape[:-1] + (nd,)) if v.ndim > 1 else r[0]
    m = np.array(fx["meta"]).copy()
    m[1] = nd
    out["meta"] = m
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [(FP64, 1e-6), (FP32, 1e-4)])
def test_nlte_at_max_depth(golden, precision, tol):
    """PYRH_NLTE_MAX_DEPTH (160) depths: the C1 atmosphere interpolated onto
    160 depths, solved to convergence on the GPU and by the NLTE oracle (35
    iterations); both precisions take the same number of iterations.  FP32
    bound: the convergence criterion itself (measured 4-7e-6)."""
    from pyrh_gb300 import nlte
    fx = deepen_nlte(golden("nlte_c1"), L.PYRH_NLTE_MAX_DEPTH)
    n_or, _, it_or, _, _ = O.nlte_solve(fx)
    cfg = nlte.make_config(fx, precision)
    dev = nlte.DeviceNlte(nlte.pack([fx], cfg.nrays), cfg)
    assert dev.solve(cfg) == L.PYRH_OK, L.lib().pyrh_last_error()
    assert int(dev.iterations.cpu()[0]) == it_or
    assert np.abs(dev.populations()[0] / n_or - 1).max() < tol


# ----------------------------------------------------------------- CPU ---

def _host_batch(fx, n):
    pk = lte.pack([fx], n)
    arrs = {k: np.ascontiguousarray(v) for k, v in pk.arrays.items()}
    return pk, arrs, lte._batch_struct(pk, lambda k: arrs[k].ctypes.data)


def test_limits_rejected_before_launch(golden):
    """Host-side checks: nothing here touches a device (the pointers are
    host arrays, which the entry points never dereference before their
    checks pass)."""
    lib = L.lib()
    from pyrh_gb300 import rf as RFm
    RFm._lib()
    fx = golden("lte_c0")
    lines, n = lte.make_lines(fx["line_const"], fx["zeeman"], fx["zeeman_n"])
    cfg = lte.make_config(precision=FP64, vmicro_char=float(fx["vmicro_char"]))
    out = np.zeros(4 * len(fx["lam"]))
    rf = np.zeros(8)
    pk, arrs, b = _host_batch(fx, n)
    # empty batch
    b.natm = 0
    assert lib.pyrh_lte_stokes(C.byref(b), lines, n, C.byref(cfg), out.ctypes.data,
                               None) == L.PYRH_ERR_ARG
    assert lib.pyrh_lte_stokes_host(C.byref(b), lines, n, C.byref(cfg),
                                    out.ctypes.data) == L.PYRH_ERR_ARG
    assert lib.pyrh_lte_rf(C.byref(b), lines, n, C.byref(cfg), out.ctypes.data,
                           rf.ctypes.data, None, None) == L.PYRH_ERR_ARG
    # one depth past each limit
    b.natm = 1
    b.max_ndep = L.PYRH_MAX_DEPTH + 1
    assert lib.pyrh_lte_stokes(C.byref(b), lines, n, C.byref(cfg), out.ctypes.data,
                               None) == L.PYRH_ERR_ARG
    b.max_ndep = L.PYRH_RF_MAX_DEPTH + 1
    b.total_depth = max(b.total_depth, b.max_ndep)
    assert lib.pyrh_lte_rf(C.byref(b), lines, n, C.byref(cfg), out.ctypes.data,
                           rf.ctypes.data, None, None) == L.PYRH_ERR_UNSUPPORTED
    # 16 lines x 160 depths: more per-(line, depth) tables than shared memory holds
    ml = many_lines(fx)
    ml = deepen(ml, L.PYRH_RF_MAX_DEPTH)
    ml_lines, nml = lte.make_lines(ml["line_const"], ml["zeeman"], ml["zeeman_n"])
    _, arrs2, b2 = _host_batch(ml, nml)
    assert lib.pyrh_lte_rf(C.byref(b2), ml_lines, nml, C.byref(cfg), out.ctypes.data,
                           rf.ctypes.data, None, None) == L.PYRH_ERR_UNSUPPORTED
    assert b"shared memory" in lib.pyrh_last_error()
    # one line and one component past the limits
    assert lib.pyrh_check_lines(lines, L.PYRH_MAX_LINES + 1, L.PYRH_FULL_STOKES) == \
        L.PYRH_ERR_ARG
    bad = (L.PyrhLine * 1)()
    C.memmove(bad, lines, C.sizeof(L.PyrhLine))
    bad[0].ncomp = L.PYRH_MAX_COMPONENTS + 1
    assert lib.pyrh_check_lines(bad, 1, L.PYRH_FULL_STOKES) == L.PYRH_ERR_ARG


def test_deepened_nlte_problem_matches_at_original_depths(golden):
    """deepen_nlte at the fixture's own depth count changes nothing: the
    oracle still reproduces the reference's converged populations."""
    fx = golden("nlte_c1")
    same = deepen_nlte(fx, len(fx["T"]))
    n, _, it, _, _ = O.nlte_solve(same)
    assert np.abs(n / fx["n_final"] - 1).max() < 1e-8


def test_deepened_atmosphere_is_a_valid_input(golden):
    fx = deepen(golden("lte_c0"), L.PYRH_MAX_DEPTH, sel=np.arange(150, 160))
    assert np.all(np.diff(fx["height"]) < 0)
    assert np.all(fx["chi_c"] > 0) and fx["chi_c"].shape == (10, L.PYRH_MAX_DEPTH)
    ml = many_lines(golden("lte_c0"))
    lines, n = lte.make_lines(ml["line_const"], ml["zeeman"], ml["zeeman_n"])
    assert n == L.PYRH_MAX_LINES
    assert L.lib().pyrh_check_lines(lines, n, L.PYRH_FULL_STOKES) == L.PYRH_OK
