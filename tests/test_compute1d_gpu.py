"""pyrh_gb300.compute1d -- the reference's pyrh.compute1d surface
(pyrh.pyx:537-668) on this library -- against the compiled reference's
outputs of the same calls: the emergent Stokes spectra on the output grid
(lambda_ref dropped), the log gf overrides, and the log gf response
functions.  The set-up state (continuum, heights, stage densities, line
list) comes from the reference's own set-up dump in each fixture; the
wavelength grid is built by the library and must equal the reference's.

Tolerances: Stokes within 1e-5 of I_c in FP64 (the reference's
single-precision 4x4 inverse, portable build) and 1e-4 in FP32; output
wavelengths identical; the log gf RFs within 1e-5 of max |dI/dlog gf| of
the reference's central differences."""
import os

import numpy as np
import pytest

from pyrh_gb300 import _lib as L
from pyrh_gb300 import compute1d as C1

pytestmark = pytest.mark.gpu


def setup_of(fx) -> C1.LteSetup:
    return C1.LteSetup(lam=fx["lam"], chi_c=fx["chi_c"], eta_c=fx["eta_c"],
                       height=fx["height"], np=fx["np"], line_pops=fx["line_pops"],
                       line_const=fx["line_const"], zeeman=fx["zeeman"],
                       zeeman_n=fx["zeeman_n"])


def keyword_dir(tmp_path, fx, stokes_mode):
    # VMACRO_TRESH: 0 makes every atmosphere moving (the fixtures' default),
    # the static fixture ran with 0.1 km/s
    tresh = "0" if int(fx["moving"]) else "0.1"
    (tmp_path / "keyword.input").write_text(
        f"# fixture keywords\n  VMICRO_CHAR = {float(fx['vmicro_char']) / 1e3}\n"
        f"  LAMBDA_REF = {float(fx['lambda_ref'])}\n  VMACRO_TRESH = {tresh}\n"
        f"  STOKES_MODE = {stokes_mode}\n  MAGNETO_OPTICAL = FALSE\n")
    return str(tmp_path)


@pytest.mark.parametrize("name,mode", [("lte_c0", "FULL_STOKES"), ("lte_edge", "FULL_STOKES"),
                                       ("lte_static", "FULL_STOKES"),
                                       ("lte_nostokes", "NO_STOKES")])
@pytest.mark.parametrize("precision,tol", [(L.PYRH_FP64, 1e-5), (L.PYRH_FP32, 1e-4)])
def test_compute1d_matches_reference(golden, tmp_path, name, mode, precision, tol):
    fx = golden(name)
    cwd = keyword_dir(tmp_path, fx, mode)
    atm = np.ascontiguousarray(fx["atm"])
    keep = atm.copy()
    sI, sQ, sU, sV, lam = C1.compute1d(cwd, float(fx["mu"]), 0, atm, fx["wave"],
                                        setup=setup_of(fx), precision=precision)
    assert np.array_equal(atm, keep)             # the caller's arrays are untouched
    assert np.array_equal(lam, fx["lam_out"])
    ref = fx["stokes_ref_portable"]
    ic = ref[0].max()
    for s, got in enumerate((sI, sQ, sU, sV)):
        assert np.abs(got - ref[s]).max() < tol * ic, (s, np.abs(got - ref[s]).max() / ic)


def test_compute1d_loggf_override_and_rfs(golden, tmp_path):
    """NO_STOKES with the line list's log gf passed back unchanged
    (kurucz.c:242-251 recomputes Aji from it) reproduces the reference's
    spectrum; the log gf RFs match the reference's central differences
    (h = 1e-3), and so do differences of overridden syntheses."""
    fx = golden("lte_loggf")
    su = setup_of(golden("lte_nostokes"))
    cwd = keyword_dir(tmp_path, golden("lte_nostokes"), "NO_STOKES")
    ids = np.array([0, 1], np.int32)
    base = fx["loggf"].astype(np.float64)
    (sI, _, _, _, lam), rf = C1.compute1d(cwd, 1.0, 0, fx["atm"], fx["wave"], loggf_ids=ids,
                                          loggf_values=base, get_atomic_rfs=True, setup=su)
    assert np.array_equal(lam, fx["lam_out"])
    assert np.abs(sI - fx["sI"]).max() < 1e-5 * fx["sI"].max()
    assert rf.shape == (2, len(lam))
    for l in range(2):
        fd = fx["fd_loggf"][l, 1]
        assert np.abs(rf[l] - fd).max() < 1e-5 * np.abs(fd).max(), l
        h = 1e-2
        up, dn = base.copy(), base.copy()
        up[l] += h
        dn[l] -= h
        Ip = C1.compute1d(cwd, 1.0, 0, fx["atm"], fx["wave"], ids, up, setup=su)[0]
        Im = C1.compute1d(cwd, 1.0, 0, fx["atm"], fx["wave"], ids, dn, setup=su)[0]
        ref = fx["fd_loggf"][l, 0]
        assert np.abs((Ip - Im) / (2 * h) - ref).max() < 1e-4 * np.abs(ref).max(), l


@pytest.mark.parametrize("lst,name", [("c0", "lte_c0"), ("broadening", "lte_broadening"),
                                      ("mixed", "lte_mixed")])
def test_compute1d_from_the_line_list_text(golden, tmp_path, lst, name):
    """The same synthesis with the line constants and Zeeman patterns read
    from the Kurucz list text by pyrh_kurucz_read instead of the reference's
    set-up dump: within 1e-5 of I_c of the reference's spectrum (FP64)."""
    from pyrh_gb300 import kurucz as K
    from test_kurucz import elements_of, tables_of
    with np.load(os.path.join(os.path.dirname(__file__), "golden", "kurucz_lists.npz")) as f:
        kz = {k: f[k] for k in f.files}
    fx = golden(name)
    lc, zm, zn = K.line_tables(*K.read_kurucz(str(kz[lst + "_text"]), elements_of(kz, lst),
                                              tables_of(kz)))
    su = setup_of(fx)
    su.line_const, su.zeeman, su.zeeman_n = lc, zm, zn
    cwd = keyword_dir(tmp_path, fx, "FULL_STOKES")
    out = C1.compute1d(cwd, float(fx["mu"]), 0, fx["atm"], fx["wave"], setup=su)
    ref = fx["stokes_ref_portable"]
    ic = ref[0].max()
    for s in range(4):
        assert np.abs(out[s] - ref[s]).max() < 1e-5 * ic, s


@pytest.mark.parametrize("precision,tol", [(L.PYRH_FP64, 1e-5), (L.PYRH_FP32, 1e-4)])
def test_compute1d_with_the_gpu_background(golden, tmp_path, precision, tol):
    """The per-wavelength set-up of the C0 synthesis on the device: the
    background continuum from the set-up's densities (pyrh_background, the
    `background` fixture's C0 atmosphere is lte_c0's) on the wavelength grid
    the library builds, then the synthesis -- against the reference's
    compute1d.  The continuum itself within 1e-12 of the reference's (FP64)."""
    from dataclasses import replace

    from pyrh_gb300 import background as B
    fx, bg = golden("lte_c0"), golden("background")
    assert np.array_equal(fx["T"], bg["T"][0]) and np.array_equal(fx["ne"], bg["ne"][0])
    dev = B.DeviceBackground(B.model_from_setup(bg))
    chi, eta = B.continuum_on(dev, B.setup_atmosphere(bg, 0), fx["lam"], precision)
    if precision == L.PYRH_FP64:
        assert np.abs(chi / fx["chi_c"] - 1).max() < 1e-12
        assert np.abs(eta / fx["eta_c"] - 1).max() < 1e-12
    setup = replace(setup_of(fx), chi_c=np.asarray(chi, np.float64),
                    eta_c=np.asarray(eta, np.float64))
    cwd = keyword_dir(tmp_path, fx, "FULL_STOKES")
    sI, sQ, sU, sV, lam = C1.compute1d(cwd, float(fx["mu"]), 0, np.ascontiguousarray(fx["atm"]),
                                        fx["wave"], setup=setup, precision=precision)
    ref = fx["stokes_ref_portable"]
    ic = ref[0].max()
    for s, got in enumerate((sI, sQ, sU, sV)):
        assert np.abs(got - ref[s]).max() < tol * ic, (s, np.abs(got - ref[s]).max() / ic)


@pytest.mark.parametrize("name", ["lte_c0", "lte_edge"])
def test_compute1d_forms_line_pops_from_the_atmosphere(golden, tmp_path, name):
    """With no line_pops in the set-up, compute1d forms the stage densities
    and partition functions of the lines on the device (pyrh_line_pops) from
    the element tables the reference read (fixture ltepops): the spectra
    equal those from the reference's own line_pops and match the
    reference's compute1d."""
    from pyrh_gb300 import ltepops as LP
    fx = golden(name)
    lp = golden("ltepops")
    meta = lp["el_meta"][0]
    ns = meta[:, 0].astype(np.int32)
    tab = LP.ElementTables(lp["Tpf"], meta[:, 2].copy(), meta[:, 1].astype(np.int32), ns,
                           np.concatenate([[0], np.cumsum(ns)[:-1]]).astype(np.int32),
                           lp["el_pf"], lp["el_ionpot"])
    cwd = keyword_dir(tmp_path, fx, "FULL_STOKES")
    atm = np.ascontiguousarray(fx["atm"])
    su = setup_of(fx)
    base = C1.compute1d(cwd, float(fx["mu"]), 0, atm, fx["wave"], setup=su)
    su.line_pops, su.elements = None, tab
    got = C1.compute1d(cwd, float(fx["mu"]), 0, atm, fx["wave"], setup=su)
    ic = base[0].max()
    for s in range(4):
        assert np.abs(got[s] - base[s]).max() < 1e-10 * ic
        assert np.abs(got[s] - fx["stokes_ref_portable"][s]).max() < 1e-5 * ic
