import ctypes as C
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)
GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden(name: str) -> dict:
    with np.load(os.path.join(GOLDEN, name + ".npz")) as f:
        return {k: f[k] for k in f.files}


def batch_member(b: dict, i: int) -> dict:
    """Atmosphere i of the stacked lte_batch fixture as a single-case dict."""
    return {k: (v[i] if isinstance(v, np.ndarray) and v.ndim >= 1 and v.shape[0] == b["T"].shape[0]
                else v) for k, v in b.items()}


@pytest.fixture(scope="session")
def golden():
    cache = {}

    def get(name):
        if name not in cache:
            cache[name] = load_golden(name)
        return cache[name]
    return get


@pytest.fixture(scope="session")
def rf_harness(tmp_path_factory):
    """tests/native/rf_host.cu compiled for the host: the response-function
    math of pyrh_gb300/csrc/lte_rf.cuh evaluated on the CPU in FP64."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    out = str(tmp_path_factory.mktemp("rf") / "librf_host.so")
    src = os.path.join(REPO, "tests", "native", "rf_host.cu")
    subprocess.run([nvcc, "-std=c++17", "-O2", "-Xcompiler", "-fPIC", "-shared",
                    "-diag-suppress", "20011,20013,20015", "-x", "cu", src, "-o", out], check=True)
    return C.CDLL(out)


def rf_eval(lib, fx, sel, single=False, jac=False, loggf=False, setup_dT=None,
            no_stokes=False):
    """Stokes [nsel, 4] and response functions [nsel, 4, 6, ndep] of one
    atmosphere at the wavelengths fx["lam"][sel] (CPU harness, FP64 or, with
    single=True, FP32; jac=True takes the opacity derivatives in forward
    mode); loggf=True also returns dS/dlog10(gf) [nsel, 4, nline].
    setup_dT: optional dict of the set-up's temperature derivatives
    (dchi_c, deta_c [lambda][depth]; dline_pops [line][2][depth]; dnp,
    dlen_up, dlen_dn [depth]); missing keys are held fixed.  no_stokes:
    STOKES_MODE = NO_STOKES (scalar solvers throughout)."""
    from pyrh_gb300 import lte
    D = C.POINTER(C.c_double)
    keep = []

    def arr(a):
        a = np.ascontiguousarray(a, np.float64)
        keep.append(a)
        return a.ctypes.data_as(D)

    lam = fx["lam"][sel]
    nd = len(fx["T"])
    lines, n = lte.make_lines(fx["line_const"], fx["zeeman"], fx["zeeman_n"])
    st = np.zeros((len(sel), 4))
    rf = np.zeros((len(sel), 4, 6, nd))
    gf = np.zeros((len(sel), 4, max(n, 1)))
    args = [nd, arr(fx["height"]), arr(fx["T"]), arr(fx["ne"]), arr(fx["nHtot"]),
            arr(fx["np"]), arr(fx["vturb"]), arr(fx["vel"]), arr(fx["B"]),
            arr(fx["gamma_B"]), arr(fx["chi_B"]), arr(fx["line_pops"]), n, lines,
            len(sel), arr(lam), arr(fx["chi_c"][sel]), arr(fx["eta_c"][sel]),
            C.c_double(float(fx["mu"])), C.c_double(float(fx["vmicro_char"])),
            st.ctypes.data_as(D), rf.ctypes.data_as(D), gf.ctypes.data_as(D)]
    if setup_dT is None:
        fn = lib.rf_eval_f32 if single else (lib.rf_eval_jac if jac else lib.rf_eval)
    else:
        fn = lib.rf_eval_f32_dT if single else (lib.rf_eval_jac_dT if jac else lib.rf_eval_dT)
        g = setup_dT.get
        args += [arr(g("dchi_c")[sel]) if g("dchi_c") is not None else None,
                 arr(g("deta_c")[sel]) if g("deta_c") is not None else None]
        args += [arr(g(k)) if g(k) is not None else None
                 for k in ("dline_pops", "dnp", "dlen_up", "dlen_dn")]
    lib.rf_set_stokes_mode(0 if no_stokes else 3)
    lib.rf_set_moving(int(fx["moving"]))
    try:
        r = fn(*args)
    finally:
        lib.rf_set_stokes_mode(3)
        lib.rf_set_moving(1)
    assert r == 0
    return (st, rf, gf) if loggf else (st, rf)


def delo_wavelengths(fx) -> np.ndarray:
    """Indices of the wavelengths where a contributing line is inside its
    window (20 VMICRO_CHAR / c, kurucz.c:593-602): the DELO-Bezier3 ones."""
    lam = fx["lam"]
    win = np.zeros(len(lam), bool)
    for l0 in fx["line_const"][:, 0]:
        win |= np.abs(lam - l0) <= lam * 20 * fx["vmicro_char"] / 2.99792458e8
    return np.nonzero(win)[0]


# elements of the passive atoms the hse fixture's run reads (H_6, He, C, N,
# O, S, Fe, Si, Al, Na, Mg), as readAtom matches their IDs
HSE_ATOM_ELEMENTS = [0, 1, 5, 6, 7, 15, 25, 13, 12, 10, 11]


def hse_oracle_inputs(golden, case: int, fixture: str = "hse"):
    """(tab, atoms, mols, ids) for oracle.hse: the element tables the case
    reads (the ltepops fixture's; its third case carries the same abundance
    overrides), the atoms as the reference parsed them (background fixture),
    the molecules of the chem fixture."""
    from oracle import chem as OC
    lp, bg, ch, h = golden("ltepops"), golden("background"), golden("chem"), golden(fixture)
    ti = 2 if case == int(h["ab_case"]) else 0
    tab = {"Tpf": lp["Tpf"], "el_meta": lp["el_meta"][ti], "el_pf": lp["el_pf"],
           "el_ionpot": lp["el_ionpot"]}
    meta = bg["atoms_meta"]
    lo, co, li = (np.concatenate([[0], np.cumsum(meta[:, c])]) for c in (0, 1, 2))
    atoms = []
    for m in range(len(meta)):
        lev = bg["atoms_lev"][lo[m]:lo[m + 1]]
        atoms.append(dict(elem=HSE_ATOM_ELEMENTS[m], E=lev[:, 0], g=lev[:, 1],
                          stage=lev[:, 2].astype(int), cont=bg["atoms_cont"][co[m]:co[m + 1]],
                          lines=bg["atoms_line"][li[m]:li[m + 1]], tab=bg["atoms_tab"]))
    aset = lp["el_meta"][ti][:, 1].astype(np.int32)
    mols = [OC.read_molecule(str(t), aset) for t in ch["molecule_text"]]
    ids = [m["id"] for m in mols]
    return tab, atoms, mols, ids


def hse_fudge(golden, case: int):
    h = golden("hse")
    if case != int(h["fudge_case"]):
        return None
    return h["fudge_wave"], h["fudge_value"]


def passive_model(golden, ab_overrides: bool = False, device: str = "cuda"):
    """pyrh_gb300.equilibria.AtomsModel of the fixtures' runs (the passive
    atoms' files, the chem fixture's molecules, the ltepops fixture's tables,
    with its abundance overrides if asked)."""
    from pyrh_gb300 import chem as CH
    from pyrh_gb300 import equilibria as EQ
    from pyrh_gb300 import grid as G
    from pyrh_gb300 import ltepops as LP
    h, lp, ch, bg = golden("hse"), golden("ltepops"), golden("chem"), golden("background")
    meta = lp["el_meta"][2 if ab_overrides else 0]
    ns = meta[:, 0].astype(np.int32)
    tab = LP.ElementTables(lp["Tpf"], meta[:, 2].copy(), meta[:, 1].astype(np.int32), ns,
                           np.concatenate([[0], np.cumsum(ns)[:-1]]).astype(np.int32),
                           lp["el_pf"], lp["el_ionpot"])
    atoms = [G.read_atom(str(t)) for t in h["atom_text"]]
    mols = [CH.read_molecule(str(t), tab.abundance_set) for t in ch["molecule_text"]]
    return EQ.AtomsModel.build(tab, atoms, mols, float(bg["misc"][0]), device=device)
