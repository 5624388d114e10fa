"""ctypes front-end of the CPU ORACLE (oracle/rt_oracle.c) -- test
infrastructure.  Only tests/, __graft_entry__.smoke() and the cpu_baseline
leg of bench.py may use it, always as the checker / baseline, never as the
product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "librt_oracle.so")
SOURCES = [os.path.join(HERE, "rt_oracle.c"), os.path.join(HERE, "nlte_oracle.c")]

RLK_NCONST = 24
_STACKED = ("mu", "line_const", "zeeman", "zeeman_n", "vmicro_char", "magneto_optical",
            "moving", "lam")
_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)


class OracleAtmos(C.Structure):
    _fields_ = [("ndep", C.c_int), ("muz", C.c_double)] + \
        [(n, _D) for n in ("height", "T", "ne", "nHtot", "np", "vturb", "vel", "B",
                           "gamma_B", "chi_B", "line_pops")]


class OracleLines(C.Structure):
    _fields_ = [("nline", C.c_int), ("maxcomp", C.c_int), ("magneto_optical", C.c_int),
                ("moving", C.c_int), ("no_stokes", C.c_int), ("vmicro_char", C.c_double),
                ("c", _D),
                ("zeeman", _D), ("ncomp", _I)]


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (OpenMP for the threaded batch driver)."""
    newest = max(os.path.getmtime(s) for s in SOURCES + [os.path.join(HERE, "rt_oracle.h"),
                                                         os.path.join(HERE, "nlte_oracle.h")])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-o", LIB] + SOURCES +
                   ["-lm"], check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
        _lib.oracle_lte_synth.restype = C.c_int
        _lib.oracle_lte_synth_batch.restype = C.c_int
        _lib.oracle_lte_opacity.restype = C.c_int
        _lib.oracle_planck.restype = C.c_double
        _lib.oracle_planck.argtypes = [C.c_double, C.c_double]
        _lib.oracle_humlicek.argtypes = [C.c_double, C.c_double, _D, _D]
        _lib.oracle_scalar_bezier3.restype = C.c_double
    return _lib


def _p(a):
    return a.ctypes.data_as(_D)


class _Keep:
    """Holds numpy arrays alive while ctypes structs point into them."""

    def __init__(self):
        self.arrays = []

    def f64(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        self.arrays.append(a)
        return a


def make_lines(line_const, zeeman, zeeman_n, vmicro_char, magneto_optical, moving,
               keep: _Keep, no_stokes: bool = False) -> OracleLines:
    lc = keep.f64(line_const)
    zm = keep.f64(zeeman)
    zn = np.ascontiguousarray(zeeman_n, dtype=np.int32)
    keep.arrays.append(zn)
    L = OracleLines()
    L.nline = lc.shape[0]
    L.maxcomp = zm.shape[-1]
    L.magneto_optical = int(magneto_optical)
    L.moving = int(moving)
    L.no_stokes = int(no_stokes)
    L.vmicro_char = float(vmicro_char)
    L.c = _p(lc)
    L.zeeman = _p(zm)
    L.ncomp = zn.ctypes.data_as(_I)
    return L


def make_atmos(fx: dict, keep: _Keep, mu=None) -> OracleAtmos:
    A = OracleAtmos()
    A.ndep = len(fx["T"])
    A.muz = float(fx["mu"] if mu is None else mu)
    for n in ("height", "T", "ne", "nHtot", "np", "vturb", "vel", "B", "gamma_B",
              "chi_B", "line_pops"):
        setattr(A, n, _p(keep.f64(fx[n])))
    return A


def lte_synth(fx: dict, md_float: bool = True, lam=None, chi_c=None, eta_c=None,
              magneto_optical=None, no_stokes: bool = False, mu=None):
    """Emergent [4][nlam] Stokes of one atmosphere given as a fixture dict with
    the keys written by tests/golden/make_golden.py."""
    keep = _Keep()
    A = make_atmos(fx, keep, mu=mu)
    mo = fx["magneto_optical"] if magneto_optical is None else magneto_optical
    L = make_lines(fx["line_const"], fx["zeeman"], fx["zeeman_n"], fx["vmicro_char"],
                   mo, fx["moving"], keep, no_stokes=no_stokes)
    lam = keep.f64(fx["lam"] if lam is None else lam)
    cc = keep.f64(fx["chi_c"] if chi_c is None else chi_c)
    ec = keep.f64(fx["eta_c"] if eta_c is None else eta_c)
    out = np.zeros((4, len(lam)))
    lib().oracle_lte_synth(C.byref(A), C.byref(L), len(lam), _p(lam), _p(cc), _p(ec),
                           int(md_float), _p(out))
    return out


def lte_synth_batch(batch: dict, nthreads: int, md_float: bool = True):
    """Threaded oracle over a batch dict whose per-atmosphere arrays carry a
    leading atmosphere axis (lam shared)."""
    keep = _Keep()
    natm = batch["T"].shape[0]

    def first(k):     # shared quantities may be stacked per atmosphere
        v = np.asarray(batch[k])
        return v[0] if v.ndim and v.shape[0] == natm and k in _STACKED else v

    atms = (OracleAtmos * natm)()
    for p in range(natm):
        fx = {k: batch[k][p] for k in ("height", "T", "ne", "nHtot", "np", "vturb",
                                        "vel", "B", "gamma_B", "chi_B", "line_pops")}
        fx["mu"] = float(first("mu"))
        atms[p] = make_atmos(fx, keep)
    L = make_lines(first("line_const"), first("zeeman"), first("zeeman_n"),
                   float(first("vmicro_char")), int(first("magneto_optical")),
                   int(first("moving")), keep)
    lam = keep.f64(first("lam"))
    cc = keep.f64(batch["chi_c"])
    ec = keep.f64(batch["eta_c"])
    out = np.zeros((natm, 4, len(lam)))
    lib().oracle_lte_synth_batch(natm, nthreads, atms, C.byref(L), len(lam), _p(lam),
                                 _p(cc), _p(ec), int(md_float), _p(out))
    return out


def lte_opacity(fx: dict, k: int, lam: float):
    keep = _Keep()
    A = make_atmos(fx, keep)
    L = make_lines(fx["line_const"], fx["zeeman"], fx["zeeman_n"], fx["vmicro_char"],
                   fx["magneto_optical"], fx["moving"], keep)
    chi = np.zeros(4); eta = np.zeros(4); chip = np.zeros(3)
    flags = lib().oracle_lte_opacity(C.byref(A), C.byref(L), int(k), C.c_double(lam),
                                     _p(chi), _p(eta), _p(chip))
    return flags, chi, eta, chip


def humlicek(a: float, v: float):
    H = C.c_double(); F = C.c_double()
    lib().oracle_humlicek(a, v, C.byref(H), C.byref(F))
    return H.value, F.value


def output_mask(lam: np.ndarray, lambda_ref: float) -> np.ndarray:
    """Indices of the spectrum that rhf1d() returns: every wavelength except
    the one equal to LAMBDA_REF (rh/rhf1d/pyrh_solveray.c:130-150)."""
    return np.nonzero(lam != lambda_ref)[0]


# ------------------------------------------------------------------ NLTE --

class NlteProblem(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("ndep", "nspect", "nrays", "nlevel", "nline",
                                       "ncont", "moving")] + \
        [(n, _D) for n in ("lambda_", "muz", "wmu", "height", "T", "vel", "vbroad", "chi_c",
                           "eta_c", "sca_c")] + [("bgline", _I)] + \
        [(n, _D) for n in ("nstar", "ntotal", "C", "lines", "adamp", "cont", "alpha")] + \
        [(n, C.c_int) for n in ("ng_delay", "ng_order", "ng_period", "isum", "nmax_iter")] + \
        [("iter_limit", C.c_double)]


def nlte_problem(fx: dict, keep: _Keep) -> NlteProblem:
    """NlteProblem from an nlte fixture dict (tests/golden/make_golden.py)."""
    P = NlteProblem()
    m = fx["meta"]
    P.nspect, P.ndep, P.nrays, P.nlevel, P.nline, P.ncont = (int(x) for x in m[:6])
    P.nmax_iter, P.ng_delay, P.ng_order, P.ng_period, P.isum = (int(x) for x in m[6:11])
    P.moving = int(m[12])
    P.iter_limit = float(fx["fmeta"][0])
    P.lambda_ = _p(keep.f64(fx["lambda"]))
    for k in ("muz", "wmu", "height", "T", "vel", "vbroad", "nstar", "ntotal", "C",
              "lines", "adamp", "alpha"):
        setattr(P, k, _p(keep.f64(fx[k])))
    P.cont = _p(keep.f64(fx["continua"]))
    bg = keep.f64(fx["background"])
    P.chi_c = _p(keep.f64(bg[0]))
    P.eta_c = _p(keep.f64(bg[1]))
    P.sca_c = _p(keep.f64(bg[2]))
    fl = np.ascontiguousarray(fx["bgflags"] & 3, dtype=np.int32)
    keep.arrays.append(fl)
    P.bgline = fl.ctypes.data_as(_I)
    return P


def nlte_J0(fx: dict) -> np.ndarray:
    """Mean intensity before the first iteration (zero when N_MAX_SCATTER = 0,
    which the fixtures use)."""
    if "J0" in fx:
        return fx["J0"]
    return np.zeros((len(fx["lambda"]), len(fx["T"])))


def _nlte_lib():
    L = lib()
    L.oracle_voigt_armstrong.restype = C.c_double
    L.oracle_voigt_armstrong.argtypes = [C.c_double, C.c_double]
    L.oracle_nlte_iterate.restype = C.c_int
    L.oracle_nlte_iterate_rates.restype = C.c_int
    L.oracle_stat_equil.restype = C.c_int
    return L


def _split_rates(fx: dict, R: np.ndarray) -> dict:
    nline, ncont, nd = len(fx["lines"]), len(fx["continua"]), len(fx["T"])
    R = R.reshape(nline + ncont, 2, nd)
    return {"lines": R[:nline], "continua": R[nline:]}


def voigt_armstrong(a, v):
    return _nlte_lib().oracle_voigt_armstrong(a, v)


def nlte_profiles(fx: dict, nrays=None, muz=None, wmu=None):
    """phi per line ([Nlambda, 2*nrays, ndep]) and wphi [nline, ndep]."""
    keep = _Keep()
    P = nlte_problem(fx, keep)
    muz = keep.f64(fx["muz"] if muz is None else muz)
    wmu = keep.f64(fx["wmu"] if wmu is None else wmu)
    nrays = len(muz)
    phis = [np.zeros((int(l[8]), 2 * nrays, P.ndep)) for l in fx["lines"]]
    arr = (_D * max(len(phis), 1))(*[_p(x) for x in phis])
    wphi = np.zeros((P.nline, P.ndep))
    _nlte_lib().oracle_nlte_profiles(C.byref(P), nrays, _p(muz), _p(wmu), arr, _p(wphi))
    return phis, wphi


def nlte_first_iteration(fx: dict, rates: bool = False):
    """Gamma and J after one formal pass with the starting populations and
    J, and the populations after one statEquil (no acceleration); with
    rates, also that pass's radiative rates {"lines": [nline, 2, ndep],
    "continua": [ncont, 2, ndep]} (R_ij, R_ji)."""
    keep = _Keep()
    P = nlte_problem(fx, keep)
    phis, wphi = nlte_profiles(fx)
    arr = (_D * max(len(phis), 1))(*[_p(x) for x in phis])
    n = np.array(fx["n0"], dtype=np.float64, order="C")
    J0 = keep.f64(nlte_J0(fx))
    J = np.zeros_like(J0)
    G = np.zeros((P.nlevel * P.nlevel, P.ndep))
    L = _nlte_lib()
    R = np.zeros(2 * (P.nline + P.ncont) * P.ndep)
    L.oracle_nlte_spectrum_rates(C.byref(P), _p(n), _p(J0), _p(J), _p(G), arr, _p(wphi),
                                 _p(R))
    n1 = n.copy()
    L.oracle_stat_equil(C.byref(P), _p(G), _p(n1))
    return (G, J, n1, _split_rates(fx, R)) if rates else (G, J, n1)


def nlte_solve(fx: dict, rates: bool = False):
    """Converged populations, final J, iteration count and dpops history;
    with rates, also the radiative rates of the last formal pass (as
    nlte_first_iteration gives them)."""
    keep = _Keep()
    P = nlte_problem(fx, keep)
    n = np.array(fx["n0"], dtype=np.float64, order="C")
    J = np.array(nlte_J0(fx), dtype=np.float64, order="C")
    dp = np.zeros(P.nmax_iter)
    acc = np.zeros(P.nmax_iter, dtype=np.int32)
    R = np.zeros(2 * (P.nline + P.ncont) * P.ndep)
    it = _nlte_lib().oracle_nlte_iterate_rates(C.byref(P), _p(n), _p(J), _p(dp),
                                               acc.ctypes.data_as(_I), _p(R))
    if rates:
        return n, J, it, dp[:it], acc[:it], _split_rates(fx, R)
    return n, J, it, dp[:it], acc[:it]


def nlte_emergent(fx: dict, n, J, mu_out=None):
    keep = _Keep()
    P = nlte_problem(fx, keep)
    n = keep.f64(n)
    J = keep.f64(J)
    out = np.zeros(P.nspect)
    mu = float(fx["fmeta"][2] if mu_out is None else mu_out)
    _nlte_lib().oracle_nlte_emergent(C.byref(P), C.c_double(mu), _p(n), _p(J), _p(out))
    return out
