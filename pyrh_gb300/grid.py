"""Host-side set-up through the C ABI (setup_host.cpp): the RH model atom,
the wavelength grids of its transitions, the global wavelength grid and the
output index.

    atom = read_atom(text)                     # pyrh_atom_read (readatom.c)
    g = nlte_grid(atom, wave, lambda_ref=500.0, vmicro_char_kms=5.0)
    g.lam, g.line_range, g.cont_range, g.alpha, g.out_index

nlte_grid() returns what the NLTE batch takes from the reference's
SortLambda (rh/sortlambda.c:42-420): the sorted, de-duplicated spectrum,
each transition's first index and point count on it (continua and lines in
the atom's order), the hydrogenic cross-sections on each continuum's range,
and the indices of the output wavelengths (lambda_ref dropped,
rh/rhf1d/pyrh_solveray.c:115-156).  lte_grid() does the same for a
synthesis without active atoms: the caller's wavelengths plus lambda_ref.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L

MAX_LEVELS, MAX_LINES, MAX_CONT, MAX_COMPONENTS = 64, 128, 64, 8
MAX_TABLE, MAX_COLL, MAX_COLLVALS, LABEL = 4096, 512, 8192, 20


class AtomLevel(C.Structure):
    _fields_ = [("E", C.c_double), ("E_cm", C.c_double), ("g", C.c_double),
                ("stage", C.c_int32), ("abo_level", C.c_int32), ("label", C.c_char * (LABEL + 4))]


class AtomLine(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("i", "j", "nlambda", "symmetric", "voigt", "prd",
                                         "vdwaals", "ncomponent")] + \
        [(n, C.c_double) for n in ("f", "lambda0", "Aji", "Bji", "Bij", "qcore", "qwing")] + \
        [("cvdw", C.c_double * 4), ("Grad", C.c_double), ("cStark", C.c_double),
         ("g_lande_eff", C.c_double), ("c_shift", C.c_double * MAX_COMPONENTS),
         ("c_fraction", C.c_double * MAX_COMPONENTS)]


class AtomCont(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("i", "j", "nlambda", "hydrogenic")] + \
        [(n, C.c_double) for n in ("alpha0", "lambda0", "lambda_min")] + \
        [("table_off", C.c_int64)]


class AtomColl(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("type", "i", "j", "ntemp", "temp_off", "value_off")]


class Atom(C.Structure):
    _fields_ = [("id", C.c_char * 4)] + \
        [(n, C.c_int32) for n in ("nlevel", "nline", "ncont", "nfixed", "ntable", "ncoll",
                                  "ncoll_values")] + \
        [("level", AtomLevel * MAX_LEVELS), ("line", AtomLine * MAX_LINES),
         ("cont", AtomCont * MAX_CONT), ("table_lambda", C.c_double * MAX_TABLE),
         ("table_alpha", C.c_double * MAX_TABLE), ("coll", AtomColl * MAX_COLL),
         ("coll_values", C.c_double * MAX_COLLVALS)]


class GridConfig(C.Structure):
    _fields_ = [("vmicro_char", C.c_double), ("B_char", C.c_double), ("moving", C.c_int32),
                ("stokes", C.c_int32)]


_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int32)


def _lib():
    lib = L.lib()
    lib.pyrh_atom_read.restype = C.c_int
    lib.pyrh_atom_read.argtypes = [C.c_char_p, C.POINTER(Atom)]
    lib.pyrh_line_grid.restype = C.c_int32
    lib.pyrh_line_grid.argtypes = [C.POINTER(Atom), C.c_int32, C.POINTER(GridConfig), _D,
                                   C.c_int32]
    lib.pyrh_cont_grid.restype = C.c_int32
    lib.pyrh_cont_grid.argtypes = [C.POINTER(Atom), C.c_int32, _D, C.c_int32]
    lib.pyrh_sort_lambda.restype = C.c_int
    lib.pyrh_sort_lambda.argtypes = [_D, C.c_int32, C.c_double, _D, _I, C.c_int32, _D,
                                     C.c_int32, _I, _I, _I, _I]
    lib.pyrh_output_index.restype = C.c_int
    lib.pyrh_output_index.argtypes = [_D, C.c_int32, C.c_double, _I, _I]
    lib.pyrh_cont_alpha.restype = C.c_int
    lib.pyrh_cont_alpha.argtypes = [C.POINTER(Atom), C.c_int32, _D, C.c_int32, _D]
    lib.pyrh_atom_lande_eff.restype = C.c_double
    lib.pyrh_atom_lande_eff.argtypes = [C.POINTER(Atom), C.c_int32]
    lib.pyrh_atom_line_polarizable.restype = C.c_int32
    lib.pyrh_atom_line_polarizable.argtypes = [C.POINTER(Atom), C.c_int32, C.c_int32]
    return lib


def _d(a):
    return a.ctypes.data_as(_D)


def _i(a):
    return a.ctypes.data_as(_I)


def read_atom(text: str) -> Atom:
    """An RH .atom file's text parsed by pyrh_atom_read."""
    atom = Atom()
    L.check(_lib().pyrh_atom_read(text.encode(), C.byref(atom)))
    return atom


def line_polarized(atom: Atom, kr: int, field_free: bool = False) -> bool:
    """Whether line kr of an active atom makes the wavelengths it covers
    angle dependent in the NLTE formal solution (the `polarized` field of
    pyrh_nlte_transition): polarizable (readatom.c:347-366, with
    atmos.Stokes, which pyrh always sets, pyrh_compute1dray.c:85) under a
    STOKES_MODE other than FIELD_FREE (containsPolarized,
    opacity.c:574-589)."""
    pol = _lib().pyrh_atom_line_polarizable(C.byref(atom), int(kr), 1)
    if pol < 0:
        raise ValueError(f"line {kr}: composite line with polarization")
    return bool(pol) and not field_free


@dataclass
class Grid:
    lam: np.ndarray          # [nspect] vacuum nm, ascending, unique
    wave_inds: np.ndarray    # [nwave] index of each caller wavelength
    line_range: np.ndarray   # [nline, 2] (nblue, nlambda)
    cont_range: np.ndarray   # [ncont, 2]
    alpha: list              # per continuum, cross-sections on its range [m^2]
    out_index: np.ndarray    # output wavelengths (lambda_ref dropped)


def _sort(wave, lambda_ref, grids):
    wave = np.ascontiguousarray(wave, np.float64)
    gn = np.array([len(g) for g in grids], np.int32)
    cat = np.ascontiguousarray(np.concatenate(grids) if grids else np.zeros(1), np.float64)
    cap = len(wave) + int(gn.sum()) + 1
    lam = np.zeros(cap)
    ns = np.zeros(1, np.int32)
    wi = np.zeros(max(len(wave), 1), np.int32)
    nb = np.zeros(max(len(grids), 1), np.int32)
    nl = np.zeros(max(len(grids), 1), np.int32)
    L.check(_lib().pyrh_sort_lambda(_d(wave), len(wave), float(lambda_ref), _d(cat), _i(gn),
                                    len(grids), _d(lam), cap, _i(ns), _i(wi), _i(nb), _i(nl)))
    n = int(ns[0])
    lam = lam[:n].copy()
    idx = np.zeros(n, np.int32)
    nout = np.zeros(1, np.int32)
    L.check(_lib().pyrh_output_index(_d(lam), n, float(lambda_ref), _i(idx), _i(nout)))
    return lam, wi[:len(wave)], nb[:len(grids)], nl[:len(grids)], idx[:int(nout[0])]


def nlte_grid(atom: Atom, wave, lambda_ref: float = 500.0, vmicro_char_kms: float = 5.0,
              B_char: float = 0.0, moving: bool = True, stokes: bool = True) -> Grid:
    lib = _lib()
    cfg = GridConfig(vmicro_char_kms * 1e3, B_char, int(moving), int(stokes))
    grids = []
    for kr in range(atom.ncont):
        n = lib.pyrh_cont_grid(C.byref(atom), kr, None, 0)
        g = np.zeros(max(n, 1))
        if n < 0 or lib.pyrh_cont_grid(C.byref(atom), kr, _d(g), n) != n:
            raise RuntimeError(L.lib().pyrh_last_error().decode())
        grids.append(g)
    for kr in range(atom.nline):
        n = lib.pyrh_line_grid(C.byref(atom), kr, C.byref(cfg), None, 0)
        g = np.zeros(max(n, 1))
        if n < 0 or lib.pyrh_line_grid(C.byref(atom), kr, C.byref(cfg), _d(g), n) != n:
            raise RuntimeError(L.lib().pyrh_last_error().decode())
        grids.append(g)
    lam, wi, nb, nl, idx = _sort(wave, lambda_ref, grids)
    nc = atom.ncont
    cont = np.stack([nb[:nc], nl[:nc]], axis=1) if nc else np.zeros((0, 2), np.int32)
    line = np.stack([nb[nc:], nl[nc:]], axis=1) if atom.nline else np.zeros((0, 2), np.int32)
    alpha = []
    for kr in range(nc):
        b, n = int(cont[kr, 0]), int(cont[kr, 1])
        a = np.zeros(n)
        seg = np.ascontiguousarray(lam[b:b + n])
        if atom.cont[kr].hydrogenic:
            L.check(lib.pyrh_cont_alpha(C.byref(atom), kr, _d(seg), n, _d(a)))
        else:
            c = atom.cont[kr]
            tl = np.array(atom.table_lambda[c.table_off:c.table_off + c.nlambda])
            ta = np.array(atom.table_alpha[c.table_off:c.table_off + c.nlambda])
            a = np.interp(seg, tl, ta)     # the reference's spline is not restated
        alpha.append(a)
    return Grid(lam, wi, line, cont, alpha, idx)


def lte_grid(wave, lambda_ref: float = 500.0) -> Grid:
    """Grid of a synthesis without active atoms: the caller's wavelengths
    and lambda_ref, sorted and de-duplicated."""
    lam, wi, _, _, idx = _sort(wave, lambda_ref, [])
    z = np.zeros((0, 2), np.int32)
    return Grid(lam, wi, z, z, [], idx)
