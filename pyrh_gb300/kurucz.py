"""Kurucz line lists through the C ABI (pyrh_kurucz_read,
pyrh_barklem_parse in setup_host.cpp): the reference's readKuruczLines /
RLKZeeman (rh/kurucz.c:121-430, 832-920) with its van der Waals
cross-sections (rh/barklem.c, rh/kurucz.c:985-1020).

    tables = barklem_tables({0: sp_text, 1: pd_text, 2: df_text})
    lines, n, extra = read_kurucz(text, elements, tables)
    line_const, zeeman, zeeman_n = line_tables(lines, n, extra)

`elements` maps an atomic number to (weight [amu], abundance relative to
hydrogen, number of stages, abundance set, ionisation potentials [J] of
the stages) -- what the reference reads from its abundance and
partition-function files; hydrogen (1) and helium (2) are required.
line_tables() returns the layout pyrh_gb300.lte.make_lines takes (and the
reference's set-up dump holds), so a list read here feeds the synthesis,
compute1d's LteSetup and the response functions directly.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L

MAX_STAGES = 4


class Element(C.Structure):
    _fields_ = [("weight", C.c_double), ("abund", C.c_double), ("nstage", C.c_int32),
                ("abundance_set", C.c_int32), ("ionpot", C.c_double * MAX_STAGES)]


class BarklemTable(C.Structure):
    _fields_ = [("n1", C.c_int32), ("n2", C.c_int32), ("neff1_0", C.c_double),
                ("neff2_0", C.c_double), ("cross", C.POINTER(C.c_double)),
                ("alpha", C.POINTER(C.c_double))]


class KuruczConfig(C.Structure):
    _fields_ = [("stokes", C.c_int32), ("ls_lande", C.c_int32),
                ("elements", C.POINTER(Element)), ("nelem", C.c_int32),
                ("barklem", C.POINTER(BarklemTable) * 3), ("nloggf", C.c_int32),
                ("loggf_ids", C.POINTER(C.c_int32)), ("loggf_values", C.POINTER(C.c_double))]


class KuruczExtra(C.Structure):
    _fields_ = [("pt_index", C.c_int32), ("stage", C.c_int32), ("gj", C.c_double),
                ("Ej", C.c_double), ("gL_i", C.c_double), ("gL_j", C.c_double)]


def _lib():
    lib = L.lib()
    lib.pyrh_kurucz_read.restype = C.c_int
    lib.pyrh_kurucz_read.argtypes = [C.c_char_p, C.POINTER(KuruczConfig), C.c_void_p,
                                     C.POINTER(KuruczExtra), C.c_int32, C.POINTER(C.c_int32)]
    lib.pyrh_barklem_parse.restype = C.c_int
    lib.pyrh_barklem_parse.argtypes = [C.c_char_p, C.c_int32, C.POINTER(C.c_double),
                                       C.POINTER(C.c_double), C.POINTER(BarklemTable)]
    return lib


class _Tables:
    """Barklem tables and the arrays behind them (kept alive together)."""

    def __init__(self):
        self.tables = {}
        self.arrays = []


def barklem_tables(texts: dict) -> _Tables:
    """Barklem tables from the reference's data files' text, by type
    (0 = s-p, 1 = p-d, 2 = d-f)."""
    out = _Tables()
    for t, text in texts.items():
        cross = np.zeros(21 * 18)
        alpha = np.zeros(21 * 18)
        tb = BarklemTable()
        L.check(_lib().pyrh_barklem_parse(text.encode(), int(t),
                                          cross.ctypes.data_as(C.POINTER(C.c_double)),
                                          alpha.ctypes.data_as(C.POINTER(C.c_double)),
                                          C.byref(tb)))
        out.arrays += [cross, alpha]
        out.tables[int(t)] = tb
    return out


def barklem_from_arrays(n1, n2, neff1_0, neff2_0, cross, alpha, tabs=None, t=0) -> _Tables:
    """A table given as arrays (row-major [n1][n2])."""
    tabs = tabs or _Tables()
    c = np.ascontiguousarray(cross, np.float64)
    a = np.ascontiguousarray(alpha, np.float64)
    tabs.arrays += [c, a]
    tabs.tables[int(t)] = BarklemTable(int(n1), int(n2), float(neff1_0), float(neff2_0),
                                       c.ctypes.data_as(C.POINTER(C.c_double)),
                                       a.ctypes.data_as(C.POINTER(C.c_double)))
    return tabs


def read_kurucz(text: str, elements: dict, tables: _Tables | None = None, stokes=True,
                ls_lande=False, loggf_ids=None, loggf_values=None, cap: int = 4096):
    """The list's pyrh_line records, their count and the extra fields."""
    nelem = max(max(elements), 2)
    els = (Element * nelem)()
    for z, (w, ab, ns, aset, ion) in elements.items():
        e = els[z - 1]
        e.weight, e.abund, e.nstage, e.abundance_set = float(w), float(ab), int(ns), int(aset)
        for s in range(min(len(ion), MAX_STAGES)):
            e.ionpot[s] = float(ion[s])
    cfg = KuruczConfig()
    cfg.stokes, cfg.ls_lande = int(stokes), int(ls_lande)
    cfg.elements = C.cast(els, C.POINTER(Element))
    cfg.nelem = nelem
    for t in range(3):
        if tables and t in tables.tables:
            cfg.barklem[t] = C.pointer(tables.tables[t])
    keep = []
    if loggf_ids is not None:
        ids = np.ascontiguousarray(loggf_ids, np.int32)
        vals = np.ascontiguousarray(loggf_values, np.float64)
        keep += [ids, vals]
        cfg.nloggf = len(ids)
        cfg.loggf_ids = ids.ctypes.data_as(C.POINTER(C.c_int32))
        cfg.loggf_values = vals.ctypes.data_as(C.POINTER(C.c_double))
    lines = (L.PyrhLine * cap)()
    extra = (KuruczExtra * cap)()
    n = C.c_int32(0)
    L.check(_lib().pyrh_kurucz_read(text.encode(), C.byref(cfg), C.cast(lines, C.c_void_p),
                                    extra, cap, C.byref(n)))
    return lines, int(n.value), extra


def line_tables(lines, n: int, extra):
    """(line_const [n, 24], zeeman [n, 3, maxcomp], zeeman_n [n]) in the
    layout of pyrh_gb300.lte.make_lines (the reference's set-up dump)."""
    maxc = max([lines[i].ncomp for i in range(n)] + [1])
    lc = np.zeros((n, 24))
    zm = np.zeros((n, 3, maxc))
    zn = np.zeros(n, np.int32)
    for i in range(n):
        ln, x = lines[i], extra[i]
        lc[i, :21] = [ln.lambda0, x.pt_index, x.stage, ln.gi, x.gj, ln.Ei, x.Ej, ln.Aji,
                      ln.Bji, ln.Bij, ln.Grad, ln.GStark, ln.GvdWaals, ln.vdwaals, ln.cross,
                      ln.alpha, ln.isotope_frac, ln.hyperfine_frac, ln.polarizable,
                      ln.weight, ln.contributes]
        lc[i, 21:23] = [x.gL_i, x.gL_j]
        zn[i] = ln.ncomp
        for c in range(ln.ncomp):
            zm[i, :, c] = [ln.comp_q[c], ln.comp_shift[c], ln.comp_strength[c]]
    return lc, zm, zn
