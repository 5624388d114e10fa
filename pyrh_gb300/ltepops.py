"""Element tables, LTE stage populations and the electron density through
the C ABI (elements_host.cpp, ltepops.cu).

    tab = element_tables(abundance_text, pf_bytes)            # host, numpy
    dev = DeviceTables(tab)                                   # device copy
    lp  = line_pops(dev, T, ne, nHtot, elem, stage)           # [nline, 2, npoint]
    ne  = solve_ne(dev, T, nHtot)                             # Solve_ne from scratch
    ne_cgs = get_ne_from_nH(cwd, atm_scale, scale, temperature, nH)   # pyrh's call

What the reference reads in readAbundance (rh/abundance.c:72-220) and
computes in LTEpops_elem (rh/ltepops.c:116-166), rlk_opacity's stage
densities (rh/kurucz.c:662-677) and Solve_ne (rh/solvene.c:55-198).
`line_pops` gives pyrh_lte_batch's line_pops input (and compute1d's
LteSetup.line_pops) from the atmosphere alone.  Elements are indexed by
atomic number - 1.  Device arrays are torch tensors (float64, one value per
depth point); the kernels run on the current CUDA stream.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import _lib as L

NELEM = 99
MAX_STAGES = 8
CM_TO_M = 1.0e-2


class ElemTables(C.Structure):
    _fields_ = [("nelem", C.c_int32), ("npf", C.c_int32), ("Tpf", C.c_void_p),
                ("abund", C.c_void_p), ("nstage", C.c_void_p), ("stage_off", C.c_void_p),
                ("lnpf", C.c_void_p), ("ionpot", C.c_void_p)]


_P = C.POINTER


def _lib():
    lib = L.lib()
    lib.pyrh_abundance_parse.restype = C.c_int
    lib.pyrh_abundance_parse.argtypes = [C.c_char_p, C.c_int32, _P(C.c_int32), _P(C.c_double),
                                         C.c_double, _P(C.c_double), _P(C.c_int32)]
    lib.pyrh_pf_parse.restype = C.c_int
    lib.pyrh_pf_parse.argtypes = [C.c_char_p, C.c_size_t, _P(C.c_int32), _P(C.c_int32),
                                  _P(C.c_int32), _P(C.c_double), _P(C.c_int32), _P(C.c_int32),
                                  _P(C.c_double), _P(C.c_double)]
    lib.pyrh_lte_stage_pops.restype = C.c_int
    lib.pyrh_lte_stage_pops.argtypes = [C.POINTER(ElemTables), C.c_int64, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_int32, _P(C.c_int32),
                                        C.c_void_p, C.c_void_p]
    lib.pyrh_line_pops.restype = C.c_int
    lib.pyrh_line_pops.argtypes = [C.POINTER(ElemTables), C.c_int64, C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_int32, _P(C.c_int32), _P(C.c_int32),
                                   C.c_void_p, C.c_void_p]
    lib.pyrh_solve_ne.restype = C.c_int
    lib.pyrh_solve_ne.argtypes = [C.POINTER(ElemTables), C.c_int64, C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]
    return lib


def _i32(a):
    return a.ctypes.data_as(_P(C.c_int32))


def _f64(a):
    return a.ctypes.data_as(_P(C.c_double))


def read_abundance(text: str, atomic_number=None, atomic_abundance=None,
                   metallicity: float = 0.0):
    """(abund [99], abundance_set [99]) from an abundance file's text.
    atomic_number / atomic_abundance replace the value of the n-th record of
    the file (1-based), as compute1d's arguments of the same name do."""
    ids = np.ascontiguousarray([] if atomic_number is None else atomic_number, np.int32)
    vals = np.ascontiguousarray([] if atomic_abundance is None else atomic_abundance, np.float64)
    if ids.shape != vals.shape:
        raise ValueError("atomic_number and atomic_abundance differ in length")
    abund = np.zeros(NELEM)
    aset = np.zeros(NELEM, np.int32)
    L.check(_lib().pyrh_abundance_parse(text.encode(), len(ids), _i32(ids), _f64(vals),
                                        float(metallicity), _f64(abund), _i32(aset)))
    return abund, aset


@dataclass
class ElementTables:
    """Host copy of the element tables (the layout of pyrh_elem_tables)."""
    Tpf: np.ndarray          # [npf] K
    abund: np.ndarray        # [99]
    abundance_set: np.ndarray
    nstage: np.ndarray       # [99] int32
    stage_off: np.ndarray    # [99] int32
    lnpf: np.ndarray         # [sum nstage, npf]
    ionpot: np.ndarray       # [sum nstage] J

    def stage_rows(self, elem: int) -> slice:
        o = int(self.stage_off[elem])
        return slice(o, o + int(self.nstage[elem]))


def read_pf(data: bytes, abundance_set) -> tuple:
    """(Tpf, nstage, stage_off, lnpf, ionpot) from the bytes of a Kurucz
    partition-function file; ln U and J for elements with abundance_set."""
    lib = _lib()
    aset = np.ascontiguousarray(abundance_set, np.int32)
    npf, nrows = C.c_int32(), C.c_int32()
    L.check(lib.pyrh_pf_parse(data, len(data), _i32(aset), C.byref(npf), C.byref(nrows),
                              None, None, None, None, None))
    Tpf = np.zeros(npf.value)
    nstage = np.zeros(NELEM, np.int32)
    off = np.zeros(NELEM, np.int32)
    lnpf = np.zeros((nrows.value, npf.value))
    ion = np.zeros(nrows.value)
    L.check(lib.pyrh_pf_parse(data, len(data), _i32(aset), C.byref(npf), C.byref(nrows),
                              _f64(Tpf), _i32(nstage), _i32(off), _f64(lnpf), _f64(ion)))
    return Tpf, nstage, off, lnpf, ion


def element_tables(abundance_text: str, pf_bytes: bytes, atomic_number=None,
                   atomic_abundance=None, metallicity: float = 0.0) -> ElementTables:
    abund, aset = read_abundance(abundance_text, atomic_number, atomic_abundance, metallicity)
    Tpf, nstage, off, lnpf, ion = read_pf(pf_bytes, aset)
    return ElementTables(Tpf, abund, aset, nstage, off, lnpf, ion)


def tables_from_files(cwd: str, atomic_number=None, atomic_abundance=None) -> ElementTables:
    """The tables the reference reads for a run in `cwd`: ABUND_FILE,
    KURUCZ_PF_DATA and METALLICITY of cwd/keyword.input, the files defaulting
    to $PYRH_PATH/rh/Atoms/abundance.input and pf_Kurucz.input as the
    reference's readInput sets them (rh/readinput.c:228-262)."""
    from .compute1d import read_keyword_input
    kw = read_keyword_input(os.path.join(str(cwd), "keyword.input"))
    root = os.path.join(os.environ.get("PYRH_PATH", ""), "rh", "Atoms")
    ab_path = kw.get("ABUND_FILE") or os.path.join(root, "abundance.input")
    pf_path = kw.get("KURUCZ_PF_DATA") or os.path.join(root, "pf_Kurucz.input")
    with open(ab_path) as f:
        ab_text = f.read()
    with open(pf_path, "rb") as f:
        pf = f.read()
    return element_tables(ab_text, pf, atomic_number, atomic_abundance,
                          float(kw.get("METALLICITY", "0.0")))


class DeviceTables:
    """The tables in device memory, with the pyrh_elem_tables that points at
    them."""

    def __init__(self, tab: ElementTables, device="cuda"):
        import torch
        self.host = tab
        t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dt)).to(device)
        self.t = {"Tpf": t(tab.Tpf, np.float64), "abund": t(tab.abund, np.float64),
                  "nstage": t(tab.nstage, np.int32), "stage_off": t(tab.stage_off, np.int32),
                  "lnpf": t(tab.lnpf, np.float64), "ionpot": t(tab.ionpot, np.float64)}
        s = ElemTables()
        s.nelem = NELEM
        s.npf = len(tab.Tpf)
        for k, v in self.t.items():
            setattr(s, k, v.data_ptr())
        self.struct = s
        self.device = device


def _dev(x, device):
    import torch
    x = torch.as_tensor(x, dtype=torch.float64, device=device)
    return x.contiguous()


def _stream():
    import torch
    return torch.cuda.current_stream().cuda_stream


def stage_pops(dev: DeviceTables, T, ne, nHtot, elements):
    """LTEpops_elem of each listed element: [sum of their nstage, npoint]."""
    import torch
    T, ne, nHtot = (_dev(x, dev.device) for x in (T, ne, nHtot))
    sel = np.ascontiguousarray(elements, np.int32)
    if np.any((sel < 0) | (sel >= NELEM)):
        raise ValueError("element index outside 0..98")
    rows = int(sum(dev.host.nstage[e] for e in sel))
    out = torch.zeros((rows, T.numel()), dtype=torch.float64, device=dev.device)
    L.check(_lib().pyrh_lte_stage_pops(C.byref(dev.struct), T.numel(), T.data_ptr(),
                                       ne.data_ptr(), nHtot.data_ptr(), len(sel), _i32(sel),
                                       out.data_ptr(), _stream()))
    return out


def line_pops(dev: DeviceTables, T, ne, nHtot, elem, stage):
    """[nline, 2, npoint]: the stage density and ln U of each line's element
    and stage (pyrh_lte_batch.line_pops)."""
    import torch
    T, ne, nHtot = (_dev(x, dev.device) for x in (T, ne, nHtot))
    el = np.ascontiguousarray(elem, np.int32)
    st = np.ascontiguousarray(stage, np.int32)
    if el.shape != st.shape:
        raise ValueError("elem and stage differ in length")
    out = torch.zeros((len(el), 2, T.numel()), dtype=torch.float64, device=dev.device)
    L.check(_lib().pyrh_line_pops(C.byref(dev.struct), T.numel(), T.data_ptr(), ne.data_ptr(),
                                  nHtot.data_ptr(), len(el), _i32(el), _i32(st), out.data_ptr(),
                                  _stream()))
    return out


def solve_ne(dev: DeviceTables, T, nHtot, ne_start=None, return_iterations=False,
             unit_hydrogen_pf=False):
    """Solve_ne: from hydrogen's ionisation (ne_start None) or from ne_start.
    With unit_hydrogen_pf the start takes hydrogen's partition function as 1,
    as the hydrostatic equilibrium's get_ne does."""
    import torch
    T, nHtot = _dev(T, dev.device), _dev(nHtot, dev.device)
    if ne_start is None:
        ne = torch.zeros_like(T)
    else:
        ne = _dev(ne_start, dev.device).clone()
    it = torch.zeros(T.numel(), dtype=torch.int32, device=dev.device)
    L.check(_lib().pyrh_solve_ne(C.byref(dev.struct), T.numel(), T.data_ptr(), nHtot.data_ptr(),
                                 ne.data_ptr(), 0 if ne_start is not None else
                                 (2 if unit_hydrogen_pf else 1), it.data_ptr(),
                                 _stream()))
    return (ne, it) if return_iterations else ne


def get_ne_from_nH(cwd, atm_scale, scale, temperature, nH, tables: ElementTables | None = None,
                   device="cuda"):
    """pyrh.get_ne_from_nH (pyrh.pyx:396-423 -> rh/rhf1d/pyrh_hse.c:555-650):
    the electron density [cm^-3] of an atmosphere from its temperature [K]
    and hydrogen density nH [cm^-3], by Solve_ne from scratch with hydrogen in
    LTE.  The depth scale does not enter the result (the reference only
    stores it).  `tables` defaults to the files the run in cwd names."""
    if atm_scale not in (0, 1, 2):
        raise ValueError(f"atm_scale {atm_scale}")
    temperature = np.ascontiguousarray(temperature, np.float64)
    nH = np.ascontiguousarray(nH, np.float64)
    if np.shape(scale) != temperature.shape or nH.shape != temperature.shape:
        raise ValueError("scale, temperature and nH differ in length")
    tab = tables if tables is not None else tables_from_files(cwd)
    dev = DeviceTables(tab, device)
    cube = CM_TO_M * CM_TO_M * CM_TO_M          # CUBE(CM_TO_M) of the reference
    ne = solve_ne(dev, temperature, nH / cube)
    return ne.cpu().numpy() * cube
