"""Chemical equilibrium through the C ABI (pyrh_molecule_read in
elements_host.cpp, pyrh_chem_equil in chem.cu): the reference's readMolecule
(rh/readmolecule.c:66-240) and ChemicalEquilibrium (rh/chemequil.c:107-390)
on the device, one thread per depth point.

    mols = [read_molecule(text, tables.abundance_set) for text in molecule_files]
    nmol, nHmin, nnuc, niter = chem_equil(DeviceTables(tables), mols, T, ne, nHtot,
                                          fn0_model={0: fn0_H, ...})

fn0_model maps an element index (atomic number - 1) to the neutral fraction
of its atom model's LTE populations at every point (what the reference takes
for nuclei with a model); the other nuclei take theirs from the element
tables' partition functions.  Returns torch tensors on the tables' device:
molecule densities [nmol, npoint], the H- density [npoint], the nuclei's
atomic densities afterwards [nnuclei, npoint] (nuclei = the elements bound in
some molecule, in element order) and the steps taken (-1: not converged).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from . import ltepops as LP

MAX_ELEMENTS = 4
MAX_COEF = 12
MAX_MOLECULES = 24
FITS = ("KURUCZ_70", "KURUCZ_85", "SAUVAL_TATUM_84", "IRWIN_81", "TSUJI_73")


class Molecule(C.Structure):
    _fields_ = [("id", C.c_char * 16), ("charge", C.c_int32), ("nelement", C.c_int32),
                ("pt_index", C.c_int32 * MAX_ELEMENTS), ("pt_count", C.c_int32 * MAX_ELEMENTS),
                ("nnuclei", C.c_int32), ("fit", C.c_int32), ("ediss", C.c_double),
                ("tmin", C.c_double), ("tmax", C.c_double), ("npf", C.c_int32),
                ("neqc", C.c_int32), ("pf_coef", C.c_double * MAX_COEF),
                ("eqc_coef", C.c_double * MAX_COEF)]


def _lib():
    lib = L.lib()
    lib.pyrh_molecule_read.restype = C.c_int
    lib.pyrh_molecule_read.argtypes = [C.c_char_p, C.POINTER(C.c_int32), C.POINTER(Molecule)]
    lib.pyrh_chem_equil.restype = C.c_int
    lib.pyrh_chem_equil.argtypes = [C.POINTER(LP.ElemTables), C.POINTER(Molecule), C.c_int32,
                                    C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.POINTER(C.c_void_p), C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.c_void_p]
    return lib


def read_molecule(text: str, abundance_set) -> Molecule:
    aset = np.ascontiguousarray(abundance_set, np.int32)
    m = Molecule()
    L.check(_lib().pyrh_molecule_read(text.encode(), aset.ctypes.data_as(C.POINTER(C.c_int32)),
                                      C.byref(m)))
    return m


def nuclei_of(mols) -> list[int]:
    """The elements bound in some molecule, in element order."""
    return sorted({m.pt_index[j] for m in mols for j in range(m.nelement)})


def chem_equil(dev: LP.DeviceTables, mols, T, ne, nHtot, fn0_model=None):
    import torch
    T, ne, nHtot = (LP._dev(x, dev.device) for x in (T, ne, nHtot))
    npoint = T.numel()
    arr = (Molecule * len(mols))(*mols)
    keep = []
    ptrs = (C.c_void_p * LP.NELEM)()
    for e, v in (fn0_model or {}).items():
        t = LP._dev(v, dev.device)
        if t.numel() != npoint:
            raise ValueError(f"fn0 of element {e}: {t.numel()} values for {npoint} points")
        keep.append(t)
        ptrs[e] = t.data_ptr()
    nuc = nuclei_of(mols)
    nmol = torch.zeros((len(mols), npoint), dtype=torch.float64, device=dev.device)
    nHmin = torch.zeros(npoint, dtype=torch.float64, device=dev.device)
    nnuc = torch.zeros((len(nuc), npoint), dtype=torch.float64, device=dev.device)
    niter = torch.zeros(npoint, dtype=torch.int32, device=dev.device)
    L.check(_lib().pyrh_chem_equil(C.byref(dev.struct), arr, len(mols), npoint, T.data_ptr(),
                                   ne.data_ptr(), nHtot.data_ptr(), ptrs, nmol.data_ptr(),
                                   nHmin.data_ptr(), nnuc.data_ptr(), niter.data_ptr(),
                                   LP._stream()))
    return nmol, nHmin, nnuc, niter
