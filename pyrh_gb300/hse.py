"""Hydrostatic equilibrium on the GPU through the C ABI (pyrh_hse, hse.cu).

    model = equilibria.AtomsModel.from_cwd(cwd)        # the run's atoms, molecules, tables
    ne, nHtot, rho, pg = hse_batch(model, 0, logtau, T, pg_top)   # [natm, ndep] SI
    ne, nHtot = hse(cwd, 0, logtau, T)                 # pyrh.hse's call

pyrh's hse() (pyrh.pyx:427-487 -> rh/rhf1d/pyrh_hse.c:67-399) builds, from
the top layer down, the gas pressure, hydrogen and electron densities of an
atmosphere given its temperature on a log tau500 (atm_scale 0) or height
[km] (atm_scale 2) scale, with every atom and molecule in LTE and the
continuum opacity at 500 nm from the background without the metals'
continua.  Here a batch of atmospheres runs at once, one vector of
atmospheres per layer.  Results are in SI (m^-3, kg m^-3, Pa), as the
reference returns them.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from . import background as BG
from . import chem as CH
from . import equilibria as EQ
from . import ltepops as LP

NMAX_ITER = 50                                           # NMAX_HSE_ITER, pyrh_hse.c:61
ETA_LIMIT = 1.0e-2                                       # pyrh_hse.c:214, 337


class HseConfig(C.Structure):
    _fields_ = [("gravity", C.c_double), ("total_abund", C.c_double), ("wght_per_H", C.c_double),
                ("scale", C.c_int32), ("nmax_iter", C.c_int32), ("eta_limit", C.c_double)]


class HseBatch(C.Structure):
    _fields_ = [("natm", C.c_int32), ("ndep", C.c_int32)] + \
        [(n, C.c_void_p) for n in ("scale", "T", "pg_top", "ne", "nHtot", "rho", "pg", "opacity",
                                   "niter")]


def _lib():
    lib = L.lib()
    lib.pyrh_hse.restype = C.c_int
    lib.pyrh_hse.argtypes = [C.POINTER(LP.ElemTables), C.POINTER(CH.Molecule), C.c_int32,
                             C.POINTER(BG.BgModel), C.POINTER(EQ.PassiveAtoms),
                             C.POINTER(HseConfig), C.POINTER(HseBatch), C.c_void_p]
    return lib


def hse_batch(model: EQ.AtomsModel, atm_scale: int, scale, T, pg_top=0.1, fudge=None,
              opacity=False, iterations=False):
    """Hydrostatic equilibrium of natm atmospheres: scale and T [natm, ndep]
    (log10 tau500 or height [km]; K), pg_top [natm] or one value (Pa).
    Returns ne, nHtot [m^-3], rho [kg m^-3], pg [Pa], each [natm, ndep] (and
    the 500 nm opacity [m^-1] and the passes per layer on request).  fudge:
    (lambda [nm], values [3, n]) as hse's fudge_wave / fudge_value."""
    import torch
    if atm_scale not in (0, 2):
        raise ValueError("atm_scale must be 0 (log tau500) or 2 (height): the reference's "
                         "column-mass branch (1) leaves its pressure step unset")
    scale = np.atleast_2d(np.asarray(scale, np.float64))
    T = np.atleast_2d(np.asarray(T, np.float64))
    if scale.shape != T.shape:
        raise ValueError("scale and T differ in shape")
    natm, ndep = T.shape
    if natm < 1 or ndep < 1:
        raise ValueError(f"{natm} atmospheres of {ndep} layers")
    dev = model.dev_tables.device
    pg0 = np.array(np.broadcast_to(np.asarray(pg_top, np.float64), (natm,)))
    lay = lambda x: torch.from_numpy(np.ascontiguousarray(x.T)).to(dev)
    t = {"scale": lay(scale), "T": lay(T),
         "pg_top": torch.from_numpy(np.ascontiguousarray(pg0)).to(dev)}
    for k in ("ne", "nHtot", "rho", "pg", "opacity"):
        t[k] = torch.zeros((ndep, natm), dtype=torch.float64, device=dev)
    t["niter"] = torch.zeros((ndep, natm), dtype=torch.int32, device=dev)
    cfg = HseConfig(gravity=EQ.GRAVITY, total_abund=model.total_abund,
                    wght_per_H=model.wght_per_H, scale=atm_scale, nmax_iter=NMAX_ITER,
                    eta_limit=ETA_LIMIT)
    bg = model.background(hse=True, fudge=fudge)
    mols = (CH.Molecule * len(model.molecules))(*model.molecules)
    out = {k: [] for k in ("ne", "nHtot", "rho", "pg", "opacity", "niter")}
    for a0 in range(0, natm, 65535):
        a1 = min(natm, a0 + 65535)
        b = HseBatch()
        b.natm, b.ndep = a1 - a0, ndep
        sub = {k: (v[:, a0:a1].contiguous() if v.dim() == 2 else v[a0:a1].contiguous())
               for k, v in t.items()}
        for k, v in sub.items():
            setattr(b, k, v.data_ptr())
        L.check(_lib().pyrh_hse(C.byref(model.dev_tables.struct), mols, len(model.molecules),
                                C.byref(bg.m), C.byref(model.atoms), C.byref(cfg),
                                C.byref(b), LP._stream()))
        for k in out:
            out[k].append(sub[k].cpu().numpy().T)
    res = [np.concatenate(out[k], axis=0) for k in ("ne", "nHtot", "rho", "pg")]
    if opacity:
        res.append(np.concatenate(out["opacity"], axis=0))
    if iterations:
        res.append(np.concatenate(out["niter"], axis=0))
    return tuple(res)


def hse(cwd, atm_scale, scale, temp, pg_top=0.1, fudge_wave=None, fudge_value=None,
        atomic_number=None, atomic_abundance=None, full_output=False, model=None,
        device="cuda"):
    """pyrh.hse (pyrh.pyx:427-487): ne and nHtot [m^-3] of one atmosphere
    (and rho [kg m^-3], pg [Pa] with full_output).  `model` skips reading the
    run's files again."""
    fudge = None
    if fudge_wave is not None or fudge_value is not None:
        fudge = (np.asarray(fudge_wave, np.float64),
                 np.asarray(fudge_value, np.float64).reshape(3, -1))
    if model is None:
        if (atomic_number is None) != (atomic_abundance is None):
            atomic_number = atomic_abundance = None   # the reference reads neither then
        elif atomic_number is not None and len(atomic_number) != len(atomic_abundance):
            raise ValueError("different number of atomic_number and atomic_abundance")
        model = EQ.AtomsModel.from_cwd(cwd, atomic_number, atomic_abundance, device)
    ne, nH, rho, pg = (x[0] for x in hse_batch(model, atm_scale, scale, temp, pg_top, fudge))
    return (ne, nH, rho, pg) if full_output else (ne, nH)
