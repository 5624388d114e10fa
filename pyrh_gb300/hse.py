"""Hydrostatic equilibrium on the GPU through the C ABI (pyrh_hse, hse.cu).

    model = HseModel.from_cwd(cwd)                     # the run's atoms, molecules, tables
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
import math
import os
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from . import background as BG
from . import chem as CH
from . import grid as G
from . import ltepops as LP

MAX_ATOMS = 24
GRAVITY = math.exp(2.30258509299404568402 * 4.4) * 1.0e-2  # MULTIatmos: 10^4.4 cm s^-2 -> m s^-2
NMAX_ITER = 50                                           # NMAX_HSE_ITER, pyrh_hse.c:61
ETA_LIMIT = 1.0e-2                                       # pyrh_hse.c:214, 337


class HseAtoms(C.Structure):
    _fields_ = [("natom", C.c_int32), ("elem", C.c_int32 * MAX_ATOMS),
                ("lev_off", C.c_int32 * (MAX_ATOMS + 1)), ("E", C.c_void_p), ("g", C.c_void_p),
                ("stage", C.c_void_p)]


class HseConfig(C.Structure):
    _fields_ = [("gravity", C.c_double), ("total_abund", C.c_double), ("wght_per_H", C.c_double),
                ("scale", C.c_int32), ("nmax_iter", C.c_int32), ("eta_limit", C.c_double)]


class HseBatch(C.Structure):
    _fields_ = [("natm", C.c_int32), ("ndep", C.c_int32)] + \
        [(n, C.c_void_p) for n in ("scale", "T", "pg_top", "ne", "nHtot", "rho", "pg", "opacity",
                                   "niter")]


def _lib():
    lib = L.lib()
    lib.pyrh_abundance_totals.restype = C.c_int
    lib.pyrh_abundance_totals.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_double),
                                          C.POINTER(C.c_double)]
    lib.pyrh_element_index.restype = C.c_int32
    lib.pyrh_element_index.argtypes = [C.c_char_p]
    lib.pyrh_hse.restype = C.c_int
    lib.pyrh_hse.argtypes = [C.POINTER(LP.ElemTables), C.POINTER(CH.Molecule), C.c_int32,
                             C.POINTER(BG.BgModel), C.POINTER(HseAtoms), C.POINTER(HseConfig),
                             C.POINTER(HseBatch), C.c_void_p]
    return lib


def abundance_totals(tab: LP.ElementTables) -> tuple[float, float]:
    """(atmos.totalAbund, atmos.wght_per_H) of the element tables."""
    ab = np.ascontiguousarray(tab.abund, np.float64)
    aset = np.ascontiguousarray(tab.abundance_set, np.int32)
    t, w = C.c_double(), C.c_double()
    L.check(_lib().pyrh_abundance_totals(ab.ctypes.data, aset.ctypes.data, C.byref(t), C.byref(w)))
    return t.value, w.value


def element_index(atom: G.Atom) -> int:
    e = _lib().pyrh_element_index(bytes(atom.id))
    if e < 0:
        raise ValueError(f"atom {atom.id!r}: no element of that symbol")
    return e


def setup_from_atoms(atoms: list, elems: list[int], vmicro_char: float, mol_present) -> dict:
    """The atomic data the background model reads (the keys
    background.model_from_setup takes) from parsed model atoms, all passive;
    vmicro_char in m/s."""
    meta, lev, cont, tab, line = [], [], [], [], []
    for a in atoms:
        meta.append((a.nlevel, a.ncont, a.nline, 0))
        lev += [(a.level[i].E, a.level[i].g, a.level[i].stage) for i in range(a.nlevel)]
        for kr in range(a.ncont):
            c = a.cont[kr]
            off = len(tab)
            if c.hydrogenic:
                lmin = c.lambda_min
            else:
                rows = range(c.table_off, c.table_off + c.nlambda)
                tab += [(a.table_lambda[r], a.table_alpha[r]) for r in rows]
                lmin = a.table_lambda[c.table_off]
            cont.append((c.i, c.j, c.lambda0, lmin, c.hydrogenic, c.alpha0, c.nlambda, off))
        line += [(a.line[kr].i, a.line[kr].j, a.line[kr].lambda0, a.line[kr].qwing,
                  a.line[kr].Aji) for kr in range(a.nline)]
    he = elems.index(1) if 1 in elems else -1
    h = elems.index(0)
    return {"atoms_meta": np.array(meta, np.int32).reshape(-1, 4),
            "atoms_lev": np.array(lev, np.float64).reshape(-1, 3),
            "atoms_cont": np.array(cont, np.float64).reshape(-1, 8),
            "atoms_tab": np.array(tab, np.float64).reshape(-1, 2),
            "atoms_line": np.array(line, np.float64).reshape(-1, 5),
            "misc": np.array([vmicro_char, he, h, len(atoms)], np.float64),
            "mol_present": np.asarray(mol_present, np.int32)}


@dataclass
class HseModel:
    """Everything hse() reads besides the atmosphere, in device memory."""
    tables: LP.ElementTables
    dev_tables: LP.DeviceTables
    molecules: list
    background: BG.DeviceBackground
    atoms: HseAtoms
    config: HseConfig
    keep: tuple

    @classmethod
    def build(cls, tables: LP.ElementTables, atoms: list, molecules: list,
              vmicro_char: float = 5.0e3, fudge=None, device="cuda") -> "HseModel":
        """tables: element tables; atoms: parsed model atoms (pyrh_gb300.grid
        .read_atom), hydrogen among them; molecules: parsed molecules
        (pyrh_gb300.chem.read_molecule), H2 first; fudge: (lambda [nm],
        values [3, n]) as hse's fudge_wave / fudge_value."""
        import torch
        if not 0 < len(atoms) <= MAX_ATOMS:
            raise ValueError(f"{len(atoms)} atoms (1..{MAX_ATOMS})")
        elems = [element_index(a) for a in atoms]
        if 0 not in elems:
            raise ValueError("hydrogen's model atom is missing")
        ids = [bytes(m.id).split(b"\0")[0] for m in molecules]
        present = [x in ids for x in (b"H2", b"OH", b"CH")]
        s = setup_from_atoms(atoms, elems, vmicro_char, present)
        model = BG.model_from_setup(s, lte=True, metals=False)
        bg = BG.DeviceBackground(model, add_scatter=True, fudge=fudge, device=device)
        lev = s["atoms_lev"]
        E = torch.from_numpy(np.ascontiguousarray(lev[:, 0])).to(device)
        g = torch.from_numpy(np.ascontiguousarray(lev[:, 1])).to(device)
        st = torch.from_numpy(np.ascontiguousarray(lev[:, 2], np.int32)).to(device)
        A = HseAtoms()
        A.natom = len(atoms)
        off = np.concatenate([[0], np.cumsum([a.nlevel for a in atoms])])
        for m, e in enumerate(elems):
            A.elem[m] = e
        for m, o in enumerate(off):
            A.lev_off[m] = int(o)
        A.E, A.g, A.stage = E.data_ptr(), g.data_ptr(), st.data_ptr()
        total, wght = abundance_totals(tables)
        cfg = HseConfig(gravity=GRAVITY, total_abund=total, wght_per_H=wght, scale=0,
                        nmax_iter=NMAX_ITER, eta_limit=ETA_LIMIT)
        return cls(tables, LP.DeviceTables(tables, device), list(molecules), bg, A, cfg,
                   (E, g, st))

    @classmethod
    def from_cwd(cls, cwd, atomic_number=None, atomic_abundance=None, fudge=None,
                 device="cuda") -> "HseModel":
        """The model the reference reads for hse() in cwd: keyword.input's
        ATOMS_FILE and MOLECULES_FILE (relative to cwd), the atom and
        molecule files under $PYRH_PATH/rh/Atoms and rh/Molecules, the
        abundance and partition-function files, VMICRO_CHAR."""
        from .compute1d import read_keyword_input
        kw = read_keyword_input(os.path.join(str(cwd), "keyword.input"))
        root = os.environ.get("PYRH_PATH", "")
        tab = LP.tables_from_files(cwd, atomic_number, atomic_abundance)
        atoms = [G.read_atom(open(os.path.join(root, "rh", "Atoms", n)).read())
                 for n in _list_file(os.path.join(str(cwd), kw.get("ATOMS_FILE", "atoms.input")))]
        mols = [CH.read_molecule(open(os.path.join(root, "rh", "Molecules", n)).read(),
                                 tab.abundance_set)
                for n in _list_file(os.path.join(str(cwd),
                                                 kw.get("MOLECULES_FILE", "molecules.input")))]
        vmc = float(kw.get("VMICRO_CHAR", "0.0")) * 1.0e3
        return cls.build(tab, atoms, mols, vmc, fudge, device)


def _list_file(path: str) -> list[str]:
    """The file names of an atoms.input / molecules.input list (count line,
    then one 'file MODE POPULATIONS [pops file]' record per entry)."""
    with open(path) as f:
        recs = [ln.split() for ln in f if ln.strip() and not ln.lstrip().startswith("#")]
    n = int(recs[0][0])
    return [r[0] for r in recs[1:1 + n]]


def hse_batch(model: HseModel, atm_scale: int, scale, T, pg_top=0.1, opacity=False,
              iterations=False):
    """Hydrostatic equilibrium of natm atmospheres: scale and T [natm, ndep]
    (log10 tau500 or height [km]; K), pg_top [natm] or one value (Pa).
    Returns ne, nHtot [m^-3], rho [kg m^-3], pg [Pa], each [natm, ndep] (and
    the 500 nm opacity [m^-1] and the passes per layer on request)."""
    import torch
    if atm_scale not in (0, 2):
        raise ValueError("atm_scale must be 0 (log tau500) or 2 (height): the reference's "
                         "column-mass branch (1) leaves its pressure step unset")
    scale = np.atleast_2d(np.asarray(scale, np.float64))
    T = np.atleast_2d(np.asarray(T, np.float64))
    if scale.shape != T.shape:
        raise ValueError("scale and T differ in shape")
    natm, ndep = T.shape
    dev = model.dev_tables.device
    pg0 = np.broadcast_to(np.asarray(pg_top, np.float64), (natm,))
    lay = lambda x: torch.from_numpy(np.ascontiguousarray(x.T)).to(dev)
    t = {"scale": lay(scale), "T": lay(T),
         "pg_top": torch.from_numpy(np.ascontiguousarray(pg0)).to(dev)}
    for k in ("ne", "nHtot", "rho", "pg", "opacity"):
        t[k] = torch.zeros((ndep, natm), dtype=torch.float64, device=dev)
    t["niter"] = torch.zeros((ndep, natm), dtype=torch.int32, device=dev)
    cfg = HseConfig.from_buffer_copy(model.config)
    cfg.scale = atm_scale
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
                                C.byref(model.background.m), C.byref(model.atoms), C.byref(cfg),
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
    if model is None:
        fudge = None
        if fudge_wave is not None or fudge_value is not None:
            fudge = (np.asarray(fudge_wave, np.float64),
                     np.asarray(fudge_value, np.float64).reshape(3, -1))
        if (atomic_number is None) != (atomic_abundance is None):
            atomic_number = atomic_abundance = None   # the reference reads neither then
        elif atomic_number is not None and len(atomic_number) != len(atomic_abundance):
            raise ValueError("different number of atomic_number and atomic_abundance")
        model = HseModel.from_cwd(cwd, atomic_number, atomic_abundance, fudge, device)
    ne, nH, rho, pg = (x[0] for x in hse_batch(model, atm_scale, scale, temp, pg_top))
    return (ne, nH, rho, pg) if full_output else (ne, nH)
