"""The run's passive atoms, molecules and element tables on the GPU, and the
per-depth set-up built from them through the C ABI (hse.cu, chem.cu,
ltepops.cu, background.cu):

    model = AtomsModel.from_cwd(cwd)                  # atoms.input, molecules.input, tables
    pops, nmol, nHmin = equilibria(model, T, ne, nHtot)            # LTE pops + chemistry
    chi_c, eta_c, np_ = continuum(model, lam, T, ne, nHtot)        # Background() of a run
    tau, cmass, height = convert_scales(model, 0, logtau, T, ne, nHtot, chi_ref)
    tau, height, cmass = get_scales(cwd, 0, scale, atmosphere, 500.0)   # pyrh's call

The reference does this inside Background() (rh/background.c:155-460 with
SOLVE_NE NONE: SetLTEQuantities, ChemicalEquilibrium, the continuum
opacities) and convertScales (rh/rhf1d/multiatmos.c:100-177); pyrh's
get_scales (pyrh.pyx:491-533 -> rh/rhf1d/pyrh_hse.c:402-554) runs them at
one reference wavelength.  All atoms are passive (LTE), as the runs these
functions serve read them.  Arrays are SI (m^-3, m, kg m^-2) unless a
function says otherwise.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from . import background as BG
from . import chem as CH
from . import grid as G
from . import ltepops as LP

MAX_ATOMS = 24
GRAVITY = math.exp(2.30258509299404568402 * 4.4) * 1.0e-2  # MULTIatmos: 10^4.4 cm s^-2 -> m s^-2


class PassiveAtoms(C.Structure):
    _fields_ = [("natom", C.c_int32), ("elem", C.c_int32 * MAX_ATOMS),
                ("lev_off", C.c_int32 * (MAX_ATOMS + 1)), ("E", C.c_void_p), ("g", C.c_void_p),
                ("stage", C.c_void_p)]


class ScalesBatch(C.Structure):
    _fields_ = [("natm", C.c_int32), ("ndep", C.c_int32), ("scale", C.c_int32),
                ("gravity", C.c_double), ("total_abund", C.c_double), ("wght_per_H", C.c_double)] + \
        [(n, C.c_void_p) for n in ("scale_in", "T", "ne", "nHtot", "chi_ref", "tau_ref", "cmass",
                                   "height")]


def _lib():
    lib = L.lib()
    lib.pyrh_abundance_totals.restype = C.c_int
    lib.pyrh_abundance_totals.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_double),
                                          C.POINTER(C.c_double)]
    lib.pyrh_element_index.restype = C.c_int32
    lib.pyrh_element_index.argtypes = [C.c_char_p]
    lib.pyrh_equilibria.restype = C.c_int
    lib.pyrh_equilibria.argtypes = [C.POINTER(LP.ElemTables), C.POINTER(CH.Molecule), C.c_int32,
                                    C.POINTER(PassiveAtoms), C.c_int64] + [C.c_void_p] * 7
    lib.pyrh_convert_scales.restype = C.c_int
    lib.pyrh_convert_scales.argtypes = [C.POINTER(ScalesBatch), C.c_void_p]
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


def list_file(path: str) -> list[tuple[str, str]]:
    """(file, mode) of each entry of an atoms.input / molecules.input list
    (count line, then one 'file MODE POPULATIONS [pops file]' record per
    entry)."""
    with open(path) as f:
        recs = [ln.split() for ln in f if ln.strip() and not ln.lstrip().startswith("#")]
    n = int(recs[0][0])
    return [(r[0], r[1].upper() if len(r) > 1 else "PASSIVE") for r in recs[1:1 + n]]


@dataclass
class AtomsModel:
    """Everything the equilibria, the background and the depth scales read
    besides the atmosphere, in device memory."""
    tables: LP.ElementTables
    dev_tables: LP.DeviceTables
    molecules: list
    atoms: PassiveAtoms
    setup: dict                   # background.model_from_setup's input
    vmicro_char: float            # m/s
    total_abund: float
    wght_per_H: float
    device: str
    keep: tuple
    _bg: dict = field(default_factory=dict)

    @classmethod
    def build(cls, tables: LP.ElementTables, atoms: list, molecules: list,
              vmicro_char: float = 5.0e3, device="cuda") -> "AtomsModel":
        """tables: element tables; atoms: parsed model atoms (grid.read_atom),
        hydrogen among them, all passive; molecules: parsed molecules
        (chem.read_molecule), H2 first; vmicro_char in m/s."""
        import torch
        if not 0 < len(atoms) <= MAX_ATOMS:
            raise ValueError(f"{len(atoms)} atoms (1..{MAX_ATOMS})")
        elems = [element_index(a) for a in atoms]
        if 0 not in elems:
            raise ValueError("hydrogen's model atom is missing")
        ids = [bytes(m.id).split(b"\0")[0] for m in molecules]
        present = [x in ids for x in (b"H2", b"OH", b"CH")]
        s = setup_from_atoms(atoms, elems, vmicro_char, present)
        lev = s["atoms_lev"]
        E = torch.from_numpy(np.ascontiguousarray(lev[:, 0])).to(device)
        g = torch.from_numpy(np.ascontiguousarray(lev[:, 1])).to(device)
        st = torch.from_numpy(np.ascontiguousarray(lev[:, 2], np.int32)).to(device)
        A = PassiveAtoms()
        A.natom = len(atoms)
        off = np.concatenate([[0], np.cumsum([a.nlevel for a in atoms])])
        for m, e in enumerate(elems):
            A.elem[m] = e
        for m, o in enumerate(off):
            A.lev_off[m] = int(o)
        A.E, A.g, A.stage = E.data_ptr(), g.data_ptr(), st.data_ptr()
        total, wght = abundance_totals(tables)
        return cls(tables, LP.DeviceTables(tables, device), list(molecules), A, s, vmicro_char,
                   total, wght, device, (E, g, st))

    @classmethod
    def from_cwd(cls, cwd, atomic_number=None, atomic_abundance=None,
                 device="cuda") -> "AtomsModel":
        """What the reference reads for a run in cwd: keyword.input's
        ATOMS_FILE and MOLECULES_FILE (relative to cwd), the atom and
        molecule files under $PYRH_PATH/rh/Atoms and rh/Molecules, the
        abundance and partition-function files, VMICRO_CHAR."""
        from .compute1d import read_keyword_input
        kw = read_keyword_input(os.path.join(str(cwd), "keyword.input"))
        root = os.environ.get("PYRH_PATH", "")
        tab = LP.tables_from_files(cwd, atomic_number, atomic_abundance)
        entries = list_file(os.path.join(str(cwd), kw.get("ATOMS_FILE", "atoms.input")))
        if any(mode == "ACTIVE" for _, mode in entries):
            raise NotImplementedError("an ACTIVE atom in the atoms list: the set-up here "
                                      "takes every atom passive")
        atoms = [G.read_atom(open(os.path.join(root, "rh", "Atoms", n)).read()) for n, _ in entries]
        mols = [CH.read_molecule(open(os.path.join(root, "rh", "Molecules", n)).read(),
                                 tab.abundance_set)
                for n, _ in list_file(os.path.join(str(cwd),
                                                   kw.get("MOLECULES_FILE", "molecules.input")))]
        vmc = float(kw.get("VMICRO_CHAR", "0.0")) * 1.0e3
        return cls.build(tab, atoms, mols, vmc, device)

    def background(self, hse: bool = False, fudge=None) -> BG.DeviceBackground:
        """The background model: Background()'s (metals' continua, no
        scattering in chi_c, as a run without active atoms has it) or, with
        hse, pyrh_Background's (no metals, scattering added)."""
        key = (hse, None if fudge is None else (tuple(np.ravel(fudge[0])),
                                                tuple(np.ravel(fudge[1]))))
        if key not in self._bg:
            model = BG.model_from_setup(self.setup, lte=True, metals=not hse)
            self._bg[key] = BG.DeviceBackground(model, add_scatter=hse, fudge=fudge,
                                                device=self.device)
        return self._bg[key]

    @property
    def h_row(self) -> tuple[int, int]:
        """Rows of hydrogen's ground level and protons in the populations."""
        m = [self.atoms.elem[i] for i in range(self.atoms.natom)].index(0)
        return int(self.atoms.lev_off[m]), int(self.atoms.lev_off[m + 1]) - 1


def equilibria(model: AtomsModel, T, ne, nHtot):
    """(pops [nlevel, npoint], nmol [nmol, npoint], nHmin [npoint]) as torch
    tensors on the model's device."""
    import torch
    T, ne, nHtot = (LP._dev(x, model.device) for x in (T, ne, nHtot))
    npt = T.numel()
    nlev = int(model.atoms.lev_off[model.atoms.natom])
    pops = torch.zeros((nlev, npt), dtype=torch.float64, device=model.device)
    nmol = torch.zeros((len(model.molecules), npt), dtype=torch.float64, device=model.device)
    nHmin = torch.zeros(npt, dtype=torch.float64, device=model.device)
    mols = (CH.Molecule * len(model.molecules))(*model.molecules)
    L.check(_lib().pyrh_equilibria(C.byref(model.dev_tables.struct), mols, len(model.molecules),
                                   C.byref(model.atoms), npt, T.data_ptr(), ne.data_ptr(),
                                   nHtot.data_ptr(), pops.data_ptr(), nmol.data_ptr(),
                                   nHmin.data_ptr(), LP._stream()))
    return pops, nmol, nHmin


def _mol_row(model: AtomsModel, nmol, name: str):
    for i, m in enumerate(model.molecules):
        if bytes(m.id).split(b"\0")[0] == name.encode():
            return nmol[i]
    return None


def continuum(model: AtomsModel, lam, T, ne, nHtot, fudge=None):
    """Background() of one atmosphere with every atom passive: chi_c, eta_c
    [nlam, ndep] on the wavelengths lam [nm] and the proton density np
    [ndep], from T [K], ne, nHtot [m^-3]."""
    pops, nmol, nHmin = equilibria(model, T, ne, nHtot)
    z = np.zeros(len(np.atleast_1d(T)))
    dens = {k: (v.cpu().numpy() if v is not None else z)
            for k, v in (("nH2", _mol_row(model, nmol, "H2")), ("nOH", _mol_row(model, nmol, "OH")),
                         ("nCH", _mol_row(model, nmol, "CH")))}
    p = pops.cpu().numpy()
    atm = {"lambda": np.asarray(lam, np.float64), "T": np.asarray(T, np.float64),
           "ne": np.asarray(ne, np.float64), "nHmin": nHmin.cpu().numpy(), "nstar": p, **dens}
    chi, eta, _ = model.background(hse=False, fudge=fudge).compute([atm], precision=L.PYRH_FP64)
    return chi[0], eta[0], p[model.h_row[1]].copy()


def convert_scales(model: AtomsModel, atm_scale: int, scale, T, ne, nHtot, chi_ref,
                   gravity: float = GRAVITY):
    """convertScales for atmospheres [natm, ndep] (or one [ndep]): the given
    scale (log10 tau_ref, log10 column mass [g cm^-2] or height [km]) and
    the continuum opacity at lambda_ref give tau_ref, column mass [kg m^-2]
    and height [m], each [natm, ndep]."""
    import torch
    x = [np.atleast_2d(np.asarray(v, np.float64)) for v in (scale, T, ne, nHtot, chi_ref)]
    natm, ndep = x[0].shape
    if any(v.shape != (natm, ndep) for v in x):
        raise ValueError("scale, T, ne, nHtot and chi_ref differ in shape")
    dev = model.device
    t = [torch.from_numpy(np.ascontiguousarray(v.T)).to(dev) for v in x]
    out = [torch.zeros((ndep, natm), dtype=torch.float64, device=dev) for _ in range(3)]
    b = ScalesBatch(natm=natm, ndep=ndep, scale=int(atm_scale), gravity=gravity,
                    total_abund=model.total_abund, wght_per_H=model.wght_per_H)
    b.scale_in, b.T, b.ne, b.nHtot, b.chi_ref = (v.data_ptr() for v in t)
    b.tau_ref, b.cmass, b.height = (v.data_ptr() for v in out)
    L.check(_lib().pyrh_convert_scales(C.byref(b), LP._stream()))
    return tuple(v.cpu().numpy().T.copy() for v in out)


def get_scales(cwd, atm_scale, scale, atmosphere, lam_ref, atomic_number=None,
               atomic_abundance=None, model: AtomsModel | None = None):
    """pyrh.get_scales (pyrh.pyx:491-533 -> rh/rhf1d/pyrh_hse.c:402-554):
    tau_ref, height [m] and column mass [kg m^-2] of an atmosphere [9, ndep]
    (the rows of compute1d: T [K], ne [cm^-3], ..., nH [cm^-3] in row 8)
    from the continuum opacity at lam_ref [nm]."""
    atmosphere = np.asarray(atmosphere, np.float64)
    if (atomic_number is None) != (atomic_abundance is None):
        atomic_number = atomic_abundance = None       # the reference reads neither then
    if model is None:
        model = AtomsModel.from_cwd(cwd, atomic_number, atomic_abundance)
    cube = 1.0e-2 * 1.0e-2 * 1.0e-2               # CUBE(CM_TO_M), pyrh_hse.c:472-478
    T, ne, nH = atmosphere[1], atmosphere[2] / cube, atmosphere[8] / cube
    chi, _, _ = continuum(model, [float(lam_ref)], T, ne, nH)
    tau, cmass, height = convert_scales(model, atm_scale, scale, T, ne, nH, chi[0])
    return tau[0], height[0], cmass[0]
