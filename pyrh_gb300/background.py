"""Background continuum on the GPU through the C ABI (pyrh_background_prepare,
pyrh_background in background.cu): the angle-independent part of the
reference's Background() (rh/background.c:329-460).

    model = model_from_setup(setup)          # atomic data of the set-up
    dev = DeviceBackground(model)            # uploads it, prepares splines
    chi, eta, sca = dev.compute(atmospheres) # per atmosphere [nspect, ndep]

`setup` holds what the reference's set-up leaves for Background(): per atom
its levels (E [J], g, stage), continua (i, j, lambda0, shortest lambda,
hydrogenic flag, alpha0, table) and lines (i, j, lambda0, qwing, Aji), which
atom is hydrogen and which helium, VMICRO_CHAR, and which molecules exist
(the keys of the `background` fixture: atoms_meta, atoms_lev, atoms_cont,
atoms_tab, atoms_line, misc, mol_present).  An atmosphere is a dict with
lambda [nspect] nm, T, ne, nHmin (and nH2, nOH, nCH where present) [ndep]
SI, and nstar [sum of the atoms' levels, ndep]: every level's LTE population
(and n, the populations, for a model made with lte=False).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L

CLIGHT = 2.99792458E+08
HPLANCK = 6.6260755E-34
M_ELECTRON = 9.1093897E-31
Q_ELECTRON = 1.60217733E-19
EPSILON_0 = 8.854187817E-12
E_RYDBERG = 2.1798741E-18
NM_TO_M = 1.0E-09
PI = 3.14159265358979
LONG_WAVELENGTH = 1.0E6
HMIN_BF_POINTS = 34       # PYRH_BG_HMIN_BF_LAMBDA_N
MAX_DEPTH = 512


class BgContinuum(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("hydrogenic", "ntab", "n_i", "n_j", "nstar_i",
                                         "nstar_j")] + \
        [("tab_off", C.c_int64)] + \
        [(n, C.c_double) for n in ("lambda0", "lambda_min", "alpha0", "n_eff", "charge", "gbf0")]


class BgRayleighLine(C.Structure):
    _fields_ = [("lambda0", C.c_double), ("lambda_red", C.c_double), ("f", C.c_double),
                ("scatterer", C.c_int32), ("reserved", C.c_int32)]


class BgModel(C.Structure):
    _fields_ = [("ncont_h", C.c_int32), ("ncont_metal", C.c_int32), ("cont", C.c_void_p),
                ("tab_lambda", C.c_void_p), ("tab_alpha", C.c_void_p), ("tab_m2", C.c_void_p),
                ("tab_f32", C.c_void_p),
                ("ntab_total", C.c_int64), ("nray", C.c_int32), ("ray", C.c_void_p),
                ("ray_limit", C.c_double * 2), ("ray_pop", C.c_int32 * 2),
                ("pop_nh0", C.c_int32), ("pop_np", C.c_int32), ("npop", C.c_int32),
                ("nonlte", C.c_int32),
                ("h_active", C.c_int32), ("has_h2", C.c_int32), ("has_oh", C.c_int32),
                ("has_ch", C.c_int32), ("add_scatter", C.c_int32), ("nfudge", C.c_int32),
                ("fudge_lambda", C.c_void_p), ("fudge", C.c_void_p)]


class BgBatch(C.Structure):
    _fields_ = [("natm", C.c_int32), ("max_nspect", C.c_int32), ("max_ndep", C.c_int32),
                ("precision", C.c_int32), ("total_depth", C.c_int64)] + \
        [(n, C.c_void_p) for n in ("ndep", "nspect", "depth_off", "lam_off", "cont_off",
                                   "lambda_", "T", "ne", "nHmin", "nH2", "nOH", "nCH", "pops",
                                   "chi_c", "eta_c", "sca_c")]


def _lib():
    lib = L.lib()
    lib.pyrh_background_prepare.restype = C.c_int
    lib.pyrh_background_prepare.argtypes = [C.POINTER(BgModel), C.c_void_p]
    lib.pyrh_background.restype = C.c_int
    lib.pyrh_background.argtypes = [C.POINTER(BgModel), C.POINTER(BgBatch), C.c_void_p]
    return lib


def gaunt_bf(lam, n_eff, charge):
    """Seaton's bound-free Gaunt factor (hydrogen.c:269-283), for the
    threshold values of the hydrogenic metal continua."""
    x = ((HPLANCK * CLIGHT) / (lam * NM_TO_M)) / (E_RYDBERG * (charge * charge))
    x3 = x ** 0.33333333
    nsqx = 1.0 / ((n_eff * n_eff) * x)
    return 1.0 + 0.1728 * x3 * (1.0 - 2.0 * nsqx) - \
        0.0496 * (x3 * x3) * (1.0 - (1.0 - nsqx) * 0.66666667 * nsqx)


@dataclass
class Model:
    """Host form of pyrh_bg_model (arrays to upload and the scalars)."""
    cont: object                  # ctypes array of BgContinuum
    ncont_h: int
    ncont_metal: int
    tab_lambda: np.ndarray
    tab_alpha: np.ndarray
    ray: object                   # ctypes array of BgRayleighLine
    nray: int
    ray_limit: tuple
    ray_pop: tuple
    pop_nh0: int
    pop_np: int
    npop: int                     # rows of pops
    lte: bool                     # pops = [nstar]; else [n, nstar]
    h_active: bool
    molecules: tuple              # (H2, OH, CH) present


def model_from_setup(s: dict, lte: bool = True, metals: bool = True) -> Model:
    """The model of a set-up (see the module docstring): continua of
    hydrogen (hydrogen.c:176-200) and of the passive metals (metal.c:
    103-140, every atom after the first), Rayleigh lines of hydrogen and
    helium (rayleigh.c:55-90).  Population rows: level l of the concatenated
    atoms is row l of nstar; with lte=False the populations n come first
    (row l) and nstar follows (row nlev + l).  With lte the populations are
    the LTE ones (the passive atoms of LTE_POPULATIONS, HYDROGEN_LTE), as
    Metal_bf and Hydrogen_bf then read them (metal.c:110, the same array).
    metals=False leaves the metals' continua out, as the hydrostatic
    equilibrium's background does (rh/rhf1d/pyrh_background.c:144-457)."""
    meta = np.asarray(s["atoms_meta"])
    lev = np.asarray(s["atoms_lev"])
    cont = np.asarray(s["atoms_cont"])
    lines = np.asarray(s["atoms_line"])
    tab = np.asarray(s["atoms_tab"]).reshape(-1, 2)
    vmicro_char, he, h = float(s["misc"][0]), int(s["misc"][1]), int(s["misc"][2])
    nlev = int(meta[:, 0].sum())
    so = 0 if lte else nlev           # first row of nstar
    lo = np.concatenate([[0], np.cumsum(meta[:, 0])]).astype(int)
    co = np.concatenate([[0], np.cumsum(meta[:, 1])]).astype(int)
    li = np.concatenate([[0], np.cumsum(meta[:, 2])]).astype(int)
    E, g, stage = lev[:, 0], lev[:, 1], lev[:, 2].astype(int)
    sigma0 = 32.0 / (3.0 * np.sqrt(3.0)) * Q_ELECTRON * Q_ELECTRON / (4.0 * PI * EPSILON_0) / \
        (M_ELECTRON * CLIGHT) * HPLANCK / (2.0 * E_RYDBERG)
    out = []

    def add(m, r, hydrogen):
        i, j = lo[m] + int(r[0]), lo[m] + int(r[1])
        c = BgContinuum()
        c.lambda0, c.lambda_min = float(r[2]), float(r[3])
        if hydrogen:
            # hydrogen.c:183-200: sigma0 n_eff g (lambda / lambda0)^3, the
            # upper level taken as hydrogen's last (the protons)
            jl = lo[m] + int(meta[m, 0]) - 1
            c.hydrogenic, c.ntab = 1, 0
            c.n_eff = np.sqrt(E_RYDBERG / (E[j] - E[i]))
            c.charge = float(stage[i] + 1)
            c.alpha0, c.gbf0 = sigma0 * c.n_eff, 1.0
            c.n_i, c.n_j, c.nstar_i, c.nstar_j = i, jl, so + i, so + jl
        else:
            c.n_i, c.n_j, c.nstar_i, c.nstar_j = i, j, so + i, so + j
            if int(r[4]):
                Z = stage[j]
                c.hydrogenic, c.ntab = 1, 0
                c.n_eff = Z * np.sqrt(E_RYDBERG / (E[j] - E[i]))
                c.charge = float(Z)
                c.alpha0 = float(r[5])
                c.gbf0 = gaunt_bf(c.lambda0, c.n_eff, c.charge)
            else:
                c.hydrogenic, c.ntab, c.tab_off = 0, int(r[6]), int(r[7])
        out.append(c)

    h_active = bool(meta[h, 3])
    for r in cont[co[h]:co[h + 1]]:
        add(h, r, True)
    ncont_h = len(out)
    for m in range(1, len(meta) if metals else 1):
        if meta[m, 3]:
            continue
        for r in cont[co[m]:co[m + 1]]:
            add(m, r, False)
    C0 = 2 * PI * (Q_ELECTRON / EPSILON_0) * (Q_ELECTRON / M_ELECTRON) / CLIGHT
    rays, limit, pop = [], [LONG_WAVELENGTH, LONG_WAVELENGTH], [-1, -1]
    for s_, m in enumerate((h, he)):
        if m < 0 or meta[m, 2] == 0:
            continue
        pop[s_] = int(lo[m])
        for r in lines[li[m]:li[m + 1]]:
            if int(r[0]) != 0:
                continue
            red = r[2] * (1.0 + r[3] * vmicro_char / CLIGHT)
            limit[s_] = min(limit[s_], red)
            ln = BgRayleighLine()
            ln.lambda0, ln.lambda_red, ln.scatterer = float(r[2]), float(red), s_
            ln.f = float(r[4] * (g[lo[m] + int(r[1])] / g[lo[m]]) * (r[2] * NM_TO_M) ** 2 / C0)
            rays.append(ln)
    mol = tuple(bool(x) for x in np.asarray(s["mol_present"]))
    return Model(cont=(BgContinuum * max(len(out), 1))(*out), ncont_h=ncont_h,
                 ncont_metal=len(out) - ncont_h,
                 tab_lambda=np.ascontiguousarray(tab[:, 0]), tab_alpha=np.ascontiguousarray(tab[:, 1]),
                 ray=(BgRayleighLine * max(len(rays), 1))(*rays), nray=len(rays),
                 ray_limit=tuple(limit),
                 ray_pop=tuple(pop), pop_nh0=int(lo[h]), pop_np=int(lo[h] + meta[h, 0] - 1),
                 npop=nlev if lte else 2 * nlev, lte=lte, h_active=h_active, molecules=mol)


def continuum_on(dev: "DeviceBackground", atm: dict, lam, precision=L.PYRH_FP64):
    """chi_c and eta_c [nlam, ndep] of one atmosphere on the wavelengths lam
    (the layout compute1d's LteSetup and pyrh_gb300.lte take)."""
    chi, eta, _ = dev.compute([dict(atm, **{"lambda": np.asarray(lam, np.float64)})],
                              precision=precision)
    return chi[0], eta[0]


def setup_atmosphere(s: dict, a: int) -> dict:
    """Atmosphere a of the `background` fixture in the form compute() takes."""
    return {"lambda": s["lambda"], "T": s["T"][a], "ne": s["ne"][a], "nHmin": s["nHmin"][a],
            "nH2": s["nH2"][a], "nOH": s["nOH"][a], "nCH": s["nCH"][a],
            "n": s["atoms_n"][a], "nstar": s["atoms_nstar"][a]}


class DeviceBackground:
    """A model in GPU memory, prepared; compute() runs batches through it."""

    def __init__(self, model: Model, add_scatter: bool = False, fudge=None, device="cuda",
                 stream_ptr: int = 0):
        import torch
        self.model = model
        self.device = device
        nb = C.sizeof(BgContinuum) * (model.ncont_h + model.ncont_metal)
        self.cont_t = torch.frombuffer(bytearray(C.string_at(C.addressof(model.cont), max(nb, 1))),
                                       dtype=torch.uint8).to(device)
        nr = C.sizeof(BgRayleighLine) * len(model.ray)
        self.ray_t = torch.frombuffer(bytearray(C.string_at(C.addressof(model.ray), nr)),
                                      dtype=torch.uint8).to(device)
        self.tl = torch.from_numpy(np.append(model.tab_lambda, 0.0)).to(device)
        self.ta = torch.from_numpy(np.append(model.tab_alpha, 0.0)).to(device)
        self.m2 = torch.zeros(len(model.tab_lambda) + HMIN_BF_POINTS, dtype=torch.float64,
                              device=device)
        self.f32 = torch.zeros(3 * max(len(model.tab_lambda), 1), dtype=torch.float32,
                               device=device)
        m = BgModel()
        m.ncont_h, m.ncont_metal = model.ncont_h, model.ncont_metal
        m.cont = self.cont_t.data_ptr()
        m.tab_lambda, m.tab_alpha, m.tab_m2 = self.tl.data_ptr(), self.ta.data_ptr(), self.m2.data_ptr()
        m.tab_f32 = self.f32.data_ptr()
        m.ntab_total = len(model.tab_lambda)
        m.nray = model.nray
        m.ray = self.ray_t.data_ptr()
        m.ray_limit[0], m.ray_limit[1] = model.ray_limit
        m.ray_pop[0], m.ray_pop[1] = model.ray_pop
        m.pop_nh0, m.pop_np, m.npop = model.pop_nh0, model.pop_np, model.npop
        m.nonlte = int(any(model.cont[c].n_i != model.cont[c].nstar_i or
                           model.cont[c].n_j != model.cont[c].nstar_j
                           for c in range(model.ncont_h, model.ncont_h + model.ncont_metal)))
        m.h_active = int(model.h_active)
        m.has_h2, m.has_oh, m.has_ch = (int(x) for x in model.molecules)
        m.add_scatter = int(add_scatter)
        if fudge is not None:
            fl, fv = fudge
            self.fl = torch.from_numpy(np.ascontiguousarray(fl, np.float64)).to(device)
            self.fv = torch.from_numpy(np.ascontiguousarray(fv, np.float64).reshape(-1)).to(device)
            m.nfudge = len(fl)
            m.fudge_lambda, m.fudge = self.fl.data_ptr(), self.fv.data_ptr()
        self.m = m
        L.check(_lib().pyrh_background_prepare(C.byref(m), stream_ptr))

    def replicated_batch(self, atm: dict, lam, natm: int, precision=L.PYRH_FP32):
        """A device batch of natm copies of one atmosphere on the wavelengths
        lam (for timing): (BgBatch, the tensors behind it)."""
        import torch
        dev = self.device
        nd, ns = len(atm["T"]), len(lam)
        rep = lambda x: torch.from_numpy(np.ascontiguousarray(
            np.tile(np.asarray(x, np.float64), natm))).to(dev)
        rows = atm["nstar"] if self.model.lte else np.concatenate([atm["n"], atm["nstar"]], axis=0)
        dt = np.float32 if precision == L.PYRH_FP32 else np.float64
        t = {"ndep": torch.full((natm,), nd, dtype=torch.int32, device=dev),
             "nspect": torch.full((natm,), ns, dtype=torch.int32, device=dev),
             "depth_off": torch.arange(natm, dtype=torch.int64, device=dev) * nd,
             "lam_off": torch.arange(natm, dtype=torch.int64, device=dev) * ns,
             "cont_off": torch.arange(natm, dtype=torch.int64, device=dev) * (nd * ns),
             "lambda_": rep(lam), "T": rep(atm["T"]), "ne": rep(atm["ne"]),
             "nHmin": rep(atm["nHmin"]), "nH2": rep(atm["nH2"]), "nOH": rep(atm["nOH"]),
             "nCH": rep(atm["nCH"]),
             "pops": torch.from_numpy(np.ascontiguousarray(np.tile(rows, (1, natm)), dt)).to(dev)}
        for k in ("chi_c", "eta_c", "sca_c"):
            t[k] = torch.empty(natm * nd * ns, dtype=torch.float32 if dt == np.float32
                               else torch.float64, device=dev)
        b = BgBatch()
        b.natm, b.max_nspect, b.max_ndep, b.total_depth = natm, ns, nd, natm * nd
        b.precision = int(precision)
        for k, v in t.items():
            setattr(b, k, v.data_ptr())
        return b, t

    def run(self, batch: BgBatch, stream_ptr: int = 0) -> None:
        L.check(_lib().pyrh_background(C.byref(self.m), C.byref(batch), stream_ptr))

    def compute(self, atms: list[dict], precision=L.PYRH_FP64, stream_ptr: int = 0):
        """(chi_c, eta_c, sca_c), each a list of [nspect, ndep] arrays, in
        FP64 or FP32."""
        import torch
        dev = self.device
        nd = np.array([len(a["T"]) for a in atms], np.int32)
        ns = np.array([len(a["lambda"]) for a in atms], np.int32)
        if nd.max() > MAX_DEPTH:
            raise ValueError(f"{nd.max()} depth points > {MAX_DEPTH}")
        doff = np.concatenate([[0], np.cumsum(nd[:-1])]).astype(np.int64)
        loff = np.concatenate([[0], np.cumsum(ns[:-1])]).astype(np.int64)
        csz = nd.astype(np.int64) * ns
        coff = np.concatenate([[0], np.cumsum(csz[:-1])]).astype(np.int64)
        td, tc = int(nd.sum()), int(csz.sum())
        cat = lambda k: torch.from_numpy(np.ascontiguousarray(
            np.concatenate([np.asarray(a.get(k, np.zeros(len(a["T"]))), np.float64)
                            for a in atms]))).to(dev)
        rows = (lambda a: a["nstar"]) if self.model.lte else \
            (lambda a: np.concatenate([a["n"], a["nstar"]], axis=0))
        pops = np.concatenate([rows(a) for a in atms], axis=1)
        if pops.shape[0] != self.model.npop:
            raise ValueError(f"{pops.shape[0]} population rows, the model has {self.model.npop}")
        t = {"ndep": torch.from_numpy(nd).to(dev), "nspect": torch.from_numpy(ns).to(dev),
             "depth_off": torch.from_numpy(doff).to(dev), "lam_off": torch.from_numpy(loff).to(dev),
             "cont_off": torch.from_numpy(coff).to(dev), "lambda_": cat("lambda"), "T": cat("T"),
             "ne": cat("ne"), "nHmin": cat("nHmin"), "nH2": cat("nH2"), "nOH": cat("nOH"),
             "nCH": cat("nCH"),
             "pops": torch.from_numpy(np.ascontiguousarray(
                 pops, np.float32 if precision == L.PYRH_FP32 else np.float64)).to(dev),
             }
        dt = torch.float32 if precision == L.PYRH_FP32 else torch.float64
        for k in ("chi_c", "eta_c", "sca_c"):
            t[k] = torch.empty(tc, dtype=dt, device=dev)
        b = BgBatch()
        b.natm, b.max_nspect, b.max_ndep, b.total_depth = len(atms), int(ns.max()), int(nd.max()), td
        b.precision = int(precision)
        for k, v in t.items():
            setattr(b, k, v.data_ptr())
        L.check(_lib().pyrh_background(C.byref(self.m), C.byref(b), stream_ptr))
        out = []
        for key in ("chi_c", "eta_c", "sca_c"):
            x = t[key].cpu().numpy()
            out.append([x[coff[p]:coff[p] + csz[p]].reshape(nd[p], ns[p]).T for p in range(len(atms))])
        return tuple(out)
