"""Host side of the batched NLTE MALI solver (libpyrh_gb300.so,
pyrh_nlte_solve / pyrh_nlte_emergent).

An atmosphere is given as a dict with the state the reference's set-up
leaves before its Iterate() (rh/rhf1d/pyrh_compute1dray.c:280-323):
  lambda [nspect] nm; height, T, vel, vbroad, ntotal [ndep] SI;
  background [3, nspect, ndep] (chi_c, eta_c, sca_c); bgflags [nspect];
  nstar, n0 [nlevel, ndep]; C [nlevel^2, ndep]; lines [nline, 16] and
  continua [ncont, 8] transition records; adamp [nline, ndep]; alpha;
  optional J0 [nspect, ndep] (zero when absent).
A line record is [i, j, lambda0, Aji, Bji, Bij, isotope_frac, Nblue,
Nlambda, symmetric, Ncomponent, c_shift, c_fraction, Voigt, PRD,
polarized], polarized = line->polarizable with STOKES_MODE other than
FIELD_FREE (the wavelengths it covers are angle dependent, opacity.c:574-589;
pyrh_atom_line_polarizable gives it from the model atom); bgflags holds
backgrflags' hasline (bit 0) and ispolarized (bit 1).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L

MAX_RAYS = 8


class PyrhNlteTransition(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("type", "i", "j", "nblue", "nlambda", "symmetric",
                                         "voigt", "line_index", "polarized", "reserved")] + \
        [("phi_off", C.c_int64), ("alpha_off", C.c_int64)] + \
        [(n, C.c_double) for n in ("lambda0", "Aji", "Bji", "Bij", "isotope_frac", "c_shift",
                                   "c_fraction")]


class PyrhNlteBatch(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("natm", "nlevel", "max_ndep", "max_nspect",
                                         "max_nline")] + \
        [(n, C.c_int64) for n in ("total_depth", "total_lambda", "total_cont")] + \
        [(n, C.c_void_p) for n in ("ndep", "nspect", "ntrans", "depth_off", "lam_off",
                                   "cont_off", "trans_off", "adamp_off", "lambda_", "height",
                                   "T", "vel", "vbroad", "ntotal", "nstar", "C", "chi_c",
                                   "eta_c", "sca_c", "bgline", "trans", "alpha", "adamp", "n",
                                   "J")] + \
        [("max_ntrans", C.c_int32), ("rates", C.c_void_p)]


class PyrhNlteConfig(C.Structure):
    _fields_ = [("precision", C.c_int32), ("nrays", C.c_int32),
                ("muz", C.c_double * MAX_RAYS), ("wmu", C.c_double * MAX_RAYS),
                ("moving", C.c_int32), ("isum", C.c_int32), ("ng_order", C.c_int32),
                ("ng_delay", C.c_int32), ("ng_period", C.c_int32), ("nmax_iter", C.c_int32),
                ("iter_limit", C.c_double)]


def _lib():
    lib = L.lib()
    lib.pyrh_nlte_workspace_bytes.restype = C.c_size_t
    lib.pyrh_nlte_workspace_bytes.argtypes = [C.POINTER(PyrhNlteBatch),
                                              C.POINTER(PyrhNlteConfig), C.c_int64]
    lib.pyrh_nlte_solve.restype = C.c_int
    lib.pyrh_nlte_solve.argtypes = [C.POINTER(PyrhNlteBatch), C.POINTER(PyrhNlteConfig),
                                    C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.pyrh_nlte_emergent.restype = C.c_int
    lib.pyrh_nlte_emergent.argtypes = [C.POINTER(PyrhNlteBatch), C.POINTER(PyrhNlteConfig),
                                       C.c_double, C.c_void_p, C.c_size_t, C.c_void_p,
                                       C.c_void_p]
    return lib


def make_config(fx: dict, precision=L.PYRH_FP64, nmax_iter=None) -> PyrhNlteConfig:
    """Iteration parameters of an NLTE fixture (keyword.input values the
    reference ran with)."""
    m = fx["meta"]
    cfg = PyrhNlteConfig()
    cfg.precision = precision
    nr = len(fx["muz"])
    if nr > MAX_RAYS:
        raise ValueError(f"{nr} rays > {MAX_RAYS}")
    cfg.nrays = nr
    for i in range(nr):
        cfg.muz[i] = float(fx["muz"][i])
        cfg.wmu[i] = float(fx["wmu"][i])
    cfg.moving = int(m[12])
    cfg.isum = int(m[10])
    cfg.ng_order, cfg.ng_delay, cfg.ng_period = int(m[8]), int(m[7]), int(m[9])
    cfg.nmax_iter = int(m[6]) if nmax_iter is None else int(nmax_iter)
    cfg.iter_limit = float(fx["fmeta"][0])
    return cfg


@dataclass
class PackedNlte:
    natm: int
    nlevel: int
    arrays: dict
    trans: object           # ctypes array of PyrhNlteTransition
    ntrans_total: int
    phi_elems: int
    shape: dict             # max_ndep, max_nspect, max_nline, totals


def pack(atms: list[dict], nrays: int) -> PackedNlte:
    natm = len(atms)
    nlevel = len(atms[0]["g"])
    ndep = np.array([len(a["T"]) for a in atms], np.int32)
    nspect = np.array([len(a["lambda"]) for a in atms], np.int32)
    depth_off = np.concatenate([[0], np.cumsum(ndep[:-1])]).astype(np.int64)
    lam_off = np.concatenate([[0], np.cumsum(nspect[:-1])]).astype(np.int64)
    csz = ndep.astype(np.int64) * nspect
    cont_off = np.concatenate([[0], np.cumsum(csz[:-1])]).astype(np.int64)
    total_depth = int(ndep.sum())
    trans, ntrans, trans_off, adamp_off = [], [], [], []
    alpha_all, adamp_all = [], []
    phi_off = 0
    aoff = 0
    adoff = 0
    for a in atms:
        trans_off.append(len(trans))
        adamp_off.append(adoff)
        nd = len(a["T"])
        for c in a["continua"]:                     # continua first (active-set order)
            t = PyrhNlteTransition()
            t.type, t.i, t.j = 1, int(c[0]), int(c[1])
            t.nblue, t.nlambda = int(c[2]), int(c[3])
            t.lambda0 = c[4]
            t.alpha_off = aoff + int(c[6])
            trans.append(t)
        for li, l in enumerate(a["lines"]):
            t = PyrhNlteTransition()
            t.type, t.i, t.j = 0, int(l[0]), int(l[1])
            t.lambda0, t.Aji, t.Bji, t.Bij, t.isotope_frac = l[2], l[3], l[4], l[5], l[6]
            t.nblue, t.nlambda, t.symmetric = int(l[7]), int(l[8]), int(l[9])
            if int(l[10]) != 1:
                raise ValueError("lines with several components are not supported")
            t.c_shift, t.c_fraction, t.voigt = l[11], l[12], int(l[13])
            if int(l[14]):
                raise ValueError("PRD lines are not supported")
            t.line_index = li
            t.polarized = int(l[15])
            t.phi_off = phi_off
            phi_off += int(l[8]) * 2 * nrays * nd
            trans.append(t)
        ntrans.append(len(trans) - trans_off[-1])
        alpha_all.append(np.asarray(a["alpha"], np.float64))
        aoff += len(a["alpha"])
        adamp_all.append(np.asarray(a["adamp"], np.float64).reshape(-1))
        adoff += a["adamp"].size
    tarr = (PyrhNlteTransition * len(trans))(*trans)
    cat = lambda k: np.concatenate([np.asarray(a[k], np.float64) for a in atms])
    lev = lambda k: np.concatenate([np.asarray(a[k], np.float64) for a in atms], axis=1)
    bgT = [np.asarray(a["background"], np.float64).transpose(0, 2, 1) for a in atms]
    arrays = dict(
        ndep=ndep, nspect=nspect, ntrans=np.array(ntrans, np.int32), depth_off=depth_off,
        lam_off=lam_off, cont_off=cont_off, trans_off=np.array(trans_off, np.int64),
        adamp_off=np.array(adamp_off, np.int64), lambda_=cat("lambda"), height=cat("height"),
        T=cat("T"), vel=cat("vel"), vbroad=cat("vbroad"), ntotal=cat("ntotal"),
        nstar=np.ascontiguousarray(lev("nstar")), C=np.ascontiguousarray(lev("C")),
        chi_c=np.concatenate([b[0].ravel() for b in bgT]),
        eta_c=np.concatenate([b[1].ravel() for b in bgT]),
        sca_c=np.concatenate([b[2].ravel() for b in bgT]),
        bgline=np.concatenate([np.asarray(a["bgflags"], np.int32) & 3 for a in atms]),
        alpha=np.concatenate(alpha_all) if alpha_all else np.zeros(1),
        adamp=np.concatenate(adamp_all) if adamp_all else np.zeros(1),
        n=np.ascontiguousarray(lev("n0")),
        J=np.concatenate([np.asarray(a.get("J0", np.zeros((len(a["lambda"]), len(a["T"])))),
                                     np.float64).T.ravel() for a in atms]),
    )
    shape = dict(max_ndep=int(ndep.max()), max_nspect=int(nspect.max()),
                 max_nline=max(len(a["lines"]) for a in atms), total_depth=total_depth,
                 total_lambda=int(nspect.sum()), total_cont=int(csz.sum()))
    return PackedNlte(natm, nlevel, arrays, tarr, len(trans), phi_off, shape)


class DeviceNlte:
    """A packed NLTE batch in GPU memory with its workspace."""

    def __init__(self, pk: PackedNlte, cfg: PyrhNlteConfig, device="cuda", rates=False):
        """rates: keep every transition's radiative rates R_ij, R_ji after
        its atmosphere's last formal solution (radiative_rates())."""
        import torch
        self.pk = pk
        self.t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(device)
                  for k, v in pk.arrays.items()}
        nb = C.sizeof(PyrhNlteTransition) * pk.ntrans_total
        self.trans_t = torch.empty(nb, dtype=torch.uint8, device=device)
        self.trans_t.copy_(torch.frombuffer(bytearray(C.string_at(C.addressof(pk.trans), nb)),
                                            dtype=torch.uint8))
        b = PyrhNlteBatch()
        b.natm, b.nlevel = pk.natm, pk.nlevel
        for k, v in pk.shape.items():
            setattr(b, k, v)
        for k, v in self.t.items():
            setattr(b, k, v.data_ptr())
        b.trans = self.trans_t.data_ptr()
        self.max_ntrans = int(pk.arrays["ntrans"].max())
        self.rates = None
        if rates:
            self.rates = torch.zeros(2 * self.max_ntrans * pk.shape["total_depth"],
                                     dtype=torch.float64, device=device)
            b.max_ntrans = self.max_ntrans
            b.rates = self.rates.data_ptr()
        self.batch = b
        self.ws_bytes = _lib().pyrh_nlte_workspace_bytes(C.byref(b), C.byref(cfg), pk.phi_elems)
        self.ws = torch.empty(self.ws_bytes, dtype=torch.uint8, device=device)
        self.iterations = torch.zeros(pk.natm, dtype=torch.int32, device=device)
        self.dpops = torch.zeros(pk.natm, dtype=torch.float64, device=device)
        self.I_out = torch.zeros(pk.shape["total_lambda"], dtype=torch.float64, device=device)

    def reset(self):
        """Restore the starting populations and J (for repeated solves)."""
        import torch
        self.t["n"].copy_(torch.from_numpy(self.pk.arrays["n"]))
        self.t["J"].copy_(torch.from_numpy(self.pk.arrays["J"]))

    def solve(self, cfg: PyrhNlteConfig, stream_ptr: int = 0) -> int:
        return _lib().pyrh_nlte_solve(C.byref(self.batch), C.byref(cfg), self.ws.data_ptr(),
                                      self.ws_bytes, self.iterations.data_ptr(),
                                      self.dpops.data_ptr(), stream_ptr)

    def emergent(self, cfg: PyrhNlteConfig, mu_out: float, stream_ptr: int = 0) -> int:
        return _lib().pyrh_nlte_emergent(C.byref(self.batch), C.byref(cfg), float(mu_out),
                                         self.ws.data_ptr(), self.ws_bytes,
                                         self.I_out.data_ptr(), stream_ptr)

    def populations(self) -> list[np.ndarray]:
        n = self.t["n"].cpu().numpy()
        out = []
        for p in range(self.pk.natm):
            o, nd = int(self.pk.arrays["depth_off"][p]), int(self.pk.arrays["ndep"][p])
            out.append(n[:, o:o + nd])
        return out

    def mean_intensity(self) -> list[np.ndarray]:
        J = self.t["J"].cpu().numpy()
        out = []
        for p in range(self.pk.natm):
            o = int(self.pk.arrays["cont_off"][p])
            nd, ns = int(self.pk.arrays["ndep"][p]), int(self.pk.arrays["nspect"][p])
            out.append(J[o:o + nd * ns].reshape(nd, ns).T)
        return out

    def radiative_rates(self) -> list[dict]:
        """Per atmosphere {"continua": [ncont, 2, ndep], "lines": [nline, 2,
        ndep]}: R_ij and R_ji [s^-1] of each transition after the
        atmosphere's last formal solution (needs rates=True)."""
        if self.rates is None:
            raise ValueError("DeviceNlte was made without rates=True")
        R = self.rates.cpu().numpy().reshape(2 * self.max_ntrans, -1)
        a = self.pk.arrays
        out = []
        for p in range(self.pk.natm):
            o, nd = int(a["depth_off"][p]), int(a["ndep"][p])
            t0, nt = int(a["trans_off"][p]), int(a["ntrans"][p])
            r = R[:2 * nt, o:o + nd].reshape(nt, 2, nd)
            ncont = sum(1 for i in range(t0, t0 + nt) if self.pk.trans[i].type == 1)
            out.append({"continua": r[:ncont], "lines": r[ncont:]})
        return out

    def emergent_spectra(self) -> list[np.ndarray]:
        I = self.I_out.cpu().numpy()
        out = []
        for p in range(self.pk.natm):
            o, ns = int(self.pk.arrays["lam_off"][p]), int(self.pk.arrays["nspect"][p])
            out.append(I[o:o + ns])
        return out


class PyrhNlteSetupBatch(C.Structure):
    _fields_ = [("total_depth", C.c_int64)] + \
        [(n, C.c_void_p) for n in ("T", "ne", "ntotal", "vturb", "nh0", "np", "nstar", "C",
                                   "vbroad")]


def device_setup(atom, weight_amu: float, T, ne, ntotal, vturb, nh0=None, np_=None,
                 device="cuda", stream_ptr: int = 0):
    """LTE populations [nlevel, nd], collision rates [nlevel^2, nd] and
    Doppler widths [nd] of one model atom (pyrh_gb300.grid.read_atom) at the
    depth points given (SI arrays, any number of atmospheres concatenated),
    computed on the device by pyrh_nlte_setup."""
    import torch
    from . import grid as G
    lib = _lib()
    lib.pyrh_nlte_setup_workspace_bytes.restype = C.c_size_t
    lib.pyrh_nlte_setup_workspace_bytes.argtypes = [C.POINTER(G.Atom)]
    lib.pyrh_nlte_setup.restype = C.c_int
    lib.pyrh_nlte_setup.argtypes = [C.POINTER(G.Atom), C.c_double,
                                    C.POINTER(PyrhNlteSetupBatch), C.c_void_p, C.c_size_t,
                                    C.c_void_p]
    f64 = lambda a: torch.as_tensor(np.ascontiguousarray(a, np.float64), device=device)
    ins = {"T": f64(T), "ne": f64(ne), "ntotal": f64(ntotal), "vturb": f64(vturb)}
    if nh0 is not None:
        ins["nh0"] = f64(nh0)
    if np_ is not None:
        ins["np"] = f64(np_)
    nd = ins["T"].numel()
    nl = atom.nlevel
    out = {"nstar": torch.empty(nl * nd, dtype=torch.float64, device=device),
           "C": torch.empty(nl * nl * nd, dtype=torch.float64, device=device),
           "vbroad": torch.empty(nd, dtype=torch.float64, device=device)}
    b = PyrhNlteSetupBatch()
    b.total_depth = nd
    for k, v in list(ins.items()) + list(out.items()):
        setattr(b, k, v.data_ptr())
    wsb = lib.pyrh_nlte_setup_workspace_bytes(C.byref(atom))
    ws = torch.empty(wsb, dtype=torch.uint8, device=device)
    L.check(lib.pyrh_nlte_setup(C.byref(atom), float(weight_amu), C.byref(b), ws.data_ptr(),
                                wsb, stream_ptr))
    return (out["nstar"].view(nl, nd).cpu().numpy(), out["C"].view(nl * nl, nd).cpu().numpy(),
            out["vbroad"].cpu().numpy())
