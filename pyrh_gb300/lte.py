"""Host side of the batched LTE Stokes synthesis: packs atmospheres into the
C-ABI layout (include/pyrh_gb300.h) and calls libpyrh_gb300.so.

Per-atmosphere inputs are dicts of numpy arrays in SI units (the reference's
internal units after rh/rhf1d/pyrh_compute1dray.c:263-270):
  height, T, ne, nHtot, np, vturb, vel, B, gamma_B, chi_B   [ndep]
  line_pops  [nline, 2, ndep]  (n of the ionisation stage, ln U(T))
  lam        [nlam]            (vacuum nm; the spectrum grid)
  chi_c, eta_c [nlam, ndep]    (continuum opacity / emissivity, as the
                                reference stores them per wavelength,
                                rh/readj.c:284-354)
Optional temperature derivatives of those set-up inputs, used by the
response functions and gradients (pyrh_lte_setup_dT; a missing key holds
that input fixed):
  dT_chi_c, dT_eta_c [nlam, ndep]   d chi_c/dT, d eta_c/dT of the same depth
  dT_line_pops [nline, 2, ndep]     d n_stage/dT, d ln U/dT
  dT_np [ndep]                      d n_p/dT
  dT_len_up, dT_len_dn [ndep]       entry k >= 1: d|h_k - h_{k-1}|/dT_{k-1},
                                    d|h_k - h_{k-1}|/dT_k
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L

DEPTH_KEYS = ("height", "T", "ne", "nHtot", "np", "vturb", "vel", "B", "gamma_B", "chi_B")
# field of the C struct for each per-depth key
_FIELD = {"vel": "vlos"}


def make_lines(line_const: np.ndarray, zeeman: np.ndarray, zeeman_n: np.ndarray):
    """pyrh_line array from the RLK_Line records (rh/atom.h:156-167) with
    the column order of the oracle's line-constant record (oracle/rt_oracle.h)."""
    n = line_const.shape[0]
    arr = (L.PyrhLine * max(n, 1))()
    for i in range(n):
        c = line_const[i]
        ln = arr[i]
        ln.lambda0, ln.Ei, ln.gi = c[0], c[5], c[3]
        ln.Aji, ln.Bji, ln.Bij = c[7], c[8], c[9]
        ln.Grad, ln.GStark, ln.GvdWaals = c[10], c[11], c[12]
        ln.vdwaals = int(c[13])
        ln.cross, ln.alpha = c[14], c[15]
        ln.isotope_frac, ln.hyperfine_frac = c[16], c[17]
        ln.polarizable = int(c[18])
        ln.weight = c[19]
        ln.contributes = int(c[20])
        nc = int(zeeman_n[i])
        if nc > L.PYRH_MAX_COMPONENTS:
            raise ValueError(f"line {i}: {nc} Zeeman components > {L.PYRH_MAX_COMPONENTS}")
        ln.ncomp = nc
        for j in range(nc):
            ln.comp_q[j] = int(zeeman[i, 0, j])
            ln.comp_shift[j] = zeeman[i, 1, j]
            ln.comp_strength[j] = zeeman[i, 2, j]
    return arr, n


@dataclass
class Packed:
    """A batch in the C-ABI layout, as host numpy arrays."""
    natm: int
    max_ndep: int
    max_nlam: int
    total_depth: int
    arrays: dict          # name -> np.ndarray
    precision: int

    @property
    def nlam_total(self) -> int:
        return int(self.arrays["lam_off"][-1] + self.arrays["nlam"][-1])


def pack(atms: list[dict], nline: int, precision: int = L.PYRH_FP64) -> Packed:
    real = np.float32 if precision == L.PYRH_FP32 else np.float64
    natm = len(atms)
    ndep = np.array([len(a["T"]) for a in atms], dtype=np.int32)
    nlam = np.array([len(a["lam"]) for a in atms], dtype=np.int32)
    depth_off = np.concatenate([[0], np.cumsum(ndep[:-1], dtype=np.int64)]).astype(np.int64)
    lam_off = np.concatenate([[0], np.cumsum(nlam[:-1], dtype=np.int64)]).astype(np.int64)
    csz = ndep.astype(np.int64) * nlam
    cont_off = np.concatenate([[0], np.cumsum(csz[:-1])]).astype(np.int64)
    total_depth = int(ndep.sum())
    arrays = dict(ndep=ndep, nlam=nlam, depth_off=depth_off, lam_off=lam_off,
                  cont_off=cont_off)
    arrays["lambda"] = np.concatenate([np.asarray(a["lam"], np.float64) for a in atms])
    for k in DEPTH_KEYS:
        arrays[k] = np.concatenate([np.asarray(a[k], np.float64) for a in atms])
    lp = np.zeros((max(nline, 1), 2, total_depth))
    if nline:
        lp[:, :, :] = np.concatenate([np.asarray(a["line_pops"], np.float64) for a in atms],
                                     axis=2)
    arrays["line_pops"] = lp
    # continuum [depth][lambda] per atmosphere
    arrays["chi_c"] = np.concatenate([np.asarray(a["chi_c"], real).T.ravel() for a in atms])
    arrays["eta_c"] = np.concatenate([np.asarray(a["eta_c"], real).T.ravel() for a in atms])
    # set-up temperature derivatives where every atmosphere has them
    have = lambda k: all(k in a for a in atms)
    for k in ("dT_chi_c", "dT_eta_c"):
        if have(k):
            arrays[k] = np.concatenate([np.asarray(a[k], real).T.ravel() for a in atms])
    if have("dT_line_pops") and nline:
        arrays["dT_line_pops"] = np.concatenate(
            [np.asarray(a["dT_line_pops"], np.float64) for a in atms], axis=2)
    for k in ("dT_np", "dT_len_up", "dT_len_dn"):
        if have(k):
            arrays[k] = np.concatenate([np.asarray(a[k], np.float64) for a in atms])
    return Packed(natm, int(ndep.max()), int(nlam.max()), total_depth, arrays, precision)


SETUP_DT_FIELDS = {"dT_chi_c": "dchi_c", "dT_eta_c": "deta_c", "dT_line_pops": "dline_pops",
                   "dT_np": "dnp", "dT_len_up": "dlen_up", "dT_len_dn": "dlen_dn"}


def _batch_struct(pk: Packed, ptr) -> L.PyrhLteBatch:
    b = L.PyrhLteBatch()
    b.natm, b.max_ndep, b.max_nlam, b.total_depth = pk.natm, pk.max_ndep, pk.max_nlam, \
        pk.total_depth
    for k in ("ndep", "depth_off", "nlam", "lam_off", "cont_off"):
        setattr(b, k, ptr(k))
    b.lambda_ = ptr("lambda")
    for k in DEPTH_KEYS:
        setattr(b, _FIELD.get(k, k), ptr(k))
    b.line_pops = ptr("line_pops")
    b.chi_c = ptr("chi_c")
    b.eta_c = ptr("eta_c")
    if any(k in pk.arrays for k in SETUP_DT_FIELDS):
        sd = L.PyrhLteSetupDT()
        for k, f in SETUP_DT_FIELDS.items():
            setattr(sd, f, ptr(k) if k in pk.arrays else None)
        b._setup_dT = sd                 # keeps the struct alive with the batch
        b.setup_dT = C.addressof(sd)
    return b


def make_config(precision=L.PYRH_FP64, mu=1.0, vmicro_char=5.0e3, magneto_optical=False,
                moving=True, stokes_mode=L.PYRH_FULL_STOKES, block_lambda=0,
                persistent_blocks=0) -> L.PyrhLteConfig:
    cfg = L.PyrhLteConfig()
    cfg.precision = precision
    cfg.stokes_mode = stokes_mode
    cfg.magneto_optical = int(bool(magneto_optical))
    cfg.moving = int(bool(moving))
    cfg.mu = float(mu)
    cfg.vmicro_char = float(vmicro_char)
    cfg.block_lambda = int(block_lambda)
    cfg.persistent_blocks = int(persistent_blocks)
    return cfg


def synth_host(pk: Packed, lines, nline: int, cfg: L.PyrhLteConfig) -> np.ndarray:
    """Runs pyrh_lte_stokes_host (host in, host out); returns the flat
    [4 * sum nlam] output in the precision's dtype."""
    arrs = {k: np.ascontiguousarray(v) for k, v in pk.arrays.items()}
    b = _batch_struct(pk, lambda k: arrs[k].ctypes.data)
    real = np.float32 if cfg.precision == L.PYRH_FP32 else np.float64
    out = np.zeros(4 * pk.nlam_total, dtype=real)
    L.check(L.lib().pyrh_lte_stokes_host(C.byref(b), lines, nline, C.byref(cfg),
                                         out.ctypes.data))
    return out


def split_output(pk: Packed, out: np.ndarray) -> list[np.ndarray]:
    """Per-atmosphere [4, nlam] views of a flat output."""
    res = []
    for p in range(pk.natm):
        o, n = int(pk.arrays["lam_off"][p]), int(pk.arrays["nlam"][p])
        res.append(out[4 * o: 4 * o + 4 * n].reshape(4, n))
    return res


class DeviceBatch:
    """A packed batch resident in GPU memory (torch tensors used as plain
    device buffers), for repeated launches of pyrh_lte_stokes."""

    def __init__(self, pk: Packed, lines, nline: int, device="cuda"):
        import torch
        self.pk = pk
        self.t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(device)
                  for k, v in pk.arrays.items()}
        nbytes = C.sizeof(L.PyrhLine) * max(nline, 1)
        self.lines_t = torch.empty(nbytes, dtype=torch.uint8, device=device)
        host = torch.frombuffer(bytearray(C.string_at(C.addressof(lines), nbytes)),
                                dtype=torch.uint8)
        self.lines_t.copy_(host)
        self.nline = nline
        real = torch.float32 if pk.precision == L.PYRH_FP32 else torch.float64
        self.out = torch.zeros(4 * pk.nlam_total, dtype=real, device=device)
        self.struct = _batch_struct(pk, lambda k: self.t[k].data_ptr())

    def run(self, cfg: L.PyrhLteConfig, stream_ptr: int = 0) -> None:
        L.check(L.lib().pyrh_lte_stokes(C.byref(self.struct), self.lines_t.data_ptr(),
                                        self.nline, C.byref(cfg), self.out.data_ptr(),
                                        stream_ptr))


class Plan:
    """pyrh_lte_plan for a resident batch: the wavelength tile tuned on the
    batch's own buffers and one launch recorded as a CUDA graph."""

    def __init__(self, dev: DeviceBatch, cfg: L.PyrhLteConfig, stream_ptr: int = 0):
        lib = L.lib()
        lib.pyrh_lte_plan_create.restype = C.c_int
        lib.pyrh_lte_plan_create.argtypes = [C.POINTER(L.PyrhLteBatch), C.c_void_p, C.c_int32,
                                             C.POINTER(L.PyrhLteConfig), C.c_void_p, C.c_void_p,
                                             C.POINTER(C.c_void_p)]
        lib.pyrh_lte_plan_launch.restype = C.c_int
        lib.pyrh_lte_plan_launch.argtypes = [C.c_void_p, C.c_void_p]
        lib.pyrh_lte_plan_block.restype = C.c_int32
        lib.pyrh_lte_plan_block.argtypes = [C.c_void_p]
        lib.pyrh_lte_plan_ms.restype = C.c_double
        lib.pyrh_lte_plan_ms.argtypes = [C.c_void_p]
        lib.pyrh_lte_plan_destroy.restype = None
        lib.pyrh_lte_plan_destroy.argtypes = [C.c_void_p]
        self.lib = lib
        self.dev = dev                      # keeps the bound buffers alive
        self.handle = C.c_void_p()
        L.check(lib.pyrh_lte_plan_create(C.byref(dev.struct), dev.lines_t.data_ptr(), dev.nline,
                                         C.byref(cfg), dev.out.data_ptr(), stream_ptr,
                                         C.byref(self.handle)))
        self.block = int(lib.pyrh_lte_plan_block(self.handle))
        self.tuned_ms = float(lib.pyrh_lte_plan_ms(self.handle))

    def launch(self, stream_ptr: int = 0) -> None:
        L.check(self.lib.pyrh_lte_plan_launch(self.handle, stream_ptr))

    def __del__(self):
        if getattr(self, "handle", None):
            self.lib.pyrh_lte_plan_destroy(self.handle)
            self.handle = None


def pack_uniform(batch: dict, nline: int, precision: int = L.PYRH_FP32) -> Packed:
    """Vectorised pack of a batch whose atmospheres share ndep and the
    wavelength grid (arrays with a leading atmosphere axis; continuum
    [natm, ndep, nlam], lambda fastest, as pyrh_gb300.workload builds it)."""
    real = np.float32 if precision == L.PYRH_FP32 else np.float64
    natm, nd = batch["T"].shape
    lam = np.asarray(batch["lam"], np.float64)
    nl = lam.shape[-1]
    arrays = dict(
        ndep=np.full(natm, nd, np.int32), nlam=np.full(natm, nl, np.int32),
        depth_off=np.arange(natm, dtype=np.int64) * nd,
        lam_off=np.arange(natm, dtype=np.int64) * nl,
        cont_off=np.arange(natm, dtype=np.int64) * nd * nl)
    arrays["lambda"] = np.broadcast_to(lam, (natm, nl)).reshape(-1).copy()
    for k in DEPTH_KEYS:
        arrays[k] = np.ascontiguousarray(batch[k], np.float64).reshape(-1)
    lp = np.asarray(batch["line_pops"], np.float64)          # [natm, nline, 2, nd]
    arrays["line_pops"] = np.ascontiguousarray(lp.transpose(1, 2, 0, 3)).reshape(nline, 2, -1)
    arrays["chi_c"] = np.ascontiguousarray(batch["chi_c"], real).reshape(-1)
    arrays["eta_c"] = np.ascontiguousarray(batch["eta_c"], real).reshape(-1)
    for k in ("dT_chi_c", "dT_eta_c"):
        if k in batch:
            arrays[k] = np.ascontiguousarray(batch[k], real).reshape(-1)
    if "dT_line_pops" in batch:
        dlp = np.asarray(batch["dT_line_pops"], np.float64)
        arrays["dT_line_pops"] = np.ascontiguousarray(dlp.transpose(1, 2, 0, 3)).reshape(nline, 2, -1)
    for k in ("dT_np", "dT_len_up", "dT_len_dn"):
        if k in batch:
            arrays[k] = np.ascontiguousarray(batch[k], np.float64).reshape(-1)
    return Packed(natm, nd, nl, natm * nd, arrays, precision)
