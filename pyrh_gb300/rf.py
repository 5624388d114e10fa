"""Response functions and gradients of the batched LTE Stokes synthesis.

Host side of pyrh_lte_rf, pyrh_lte_chi2_grad and pyrh_lte_stokes_vjp
(include/pyrh_gb300.h) and a torch.autograd.Function around the synthesis.
The derivatives are taken with respect to the six atmosphere parameters of
every depth, in this order and in SI units:
    T [K], v_los [m/s], v_mic [m/s], B [T], gamma_B [rad], chi_B [rad]
(the depth-resolved quantities the reference perturbs for its finite-
difference response functions, rh/rhf1d/rf_ray.c:205-235).

The reference re-runs its set-up for every perturbed temperature
(Background() and convertScales(), rf_ray.c:257-283), so its temperature
response also moves the continuum, the stage densities, the proton density
and, on a tau_500 depth scale, the interval lengths.  A batch packed with the
dT_* keys of pyrh_gb300.lte (pyrh_lte_setup_dT) gets those terms as well;
without them the set-up is held fixed and the temperature derivative is the
partial one at fixed continuum, populations and heights.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .lte import DeviceBatch, Packed

PARAMS = ("T", "vel", "vturb", "B", "gamma_B", "chi_B")
NPARAM = len(PARAMS)

_bound = None


def _lib():
    global _bound
    lib = L.lib()
    if _bound is not lib:
        B, P, I32, V = C.POINTER(L.PyrhLteBatch), C.POINTER(L.PyrhLteConfig), C.c_int32, C.c_void_p
        lib.pyrh_lte_rf.restype = C.c_int
        lib.pyrh_lte_rf.argtypes = [B, V, I32, P, V, V, V, V]
        lib.pyrh_lte_chi2_grad.restype = C.c_int
        lib.pyrh_lte_chi2_grad.argtypes = [B, V, I32, P, V, V, V, V, V, V, V]
        lib.pyrh_lte_stokes_vjp.restype = C.c_int
        lib.pyrh_lte_stokes_vjp.argtypes = [B, V, I32, P, V, V, V, V, V]
        _bound = lib
    return lib


def _real(dev: DeviceBatch):
    import torch
    return torch.float32 if dev.pk.precision == L.PYRH_FP32 else torch.float64


def tau500_interval_dT(height, chi_ref, dchi_ref_dT):
    """Temperature derivatives of the interval lengths |h_k - h_{k-1}| of a
    height scale built from tau_500 (convertScales, TAU500 branch,
    rh/rhf1d/multiatmos.c:126-138: h_k = h_{k-1} - 2 (tau_k - tau_{k-1}) /
    (chi_ref_{k-1} + chi_ref_k), chi_ref the continuum opacity at
    LAMBDA_REF).  Returns (dT_len_up, dT_len_dn) [ndep]: entry k >= 1 is
    the derivative with respect to T_{k-1} and T_k; entry 0 is zero."""
    h = np.asarray(height, np.float64)
    c = np.asarray(chi_ref, np.float64)
    dc = np.asarray(dchi_ref_dT, np.float64)
    up, dn = np.zeros(len(h)), np.zeros(len(h))
    length = np.abs(h[1:] - h[:-1])
    den = c[:-1] + c[1:]
    up[1:] = -length * dc[:-1] / den
    dn[1:] = -length * dc[1:] / den
    return up, dn


def rf_size(pk: Packed) -> int:
    """Length of the flat response-function array of a batch."""
    last = pk.natm - 1
    cont = int(pk.arrays["cont_off"][last] + int(pk.arrays["ndep"][last]) * int(pk.arrays["nlam"][last]))
    return 4 * NPARAM * cont


def response_functions(dev: DeviceBatch, cfg: L.PyrhLteConfig, stream_ptr: int = 0,
                       loggf: bool = False):
    """Runs pyrh_lte_rf; returns the flat RF tensor (layout of the header),
    with loggf=True also the flat log gf RFs ([line][stokes][lambda] per
    atmosphere), and leaves the emergent Stokes vectors in dev.out."""
    import torch
    rf = torch.empty(rf_size(dev.pk), dtype=_real(dev), device=dev.out.device)
    gf = (torch.empty(4 * dev.nline * dev.pk.nlam_total, dtype=_real(dev), device=dev.out.device)
          if loggf else None)
    L.check(_lib().pyrh_lte_rf(C.byref(dev.struct), dev.lines_t.data_ptr(), dev.nline,
                               C.byref(cfg), dev.out.data_ptr(), rf.data_ptr(),
                               gf.data_ptr() if loggf else None, stream_ptr))
    return (rf, gf) if loggf else rf


def split_loggf_rf(pk: Packed, nline: int, gf) -> list:
    """Per-atmosphere [nline, 4, nlam] views of the flat log gf RFs."""
    out = []
    for p in range(pk.natm):
        o, nl = int(pk.arrays["lam_off"][p]), int(pk.arrays["nlam"][p])
        out.append(gf[4 * nline * o: 4 * nline * (o + nl)].reshape(nline, 4, nl))
    return out


def split_rf(pk: Packed, rf) -> list:
    """Per-atmosphere [4, 6, ndep, nlam] views of a flat RF array."""
    out = []
    for p in range(pk.natm):
        o = int(pk.arrays["cont_off"][p])
        nd, nl = int(pk.arrays["ndep"][p]), int(pk.arrays["nlam"][p])
        out.append(rf[4 * NPARAM * o: 4 * NPARAM * (o + nd * nl)].reshape(4, NPARAM, nd, nl))
    return out


def chi2_grad(dev: DeviceBatch, cfg: L.PyrhLteConfig, obs, weights, stream_ptr: int = 0,
              loggf: bool = False):
    """chi2[p] = sum w (S - obs)^2 and its gradient [6, total_depth] in one
    forward + adjoint pass (obs, weights: flat tensors laid out like dev.out);
    with loggf=True also d chi2 / d log10(gf) [natm, nline]."""
    import torch
    real = _real(dev)
    obs = obs.to(device=dev.out.device, dtype=real).contiguous()
    weights = weights.to(device=dev.out.device, dtype=real).contiguous()
    chi2 = torch.empty(dev.pk.natm, dtype=real, device=dev.out.device)
    grad = torch.empty(NPARAM * dev.pk.total_depth, dtype=real, device=dev.out.device)
    gf = torch.empty(dev.pk.natm * dev.nline, dtype=real, device=dev.out.device) if loggf else None
    L.check(_lib().pyrh_lte_chi2_grad(C.byref(dev.struct), dev.lines_t.data_ptr(), dev.nline,
                                      C.byref(cfg), obs.data_ptr(), weights.data_ptr(),
                                      dev.out.data_ptr(), chi2.data_ptr(), grad.data_ptr(),
                                      gf.data_ptr() if loggf else None, stream_ptr))
    g = grad.view(NPARAM, dev.pk.total_depth)
    return (chi2, g, gf.view(dev.pk.natm, dev.nline)) if loggf else (chi2, g)


def vjp(dev: DeviceBatch, cfg: L.PyrhLteConfig, dL_dstokes, stream_ptr: int = 0,
        loggf: bool = False):
    """sum over wavelengths and Stokes of dL/dS * dS/dx: [6, total_depth]
    (and with loggf=True the same for log10(gf) of every line: [natm, nline])."""
    import torch
    real = _real(dev)
    g = dL_dstokes.to(device=dev.out.device, dtype=real).contiguous()
    grad = torch.empty(NPARAM * dev.pk.total_depth, dtype=real, device=dev.out.device)
    gf = torch.empty(dev.pk.natm * dev.nline, dtype=real, device=dev.out.device) if loggf else None
    L.check(_lib().pyrh_lte_stokes_vjp(C.byref(dev.struct), dev.lines_t.data_ptr(), dev.nline,
                                       C.byref(cfg), g.data_ptr(), dev.out.data_ptr(),
                                       grad.data_ptr(), gf.data_ptr() if loggf else None,
                                       stream_ptr))
    out = grad.view(NPARAM, dev.pk.total_depth)
    return (out, gf.view(dev.pk.natm, dev.nline)) if loggf else out


def set_params(dev: DeviceBatch, params) -> None:
    """Writes a [6, total_depth] float64 tensor into the batch's per-depth
    arrays (T, v_los, v_mic, B, gamma_B, chi_B)."""
    for i, k in enumerate(PARAMS):
        dev.t[k].copy_(params[i])


def get_params(dev: DeviceBatch):
    import torch
    return torch.stack([dev.t[k] for k in PARAMS])


def _autograd_function():
    import torch

    class LteStokes(torch.autograd.Function):
        """Emergent Stokes vectors of a resident batch as a function of the
        [6, total_depth] atmosphere parameters; backward is the hand-written
        adjoint (pyrh_lte_stokes_vjp), which recomputes the forward sweep per
        pixel instead of storing it."""

        @staticmethod
        def forward(ctx, params, dev, cfg):
            set_params(dev, params.detach())
            dev.run(cfg)
            ctx.dev, ctx.cfg = dev, cfg
            ctx.save_for_backward(params.detach().clone())
            return dev.out.clone()

        @staticmethod
        def backward(ctx, g):
            (params,) = ctx.saved_tensors
            set_params(ctx.dev, params)
            grad = vjp(ctx.dev, ctx.cfg, g)
            return grad.to(params.dtype), None, None

    return LteStokes


_fn = None


def synthesize(dev: DeviceBatch, cfg: L.PyrhLteConfig, params):
    """Differentiable synthesis: Stokes (flat, like dev.out) from params
    [6, total_depth] (float64, on the device of dev)."""
    global _fn
    if _fn is None:
        _fn = _autograd_function()
    return _fn.apply(params, dev, cfg)
