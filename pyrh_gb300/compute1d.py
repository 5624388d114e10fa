"""pyrh.compute1d on this library: the reference's Python surface for one
atmosphere (pyrh.pyx:537-668), with the synthesis running through the C ABI
(pyrh_lte_stokes, and pyrh_lte_rf for the log gf response functions).

    out = compute1d(cwd, mu, atm_scale, atmosphere, wave, setup=setup)
    sI, sQ, sU, sV, lam = out

Arguments, units and return values follow the reference:
  cwd          directory holding keyword.input (read here for STOKES_MODE,
               LAMBDA_REF, VMICRO_CHAR, VMACRO_TRESH, MAGNETO_OPTICAL)
  mu           cosine of the viewing angle
  atm_scale    0 = tau500, 1 = column mass, 2 = height (the depth scale of
               row 0; the heights of the depth points come with the set-up)
  atmosphere   [9, ndep] C-contiguous float64 rows: scale, T [K],
               ne [cm^-3], v_los [km/s], v_mic [km/s], B [G],
               inclination [rad], azimuth [rad], nH [cm^-3]
  wave         [nwave] vacuum nm
  loggf_ids, loggf_values   new log gf of the listed lines (line index in
               the set-up's line list)
  get_atomic_rfs   also return the log gf response functions of Stokes I
  get_populations  also return the active atoms' populations (none in an
               LTE synthesis: an empty tuple)
Returns (sI, sQ, sU, sV, lam) on the output grid (the caller's wavelengths
sorted and de-duplicated, lambda_ref dropped: pyrh_solveray.c:115-156); Q,
U, V are always returned, since pyrh sets atmos.Stokes in every mode
(pyrh_compute1dray.c:258), and are zero with STOKES_MODE = NO_STOKES.  With
get_atomic_rfs: ((sI, sQ, sU, sV, lam), rf) with rf [Nloggf + Nlam, nlw]
(pyrh.pyx:658-660); with get_populations the populations are appended
likewise.

Differences from the reference, by design:
  * the caller's arrays are never modified (the reference converts them to
    SI in place and back, pyrh_compute1dray.c:263-270, 351-357);
  * errors raise exceptions instead of exiting the process;
  * the log gf response functions are the exact derivatives
    dI/dlog10(gf) of the synthesis (the adjoint of the formal solution);
    the reference's analytical ones are about half of that (its
    approximate derivative equation, bezier_1D.c:416-490); the rows for
    lam_ids stay zero, as in the reference, which never fills them;
  * what the reference computes in its set-up before the formal solution
    (background continuum, stage densities and partition functions, the
    tau500-to-height conversion, line constants and Zeeman patterns) is
    taken from `setup` (an LteSetup): the wavelength grid is built here
    (pyrh_sort_lambda) and must equal the set-up's.
Arguments that change that set-up (lam_ids / lam_values, fudge_wave /
fudge_value, atomic_number / atomic_abundance) raise NotImplementedError.
"""
from __future__ import annotations

import os
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from . import grid as G
from . import lte

# rh/constant.h
CLIGHT = 2.99792458E+08
HPLANCK = 6.6260755E-34
Q_ELECTRON = 1.60217733E-19
EPSILON_0 = 8.854187817E-12
M_ELECTRON = 9.1093897E-31
PI = 3.14159265358979
NM_TO_M = 1.0E-09

# keyword.input entries this entry point reads, with the reference's
# defaults (rh/readinput.c:51-204)
KEYWORD_DEFAULTS = {"STOKES_MODE": "NO_STOKES", "LAMBDA_REF": "500.0",
                    "VMACRO_TRESH": "0.1", "MAGNETO_OPTICAL": "TRUE", "VMICRO_CHAR": None}


def read_keyword_input(path: str) -> dict:
    """keyword.input as a dict of upper-case keys to string values
    (KEY = VALUE lines; '#' starts a comment)."""
    out = {}
    with open(path) as f:
        for raw in f:
            line = raw.split("#", 1)[0].strip()
            if "=" not in line:
                continue
            k, v = line.split("=", 1)
            out[k.strip().upper()] = v.strip()
    return out


def _flag(v: str) -> bool:
    return v.strip().upper() in ("TRUE", "YES", "1")


@dataclass
class LteSetup:
    """The state the reference's set-up leaves for the formal solution of
    one atmosphere, on the global wavelength grid `lam` (vacuum nm,
    lambda_ref included): continuum chi_c, eta_c [nlam, ndep] (SI),
    heights [ndep] (m), proton density np [ndep] (m^-3), stage densities
    and ln U of each line's element line_pops [nline, 2, ndep], and the
    line list (line_const, zeeman, zeeman_n: the layout of
    pyrh_gb300.lte.make_lines).  With line_pops None, compute1d forms them
    on the device from the atmosphere (pyrh_line_pops) and the element
    tables: `elements` (a pyrh_gb300.ltepops.ElementTables), else the
    abundance and partition-function files the run in cwd names.  With
    chi_c, eta_c, height and np None, compute1d forms them on the device as
    the reference's Background() and convertScales do: LTE populations and
    chemical equilibrium of the run's passive atoms and molecules
    (`atoms_model`, a pyrh_gb300.equilibria.AtomsModel, else the files the
    run in cwd names), the continuum on the grid, the heights from the
    opacity at LAMBDA_REF."""
    lam: np.ndarray
    chi_c: np.ndarray | None
    eta_c: np.ndarray | None
    height: np.ndarray | None
    np: np.ndarray | None
    line_pops: np.ndarray | None
    line_const: np.ndarray
    zeeman: np.ndarray
    zeeman_n: np.ndarray
    elements: object = None
    atoms_model: object = None


def _line_constants(setup: LteSetup, loggf_ids, loggf_values) -> np.ndarray:
    """The line list with new log gf for the listed lines
    (kurucz.c:232-246: Aji, then Bji and Bij from it)."""
    lc = np.array(setup.line_const, np.float64, copy=True)
    if loggf_ids is None or loggf_values is None:
        return lc
    ids = np.asarray(loggf_ids)
    vals = np.asarray(loggf_values, np.float64)
    if ids.shape != vals.shape:
        raise ValueError("different number of 'loggf_ids' and 'loggf_values'")
    Cf = 2.0 * PI * (Q_ELECTRON / EPSILON_0) * (Q_ELECTRON / M_ELECTRON) / CLIGHT
    for i, v in zip(ids, vals):
        if not 0 <= int(i) < lc.shape[0]:
            raise ValueError(f"loggf id {int(i)} outside the line list")
        row = lc[int(i)]
        lam0 = row[0] * NM_TO_M
        gi, gj = row[3], row[4]
        Aji = Cf / (lam0 * lam0) * 10.0 ** v / gj
        Bji = (lam0 * lam0 * lam0) / (2.0 * HPLANCK * CLIGHT) * Aji
        row[7], row[8], row[9] = Aji, Bji, (gj / gi) * Bji
    return lc


def compute1d(cwd, mu, atm_scale, atmosphere, wave, loggf_ids=None, loggf_values=None,
              lam_ids=None, lam_values=None, fudge_wave=None, fudge_value=None,
              atomic_number=None, atomic_abundance=None, get_atomic_rfs=False,
              get_populations=False, *, setup: LteSetup, precision=L.PYRH_FP64,
              device="cuda"):
    import torch
    if lam_ids is not None or lam_values is not None:
        raise NotImplementedError("lam_ids / lam_values change the line list's wavelengths")
    continuum_here = all(x is None for x in (setup.chi_c, setup.eta_c, setup.height, setup.np))
    if not continuum_here and any(x is None for x in (setup.chi_c, setup.eta_c, setup.height,
                                                      setup.np)):
        raise ValueError("chi_c, eta_c, height and np are given together or not at all")
    fudge = None
    if fudge_wave is not None or fudge_value is not None:
        if not continuum_here:
            raise NotImplementedError("fudge_wave / fudge_value change the background opacity "
                                      "the caller's set-up holds")
        fudge = (np.asarray(fudge_wave, np.float64),
                 np.asarray(fudge_value, np.float64).reshape(3, -1))
    if (atomic_number is None) != (atomic_abundance is None):
        atomic_number = atomic_abundance = None   # the reference reads neither then
    if atomic_number is not None:
        if not continuum_here or setup.line_pops is not None or setup.elements is not None \
                or setup.atoms_model is not None:
            raise NotImplementedError("atomic_number / atomic_abundance change the set-up the "
                                      "caller holds")
    atmosphere = np.asarray(atmosphere, np.float64)
    if atmosphere.ndim != 2 or atmosphere.shape[0] != 9:
        raise ValueError("atmosphere must be [9, ndep]")
    if atm_scale not in (0, 1, 2):
        raise ValueError(f"atm_scale {atm_scale}")
    kw = dict(KEYWORD_DEFAULTS)
    kw.update(read_keyword_input(os.path.join(str(cwd), "keyword.input")))
    if kw["VMICRO_CHAR"] is None:
        raise ValueError("keyword.input has no VMICRO_CHAR (a required keyword)")
    stokes_mode = kw["STOKES_MODE"].upper()
    if stokes_mode not in ("NO_STOKES", "FULL_STOKES"):
        raise NotImplementedError(f"STOKES_MODE = {stokes_mode}")
    lambda_ref = float(kw["LAMBDA_REF"])
    vmicro_char = float(kw["VMICRO_CHAR"]) * 1e3
    vmacro_tresh = float(kw["VMACRO_TRESH"]) * 1e3
    mo = _flag(kw["MAGNETO_OPTICAL"])

    # units of the reference's set-up (pyrh_compute1dray.c:263-270)
    T, ne, vel = atmosphere[1], atmosphere[2] * 1e6, atmosphere[3] * 1e3
    vturb, B = atmosphere[4] * 1e3, atmosphere[5] * 1e-4
    gam, chi, nH = atmosphere[6], atmosphere[7], atmosphere[8] * 1e6
    moving = bool(np.any(np.abs(vel) >= vmacro_tresh))       # pyrh_compute1dray.c:273-278

    g = G.lte_grid(np.asarray(wave, np.float64), lambda_ref)
    if not np.array_equal(g.lam, np.asarray(setup.lam)):
        raise ValueError("the set-up's wavelength grid is not the one these wavelengths make")
    lc = _line_constants(setup, loggf_ids, loggf_values)
    lines, nline = lte.make_lines(lc, setup.zeeman, setup.zeeman_n)
    model = None
    if continuum_here:
        from . import equilibria as EQ
        model = setup.atoms_model if setup.atoms_model is not None else \
            EQ.AtomsModel.from_cwd(cwd, atomic_number, atomic_abundance, device)
        chi_c, eta_c, np_ = EQ.continuum(model, g.lam, T, ne, nH, fudge)
        iref = int(np.searchsorted(g.lam, lambda_ref))
        _, _, height = EQ.convert_scales(model, atm_scale, atmosphere[0], T, ne, nH, chi_c[iref])
        height = height[0]
    else:
        chi_c, eta_c, np_, height = setup.chi_c, setup.eta_c, setup.np, setup.height
    line_pops = setup.line_pops
    if line_pops is None:
        from . import ltepops as LP
        if setup.elements is not None:
            tab = setup.elements
        elif model is not None:
            tab = model.tables
        else:
            tab = LP.tables_from_files(cwd)
        line_pops = LP.line_pops(LP.DeviceTables(tab, device), T, ne, nH,
                                 lc[:, 1].astype(np.int32) - 1,
                                 lc[:, 2].astype(np.int32)).cpu().numpy()
    atm = dict(height=height, T=T, ne=ne, nHtot=nH, np=np_, vturb=vturb, vel=vel,
               B=B, gamma_B=gam, chi_B=chi, line_pops=line_pops, lam=g.lam,
               chi_c=chi_c, eta_c=eta_c)
    pk = lte.pack([atm], nline, precision)
    dev = lte.DeviceBatch(pk, lines, nline, device=device)
    cfg = lte.make_config(precision=precision, mu=mu, vmicro_char=vmicro_char,
                          magneto_optical=mo, moving=moving,
                          stokes_mode=(L.PYRH_FULL_STOKES if stokes_mode == "FULL_STOKES"
                                       else L.PYRH_NO_STOKES))
    rf_loggf = None
    if get_atomic_rfs:
        from . import rf as RF
        _, gf = RF.response_functions(dev, cfg, loggf=True)
        torch.cuda.synchronize()
        rf_loggf = gf.double().cpu().numpy().reshape(nline, 4, -1)
    else:
        dev.run(cfg)
        torch.cuda.synchronize()
    S = dev.out.double().cpu().numpy().reshape(4, -1)
    idx = g.out_index
    sI, sQ, sU, sV = (S[s][idx].copy() for s in range(4))
    output = (sI, sQ, sU, sV, g.lam[idx].copy())
    if get_atomic_rfs:
        ids = [] if loggf_ids is None else [int(i) for i in np.asarray(loggf_ids)]
        nlam_ids = 0 if lam_ids is None else len(lam_ids)
        rf = np.zeros((len(ids) + nlam_ids, len(idx)))
        for r, i in enumerate(ids):
            rf[r] = rf_loggf[i, 0][idx]
        output = (output, rf)
    if get_populations:
        output = (output, ())
    return output
