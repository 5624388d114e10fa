"""TEST INFRASTRUCTURE: numpy restatement of the reference's hydrostatic
equilibrium, the checker of hse.cu.  Nothing in the product imports it.

    hse(tab, atoms, mols, atm_scale, scale, T, pg_top)    rh/rhf1d/pyrh_hse.c:67-399

per pass of a layer:
    get_ne            rh/rhf1d/pyrh_background.c:459-540  (ltepops.solve_ne, U_H = 1)
    LTEpops           rh/ltepops.c:33-109                 (no Debye lowering)
    ChemicalEquilibrium rh/chemequil.c:107-390            (chem.chem_equil; the model
                                                           atoms' neutral fractions and
                                                           population scaling here)
    pyrh_Background   rh/rhf1d/pyrh_background.c:144-457  (background.background
                                                           without Metal_bf, scattering
                                                           added)
    totals            rh/abundance.c:168-221              (totalAbund, wght_per_H)

and the same pieces for a run's set-up and pyrh's get_scales:
    equilibria(...)   SetLTEQuantities + ChemicalEquilibrium (background.c:155-170)
    continuum(...)    Background() at given wavelengths (passive atoms, SOLVE_NE NONE)
    convert_scales(...) convertScales, rh/rhf1d/multiatmos.c:100-177
    get_scales(...)   rh/rhf1d/pyrh_hse.c:402-554

`tab` has the layout of oracle.ltepops (tests/golden/ltepops.npz); `atoms`
is a list of dicts (elem, E, g, stage, cont rows, line rows, tab rows as
the background fixture keeps them), hydrogen among them; `mols` are
oracle.chem molecules.  Every layer of every atmosphere is computed point by
point in the reference's order; atmospheres run side by side.
"""
from __future__ import annotations

import math
import os
import re

import numpy as np

from . import background as OB
from . import chem as OC
from . import ltepops as OL

KBOLTZMANN = 1.380658E-23
AMU = 1.6605402E-27
KM_TO_M = 1.0E+03
LG10 = 2.30258509299404568402
HPLANCK = 6.6260755E-34
M_ELECTRON = 9.1093897E-31
PI = 3.14159265358979
C1 = (HPLANCK / (2.0 * PI * M_ELECTRON)) * (HPLANCK / KBOLTZMANN)
GRAVITY = math.exp(LG10 * 4.4) * 1.0E-02        # MULTIatmos, rh/rhf1d/multiatmos.c:70,80
NMAX_HSE_ITER = 50
ETA_LIMIT = 1.0E-2


def element_weights() -> np.ndarray:
    """The 99 atomic weights, read from the table in elements_host.cpp (the
    reference's rh/atomweights.h values)."""
    src = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                       "pyrh_gb300", "csrc", "elements_host.cpp")
    text = open(src).read()
    body = re.search(r"kElementWeight\[PYRH_NELEM\]\s*=\s*\{([^}]*)\}", text).group(1)
    w = np.array([float(x) for x in body.replace("\n", " ").split(",") if x.strip()])
    assert len(w) == 99
    return w


def totals(tab) -> tuple[float, float]:
    """(totalAbund, wght_per_H): sums in element order over the elements with
    an abundance."""
    w = element_weights()
    total = weight = 0.0
    for e in range(99):
        if tab["el_meta"][e, 1]:
            total += tab["el_meta"][e, 2]
            weight += tab["el_meta"][e, 2] * w[e]
    return total, weight


def lte_pops(atom, T, ne, ntotal):
    """LTEpops (ltepops.c:72-107) at every point: [nlevel, npoint]."""
    E, g, stage = atom["E"], atom["g"], atom["stage"]
    nl = len(E)
    n = np.zeros((nl, len(T)))
    cNe_T = 0.5 * ne * (C1 / T) ** 1.5
    s = np.ones(len(T))
    for i in range(1, nl):
        dE_kT = (E[i] - E[0]) / (KBOLTZMANN * T)
        v = g[i] / g[0] * np.exp(-dE_kT)
        for _ in range(int(stage[i]) - int(stage[0])):
            v = v / cNe_T
        n[i] = v
        s = s + v
    n[0] = ntotal / s
    for i in range(1, nl):
        n[i] = n[i] * n[0]
    return n


def neutral_fraction(atom, n, ntotal):
    """chemequil.c:224-236 for a passive atom."""
    f = np.zeros(n.shape[1])
    for j in range(len(atom["E"])):
        if atom["stage"][j] > 0:
            break
        f = f + n[j]
    return f / ntotal


def _layer_fixture(atoms, pops, T, ne, nHmin, nmol_by_id, vmicro_char, mol_present):
    """The background fixture's fields for one layer (points as depths)."""
    h = [a["elem"] for a in atoms].index(0)
    he = [a["elem"] for a in atoms].index(1) if 1 in [a["elem"] for a in atoms] else -1
    z = np.zeros(len(T))
    return {"lambda": np.array([500.0]), "T": T[None], "ne": ne[None], "nHmin": nHmin[None],
            "nH2": nmol_by_id.get("H2", z)[None], "nOH": nmol_by_id.get("OH", z)[None],
            "nCH": nmol_by_id.get("CH", z)[None], "mol_present": np.asarray(mol_present),
            "atoms_meta": np.array([(len(a["E"]), len(a["cont"]), len(a["lines"]), 0)
                                    for a in atoms]),
            "atoms_lev": np.concatenate([np.stack([a["E"], a["g"], a["stage"]], 1) for a in atoms]),
            "atoms_n": np.concatenate(pops)[None], "atoms_nstar": np.concatenate(pops)[None],
            "atoms_cont": np.concatenate([np.asarray(a["cont"]).reshape(-1, 8) for a in atoms]),
            "atoms_tab": np.concatenate([np.asarray(a["tab"]).reshape(-1, 2) for a in atoms]),
            "atoms_line": np.concatenate([np.asarray(a["lines"]).reshape(-1, 5) for a in atoms]),
            "misc": np.array([vmicro_char, he, h, len(atoms)], np.float64)}


def equilibria(tab, atoms, mols, T, ne, nH):
    """SetLTEQuantities and ChemicalEquilibrium at every point: the atoms'
    populations (list of [nlevel, npoint], scaled for the nuclei bound in
    molecules), the molecule densities [nmol, npoint] and nHmin [npoint]."""
    ntot = [tab["el_meta"][a["elem"], 2] * nH for a in atoms]
    pops = [lte_pops(a, T, ne, nt) for a, nt in zip(atoms, ntot)]
    fn0 = {a["elem"]: neutral_fraction(a, p, nt) for a, p, nt in zip(atoms, pops, ntot)}
    nmol, nHmin, nnuc, _ = OC.chem_equil(tab, mols, T, ne, nH, fn0)
    nuc = sorted({e for m in mols for e in m["pt_index"]})
    for i, e in enumerate(nuc):
        for m, a in enumerate(atoms):
            if a["elem"] == e:
                pops[m] = pops[m] * (nnuc[i] / ntot[m])
    return pops, nmol, nHmin


def continuum(tab, atoms, mols, mol_ids, lam, T, ne, nH, vmicro_char=5.0e3, fudge=None,
              hse=False):
    """Background() at the wavelengths lam (or, with hse, pyrh_Background:
    no metals, scattering added): chi, eta [nlam, npoint] and the protons."""
    pops, nmol, nHmin = equilibria(tab, atoms, mols, T, ne, nH)
    by_id = {mol_ids[i]: nmol[i] for i in range(len(mols))}
    present = [x in by_id for x in ("H2", "OH", "CH")]
    fx = _layer_fixture(atoms, pops, T, ne, nHmin, by_id, vmicro_char, present)
    fx["lambda"] = np.atleast_1d(np.asarray(lam, np.float64))
    chi, eta, _, _ = OB.background(fx, 0, add_scatter=hse, fudge=fudge, metals=not hse)
    h = [a["elem"] for a in atoms].index(0)
    return chi, eta, pops[h][-1]


def convert_scales(atm_scale, scale, T, ne, nH, chi, total_abund, wght, gravity=GRAVITY):
    """convertScales (rh/rhf1d/multiatmos.c:100-177) of one atmosphere:
    tau_ref, cmass [kg m^-2], height [m] from the given scale (log10 tau,
    log10 g cm^-2 or km) and the opacity at lambda_ref."""
    nd = len(T)
    rho = (AMU * wght) * np.asarray(nH)
    tau, cm, h = np.zeros(nd), np.zeros(nd), np.zeros(nd)
    if atm_scale == 0:
        tau = np.exp(LG10 * np.asarray(scale))
        cm[0] = (tau[0] / chi[0]) * rho[0]
        for k in range(1, nd):
            h[k] = h[k - 1] - 2.0 * (tau[k] - tau[k - 1]) / (chi[k - 1] + chi[k])
            cm[k] = cm[k - 1] + 0.5 * (rho[k - 1] + rho[k]) * (h[k - 1] - h[k])
    elif atm_scale == 1:
        cm = np.exp(LG10 * np.asarray(scale)) * (1.0E-03 / (1.0E-02 * 1.0E-02))
        tau[0] = chi[0] / rho[0] * cm[0]
        for k in range(1, nd):
            h[k] = h[k - 1] - 2.0 * (cm[k] - cm[k - 1]) / (rho[k - 1] + rho[k])
            tau[k] = tau[k - 1] + 0.5 * (chi[k - 1] + chi[k]) * (h[k - 1] - h[k])
    else:
        h = np.asarray(scale) * KM_TO_M
        cm[0] = (nH[0] * total_abund + ne[0]) * (KBOLTZMANN * T[0] / gravity)
        tau[0] = 0.5 * chi[0] * (h[0] - h[1])
        if tau[0] > 1.0:
            tau[0] = 0.0
        for k in range(1, nd):
            cm[k] = cm[k - 1] + 0.5 * (rho[k - 1] + rho[k]) * (h[k - 1] - h[k])
            tau[k] = tau[k - 1] + 0.5 * (chi[k - 1] + chi[k]) * (h[k - 1] - h[k])
    if atm_scale in (0, 1):
        if tau[1] > tau[0]:
            h0 = OL.linear(tau, h, 1.0)[0]
        else:
            h0 = OL.linear(tau[::-1], h[::-1], 1.0)[0]
        h = h - h0
    return tau, cm, h


def get_scales(tab, atoms, mols, mol_ids, atm_scale, scale, atm, lam_ref, vmicro_char=5.0e3):
    """pyrh.get_scales of an atmosphere [9, ndep] (compute1d's rows)."""
    cube = 1.0E-02 * 1.0E-02 * 1.0E-02
    T, ne, nH = atm[1], atm[2] / cube, atm[8] / cube
    chi, _, _ = continuum(tab, atoms, mols, mol_ids, [lam_ref], T, ne, nH, vmicro_char)
    tA, wght = totals(tab)
    return convert_scales(atm_scale, scale, T, ne, nH, chi[0], tA, wght)


def layer_pass(tab, atoms, mols, mol_ids, T, nH, vmicro_char, fudge=None):
    """One pass at a layer: (ne, opacity at 500 nm) at every point."""
    ne, _ = OL.solve_ne(tab, T, nH, unit_hydrogen_pf=True)
    chi, _, _ = continuum(tab, atoms, mols, mol_ids, [500.0], T, ne, nH, vmicro_char, fudge,
                          hse=True)
    return ne, chi[0]


def hse(tab, atoms, mols, mol_ids, atm_scale, scale, T, pg_top=0.1, vmicro_char=5.0e3,
        fudge=None):
    """ne, nHtot [m^-3], rho [kg m^-3], pg [Pa] and the passes per layer, each
    [natm, ndep], for atmospheres scale / T [natm, ndep]."""
    if atm_scale not in (0, 2):
        raise ValueError("atm_scale 0 or 2")
    scale = np.atleast_2d(np.asarray(scale, np.float64))
    T = np.atleast_2d(np.asarray(T, np.float64))
    natm, ndep = T.shape
    tA, wght = totals(tab)
    ne, nH, rho, pg, op = (np.zeros((natm, ndep)) for _ in range(5))
    passes = np.zeros((natm, ndep), int)
    pg[:, 0] = pg_top
    for k in range(ndep):
        if k == 0:
            nH[:, 0] = (pg[:, 0] / KBOLTZMANN / T[:, 0] - 0.0) / tA
        else:
            if atm_scale == 0:
                tk, tu = np.exp(LG10 * scale[:, k]), np.exp(LG10 * scale[:, k - 1])
                dP = GRAVITY * rho[:, k - 1] / op[:, k - 1] * (tk - tu)
            else:
                dP = GRAVITY * rho[:, k - 1] * (scale[:, k - 1] * KM_TO_M - scale[:, k] * KM_TO_M)
            pg[:, k] = pg[:, k - 1] + dP
            nH[:, k] = (pg[:, k] / KBOLTZMANN / T[:, k] - ne[:, k - 1]) / tA
        act = np.arange(natm)
        it = 0
        while len(act) and it < NMAX_HSE_ITER:
            old = nH[act, k].copy()
            r = (AMU * wght) * old
            n_e, chi = layer_pass(tab, atoms, mols, mol_ids, T[act, k], old, vmicro_char, fudge)
            rho[act, k], ne[act, k], op[act, k] = r, n_e, chi
            if k > 0:
                u = k - 1
                if atm_scale == 0:
                    tk, tu = np.exp(LG10 * scale[act, k]), np.exp(LG10 * scale[act, u])
                    dlogtau = np.log10(tk) - np.log10(tu)
                    beta1 = rho[act, u] / op[act, u] * tu
                    beta2 = r / chi * tk
                    pg[act, k] = pg[act, u] + LG10 * GRAVITY * (beta2 + beta1) / 2 * dlogtau
                else:
                    dP = GRAVITY * (scale[act, u] * KM_TO_M - scale[act, k] * KM_TO_M) * \
                        np.sqrt(r * rho[act, u])
                    pg[act, k] = pg[act, u] + dP
            new = (pg[act, k] / KBOLTZMANN / T[act, k] - n_e) / tA
            nH[act, k] = new
            it += 1
            eta = np.abs((new - old) / new)
            done = eta <= ETA_LIMIT
            passes[act[done], k] = it
            act = act[~done]
        passes[act, k] = -1
    return ne, nH, rho, pg, passes
