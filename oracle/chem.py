"""TEST INFRASTRUCTURE: numpy restatement of the reference's chemical
equilibrium, the checker of chem.cu.  Nothing in the product imports it.

    read_molecule(text, abundance_set)      readMolecule   rh/readmolecule.c:66-240
    equilconstant(mol, T)                   equilconstant  rh/chemequil.c:456-535
    chem_equil(tab, mols, T, ne, nHtot, fn0_model)
                                            ChemicalEquilibrium rh/chemequil.c:107-390

`tab` has the layout of tests/golden/ltepops.npz (case 0).  Pinned to the
reference's own ChemicalEquilibrium output (tests/golden/chem.npz) in
tests/test_chem.py.
"""
from __future__ import annotations

import math

import numpy as np

from oracle import ltepops as LT

KBOLTZMANN = 1.380658E-23
EV = 1.60217733E-19
THETA0 = 5.03974756E+03
CM_TO_M = 1.0E-02
ERG_TO_JOULE = 1.0E-07
LG10 = 2.30258509299404568402
ELEMENT_ID = ("H ,HE,LI,BE,B ,C ,N ,O ,F ,NE,NA,MG,AL,SI,P ,S ,CL,AR,K ,CA,SC,TI,V ,CR,MN,FE,CO,"
              "NI,CU,ZN,GA,GE,AS,SE,BR,KR,RB,SR,Y ,ZR,NB,MO,TC,RU,RH,PD,AG,CD,IN,SN,SB,TE,I ,XE,"
              "CS,BA,LA,CE,PR,ND,PM,SM,EU,GD,TB,DY,HO,ER,TM,YB,LU,HF,TA,W ,RE,OS,IR,PT,AU,HG,TL,"
              "PB,BI,PO,AT,RN,FR,RA,AC,TH,PA,U ,NP,PU,AM,CM,BK,CF,ES").split(",")
FITS = ("KURUCZ_70", "KURUCZ_85", "SAUVAL_TATUM_84", "IRWIN_81", "TSUJI_73")


def _lines(text):
    for ln in text.splitlines():
        if not ln or ln[0] == "#" or not ln.split():
            continue
        yield ln


def read_molecule(text, abundance_set):
    it = _lines(text)
    m = {"id": next(it).split()[0], "charge": int(next(it).split()[0])}
    m["pt_index"], m["pt_count"] = [], []
    for tok in next(it).replace(",", " ").split():
        j = 0
        while j < len(tok) and tok[j].isdigit():
            j += 1
        count, el = (int(tok[:j]), tok[j:]) if j else (1, tok)
        el = el.upper()
        if len(el) == 1:
            el += " "
        idx = next(n for n, e in enumerate(ELEMENT_ID) if e in el)
        assert abundance_set[idx]
        m["pt_index"].append(idx)
        m["pt_count"].append(count)
    m["nnuclei"] = sum(m["pt_count"])
    m["ediss"] = float(next(it).split()[0]) * EV
    fit = next(it).split()[0]
    m["fit"] = next(i for i, f in enumerate(FITS) if f in fit)
    m["tmin"], m["tmax"] = (float(x) for x in next(it).split()[:2])
    for key in ("pf_coef", "eqc_coef"):
        tok = next(it).split()
        n = int(tok[0])
        m[key] = [float(x) for x in tok[1:n + 1]][::-1]
    return m


def equilconstant(m, T):
    if T < m["tmin"] or T > m["tmax"]:
        return 0.0
    c = m["eqc_coef"]
    fit = m["fit"]
    if fit in (0, 1):
        t = T if fit == 0 else T * 1.0E-4
        kT = KBOLTZMANN * T
        mk = m["nnuclei"] - 1 - m["charge"]
        eqc = c[0]
        for x in c[1:]:
            eqc = eqc * t + x
        eqc = math.exp(m["ediss"] / kT + eqc - 1.5 * mk * math.log(T))
        return eqc * (CM_TO_M * CM_TO_M * CM_TO_M) ** mk
    if fit in (2, 3):
        theta = THETA0 / T
        t = math.log10(theta)
        kT = KBOLTZMANN * T
        eqc = c[0]
        for x in c[1:]:
            eqc = eqc * t + x
        return math.exp(LG10 * ((m["ediss"] / EV) * theta - eqc)) * kT
    theta = THETA0 / T
    kT = KBOLTZMANN * T
    eqc = c[0]
    for x in c[1:]:
        eqc = eqc * theta + x
    eqc = (kT * kT) * math.exp(LG10 * (-eqc))
    return eqc * ((CM_TO_M * CM_TO_M * CM_TO_M) / ERG_TO_JOULE) ** (m["nnuclei"] - 1)


def _solve(A, b):
    x = np.linalg.solve(A, b)
    return x + np.linalg.solve(A, b - A @ x)     # one improvement step, as SolveLinearEq


def chem_equil(tab, mols, T, ne, nHtot, fn0_model=None):
    """(nmol [nmol, npoint], nHmin [npoint], nnuc [nnuclei, npoint], steps)."""
    fn0_model = fn0_model or {}
    nuc = sorted({e for m in mols for e in m["pt_index"]})
    Nn, Nm = len(nuc), len(mols)
    Neq = Nn + Nm
    CI = LT.C1
    npt = len(T)
    nmol = np.zeros((Nm, npt))
    nHmin = np.zeros(npt)
    nnuc = np.zeros((Nn, npt))
    steps = np.zeros(npt, int)
    index = {e: i for i, e in enumerate(nuc)}
    for k in range(npt):
        fn0 = np.zeros(Nn)
        a = np.zeros(Neq)
        for i, e in enumerate(nuc):
            if e in fn0_model:
                fn0[i] = fn0_model[e][k]
            else:
                fn0[i] = LT._fjk(tab, e, ne[k], T[k])[0][0]
            a[i] = tab["el_meta"][e, 2] * nHtot[k]
        PhiHmin = 0.25 * (CI / T[k]) ** 1.5 * math.exp(0.754 * EV / (KBOLTZMANN * T[k]))
        fHmin = ne[k] * fn0[0] * PhiHmin
        Phi = [equilconstant(m, T[k]) for m in mols]
        n = a.copy()
        prev = n.copy()
        dnmax, it = 0.0, 1
        while it <= 10:
            f = n - a
            df = np.eye(Neq)
            f[0] += fHmin * n[0]
            df[0, 0] += fHmin
            for i, m in enumerate(mols):
                saha = Phi[i]
                for e, c in zip(m["pt_index"], m["pt_count"]):
                    nu = index[e]
                    saha *= (fn0[nu] * n[nu]) ** float(c)
                    f[nu] += c * n[Nn + i]
                saha /= ne[k] ** float(m["charge"])
                f[Nn + i] -= saha
                for e, c in zip(m["pt_index"], m["pt_count"]):
                    nu = index[e]
                    df[nu, Nn + i] += c
                    df[Nn + i, nu] = -saha * (c / n[nu])
            n = n - _solve(df, f)
            nz = n != 0
            dnmax = np.max(np.abs((n[nz] - prev[nz]) / n[nz])) if nz.any() else 0.0
            prev = n.copy()
            if dnmax <= 1.0E-3:
                break
            it += 1
        nmol[:, k] = n[Nn:]
        nHmin[k] = ne[k] * (n[0] * PhiHmin)
        nnuc[:, k] = n[:Nn]
        steps[k] = -1 if dnmax > 1.0E-3 else min(it, 10)
    return nmol, nHmin, nnuc, steps
