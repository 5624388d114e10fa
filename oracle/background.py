"""Background continuum oracle -- TEST INFRASTRUCTURE (not shipped, not used
by the product).

numpy restatement of the angle-independent part of the reference's
Background() (rh/background.c:329-460) for one atmosphere, from the
densities and atomic data its set-up leaves (the fields of the
`background` fixture):

  Thomson            rh/thomson.c:35-50
  Hminus_bf          rh/hydrogen.c:310-365  (Geltman table, natural spline)
  Hminus_ff          rh/hydrogen.c:367-545  (Stilley-Callaway table, bilinear)
  Hminus_ff_long     rh/hydrogen.c:553-615  (John 1988, beyond 9113 nm)
  OH_bf_opac         rh/ohchbf.c:53-398, CH_bf_opac rh/ohchbf.c:402-691
  Hydrogen_bf/_ff    rh/hydrogen.c:151-265, Gaunt_bf/_ff :269-305
  Rayleigh (H, He)   rh/rayleigh.c:33-100
  H2plus_ff          rh/hydrogen.c:797-935, Rayleigh_H2 :941-995,
  H2minus_ff         rh/hydrogen.c:621-790, bilinear :998-1020
  Metal_bf           rh/metal.c:71-171
  splineCoef/Eval    rh/spline.c (natural cubic spline), Hunt rh/hunt.c,
  Linear             rh/linear.c:22-51 (fudge factors), Planck rh/planck.c

The tables are read from pyrh_gb300/csrc/background_tables.h (published
data; the algorithms here are restated independently of the CUDA code).
"""
from __future__ import annotations

import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TABLES_H = os.path.join(os.path.dirname(HERE), "pyrh_gb300", "csrc", "background_tables.h")

CLIGHT = 2.99792458E+08
HPLANCK = 6.6260755E-34
KBOLTZMANN = 1.380658E-23
M_ELECTRON = 9.1093897E-31
Q_ELECTRON = 1.60217733E-19
EPSILON_0 = 8.854187817E-12
E_RYDBERG = 2.1798741E-18
EV = 1.60217733E-19
THETA0 = 5.03974756E+03
NM_TO_M = 1.0E-09
CM_TO_M = 1.0E-02
MICRON_TO_NM = 1.0E+03
MEGABARN_TO_M2 = 1.0E-22
PI = 3.14159265358979
LG10 = 2.30258509299404568402
LONG_WAVELENGTH = 1.0E6
RAYLEIGH_H2_LIMIT = 121.57

NAMES = ["Thomson", "Hminus_bf", "Hminus_ff", "OH_bf", "CH_bf", "Hydrogen_bf", "Hydrogen_ff",
         "Rayleigh_H", "Rayleigh_He", "H2plus_ff", "Rayleigh_H2", "H2minus_ff", "Metal_bf"]


def tables() -> dict:
    """The PYRH_BG_* lists of the tables header as arrays."""
    text = open(TABLES_H).read()
    out = {}
    for m in re.finditer(r"#define PYRH_BG_(\w+) \\\n(.*?)(?=\n#define|\n\n|\Z)", text, re.S):
        out[m.group(1)] = np.array([float(x) for x in m.group(2).replace("\\", "").split(",")])
    return out


T_ = tables()


def hunt(table, x):
    """Index j with table[j] <= x < table[j+1] (ascending table), the
    bracket Hunt and Locate return."""
    return int(np.clip(np.searchsorted(table, x, side="right") - 1, 0, len(table) - 1))


def spline_coef(x, y):
    """Second derivatives of the natural cubic spline (spline.c:38-66)."""
    n = len(x)
    M = np.zeros(n)
    q = np.zeros(n)
    u = np.zeros(n)
    hj = x[1] - x[0]
    D = (y[1] - y[0]) / hj
    for j in range(1, n - 1):
        hj1 = x[j + 1] - x[j]
        mu = hj / (hj + hj1)
        D1 = (y[j + 1] - y[j]) / hj1
        p = mu * q[j - 1] + 2
        q[j] = (mu - 1) / p
        u[j] = ((D1 - D) * 6 / (hj + hj1) - mu * u[j - 1]) / p
        hj, D = hj1, D1
    for j in range(n - 2, -1, -1):
        M[j] = q[j] * M[j + 1] + u[j]
    return M


def spline_eval(x, y, M, v):
    """spline.c:70-96 for an ascending table."""
    if v <= x[0]:
        return y[0]
    if v >= x[-1]:
        return y[-1]
    j = hunt(x, v)
    hj = x[j + 1] - x[j]
    fx = (v - x[j]) / hj
    fx1 = 1 - fx
    return (fx1 * y[j] + fx * y[j + 1] +
            (fx1 * (fx1 * fx1 - 1) * M[j] + fx * (fx * fx - 1) * M[j + 1]) * hj * hj / 6.0)


def linear(xt, yt, v):
    """linear.c:22-51 for one value."""
    asc = xt[1] > xt[0]
    lo, hi = (xt[0], xt[-1]) if asc else (xt[-1], xt[0])
    if v <= lo:
        return yt[0] if asc else yt[-1]
    if v >= hi:
        return yt[-1] if asc else yt[0]
    j = hunt(xt, v) if asc else len(xt) - 2 - hunt(xt[::-1], v)
    fx = (xt[j + 1] - v) / (xt[j + 1] - xt[j])
    return fx * yt[j] + (1 - fx) * yt[j + 1]


def frac_index(table, x):
    """Fractional table index, clamped to the ends (hydrogen.c:497-508)."""
    if x <= table[0]:
        return 0.0
    if x >= table[-1]:
        return float(len(table) - 1)
    j = hunt(table, x)
    return j + (x - table[j]) / (table[j + 1] - table[j])


def bilinear(ncol, nrow, f, x, y):
    """hydrogen.c:998-1020: f[j * ncol + i] at fractional (x = i, y = j)."""
    i = int(x)
    fx = x - i
    i1 = i if i == ncol - 1 else i + 1
    j = int(y)
    fy = y - j
    j1 = j if j == nrow - 1 else j + 1
    return ((1.0 - fx) * (1.0 - fy) * f[j * ncol + i] + fx * (1.0 - fy) * f[j * ncol + i1] +
            (1.0 - fx) * fy * f[j1 * ncol + i] + fx * fy * f[j1 * ncol + i1])


def gaunt_bf(lam, n_eff, charge):
    x = ((HPLANCK * CLIGHT) / (lam * NM_TO_M)) / (E_RYDBERG * charge * charge)
    x3 = x ** 0.33333333
    nsqx = 1.0 / (n_eff * n_eff * x)
    return 1.0 + 0.1728 * x3 * (1.0 - 2.0 * nsqx) - \
        0.0496 * x3 * x3 * (1.0 - (1.0 - nsqx) * 0.66666667 * nsqx)


def gaunt_ff(lam, charge, T):
    x = ((HPLANCK * CLIGHT) / (lam * NM_TO_M)) / (E_RYDBERG * charge * charge)
    x3 = x ** 0.33333333
    y = (2.0 * lam * NM_TO_M * KBOLTZMANN * T) / (HPLANCK * CLIGHT)
    g = 1.0 + 0.1728 * x3 * (1.0 + y) - 0.0496 * x3 * x3 * (1.0 + (1.0 + y) * 0.33333333 * y)
    return np.maximum(g, 1.0)


def planck(T, lam):
    hc_kla = (HPLANCK * CLIGHT) / (KBOLTZMANN * NM_TO_M * lam)
    l = NM_TO_M * lam
    twohnu3_c2 = (2.0 * HPLANCK * CLIGHT) / (l * l * l)
    x = hc_kla / T
    with np.errstate(over="ignore"):
        return np.where(x <= 150.0, twohnu3_c2 / (np.exp(np.minimum(x, 150.0)) - 1.0), 0.0)


class Atoms:
    """The fixture's atomic data split per atom."""

    def __init__(self, fx: dict, a: int):
        meta = fx["atoms_meta"]
        self.n_atoms = len(meta)
        lo = np.concatenate([[0], np.cumsum(meta[:, 0])])
        co = np.concatenate([[0], np.cumsum(meta[:, 1])])
        li = np.concatenate([[0], np.cumsum(meta[:, 2])])
        self.atoms = []
        for m in range(self.n_atoms):
            sl = slice(lo[m], lo[m + 1])
            self.atoms.append(dict(
                active=bool(meta[m, 3]), E=fx["atoms_lev"][sl, 0], g=fx["atoms_lev"][sl, 1],
                stage=fx["atoms_lev"][sl, 2].astype(int), n=fx["atoms_n"][a][sl],
                nstar=fx["atoms_nstar"][a][sl], cont=fx["atoms_cont"][co[m]:co[m + 1]],
                lines=fx["atoms_line"][li[m]:li[m + 1]]))
        self.tab = fx["atoms_tab"]
        self.h = int(fx["misc"][2])
        self.he = int(fx["misc"][1])
        self.vmicro_char = float(fx["misc"][0])


def rayleigh(lam, atom, vmicro_char):
    """Cross-section of rayleigh.c:33-100 (None where the routine adds
    nothing)."""
    lines = atom["lines"]
    if len(lines) == 0:
        return None
    lim = LONG_WAVELENGTH
    for l in lines:
        if int(l[0]) == 0:
            lim = min(lim, l[2] * (1.0 + l[3] * vmicro_char / CLIGHT))
    if not lam > lim:
        return None
    C = 2 * PI * (Q_ELECTRON / EPSILON_0) * (Q_ELECTRON / M_ELECTRON) / CLIGHT
    sigma_e = 8.0 * PI / 3.0 * (Q_ELECTRON / (np.sqrt(4.0 * PI * EPSILON_0) *
                                              (np.sqrt(M_ELECTRON) * CLIGHT))) ** 4
    fomega = 0.0
    for l in lines:
        red = l[2] * (1.0 + l[3] * vmicro_char / CLIGHT)
        if int(l[0]) == 0 and lam > red:
            lambda2 = 1.0 / ((lam / l[2]) ** 2 - 1.0)
            f = l[4] * (atom["g"][int(l[1])] / atom["g"][0]) * (l[2] * NM_TO_M) ** 2 / C
            fomega += f * lambda2 * lambda2
    return sigma_e * fomega


def background(fx: dict, a: int = 0, add_scatter: bool = False, fudge=None, metals=True):
    """(chi, eta, sca) [nspect, ndep] of atmosphere a, and the per-process
    contributions [13, 2, nspect, ndep] in the order of NAMES (opacity, then
    emissivity or scattering opacity).  fudge = (lambda [N], [3, N]) applies
    the reference's H-minus, scattering and metal fudge factors; metals
    False leaves Metal_bf out (the hydrostatic equilibrium's background,
    rh/rhf1d/pyrh_background.c:144-457)."""
    lam_all = fx["lambda"]
    T, ne = fx["T"][a], fx["ne"][a]
    nHmin, nH2, nOH, nCH = fx["nHmin"][a], fx["nH2"][a], fx["nOH"][a], fx["nCH"][a]
    mol = fx["mol_present"]
    at = Atoms(fx, a)
    H = at.atoms[at.h]
    He = at.atoms[at.he] if at.he >= 0 else None
    nH0, npr = H["n"][0], H["n"][-1]
    ns, nd = len(lam_all), len(T)
    comp = np.zeros((13, 2, ns, nd))
    chi_t = np.zeros((ns, nd))
    eta_t = np.zeros((ns, nd))
    sca_t = np.zeros((ns, nd))
    hm_M = spline_coef(T_["HMIN_BF_LAMBDA"], T_["HMIN_BF_ALPHA"])
    sigma_T = 8.0 * PI / 3.0 * (Q_ELECTRON / (np.sqrt(4.0 * PI * EPSILON_0) *
                                              (np.sqrt(M_ELECTRON) * CLIGHT))) ** 4
    metal_M = {}
    for la, lam in enumerate(lam_all):
        hc_kla = (HPLANCK * CLIGHT) / (KBOLTZMANN * NM_TO_M * lam)
        twohnu3_c2 = (2.0 * HPLANCK * CLIGHT) / (NM_TO_M * lam) ** 3
        ex = np.exp(-hc_kla / T)
        B = planck(T, lam)
        c = comp[:, :, la]
        c[0, 1] = ne * sigma_T
        # H- bound-free
        tl = T_["HMIN_BF_LAMBDA"]
        if tl[0] < lam < tl[-1]:
            al = spline_eval(tl, T_["HMIN_BF_ALPHA"], hm_M, lam) * 1.0e-21
            c[1, 0] = nHmin * (1.0 - ex) * al
            c[1, 1] = nHmin * twohnu3_c2 * ex * al
        # H- free-free
        tl = T_["HMIN_FF_LAMBDA"]
        if lam >= tl[-1]:
            lmu = lam / MICRON_TO_NM
            linv = 1.0 / lmu
            Cl = [0.0] * 6
            for n in range(1, 6):
                Cl[n] = lmu * lmu * T_["HMIN_FF_LONG_A"][n] + T_["HMIN_FF_LONG_B"][n] + linv * (
                    T_["HMIN_FF_LONG_C"][n] + linv * (T_["HMIN_FF_LONG_D"][n] + linv * (
                        T_["HMIN_FF_LONG_E"][n] + linv * T_["HMIN_FF_LONG_F"][n])))
            Ck = KBOLTZMANN * THETA0 * 1.0E-32
            for k in range(nd):
                s, tn, st = 0.0, 1.0, np.sqrt(THETA0 / T[k])
                for n in range(1, 6):
                    tn *= st
                    s += tn * Cl[n]
                c[2, 0, k] = s * nH0[k] * (ne[k] * Ck)
        else:
            li = frac_index(tl, lam)
            th = T_["HMIN_FF_THETA"]
            for k in range(nd):
                ti = frac_index(th, THETA0 / T[k])
                kap = bilinear(len(th), len(tl), T_["HMIN_FF_KAPPA"], ti, li)
                c[2, 0, k] = (nH0[k] * 1.0E-29) * (ne[k] * KBOLTZMANN * T[k]) * kap
        # OH and CH bound-free
        for slot, key, dens, present in ((3, "OH_BF", nOH, mol[1]), (4, "CH_BF", nCH, mol[2])):
            if not present:
                continue
            E = T_[key + "_EV"]
            Tt = T_[key + "_TEMP"]
            Eev = (HPLANCK * CLIGHT) / (lam * NM_TO_M) / EV
            if Eev < E[0] or Eev > E[-1]:
                continue
            ei = frac_index(E, Eev)
            for k in range(nd):
                if T[k] < Tt[0] or T[k] > Tt[-1]:
                    continue
                ti = frac_index(Tt, T[k])
                kap = np.exp(LG10 * bilinear(len(Tt), len(E), T_[key + "_LOGSIGMA"], ti, ei)) * \
                    CM_TO_M * CM_TO_M
                c[slot, 0, k] = dens[k] * (1.0 - ex[k]) * kap
                c[slot, 1, k] = dens[k] * twohnu3_c2 * ex[k] * kap
        # hydrogen bound-free and free-free
        if not H["active"]:
            sigma0 = 32.0 / (3.0 * np.sqrt(3.0)) * Q_ELECTRON ** 2 / (4.0 * PI * EPSILON_0) / \
                (M_ELECTRON * CLIGHT) * HPLANCK / (2.0 * E_RYDBERG)
            for cr in H["cont"]:
                i, j, lam0, lmin = int(cr[0]), int(cr[1]), cr[2], cr[3]
                if lam <= lam0 and lam >= lmin:
                    n_eff = np.sqrt(E_RYDBERG / (H["E"][j] - H["E"][i]))
                    g = gaunt_bf(lam, n_eff, H["stage"][i] + 1)
                    sig = sigma0 * n_eff * g * (lam / lam0) ** 3
                    gij = H["nstar"][i] / H["nstar"][-1] * ex
                    c[5, 0] += sig * (1.0 - ex) * H["n"][i]
                    c[5, 1] += twohnu3_c2 * gij * sig * npr
        C0 = Q_ELECTRON ** 2 / (4.0 * PI * EPSILON_0) / np.sqrt(M_ELECTRON)
        sigma = 4.0 / 3.0 * np.sqrt(2.0 * PI / (3.0 * KBOLTZMANN)) * C0 ** 3 / (HPLANCK * CLIGHT)
        nu3 = ((lam * NM_TO_M) / CLIGHT) ** 3
        c[6, 0] = sigma / np.sqrt(T) * nu3 * ne * npr * (1.0 - ex) * gaunt_ff(lam, 1, T)
        # Rayleigh by H and He
        s = rayleigh(lam, H, at.vmicro_char)
        if s is not None:
            c[7, 1] = s * H["n"][0]
        if He is not None:
            s = rayleigh(lam, He, at.vmicro_char)
            if s is not None:
                c[8, 1] = s * He["n"][0]
        # H + H+ free-free
        tl = T_["H2PLUS_FF_LAMBDA"]
        if lam < tl[-1]:
            li = frac_index(tl, lam)
            tt = T_["H2PLUS_FF_TEMP"]
            for k in range(nd):
                kap = bilinear(len(tt), len(tl), T_["H2PLUS_FF_KAPPA"], frac_index(tt, T[k]), li)
                c[9, 0, k] = (nH0[k] * 1.0E-29) * (npr[k] * 1.0E-20) * kap
        # H2 Rayleigh and H2- free-free
        if mol[0] and lam >= RAYLEIGH_H2_LIMIT:
            tl = T_["RAYLEIGH_H2_LAMBDA"]
            if lam <= tl[-1]:
                s = linear(tl, T_["RAYLEIGH_H2_SIGMA"], lam)
            else:
                l2 = 1.0 / (lam * lam)
                a_ = T_["RAYLEIGH_H2_COEF"]
                s = (a_[0] + (a_[1] + a_[2] * l2) * l2) * l2 * l2
            c[10, 1] = s * MEGABARN_TO_M2 * nH2
        tl = T_["H2MIN_FF_LAMBDA"]
        if mol[0] and lam < tl[-1]:
            li = frac_index(tl, lam)
            th = T_["H2MIN_FF_THETA"]
            for k in range(nd):
                if nH2[k] > 0.0:
                    kap = bilinear(len(th), len(tl), T_["H2MIN_FF_KAPPA"],
                                   frac_index(th, THETA0 / T[k]), li)
                    c[11, 0, k] = (nH2[k] * 1.0E-29) * (ne[k] * KBOLTZMANN * T[k]) * kap
        # metals (every atom after the first that is not active)
        for m in range(1, at.n_atoms if metals else 1):
            A = at.atoms[m]
            if A["active"]:
                continue
            for q, cr in enumerate(A["cont"]):
                i, j, lam0, lmin = int(cr[0]), int(cr[1]), cr[2], cr[3]
                if not (lam <= lam0 and lam >= lmin):
                    continue
                if int(cr[4]):
                    Z = A["stage"][j]
                    n_eff = Z * np.sqrt(E_RYDBERG / (A["E"][j] - A["E"][i]))
                    alpha = cr[5] * (lam / lam0) ** 3 * gaunt_bf(lam, n_eff, Z) / \
                        gaunt_bf(lam0, n_eff, Z)
                else:
                    off, nt = int(cr[7]), int(cr[6])
                    x, y = at.tab[off:off + nt, 0], at.tab[off:off + nt, 1]
                    key = (m, q)
                    if key not in metal_M:
                        metal_M[key] = spline_coef(x, y)
                    alpha = spline_eval(x, y, metal_M[key], lam)
                gij = A["nstar"][i] / A["nstar"][j] * ex
                c[12, 0] += alpha * (1.0 - ex) * A["n"][i]
                c[12, 1] += twohnu3_c2 * gij * alpha * A["n"][j]
        # totals in the order of background.c:341-460
        hf = mf = sf = 1.0
        if fudge is not None:
            fl, fv = fudge
            hf, sf, mf = (linear(fl, fv[r], lam) for r in range(3))
        chi = c[1, 0] + c[2, 0]
        eta = c[1, 1] + c[2, 0] * B
        chi, eta = chi * hf, eta * hf
        chi = chi + c[3, 0] + c[4, 0] + c[5, 0] + c[6, 0]
        eta = eta + c[3, 1] + c[4, 1] + c[5, 1] + c[6, 0] * B
        sca = c[0, 1] + c[7, 1] + c[8, 1]
        chi = chi + c[9, 0]
        eta = eta + c[9, 0] * B
        sca = sca + c[10, 1]
        chi = chi + c[11, 0] + c[12, 0] * mf
        eta = eta + c[11, 0] * B + c[12, 1] * mf
        sca = sca * sf
        if add_scatter:
            chi = chi + sca
        chi_t[la], eta_t[la], sca_t[la] = chi, eta, sca
    return chi_t, eta_t, sca_t, comp
