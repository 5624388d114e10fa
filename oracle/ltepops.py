"""TEST INFRASTRUCTURE: numpy restatement of the reference's LTE ionisation
populations and electron density, the checker of ltepops.cu.  Nothing in
the product imports it.

    stage_pops(tab, e, T, ne, nHtot)   LTEpops_elem    rh/ltepops.c:116-166
    solve_ne(tab, T, nHtot, ne0)       Solve_ne        rh/solvene.c:55-141
                                       with getfjk     rh/solvene.c:145-198
    linear(Tpf, y, T)                  Linear          rh/linear.c:22-51

`tab` is a dict with the fixture's layout (tests/golden/ltepops.npz):
Tpf [npf], el_meta [99][4] (Nstage, abundance_set, abund, weight), el_pf
[sum Nstage][npf] (ln U), el_ionpot [sum Nstage] (J).  Pinned to the
reference's own LTEpops_elem and Solve_ne output in that fixture
(tests/test_ltepops.py).
"""
from __future__ import annotations

import numpy as np

HPLANCK = 6.6260755E-34
KBOLTZMANN = 1.380658E-23
M_ELECTRON = 9.1093897E-31
PI = 3.14159265358979
EV = 1.60217733E-19
C1 = (HPLANCK / (2.0 * PI * M_ELECTRON)) * (HPLANCK / KBOLTZMANN)
MAX_ELECTRON_ERROR = 1.0E-2
N_MAX_ELECTRON_ITERATIONS = 10


def linear(xt, yt, x):
    """Linear() of rh/linear.c: held at the ends of an ascending table."""
    x = np.atleast_1d(np.asarray(x, np.float64))
    out = np.empty_like(x)
    n = len(xt)
    for i, v in enumerate(x):
        if v <= xt[0]:
            out[i] = yt[0]
        elif v >= xt[n - 1]:
            out[i] = yt[n - 1]
        else:
            j = int(np.searchsorted(xt, v, side="right")) - 1
            fx = (xt[j + 1] - v) / (xt[j + 1] - xt[j])
            out[i] = fx * yt[j] + (1 - fx) * yt[j + 1]
    return out


def _rows(tab, e):
    ns = tab["el_meta"][:, 0].astype(int)
    off = int(ns[:e].sum())
    return off, int(ns[e])


def stage_pops(tab, e, T, ne, nHtot):
    """[Nstage, npoint] LTE stage populations of element e (0-based)."""
    off, ns = _rows(tab, e)
    T = np.asarray(T, np.float64)
    ne = np.asarray(ne, np.float64)
    abund = tab["el_meta"][e, 2]
    n = np.zeros((ns, len(T)))
    for k in range(len(T)):
        CT_ne = 2.0 * (C1 / T[k]) ** -1.5 / ne[k]
        s = 1.0
        n[0, k] = 1.0
        Uk = linear(tab["Tpf"], tab["el_pf"][off], T[k])[0]
        for i in range(1, ns):
            Ukp1 = linear(tab["Tpf"], tab["el_pf"][off + i], T[k])[0]
            n[i, k] = n[i - 1, k] * CT_ne * np.exp(
                Ukp1 - Uk - tab["el_ionpot"][off + i - 1] / (KBOLTZMANN * T[k]))
            s += n[i, k]
            Uk = Ukp1
        n[0, k] = abund * nHtot[k] / s
        for i in range(1, ns):
            n[i, k] *= n[0, k]
    return n


def _fjk(tab, e, ne, T):
    off, ns = _rows(tab, e)
    CT_ne = 2.0 * (C1 / T) ** -1.5 / ne
    f = np.zeros(ns)
    df = np.zeros(ns)
    f[0], s1, s2 = 1.0, 1.0, 0.0
    Uk = linear(tab["Tpf"], tab["el_pf"][off], T)[0]
    for j in range(1, ns):
        Ukp1 = linear(tab["Tpf"], tab["el_pf"][off + j], T)[0]
        f[j] = f[j - 1] * CT_ne * np.exp(Ukp1 - Uk - tab["el_ionpot"][off + j - 1] / (KBOLTZMANN * T))
        df[j] = -j * f[j] / ne
        s1 += f[j]
        s2 += df[j]
        Uk = Ukp1
    for j in range(ns):
        f[j] /= s1
        df[j] = (df[j] - f[j] * s2) / s1
    return f, df


def solve_ne(tab, T, nHtot, ne0=None, unit_hydrogen_pf=False):
    """Solve_ne at every point: from hydrogen's ionisation (ne0 None, H in
    LTE) or from ne0.  Returns (ne, steps) with steps -1 where it did not
    reach its limit.  unit_hydrogen_pf starts from U_H = 1 instead, as get_ne
    does (rh/rhf1d/pyrh_background.c:485-492)."""
    T = np.asarray(T, np.float64)
    nHtot = np.asarray(nHtot, np.float64)
    nelem = tab["el_meta"].shape[0]
    out = np.zeros(len(T))
    steps = np.zeros(len(T), int)
    for k in range(len(T)):
        if ne0 is None:
            off, _ = _rows(tab, 0)
            Uk = 0.0 if unit_hydrogen_pf else linear(tab["Tpf"], tab["el_pf"][off], T[k])[0]
            PhiH = 0.5 * (C1 / T[k]) ** 1.5 * np.exp(Uk + tab["el_ionpot"][off] / (KBOLTZMANN * T[k]))
            ne_old = (np.sqrt(1.0 + 4.0 * nHtot[k] * PhiH) - 1.0) / (2.0 * PhiH)
        else:
            ne_old = float(ne0[k])
        niter = 0
        ne_new, dne = ne_old, 0.0
        while niter < N_MAX_ELECTRON_ITERATIONS:
            error = ne_old / nHtot[k]
            s = 0.0
            for e in range(nelem):
                f, df = _fjk(tab, e, ne_old, T[k])
                if e == 0:
                    PhiHmin = 0.25 * (C1 / T[k]) ** 1.5 * np.exp(0.754 * EV / (KBOLTZMANN * T[k]))
                    error += ne_old * f[0] * PhiHmin
                    s -= (f[0] + ne_old * df[0]) * PhiHmin
                for j in range(1, len(f)):
                    akj = tab["el_meta"][e, 2] * j
                    error -= akj * f[j]
                    s += akj * df[j]
            ne_new = ne_old - nHtot[k] * error / (1.0 - nHtot[k] * s)
            dne = abs((ne_new - ne_old) / ne_old)
            ne_old = ne_new
            if dne <= MAX_ELECTRON_ERROR:
                break
            niter += 1
        out[k] = ne_new
        steps[k] = -1 if dne > MAX_ELECTRON_ERROR else niter + 1
    return out, steps
