"""Synthetic atmospheres, line lists and wavelength grids for the benchmark
workloads (plain LTE synthesis of one 71-depth atmosphere; the batched form of
16384 perturbed atmospheres; the NLTE six-level atom cases).

The atmosphere model follows the stated generator: log tau500 uniform from -6
to +1, T = 5777 (0.75 (tau + 2/3))^0.25 + 2000 exp(-(log tau + 5)^2) K,
v_mic 1 km/s, B 1000 G, inclination 45 deg, azimuth 30 deg.  Atmosphere rows
follow pyrh.compute1d (reference pyrh.pyx:621-625): scale, T [K], ne [cm^-3],
v_los [km/s], v_mic [km/s], B [G], gamma [rad], chi [rad], nH [cm^-3].

Perturbations for the batched workloads: T offsets drawn N(0, 300 K) at the
nodes log tau = -2, -0.8, 0 and interpolated with a natural cubic spline
(held constant outside the node range); v_los uniform in [-3, 3] km/s;
B log-uniform in [10, 3000] G; cos(inclination) uniform in [-1, 1];
azimuth uniform in [0, pi).
"""
from __future__ import annotations

import numpy as np

# Physical constants with the values the reference uses (rh/constant.h:28-68).
CLIGHT = 2.99792458e8
HPLANCK = 6.6260755e-34
KBOLTZMANN = 1.380658e-23
EV = 1.60217733e-19
CM_TO_M = 1.0e-2

T_NODES = (-2.0, -0.8, 0.0)

# Two Zeeman-split Fe I-like lines: vacuum centre [nm], log gf, chi_low [eV],
# (J_low, J_up), (gL_low, gL_up) giving g_eff 1.67 and 2.49, terms, damping
# (log Grad, log GStark, log GvdW), orbital l of (low, up) for ABO broadening.
FE_LINES = (
    dict(lam_vac=630.15, loggf=-0.72, chi_low=3.65, J=(2.0, 2.0),
         gL=(1.835, 1.503), labels=("5Dsp3P z5P", "4s6D5s e5D"),
         damp=(8.08, -5.42, -7.54), orbital=(1, 0)),
    dict(lam_vac=630.25, loggf=-1.24, chi_low=3.69, J=(1.0, 0.0),
         gL=(2.487, 0.000), labels=("5Dsp3P z5P", "4s6D5s e5D"),
         damp=(8.08, -5.40, -7.54), orbital=(1, 0)),
)


def logtau_grid(ndep: int = 71) -> np.ndarray:
    return np.linspace(-6.0, 1.0, ndep)


def base_temperature(logtau: np.ndarray) -> np.ndarray:
    tau = 10.0 ** logtau
    return 5777.0 * (0.75 * (tau + 2.0 / 3.0)) ** 0.25 + \
        2000.0 * np.exp(-(logtau + 5.0) ** 2)


def natural_spline(xn, yn, x):
    """Natural cubic spline through (xn, yn), constant outside [xn0, xn-1]."""
    xn = np.asarray(xn, dtype=np.float64)
    yn = np.asarray(yn, dtype=np.float64)
    n = len(xn)
    h = np.diff(xn)
    A = np.zeros((n, n))
    r = np.zeros(n)
    A[0, 0] = A[-1, -1] = 1.0
    for i in range(1, n - 1):
        A[i, i - 1] = h[i - 1]
        A[i, i] = 2.0 * (h[i - 1] + h[i])
        A[i, i + 1] = h[i]
        r[i] = 6.0 * ((yn[i + 1] - yn[i]) / h[i] - (yn[i] - yn[i - 1]) / h[i - 1])
    M = np.linalg.solve(A, r)
    xc = np.clip(x, xn[0], xn[-1])
    j = np.clip(np.searchsorted(xn, xc) - 1, 0, n - 2)
    t0 = xn[j + 1] - xc
    t1 = xc - xn[j]
    hj = h[j]
    return (M[j] * t0 ** 3 + M[j + 1] * t1 ** 3) / (6.0 * hj) + \
        (yn[j] / hj - M[j] * hj / 6.0) * t0 + (yn[j + 1] / hj - M[j + 1] * hj / 6.0) * t1


def perturbations(n: int, seed: int, logtau: np.ndarray) -> dict:
    """Seeded per-atmosphere perturbations (T offsets, v_los, B, angles)."""
    rng = np.random.default_rng(seed)
    dT_nodes = rng.normal(0.0, 300.0, size=(n, len(T_NODES)))
    dT = np.stack([natural_spline(T_NODES, dT_nodes[i], logtau) for i in range(n)])
    vlos = rng.uniform(-3.0, 3.0, size=n)
    B = 10.0 ** rng.uniform(1.0, np.log10(3000.0), size=n)
    gamma = np.arccos(rng.uniform(-1.0, 1.0, size=n))
    chi = rng.uniform(0.0, np.pi, size=n)
    return dict(dT=dT, vlos=vlos, B=B, gamma=gamma, chi=chi)


def atmosphere_rows(logtau, T, ne_cm3, nH_cm3, vlos=0.0, vmic=1.0, B=1000.0,
                    gamma=np.deg2rad(45.0), chi=np.deg2rad(30.0)) -> np.ndarray:
    nd = len(logtau)
    atm = np.zeros((9, nd))
    atm[0] = logtau
    atm[1] = T
    atm[2] = ne_cm3
    atm[3] = vlos
    atm[4] = vmic
    atm[5] = B
    atm[6] = gamma
    atm[7] = chi
    atm[8] = nH_cm3
    return atm


def line_wavelengths(n_per_line: int = 201, half_width: float = 0.05,
                     centres=(630.15, 630.25)) -> np.ndarray:
    return np.concatenate([np.linspace(c - half_width, c + half_width, n_per_line)
                           for c in centres])


def kurucz_record(lam_air, loggf, code, E_low_cm, J_low, label_low, E_up_cm,
                  J_up, label_up, damp, gL_low, gL_up, l_low, l_up,
                  iso_log=0.0, hfs_log=0.0) -> str:
    """One line of a Kurucz-format list at the fixed columns that the
    reference reader uses (rh/kurucz.c:187-373): wavelength, log gf, code and
    first energy by whitespace, J at +35, labels at +41 and +69, second energy
    at +53, J at +63, damping at +79, isotope data at +106/+108/+117,
    hyperfine shifts at +123, Lande factors x1000 at +143, orbital l at +160.
    iso_log, hfs_log: log10 of the isotope and hyperfine fractions."""
    rec = (f"{lam_air:11.4f}{loggf:7.3f}{code:6.2f}{E_low_cm:11.3f}{J_low:5.1f} "
           f"{label_low:10s}  {E_up_cm:10.3f}{J_up:5.1f} {label_up:10s}"
           f"{damp[0]:6.2f}{damp[1]:6.2f}{damp[2]:6.2f}"
           f"{'SYNT':4s} 0 0{0:3d}{iso_log:6.3f}{0:3d}{hfs_log:6.3f}{0:5d}{0:5d}"
           f"{'':10s}{int(round(gL_low * 1000)):5d}{int(round(gL_up * 1000)):5d}"
           f"{'':7s}{l_low} {l_up}")
    assert rec[35:40].strip() and rec[143:153].strip() and len(rec) <= 171
    return rec


def vacuum_to_air(lam_vac: np.ndarray) -> np.ndarray:
    """Vacuum to air wavelength [nm] with the reference's formula for
    lambda >= 200 nm (rh/vacuumtoair.c:29-48)."""
    lam_vac = np.asarray(lam_vac, dtype=np.float64)
    sq = 1.0 / lam_vac ** 2
    red = 1.0 + 2.735182e-4 + (1.314182 + 2.76249e4 * sq) * sq
    return np.where(lam_vac >= 200.0, lam_vac / red, lam_vac)


def fe_linelist(lines=FE_LINES) -> str:
    out = []
    hc_cm = HPLANCK * CLIGHT / CM_TO_M          # J per cm^-1
    for L in lines:
        lam_air = float(vacuum_to_air(np.array([L["lam_vac"]]))[0])
        E_low = L["chi_low"] * EV / hc_cm
        E_up = E_low + 1.0e7 / lam_air
        out.append(kurucz_record(lam_air, L["loggf"], 26.00, E_low, L["J"][0],
                                 L["labels"][0], E_up, L["J"][1], L["labels"][1],
                                 L["damp"], L["gL"][0], L["gL"][1],
                                 L["orbital"][0], L["orbital"][1],
                                 L.get("iso_log", 0.0), L.get("hfs_log", 0.0)))
    return "\n".join(out) + "\n"


# ------------------------------------------------------------------------
# Batched synthetic workload built on the base atmosphere's hot-path inputs
# (continuum, stage densities, height scale from the reference's set-up for
# the base model, stored in pyrh_gb300/data/base_atmosphere.npz).  The
# temperature perturbations rescale the inputs that depend on T:
#   continuum opacity  ~ n(H-)   ~ T^-3/2 exp(0.754 eV / kT)  (Saha, H- bf)
#   continuum emission = opacity x Planck(T)                 (LTE)
#   Fe I stage density ~ T^-3/2 exp(7.87 eV / kT)            (Saha, minority)
# with ne, nH, height held fixed.  The result has the shapes and value
# distributions of the batched form; its spectra are not reference spectra.
# ------------------------------------------------------------------------

import os as _os

E_HMINUS = 0.754 * EV
E_FE_ION = 7.87 * EV
DATA = _os.path.join(_os.path.dirname(_os.path.abspath(__file__)), "data")


def load_base() -> dict:
    with np.load(_os.path.join(DATA, "base_atmosphere.npz")) as f:
        return {k: f[k] for k in f.files}


def planck_lambda(T, lam_nm):
    """Planck function B_nu(T) at wavelength lam [nm] (rh/planck.c:38-63)."""
    l = lam_nm * 1e-9
    x = HPLANCK * CLIGHT / (KBOLTZMANN * l * T)
    return (2.0 * HPLANCK * CLIGHT / l ** 3) / np.expm1(x)


def synthetic_batch(natm: int, seed: int = 2024, n_per_line: int = 112,
                    half_width: float = 0.05, dtype=np.float32, setup_dT: bool = False) -> dict:
    """natm perturbed copies of the base atmosphere on the 2 x n_per_line
    grid.  Arrays carry a leading atmosphere axis; continuum is
    [natm, ndep, nlam] (lambda fastest) in `dtype`.  With setup_dT, also the
    temperature derivatives of this set-up (dT_chi_c, dT_eta_c [natm, ndep,
    nlam]; dT_line_pops [natm, nline, 2, ndep]) for response functions that
    follow T through it; ne, nH, the proton density and the heights do not
    depend on T here."""
    base = load_base()
    lam = line_wavelengths(n_per_line, half_width)
    nd = len(base["T"])
    T0 = base["T"]
    # continuum of the base model interpolated to the new grid (it varies by
    # ~1e-4 across 0.2 nm)
    chi0 = np.stack([np.interp(lam, base["lam"][1:], base["chi_c"][1:, k]) for k in range(nd)])
    logtau = base["atm"][0]
    pert = perturbations(natm, seed, logtau)
    T = T0[None, :] + pert["dT"]
    T = np.maximum(T, 2500.0)
    r = T0[None, :] / T
    f_cont = r ** 1.5 * np.exp(E_HMINUS / KBOLTZMANN * (1.0 / T - 1.0 / T0[None, :]))
    f_fe = r ** 1.5 * np.exp(E_FE_ION / KBOLTZMANN * (1.0 / T - 1.0 / T0[None, :]))
    chi_c = (chi0[None, :, :] * f_cont[:, :, None]).astype(dtype)
    eta_c = (chi_c * planck_lambda(T[:, :, None], lam[None, None, :])).astype(dtype)
    ones = np.ones((natm, nd))
    out = dict(
        lam=lam, T=T, ne=ones * base["ne"], nHtot=ones * base["nHtot"], np=ones * base["np"],
        height=ones * base["height"], vturb=ones * base["vturb"],
        vel=ones * (pert["vlos"][:, None] * 1e3), B=ones * (pert["B"][:, None] * 1e-4),
        gamma_B=ones * pert["gamma"][:, None], chi_B=ones * pert["chi"][:, None],
        chi_c=chi_c, eta_c=eta_c,
        line_const=base["line_const"], zeeman=base["zeeman"], zeeman_n=base["zeeman_n"],
        vmicro_char=float(base["vmicro_char"]), mu=1.0,
    )
    lp = np.repeat(base["line_pops"][None], natm, axis=0)    # [natm, nline, 2, nd]
    lp[:, :, 0, :] *= f_fe[:, None, :]
    out["line_pops"] = lp
    if setup_dT:
        # d ln f / dT of the Saha factors above; d B / dT = B x e^x / ((e^x - 1) T)
        g_cont = -1.5 / T - E_HMINUS / (KBOLTZMANN * T * T)
        g_fe = -1.5 / T - E_FE_ION / (KBOLTZMANN * T * T)
        x = HPLANCK * CLIGHT / (KBOLTZMANN * lam[None, None, :] * 1e-9 * T[:, :, None])
        dlnB = x / (-np.expm1(-x) * T[:, :, None])
        dchi = chi_c.astype(np.float64) * g_cont[:, :, None]
        out["dT_chi_c"] = dchi.astype(dtype)
        out["dT_eta_c"] = (eta_c.astype(np.float64) * (g_cont[:, :, None] + dlnB)).astype(dtype)
        dlp = np.zeros_like(lp)
        dlp[:, :, 0, :] = lp[:, :, 0, :] * g_fe[:, None, :]
        out["dT_line_pops"] = dlp
    return out


# ------------------------------------------------------------------------
# Six-level Ca II-like model atom in RH .atom format (5 bound levels plus
# the continuum, 5 bound-bound CRD Voigt lines, 5 hydrogenic bound-free
# edges, electron-impact collisions tabulated on TEMP).  Level energies,
# log gf and collision strengths are drawn from a seeded table around Ca II
# like values (energies 0-11.9 eV, log gf in [-1.5, 0.2]).  Field layout as
# the reference reader expects it (rh/readatom.c:108-470).
# ------------------------------------------------------------------------

_CAII_LEVELS = (  # E [cm^-1], g, label, stage
    (0.0, 2.0, "CA II 3P6 4S 2SE"),
    (13650.0, 4.0, "CA II 3P6 3D 2DE 3"),
    (13711.0, 6.0, "CA II 3P6 3D 2DE 5"),
    (25192.0, 2.0, "CA II 3P6 4P 2PO 1"),
    (25414.0, 4.0, "CA II 3P6 4P 2PO 3"),
    (95752.0, 1.0, "CA III 3P6 1SE"),
)
# (upper, lower, Nlambda, qcore, qwing) of the five lines
_CAII_LINES = ((3, 0, 150, 15.0, 600.0), (4, 0, 150, 15.0, 600.0),
               (3, 1, 110, 4.0, 150.0), (4, 1, 110, 4.0, 150.0), (4, 2, 120, 4.0, 200.0))


def caii_like_atom(seed: int = 11, nlambda_scale: float = 1.0) -> str:
    rng = np.random.default_rng(seed)
    E = [lv[0] for lv in _CAII_LEVELS]
    # jitter bound excited levels by +-1 %, keep ordering
    for i in range(1, 5):
        E[i] *= 1.0 + rng.uniform(-0.01, 0.01)
    E[1], E[2] = sorted(E[1:3])
    E[3], E[4] = sorted(E[3:5])
    out = ["# Ca II-like six-level model atom (seeded synthetic table)",
           "  CA", "", "    6   5   5   0", ""]
    for i, (e, (_, g, lab)) in enumerate(zip(E, _CAII_LEVELS)):
        stage = 2 if i == 5 else 1
        out.append(f"  {e:12.3f}   {g:4.1f}   '{lab:<20s}'   {stage:d}   {i:d}")
    out.append("")
    for (j, i, nl, qc, qw) in _CAII_LINES:
        loggf = rng.uniform(-1.5, 0.2)
        f = 10.0 ** loggf / _CAII_LEVELS[i][1]
        nl = max(21, int(round(nl * nlambda_scale)) | 1)
        out.append(f"  {j:d}  {i:d}  {f:10.4E}   VOIGT  {nl:4d}   ASYMM  {qc:6.1f}  {qw:7.1f}"
                   f"  UNSOLD   1.00   0.00   1.00   0.00   1.50E+08   1.0E-00")
    out.append("")
    for i in range(5):
        alpha0 = 10.0 ** rng.uniform(-23.0, -21.2)
        edge_nm = 1.0e7 / (E[5] - E[i])
        out.append(f"  5  {i:d}  {alpha0:11.4E}  {max(9, int(round(30 * nlambda_scale))):4d}"
                   f"  HYDROGENIC  {0.35 * edge_nm:9.3f}")
    out.append("")
    temps = (3000.0, 5000.0, 7000.0, 15000.0, 50000.0, 100000.0)
    out.append(" TEMP    6   " + "".join(f"{t:11.1f}" for t in temps))
    out.append("")
    for j in range(1, 5):
        for i in range(j):
            om = 10.0 ** rng.uniform(0.0, 1.4) * np.linspace(0.9, 1.3, 6)
            out.append(f" OMEGA   {j:d}  {i:d}  " + "".join(f"{v:11.3E}" for v in om))
    out.append("")
    for i in range(5):
        ci = 10.0 ** rng.uniform(-17.5, -15.7)
        out.append(f" CI      {i:d}  5  " + "".join(f"{ci:11.3E}" for _ in temps))
    out.append("")
    out.append(" END")
    return "\n".join(out) + "\n"


# ------------------------------------------------------------------------
# Batched uneven NLTE workload: atmospheres derived from NLTE set-ups that
# the reference produced (its own background, LTE populations, collision
# rates, damping and continuum cross-sections for the six-level atom), each
# re-gridded to its own depth count (uniform in 50..150) and wavelength
# count (uniform in 700..1100), with the temperature and velocity
# perturbations of the batched LTE workload.  The temperature moves the
# set-up consistently to first order: LTE populations by Saha-Boltzmann at
# fixed n_e and total population, upward collision rates by detailed balance
# with the downward ones kept, thermal continuum emissivity by the Planck
# function, Doppler widths by the thermal speed.  The oracle solves the same
# inputs, so these atmospheres are parity cases in their own right.
# ------------------------------------------------------------------------

NLTE_DEPTH_LOG = ("T", "ne", "nHtot", "ntotal", "vbroad", "nstar", "n0", "adamp")
NLTE_DEPTH_LIN = ("vel", "vturb", "height", "C", "wphi", "atm")
NLTE_RESULTS = ("Gamma1", "J1", "n1", "n_final", "J_final", "I_out", "phi_sample",
                "phi_sample_la", "J0")
AMU = 1.6605402e-27
CA_MASS = 40.08


def _lin_weights(x0: np.ndarray, x: np.ndarray):
    """Indices and weights of linear interpolation from the increasing grid
    x0 onto x (clamped at the ends), shared by every row interpolated."""
    j = np.clip(np.searchsorted(x0, x, side="right") - 1, 0, len(x0) - 2)
    f = np.clip((x - x0[j]) / (x0[j + 1] - x0[j]), 0.0, 1.0)
    return j, f


def _interp_last(v: np.ndarray, jw, log: bool) -> np.ndarray:
    """Interpolate v along its last axis with _lin_weights (in log for
    positive quantities)."""
    j, f = jw
    a = np.asarray(v, np.float64)
    if log:
        a = np.log(np.maximum(a, 1e-300))
    r = a[..., j] * (1.0 - f) + a[..., j + 1] * f
    return np.ascontiguousarray(np.exp(r) if log else r)


def nlte_regrid_depth(fx: dict, nd: int) -> dict:
    """An NLTE set-up on nd depths, interpolated in depth index (logarithm of
    the positive quantities); results of the source run are dropped."""
    n0 = len(fx["T"])
    jw = _lin_weights(np.arange(n0, dtype=np.float64), np.linspace(0, n0 - 1, nd))
    out = {k: v for k, v in fx.items() if k not in NLTE_RESULTS}
    for k in NLTE_DEPTH_LOG + NLTE_DEPTH_LIN:
        out[k] = _interp_last(fx[k], jw, k in NLTE_DEPTH_LOG)
    bg = np.asarray(fx["background"], np.float64)              # [3, nspect, ndep]
    out["background"] = np.stack([_interp_last(bg[0], jw, True), _interp_last(bg[1], jw, True),
                                  _interp_last(np.maximum(bg[2], 0.0), jw, False)])
    m = np.array(fx["meta"]).copy()
    m[1] = nd
    out["meta"] = m
    return out


def nlte_regrid_lambda(fx: dict, ns: int) -> dict:
    """The same set-up on ns spectrum points: the sorted wavelength grid
    resampled in index, each transition's range mapped onto the new grid,
    the background interpolated in wavelength and the continuum
    cross-sections in wavelength along each edge."""
    lam0 = np.asarray(fx["lambda"], np.float64)
    n_old = len(lam0)
    s = (ns - 1) / (n_old - 1)
    xi = np.linspace(0.0, n_old - 1.0, ns)
    lam = np.interp(xi, np.arange(n_old), lam0)
    out = dict(fx)
    out["lambda"] = lam

    def span(nblue, nl):
        lo = int(np.ceil(nblue * s - 1e-9))
        hi = int(np.floor((nblue + nl - 1) * s + 1e-9))
        return lo, max(hi - lo + 1, 3 if hi >= lo else 0)

    lines = np.array(fx["lines"], np.float64).copy()
    for r in lines:
        lo, nl = span(int(r[7]), int(r[8]))
        r[7], r[8] = lo, min(nl, ns - lo)
    cont = np.array(fx["continua"], np.float64).copy()
    alpha_old = np.asarray(fx["alpha"], np.float64)
    alpha = []
    off = 0
    for r in cont:
        nb, nl, ao = int(r[2]), int(r[3]), int(r[6])
        lo, nl2 = span(nb, nl)
        nl2 = min(nl2, ns - lo)
        a_old = alpha_old[ao:ao + nl]
        alpha.append(np.exp(np.interp(lam[lo:lo + nl2], lam0[nb:nb + nl], np.log(a_old))))
        r[2], r[3], r[6] = lo, nl2, off
        off += nl2
    out["lines"], out["continua"] = lines, cont
    out["alpha"] = np.concatenate(alpha) if alpha else np.zeros(1)
    bg = np.asarray(fx["background"], np.float64)              # [3, nspect, ndep]
    jw = _lin_weights(lam0, lam)
    bgT = bg.transpose(0, 2, 1)                                # wavelength last
    out["background"] = np.stack([_interp_last(bgT[0], jw, True), _interp_last(bgT[1], jw, True),
                                  _interp_last(bgT[2], jw, False)]).transpose(0, 2, 1).copy()
    idx = np.clip(np.rint(xi).astype(np.int64), 0, n_old - 1)
    out["bgflags"] = np.asarray(fx["bgflags"])[idx]
    m = np.array(fx["meta"]).copy()
    m[0] = ns
    out["meta"] = m
    return out


def nlte_perturb(fx: dict, dT: np.ndarray, vlos_kms: float) -> dict:
    """Temperature offsets dT [ndep] and a line-of-sight velocity offset,
    with the set-up moved along with T (see the section comment)."""
    out = dict(fx)
    T0 = np.asarray(fx["T"], np.float64)
    T = np.maximum(T0 + dT, 2500.0)
    out["T"] = T
    atm = np.array(fx["atm"], np.float64).copy()
    atm[1] = T
    atm[3] = atm[3] + vlos_kms
    out["atm"] = atm
    out["vel"] = np.asarray(fx["vel"], np.float64) + vlos_kms * 1e3
    vb2 = np.asarray(fx["vbroad"], np.float64) ** 2 + 2.0 * KBOLTZMANN * (T - T0) / (CA_MASS * AMU)
    out["vbroad"] = np.sqrt(np.maximum(vb2, 1e4))
    E = np.asarray(fx["E"], np.float64)[:, None]
    stage = np.asarray(fx["stage"], np.float64)[:, None]
    nst = np.asarray(fx["nstar"], np.float64)
    lf = -E / KBOLTZMANN * (1.0 / T - 1.0 / T0)[None, :] + \
        1.5 * (stage - stage.min()) * np.log(T / T0)[None, :]
    w = nst * np.exp(lf - lf.max(axis=0, keepdims=True))
    nstar = w * (nst.sum(axis=0) / w.sum(axis=0))[None, :]
    out["nstar"] = nstar
    out["n0"] = nstar.copy()
    nl = nstar.shape[0]
    C = np.array(fx["C"], np.float64).copy()
    for i in range(nl):
        for j in range(i + 1, nl):
            C[j * nl + i] = C[i * nl + j] * nstar[j] / nstar[i]
    out["C"] = C
    bg = np.array(fx["background"], np.float64).copy()
    lam = np.asarray(fx["lambda"], np.float64)
    ratio = planck_lambda(T[None, :], lam[:, None]) / planck_lambda(T0[None, :], lam[:, None])
    bg[1] *= ratio
    out["background"] = bg
    return out


def nlte_batch(bases: list, natm: int, seed: int = 4096, depth_range=(50, 150),
               lambda_range=(700, 1100)) -> list:
    """natm NLTE atmospheres for the batched uneven workload: base set-up
    drawn from `bases`, depth count uniform in depth_range, spectrum points
    uniform in lambda_range, T nodes N(0, 300 K) at log tau -2, -0.8, 0
    (natural spline, constant outside) and v_los uniform in [-3, 3] km/s."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(natm):
        b = bases[int(rng.integers(len(bases)))]
        nd = int(rng.integers(depth_range[0], depth_range[1] + 1))
        ns = int(rng.integers(lambda_range[0], lambda_range[1] + 1))
        fx = nlte_regrid_lambda(nlte_regrid_depth(b, nd), ns)
        logtau = np.asarray(fx["atm"][0], np.float64)
        dT = natural_spline(T_NODES, rng.normal(0.0, 300.0, len(T_NODES)), logtau)
        out.append(nlte_perturb(fx, dT, float(rng.uniform(-3.0, 3.0))))
    return out
