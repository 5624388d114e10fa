"""Generates the golden fixtures in tests/golden/ from the compiled REFERENCE.

Run in a checkout where the reference sources are available (it builds
oracle/_ref/librh_ref.so from them with oracle/Makefile.ref):

    python tests/golden/make_golden.py [--only NAME ...]

Every number stored here comes out of the reference's own C code
(rhf1d(), hse(), Background(), RLKZeeman(), LTEpops_elem()), driven through
oracle/ref_harness.c.  Nothing in the product reads these files; tests do.

Fixtures (npz, float64):
  lte_c0          plain LTE polarized synthesis, 71 depths, 2 x 201 lambda,
                  mu=1 (MAGNETO_OPTICAL = FALSE: with TRUE the reference
                  writes four records into the three-record chip_c_lam buffer,
                  rh/readj.c:330 vs rh/sortlambda.c:574, and crashes)
  lte_edge        mu=0.5, velocity gradient, strong field, lambda points
                  outside every line window, duplicate and unsorted lambda
  lte_b0          B = 0 (polarizable lines with no splitting)
  lte_nostokes    C0 in STOKES_MODE = NO_STOKES
  lte_mixed       C0 with two unpolarizable lines (Armstrong's Voigt), one
                  alone in its window and one among the polarized lines
  lte_static      the lines of lte_mixed in a static atmosphere (VMACRO_TRESH
                  0.1 km/s, no velocity: atmos.moving FALSE), mu = 0.8
  lte_static_v    the same with velocities below the threshold (+-0.09 km/s),
                  which the reference then ignores
  lte_broadening  C0 with one line on Unsold's van der Waals broadening and
                  one with isotope and hyperfine fractions below one
  lte_loggf       the reference's analytical log gf RFs of Stokes I (NO_STOKES
                  C0, both lines) and central differences of its synthesis in
                  log gf
  lte_batch       6 atmospheres of the batched generator (2 x 112 lambda)
  lte_c0_dT, lte_edge_dT
                  temperature derivatives of the set-up inputs of lte_c0 /
                  lte_edge (continuum, stage densities and ln U, proton
                  density: central differences of harness_dump_lte at
                  T (1 +- 1e-5), every depth at once, since the set-up is
                  local in depth; interval lengths from convertScales'
                  tau_500 rule, rh/rhf1d/multiatmos.c:126-138), and the
                  reference's own temperature response functions: central
                  differences of rhf1d() (portable build) with T perturbed at
                  one depth, the definition of rh/rhf1d/rf_ray.c:205-293
  nlte_c1         six-level Ca II-like atom ACTIVE, 82 depths, 5 rays
  nlte_c4_50/120  the same atom on perturbed 50- and 120-depth atmospheres
                  with velocity fields and other wavelength counts
  nlte_static     nlte_c1 in a static atmosphere (VMACRO_TRESH 0.1 km/s, no
                  velocity): every wavelength takes the Feautrier solver
  background      the background continuum of the LTE set-up (Background()
                  without line lists) at 240 wavelengths from 120 to 20000
                  nm for the C0 atmosphere and a cooler one, with the
                  densities and atomic data it reads, and for C0 each
                  process alone
  ltepops         the element tables (Kurucz partition functions, ionisation
                  potentials, abundances) as the reference parsed them,
                  LTEpops_elem() of every element and Solve_ne() for three
                  atmospheres, one with abundance overrides
  chem            ChemicalEquilibrium() of the molecules of tests/molecules.input
                  (their files' text kept) on three atmospheres: the neutral
                  fractions it starts from and the densities it leaves
  scales          pyrh.get_scales() of the C0 atmosphere on its three depth
                  scales, at two reference wavelengths, and with abundance
                  overrides
  lte_scales      compute1d of C0 given on the column-mass and height scales
  hse             pyrh.hse() (ne, nHtot, rho, pg) on five atmospheres: C0 on
                  its log tau500 scale, a cooler one with another top
                  pressure, a height scale, abundance overrides, and opacity
                  fudge factors; the text of the model atoms it reads

stokes_ref comes from the reference as setup.py builds it on x86 (-DSIMDON,
SSE reciprocal-estimate 4x4 inverse); stokes_ref_portable from the same
sources without -DSIMDON (scalar float inverse, the Arm build).
"""
from __future__ import annotations

import argparse
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import ref_runner as rr  # noqa: E402
from pyrh_gb300 import workload as wl  # noqa: E402

PORTABLE = None
OPAC_STRIDE = 8      # keep the reference's total background record every 8th lambda


def base_c0(ref: rr.Reference, workdir: str, ndep: int = 71):
    logtau = wl.logtau_grid(ndep)
    T = wl.base_temperature(logtau)
    ne, nH = ref.hse(workdir, logtau, T)
    return logtau, T, ne / 1e6, nH / 1e6


def lte_case(ref, name, atm, wave, mu=1.0, magneto_optical="FALSE",
             extra=None, stokes_mode="FULL_STOKES", linelist=None, vmacro_tresh="0"):
    wd = rr.scratch_dir()
    rr.write_inputs(wd, linelist or wl.fe_linelist(), magneto_optical=magneto_optical,
                    stokes_mode=stokes_mode, vmacro_tresh=vmacro_tresh)
    lam_out, stokes, flag = ref.synth(wd, mu, atm, wave)
    _, stokes_portable, _ = PORTABLE.synth(wd, mu, atm, wave)
    dd = os.path.join(wd, "dump")
    ref.dump_lte(wd, mu, atm, wave, dd)
    d = rr.read_dump(dd)
    nspect = len(d["lambda"])
    sel = np.arange(0, nspect, OPAC_STRIDE)
    out = dict(
        atm=atm, wave=wave, mu=np.float64(mu),
        magneto_optical=np.int32(magneto_optical == "TRUE"),
        vmicro_char=np.float64(d["fmeta"][0]), lambda_ref=np.float64(d["fmeta"][1]),
        moving=np.int32(d["meta"][5]),
        lam_out=lam_out, stokes_ref=stokes, stokes_flag=np.int32(flag),
        stokes_ref_portable=stokes_portable,
        lam=d["lambda"], chi_c=d["cont"][0], eta_c=d["cont"][1],
        cont_flags=d["cont_flags"],
        height=d["height"], T=d["T"], ne=d["ne"], nHtot=d["nHtot"], np=d["np"],
        vturb=d["vturb"], vel=d["vel"], B=d["B"], gamma_B=d["gamma_B"],
        chi_B=d["chi_B"], cos_gamma=d["cos_gamma"], cos_2chi=d["cos_2chi"],
        sin_2chi=d["sin_2chi"],
        line_const=d["line_const"], line_pops=d["line_pops"],
        zeeman=d["zeeman"], zeeman_n=d["zeeman_n"],
        opac_idx=sel, tot_chi=d["tot_chi"][sel], tot_eta=d["tot_eta"][sel],
        tot_chip=d["tot_chip"][sel], tot_flags=d["tot_flags"],
    )
    if extra:
        out.update(extra)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    shutil.rmtree(wd, ignore_errors=True)
    print(f"{name}: {len(lam_out)} lambda, {atm.shape[1]} depths, "
          f"{os.path.getsize(path) / 1e3:.0f} kB")
    return out


def make_lte_c0(ref, wd):
    logtau, T, ne, nH = base_c0(ref, wd)
    atm = wl.atmosphere_rows(logtau, T, ne, nH)
    wave = wl.line_wavelengths(201, 0.05)
    lte_case(ref, "lte_c0", atm, wave)


def make_base_model(ref, wd):
    """Package data for the synthetic batched workloads: the reference's
    hot-path inputs for the base 71-depth atmosphere (continuum on the
    2 x 201 lambda grid, height scale, stage densities, line table)."""
    fx = np.load(os.path.join(HERE, "lte_c0.npz"))
    keep = ["atm", "lam", "chi_c", "eta_c", "height", "T", "ne", "nHtot", "np", "vturb",
            "vel", "B", "gamma_B", "chi_B", "line_const", "line_pops", "zeeman", "zeeman_n",
            "vmicro_char", "lambda_ref", "moving", "mu"]
    path = os.path.join(REPO, "pyrh_gb300", "data", "base_atmosphere.npz")
    os.makedirs(os.path.dirname(path), exist_ok=True)
    np.savez_compressed(path, **{k: fx[k] for k in keep})
    print(f"base_atmosphere: {os.path.getsize(path) / 1e3:.0f} kB")


def make_lte_edge(ref, wd):
    logtau, T, ne, nH = base_c0(ref, wd)
    atm = wl.atmosphere_rows(logtau, T, ne, nH, B=3000.0,
                             gamma=np.deg2rad(70.0), chi=np.deg2rad(120.0))
    atm[3] = np.linspace(-2.5, 1.5, len(logtau))      # velocity gradient
    atm[4] = np.linspace(2.0, 0.5, len(logtau))
    core = wl.line_wavelengths(21, 0.04)
    far = np.array([629.70, 629.85, 630.55, 630.80])    # outside 20 v_char/c
    wave = np.concatenate([core[::-1][:30], far, core[::-1][30:], core[5:8]])
    lte_case(ref, "lte_edge", atm, wave, mu=0.5)


UNPOLARIZED = dict(loggf=-1.0, chi_low=3.0, J=(2.0, 2.0), gL=(-0.099, -0.099),
                   labels=("unknown ab", "unknown ab"), damp=(8.08, -5.42, -7.54),
                   orbital=(1, 0))


def make_lte_modes(ref, wd):
    """NO_STOKES (pyrh keeps atmos.Stokes = TRUE, pyrh_compute1dray.c:258, so
    the lines stay polarizable and only the solver is scalar), and a list
    with two unpolarizable lines: labels without a term designation and
    Lande factors of -99 (kurucz.c:296, 384-387), which RLKProfile gives
    Armstrong's Voigt function (kurucz.c:824).  The one at 629.60 nm is the
    only line in its window (scalar Bezier3 there); the one at 630.20 nm
    shares its window with the two polarized lines (DELO-Bezier3, Stokes I
    opacity only)."""
    logtau, T, ne, nH = base_c0(ref, wd)
    atm = wl.atmosphere_rows(logtau, T, ne, nH)
    lte_case(ref, "lte_nostokes", atm, wl.line_wavelengths(101, 0.05),
             stokes_mode="NO_STOKES")
    lines = sorted([dict(UNPOLARIZED, lam_vac=629.60), dict(UNPOLARIZED, lam_vac=630.20),
                    *wl.FE_LINES], key=lambda L: L["lam_vac"])
    wave = np.concatenate([wl.line_wavelengths(41, 0.05, centres=(629.60,)),
                           np.linspace(630.10, 630.30, 121)])
    lte_case(ref, "lte_mixed", atm, wave, linelist=wl.fe_linelist(lines))


def make_lte_static(ref, wd):
    """A static atmosphere: VMACRO_TRESH = 0.1 km/s and no velocity, so
    atmos.moving stays FALSE (pyrh_compute1dray.c:261-278).  Wavelengths
    covered only by lines that are not polarizable are then not angle
    dependent and take the Feautrier solver (formal.c:96-101, 284-304)
    instead of scalar Bezier3; line shifts are ignored.  The line list of
    lte_mixed, mu = 0.8."""
    logtau, T, ne, nH = base_c0(ref, wd)
    atm = wl.atmosphere_rows(logtau, T, ne, nH, vlos=0.0)
    lines = sorted([dict(UNPOLARIZED, lam_vac=629.60), dict(UNPOLARIZED, lam_vac=630.20),
                    *wl.FE_LINES], key=lambda L: L["lam_vac"])
    wave = np.concatenate([wl.line_wavelengths(41, 0.05, centres=(629.60,)),
                           np.linspace(630.10, 630.30, 121)])
    lte_case(ref, "lte_static", atm, wave, mu=0.8, linelist=wl.fe_linelist(lines),
             vmacro_tresh="0.1")
    # velocities below the threshold: still static, and the reference
    # ignores them (no line shifts)
    atm = wl.atmosphere_rows(logtau, T, ne, nH)
    atm[3] = np.linspace(-0.09, 0.09, len(logtau))
    lte_case(ref, "lte_static_v", atm, wave, mu=0.8, linelist=wl.fe_linelist(lines),
             vmacro_tresh="0.1")


def make_lte_broadening(ref, wd):
    """Line-list variants of C0: the 630.15 nm line with orbital numbers
    (s, d) that no Barklem table covers, so the reader falls back to
    Unsold's van der Waals cross-section (kurucz.c:313-346), and the
    630.25 nm line with isotope and hyperfine fractions of 10^-0.3 and
    10^-0.1 (kurucz.c:359-365)."""
    logtau, T, ne, nH = base_c0(ref, wd)
    atm = wl.atmosphere_rows(logtau, T, ne, nH)
    lines = [dict(wl.FE_LINES[0], orbital=(0, 2)),
             dict(wl.FE_LINES[1], iso_log=-0.3, hfs_log=-0.1)]
    lte_case(ref, "lte_broadening", atm, wl.line_wavelengths(101, 0.05),
             linelist=wl.fe_linelist(lines))


def make_lte_loggf(ref, wd):
    """The reference's analytical log gf response functions of Stokes I
    (compute1d(..., loggf_ids, loggf_values, get_atomic_rfs=True); only its
    scalar solver propagates them, so STOKES_MODE = NO_STOKES,
    formal.c:214-235) for both lines of C0, and central differences of the
    same synthesis in log gf (the line list's values moved by +-h through
    the same override, kurucz.c:250-260) for comparison."""
    logtau, T, ne, nH = base_c0(ref, wd)
    atm = wl.atmosphere_rows(logtau, T, ne, nH)
    wave = wl.line_wavelengths(101, 0.05)
    w = rr.scratch_dir()
    rr.write_inputs(w, wl.fe_linelist(), stokes_mode="NO_STOKES")
    ids = np.array([0, 1], np.int32)
    base = np.array([L["loggf"] for L in wl.FE_LINES])
    lam, sI, rfs = ref.synth_loggf(w, 1.0, atm, wave, ids, base, True)
    steps = np.array([1e-2, 1e-3, 1e-4])
    jobs = []
    for l in range(2):
        for h in steps:
            for sgn in (1, -1):
                v = base.copy()
                v[l] += sgn * h
                jobs.append((w, ref.pyrh_path, 1.0, atm, wave, ids, v, False))
    res = ref.map(rr._loggf_job, jobs)
    fd = np.zeros((2, len(steps), len(lam)))
    i = 0
    for l in range(2):
        for b, h in enumerate(steps):
            fd[l, b] = (res[i][1] - res[i + 1][1]) / (2 * h)
            i += 2
    path = os.path.join(HERE, "lte_loggf.npz")
    np.savez_compressed(path, lam_out=lam, sI=sI, rf_analytic=rfs, fd_steps=steps, fd_loggf=fd,
                        loggf=base, atm=atm, wave=wave)
    shutil.rmtree(w, ignore_errors=True)
    print(f"lte_loggf: {len(lam)} lambda, {os.path.getsize(path) / 1e3:.0f} kB")


def make_lte_b0(ref, wd):
    logtau, T, ne, nH = base_c0(ref, wd)
    atm = wl.atmosphere_rows(logtau, T, ne, nH, B=0.0)
    wave = wl.line_wavelengths(31, 0.05)
    lte_case(ref, "lte_b0", atm, wave)


def make_lte_batch(ref, wd, n=6, seed=2024):
    logtau = wl.logtau_grid(71)
    T0 = wl.base_temperature(logtau)
    pert = wl.perturbations(n, seed, logtau)
    wave = wl.line_wavelengths(112, 0.05)
    jobs = [(wd, ref.pyrh_path, logtau, T0 + pert["dT"][i]) for i in range(n)]
    hse = ref.map(rr._hse_job, jobs)
    cases = []
    for i in range(n):
        ne, nH = hse[i]
        atm = wl.atmosphere_rows(logtau, T0 + pert["dT"][i], ne / 1e6, nH / 1e6,
                                 vlos=pert["vlos"][i], B=pert["B"][i],
                                 gamma=pert["gamma"][i], chi=pert["chi"][i])
        cases.append(lte_case(ref, f"_tmp_batch{i}", atm, wave))
    keys = [k for k in cases[0] if k not in ("opac_idx", "tot_chi", "tot_eta",
                                              "tot_chip", "tot_flags")]
    out = {k: np.stack([c[k] for c in cases]) for k in keys}
    path = os.path.join(HERE, "lte_batch.npz")
    np.savez_compressed(path, **out)
    for i in range(n):
        os.remove(os.path.join(HERE, f"_tmp_batch{i}.npz"))
    print(f"lte_batch: {n} atmospheres, {os.path.getsize(path) / 1e3:.0f} kB")


def tau500_len_dT(height, chi_ref, dchi_ref):
    """d|h_k - h_{k-1}| / dT_{k-1} and / dT_k (entry k >= 1) on a tau_500
    scale: convertScales sets h_k = h_{k-1} - 2 (tau_k - tau_{k-1}) /
    (chi_ref_{k-1} + chi_ref_k) (rh/rhf1d/multiatmos.c:126-138), so the
    interval length scales as 1 / (chi_ref_{k-1} + chi_ref_k)."""
    n = len(height)
    up, dn = np.zeros(n), np.zeros(n)
    dh = np.abs(height[1:] - height[:-1])
    den = chi_ref[:-1] + chi_ref[1:]
    up[1:] = -dh * dchi_ref[:-1] / den
    dn[1:] = -dh * dchi_ref[1:] / den
    return up, dn


FD_STEPS = np.array([3e-3, 1e-3, 3e-4])     # relative temperature steps


def lte_dT_case(ref, name, depths, eps=1e-5):
    fx = dict(np.load(os.path.join(HERE, name + ".npz")))
    atm, wave, mu = fx["atm"], fx["wave"], float(fx["mu"])
    wd = rr.scratch_dir()
    rr.write_inputs(wd, wl.fe_linelist())
    dumps = []
    for sgn in (1, -1):
        a = atm.copy()
        a[1] = atm[1] * (1 + sgn * eps)
        dd = os.path.join(wd, f"dump{sgn:+d}")
        ref.dump_lte(wd, mu, a, wave, dd)
        dumps.append(rr.read_dump(dd))
    h = eps * atm[1]
    dif = lambda f: (f(dumps[0]) - f(dumps[1])) / (2 * h)
    dchi = dif(lambda d: d["cont"][0])
    deta = dif(lambda d: d["cont"][1])
    iref = int(np.argmin(np.abs(fx["lam"] - fx["lambda_ref"])))
    up, dn = tau500_len_dT(fx["height"], fx["chi_c"][iref], dchi[iref])
    jobs, keys = [], []
    for k in depths:
        for rel in FD_STEPS:
            for sgn in (1, -1):
                a = atm.copy()
                a[1, k] += sgn * rel * atm[1, k]
                jobs.append((wd, PORTABLE.pyrh_path, mu, a, wave))
    res = PORTABLE.map(rr._synth_job, jobs)
    fd = np.zeros((len(depths), len(FD_STEPS), 4, len(res[0][0])))
    i = 0
    for a, k in enumerate(depths):
        for b, rel in enumerate(FD_STEPS):
            fd[a, b] = (res[i][1] - res[i + 1][1]) / (2 * rel * atm[1, k])
            i += 2
    out = dict(dT_chi_c=dchi, dT_eta_c=deta,
               dT_line_pops=dif(lambda d: d["line_pops"]), dT_np=dif(lambda d: d["np"]),
               dT_len_up=up, dT_len_dn=dn, fd_depths=np.array(depths, np.int32),
               fd_steps=FD_STEPS, fd_stokes=fd)
    path = os.path.join(HERE, name + "_dT.npz")
    np.savez_compressed(path, **out)
    shutil.rmtree(wd, ignore_errors=True)
    print(f"{name}_dT: {len(depths)} depths x {len(FD_STEPS)} steps, "
          f"{os.path.getsize(path) / 1e3:.0f} kB")


def make_lte_dT(ref, wd):
    lte_dT_case(ref, "lte_c0", [3, 20, 35, 45, 50, 55, 60, 65, 68, 70])
    lte_dT_case(ref, "lte_edge", [3, 30, 45, 55, 62, 68, 70])


NLTE_ATOM = "CaII_synth.atom"


def nlte_case(name, ndep=82, nlambda_scale=1.0, atom_seed=11, dT=None, vlos=0.0,
              mu_out=1.0, nrays=5, vmacro_tresh="0"):
    """NLTE MALI with the six-level Ca II-like atom ACTIVE: the reference's
    set-up state, one hand-made iteration (Gamma, J, statEquil), and the
    converged populations and emergent intensity (N_MAX_SCATTER = 0, Ng
    order 2 / delay 5 / period 5, ITER_LIMIT 1e-4, I_SUM = -1)."""
    root = rr.make_pyrh_root(NLTE_ATOM, wl.caii_like_atom(atom_seed, nlambda_scale))
    ref = rr.Reference(pyrh_path=root)
    wd = rr.scratch_dir()
    rr.write_inputs(wd, None, atoms=list(rr.PASSIVE_ATOMS) + [NLTE_ATOM], active=NLTE_ATOM,
                    nrays=nrays, nmax_iter=200, iter_limit="1.0E-4", ng_order=2, ng_delay=5,
                    ng_period=5, stokes_mode="NO_STOKES", nmax_scatter=0,
                    vmacro_tresh=vmacro_tresh)
    lt = wl.logtau_grid(ndep)
    T = wl.base_temperature(lt) + (0.0 if dT is None else dT)
    ne, nH = ref.hse(wd, lt, T)
    atm = wl.atmosphere_rows(lt, T, ne / 1e6, nH / 1e6, vlos=vlos, B=0.0)
    wave = np.array([393.4])
    ref.nlte(wd, mu_out, atm, wave, os.path.join(wd, "d0"), 0)
    ref.nlte(wd, mu_out, atm, wave, os.path.join(wd, "d1"), 1)
    d = rr.read_nlte_dump(os.path.join(wd, "d0"))
    d1 = rr.read_nlte_dump(os.path.join(wd, "d1"))
    nl = len(d["g"])
    out = {k: v for k, v in d.items() if k not in ("J0",)}
    assert not np.any(d["J0"]), "N_MAX_SCATTER = 0 leaves J = 0 before the first iteration"
    out.update(atm=atm, wave=wave, atom_text=np.array(wl.caii_like_atom(atom_seed, nlambda_scale)),
               n_final=d1["n_final"].reshape(nl, -1), J_final=d1["J_final"].reshape(d["J1"].shape),
               lam_out=d1["lam_out"], I_out=d1["I_out"],
               R_final_line=d1["R_final_line"].reshape(len(d["lines"]), 2, ndep),
               R_final_cont=d1["R_final_cont"].reshape(len(d["continua"]), 2, ndep))
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    shutil.rmtree(wd, ignore_errors=True)
    shutil.rmtree(root, ignore_errors=True)
    print(f"{name}: {len(d['lambda'])} lambda, {ndep} depths, "
          f"{os.path.getsize(path) / 1e3:.0f} kB")


def make_nlte(ref, wd):
    nlte_case("nlte_c1", ndep=82)
    lt50 = wl.logtau_grid(50)
    pert = wl.perturbations(2, 99, lt50)
    nlte_case("nlte_c4_50", ndep=50, nlambda_scale=0.8, dT=pert["dT"][0], vlos=1.5,
              mu_out=0.7)
    lt120 = wl.logtau_grid(120)
    pert = wl.perturbations(2, 98, lt120)
    nlte_case("nlte_c4_120", ndep=120, nlambda_scale=1.25, dT=pert["dT"][1], vlos=-2.0)


def make_nlte_static(ref, wd):
    """nlte_c1 with VMACRO_TRESH = 0.1 km/s and no velocity: atmos.moving
    stays FALSE, so no wavelength is angle dependent and every one takes
    the Feautrier solver (formal.c:96-101, 284-304), and the line profiles
    are stored once per wavelength (profile.c:154-170)."""
    nlte_case("nlte_static", ndep=82, vmacro_tresh="0.1")


def make_background(ref, wd):
    """Background() (background.c:139-631, no Kurucz list, no passive
    lines) on the C0 atmosphere and on a cooler one (T - 1500 K above log
    tau 0, at least 2600 K, so that the molecules and the low-temperature
    ends of the tables matter), both with their own hse() densities."""
    wave = np.geomspace(120.0, 20000.0, 240)
    out = {}
    for a, shift in enumerate((0.0, 1500.0)):
        logtau = wl.logtau_grid(71)
        T = wl.base_temperature(logtau)
        T = np.where(logtau < 0.0, np.maximum(T - shift, 2600.0), T)
        w = rr.scratch_dir()
        rr.write_inputs(w, None)
        ne, nH = ref.hse(w, logtau, T)
        atm = wl.atmosphere_rows(logtau, T, ne / 1e6, nH / 1e6)
        d = rr.read_background_dump(_dump_background(ref, w, atm, wave))
        if a == 0:
            for k in ("lambda", "mol_present", "misc", "atoms_meta", "atoms_lev", "atoms_cont",
                      "atoms_tab", "atoms_line", "comp"):
                out[k] = d[k]
        else:
            assert np.array_equal(d["lambda"], out["lambda"])
            assert np.array_equal(d["atoms_cont"], out["atoms_cont"])
        for k in ("T", "ne", "nHmin", "nH2", "nOH", "nCH", "atoms_n", "atoms_nstar", "cont"):
            out.setdefault(k, []).append(d[k])
        shutil.rmtree(w, ignore_errors=True)
    for k in ("T", "ne", "nHmin", "nH2", "nOH", "nCH", "atoms_n", "atoms_nstar", "cont"):
        out[k] = np.stack(out[k])
    path = os.path.join(HERE, "background.npz")
    np.savez_compressed(path, **out)
    print(f"background: {len(out['lambda'])} lambda, {os.path.getsize(path) / 1e3:.0f} kB")


def _dump_background(ref, workdir, atm, wave):
    outdir = os.path.join(workdir, "bg")
    ref.dump_background(workdir, 1.0, atm, wave, outdir)
    return outdir


def make_kurucz(ref, wd):
    """Inputs and outputs of the reference's Kurucz line-list reader
    (readKuruczLines, RLKZeeman, the Barklem and Unsold cross-sections) for
    the line lists of lte_c0 (Barklem s-p broadening), lte_broadening
    (orbital numbers no table covers: Unsold; isotope and hyperfine
    fractions) and lte_mixed (two lines that are not polarizable): the list
    text, each line's element data, hydrogen and helium, the Barklem tables
    as the reference parsed them, and the line constants and Zeeman patterns
    it produced."""
    logtau, T, ne, nH = base_c0(ref, wd)
    atm = wl.atmosphere_rows(logtau, T, ne, nH)
    wave = wl.line_wavelengths(21, 0.05)
    lists = {
        "c0": wl.fe_linelist(),
        "broadening": wl.fe_linelist([dict(wl.FE_LINES[0], orbital=(0, 2)),
                                      dict(wl.FE_LINES[1], iso_log=-0.3, hfs_log=-0.1)]),
        "mixed": wl.fe_linelist(sorted([dict(UNPOLARIZED, lam_vac=629.60),
                                        dict(UNPOLARIZED, lam_vac=630.20), *wl.FE_LINES],
                                       key=lambda L: L["lam_vac"])),
    }
    out = {}
    for name, text in lists.items():
        w = rr.scratch_dir()
        rr.write_inputs(w, text)
        dd = os.path.join(w, "dump")
        ref.dump_lte(w, 1.0, atm, wave, dd)
        d = rr.read_dump(dd)
        out[f"{name}_text"] = np.array(text)
        for k in ("line_const", "zeeman", "zeeman_n", "rlk_element", "rlk_hhe"):
            out[f"{name}_{k}"] = d[k]
        for t in ("sp", "pd", "df"):
            if f"barklem_{t}" in d:
                out[f"barklem_{t}"] = d[f"barklem_{t}"]
        shutil.rmtree(w, ignore_errors=True)
    path = os.path.join(HERE, "kurucz_lists.npz")
    np.savez_compressed(path, **out)
    print(f"kurucz_lists: {os.path.getsize(path) / 1e3:.0f} kB")


def make_ltepops(ref, wd):
    """Element tables as readAbundance() parsed them (partition functions and
    ionisation potentials of the Kurucz pf file, abundances of the abundance
    file), LTEpops_elem() of every element at the atmosphere's own electron
    density, and Solve_ne() from scratch (hydrogen in LTE) and from the
    given electron density, for the C0 atmosphere, a cooler one (T - 1500 K
    above log tau 0, at least 2600 K) and C0 with overridden abundances
    (entries 1 and 26 of the abundance file, as compute1d's atomic_number /
    atomic_abundance give them)."""
    cases = []
    for shift, ab_id, ab_val in ((0.0, [], []), (1500.0, [], []),
                                 (0.0, [1, 26], [12.0, 7.10])):
        logtau = wl.logtau_grid(71)
        T = wl.base_temperature(logtau)
        T = np.where(logtau < 0.0, np.maximum(T - shift, 2600.0), T)
        w = rr.scratch_dir()
        rr.write_inputs(w, None)
        ne, nH = ref.hse(w, logtau, T)
        atm = wl.atmosphere_rows(logtau, T, ne / 1e6, nH / 1e6)
        outdir = os.path.join(w, "lp")
        ref.dump_ltepops(w, atm, ab_id, ab_val, outdir)
        d = rr.read_ltepops_dump(outdir)
        d["ab_id"] = np.array(ab_id, np.int32)
        d["ab_val"] = np.array(ab_val, np.float64)
        cases.append(d)
        shutil.rmtree(w, ignore_errors=True)
    out = {"Tpf": cases[0]["Tpf"], "el_pf": cases[0]["el_pf"],
           "el_ionpot": cases[0]["el_ionpot"],
           "abundance_text": np.array(open(os.path.join(rr.REF_ROOT, "rh", "Atoms",
                                                        "abundance.input")).read())}
    for c in cases[1:]:
        assert np.array_equal(c["Tpf"], out["Tpf"])
    for k in ("el_meta", "T", "ne", "nHtot", "el_n", "ne_solved", "ne_warm"):
        out[k] = np.stack([c[k] for c in cases])
    out["ab_id"] = np.array([np.pad(c["ab_id"], (0, 2 - len(c["ab_id"])), constant_values=-1)
                             for c in cases])
    out["ab_val"] = np.array([np.pad(c["ab_val"], (0, 2 - len(c["ab_val"]))) for c in cases])
    path = os.path.join(HERE, "ltepops.npz")
    np.savez_compressed(path, **out)
    print(f"ltepops: {len(out['Tpf'])} pf temperatures, {out['el_meta'].shape[1]} elements, "
          f"{os.path.getsize(path) / 1e3:.0f} kB")


def make_chem(ref, wd):
    """ChemicalEquilibrium() with the molecules of tests/molecules.input
    (the reference's molecule files, their text kept here) on the C0
    atmosphere and on two cooler ones (T - 1000 K and T - 2000 K above log
    tau 0, at least 2200 K), each with its own hse() densities: the neutral
    fractions it starts from, the molecule and H- densities and the model
    atoms' totals it leaves."""
    mol_list = [ln.split()[0] for ln in open(os.path.join(rr.REF_ROOT, "tests", "molecules.input"))
                if ln.strip() and not ln.lstrip().startswith("#") and ".molecule" in ln]
    texts = [open(os.path.join(rr.REF_ROOT, "rh", "Molecules", m)).read() for m in mol_list]
    cases = []
    for shift in (0.0, 1000.0, 2000.0):
        logtau = wl.logtau_grid(71)
        T = wl.base_temperature(logtau)
        T = np.where(logtau < 0.0, np.maximum(T - shift, 2200.0), T)
        w = rr.scratch_dir()
        rr.write_inputs(w, None)
        ne, nH = ref.hse(w, logtau, T)
        atm = wl.atmosphere_rows(logtau, T, ne / 1e6, nH / 1e6)
        outdir = os.path.join(w, "chem")
        ref.dump_chem(w, atm, outdir)
        cases.append(rr.read_chem_dump(outdir))
        shutil.rmtree(w, ignore_errors=True)
    out = {"molecule_files": np.array(mol_list), "molecule_text": np.array(texts),
           "nuclei": cases[0]["nuclei"], "nuc_model": cases[0]["nuc_model"]}
    for c in cases[1:]:
        assert np.array_equal(c["nuclei"], out["nuclei"])
    for k in ("T", "ne", "nHtot", "fn0", "nmol", "nHmin", "ntot_model"):
        out[k] = np.stack([c[k] for c in cases])
    path = os.path.join(HERE, "chem.npz")
    np.savez_compressed(path, **out)
    print(f"chem: {len(mol_list)} molecules, nuclei {out['nuclei']}, "
          f"{os.path.getsize(path) / 1e3:.0f} kB")


def make_hse(ref, wd):
    """hse() with the run's passive atoms and molecules, cases: C0 (log
    tau500, pg_top 0.1 Pa); T - 1500 K above log tau 0 (at least 2600 K),
    pg_top 0.3 Pa; C0's temperatures on heights from 2000 to -100 km; C0 with
    the abundance overrides of the ltepops fixture (records 1 and 26); C0
    with H-minus and scattering fudge factors.  Keeps the atom files' text
    (the background fixture keeps the arrays the reference made of them)."""
    logtau = wl.logtau_grid(71)
    T0 = wl.base_temperature(logtau)
    Tc = np.where(logtau < 0.0, np.maximum(T0 - 1500.0, 2600.0), T0)
    height = np.linspace(2000.0, -100.0, 71)
    fw = np.array([300.0, 450.0, 700.0])
    fv = np.array([[1.30, 1.20, 1.10], [1.05, 1.10, 1.00], [1.0, 1.0, 1.0]])
    cases = [dict(atm_scale=0, scale=logtau, T=T0, pg_top=0.1),
             dict(atm_scale=0, scale=logtau, T=Tc, pg_top=0.3),
             dict(atm_scale=2, scale=height, T=T0, pg_top=0.1),
             dict(atm_scale=0, scale=logtau, T=T0, pg_top=0.1, ab_id=[1, 26], ab_val=[12.0, 7.10]),
             dict(atm_scale=0, scale=logtau, T=T0, pg_top=0.1, fudge_wave=fw, fudge_value=fv)]
    out = {k: [] for k in ("atm_scale", "scale", "T", "pg_top", "ne", "nHtot", "rho", "pg")}
    for c in cases:
        w = rr.scratch_dir()
        rr.write_inputs(w, None)
        ne, nH, rho, pg = ref.hse_full(w, c["atm_scale"], c["scale"], c["T"], c["pg_top"],
                                       c.get("fudge_wave"), c.get("fudge_value"),
                                       c.get("ab_id"), c.get("ab_val"))
        shutil.rmtree(w, ignore_errors=True)
        for k, v in (("atm_scale", c["atm_scale"]), ("scale", c["scale"]), ("T", c["T"]),
                     ("pg_top", c["pg_top"]), ("ne", ne), ("nHtot", nH), ("rho", rho),
                     ("pg", pg)):
            out[k].append(v)
    out = {k: np.array(v) for k, v in out.items()}
    out["ab_case"] = np.array(3)
    out["ab_id"], out["ab_val"] = np.array([1, 26], np.int32), np.array([12.0, 7.10])
    out["fudge_case"] = np.array(4)
    out["fudge_wave"], out["fudge_value"] = fw, fv
    out["atom_files"] = np.array(rr.PASSIVE_ATOMS)
    out["atom_text"] = np.array([open(os.path.join(rr.REF_ROOT, "rh", "Atoms", a)).read()
                                 for a in rr.PASSIVE_ATOMS])
    path = os.path.join(HERE, "hse.npz")
    np.savez_compressed(path, **out)
    print(f"hse: {len(cases)} atmospheres, {os.path.getsize(path) / 1e3:.0f} kB")


def make_scales(ref, wd):
    """get_scales() on the C0 atmosphere given on its log tau500 scale, on
    the column-mass scale and on the height scale that run returned, at
    lambda_ref 500 nm; on log tau500 at 450 nm; and with the abundance
    overrides of the ltepops fixture.  The run reads the two Fe I lines'
    Kurucz list (get_scales requires one), which adds no opacity at 450 or
    500 nm."""
    logtau, T, ne, nH = base_c0(ref, wd)
    atm = wl.atmosphere_rows(logtau, T, ne, nH)
    w = rr.scratch_dir()
    rr.write_inputs(w, wl.fe_linelist())    # get_scales reads a Kurucz list (cwd/KURUCZ_DATA)
    tau0, h0, cm0 = ref.get_scales(w, 0, logtau, atm, 500.0)
    g_cm2 = 1.0e-3 / (1.0e-2 * 1.0e-2)                  # G_TO_KG / SQ(CM_TO_M)
    cases = [(0, logtau, 500.0, None, None), (1, np.log10(cm0 / g_cm2), 500.0, None, None),
             (2, h0 / 1.0e3, 500.0, None, None), (0, logtau, 450.0, None, None),
             (0, logtau, 500.0, [1, 26], [12.0, 7.10])]
    out = {k: [] for k in ("atm_scale", "scale", "lam_ref", "tau", "height", "cmass")}
    for sc, scale, lr, ai, av in cases:
        tau, h, cm = ref.get_scales(w, sc, scale, atm, lr, ai, av)
        for k, v in (("atm_scale", sc), ("scale", scale), ("lam_ref", lr), ("tau", tau),
                     ("height", h), ("cmass", cm)):
            out[k].append(v)
    shutil.rmtree(w, ignore_errors=True)
    out = {k: np.array(v) for k, v in out.items()}
    out["atm"] = atm
    out["ab_case"] = np.array(4)
    path = os.path.join(HERE, "scales.npz")
    np.savez_compressed(path, **out)
    print(f"scales: {len(cases)} cases, {os.path.getsize(path) / 1e3:.0f} kB")


def make_lte_scales(ref, wd):
    """compute1d of the C0 atmosphere and its two Fe I lines given on the
    column-mass scale (log10 g cm^-2) and on the height scale (km) that
    get_scales made of it (fixture scales), by both reference builds."""
    d = np.load(os.path.join(HERE, "scales.npz"))
    atm0 = d["atm"]
    wave = wl.line_wavelengths(201, 0.05)
    g_cm2 = 1.0e-3 / (1.0e-2 * 1.0e-2)
    out = {"wave": wave}
    for sc, row in ((1, np.log10(d["cmass"][0] / g_cm2)), (2, d["height"][0] / 1.0e3)):
        atm = atm0.copy()
        atm[0] = row
        w = rr.scratch_dir()
        rr.write_inputs(w, wl.fe_linelist())
        lam_out, stokes, _ = ref.synth(w, 1.0, atm, wave, atm_scale=sc)
        _, stokes_p, _ = PORTABLE.synth(w, 1.0, atm, wave, atm_scale=sc)
        shutil.rmtree(w, ignore_errors=True)
        out[f"atm_{sc}"], out[f"stokes_ref_{sc}"] = atm, stokes
        out[f"stokes_ref_portable_{sc}"], out["lam_out"] = stokes_p, lam_out
    path = os.path.join(HERE, "lte_scales.npz")
    np.savez_compressed(path, **out)
    print(f"lte_scales: {os.path.getsize(path) / 1e3:.0f} kB")


MAKERS = {"lte_c0": make_lte_c0, "base_model": make_base_model, "lte_edge": make_lte_edge,
          "lte_b0": make_lte_b0, "lte_batch": make_lte_batch, "lte_dT": make_lte_dT,
          "lte_modes": make_lte_modes, "lte_loggf": make_lte_loggf,
          "lte_static": make_lte_static, "lte_broadening": make_lte_broadening,
          "nlte": make_nlte, "nlte_static": make_nlte_static, "kurucz": make_kurucz,
          "background": make_background, "ltepops": make_ltepops, "chem": make_chem,
          "hse": make_hse, "scales": make_scales, "lte_scales": make_lte_scales}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", nargs="*", default=None)
    args = ap.parse_args()
    global PORTABLE
    ref = rr.Reference()
    PORTABLE = rr.Reference(lib_path=rr.REF_LIB_PORTABLE)
    wd = rr.scratch_dir()
    rr.write_inputs(wd, None)
    for name, fn in MAKERS.items():
        if args.only and name not in args.only:
            continue
        fn(ref, wd)
    shutil.rmtree(wd, ignore_errors=True)


if __name__ == "__main__":
    main()
