#!/usr/bin/env python
"""Benchmark of the batched polarized LTE synthesis on GB300.

Workload (the batched precision form): 16384 atmospheres with 71 depth
points, perturbed from the base model (T nodes +-300 K, v_los, B, angles),
two Zeeman-split Fe I-like lines with 112 wavelengths each (224 per
atmosphere), mu = 1, FP32 DELO-Bezier3 Stokes.  One step = one launch of
pyrh_lte_stokes over the whole batch.  Inputs (continuum 2.1 GB) are larger
than L2, so no flush is needed between steps.

Prints one JSON line (rank 0).  --impl reference times the CPU path instead.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = ("pixel·λ·μ formal solutions/s and RF gradients/s vs plain FP64 "
          "GPU, at 1e-4 rel err")
UNIT = "pixel*lambda*mu/s"
WORKLOAD = "batched LTE Stokes synthesis: 16384 atm x 71 depths x 2x112 lambda, mu=1, FP32"
# ncu figures of the synthesis kernel (DRAM traffic, FP32 flops), recorded
# with the digest of the kernel sources they were measured on; reported only
# while those sources are unchanged.
NCU_TRAFFIC = os.path.join(HERE, "pyrh_gb300", "data", "ncu_traffic.json")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--natm", type=int, default=16384)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-rf", action="store_true")
    ap.add_argument("--skip-nlte", action="store_true")
    ap.add_argument("--skip-background", action="store_true")
    ap.add_argument("--skip-accuracy", action="store_true")
    ap.add_argument("--rf-natm", type=int, default=4096)
    ap.add_argument("--nlte-natm", type=int, default=1024)
    return ap.parse_args()


def config_dict(natm):
    return {"workload": WORKLOAD, "atmospheres": natm, "depths": 71, "lambda_per_atm": 224,
            "lines": 2, "zeeman_components": [13, 3], "mu": 1, "solver": "DELO-Bezier3",
            "magneto_optical": False, "l2": "inputs 2.1 GB > L2, no flush"}


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.proc = None
        self.gpu = gpu_index
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={gpu_index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline_port(batch, nthreads, seconds):
    """Times the CPU oracle (FP64 C port of the reference path, OpenMP over
    atmospheres) on a bounded sample of the same workload."""
    from oracle import oracle as O
    natm = batch["T"].shape[0]

    def sub(n):
        d = {k: batch[k][:n] for k in ("height", "T", "ne", "nHtot", "np", "vturb", "vel",
                                        "B", "gamma_B", "chi_B")}
        d["line_pops"] = batch["line_pops"][:n]
        d["chi_c"] = np.ascontiguousarray(batch["chi_c"][:n].transpose(0, 2, 1), np.float64)
        d["eta_c"] = np.ascontiguousarray(batch["eta_c"][:n].transpose(0, 2, 1), np.float64)
        for k in ("lam", "line_const", "zeeman", "zeeman_n", "vmicro_char", "mu"):
            d[k] = batch[k]
        d["magneto_optical"] = 0
        d["moving"] = 1
        return d

    n = min(natm, max(nthreads, 8))
    t0 = time.perf_counter()
    O.lte_synth_batch(sub(n), nthreads)
    t = time.perf_counter() - t0
    n2 = int(min(natm, max(n, n * seconds / max(t, 1e-3))))
    d = sub(n2)
    t0 = time.perf_counter()
    O.lte_synth_batch(d, nthreads)
    t = time.perf_counter() - t0
    units = n2 * len(batch["lam"])
    return {"value": units / t, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": f"{n2} of the {natm} atmospheres x {len(batch['lam'])} lambda, "
                      f"FP64 oracle (oracle/rt_oracle.c), {t:.1f} s", "seconds": t}


def _ncu_record(kernel: str):
    from pyrh_gb300 import build as B
    if not os.path.exists(NCU_TRAFFIC):
        return None, "no ncu capture recorded"
    with open(NCU_TRAFFIC) as f:
        rec = json.load(f).get(kernel)
    if not rec:
        return None, "no ncu capture recorded for this kernel"
    if rec["sources_digest"] != B.sources_digest(rec["sources"]):
        return None, "kernel sources changed since the recorded ncu capture"
    return rec, None


def measured_traffic(kernel: str, natm: int):
    """DRAM bytes of one launch over natm atmospheres from the recorded ncu
    capture of `kernel` (scaled by atmospheres), or None when the kernel's
    sources changed since that capture."""
    rec, why = _ncu_record(kernel)
    if rec is None:
        return None, why
    per_atm = (rec["dram_bytes_read"] + rec["dram_bytes_write"]) / rec["atmospheres"]
    return per_atm * natm, (f"ncu dram__bytes_read+write of one launch at {rec['atmospheres']} "
                            f"atmospheres, scaled by atmospheres ({rec['command']})")


def fp32_flops_per_unit(kernel: str):
    """FP32 flops per (pixel, wavelength) of `kernel` (FADD + FMUL + 2 FFMA
    thread instructions of the recorded ncu capture), or None."""
    rec, _ = _ncu_record(kernel)
    if rec is None:
        return None
    return rec["fp32_flops"] / (rec["atmospheres"] * rec["lambda_per_atm"])


def lte_accuracy(batch, db, pk, lines, nline, local, sp, nsample=16):
    """Error of the timed FP32 batch: the FP64 kernel on the same inputs, and
    the FP64 kernel against the FP64 oracle on a sample of atmospheres."""
    import torch
    from oracle import oracle as O
    from pyrh_gb300 import _lib as L
    from pyrh_gb300 import lte
    natm, nl = batch["T"].shape[0], pk.max_nlam
    pk64 = lte.pack_uniform(batch, nline, L.PYRH_FP64)
    d64 = lte.DeviceBatch(pk64, lines, nline, device=f"cuda:{local}")
    cfg64 = lte.make_config(precision=L.PYRH_FP64, mu=1.0, vmicro_char=batch["vmicro_char"])
    d64.run(cfg64, sp)
    torch.cuda.synchronize()
    s64 = d64.out.view(natm, 4, nl)
    s32 = db.out.view(natm, 4, nl).double()
    ic = s64[:, 0].amax(dim=1)[:, None, None]
    err_ic = ((s32 - s64).abs() / ic).amax(dim=(0, 2)).cpu().numpy()
    rel_I = float(((s32[:, 0] - s64[:, 0]).abs() / s64[:, 0].abs()).max())
    sub = {k: (v[:nsample] if isinstance(v, np.ndarray) and v.ndim and v.shape[0] == natm
               else v) for k, v in batch.items()}
    sub["chi_c"] = np.ascontiguousarray(batch["chi_c"][:nsample].transpose(0, 2, 1), np.float64)
    sub["eta_c"] = np.ascontiguousarray(batch["eta_c"][:nsample].transpose(0, 2, 1), np.float64)
    sub["magneto_optical"] = 0
    sub["moving"] = 1
    ref = O.lte_synth_batch(sub, os.cpu_count() or 1, md_float=False)
    g = s64[:nsample].cpu().numpy()
    err_or = float((np.abs(g - ref) / ref[:, 0].max(axis=1)[:, None, None]).max())
    del d64
    return {"fp32_vs_fp64_max_abs_over_Ic": {s: float(e) for s, e in zip("IQUV", err_ic)},
            "fp32_vs_fp64_max_rel_I": rel_I,
            "fp64_vs_oracle_max_abs_over_Ic": err_or,
            "oracle_sample_atmospheres": nsample,
            "metric": f"|S_fp32 - S_fp64| / I_c per atmosphere (I_c = max I of the atmosphere), "
                      f"over all {natm} atmospheres and wavelengths; rel_I = |dI| / I per point"}


def _events_ms(fn, stream, n):
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(n):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / n


def rf_measure(natm, local, stream, steps, warmup):
    """Adjoint of the batched synthesis: chi^2 against noisy targets
    synthesised from perturbed copies (sigma = 1e-3 I_c), its gradient with
    respect to T, v_los, v_mic, B, gamma, chi at every depth, and the full
    depth-resolved response functions, for natm atmospheres (FP32)."""
    import torch
    from pyrh_gb300 import _lib as L
    from pyrh_gb300 import lte, rf as RF, workload
    batch = workload.synthetic_batch(natm, seed=3000 + local, dtype=np.float32, setup_dT=True)
    pert = workload.synthetic_batch(natm, seed=4000 + local, dtype=np.float32)
    lines, nline = lte.make_lines(batch["line_const"], batch["zeeman"], batch["zeeman_n"])
    dev = lte.DeviceBatch(lte.pack_uniform(batch, nline, L.PYRH_FP32), lines, nline,
                          device=f"cuda:{local}")
    tgt = lte.DeviceBatch(lte.pack_uniform(pert, nline, L.PYRH_FP32), lines, nline,
                          device=f"cuda:{local}")
    cfg = lte.make_config(precision=L.PYRH_FP32, mu=1.0, vmicro_char=batch["vmicro_char"])
    sp = stream.cuda_stream
    tgt.run(cfg, sp)
    torch.cuda.synchronize()
    nl = dev.pk.max_nlam
    S = tgt.out.view(natm, 4, nl)
    ic = S[:, 0].max(dim=1).values[:, None, None]
    gen = torch.Generator(device=S.device).manual_seed(5)
    sigma = 1e-3 * ic
    obs = (S + sigma * torch.randn(S.shape, device=S.device, generator=gen)).reshape(-1)
    w = (1.0 / sigma ** 2).expand(natm, 4, nl).reshape(-1).contiguous()
    with torch.cuda.stream(stream):
        for _ in range(max(warmup, 3)):
            dev.run(cfg, sp)
            RF.chi2_grad(dev, cfg, obs, w, sp)
        fwd_ms = _events_ms(lambda: dev.run(cfg, sp), stream, steps)
        grad_ms = _events_ms(lambda: RF.chi2_grad(dev, cfg, obs, w, sp), stream, steps)
        RF.response_functions(dev, cfg, sp)
        rf_ms = _events_ms(lambda: RF.response_functions(dev, cfg, sp), stream, 2)
        # the same gradient with the set-up held fixed (partial T derivative)
        held = dev.struct.setup_dT
        dev.struct.setup_dT = None
        RF.chi2_grad(dev, cfg, obs, w, sp)
        fixed_ms = _events_ms(lambda: RF.chi2_grad(dev, cfg, obs, w, sp), stream, steps)
        dev.struct.setup_dT = held
    # FP32 gradient against the FP64 gradient of the same atmospheres
    nchk = min(natm, 256)
    nd = dev.pk.total_depth // natm
    with torch.cuda.stream(stream):
        g32 = RF.chi2_grad(dev, cfg, obs, w, sp)[1].view(6, natm, nd)[:, :nchk].double()
        sub = {k: (v[:nchk] if isinstance(v, np.ndarray) and v.ndim and v.shape[0] == natm
                   else v) for k, v in batch.items()}
        d64 = lte.DeviceBatch(lte.pack_uniform(sub, nline, L.PYRH_FP64), lines, nline,
                              device=f"cuda:{local}")
        cfg64 = lte.make_config(precision=L.PYRH_FP64, mu=1.0, vmicro_char=batch["vmicro_char"])
        g64 = RF.chi2_grad(d64, cfg64, obs.view(natm, -1)[:nchk].reshape(-1).double(),
                           w.view(natm, -1)[:nchk].reshape(-1).double(), sp)[1]
        g64 = g64.view(6, nchk, nd)
    torch.cuda.synchronize()
    diff = (g32 - g64).abs().amax(dim=2)
    per_atm = (diff / g64.abs().amax(dim=2)).amax(dim=1).cpu().numpy()
    batch_scale = (diff.amax(dim=1) / g64.abs().amax(dim=(1, 2))).cpu().numpy()
    del d64
    units = natm * nl
    return {"workload": f"chi^2 gradient and response functions: {natm} atm x 71 depths x "
                        f"{nl} lambda, FP32, targets from perturbed copies + noise 1e-3 I_c; "
                        "the temperature derivative follows T through the set-up (continuum "
                        "and stage densities) as the reference's finite differences do",
            "gradients_per_s": {"value": units / (grad_ms / 1e3), "unit": UNIT},
            "ms_forward": fwd_ms, "ms_chi2_gradient": grad_ms,
            "gradient_cost_vs_forward": grad_ms / fwd_ms,
            "ms_chi2_gradient_setup_fixed": fixed_ms,
            "ms_response_functions": rf_ms,
            "gradient_fp32_vs_fp64_rel_err": {p: float(e) for p, e in zip(RF.PARAMS, per_atm)},
            "gradient_fp32_vs_fp64_rel_err_batch_scale": {p: float(e) for p, e in
                                                          zip(RF.PARAMS, batch_scale)},
            "gradient_error_metric": f"{nchk} atmospheres, per parameter: max over atmospheres "
                                     "of max_depth |g32 - g64| / max_depth |g64| (the weakest "
                                     "fields dominate: their Q, U, V are small differences of "
                                     "Zeeman components), and max |g32 - g64| / max |g64| over "
                                     "the whole sample",
            "rf_bytes_written": int(4 * 6 * 71 * units * 4)}


def nlte_oracle_solve(atms, nthreads):
    """Converged populations and iteration counts of the FP64 NLTE oracle
    (oracle/nlte_oracle.c, one atmosphere per thread), and its wall time."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle import oracle as O
    t0 = time.perf_counter()
    with ThreadPoolExecutor(nthreads) as ex:
        res = list(ex.map(O.nlte_solve, atms))
    return [r[0] for r in res], [int(r[2]) for r in res], time.perf_counter() - t0


def background_measure(natm, local, stream, steps, warmup):
    """GPU background continuum (Background(), rh/background.c:329-460) at
    the batched synthesis' shape: natm atmospheres x 224 wavelengths x 71
    depths (the C0 atmosphere of the background fixture, whose densities and
    atomic data the reference's set-up produced), FP32 and FP64, CUDA
    events; the FP64 result against the reference's own Background() on the
    fixture's two atmospheres (120-20000 nm) and FP32 against FP64."""
    import torch
    from pyrh_gb300 import _lib as L
    from pyrh_gb300 import background as BGR
    fx = dict(np.load(os.path.join(HERE, "tests", "golden", "background.npz")))
    dev = BGR.DeviceBackground(BGR.model_from_setup(fx), device=f"cuda:{local}")
    lam = np.linspace(630.0, 630.35, 224)
    atm = BGR.setup_atmosphere(fx, 0)
    out = {"workload": f"{natm} atmospheres x 224 wavelengths (630.0-630.35 nm) x 71 depths; "
                       "11 passive atoms (157 continua), H2, OH, CH"}
    units = natm * 224 * 71
    for prec, tag in ((L.PYRH_FP32, "fp32"), (L.PYRH_FP64, "fp64")):
        b, keep = dev.replicated_batch(atm, lam, natm, prec)
        for _ in range(warmup):
            dev.run(b, stream.cuda_stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            dev.run(b, stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        out[tag] = {"ms": ms, "value": units / (ms / 1e3), "unit": "lambda*depth points/s",
                    "bytes_written": 3 * units * (4 if prec == L.PYRH_FP32 else 8)}
        del keep
        torch.cuda.empty_cache()
    atms = [BGR.setup_atmosphere(fx, a) for a in range(2)]
    r64 = dev.compute(atms)
    r32 = dev.compute(atms, precision=L.PYRH_FP32)
    err_ref, err_32 = 0.0, 0.0
    for q in range(3):
        for a in range(2):
            err_ref = max(err_ref, float(np.abs(r64[q][a] / fx["cont"][a][q] - 1).max()))
            m = np.abs(r64[q][a]) > 1e-30
            err_32 = max(err_32, float(np.abs(r32[q][a][m] / r64[q][a][m] - 1).max()))
    out["fp64_vs_reference_max_rel_err"] = err_ref
    out["fp32_vs_fp64_max_rel_err"] = err_32
    out["error_metric"] = ("chi_c, eta_c, sca_c element-wise relative, 2 atmospheres x 241 "
                           "wavelengths x 71 depths (FP32: where |FP64| > 1e-30)")
    return out


def setup_measure(natm, local, stream, steps, warmup):
    """The per-depth set-up on the GPU at the batched synthesis' shape (natm
    atmospheres x 71 depths, the three atmospheres of the chemistry fixture
    repeated): the two lines' stage densities and ln U (pyrh_line_pops), the
    electron density from scratch (pyrh_solve_ne) and the chemical
    equilibrium of the twelve molecules (pyrh_chem_equil), CUDA events; each
    against the reference's own LTEpops_elem / Solve_ne / ChemicalEquilibrium
    output on the fixtures' atmospheres."""
    import torch
    from pyrh_gb300 import chem as CH
    from pyrh_gb300 import ltepops as LP
    g = lambda n: dict(np.load(os.path.join(HERE, "tests", "golden", n + ".npz")))
    lp, ch, c0 = g("ltepops"), g("chem"), g("lte_c0")
    meta = lp["el_meta"][0]
    ns = meta[:, 0].astype(np.int32)
    tab = LP.ElementTables(lp["Tpf"], meta[:, 2].copy(), meta[:, 1].astype(np.int32), ns,
                           np.concatenate([[0], np.cumsum(ns)[:-1]]).astype(np.int32),
                           lp["el_pf"], lp["el_ionpot"])
    dev = LP.DeviceTables(tab, device=f"cuda:{local}")
    mols = [CH.read_molecule(str(t), tab.abundance_set) for t in ch["molecule_text"]]
    npt = natm * 71
    rep = -(-npt // ch["T"].size)
    T, ne, nH = (torch.from_numpy(np.tile(ch[k].ravel(), rep)[:npt]).to(f"cuda:{local}")
                 for k in ("T", "ne", "nHtot"))
    elem = c0["line_const"][:, 1].astype(np.int32) - 1
    stage = c0["line_const"][:, 2].astype(np.int32)
    legs = {"line_pops": lambda: LP.line_pops(dev, T, ne, nH, elem, stage),
            "solve_ne": lambda: LP.solve_ne(dev, T, nH),
            "chem_equil": lambda: CH.chem_equil(dev, mols, T, ne, nH)}
    out = {"workload": f"{natm} atmospheres x 71 depths ({npt} points); 2 Fe I lines; "
                       "99 elements; 12 molecules (H, C, N, O nuclei, partition-function "
                       "neutral fractions)"}
    with torch.cuda.stream(stream):
        for name, fn in legs.items():
            for _ in range(warmup):
                fn()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(steps):
                fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / steps
            out[name] = {"ms": ms, "value": npt / (ms / 1e3), "unit": "depth points/s"}
    # errors against the reference on the fixtures
    err = {}
    r = LP.line_pops(dev, c0["T"], c0["ne"], c0["nHtot"], elem, stage).cpu().numpy()
    err["line_pops_vs_reference"] = float(np.abs(r / c0["line_pops"] - 1).max())
    e_ne, e_ch = 0.0, 0.0
    for c in range(2):     # the ltepops fixture's atmospheres with the file's own abundances
        v = LP.solve_ne(dev, lp["T"][c], lp["nHtot"][c]).cpu().numpy()
        e_ne = max(e_ne, float(np.abs(v / lp["ne_solved"][c] - 1).max()))
    for c in range(3):
        fn0 = {int(e): ch["fn0"][c][i] for i, e in enumerate(ch["nuclei"]) if ch["nuc_model"][i]}
        nm, nh, nn, _ = CH.chem_equil(dev, mols, ch["T"][c], ch["ne"][c], ch["nHtot"][c], fn0)
        ref = ch["nmol"][c]
        m = ref != 0
        e_ch = max(e_ch, float(np.abs(nm.cpu().numpy()[m] / ref[m] - 1).max()),
                   float(np.abs(nh.cpu().numpy() / ch["nHmin"][c] - 1).max()))
    err["solve_ne_vs_reference"] = e_ne
    err["chem_equil_vs_reference"] = e_ch
    out["hse"], err["hse_vs_reference"] = hse_measure(natm, local, tab, lp, ch)
    out["accuracy"] = err
    out["error_metric"] = ("max relative error against the reference's LTEpops_elem / "
                           "Solve_ne / ChemicalEquilibrium / hse output (fixtures lte_c0, "
                           "ltepops, chem, hse)")
    return out


def hse_measure(natm, local, tab, lp, ch):
    """Hydrostatic equilibrium (pyrh_hse) of natm atmospheres x 71 layers on
    log tau500 (the hse fixture's first two atmospheres alternating), one
    timed call after one untimed, CUDA events; the oracle's time for one
    atmosphere on one host core beside it; the largest relative error of ne,
    nHtot, rho and pg against the reference's hse() on the fixture's five
    atmospheres."""
    import torch
    from pyrh_gb300 import chem as CH
    from pyrh_gb300 import grid as G
    from pyrh_gb300 import equilibria as EQ
    from pyrh_gb300 import hse as H
    from pyrh_gb300 import ltepops as LP
    g = lambda n: dict(np.load(os.path.join(HERE, "tests", "golden", n + ".npz")))
    h, bg = g("hse"), g("background")
    atoms = [G.read_atom(str(t)) for t in h["atom_text"]]
    dev = f"cuda:{local}"

    def model(case):
        ti = 2 if case == int(h["ab_case"]) else 0
        meta = lp["el_meta"][ti]
        ns = meta[:, 0].astype(np.int32)
        t = LP.ElementTables(lp["Tpf"], meta[:, 2].copy(), meta[:, 1].astype(np.int32), ns,
                             np.concatenate([[0], np.cumsum(ns)[:-1]]).astype(np.int32),
                             lp["el_pf"], lp["el_ionpot"])
        mols = [CH.read_molecule(str(x), t.abundance_set) for x in ch["molecule_text"]]
        return EQ.AtomsModel.build(t, atoms, mols, float(bg["misc"][0]), device=dev)

    m0 = model(0)
    from pyrh_gb300 import _lib as L

    def timed(n):
        sel = np.arange(n) % 2
        scale, T, pg_top = h["scale"][sel], h["T"][sel], h["pg_top"][sel]
        H.hse_batch(m0, 0, scale, T, pg_top)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s = torch.cuda.current_stream()
        e0.record(s)
        H.hse_batch(m0, 0, scale, T, pg_top)
        e1.record(s)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), int(L.lib().pyrh_last_launch_count())

    ms, launches = timed(natm)
    ms_small, _ = timed(1024)
    err = 0.0
    for c in range(len(h["T"])):
        m = model(c) if c == int(h["ab_case"]) else m0
        fudge = (h["fudge_wave"], h["fudge_value"]) if c == int(h["fudge_case"]) else None
        got = H.hse_batch(m, int(h["atm_scale"][c]), h["scale"][c][None], h["T"][c][None],
                          float(h["pg_top"][c]), fudge)
        for x, k in zip(got, ("ne", "nHtot", "rho", "pg")):
            err = max(err, float(np.abs(x[0] / h[k][c] - 1).max()))
    # the oracle (numpy restatement, one core) on the first atmosphere
    from oracle import chem as OC
    from oracle import hse as OH
    otab = {"Tpf": lp["Tpf"], "el_meta": lp["el_meta"][0], "el_pf": lp["el_pf"],
            "el_ionpot": lp["el_ionpot"]}
    elems = [EQ.element_index(a) for a in atoms]
    meta = bg["atoms_meta"]
    lo = np.concatenate([[0], np.cumsum(meta[:, 0])])
    co = np.concatenate([[0], np.cumsum(meta[:, 1])])
    li = np.concatenate([[0], np.cumsum(meta[:, 2])])
    oatoms = [dict(elem=elems[m], E=bg["atoms_lev"][lo[m]:lo[m + 1], 0],
                   g=bg["atoms_lev"][lo[m]:lo[m + 1], 1],
                   stage=bg["atoms_lev"][lo[m]:lo[m + 1], 2].astype(int),
                   cont=bg["atoms_cont"][co[m]:co[m + 1]], lines=bg["atoms_line"][li[m]:li[m + 1]],
                   tab=bg["atoms_tab"]) for m in range(len(meta))]
    omols = [OC.read_molecule(str(x), lp["el_meta"][0][:, 1].astype(np.int32))
             for x in ch["molecule_text"]]
    t0 = time.perf_counter()
    OH.hse(otab, oatoms, omols, [x["id"] for x in omols], 0, h["scale"][0][None],
           h["T"][0][None], float(h["pg_top"][0]))
    cpu_s = time.perf_counter() - t0
    return {"workload": f"{natm} atmospheres x 71 layers, log tau500, 11 passive atoms, "
                        "12 molecules, 500 nm background", "ms": ms,
            "value": natm / (ms / 1e3), "unit": "atmospheres/s",
            "launches": launches, "ms_1024_atmospheres": ms_small,
            "cpu_baseline": {"value": 1.0 / cpu_s, "unit": "atmospheres/s", "cores": 1,
                             "kind": "port", "sample": "one atmosphere of 71 layers"}}, err



def nlte_measure(natm, local, nsample=32):
    """Batched uneven NLTE (the six-level atom, five rays, Ng order 2 every 5
    iterations after 5): natm atmospheres with 50..150 depths and 700..1100
    wavelengths, generated from the reference's NLTE set-ups with the
    batched workload's T and v_los perturbations, solved in one batch.
    Converged atmospheres per second, FP32 against FP64 on the whole batch,
    both against the FP64 oracle on a sample, and the oracle's own rate on
    the host cores (the CPU baseline of this leg)."""
    import torch
    from pyrh_gb300 import _lib as L
    from pyrh_gb300 import nlte, workload
    names = ["nlte_c1", "nlte_c4_50", "nlte_c4_120"]
    bases = [dict(np.load(os.path.join(HERE, "tests", "golden", n + ".npz"))) for n in names]
    atms = workload.nlte_batch(bases, natm, seed=4096)
    nd = [len(a["T"]) for a in atms]
    ns = [len(a["lambda"]) for a in atms]
    out = {"workload": f"batched uneven NLTE: {natm} atmospheres, {min(nd)}-{max(nd)} depths, "
                       f"{min(ns)}-{max(ns)} wavelengths, 5 rays, 6-level atom (5 lines, 5 "
                       "continua); T nodes +-300 K and v_los +-3 km/s on the reference's NLTE "
                       "set-ups re-gridded per atmosphere"}
    pops, its = {}, {}
    for prec, tag in ((L.PYRH_FP32, "fp32"), (L.PYRH_FP64, "fp64")):
        cfg = nlte.make_config(atms[0], prec)
        pk = nlte.pack(atms, cfg.nrays)
        dev = nlte.DeviceNlte(pk, cfg, device=f"cuda:{local}")
        st = dev.solve(cfg)                      # warm-up (first-touch of the workspace)
        runs, raw = [], []
        for _ in range(2 if prec == L.PYRH_FP32 else 1):
            dev.reset()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            st = dev.solve(cfg)
            torch.cuda.synchronize()
            runs.append(time.perf_counter() - t0)
            raw.append(dev.t["n"].cpu().numpy().copy())
        t = min(runs)
        it = dev.iterations.cpu().numpy()
        out[tag] = {"status": int(st), "seconds": t, "converged_atm_per_s": natm / t,
                    "iterations_min_max": [int(it.min()), int(it.max())],
                    "launches": int(L.lib().pyrh_last_launch_count())}
        if prec == L.PYRH_FP32:
            out[tag]["bit_identical_rerun"] = bool(np.array_equal(raw[0], raw[1]))
        pops[tag], its[tag] = dev.populations(), it
        del dev
        torch.cuda.empty_cache()
    p32, p64 = pops["fp32"], pops["fp64"]
    errs = np.array([float(np.abs(a / b - 1).max()) for a, b in zip(p32, p64)])
    same = np.asarray(its["fp32"]) == np.asarray(its["fp64"])
    out["fp32_vs_fp64_max_population_rel_err"] = float(errs.max())
    # an FP32 run that meets the convergence limit one iteration earlier or
    # later than the FP64 run stops at another point of the same path
    out["fp32_vs_fp64_by_iteration_count"] = {
        "same_count_atmospheres": int(same.sum()),
        "same_count_max_rel_err": float(errs[same].max()) if same.any() else None,
        "different_count_atmospheres": int((~same).sum()),
        "different_count_max_rel_err": float(errs[~same].max()) if (~same).any() else None}
    # Both runs stop once no population changes by more than the limit in an
    # iteration, so each lies within about that change (times the Ng
    # amplification of a slowly converging atmosphere) of the fixed point.
    # Where FP32 and FP64 differ most, measure how far each is from the
    # fixed point itself: an FP64 solve run to a 1e-9 limit.
    worst = np.argsort(-errs)[:min(64, natm)]
    cfg = nlte.make_config(atms[0], L.PYRH_FP64, nmax_iter=400)
    cfg.iter_limit = 1e-9
    dev = nlte.DeviceNlte(nlte.pack([atms[i] for i in worst], cfg.nrays), cfg,
                          device=f"cuda:{local}")
    st = dev.solve(cfg)
    pfix = dev.populations()
    del dev
    torch.cuda.empty_cache()
    out["fixed_point_sample"] = {
        "atmospheres": len(worst), "selection": "largest FP32-vs-FP64 difference",
        "status": int(st),
        "fp32_max_rel_err": max(float(np.abs(p32[i] / f - 1).max()) for i, f in zip(worst, pfix)),
        "fp64_max_rel_err": max(float(np.abs(p64[i] / f - 1).max()) for i, f in zip(worst, pfix))}
    nthreads = os.cpu_count() or 1
    n_or, it_or, t_or = nlte_oracle_solve(atms[:nsample], nthreads)
    out["oracle_sample"] = {
        "atmospheres": nsample,
        "fp64_max_population_rel_err": max(float(np.abs(p64[i] / n_or[i] - 1).max())
                                           for i in range(nsample)),
        "fp32_max_population_rel_err": max(float(np.abs(p32[i] / n_or[i] - 1).max())
                                           for i in range(nsample)),
        "fp64_same_iteration_count": bool(all(int(its["fp64"][i]) == it_or[i]
                                              for i in range(nsample))),
        "fp32_iteration_count_diff_max": int(max(abs(int(its["fp32"][i]) - it_or[i])
                                                 for i in range(nsample)))}
    out["cpu_baseline"] = {"value": nsample / t_or, "unit": "converged atmospheres/s",
                           "cores": nthreads, "kind": "port",
                           "sample": f"{nsample} of the {natm} atmospheres, FP64 NLTE oracle "
                                     f"(oracle/nlte_oracle.c), one per thread, {t_or:.1f} s"}
    return out


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from pyrh_gb300 import workload
    nthreads = os.cpu_count() or 1
    batch = workload.synthetic_batch(min(args.natm, 4096), seed=1000, dtype=np.float64)
    vals, secs = [], []
    info = None
    for _ in range(args.warmup):
        cpu_baseline_port(batch, nthreads, min(args.cpu_seconds, 3.0))
    for _ in range(args.steps):
        info = cpu_baseline_port(batch, nthreads, args.cpu_seconds / max(args.steps, 1))
        vals.append(info["value"])
        secs.append(info.pop("seconds"))
    v = statistics.median(vals)
    info["value"] = v
    line = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * statistics.mean(secs), "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_dict(args.natm),
            "cpu_baseline": info,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "reference C sources are not available on this machine; the CPU arm runs "
                    "the oracle port of the same path with all host threads"}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
        return
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    from pyrh_gb300 import _lib as L
    from pyrh_gb300 import lte, workload

    natm = args.natm
    from pyrh_gb300.shard import max_over_ranks, rank_seed
    # weak scaling: every rank synthesises its own natm atmospheres
    batch = workload.synthetic_batch(natm, seed=rank_seed(1000, rank), dtype=np.float32)
    lines, nline = lte.make_lines(batch["line_const"], batch["zeeman"], batch["zeeman_n"])
    pk = lte.pack_uniform(batch, nline, L.PYRH_FP32)
    db = lte.DeviceBatch(pk, lines, nline, device=f"cuda:{local}")
    cfg = lte.make_config(precision=L.PYRH_FP32, mu=1.0, vmicro_char=batch["vmicro_char"])
    units = natm * pk.max_nlam
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream

    # autotuned wavelength tile, one launch recorded as a CUDA graph
    plan = lte.Plan(db, cfg, sp)
    for _ in range(max(args.warmup, 3)):
        plan.launch(sp)
    torch.cuda.synchronize()

    # ---- device-resident timing ----
    clocks = ClockSampler(local)
    time.sleep(0.3)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches = 0
    with torch.cuda.stream(stream):
        e0.record(stream)
        for _ in range(args.steps):
            plan.launch(sp)
            launches += L.lib().pyrh_last_launch_count()
        e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    clk = clocks.stop()
    ms = max_over_ranks(ms, dist)
    value = units * world / (ms / 1e3)

    # algorithmic bytes of one launch: every input array once + the output
    alg_bytes = sum(a.nbytes for a in pk.arrays.values()) + db.out.numel() * db.out.element_size()
    achieved = alg_bytes / (ms / 1e3) / 1e9
    traffic, traffic_src = measured_traffic("lte_stokes_kernel<float,false>", natm)
    # the FP32 roofline: SMs x 128 FP32 lanes x 2 flops (FMA) x the SM clock
    # sampled during the timed region
    fpu = fp32_flops_per_unit("lte_stokes_kernel<float,false>")
    props = torch.cuda.get_device_properties(local)
    clock_hz = (clk.get("sm_mhz") or 2070.0) * 1e6
    fp32_peak = props.multi_processor_count * 128 * 2 * clock_hz / 1e12
    fp32 = None
    if fpu is not None:
        fp32_ach = fpu * units / (ms / 1e3) / 1e12      # one GPU's launch
        fp32 = {"achieved": fp32_ach, "peak": fp32_peak, "unit": "TFLOP/s",
                "frac": fp32_ach / fp32_peak, "flops_per_unit": fpu,
                "peak_derivation": f"{props.multi_processor_count} SMs x 128 FP32 lanes x 2 "
                                   f"flops x {clock_hz / 1e6:.0f} MHz (sampled SM clock)",
                "flops_source": "ncu FADD + FMUL + 2 FFMA thread instructions of one launch "
                                "(pyrh_gb300/data/ncu_traffic.json)"}
    peaks_path = os.path.join(HERE, "MEASURED_PEAKS.json")
    peak, peak_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        with open(peaks_path) as f:
            peak = float(json.load(f)["hbm_gbs"])
        peak_src = "measured"

    accuracy = (lte_accuracy(batch, db, pk, lines, nline, local, sp)
                if rank == 0 and not args.skip_accuracy else None)

    # ---- end to end through the host-buffer C ABI (pinned host memory) ----
    pinned = {k: torch.from_numpy(np.ascontiguousarray(v)).pin_memory()
              for k, v in pk.arrays.items()}
    out_h = torch.empty(db.out.numel(), dtype=db.out.dtype).pin_memory()
    import ctypes as C
    hb = lte._batch_struct(pk, lambda k: pinned[k].data_ptr())
    h2d = sum(t.numel() * t.element_size() for t in pinned.values()) + C.sizeof(L.PyrhLine) * nline
    d2h = out_h.numel() * out_h.element_size()

    def host_call():
        L.check(L.lib().pyrh_lte_stokes_host(C.byref(hb), lines, nline, C.byref(cfg),
                                             out_h.data_ptr()))

    for _ in range(max(args.warmup, 3)):
        host_call()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        host_call()
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / args.steps
    e2e_s = max_over_ranks(e2e_s, dist)
    e2e = {"value": units * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_s * 1e3,
           "path": "pyrh_lte_stokes_host (host arrays in, Stokes out)"}

    extra = {}
    if rank == 0 and not args.skip_fp64:
        # plain FP64 one-pixel-per-call GPU form (the comparator of the target)
        b64 = workload.synthetic_batch(64, seed=77, dtype=np.float64)
        cfg64 = lte.make_config(precision=L.PYRH_FP64, mu=1.0, vmicro_char=b64["vmicro_char"])
        singles = []
        for i in range(64):
            one = {k: (v[i:i + 1] if isinstance(v, np.ndarray) and v.ndim and v.shape[0] == 64
                       else v) for k, v in b64.items()}
            p1 = lte.pack_uniform(one, nline, L.PYRH_FP64)
            singles.append(lte.DeviceBatch(p1, lines, nline, device=f"cuda:{local}"))
        for s in singles[:4]:
            s.run(cfg64, sp)
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for s in singles:
            s.run(cfg64, sp)
        f1.record(stream)
        torch.cuda.synchronize()
        per_call_ms = f0.elapsed_time(f1) / len(singles)
        fp64_single = pk.max_nlam / (per_call_ms / 1e3)
        # FP64 batched (same kernel, whole batch, one launch)
        pk64 = lte.pack_uniform(workload.synthetic_batch(2048, seed=78, dtype=np.float64),
                                nline, L.PYRH_FP64)
        db64 = lte.DeviceBatch(pk64, lines, nline, device=f"cuda:{local}")
        db64.run(cfg64, sp)
        torch.cuda.synchronize()
        g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        g0.record(stream)
        db64.run(cfg64, sp)
        g1.record(stream)
        torch.cuda.synchronize()
        fp64_batched = 2048 * pk64.max_nlam / (g0.elapsed_time(g1) / 1e3)
        extra = {"fp64_single_pixel_per_call": {"value": fp64_single, "unit": UNIT,
                                                "ms_per_call": per_call_ms, "sample": "64 calls"},
                 "fp64_batched": {"value": fp64_batched, "unit": UNIT, "atmospheres": 2048},
                 "speedup_vs_fp64_single_pixel": value / world / fp64_single}
        del singles, db64

    tile = {"block_lambda": plan.block, "tuned_ms": plan.tuned_ms, "cuda_graph": True}
    del plan, db
    torch.cuda.empty_cache()
    if rank == 0 and not args.skip_rf:
        extra["rf"] = rf_measure(args.rf_natm, local, stream, max(2, min(args.steps, 5)),
                                 args.warmup)
        torch.cuda.empty_cache()
    if rank == 0 and not args.skip_nlte:
        extra["nlte"] = nlte_measure(args.nlte_natm, local)
        torch.cuda.empty_cache()
    if rank == 0 and not args.skip_background:
        extra["background"] = background_measure(args.natm, local, stream,
                                                 max(2, min(args.steps, 5)), args.warmup)
        torch.cuda.empty_cache()
    if rank == 0 and not args.skip_background:
        extra["setup"] = setup_measure(args.natm, local, stream, max(2, min(args.steps, 5)),
                                       args.warmup)
        torch.cuda.empty_cache()

    cpu = None
    if rank == 0:
        batch64 = {k: v for k, v in batch.items()}
        cpu = cpu_baseline_port(batch64, os.cpu_count() or 1, args.cpu_seconds)
        cpu.pop("seconds")

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32", "data": "synthetic", "config": config_dict(natm),
                "clocks": clk, "e2e": e2e, "gpu_launches": launches, "plan": tile,
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak,
                             "traffic": traffic, "traffic_source": traffic_src,
                             "peak_source": peak_src, "alg_bytes_per_launch": alg_bytes,
                             "kernel": "lte_stokes_kernel<float,false>",
                             "fp32": fp32,
                             "note": "bound by FP32 issue, not HBM: the fp32 entry is the "
                                     "roofline that binds; the HBM fraction is small by "
                                     "construction"},
                "cpu_baseline": cpu, "accuracy": accuracy}
        line.update(extra)
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
