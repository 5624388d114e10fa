"""Runs one hot-path kernel on a synthetic case a few times, for profilers.

    python -m pyrh_gb300.profile_case lte  --natm 2048 --reps 2
    python -m pyrh_gb300.profile_case grad --natm 2048 --reps 2
    python -m pyrh_gb300.profile_case rf   --natm 512  --reps 2
    python -m pyrh_gb300.profile_case nlte --natm 64   --reps 1
    python -m pyrh_gb300.profile_case background --natm 1024 --reps 3
    python -m pyrh_gb300.profile_case hse  --natm 1024 --reps 2

lte:  pyrh_lte_stokes (FP32) over natm perturbed atmospheres, 71 depths,
      2 x 112 wavelengths (the batched synthesis workload at a smaller size).
grad: pyrh_lte_chi2_grad (FP32) on the same shape.
rf:   pyrh_lte_rf (FP32): full depth-resolved response functions.
nlte: pyrh_nlte_solve (FP32 formal solution) over natm atmospheres cycled
      from the three NLTE fixtures of tests/golden.
background: pyrh_background (FP32) for natm copies of the C0 atmosphere of
      the background fixture on 224 wavelengths at 630.0-630.35 nm.
hse:  pyrh_hse (FP64) for natm atmospheres of 71 layers on log tau500 (the
      hse fixture's first two atmospheres alternating), with the passive
      atoms, molecules and element tables of the fixtures' runs.
Prints one line per case with the time of the last repetition (CUDA events).
"""
from __future__ import annotations

import argparse
import os

import numpy as np


def _time(fn, reps):
    import torch
    t = 0.0
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1)
    return t


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["lte", "grad", "rf", "nlte", "background", "hse"])
    ap.add_argument("--natm", type=int, default=2048)
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--fp64", action="store_true")
    a = ap.parse_args(argv)
    import torch
    from . import _lib as L
    from . import lte, nlte, rf as RF, workload
    prec = L.PYRH_FP64 if a.fp64 else L.PYRH_FP32
    if a.case == "hse":
        from . import chem as CH
        from . import equilibria as EQ
        from . import grid as G
        from . import hse as H
        from . import ltepops as LP
        here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
        g = lambda n: dict(np.load(os.path.join(here, "tests", "golden", n + ".npz")))
        h, lp, ch, bg = g("hse"), g("ltepops"), g("chem"), g("background")
        meta = lp["el_meta"][0]
        ns = meta[:, 0].astype(np.int32)
        tab = LP.ElementTables(lp["Tpf"], meta[:, 2].copy(), meta[:, 1].astype(np.int32), ns,
                               np.concatenate([[0], np.cumsum(ns)[:-1]]).astype(np.int32),
                               lp["el_pf"], lp["el_ionpot"])
        model = EQ.AtomsModel.build(tab, [G.read_atom(str(t)) for t in h["atom_text"]],
                                    [CH.read_molecule(str(t), tab.abundance_set)
                                     for t in ch["molecule_text"]], float(bg["misc"][0]))
        sel = np.arange(a.natm) % 2

        def run():
            H.hse_batch(model, 0, h["scale"][sel], h["T"][sel], h["pg_top"][sel])
    elif a.case == "background":
        from . import background as BGR
        here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
        fx = dict(np.load(os.path.join(here, "tests", "golden", "background.npz")))
        dev = BGR.DeviceBackground(BGR.model_from_setup(fx))
        batch, keep = dev.replicated_batch(BGR.setup_atmosphere(fx, 0),
                                           np.linspace(630.0, 630.35, 224), a.natm, prec)

        def run():
            dev.run(batch)
    elif a.case == "nlte":
        here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
        names = ["nlte_c1", "nlte_c4_50", "nlte_c4_120"]
        gold = [dict(np.load(os.path.join(here, "tests", "golden", n + ".npz"))) for n in names]
        atms = [gold[i % 3] for i in range(a.natm)]
        cfg = nlte.make_config(gold[0], prec)
        dev = nlte.DeviceNlte(nlte.pack(atms, cfg.nrays), cfg)

        def run():
            dev.reset()
            L.check(dev.solve(cfg))
    else:
        dt = np.float64 if a.fp64 else np.float32
        batch = workload.synthetic_batch(a.natm, seed=5, dtype=dt)
        lines, nline = lte.make_lines(batch["line_const"], batch["zeeman"], batch["zeeman_n"])
        dev = lte.DeviceBatch(lte.pack_uniform(batch, nline, prec), lines, nline)
        cfg = lte.make_config(precision=prec, mu=1.0, vmicro_char=batch["vmicro_char"])
        obs = torch.zeros_like(dev.out)
        w = torch.ones_like(dev.out)
        run = {"lte": lambda: dev.run(cfg),
               "grad": lambda: RF.chi2_grad(dev, cfg, obs, w),
               "rf": lambda: RF.response_functions(dev, cfg)}[a.case]
    ms = _time(run, a.reps)
    print(f"{a.case} natm={a.natm} precision={'fp64' if a.fp64 else 'fp32'} ms={ms:.3f}",
          flush=True)


if __name__ == "__main__":
    main()
