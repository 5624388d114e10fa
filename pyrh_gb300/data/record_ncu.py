"""Records the ncu figures of the synthesis kernel that bench.py reports
(DRAM traffic and FP32 / FP64 flops of one launch) in ncu_traffic.json,
with the digest of the kernel sources they were measured on.

    python -m pyrh_gb300.profile_case lte --natm 2048 --reps 1
    ncu --metrics gpu__time_duration.sum,dram__bytes_read.sum,dram__bytes_write.sum,\
smsp__sass_thread_inst_executed_op_fadd_pred_on.sum,\
smsp__sass_thread_inst_executed_op_fmul_pred_on.sum,\
smsp__sass_thread_inst_executed_op_ffma_pred_on.sum,\
smsp__sass_thread_inst_executed_op_dadd_pred_on.sum,\
smsp__sass_thread_inst_executed_op_dmul_pred_on.sum,\
smsp__sass_thread_inst_executed_op_dfma_pred_on.sum \
        --clock-control none -k regex:lte_stokes_kernel -c 1 --csv --log-file launch.csv \
        python -m pyrh_gb300.profile_case lte --natm 2048 --reps 1
    python -m pyrh_gb300.data.record_ncu launch.csv --natm 2048

The flop count is FADD + FMUL + 2 FFMA (FP32) and DADD + DMUL + 2 DFMA
(FP64) thread instructions.
"""
from __future__ import annotations

import argparse
import csv
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "ncu_traffic.json")
KERNEL = "lte_stokes_kernel<float,false>"
SOURCES = ["pyrh_gb300/csrc/lte_stokes.cu", "pyrh_gb300/csrc/lte_stokes.cuh",
           "pyrh_gb300/csrc/rt_device.cuh", "pyrh_gb300/csrc/voigt_armstrong.cuh"]
COMMAND = ("python -m pyrh_gb300.profile_case lte --natm {natm} --reps 1 under ncu --metrics "
           "gpu__time_duration.sum,dram__bytes_read.sum,dram__bytes_write.sum,"
           "smsp__sass_thread_inst_executed_op_{{fadd,fmul,ffma,dadd,dmul,dfma}}_pred_on.sum "
           "--clock-control none -k regex:lte_stokes_kernel -c 1")


def read_metrics(path: str) -> dict:
    """Metric name -> value (as float, in the unit ncu printed) of the one
    captured launch in an ncu --csv log."""
    with open(path, newline="") as f:
        lines = [ln for ln in f if ln.startswith('"')]     # skip ncu's own log lines
    rows = list(csv.DictReader(lines))
    if not rows:
        raise ValueError(f"{path}: no metric rows")
    ids = {r["ID"] for r in rows}
    if len(ids) != 1:
        raise ValueError(f"{path}: {len(ids)} launches captured, expected one")
    out = {}
    for r in rows:
        v = float(r["Metric Value"].replace(",", ""))
        unit = r.get("Metric Unit", "")
        scale = {"byte": 1, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9,
                 "nsecond": 1, "usecond": 1e3, "msecond": 1e6}.get(unit, 1)
        out[r["Metric Name"]] = v * scale
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("csv")
    ap.add_argument("--natm", type=int, required=True)
    ap.add_argument("--lambda-per-atm", type=int, default=224)
    ap.add_argument("--depths", type=int, default=71)
    a = ap.parse_args(argv)
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from pyrh_gb300 import build as B
    m = read_metrics(a.csv)
    op = "smsp__sass_thread_inst_executed_op_{}_pred_on.sum"
    rec = {
        "sources": SOURCES,
        "sources_digest": B.sources_digest(SOURCES),
        "atmospheres": a.natm,
        "lambda_per_atm": a.lambda_per_atm,
        "depths": a.depths,
        "dram_bytes_read": int(m["dram__bytes_read.sum"]),
        "dram_bytes_write": int(m["dram__bytes_write.sum"]),
        "fp32_flops": int(m[op.format("fadd")] + m[op.format("fmul")] + 2 * m[op.format("ffma")]),
        "fp64_flops": int(m[op.format("dadd")] + m[op.format("dmul")] + 2 * m[op.format("dfma")]),
        "ncu_duration_ns": int(m["gpu__time_duration.sum"]),
        "command": COMMAND.format(natm=a.natm),
    }
    data = {}
    if os.path.exists(OUT):
        with open(OUT) as f:
            data = json.load(f)
    data[KERNEL] = rec
    with open(OUT, "w") as f:
        json.dump(data, f, indent=1)
        f.write("\n")
    print(json.dumps(rec, indent=1))


if __name__ == "__main__":
    main()
