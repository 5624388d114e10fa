"""Builds libpyrh_gb300.so in-tree with nvcc for sm_103a (no torch extension
machinery: the library exposes a plain C ABI, include/pyrh_gb300.h)."""
from __future__ import annotations

import hashlib
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpyrh_gb300.so")
# the response-function kernels: one unit per precision and mode, so that
# the largest instantiations compile in parallel
UNITS = ["capi.cu", "lte_stokes.cu", "lte_rf.cu"] + \
    [f"lte_rf_fp{p}_{m}.cu" for p in ("32", "64") for m in ("rf", "chi2", "vjp")] + \
    ["nlte.cu", "nlte_capi.cu", "nlte_setup.cu", "setup_host.cpp", "background.cu",
     "ltepops.cu", "elements_host.cpp", "chem.cu", "hse.cu"]
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def sources_digest(files) -> str:
    """Digest of source files given relative to the repository root (ties a
    recorded measurement to the kernel sources it was taken on)."""
    repo = os.path.dirname(HERE)
    h = hashlib.sha256()
    for f in files:
        with open(os.path.join(repo, f), "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()[:16]


def _sources_mtime() -> float:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(os.path.dirname(HERE), "include", "pyrh_gb300.h"))
    return max(os.path.getmtime(f) for f in files)


def build(force: bool = False, verbose: bool = False, out: str | None = None,
          defines: tuple = ()) -> str:
    """Compile the library; `out` and `defines` (e.g. "PYRH_LTE_MIN_BLOCKS=3")
    build a variant next to the default one (used for tile/occupancy sweeps)."""
    target = out or LIB
    if not force and os.path.exists(target) and os.path.getmtime(target) >= _sources_mtime():
        return target
    bdir = BUILD if out is None else os.path.join(BUILD, os.path.basename(out) + ".d")
    os.makedirs(bdir, exist_ok=True)
    dflags = [f"-D{d}" for d in defines]

    def compile_unit(u):
        obj = os.path.join(bdir, os.path.splitext(u)[0] + ".o")
        cmd = [NVCC, *GENCODE, *FLAGS, *dflags, "-c", os.path.join(CSRC, u), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {u}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = target + ".tmp"
    subprocess.run([NVCC, *GENCODE, "-shared", "-o", tmp, *objs, "-lcudart"], check=True)
    os.replace(tmp, target)
    return target


if __name__ == "__main__":
    print(build(force=True, verbose=True))
