"""Runs the compiled REFERENCE (oracle/_ref/librh_ref.so) -- test infrastructure.

Only the golden-vector generator (tests/golden/make_golden.py) and the
reference arm of the CPU baseline use this module, and only where the
reference sources were available to build oracle/_ref (never on a machine
without them).  Every reference call runs in a fresh spawned process because
the reference keeps process-global state and is not re-entrant
(rh/rhf1d/pyrh_compute1dray.c:86-92).

Reference entry points driven here:
  hse()    rh/rhf1d/pyrh_hse.c:67   (ne, nHtot in m^-3 for a T(log tau) model)
  rhf1d()  rh/rhf1d/pyrh_compute1dray.c:112 via harness_synth
  set-up of rhf1d() + Background() dump via harness_dump_lte
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_LIB = os.path.join(HERE, "_ref", "librh_ref.so")
# Same sources built without -DSIMDON: the scalar float 4x4 inverse of
# rh/bezier_aux.c:235-328 (what the reference compiles to on Arm) instead of
# the SSE reciprocal-estimate inverse of rh/bezier_aux.c:133-232.
REF_LIB_PORTABLE = os.path.join(HERE, "_ref", "portable", "librh_ref.so")


def reference_root() -> str:
    """The reference checkout: PYRH_REFERENCE_ROOT, else the default of the
    build recipe oracle/Makefile.ref; empty when neither holds the sources."""
    env = os.environ.get("PYRH_REFERENCE_ROOT")
    if env:
        return env if os.path.isdir(os.path.join(env, "rh")) else ""
    r = subprocess.run(["make", "-s", "-f", os.path.join(HERE, "Makefile.ref"), "print-ref"],
                       capture_output=True, text=True)
    return r.stdout.strip() if r.returncode == 0 else ""


REF_ROOT = reference_root()

_P = C.POINTER(C.c_double)


def build_ref(ref_root: str = REF_ROOT) -> str:
    """Compile the reference sources into oracle/_ref/librh_ref.so and the
    portable variant into oracle/_ref/portable/librh_ref.so."""
    repo = os.path.dirname(HERE)
    jobs = f"-j{os.cpu_count() or 4}"
    subprocess.run(["make", "-s", "-f", "oracle/Makefile.ref", f"REF={ref_root}", jobs],
                   cwd=repo, check=True)
    subprocess.run(["make", "-s", "-f", "oracle/Makefile.ref", f"REF={ref_root}",
                    "OUT=oracle/_ref/portable", "SIMD=", jobs], cwd=repo, check=True)
    return REF_LIB


def _p(a: np.ndarray):
    return a.ctypes.data_as(_P)


# ---------------------------------------------------------------- input set --

KEYWORD_TEMPLATE = """\
  NRAYS = {nrays}
  ATOMS_FILE = atoms.input
  MOLECULES_FILE = molecules.input
  N_MAX_SCATTER = {nmax_scatter}
  I_SUM = -1
  N_MAX_ITER = {nmax_iter}
  ITER_LIMIT = {iter_limit}
  NG_ORDER  = {ng_order}
  NG_DELAY  = {ng_delay}
  NG_PERIOD = {ng_period}
  PRD_N_MAX_ITER = 1
  PRD_ITER_LIMIT = 1.0E-2
  J_FILE          = J.dat
  STARTING_J      = NEW_J
  BACKGROUND_FILE = background.dat
  OLD_BACKGROUND  = FALSE
  KURUCZ_DATA = {kurucz}
  SOLVE_NE = NONE
  RLK_SCATTER = FALSE
  HYDROGEN_LTE = TRUE
  VMICRO_CHAR = {vmicro_char}
  VMACRO_TRESH = {vmacro_tresh}
  S_INTERPOLATION = S_BEZIER3
  S_INTERPOLATION_STOKES = DELO_BEZIER3
  VACUUM_TO_AIR = FALSE
  STOKES_MODE = {stokes_mode}
  MAGNETO_OPTICAL = {magneto_optical}
  LS_LANDE = FALSE
  LIMIT_MEMORY = FALSE
  ALLOW_PASSIVE_BB = FALSE
  PRINT_CPU = FALSE
{extra}"""

PASSIVE_ATOMS = ["H_6.atom", "He.atom", "C.atom", "N.atom", "O.atom", "S.atom",
                 "Fe.atom", "Si.atom", "Al.atom", "Na.atom", "Mg.atom"]


def write_inputs(workdir: str, kurucz_lines: str | None, atoms=None,
                 active: str | None = None, **kw) -> None:
    """Write keyword.input, atoms.input, molecules.input, kurucz.input."""
    opts = dict(nrays=1, nmax_scatter=0, nmax_iter=1, iter_limit="1.0E-2",
                ng_order=0, ng_delay=10, ng_period=3, vmicro_char=5.0,
                stokes_mode="FULL_STOKES", magneto_optical="FALSE",
                kurucz="kurucz.input" if kurucz_lines else "none", extra="",
                vmacro_tresh="0")
    opts.update(kw)
    with open(os.path.join(workdir, "keyword.input"), "w") as f:
        f.write(KEYWORD_TEMPLATE.format(**opts))
    atoms = list(atoms or PASSIVE_ATOMS)
    with open(os.path.join(workdir, "atoms.input"), "w") as f:
        f.write(f"{len(atoms)}\n")
        for a in atoms:
            mode = "ACTIVE" if a == active else "PASSIVE"
            f.write(f"  {a}  {mode}  LTE_POPULATIONS  pops.out\n")
    shutil.copy(os.path.join(REF_ROOT, "tests", "molecules.input"), workdir)
    if kurucz_lines:
        path = os.path.join(workdir, "lines.kurucz")
        with open(path, "w") as f:
            f.write(kurucz_lines)
        with open(os.path.join(workdir, "kurucz.input"), "w") as f:
            f.write(path + "\n")


# ------------------------------------------------------------ subprocesses --

def _lib(pyrh_path: str):
    os.environ["PYRH_PATH"] = pyrh_path
    return C.CDLL(os.environ.get("PYRH_REF_LIB", REF_LIB))


def _hse_job(args):
    workdir, pyrh_path, logtau, T = args
    lib = _lib(pyrh_path)
    n = len(logtau)
    logtau = np.ascontiguousarray(logtau, dtype=np.float64)
    T = np.ascontiguousarray(T, dtype=np.float64)
    ne, nH, rho, pg = (np.zeros(n) for _ in range(4))
    pg[0] = 0.1
    lib.hse.restype = None
    lib.hse(workdir.encode(), n, _p(logtau), _p(T), _p(ne), _p(nH), _p(rho),
            _p(pg), 0, 0, None, None, 0, None, None)
    return ne, nH


def _hse_full_job(args):
    """hse() with every argument of pyrh.hse (pyrh.pyx:427-487): the depth
    scale type, pg_top, fudge factors and abundance overrides; returns ne,
    nHtot, rho, pg (SI)."""
    workdir, pyrh_path, atm_scale, scale, T, pg_top, fudge_wave, fudge_value, ab_id, ab_val = args
    lib = _lib(pyrh_path)
    n = len(scale)
    scale = np.ascontiguousarray(scale, dtype=np.float64)
    T = np.ascontiguousarray(T, dtype=np.float64)
    ne, nH, rho, pg = (np.zeros(n) for _ in range(4))
    pg[0] = pg_top
    nf, fw, fv = 0, None, None
    if fudge_wave is not None:
        fudge_wave = np.ascontiguousarray(fudge_wave, dtype=np.float64)
        fudge_value = np.ascontiguousarray(fudge_value, dtype=np.float64)
        nf, fw, fv = len(fudge_wave), _p(fudge_wave), _p(fudge_value)
    na, ai, av = 0, None, None
    if ab_id is not None:
        ab_id = np.ascontiguousarray(ab_id, dtype=np.int32)
        ab_val = np.ascontiguousarray(ab_val, dtype=np.float64)
        na, ai, av = len(ab_id), ab_id.ctypes.data_as(C.POINTER(C.c_int)), _p(ab_val)
    lib.hse.restype = None
    lib.hse(workdir.encode(), n, _p(scale), _p(T), _p(ne), _p(nH), _p(rho), _p(pg),
            int(atm_scale), nf, fw, fv, na, ai, av)
    return ne, nH, rho, pg


def _scales_job(args):
    """get_scales() (pyrh.pyx:491-533): tau, height, cmass of an atmosphere
    [9, ndep] (compute1d's rows) on its scale."""
    workdir, pyrh_path, atm_scale, scale, atm, lam_ref, ab_id, ab_val = args
    lib = _lib(pyrh_path)
    atm = np.array(atm, dtype=np.float64, order="C")
    n = atm.shape[1]
    scale = np.ascontiguousarray(scale, dtype=np.float64)
    tau, height, cmass = (np.zeros(n) for _ in range(3))
    na, ai, av = 0, None, None
    if ab_id is not None:
        ab_id = np.ascontiguousarray(ab_id, dtype=np.int32)
        ab_val = np.ascontiguousarray(ab_val, dtype=np.float64)
        na, ai, av = len(ab_id), ab_id.ctypes.data_as(C.POINTER(C.c_int)), _p(ab_val)
    rows = [np.ascontiguousarray(atm[r]) for r in (1, 2, 3, 4, 8)]
    lib.get_scales.restype = None
    lib.get_scales(workdir.encode(), n, _p(scale), *[_p(r) for r in rows], int(atm_scale),
                   C.c_double(lam_ref), _p(tau), _p(height), _p(cmass), na, ai, av)
    return tau, height, cmass


def _synth_job(args):
    workdir, pyrh_path, mu, atm, wave = args[:5]
    atm_scale = args[5] if len(args) > 5 else 0
    lib = _lib(pyrh_path)
    atm = np.ascontiguousarray(atm, dtype=np.float64)
    wave = np.ascontiguousarray(wave, dtype=np.float64)
    cap = len(wave) + 4096
    out = [np.zeros(cap) for _ in range(5)]
    flag = C.c_int(0)
    lib.harness_synth.restype = C.c_int
    n = lib.harness_synth(workdir.encode(), C.c_double(mu), atm.shape[1],
                          _p(atm), int(atm_scale), len(wave), _p(wave), cap,
                          *[_p(o) for o in out], C.byref(flag))
    if n < 0:
        raise RuntimeError("reference output larger than capacity")
    lam, sI, sQ, sU, sV = (o[:n].copy() for o in out)
    return lam, np.stack([sI, sQ, sU, sV]), flag.value


def _loggf_job(args):
    workdir, pyrh_path, mu, atm, wave, ids, vals, get_rfs = args
    lib = _lib(pyrh_path)
    atm = np.ascontiguousarray(atm, dtype=np.float64)
    wave = np.ascontiguousarray(wave, dtype=np.float64)
    ids = np.ascontiguousarray(ids, dtype=np.int32)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    cap = len(wave) + 4096
    lam, sI = np.zeros(cap), np.zeros(cap)
    rfs = np.zeros((len(ids), cap))
    lib.harness_synth_loggf.restype = C.c_int
    n = lib.harness_synth_loggf(workdir.encode(), C.c_double(mu), atm.shape[1], _p(atm),
                                len(wave), _p(wave), len(ids),
                                ids.ctypes.data_as(C.POINTER(C.c_int)), _p(vals), int(get_rfs),
                                cap, _p(lam), _p(sI), _p(rfs))
    if n < 0:
        raise RuntimeError("reference output larger than capacity")
    return lam[:n].copy(), sI[:n].copy(), rfs[:, :n].copy()


def _dump_job(args):
    workdir, pyrh_path, mu, atm, wave, outdir = args
    lib = _lib(pyrh_path)
    atm = np.ascontiguousarray(atm, dtype=np.float64)
    wave = np.ascontiguousarray(wave, dtype=np.float64)
    os.makedirs(outdir, exist_ok=True)
    lib.harness_dump_lte.restype = C.c_int
    return lib.harness_dump_lte(workdir.encode(), C.c_double(mu), atm.shape[1],
                                _p(atm), len(wave), _p(wave), outdir.encode())


def _background_job(args):
    workdir, pyrh_path, mu, atm, wave, outdir = args
    lib = _lib(pyrh_path)
    atm = np.ascontiguousarray(atm, dtype=np.float64)
    wave = np.ascontiguousarray(wave, dtype=np.float64)
    os.makedirs(outdir, exist_ok=True)
    lib.harness_dump_background.restype = C.c_int
    return lib.harness_dump_background(workdir.encode(), C.c_double(mu), atm.shape[1],
                                       _p(atm), len(wave), _p(wave), outdir.encode())


def _ltepops_job(args):
    workdir, pyrh_path, atm, ab_id, ab_val, outdir = args
    lib = _lib(pyrh_path)
    atm = np.ascontiguousarray(atm, dtype=np.float64)
    ab_id = np.ascontiguousarray(ab_id, dtype=np.int32)
    ab_val = np.ascontiguousarray(ab_val, dtype=np.float64)
    os.makedirs(outdir, exist_ok=True)
    lib.harness_dump_ltepops.restype = C.c_int
    return lib.harness_dump_ltepops(workdir.encode(), atm.shape[1], _p(atm), len(ab_id),
                                    ab_id.ctypes.data_as(C.POINTER(C.c_int)), _p(ab_val),
                                    outdir.encode())


def read_ltepops_dump(outdir: str) -> dict:
    """The files of harness_dump_ltepops as arrays."""
    f64 = lambda n: np.fromfile(os.path.join(outdir, n + ".f64"))
    d = {k: f64(k) for k in ("Tpf", "el_ionpot", "T", "ne", "nHtot", "ne_solved", "ne_warm")}
    d["el_meta"] = f64("el_meta").reshape(-1, 4)
    d["el_pf"] = f64("el_pf").reshape(-1, len(d["Tpf"]))
    d["el_n"] = f64("el_n").reshape(-1, len(d["T"]))
    return d


def _chem_job(args):
    workdir, pyrh_path, atm, outdir = args
    lib = _lib(pyrh_path)
    atm = np.ascontiguousarray(atm, dtype=np.float64)
    os.makedirs(outdir, exist_ok=True)
    lib.harness_dump_chem.restype = C.c_int
    return lib.harness_dump_chem(workdir.encode(), atm.shape[1], _p(atm), outdir.encode())


def read_chem_dump(outdir: str) -> dict:
    """The files of harness_dump_chem as arrays."""
    f64 = lambda n: np.fromfile(os.path.join(outdir, n + ".f64"))
    i32 = lambda n: np.fromfile(os.path.join(outdir, n + ".i32"), dtype=np.int32)
    d = {k: f64(k) for k in ("T", "ne", "nHtot", "nHmin")}
    nd = len(d["T"])
    d["nuclei"], d["nuc_model"] = i32("nuclei"), i32("nuc_model")
    for k in ("fn0", "nmol", "ntot_model"):
        d[k] = f64(k).reshape(-1, nd)
    return d


def read_background_dump(outdir: str) -> dict:
    """The files of harness_dump_background as arrays."""
    f64 = lambda n: np.fromfile(os.path.join(outdir, n + ".f64"))
    i32 = lambda n: np.fromfile(os.path.join(outdir, n + ".i32"), dtype=np.int32)
    d = {"lambda": f64("lambda")}
    ns, nd = len(d["lambda"]), len(f64("T"))
    for k in ("T", "ne", "nHmin", "nH2", "nOH", "nCH", "misc"):
        d[k] = f64(k)
    d["mol_present"] = i32("mol_present")
    d["cont"] = f64("cont").reshape(3, ns, nd)
    d["comp"] = f64("comp").reshape(13, 2, ns, nd)
    d["atoms_meta"] = i32("atoms_meta").reshape(-1, 4)
    d["atoms_lev"] = f64("atoms_lev").reshape(-1, 3)
    d["atoms_n"] = f64("atoms_n").reshape(-1, nd)
    d["atoms_nstar"] = f64("atoms_nstar").reshape(-1, nd)
    d["atoms_cont"] = f64("atoms_cont").reshape(-1, 8)
    d["atoms_tab"] = f64("atoms_tab").reshape(-1, 2)
    d["atoms_line"] = f64("atoms_line").reshape(-1, 5)
    return d


def _vac2air_job(args):
    pyrh_path, lam_vac = args
    lib = _lib(pyrh_path)
    lam_vac = np.ascontiguousarray(lam_vac, dtype=np.float64)
    out = np.zeros_like(lam_vac)
    lib.vacuum_to_air.restype = None
    lib.vacuum_to_air(len(lam_vac), _p(lam_vac), _p(out))
    return out


class Reference:
    """Runs every reference call in a fresh interpreter (subprocess with a
    time limit), since the reference keeps global state, leaks memory and
    calls exit() on errors (rh/error.c:45-60)."""

    def __init__(self, pyrh_path: str = REF_ROOT, timeout: float = 600.0,
                 lib_path: str = REF_LIB):
        if not (os.path.exists(REF_LIB) and os.path.exists(REF_LIB_PORTABLE)):
            build_ref()
        self.pyrh_path = pyrh_path
        self.timeout = timeout
        self.lib_path = lib_path

    def _run(self, fn, args):
        import pickle
        import sys
        with tempfile.TemporaryDirectory(prefix="rhjob_") as td:
            src, dst = os.path.join(td, "in.pkl"), os.path.join(td, "out.pkl")
            with open(src, "wb") as f:
                pickle.dump((fn.__name__, args), f)
            repo = os.path.dirname(HERE)
            env = dict(os.environ, PYRH_REF_LIB=self.lib_path)
            r = subprocess.run([sys.executable, "-m", "oracle.ref_runner", src, dst],
                               cwd=repo, timeout=self.timeout, capture_output=True,
                               text=True, env=env)
            if r.returncode != 0 or not os.path.exists(dst):
                raise RuntimeError(f"reference call {fn.__name__} failed "
                                   f"(rc={r.returncode}): {r.stderr[-2000:]}"
                                   f"{r.stdout[-2000:]}")
            with open(dst, "rb") as f:
                return pickle.load(f)

    def map(self, fn, arglist, procs=None):
        from concurrent.futures import ThreadPoolExecutor
        procs = procs or min(len(arglist), os.cpu_count() or 4)
        with ThreadPoolExecutor(procs) as ex:
            return list(ex.map(lambda a: self._run(fn, a), arglist))

    def hse(self, workdir, logtau, T):
        return self._run(_hse_job, (workdir, self.pyrh_path, logtau, T))

    def hse_full(self, workdir, atm_scale, scale, T, pg_top=0.1, fudge_wave=None,
                 fudge_value=None, ab_id=None, ab_val=None):
        return self._run(_hse_full_job, (workdir, self.pyrh_path, atm_scale, scale, T, pg_top,
                                         fudge_wave, fudge_value, ab_id, ab_val))

    def get_scales(self, workdir, atm_scale, scale, atm, lam_ref, ab_id=None, ab_val=None):
        return self._run(_scales_job, (workdir, self.pyrh_path, atm_scale, scale, atm, lam_ref,
                                       ab_id, ab_val))

    def synth(self, workdir, mu, atm, wave, atm_scale=0):
        return self._run(_synth_job, (workdir, self.pyrh_path, mu, atm, wave, atm_scale))

    def synth_loggf(self, workdir, mu, atm, wave, ids, vals, get_rfs=True):
        return self._run(_loggf_job, (workdir, self.pyrh_path, mu, atm, wave, ids, vals, get_rfs))

    def dump_lte(self, workdir, mu, atm, wave, outdir):
        return self._run(_dump_job, (workdir, self.pyrh_path, mu, atm, wave, outdir))

    def dump_background(self, workdir, mu, atm, wave, outdir):
        return self._run(_background_job, (workdir, self.pyrh_path, mu, atm, wave, outdir))

    def dump_ltepops(self, workdir, atm, ab_id, ab_val, outdir):
        return self._run(_ltepops_job, (workdir, self.pyrh_path, atm, ab_id, ab_val, outdir))

    def dump_chem(self, workdir, atm, outdir):
        return self._run(_chem_job, (workdir, self.pyrh_path, atm, outdir))

    def nlte(self, workdir, mu, atm, wave, outdir, mode):
        return self._run(_nlte_job, (workdir, self.pyrh_path, mu, atm, wave, outdir, mode))

    def vacuum_to_air(self, lam_vac):
        return self._run(_vac2air_job, (self.pyrh_path, lam_vac))


def read_dump(outdir: str) -> dict:
    """Load the files written by harness_dump_lte into numpy arrays."""
    meta = np.fromfile(os.path.join(outdir, "meta.i32"), dtype=np.int32)
    nspect, nspace, nrlk, maxcomp = (int(x) for x in meta[:4])
    d = {"meta": meta, "fmeta": np.fromfile(os.path.join(outdir, "fmeta.f64"))}
    f64 = lambda n: np.fromfile(os.path.join(outdir, n + ".f64"))
    i32 = lambda n: np.fromfile(os.path.join(outdir, n + ".i32"), dtype=np.int32)
    d["lambda"] = f64("lambda")
    d["cont"] = f64("cont").reshape(3, nspect, nspace)
    d["cont_flags"] = i32("cont_flags").reshape(nspect, 2)
    d["tot_chi"] = f64("tot_chi").reshape(nspect, 4, nspace)
    d["tot_eta"] = f64("tot_eta").reshape(nspect, 4, nspace)
    d["tot_chip"] = f64("tot_chip").reshape(nspect, 3, nspace)
    d["tot_flags"] = i32("tot_flags").reshape(nspect, 2)
    for n in ["height", "T", "ne", "nHtot", "vturb", "vel", "B", "gamma_B",
              "chi_B", "np", "cos_gamma", "cos_2chi", "sin_2chi"]:
        d[n] = f64(n)
    d["line_const"] = f64("line_const").reshape(nrlk, 24)
    d["line_pops"] = f64("line_pops").reshape(nrlk, 2, nspace)
    mc = max(maxcomp, 1)
    d["zeeman"] = f64("zeeman").reshape(nrlk, 3, mc)
    d["zeeman_n"] = i32("zeeman_n")[:nrlk]
    # inputs of the line-list reader (element data, Barklem tables), when
    # the harness wrote them
    if os.path.exists(os.path.join(outdir, "rlk_element.f64")):
        d["rlk_element"] = f64("rlk_element").reshape(-1, 8)[:nrlk]
        d["rlk_hhe"] = f64("rlk_hhe")
        for t in ("sp", "pd", "df"):
            path = os.path.join(outdir, f"barklem_{t}.f64")
            if os.path.exists(path):
                d[f"barklem_{t}"] = np.fromfile(path)
    return d


def scratch_dir(prefix="rhref_") -> str:
    return tempfile.mkdtemp(prefix=prefix)



# ------------------------------------------------------------------ NLTE --

def make_pyrh_root(atom_name: str, atom_text: str, ref_root: str = REF_ROOT) -> str:
    """Scratch PYRH_PATH: the reference looks model atoms up under
    $PYRH_PATH/rh/Atoms (rh/readatom.c:839-842), so the reference's data files
    are linked there next to the generated model atom."""
    root = tempfile.mkdtemp(prefix="pyrh_root_")
    atoms = os.path.join(root, "rh", "Atoms")
    os.makedirs(atoms)
    src = os.path.join(ref_root, "rh", "Atoms")
    for f in os.listdir(src):
        os.symlink(os.path.join(src, f), os.path.join(atoms, f))
    os.symlink(os.path.join(ref_root, "rh", "Molecules"), os.path.join(root, "rh", "Molecules"))
    with open(os.path.join(atoms, atom_name), "w") as f:
        f.write(atom_text)
    return root


def _nlte_job(args):
    workdir, pyrh_path, mu, atm, wave, outdir, mode = args
    lib = _lib(pyrh_path)
    atm = np.ascontiguousarray(atm, dtype=np.float64)
    wave = np.ascontiguousarray(wave, dtype=np.float64)
    os.makedirs(outdir, exist_ok=True)
    lib.harness_nlte.restype = C.c_int
    return lib.harness_nlte(workdir.encode(), C.c_double(mu), atm.shape[1], _p(atm),
                            len(wave), _p(wave), outdir.encode(), int(mode))


def read_nlte_dump(outdir: str) -> dict:
    f64 = lambda n: np.fromfile(os.path.join(outdir, n + ".f64"))
    i32 = lambda n: np.fromfile(os.path.join(outdir, n + ".i32"), dtype=np.int32)
    ex = lambda n, s: os.path.exists(os.path.join(outdir, n + s))
    d = {}
    if ex("meta", ".i32"):
        m = i32("meta")
        ns, nd, nr, nl, nline, ncont = (int(x) for x in m[:6])
        d["meta"] = m
        d["fmeta"] = f64("fmeta")
        d["lambda"] = f64("lambda")
        for k in ("muz", "wmu", "T", "ne", "nHtot", "vel", "vturb", "height", "g", "E",
                  "ntotal", "vbroad"):
            d[k] = f64(k)
        d["stage"] = i32("stage")
        d["background"] = f64("background").reshape(3, ns, nd)
        d["bgflags"] = i32("bgflags")
        d["J0"] = f64("J0").reshape(ns, nd)
        d["nstar"] = f64("nstar").reshape(nl, nd)
        d["n0"] = f64("n0").reshape(nl, nd)
        d["C"] = f64("C").reshape(nl * nl, nd)
        d["lines"] = f64("lines").reshape(nline, 16)
        d["adamp"] = f64("adamp").reshape(nline, nd)
        d["wphi"] = f64("wphi").reshape(nline, nd)
        d["phi_sample"] = f64("phi_sample").reshape(nline, 5, 2 * nr, nd)
        d["phi_sample_la"] = i32("phi_sample_la").reshape(nline, 5)
        d["continua"] = f64("continua").reshape(ncont, 8)
        d["alpha"] = f64("alpha")
        d["Gamma1"] = f64("Gamma1").reshape(nl * nl, nd)
        d["J1"] = f64("J1").reshape(ns, nd)
        d["n1"] = f64("n1").reshape(nl, nd)
        if ex("R1_line", ".f64"):
            d["R1_line"] = f64("R1_line").reshape(nline, 2, nd)
            d["R1_cont"] = f64("R1_cont").reshape(ncont, 2, nd)
    if ex("n_final", ".f64"):
        nl = len(f64("g")) if ex("g", ".f64") else None
        d["n_final"] = f64("n_final")
        d["J_final"] = f64("J_final")
        d["lam_out"] = f64("lam_out")
        d["I_out"] = f64("I_out")
        if ex("R_final_line", ".f64"):
            d["R_final_line"] = f64("R_final_line")
            d["R_final_cont"] = f64("R_final_cont")
    return d


if __name__ == "__main__":
    import pickle
    import sys
    with open(sys.argv[1], "rb") as f:
        name, args = pickle.load(f)
    result = globals()[name](args)
    with open(sys.argv[2], "wb") as f:
        pickle.dump(result, f)
