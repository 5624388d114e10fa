"""ctypes view of libpyrh_gb300.so (declarations mirror include/pyrh_gb300.h)."""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("PYRH_GB300_LIB", os.path.join(HERE, "libpyrh_gb300.so"))

PYRH_OK = 0
PYRH_ERR_ARG = 1
PYRH_ERR_UNSUPPORTED = 2
PYRH_ERR_CUDA = 3
PYRH_ERR_NONCONVERGED = 4
PYRH_ERR_SINGULAR = 5
PYRH_ERR_TIMEOUT = 6

PYRH_FP64 = 0
PYRH_FP32 = 1
PYRH_NO_STOKES = 0
PYRH_FULL_STOKES = 3

PYRH_MAX_LINES = 16
PYRH_MAX_COMPONENTS = 32
PYRH_MAX_DEPTH = 512
PYRH_RF_NPARAM = 6
PYRH_RF_MAX_DEPTH = 160
PYRH_NLTE_MAX_LEVELS = 8
PYRH_NLTE_MAX_ACTIVE = 16
PYRH_NLTE_MAX_RAYS = 8
PYRH_NLTE_MAX_DEPTH = 160
PYRH_NLTE_MAX_NG = 4

_D = C.POINTER(C.c_double)
_I32 = C.POINTER(C.c_int32)
_I64 = C.POINTER(C.c_int64)


class PyrhLine(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "lambda0", "Ei", "gi", "Aji", "Bji", "Bij", "Grad", "GStark", "GvdWaals",
        "cross", "alpha", "isotope_frac", "hyperfine_frac", "weight")] + [
        ("vdwaals", C.c_int32), ("contributes", C.c_int32), ("polarizable", C.c_int32),
        ("ncomp", C.c_int32), ("comp_q", C.c_int32 * PYRH_MAX_COMPONENTS),
        ("comp_shift", C.c_double * PYRH_MAX_COMPONENTS),
        ("comp_strength", C.c_double * PYRH_MAX_COMPONENTS)]


class PyrhLteBatch(C.Structure):
    _fields_ = [("natm", C.c_int32), ("max_ndep", C.c_int32), ("max_nlam", C.c_int32),
                ("total_depth", C.c_int64),
                ("ndep", C.c_void_p), ("depth_off", C.c_void_p), ("nlam", C.c_void_p),
                ("lam_off", C.c_void_p), ("cont_off", C.c_void_p), ("lambda_", C.c_void_p)] + \
        [(n, C.c_void_p) for n in ("height", "T", "ne", "nHtot", "np", "vturb", "vlos", "B",
                                   "gamma_B", "chi_B", "line_pops", "chi_c", "eta_c",
                                   "setup_dT")]


class PyrhLteSetupDT(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("dchi_c", "deta_c", "dline_pops", "dnp", "dlen_up",
                                          "dlen_dn")]


class PyrhLteConfig(C.Structure):
    _fields_ = [("precision", C.c_int32), ("stokes_mode", C.c_int32),
                ("magneto_optical", C.c_int32), ("moving", C.c_int32),
                ("mu", C.c_double), ("vmicro_char", C.c_double),
                ("block_lambda", C.c_int32), ("persistent_blocks", C.c_int32)]


class PyrhError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"pyrh_gb300 status {status}: {msg}")
        self.status = status


_lib = None


def lib(build_if_missing: bool = True):
    """Load the CUDA library.  There is no CPU fallback: a missing library
    is an error (or is built from source when nvcc is available)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise ImportError(f"{LIB_PATH} is missing; run pyrh_gb300.build.build()")
        from . import build as _build
        _build.build()
    L = C.CDLL(LIB_PATH)
    L.pyrh_version.restype = C.c_char_p
    L.pyrh_last_error.restype = C.c_char_p
    L.pyrh_last_launch_count.restype = C.c_int32
    L.pyrh_lte_stokes.restype = C.c_int
    L.pyrh_lte_stokes.argtypes = [C.POINTER(PyrhLteBatch), C.c_void_p, C.c_int32,
                                  C.POINTER(PyrhLteConfig), C.c_void_p, C.c_void_p]
    L.pyrh_lte_stokes_host.restype = C.c_int
    L.pyrh_lte_stokes_host.argtypes = [C.POINTER(PyrhLteBatch), C.POINTER(PyrhLine), C.c_int32,
                                       C.POINTER(PyrhLteConfig), C.c_void_p]
    L.pyrh_check_lines.restype = C.c_int
    L.pyrh_check_lines.argtypes = [C.POINTER(PyrhLine), C.c_int32, C.c_int32]
    _lib = L
    return L


def check(status: int) -> None:
    if status != PYRH_OK:
        raise PyrhError(status, lib().pyrh_last_error().decode())


EXPORTED = ["pyrh_lte_stokes", "pyrh_lte_stokes_host", "pyrh_check_lines",
            "pyrh_last_launch_count", "pyrh_version", "pyrh_last_error"]
