"""The C ABI library loads and exports every entry point that
include/pyrh_gb300.h declares; argument checks run without a GPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import REPO
from pyrh_gb300 import _lib as L
from pyrh_gb300 import lte


def _declared():
    names = set()
    for f in os.listdir(os.path.join(REPO, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(REPO, "include", f)).read()
            names |= set(re.findall(r"^\s*(?:pyrh_status|int32_t|size_t|double|void|const char \*)\s*(pyrh_\w+)\s*\(",
                                    src, re.M))
    return names


def test_library_exports_all_declared_symbols():
    lib = L.lib()
    declared = _declared()
    assert declared, "no declarations parsed"
    for name in declared:
        assert hasattr(lib, name), name
    assert set(L.EXPORTED) <= declared
    assert b"sm_103a" in lib.pyrh_version()


def test_struct_sizes_match_header_layout():
    # 14 doubles + 4 int32 + 32 int32 + 64 doubles
    assert C.sizeof(L.PyrhLine) == 14 * 8 + 4 * 4 + 32 * 4 + 64 * 8
    assert C.sizeof(L.PyrhLteConfig) == 4 * 4 + 2 * 8 + 2 * 4
    # 3 int32 (+4 padding), 1 int64, 19 array pointers, the set-up derivative pointer
    assert C.sizeof(L.PyrhLteBatch) == 16 + 8 + 20 * 8
    assert L.PyrhLteBatch.setup_dT.offset == 16 + 8 + 19 * 8
    assert C.sizeof(L.PyrhLteSetupDT) == 6 * 8


def test_constants_match_header():
    """Every numeric #define of include/pyrh_gb300.h that the Python layer
    mirrors has the header's value."""
    hdr = open(os.path.join(REPO, "include", "pyrh_gb300.h")).read()
    defines = dict(re.findall(r"#define\s+(PYRH_\w+)\s+(\d+)\b", hdr))
    enums = dict(re.findall(r"\b(PYRH_\w+)\s*=\s*(\d+)", hdr))
    mirrored = {k: getattr(L, k) for k in dir(L) if k.startswith("PYRH_")
                and isinstance(getattr(L, k), int)}
    assert mirrored
    for k, v in mirrored.items():
        assert k in defines or k in enums, k
        assert int(defines.get(k, enums.get(k))) == v, k


def test_struct_layout_matches_compiled_header(tmp_path):
    """sizeof/offsetof of the batch structs as a C compiler lays them out
    from include/pyrh_gb300.h, against the ctypes mirror."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "layout.c"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "pyrh_gb300.h"\n'
                   'int main(void) { printf("%zu %zu %zu %zu\\n", sizeof(pyrh_lte_batch), '
                   'offsetof(pyrh_lte_batch, setup_dT), sizeof(pyrh_lte_setup_dT), '
                   'sizeof(pyrh_lte_config)); return 0; }\n')
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", inc, str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True,
                                          text=True).stdout.split()]
    assert got == [C.sizeof(L.PyrhLteBatch), L.PyrhLteBatch.setup_dT.offset,
                   C.sizeof(L.PyrhLteSetupDT), C.sizeof(L.PyrhLteConfig)]


def test_config_validation_without_gpu(golden):
    fx = golden("lte_c0")
    lines, n = lte.make_lines(fx["line_const"], fx["zeeman"], fx["zeeman_n"])
    pk = lte.pack([fx], n)
    for bad in (dict(mu=0.0), dict(mu=1.5), dict(precision=7), dict(block_lambda=48),
                dict(stokes_mode=1)):
        cfg = lte.make_config(**bad)
        with pytest.raises(L.PyrhError) as e:
            lte.synth_host(pk, lines, n, cfg)
        assert e.value.status == L.PYRH_ERR_ARG


def test_line_checks(golden):
    fx = golden("lte_c0")
    lines, n = lte.make_lines(fx["line_const"], fx["zeeman"], fx["zeeman_n"])
    lib = L.lib()
    assert lib.pyrh_check_lines(lines, n, L.PYRH_FULL_STOKES) == L.PYRH_OK
    bad, _ = lte.make_lines(fx["line_const"][::-1].copy(), fx["zeeman"][::-1].copy(),
                            fx["zeeman_n"][::-1].copy())
    assert lib.pyrh_check_lines(bad, n, L.PYRH_FULL_STOKES) == L.PYRH_ERR_ARG
    lc = fx["line_const"].copy()
    lc[0, 18] = 0   # not polarizable: Armstrong's Voigt function, Stokes I only
    unp, _ = lte.make_lines(lc, fx["zeeman"], fx["zeeman_n"])
    assert lib.pyrh_check_lines(unp, n, L.PYRH_FULL_STOKES) == L.PYRH_OK
    assert lib.pyrh_check_lines(lines, L.PYRH_MAX_LINES + 1, 3) == L.PYRH_ERR_ARG


def test_pack_layout(golden):
    fx = golden("lte_c0")
    b = golden("lte_batch")
    from conftest import batch_member
    atms = [fx, batch_member(b, 0)]
    pk = lte.pack(atms, 2)
    a = pk.arrays
    assert list(a["ndep"]) == [71, 71]
    assert list(a["nlam"]) == [len(fx["lam"]), len(b["lam"][0])]
    assert a["cont_off"][1] == 71 * len(fx["lam"])
    # continuum is [depth][lambda] per atmosphere
    assert a["chi_c"][5 * len(fx["lam"]) + 7] == fx["chi_c"][7, 5]


def test_nlte_structs_and_workspace_without_gpu(golden):
    import ctypes as C
    from pyrh_gb300 import nlte
    assert C.sizeof(nlte.PyrhNlteTransition) == 10 * 4 + 2 * 8 + 7 * 8
    fx = golden("nlte_c1")
    cfg = nlte.make_config(fx)
    pk = nlte.pack([fx], cfg.nrays)
    b = nlte.PyrhNlteBatch()
    b.natm, b.nlevel = pk.natm, pk.nlevel
    for k, v in pk.shape.items():
        setattr(b, k, v)
    n = nlte._lib().pyrh_nlte_workspace_bytes(C.byref(b), C.byref(cfg), pk.phi_elems)
    # profiles dominate: 663 line wavelengths x 10 ray-directions x 82 depths
    assert n >= 8 * pk.phi_elems
    assert pk.phi_elems == sum(int(l[8]) for l in fx["lines"]) * 10 * 82
    # transitions: continua first, then lines, as the active sets are built
    types = [pk.trans[i].type for i in range(pk.ntrans_total)]
    assert types == [1] * len(fx["continua"]) + [0] * len(fx["lines"])


def test_rf_tile_width_checked_without_gpu(golden):
    """The response-function kernel takes tiles up to its block size (512
    threads in FP32, 128 in FP64): wider tiles are refused before any
    device work."""
    fx = golden("lte_c0")
    lines, n = lte.make_lines(fx["line_const"], fx["zeeman"], fx["zeeman_n"])
    pk = lte.pack([fx], n)
    arrs = {k: np.ascontiguousarray(v) for k, v in pk.arrays.items()}
    b = lte._batch_struct(pk, lambda k: arrs[k].ctypes.data)
    cfg = lte.make_config(precision=L.PYRH_FP64, block_lambda=160)
    lib = L.lib()
    dummy = C.c_void_p(1)
    s = lib.pyrh_lte_rf(C.byref(b), C.cast(lines, C.c_void_p), n, C.byref(cfg), dummy, dummy,
                        None, None)
    assert s == L.PYRH_ERR_ARG
    assert b"block_lambda 160 above 128" in lib.pyrh_last_error()
