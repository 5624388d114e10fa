"""Hydrostatic equilibrium on the CPU: the oracle's restatement of pyrh's
hse() (oracle/hse.py) against the reference's own output (fixture hse:
log tau500 and height scales, another top pressure and a cooler
atmosphere, abundance overrides, fudge factors), and the host pieces of
the GPU path -- the model atoms' data as pyrh_atom_read and
pyrh_gb300.equilibria.setup_from_atoms give them against the reference's parse,
the abundance totals and the element lookup."""
import numpy as np
import pytest

from conftest import HSE_ATOM_ELEMENTS, hse_fudge, hse_oracle_inputs
from oracle import hse as OH
from pyrh_gb300 import grid as G
from pyrh_gb300 import equilibria as EQ
from pyrh_gb300 import hse as H
from pyrh_gb300 import ltepops as LP


@pytest.mark.parametrize("case", range(5))
def test_oracle_hse_matches_reference(golden, case):
    h = golden("hse")
    tab, atoms, mols, ids = hse_oracle_inputs(golden, case)
    ne, nH, rho, pg, passes = OH.hse(tab, atoms, mols, ids, int(h["atm_scale"][case]),
                                     h["scale"][case][None], h["T"][case][None],
                                     float(h["pg_top"][case]), fudge=hse_fudge(golden, case))
    for got, key in ((ne, "ne"), (nH, "nHtot"), (rho, "rho"), (pg, "pg")):
        np.testing.assert_allclose(got[0], h[key][case], rtol=1e-13, atol=0, err_msg=key)
    assert np.all(passes >= 1)


def test_setup_from_atoms_matches_reference_parse(golden):
    """The atom files' levels, continua and lines as the GPU path reads them
    equal the arrays the reference made of the same files."""
    h, bg = golden("hse"), golden("background")
    atoms = [G.read_atom(str(t)) for t in h["atom_text"]]
    elems = [EQ.element_index(a) for a in atoms]
    assert elems == HSE_ATOM_ELEMENTS
    s = EQ.setup_from_atoms(atoms, elems, float(bg["misc"][0]), bg["mol_present"])
    assert np.array_equal(s["atoms_meta"][:, :3], bg["atoms_meta"][:, :3])
    np.testing.assert_array_equal(s["atoms_lev"], bg["atoms_lev"])
    np.testing.assert_array_equal(s["atoms_line"], bg["atoms_line"])
    np.testing.assert_array_equal(s["atoms_cont"][:, :7], bg["atoms_cont"][:, :7])
    assert np.array_equal(s["misc"][:4], bg["misc"][:4])
    # the explicit cross-section tables, row for row
    for r, q in zip(s["atoms_cont"], bg["atoms_cont"]):
        if not int(r[4]):
            n = int(r[6])
            np.testing.assert_array_equal(s["atoms_tab"][int(r[7]):int(r[7]) + n],
                                          bg["atoms_tab"][int(q[7]):int(q[7]) + n])


@pytest.mark.parametrize("ti", [0, 2])
def test_abundance_totals_match_oracle(golden, ti):
    lp = golden("ltepops")
    meta = lp["el_meta"][ti]
    ns = meta[:, 0].astype(np.int32)
    tab = LP.ElementTables(lp["Tpf"], meta[:, 2].copy(), meta[:, 1].astype(np.int32), ns,
                           np.concatenate([[0], np.cumsum(ns)[:-1]]).astype(np.int32),
                           lp["el_pf"], lp["el_ionpot"])
    got = EQ.abundance_totals(tab)
    want = OH.totals({"el_meta": meta})
    assert got == want


def test_element_index():
    lib = EQ._lib()
    for s, e in ((b"H ", 0), (b"H", 0), (b"HE", 1), (b"C ", 5), (b"FE", 25), (b"ES", 98),
                 (b"he", 1), (b"XX", -1)):
        assert lib.pyrh_element_index(s) == e, s


def test_hse_rejects_the_column_mass_scale():
    with pytest.raises(ValueError, match="column-mass"):
        H.hse_batch(None, 1, np.zeros((1, 3)), np.ones((1, 3)))


@pytest.mark.parametrize("case", range(5))
def test_oracle_get_scales_matches_reference(golden, case):
    """The two scales get_scales derives (the given one it leaves unset)."""
    d = golden("scales")
    tab, atoms, mols, ids = hse_oracle_inputs(golden, case, "scales")
    sc = int(d["atm_scale"][case])
    tau, cm, h = OH.get_scales(tab, atoms, mols, ids, sc, d["scale"][case], d["atm"],
                               float(d["lam_ref"][case]))
    got = {"tau": tau, "cmass": cm, "height": h}
    for key in [("cmass", "height"), ("tau", "height"), ("tau", "cmass")][sc]:
        np.testing.assert_allclose(got[key], d[key][case], rtol=1e-13, atol=1e-9, err_msg=key)


def test_oracle_setup_matches_reference_lte_setup(golden):
    """The set-up of a synthesis from the atmosphere alone -- continuum on
    the whole wavelength grid, protons, heights from tau500 -- against the
    reference's own set-up of the lte_c0 run."""
    fx = golden("lte_c0")
    tab, atoms, mols, ids = hse_oracle_inputs(golden, 0)
    chi, eta, npr = OH.continuum(tab, atoms, mols, ids, fx["lam"], fx["T"], fx["ne"],
                                 fx["nHtot"])
    np.testing.assert_allclose(chi, fx["chi_c"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(eta, fx["eta_c"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(npr, fx["np"], rtol=1e-13, atol=0)
    iref = int(np.searchsorted(fx["lam"], float(fx["lambda_ref"])))
    assert fx["lam"][iref] == fx["lambda_ref"]
    tA, w = OH.totals(tab)
    _, _, h = OH.convert_scales(0, fx["atm"][0], fx["T"], fx["ne"], fx["nHtot"], chi[iref], tA, w)
    np.testing.assert_allclose(h, fx["height"], rtol=1e-12, atol=1e-6)


def test_hse_structs_match_compiled_header(tmp_path):
    """sizeof/offsetof of the passive-atom, depth-scale and hse structs as a
    C compiler lays them out from include/pyrh_gb300.h, against the ctypes
    mirrors."""
    import ctypes as C
    import os
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    src = tmp_path / "layout.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "pyrh_gb300.h"\n'
        'int main(void) { printf("%zu %zu %zu %zu %zu %zu %zu %zu\\n", '
        'sizeof(pyrh_passive_atoms), offsetof(pyrh_passive_atoms, E), '
        'sizeof(pyrh_scales_batch), offsetof(pyrh_scales_batch, scale_in), '
        'sizeof(pyrh_hse_config), offsetof(pyrh_hse_config, eta_limit), '
        'sizeof(pyrh_hse_batch), offsetof(pyrh_hse_batch, niter)); return 0; }\n')
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", inc, str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True,
                                          text=True).stdout.split()]
    assert got == [C.sizeof(EQ.PassiveAtoms), EQ.PassiveAtoms.E.offset,
                   C.sizeof(EQ.ScalesBatch), EQ.ScalesBatch.scale_in.offset,
                   C.sizeof(H.HseConfig), H.HseConfig.eta_limit.offset,
                   C.sizeof(H.HseBatch), H.HseBatch.niter.offset]


def test_argument_checks_before_any_device_work():
    """The entry points refuse bad arguments with a status and a message,
    before they touch the device (so these run without a GPU)."""
    import ctypes as C
    from pyrh_gb300 import _lib as L
    lib = EQ._lib()
    H._lib()
    b = EQ.ScalesBatch(natm=1, ndep=1, scale=0)           # fewer than 2 depth points
    assert lib.pyrh_convert_scales(C.byref(b), None) == L.PYRH_ERR_ARG
    assert b"convert scales" in lib.pyrh_last_error()
    b = EQ.ScalesBatch(natm=1, ndep=4, scale=3)
    for f in ("scale_in", "T", "ne", "nHtot", "chi_ref", "tau_ref", "cmass", "height"):
        setattr(b, f, 8)
    assert lib.pyrh_convert_scales(C.byref(b), None) == L.PYRH_ERR_ARG
    assert b"scale" in lib.pyrh_last_error()
    # no atoms, no molecules: refused before any allocation
    tabs = LP.ElemTables()
    atoms = EQ.PassiveAtoms()
    assert lib.pyrh_equilibria(C.byref(tabs), None, 0, C.byref(atoms), 4, *([None] * 7)) == \
        L.PYRH_ERR_ARG
    assert lib.pyrh_equilibria(C.byref(tabs), None, 0, C.byref(atoms), 0, *([None] * 7)) == \
        L.PYRH_ERR_ARG
    cfg = H.HseConfig(scale=1, nmax_iter=50, total_abund=1.1, wght_per_H=1.4)
    hb = H.HseBatch(natm=2, ndep=3)
    for f in ("scale", "T", "pg_top", "ne", "nHtot", "rho", "pg"):
        setattr(hb, f, 8)
    from pyrh_gb300 import background as BG
    from pyrh_gb300 import chem as CH
    mols = (CH.Molecule * 1)()
    st = lib.pyrh_hse(C.byref(tabs), mols, 1, C.byref(BG.BgModel()), C.byref(atoms),
                      C.byref(cfg), C.byref(hb), None)
    assert st == L.PYRH_ERR_UNSUPPORTED and b"column-mass" in lib.pyrh_last_error()
    hb.natm = 0
    st = lib.pyrh_hse(C.byref(tabs), mols, 1, C.byref(BG.BgModel()), C.byref(atoms),
                      C.byref(cfg), C.byref(hb), None)
    assert st == L.PYRH_ERR_ARG
