"""Element tables, LTE stage populations and the electron density, on the
CPU: the oracle restatement (oracle/ltepops.py) against the reference's own
LTEpops_elem and Solve_ne output (fixture ltepops, made by
tests/golden/make_golden.py), and the host readers of the abundance and
partition-function files (elements_host.cpp) against the tables the
reference parsed."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import REPO
from oracle import ltepops as O
from oracle import ref_runner
from pyrh_gb300 import ltepops as LP


def _tab(fx, case=0):
    return {"Tpf": fx["Tpf"], "el_meta": fx["el_meta"][case], "el_pf": fx["el_pf"],
            "el_ionpot": fx["el_ionpot"]}


@pytest.mark.parametrize("case", [0, 1, 2])
def test_oracle_stage_pops_match_reference(golden, case):
    fx = golden("ltepops")
    tab = _tab(fx, case)
    ns = fx["el_meta"][case][:, 0].astype(int)
    off = np.concatenate([[0], np.cumsum(ns)[:-1]])
    for e in (0, 1, 5, 10, 11, 19, 25, 27, 55):     # H He C Na Mg Ca Fe Ni Ba
        n = O.stage_pops(tab, e, fx["T"][case], fx["ne"][case], fx["nHtot"][case])
        ref = fx["el_n"][case][off[e]:off[e] + ns[e]]
        np.testing.assert_allclose(n, ref, rtol=1e-13, atol=0, err_msg=f"element {e + 1}")


@pytest.mark.parametrize("case", [0, 1, 2])
def test_oracle_solve_ne_matches_reference(golden, case):
    fx = golden("ltepops")
    tab = _tab(fx, case)
    sel = np.arange(0, 71, 7)
    ne, steps = O.solve_ne(tab, fx["T"][case][sel], fx["nHtot"][case][sel])
    np.testing.assert_allclose(ne, fx["ne_solved"][case][sel], rtol=1e-12, atol=0)
    assert np.all(steps >= 1)
    ne, _ = O.solve_ne(tab, fx["T"][case][sel], fx["nHtot"][case][sel], fx["ne"][case][sel])
    np.testing.assert_allclose(ne, fx["ne_warm"][case][sel], rtol=1e-12, atol=0)


def test_abundance_reader_matches_reference(golden):
    """Record matching, DEX conversion and the overrides by record number:
    the abundances the reference's readAbundance produced, in all three
    cases (the third overrides records 1 and 26)."""
    fx = golden("ltepops")
    text = str(fx["abundance_text"])
    for case in range(3):
        ids = fx["ab_id"][case]
        keep = ids >= 0
        abund, aset = LP.read_abundance(text, ids[keep], fx["ab_val"][case][keep])
        ref = fx["el_meta"][case]
        assert np.array_equal(aset, ref[:, 1].astype(np.int32))
        np.testing.assert_allclose(abund, ref[:, 2], rtol=2e-16, atol=0)


def test_abundance_reader_rules():
    text = "# comment\n\n  H  12.00\n  he 10.99\n#  C  8.60\n  C  8.39  ## note\n  XX 1.0\n"
    abund, aset = LP.read_abundance(text, metallicity=0.5)
    assert aset[0] == aset[1] == aset[5] == 1 and aset.sum() == 3
    assert abund[0] == 1.0
    np.testing.assert_allclose(abund[1], 10 ** (10.99 - 12) * 10 ** 0.5, rtol=1e-14)
    np.testing.assert_allclose(abund[5], 10 ** (8.39 - 12) * 10 ** 0.5, rtol=1e-14)
    # override of the third record (C), not of element 3
    abund, _ = LP.read_abundance(text, [3], [7.0])
    np.testing.assert_allclose(abund[5], 1e-5, rtol=1e-14)
    assert abund[2] == 0.0
    # linear scale when hydrogen is not 12.0
    abund, _ = LP.read_abundance("H 1.0\nHE 0.1\n")
    assert abund[0] == 1.0 and abund[1] == 0.1
    with pytest.raises(RuntimeError):
        LP.read_abundance("H\n")


def _pf_bytes(tab_T, rows):
    """An XDR partition-function file of 99 elements with the given
    [nstage, npf] U tables and potentials (cm^-1)."""
    out = [np.array([len(tab_T)], ">i4").tobytes(), np.asarray(tab_T, ">f8").tobytes()]
    for z, (U, ion) in enumerate(rows, start=1):
        out.append(np.array([z, U.shape[0]], ">i4").tobytes())
        out.append(np.asarray(U, ">f8").tobytes())
        out.append(np.asarray(ion, ">f8").tobytes())
    return b"".join(out)


def test_pf_reader_layout_and_conversion():
    T = np.array([1000.0, 2000.0, 4000.0])
    rng = np.random.default_rng(3)
    rows = [(1.0 + rng.random((1 + z % 4, 3)), 1000.0 * (1 + np.arange(1 + z % 4)))
            for z in range(99)]
    data = _pf_bytes(T, rows)
    aset = np.ones(99, np.int32)
    aset[7] = 0
    Tpf, nstage, off, lnpf, ion = LP.read_pf(data, aset)
    assert np.array_equal(Tpf, T)
    assert np.array_equal(nstage, [r[0].shape[0] for r in rows])
    assert np.array_equal(off, np.concatenate([[0], np.cumsum(nstage)[:-1]]))
    for e, (U, v) in enumerate(rows):
        s = slice(off[e], off[e] + nstage[e])
        if aset[e]:
            np.testing.assert_allclose(lnpf[s], np.log(U), rtol=4e-16, atol=0)   # numpy's log
            np.testing.assert_array_equal(ion[s], v * ((6.6260755E-34 * 2.99792458E+08) / 1.0E-02))
        else:    # kept as read, as the reference keeps elements without an abundance
            np.testing.assert_array_equal(lnpf[s], U)
            np.testing.assert_array_equal(ion[s], v)
    with pytest.raises(RuntimeError):
        LP.read_pf(data[:-8], aset)          # truncated


def test_pf_reader_matches_reference_file(golden):
    """The reference's own pf_Kurucz.input, read here, against the tables
    its readAbundance produced (only where the reference sources exist)."""
    if not ref_runner.REF_ROOT:
        pytest.skip("reference sources not present")
    fx = golden("ltepops")
    with open(os.path.join(ref_runner.REF_ROOT, "rh", "Atoms", "pf_Kurucz.input"), "rb") as f:
        data = f.read()
    Tpf, nstage, off, lnpf, ion = LP.read_pf(data, fx["el_meta"][0][:, 1].astype(np.int32))
    assert np.array_equal(Tpf, fx["Tpf"])
    assert np.array_equal(nstage, fx["el_meta"][0][:, 0].astype(np.int32))
    np.testing.assert_array_equal(lnpf, fx["el_pf"])
    np.testing.assert_array_equal(ion, fx["el_ionpot"])


def test_elem_tables_struct_layout():
    assert C.sizeof(LP.ElemTables) == 8 + 6 * 8
