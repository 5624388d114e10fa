"""The Kurucz line-list reader (pyrh_kurucz_read, pyrh_barklem_parse through
the C ABI) against the reference's own reader: for the line lists of
lte_c0 (Barklem s-p broadening), lte_broadening (orbital numbers no table
covers, so Unsold; isotope and hyperfine fractions) and lte_mixed (lines
that are not polarizable), the fixture tests/golden/kurucz_lists.npz holds
the list text, the element data and Barklem tables the reference used, and
the line constants and Zeeman patterns its readKuruczLines / RLKZeeman made.

Every field must be identical except the van der Waals cross-section
(within 1e-13: the log-gamma function of the C library against the
reference's series) and alpha of lines with Unsold broadening (unset and
unused in the reference)."""
import os

import numpy as np
import pytest

from pyrh_gb300 import kurucz as K

LISTS = ["c0", "broadening", "mixed"]


@pytest.fixture(scope="module")
def kz():
    with np.load(os.path.join(os.path.dirname(__file__), "golden", "kurucz_lists.npz")) as f:
        return {k: f[k] for k in f.files}


def tables_of(kz):
    tabs = K._Tables()
    for t, name in enumerate(("sp", "pd", "df")):
        a = kz["barklem_" + name]
        n1, n2 = int(a[0]), int(a[1])
        n12 = n1 * n2
        K.barklem_from_arrays(n1, n2, a[2], a[3], a[4:4 + n12], a[4 + n12:4 + 2 * n12], tabs, t)
    return tabs


def elements_of(kz, lst):
    lc, el, hhe = kz[lst + "_line_const"], kz[lst + "_rlk_element"], kz[lst + "_rlk_hhe"]
    elements = {1: (hhe[0], hhe[1], 2, 1, [0.0, 0.0]), 2: (hhe[2], hhe[3], 3, 1, [0.0] * 3)}
    for i in range(len(lc)):
        e = el[i]
        elements[int(lc[i, 1])] = (e[0], e[2], int(e[1]), int(e[3]), list(e[4:8]))
    return elements


@pytest.mark.parametrize("lst", LISTS)
def test_reader_matches_reference(kz, lst):
    lines, n, extra = K.read_kurucz(str(kz[lst + "_text"]), elements_of(kz, lst), tables_of(kz))
    lc, zm, zn = K.line_tables(lines, n, extra)
    ref = kz[lst + "_line_const"]
    assert lc.shape[0] == ref.shape[0]
    exact = [c for c in range(23) if c not in (14, 15)]
    assert np.array_equal(lc[:, exact], ref[:, exact])
    assert np.allclose(lc[:, 14], ref[:, 14], rtol=1e-13, atol=0)
    barklem = ref[:, 13] == 2
    assert np.array_equal(lc[barklem, 15], ref[barklem, 15])
    assert np.array_equal(zn, kz[lst + "_zeeman_n"])
    nc = zm.shape[2]
    assert np.array_equal(zm, kz[lst + "_zeeman"][:, :, :nc])
    assert not np.any(kz[lst + "_zeeman"][:, :, nc:])


def test_loggf_override(kz):
    """A log gf override by record index recomputes Aji, Bji, Bij (and the
    radiative damping only where it follows Aji) of that line alone."""
    base = K.line_tables(*K.read_kurucz(str(kz["c0_text"]), elements_of(kz, "c0"),
                                        tables_of(kz)))[0]
    mod = K.line_tables(*K.read_kurucz(str(kz["c0_text"]), elements_of(kz, "c0"), tables_of(kz),
                                       loggf_ids=[1], loggf_values=[-0.24]))[0]
    assert np.array_equal(mod[0], base[0])
    assert np.allclose(mod[1, 7:10] / base[1, 7:10], 10.0, rtol=1e-12)
    assert np.array_equal(np.delete(mod[1], [7, 8, 9]), np.delete(base[1], [7, 8, 9]))


def test_barklem_text_parser(kz):
    """pyrh_barklem_parse on the reference's own table files (only where the
    reference's sources are on this machine) gives the tables its reader
    parsed."""
    from oracle import ref_runner
    if not ref_runner.REF_ROOT:
        pytest.skip("reference sources not on this machine")
    for t, name in enumerate(("sp", "pd", "df")):
        path = os.path.join(ref_runner.REF_ROOT, "rh", "Atoms", f"Barklem_{name}data.dat")
        with open(path) as f:
            tabs = K.barklem_tables({t: f.read()})
        tb = tabs.tables[t]
        a = kz["barklem_" + name]
        n12 = int(a[0]) * int(a[1])
        assert (tb.n1, tb.n2, tb.neff1_0, tb.neff2_0) == (int(a[0]), int(a[1]), a[2], a[3])
        assert np.array_equal(np.ctypeslib.as_array(tb.cross, (n12,)), a[4:4 + n12])
        assert np.array_equal(np.ctypeslib.as_array(tb.alpha, (n12,)), a[4 + n12:4 + 2 * n12])


def test_reader_rejects_bad_records(kz):
    els = elements_of(kz, "c0")
    with pytest.raises(Exception):
        K.read_kurucz("630.0 -1.0 26.00\n", els)          # truncated record
    bad = str(kz["c0_text"]).replace("26.00", "99.00", 1)  # element outside the table
    with pytest.raises(Exception):
        K.read_kurucz(bad, els)
