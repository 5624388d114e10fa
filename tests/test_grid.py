"""Host-side set-up through the C ABI (pyrh_atom_read, pyrh_line_grid,
pyrh_cont_grid, pyrh_sort_lambda, pyrh_output_index, pyrh_cont_alpha)
against the compiled reference's own set-up state: the global wavelength
grid, each transition's index range and the hydrogenic cross-sections of
the NLTE fixtures (made by the reference's readAtom / getLambda /
SortLambda), and the grid and output wavelengths of every LTE fixture.
Integers and wavelengths must be identical, not close."""
import numpy as np
import pytest

from pyrh_gb300 import _lib as L
from pyrh_gb300 import grid as G

NLTE = ["nlte_c1", "nlte_c4_50", "nlte_c4_120", "nlte_static"]
LTE = ["lte_c0", "lte_edge", "lte_b0", "lte_mixed", "lte_static", "lte_static_v",
       "lte_nostokes", "lte_broadening"]


@pytest.mark.parametrize("name", NLTE)
def test_nlte_grid_matches_reference(golden, name):
    fx = golden(name)
    atom = G.read_atom(str(fx["atom_text"]))
    assert (atom.nlevel, atom.nline, atom.ncont) == tuple(int(x) for x in fx["meta"][3:6])
    # VMICRO_CHAR = 5 km/s and B_STRENGTH_CHAR = 0 in the fixtures' keyword.input
    g = G.nlte_grid(atom, fx["wave"], float(fx["fmeta"][1]), 5.0, moving=bool(fx["meta"][12]))
    assert np.array_equal(g.lam, fx["lambda"])
    assert np.array_equal(g.line_range, fx["lines"][:, 7:9].astype(np.int32))
    assert np.array_equal(g.cont_range, fx["continua"][:, 2:4].astype(np.int32))
    assert np.array_equal(np.concatenate(g.alpha), fx["alpha"])
    assert np.array_equal(g.lam[g.out_index], fx["lam_out"])
    # the caller's wavelength sits where the reference put it
    assert np.all(g.lam[g.wave_inds] == fx["wave"])
    # line constants of the reader against the reference's transition table
    for kr in range(atom.nline):
        ln, ref = atom.line[kr], fx["lines"][kr]
        assert (ln.i, ln.j) == (int(ref[0]), int(ref[1]))
        assert ln.lambda0 == ref[2] and ln.Aji == ref[3] and ln.Bji == ref[4] and ln.Bij == ref[5]
        # whether the line polarizes the active set (NO_STOKES: only
        # FIELD_FREE would not)
        assert G.line_polarized(atom, kr) == bool(ref[15])
        assert not G.line_polarized(atom, kr, field_free=True)


@pytest.mark.parametrize("name", LTE)
def test_lte_grid_matches_reference(golden, name):
    fx = golden(name)
    g = G.lte_grid(fx["wave"], float(fx["lambda_ref"]))
    assert np.array_equal(g.lam, fx["lam"])
    assert np.array_equal(g.lam[g.out_index], fx["lam_out"])


def test_sort_lambda_edge_cases():
    # duplicates (strictly larger kept), unsorted input, lambda_ref among the
    # caller's wavelengths (then dropped from the output with it)
    g = G.lte_grid([630.2, 630.1, 630.2, 500.0, 630.15], 500.0)
    assert np.array_equal(g.lam, [500.0, 630.1, 630.15, 630.2])
    assert np.array_equal(g.out_index, [1, 2, 3])
    # the reference searches each caller wavelength from the previous one's
    # index on (its spectrum.wave_inds assume an ascending table); one not
    # found that way is -1 here
    assert np.array_equal(g.wave_inds, [3, -1, 3, -1, -1])
    assert np.array_equal(G.lte_grid([500.0, 630.1, 630.15], 500.0).wave_inds, [0, 1, 2])
    # lambda_ref off the grid cannot happen with lambda_ref > 0; with 0 it
    # is not added, and the output index refuses a grid without it
    with pytest.raises(RuntimeError):
        G.lte_grid([630.1, 630.2], 0.0)


def test_atom_reader_rejects_bad_input():
    lib = G._lib()
    atom = G.Atom()
    assert lib.pyrh_atom_read(b"CA\n 2 1 0 0\n 0.0 2.0 'A' 1 0\n", atom) == L.PYRH_ERR_ARG
    bad_coll = ("CA\n 2 0 1 0\n 0.0 2.0 'CA II 3P6 4S 2SE    ' 1 0\n"
                " 95752.0 1.0 'CA III 3P6 1SE      ' 2 1\n"
                " 1 0 1.0E-22 10 HYDROGENIC 36.0\n TEMP 2 3000.0 5000.0\n"
                " SHULL82 0 1 1.0 2.0\n END\n")
    assert lib.pyrh_atom_read(bad_coll.encode(), atom) == L.PYRH_ERR_UNSUPPORTED
