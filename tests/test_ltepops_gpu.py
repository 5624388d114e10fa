"""LTE stage populations, line stage densities and the electron density on
the GPU (ltepops.cu through the C ABI) against the reference's own output:
LTEpops_elem and Solve_ne of the ltepops fixture, and the stage densities
and ln U that rlk_opacity read in the LTE fixtures (their line_pops)."""
import numpy as np
import pytest

from pyrh_gb300 import _lib as L
from pyrh_gb300 import ltepops as LP

pytestmark = pytest.mark.gpu


def _tables(fx, case=0):
    meta = fx["el_meta"][case]
    ns = meta[:, 0].astype(np.int32)
    off = np.concatenate([[0], np.cumsum(ns)[:-1]]).astype(np.int32)
    return LP.ElementTables(fx["Tpf"], meta[:, 2].copy(), meta[:, 1].astype(np.int32), ns, off,
                            fx["el_pf"], fx["el_ionpot"])


@pytest.mark.parametrize("case", [0, 1, 2])
def test_stage_pops_match_reference(golden, case):
    fx = golden("ltepops")
    tab = _tables(fx, case)
    dev = LP.DeviceTables(tab)
    sel = np.arange(99)
    n = LP.stage_pops(dev, fx["T"][case], fx["ne"][case], fx["nHtot"][case], sel).cpu().numpy()
    np.testing.assert_allclose(n, fx["el_n"][case], rtol=1e-12, atol=0)
    assert L.lib().pyrh_last_launch_count() == 1


@pytest.mark.parametrize("case", [0, 1, 2])
def test_solve_ne_matches_reference(golden, case):
    fx = golden("ltepops")
    dev = LP.DeviceTables(_tables(fx, case))
    ne, it = LP.solve_ne(dev, fx["T"][case], fx["nHtot"][case], return_iterations=True)
    np.testing.assert_allclose(ne.cpu().numpy(), fx["ne_solved"][case], rtol=1e-12, atol=0)
    assert np.all(it.cpu().numpy() >= 1)
    ne = LP.solve_ne(dev, fx["T"][case], fx["nHtot"][case], ne_start=fx["ne"][case])
    np.testing.assert_allclose(ne.cpu().numpy(), fx["ne_warm"][case], rtol=1e-12, atol=0)


@pytest.mark.parametrize("name", ["lte_c0", "lte_edge", "lte_broadening", "lte_mixed"])
def test_line_pops_match_reference(golden, name):
    """line_pops of an LTE fixture (the reference's element->n[stage] and
    Linear(pf[stage]) in rlk_opacity) from the atmosphere alone."""
    fx = golden(name)
    lp = golden("ltepops")
    dev = LP.DeviceTables(_tables(lp, 0))
    elem = fx["line_const"][:, 1].astype(np.int32) - 1
    stage = fx["line_const"][:, 2].astype(np.int32)
    out = LP.line_pops(dev, fx["T"], fx["ne"], fx["nHtot"], elem, stage).cpu().numpy()
    np.testing.assert_allclose(out, fx["line_pops"], rtol=1e-12, atol=0)


def test_batched_points_and_limits(golden):
    """Many atmospheres in one launch equal each alone; bad indices are
    refused before any launch; empty batches are no-ops."""
    fx = golden("ltepops")
    dev = LP.DeviceTables(_tables(fx, 0))
    cases = (0, 1)           # the two atmospheres with the file's own abundances
    T = np.concatenate([fx["T"][c] for c in cases] * 50)
    nH = np.concatenate([fx["nHtot"][c] for c in cases] * 50)
    ne = LP.solve_ne(dev, T, nH).cpu().numpy()
    ref = np.concatenate([fx["ne_solved"][c] for c in cases] * 50)
    np.testing.assert_allclose(ne, ref, rtol=1e-12, atol=0)
    with pytest.raises(RuntimeError):
        LP.line_pops(dev, T, T, nH, [25], [7])       # Fe has fewer stages
    with pytest.raises(ValueError):
        LP.stage_pops(dev, T, T, nH, [99])
    assert LP.line_pops(dev, T[:0], T[:0], nH[:0], [25], [0]).numel() == 0


def test_get_ne_from_nH_units(golden):
    """pyrh.get_ne_from_nH's units: nH and the result in cm^-3."""
    fx = golden("ltepops")
    tab = _tables(fx, 0)
    ne = LP.get_ne_from_nH(".", 0, np.zeros(71), fx["T"][0], fx["nHtot"][0] * 1e-6, tables=tab)
    np.testing.assert_allclose(ne, fx["ne_solved"][0] * (1e-2 * 1e-2 * 1e-2), rtol=1e-12, atol=0)
