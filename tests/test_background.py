"""Background continuum (Background(), rh/background.c:329-460): the numpy
oracle (oracle/background.py) against the reference's own output in the
`background` fixture -- every process alone and the totals, for the C0
atmosphere and a cooler one over 120-20000 nm -- and the host side of the
GPU entry points (model layout, struct sizes).

Tolerances (relative): totals 1e-13, each process 1e-12 of its largest
value (the same formulas; libm pow/exp against the reference's)."""
import ctypes as C

import numpy as np
import pytest

from oracle import background as BG
from pyrh_gb300 import background as B


@pytest.fixture(scope="module")
def bgfx(golden):
    return golden("background")


@pytest.mark.parametrize("a", [0, 1])
def test_oracle_totals_match_reference(bgfx, a):
    chi, eta, sca, _ = BG.background(bgfx, a)
    ref = bgfx["cont"][a]
    for x, r in ((chi, ref[0]), (eta, ref[1]), (sca, ref[2])):
        assert np.abs(x / r - 1).max() < 1e-13


def test_oracle_processes_match_reference(bgfx):
    _, _, _, comp = BG.background(bgfx, 0)
    ref = bgfx["comp"]
    for c, name in enumerate(BG.NAMES):
        for s in range(2):
            den = np.abs(ref[c, s]).max()
            if den == 0:
                assert not comp[c, s].any(), name
                continue
            assert np.abs(comp[c, s] - ref[c, s]).max() <= 1e-12 * den, (name, s)
            # zero exactly where the reference's routine adds nothing
            assert np.array_equal(comp[c, s] == 0, ref[c, s] == 0), (name, s)


def test_every_process_contributes_somewhere(bgfx):
    assert bgfx["mol_present"].tolist() == [1, 1, 1]
    for c in range(13):
        assert np.abs(bgfx["comp"][c]).max() > 0, BG.NAMES[c]


def test_model_layout(bgfx):
    assert C.sizeof(B.BgContinuum) == 6 * 4 + 8 + 6 * 8
    assert C.sizeof(B.BgRayleighLine) == 3 * 8 + 2 * 4
    m = B.model_from_setup(bgfx)
    meta = bgfx["atoms_meta"]
    assert m.ncont_h == meta[0, 1] and m.ncont_metal == meta[1:, 1].sum()
    assert m.npop == meta[:, 0].sum()
    assert B.model_from_setup(bgfx, lte=False).npop == 2 * meta[:, 0].sum()
    # hydrogen's continua: sigma0 n_eff, upper level the protons
    c0 = m.cont[0]
    assert c0.hydrogenic == 1 and c0.gbf0 == 1.0 and c0.n_j == meta[0, 0] - 1
    # Rayleigh lines only from ground levels, limits the shortest red edge
    for s in range(2):
        red = [m.ray[i].lambda_red for i in range(m.nray) if m.ray[i].scatterer == s]
        assert red and m.ray_limit[s] == min(red)


def test_fudge_factors_in_the_oracle(bgfx):
    """compute1d's fudge factors scale the H-minus, scattering and metal
    terms (background.c:365-455): with all three at 1 nothing changes."""
    fl = np.array([100.0, 30000.0])
    ones = np.ones((3, 2))
    a = BG.background(bgfx, 0)
    b = BG.background(bgfx, 0, fudge=(fl, ones))
    for x, y in zip(a[:3], b[:3]):
        assert np.array_equal(x, y)
