"""NLTE set-up on the device (pyrh_nlte_setup through the C ABI) against the
reference's own set-up state in the NLTE fixtures: LTE populations, the
collision rate matrix and the Doppler widths, from the model atom's text
(pyrh_atom_read) and the atmosphere; and a converged FP64 solve whose
populations, collision rates, wavelength grid, transition ranges and
continuum cross-sections all come from this library (only the background
opacity and the line damping are the reference's) against the reference's
converged populations.

Tolerances: nstar and C within 1e-12 relative (device exp/pow against the
host's), vbroad within 1e-14; the converged populations within 1e-6, the
solver's FP64 parity bound."""
import numpy as np
import pytest

from pyrh_gb300 import _lib as L
from pyrh_gb300 import grid as G
from pyrh_gb300 import nlte

pytestmark = pytest.mark.gpu

CASES = ["nlte_c1", "nlte_c4_50", "nlte_c4_120"]
CA_WEIGHT = 40.08       # the reference's element table (rh/Atoms)


def _setup(fx):
    atom = G.read_atom(str(fx["atom_text"]))
    return atom, nlte.device_setup(atom, CA_WEIGHT, fx["T"], fx["ne"], fx["ntotal"], fx["vturb"])


@pytest.mark.parametrize("name", CASES)
def test_setup_matches_reference(golden, name):
    fx = golden(name)
    _, (nstar, Cm, vb) = _setup(fx)
    assert np.abs(nstar / fx["nstar"] - 1).max() < 1e-12
    ref = fx["C"]
    nz = ref != 0
    assert np.array_equal(Cm != 0, nz)
    assert np.abs(Cm[nz] / ref[nz] - 1).max() < 1e-12
    assert np.abs(vb / fx["vbroad"] - 1).max() < 1e-14


@pytest.mark.parametrize("name", ["nlte_c1", "nlte_c4_120", "nlte_static"])
def test_solve_from_atom_file(golden, name):
    fx = golden(name)
    atom, (nstar, Cm, vb) = _setup(fx)
    g = G.nlte_grid(atom, fx["wave"], float(fx["fmeta"][1]), 5.0, moving=bool(fx["meta"][12]))
    mine = dict(fx)
    for k in ("Gamma1", "J1", "n1", "n_final", "J_final", "I_out"):
        mine.pop(k, None)
    mine["lambda"] = g.lam
    lines = np.array(fx["lines"], np.float64).copy()
    lines[:, 7:9] = g.line_range
    lines[:, 15] = [G.line_polarized(atom, kr) for kr in range(atom.nline)]
    cont = np.array(fx["continua"], np.float64).copy()
    cont[:, 2:4] = g.cont_range
    off = np.concatenate([[0], np.cumsum(cont[:, 3])[:-1]])
    cont[:, 6] = off
    mine["lines"], mine["continua"] = lines, cont
    mine["alpha"] = np.concatenate(g.alpha)
    mine["nstar"], mine["n0"], mine["C"], mine["vbroad"] = nstar, nstar.copy(), Cm, vb
    cfg = nlte.make_config(mine, L.PYRH_FP64)
    dev = nlte.DeviceNlte(nlte.pack([mine], cfg.nrays), cfg)
    assert dev.solve(cfg) == L.PYRH_OK, L.lib().pyrh_last_error()
    assert np.abs(dev.populations()[0] / fx["n_final"] - 1).max() < 1e-6
