"""The per-depth set-up of a synthesis from the atmosphere alone, on the
GPU through the C ABI (pyrh_equilibria, pyrh_background, pyrh_convert_scales):
against the reference's own set-up of the LTE runs (continuum on the whole
grid, protons, heights from tau500: fixtures lte_c0, lte_edge, lte_static,
lte_batch), against pyrh.get_scales (fixture scales: three depth scales,
two reference wavelengths, abundance overrides), and compute1d with that
set-up against the reference's spectra."""
import numpy as np
import pytest

from conftest import batch_member, passive_model
from pyrh_gb300 import _lib as L
from pyrh_gb300 import compute1d as C1
from pyrh_gb300 import equilibria as EQ
from test_compute1d_gpu import keyword_dir, setup_of

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def model(golden):
    return passive_model(golden)


def _cases(golden):
    out = [golden(n) for n in ("lte_c0", "lte_edge", "lte_static")]
    b = golden("lte_batch")
    out += [batch_member(b, i) for i in range(b["T"].shape[0])]
    return out


def test_continuum_protons_and_heights_match_reference_setup(golden, model):
    for fx in _cases(golden):
        chi, eta, npr = EQ.continuum(model, fx["lam"], fx["T"], fx["ne"], fx["nHtot"])
        np.testing.assert_allclose(chi, fx["chi_c"], rtol=1e-12, atol=0)
        np.testing.assert_allclose(eta, fx["eta_c"], rtol=1e-12, atol=0)
        np.testing.assert_allclose(npr, fx["np"], rtol=1e-12, atol=0)
        iref = int(np.searchsorted(fx["lam"], float(fx["lambda_ref"])))
        tau, cm, h = EQ.convert_scales(model, 0, fx["atm"][0], fx["T"], fx["ne"], fx["nHtot"],
                                       chi[iref])
        assert L.lib().pyrh_last_launch_count() == 1
        np.testing.assert_allclose(h[0], fx["height"], rtol=1e-12, atol=1e-6)


def test_equilibria_batch_equals_points_alone(golden, model):
    """Every point is independent: a batch of two atmospheres' points gives
    each atmosphere's values bit for bit."""
    a, b = golden("lte_c0"), golden("lte_edge")
    T = np.concatenate([a["T"], b["T"][::-1]])
    ne = np.concatenate([a["ne"], b["ne"][::-1]])
    nH = np.concatenate([a["nHtot"], b["nHtot"][::-1]])
    pops, nmol, nHmin = EQ.equilibria(model, T, ne, nH)
    one = EQ.equilibria(model, a["T"], a["ne"], a["nHtot"])
    for x, y in zip((pops, nmol, nHmin), one):
        assert np.array_equal(x.cpu().numpy()[..., :71], y.cpu().numpy())


@pytest.mark.parametrize("case", range(5))
def test_get_scales_matches_reference(golden, model, case):
    d = golden("scales")
    m = passive_model(golden, ab_overrides=True) if case == int(d["ab_case"]) else model
    sc = int(d["atm_scale"][case])
    tau, h, cm = EQ.get_scales(None, sc, d["scale"][case], d["atm"], float(d["lam_ref"][case]),
                               model=m)
    got = {"tau": tau, "cmass": cm, "height": h}
    for key in [("cmass", "height"), ("tau", "height"), ("tau", "cmass")][sc]:
        np.testing.assert_allclose(got[key], d[key][case], rtol=1e-12, atol=1e-6, err_msg=key)


@pytest.mark.parametrize("name", ["lte_c0", "lte_edge", "lte_static"])
def test_compute1d_with_the_setup_from_the_atmosphere(golden, tmp_path, model, name):
    """compute1d with neither continuum, heights nor protons given forms
    them on the device: the spectra match the reference's compute1d and the
    run with the reference's own set-up."""
    fx = golden(name)
    cwd = keyword_dir(tmp_path, fx, "FULL_STOKES")
    atm = np.ascontiguousarray(fx["atm"])
    base = C1.compute1d(cwd, float(fx["mu"]), 0, atm, fx["wave"], setup=setup_of(fx))
    su = setup_of(fx)
    su.chi_c = su.eta_c = su.height = su.np = None
    su.line_pops, su.atoms_model = None, model
    got = C1.compute1d(cwd, float(fx["mu"]), 0, atm, fx["wave"], setup=su)
    ic = base[0].max()
    for s in range(4):
        assert np.abs(got[s] - base[s]).max() < 1e-9 * ic
        assert np.abs(got[s] - fx["stokes_ref_portable"][s]).max() < 1e-5 * ic


@pytest.mark.parametrize("case", [0, 1, 2])
def test_equilibria_match_reference_chemistry(golden, model, case):
    """pyrh_equilibria from T, n_e and nHtot alone -- the passive atoms' LTE
    populations and their neutral fractions, then the chemistry (a warp per
    point) -- against the reference's SetLTEQuantities + ChemicalEquilibrium
    (fixture chem, down to 2900 K)."""
    d = golden("chem")
    pops, nmol, nHmin = EQ.equilibria(model, d["T"][case], d["ne"][case], d["nHtot"][case])
    ref = d["nmol"][case]
    np.testing.assert_allclose(nmol.cpu().numpy(), ref, rtol=1e-12, atol=0)
    np.testing.assert_allclose(nHmin.cpu().numpy(), d["nHmin"][case], rtol=1e-12, atol=0)
    # the model atoms of the nuclei keep their atomic share (rows of H, C, N, O)
    p = pops.cpu().numpy()
    for i, e in enumerate(d["nuclei"]):
        m = [model.atoms.elem[q] for q in range(model.atoms.natom)].index(int(e))
        lo, hi = model.atoms.lev_off[m], model.atoms.lev_off[m + 1]
        np.testing.assert_allclose(p[lo:hi].sum(axis=0), d["ntot_model"][case][i], rtol=1e-12,
                                   atol=0)


@pytest.mark.parametrize("atm_scale", [1, 2])
def test_compute1d_on_column_mass_and_height_scales(golden, tmp_path, model, atm_scale):
    """compute1d of C0 given on the column-mass or the height scale, its
    heights from the device's convertScales: the reference's spectra of the
    same calls (fixture lte_scales)."""
    fx, d = golden("lte_c0"), golden("lte_scales")
    cwd = keyword_dir(tmp_path, fx, "FULL_STOKES")
    su = setup_of(fx)
    su.chi_c = su.eta_c = su.height = su.np = None
    su.line_pops, su.atoms_model = None, model
    atm = np.ascontiguousarray(d[f"atm_{atm_scale}"])
    got = C1.compute1d(cwd, 1.0, atm_scale, atm, d["wave"], setup=su)
    ref = d[f"stokes_ref_portable_{atm_scale}"]
    ic = ref[0].max()
    assert np.array_equal(got[4], d["lam_out"])
    for s in range(4):
        assert np.abs(got[s] - ref[s]).max() < 1e-5 * ic
