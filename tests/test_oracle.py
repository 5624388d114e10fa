"""The CPU oracle (oracle/rt_oracle.c) against golden vectors produced by the
compiled reference (tests/golden/make_golden.py).  Stokes errors are
normalised by the continuum intensity I_c = max(I) of each spectrum."""
import numpy as np
import pytest

from conftest import batch_member
from oracle import oracle as O

# lte_mixed: two unpolarizable lines (Armstrong's Voigt, kurucz.c:824);
# lte_static: the same lines in a static atmosphere (Feautrier where only
# unpolarizable lines cover the wavelength, formal.c:96-101); lte_static_v:
# velocities below VMACRO_TRESH, which the static case ignores
# lte_broadening: Unsold van der Waals broadening, isotope and hyperfine
# fractions below one
LTE_CASES = ["lte_c0", "lte_edge", "lte_b0", "lte_mixed", "lte_static", "lte_static_v",
             "lte_broadening"]


def _err(mine, ref):
    return np.abs(mine - ref).max(axis=1) / ref[0].max()


@pytest.mark.parametrize("name", LTE_CASES)
def test_output_grid_matches_reference(golden, name):
    fx = golden(name)
    m = O.output_mask(fx["lam"], fx["lambda_ref"])
    # rhf1d returns the sorted, de-duplicated grid without LAMBDA_REF
    assert np.array_equal(fx["lam"][m], fx["lam_out"])
    assert np.all(np.diff(fx["lam"]) > 0)
    assert np.array_equal(np.unique(np.append(fx["wave"], fx["lambda_ref"])), fx["lam"])


@pytest.mark.parametrize("name", LTE_CASES)
def test_oracle_vs_portable_reference(golden, name):
    """Same 4x4 float inverse as the reference's portable build: 1e-6 I_c."""
    fx = golden(name)
    m = O.output_mask(fx["lam"], fx["lambda_ref"])
    out = O.lte_synth(fx, md_float=True)[:, m]
    assert _err(out, fx["stokes_ref_portable"]).max() < 1e-6


@pytest.mark.parametrize("name", LTE_CASES)
@pytest.mark.parametrize("md_float", [True, False])
def test_oracle_vs_sse_reference(golden, name, md_float):
    """The x86 reference inverts with an SSE reciprocal estimate
    (rh/bezier_aux.c:216-218), 3.5e-6 I_c away from an exact inverse."""
    fx = golden(name)
    m = O.output_mask(fx["lam"], fx["lambda_ref"])
    out = O.lte_synth(fx, md_float=md_float)[:, m]
    assert _err(out, fx["stokes_ref"]).max() < 1e-5


@pytest.mark.parametrize("name", LTE_CASES)
def test_oracle_opacity_matches_background_record(golden, name):
    fx = golden(name)
    worst = 0.0
    for j, la in enumerate(fx["opac_idx"]):
        for k in range(len(fx["T"])):
            flags, chi, eta, chip = O.lte_opacity(fx, k, fx["lam"][la])
            tot_c = fx["tot_chi"][j][:, k]
            tot_e = fx["tot_eta"][j][:, k]
            mine_c = np.array([fx["chi_c"][la, k] + chi[0], chi[1], chi[2], chi[3]])
            mine_e = np.array([fx["eta_c"][la, k] + eta[0], eta[1], eta[2], eta[3]])
            worst = max(worst, (np.abs(mine_c - tot_c) / abs(tot_c[0])).max(),
                        (np.abs(mine_e - tot_e) / abs(tot_e[0])).max())
            assert flags == (fx["tot_flags"][la][0] | (fx["tot_flags"][la][1] << 1))
    assert worst < 1e-12


def test_oracle_no_stokes_vs_reference(golden):
    """STOKES_MODE = NO_STOKES: pyrh keeps atmos.Stokes = TRUE
    (pyrh_compute1dray.c:258), so the lines stay polarizable and their
    Zeeman-summed Stokes I profile goes into the scalar Bezier3 solver
    (formal.c:94-95); no 4x4 inverse is involved, and the oracle reproduces
    the reference to rounding."""
    fx = golden("lte_nostokes")
    m = O.output_mask(fx["lam"], fx["lambda_ref"])
    out = O.lte_synth(fx, no_stokes=True)[:, m]
    assert _err(out, fx["stokes_ref"]).max() < 1e-12
    assert np.all(fx["stokes_ref"][1:] == 0.0)


def test_unpolarizable_lines_use_armstrong(golden):
    fx = golden("lte_mixed")
    pol = fx["line_const"][:, 18]
    assert list(pol) == [0, 1, 0, 1] and list(fx["zeeman_n"][pol == 0]) == [0, 0]
    # near 629.60 nm only the unpolarizable line is in its window: no Q, U, V
    m = O.output_mask(fx["lam"], fx["lambda_ref"])
    near = np.abs(fx["lam_out"] - 629.60) < 0.06
    assert np.all(fx["stokes_ref"][1:, near] == 0.0)
    assert fx["stokes_ref"][0, near].min() < 0.9 * fx["stokes_ref"][0, near].max()


def test_oracle_batch_fixture(golden):
    b = golden("lte_batch")
    for i in range(b["T"].shape[0]):
        fx = batch_member(b, i)
        m = O.output_mask(fx["lam"], fx["lambda_ref"])
        out = O.lte_synth(fx)[:, m]
        assert _err(out, fx["stokes_ref_portable"]).max() < 1e-6
        assert _err(out, fx["stokes_ref"]).max() < 1e-5


def test_oracle_threaded_batch_equals_serial(golden):
    b = golden("lte_batch")
    out = O.lte_synth_batch(b, nthreads=4)
    for i in range(b["T"].shape[0]):
        assert np.array_equal(out[i], O.lte_synth(batch_member(b, i)))


def test_far_wavelengths_use_feautrier(golden):
    """lte_edge holds wavelengths outside every line window: the reference
    solves those with Feautrier (formal.c:285-310) and returns Q=U=V=0."""
    fx = golden("lte_edge")
    m = O.output_mask(fx["lam"], fx["lambda_ref"])
    far = fx["tot_flags"][m][:, 0] == 0
    assert far.sum() == 4
    assert np.all(fx["stokes_ref"][1:, far] == 0.0)
    out = O.lte_synth(fx)[:, m]
    assert _err(out[:, far], fx["stokes_ref_portable"][:, far]).max() < 1e-6


def test_humlicek_regions_continuous():
    """W4 is piecewise; values on both sides of each region boundary agree
    to the method's ~1e-4 accuracy (Humlicek 1982)."""
    for a in (1e-3, 0.05, 0.5, 2.0):
        for s_edge in (5.5, 15.0):
            v = s_edge - a
            h1, f1 = O.humlicek(a, v - 1e-9)
            h2, f2 = O.humlicek(a, v + 1e-9)
            assert abs(h1 - h2) <= 2e-4 * max(abs(h1), 1e-3)
    h, f = O.humlicek(1e-4, 0.0)
    assert abs(h - 1.0) < 1e-3
