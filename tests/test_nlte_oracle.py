"""The NLTE CPU oracle (oracle/nlte_oracle.c) against the compiled
reference's golden vectors: profiles, the rate matrix after one formal pass,
one statistical-equilibrium solve, the converged populations at the same
convergence criterion, and the emergent intensity."""
import numpy as np
import pytest

from oracle import oracle as O

CASES = ["nlte_c1", "nlte_c4_50", "nlte_c4_120"]
# nlte_static: the C1 atmosphere without velocities below VMACRO_TRESH, so
# every wavelength takes the Feautrier solver
PINNED = CASES + ["nlte_static"]


@pytest.mark.parametrize("name", PINNED)
def test_profiles(golden, name):
    fx = golden(name)
    phis, wphi = O.nlte_profiles(fx)
    assert np.abs(wphi / fx["wphi"] - 1).max() < 1e-12
    for kr, ph in enumerate(phis):
        for s, la in enumerate(fx["phi_sample_la"][kr]):
            ref = fx["phi_sample"][kr, s]
            assert np.abs(ph[la] - ref).max() <= 1e-10 * np.abs(ref).max()   # GH nodes: 10 vs 17 digits


@pytest.mark.parametrize("name", PINNED)
def test_first_iteration(golden, name):
    fx = golden(name)
    G, J, n1 = O.nlte_first_iteration(fx)
    g = fx["Gamma1"]
    assert np.abs(G - g).max() <= 1e-12 * np.abs(g).max()
    assert np.abs(J - fx["J1"]).max() <= 1e-10 * np.abs(fx["J1"]).max()
    assert np.abs(n1 / fx["n1"] - 1).max() < 1e-7


@pytest.mark.parametrize("name", PINNED)
def test_converged_populations_and_emergent(golden, name):
    fx = golden(name)
    n, J, it, dp, acc = O.nlte_solve(fx)
    assert dp[-1] < fx["fmeta"][0] <= dp[-2]
    assert acc.sum() >= 1                       # Ng acceleration was exercised
    assert np.abs(n / fx["n_final"] - 1).max() < 1e-6
    Iem = O.nlte_emergent(fx, n, J)
    m = O.output_mask(fx["lambda"], fx["fmeta"][1])
    assert np.array_equal(fx["lambda"][m], fx["lam_out"])
    assert np.abs(Iem[m] / fx["I_out"] - 1).max() < 1e-6


@pytest.mark.parametrize("name", PINNED)
def test_radiative_rates(golden, name):
    """R_ij and R_ji of every transition (addtoRates) after the first
    formal pass and after the last one of the converged run."""
    fx = golden(name)
    R1 = O.nlte_first_iteration(fx, rates=True)[3]
    for kind, key in (("lines", "R1_line"), ("continua", "R1_cont")):
        assert np.abs(R1[kind] / fx[key] - 1).max() < 1e-12, kind
    R = O.nlte_solve(fx, rates=True)[5]
    for kind, key in (("lines", "R_final_line"), ("continua", "R_final_cont")):
        assert np.abs(R[kind] / fx[key] - 1).max() < 1e-7, kind


def test_armstrong_voigt_limits():
    # H(0, v) = exp(-v^2); Lorentz wings H ~ a / (sqrt(pi) v^2)
    for v in (0.0, 0.5, 1.7, 3.9):
        assert abs(O.voigt_armstrong(0.0, v) - np.exp(-v * v)) < 1e-12
    a, v = 0.01, 40.0
    assert abs(O.voigt_armstrong(a, v) / (a / (np.sqrt(np.pi) * v * v)) - 1) < 1e-3


# ------------------------------------------- batched uneven NLTE workload --

@pytest.mark.parametrize("name", CASES)
def test_regrid_at_own_shape_keeps_the_reference_solution(golden, name):
    """The workload's depth and wavelength re-gridding at the set-up's own
    shape changes nothing: the oracle still converges to the reference's
    populations after the reference's iteration count."""
    from pyrh_gb300 import workload as W
    fx = golden(name)
    same = W.nlte_regrid_lambda(W.nlte_regrid_depth(fx, len(fx["T"])), len(fx["lambda"]))
    n, _, it, _, _ = O.nlte_solve(same)
    assert np.abs(n / fx["n_final"] - 1).max() < 1e-8
    assert it == O.nlte_solve(fx)[2]


def test_uneven_batch_shapes_and_convergence(golden):
    """Atmospheres of the batched uneven workload have 50..150 depths and
    700..1100 wavelengths, consistent transition ranges, and converge in the
    oracle at the set-ups' convergence limit."""
    from pyrh_gb300 import workload as W
    bases = [golden(n) for n in CASES]
    atms = W.nlte_batch(bases, 12, seed=7)
    for a in atms:
        nd, ns = len(a["T"]), len(a["lambda"])
        assert 50 <= nd <= 150 and 700 <= ns <= 1100
        assert np.all(np.diff(a["lambda"]) > 0)
        for r in list(a["lines"]) + list(a["continua"]):
            nb, nl = (int(r[7]), int(r[8])) if len(r) == 16 else (int(r[2]), int(r[3]))
            assert nl >= 3 and 0 <= nb and nb + nl <= ns
        assert a["background"].shape == (3, ns, nd) and a["C"].shape[1] == nd
        assert np.all(a["nstar"] > 0) and np.all(np.isfinite(a["C"]))
    for a in atms[:3]:
        n, _, it, dp, _ = O.nlte_solve(a)
        assert np.all(np.isfinite(n)) and dp[-1] < float(a["fmeta"][0])
