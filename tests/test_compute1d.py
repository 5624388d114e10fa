"""Host logic of pyrh_gb300.compute1d that runs before any device work:
keyword.input parsing and defaults, argument checks, the log gf override of
the line constants (kurucz.c:242-251)."""
import numpy as np
import pytest

from pyrh_gb300 import compute1d as C1
from test_compute1d_gpu import keyword_dir, setup_of


def test_keyword_reader(tmp_path):
    (tmp_path / "keyword.input").write_text(
        "# comment\n  ATOMS_FILE = atoms.input\n  stokes_mode = FULL_STOKES  # trailing\n"
        "VMICRO_CHAR=5.0\n\n")
    kw = C1.read_keyword_input(str(tmp_path / "keyword.input"))
    assert kw == {"ATOMS_FILE": "atoms.input", "STOKES_MODE": "FULL_STOKES",
                  "VMICRO_CHAR": "5.0"}


def test_rejects_set_up_changes_and_wrong_grids(golden, tmp_path):
    fx = golden("lte_c0")
    cwd = keyword_dir(tmp_path, fx, "FULL_STOKES")
    with pytest.raises(NotImplementedError):
        C1.compute1d(cwd, 1.0, 0, fx["atm"], fx["wave"], lam_ids=np.array([0], np.int32),
                     lam_values=np.array([0.001]), setup=setup_of(fx))
    with pytest.raises(NotImplementedError):
        C1.compute1d(cwd, 1.0, 0, fx["atm"], fx["wave"], atomic_number=np.array([26], np.int32),
                     atomic_abundance=np.array([7.5]), setup=setup_of(fx))
    with pytest.raises(NotImplementedError):   # fudge factors and the caller's continuum
        C1.compute1d(cwd, 1.0, 0, fx["atm"], fx["wave"], fudge_wave=np.array([400.0, 700.0]),
                     fudge_value=np.ones((3, 2)), setup=setup_of(fx))
    part = setup_of(fx)
    part.height = None
    with pytest.raises(ValueError):        # continuum, heights and protons go together
        C1.compute1d(cwd, 1.0, 0, fx["atm"], fx["wave"], setup=part)
    with pytest.raises(ValueError):        # the set-up was made for other wavelengths
        C1.compute1d(cwd, 1.0, 0, fx["atm"], fx["wave"][:-3], setup=setup_of(fx))
    with pytest.raises(ValueError):
        C1.compute1d(cwd, 1.0, 0, fx["atm"][:8], fx["wave"], setup=setup_of(fx))


def test_loggf_override_reproduces_line_constants(golden):
    """Passing each line's own log gf back recomputes Aji, Bji, Bij as the
    reference's reader does, to rounding."""
    fx = golden("lte_c0")
    su = setup_of(fx)
    base = np.array([-0.72, -1.24])
    lc = C1._line_constants(su, np.array([0, 1]), base)
    assert np.allclose(lc[:, 7:10], fx["line_const"][:, 7:10], rtol=1e-13, atol=0)
    lc2 = C1._line_constants(su, np.array([1]), np.array([-0.24]))
    assert np.allclose(lc2[1, 7] / fx["line_const"][1, 7], 10.0, rtol=1e-12)
    assert np.array_equal(lc2[0], fx["line_const"][0])
