"""Chemical equilibrium on the CPU: the oracle restatement (oracle/chem.py)
against the reference's own ChemicalEquilibrium output (fixture chem, made
by tests/golden/make_golden.py), and the product's molecule-file reader
(pyrh_molecule_read) against the oracle's parse of the same files."""
import ctypes as C

import numpy as np
import pytest

from oracle import chem as OC
from pyrh_gb300 import chem as CH


def _tab(golden):
    lp = golden("ltepops")
    return {"Tpf": lp["Tpf"], "el_meta": lp["el_meta"][0], "el_pf": lp["el_pf"],
            "el_ionpot": lp["el_ionpot"]}


@pytest.mark.parametrize("case", [0, 1, 2])
def test_oracle_matches_reference(golden, case):
    d = golden("chem")
    tab = _tab(golden)
    mols = [OC.read_molecule(str(t), tab["el_meta"][:, 1]) for t in d["molecule_text"]]
    fn0 = {int(e): d["fn0"][case][i] for i, e in enumerate(d["nuclei"]) if d["nuc_model"][i]}
    sel = np.arange(0, 71, 5)
    nm, nh, nn, _ = OC.chem_equil(tab, mols, d["T"][case][sel], d["ne"][case][sel],
                                  d["nHtot"][case][sel], {e: v[sel] for e, v in fn0.items()})
    np.testing.assert_allclose(nm, d["nmol"][case][:, sel], rtol=1e-13, atol=0)
    np.testing.assert_allclose(nh, d["nHmin"][case][sel], rtol=1e-13, atol=0)
    np.testing.assert_allclose(nn, d["ntot_model"][case][:, sel], rtol=1e-13, atol=0)


def test_molecule_reader_matches_oracle_parse(golden):
    d = golden("chem")
    aset = golden("ltepops")["el_meta"][0][:, 1].astype(np.int32)
    for text in d["molecule_text"]:
        m = CH.read_molecule(str(text), aset)
        o = OC.read_molecule(str(text), aset)
        assert m.id.decode() == o["id"] and m.charge == o["charge"] and m.fit == o["fit"]
        assert list(m.pt_index[:m.nelement]) == o["pt_index"]
        assert list(m.pt_count[:m.nelement]) == o["pt_count"] and m.nnuclei == o["nnuclei"]
        assert m.ediss == o["ediss"] and (m.tmin, m.tmax) == (o["tmin"], o["tmax"])
        assert list(m.pf_coef[:m.npf]) == o["pf_coef"]
        assert list(m.eqc_coef[:m.neqc]) == o["eqc_coef"]


def test_molecule_reader_rules(golden):
    aset = golden("ltepops")["el_meta"][0][:, 1].astype(np.int32)
    base = "# a comment\n  XY\n\n  1\n  C, 2O\n  5.0\n  KURUCZ_85\n  1.0E+3  9.0E+3\n  2  1.0  2.0\n  3  4.0  5.0  6.0\n"
    m = CH.read_molecule(base, aset)
    assert m.charge == 1 and m.nelement == 2 and list(m.pt_index[:2]) == [5, 7]
    assert list(m.pt_count[:2]) == [1, 2] and m.nnuclei == 3
    assert list(m.pf_coef[:2]) == [2.0, 1.0] and list(m.eqc_coef[:3]) == [6.0, 5.0, 4.0]
    with pytest.raises(RuntimeError):      # a charged molecule needs a KURUCZ fit
        CH.read_molecule(base.replace("KURUCZ_85", "SAUVAL_TATUM_84"), aset)
    with pytest.raises(RuntimeError):      # charge 2
        CH.read_molecule(base.replace("  1\n", "  2\n", 1), aset)
    with pytest.raises(RuntimeError):      # unknown element
        CH.read_molecule(base.replace("C, 2O", "C, 2QQ"), aset)


def test_structs_match_compiled_header(tmp_path):
    """sizeof and a late member's offset of pyrh_molecule, and sizeof
    pyrh_elem_tables, as a C compiler lays them out from the header."""
    import os
    import shutil
    import subprocess
    from pyrh_gb300 import ltepops as LP
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    src = tmp_path / "layout.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "pyrh_gb300.h"\n'
                   'int main(void) { printf("%zu %zu %zu\\n", sizeof(pyrh_molecule), '
                   'offsetof(pyrh_molecule, eqc_coef), sizeof(pyrh_elem_tables)); return 0; }\n')
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", inc, str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True,
                                          text=True).stdout.split()]
    assert got == [C.sizeof(CH.Molecule), CH.Molecule.eqc_coef.offset, C.sizeof(LP.ElemTables)]
