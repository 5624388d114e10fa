"""Chemical equilibrium on the GPU (pyrh_chem_equil through the C ABI)
against the reference's own ChemicalEquilibrium output (fixture chem): the
molecule densities, the H- density and the nuclei's atomic densities, on
three atmospheres down to 2900 K (37 % of hydrogen in H2), with the neutral
fractions of the model atoms the reference started from; and, without atom
models, against the oracle with the element tables' partition functions."""
import numpy as np
import pytest

from oracle import chem as OC
from pyrh_gb300 import _lib as L
from pyrh_gb300 import chem as CH
from pyrh_gb300 import ltepops as LP

pytestmark = pytest.mark.gpu


def _tables(golden):
    lp = golden("ltepops")
    meta = lp["el_meta"][0]
    ns = meta[:, 0].astype(np.int32)
    off = np.concatenate([[0], np.cumsum(ns)[:-1]]).astype(np.int32)
    return LP.ElementTables(lp["Tpf"], meta[:, 2].copy(), meta[:, 1].astype(np.int32), ns, off,
                            lp["el_pf"], lp["el_ionpot"])


@pytest.mark.parametrize("case", [0, 1, 2])
def test_chem_matches_reference(golden, case):
    d = golden("chem")
    tab = _tables(golden)
    dev = LP.DeviceTables(tab)
    mols = [CH.read_molecule(str(t), tab.abundance_set) for t in d["molecule_text"]]
    assert CH.nuclei_of(mols) == list(d["nuclei"])
    fn0 = {int(e): d["fn0"][case][i] for i, e in enumerate(d["nuclei"]) if d["nuc_model"][i]}
    nm, nh, nn, it = CH.chem_equil(dev, mols, d["T"][case], d["ne"][case], d["nHtot"][case], fn0)
    assert L.lib().pyrh_last_launch_count() == 1
    np.testing.assert_allclose(nm.cpu().numpy(), d["nmol"][case], rtol=1e-12, atol=0)
    np.testing.assert_allclose(nh.cpu().numpy(), d["nHmin"][case], rtol=1e-12, atol=0)
    np.testing.assert_allclose(nn.cpu().numpy(), d["ntot_model"][case], rtol=1e-12, atol=0)
    it = it.cpu().numpy()
    assert np.all((it >= 1) | (it == -1))


def test_chem_without_models_matches_oracle(golden):
    """Every nucleus' neutral fraction from the partition functions
    (getfjk), batched over the three atmospheres in one launch."""
    d = golden("chem")
    tab = _tables(golden)
    lp = golden("ltepops")
    otab = {"Tpf": lp["Tpf"], "el_meta": lp["el_meta"][0], "el_pf": lp["el_pf"],
            "el_ionpot": lp["el_ionpot"]}
    mols = [CH.read_molecule(str(t), tab.abundance_set) for t in d["molecule_text"]]
    omols = [OC.read_molecule(str(t), tab.abundance_set) for t in d["molecule_text"]]
    sel = np.arange(0, 71, 7)
    T = np.concatenate([d["T"][c][sel] for c in range(3)])
    ne = np.concatenate([d["ne"][c][sel] for c in range(3)])
    nH = np.concatenate([d["nHtot"][c][sel] for c in range(3)])
    nm, nh, nn, _ = CH.chem_equil(LP.DeviceTables(tab), mols, T, ne, nH)
    om, oh, on, _ = OC.chem_equil(otab, omols, T, ne, nH)
    np.testing.assert_allclose(nm.cpu().numpy(), om, rtol=1e-12, atol=0)
    np.testing.assert_allclose(nh.cpu().numpy(), oh, rtol=1e-12, atol=0)
    np.testing.assert_allclose(nn.cpu().numpy(), on, rtol=1e-12, atol=0)


def test_chem_rejects_bad_input(golden):
    d = golden("chem")
    tab = _tables(golden)
    dev = LP.DeviceTables(tab)
    mols = [CH.read_molecule(str(t), tab.abundance_set) for t in d["molecule_text"]]
    with pytest.raises(RuntimeError):          # H2 must come first
        CH.chem_equil(dev, mols[1:], d["T"][0], d["ne"][0], d["nHtot"][0])
    nm, nh, nn, it = CH.chem_equil(dev, mols, d["T"][0][:0], d["ne"][0][:0], d["nHtot"][0][:0])
    assert nm.numel() == 0
