"""r-ccsd(t) on the GPU (hx_ccsd_triples) against the oracle (oracle/triples.py).

The GPU's own converged amplitudes and orbitals are handed to the oracle:
the closed-shell (T) must agree to 1e-10 relative, and for the smallest
molecules the reference's spin-orbital loop (mod_cc.f90:2028-2111) must give
the GPU's reference term (-(T)). A mixed-precision solve must give the same
(T) as the FP64 one.
"""
import numpy as np
import pytest

from helios_gb300 import molecules

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    from helios_gb300 import build
    build.build()
    from helios_gb300 import api as a
    return a


def _gpu(api, mol, precision="fp64"):
    cc = api.CoupledCluster(mol, api.Keywords(bond_alternation=0.1, accuracy=12, precision=precision))
    cc.initCC()
    r = cc.iterate()
    assert r["status"] == 1
    t = cc.triples(0)
    t1, t2 = cc.amplitudes(0)
    s = cc.scf(0)
    cc.finalizeCC()
    return t, t1, t2, s


@pytest.mark.parametrize("mol", [molecules.polyene(6), molecules.ladder(8), molecules.dodecahexaene(),
                                 molecules.polyene(20), molecules.random_molecule(11, 14, 18)],
                         ids=["polyene-6", "ladder-8", "dodecahexaene", "polyene-20", "random-11"])
def test_triples_match_the_oracle(api, mol):
    from oracle import triples
    from oracle.ppp import build_model
    t, t1, t2, s = _gpu(api, mol)
    model = build_model(mol, alternation=0.1)
    o = t1.shape[0]
    want = triples.closed_shell_triples(s["C"], model["G"], np.diag(s["F"]), o, t1, t2)
    assert t["T"] == pytest.approx(want, rel=1e-10)
    assert t["T"] == pytest.approx(t["E4"] + t["E5"], rel=1e-14) and t["T"] < 0
    assert t["reference_term"] == -t["T"]
    if mol.n_sites <= 8:
        e_ref, c1, c2, c3 = triples.spin_triples(s["C"], model["G"], model["core"], o, t1, t2)
        assert t["reference_term"] == pytest.approx(e_ref, rel=1e-10)
        assert t["E4"] == pytest.approx(-c1, rel=1e-10)


def test_mixed_precision_gives_the_same_triples(api):
    mol = molecules.ladder(16)
    t64, *_ = _gpu(api, mol, "fp64")
    tmx, *_ = _gpu(api, mol, "mixed")
    assert tmx["T"] == pytest.approx(t64["T"], rel=1e-8)
