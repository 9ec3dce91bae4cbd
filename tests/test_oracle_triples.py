"""The (T) oracle (oracle/triples.py), no GPU: the reference's spin-orbital
loop (mod_cc.f90:2028-2111), the published spin-orbital (T) and the
closed-shell form the GPU evaluates, on converged oracle amplitudes."""
import numpy as np
import pytest

from helios_gb300 import molecules
from oracle import ccsd_fact, triples
from oracle.ppp import build_model
from oracle.rhf import mo_fock, rhf


def _solved(mol):
    model = build_model(mol, alternation=0.1)
    scf = rhf(model)
    F, eref = mo_fock(model, scf["V"], scf["D"])
    o = model["nel"] // 2
    out = ccsd_fact.ccsd(F, scf["V"], model["G"], eref, o, eps=1e-12)
    return model, scf, F, eref, o, out


@pytest.mark.parametrize("mol", [molecules.polyene(6), molecules.ladder(8), molecules.random_molecule(5, 8, 10)],
                         ids=["polyene-6", "ladder-8", "random-5"])
def test_three_forms_of_the_triples_agree(mol):
    model, scf, F, eref, o, out = _solved(mol)
    C, G, h = scf["V"], model["G"], model["core"]
    t1, t2 = out["t1"], out["t2"]
    # the spin-orbital amplitudes reproduce the closed-shell CCSD energy
    from oracle.spin_ccsd import spin_integrals
    f, g, no, ns = spin_integrals(C, G, h, o)
    t1s, t2s = triples.spin_amplitudes(t1, t2)
    Oo, Vv = slice(0, no), slice(no, ns)
    es = (np.einsum("ia,ia->", f[Oo, Vv], t1s) + 0.25 * np.einsum("ijab,ijab->", g[Oo, Oo, Vv, Vv], t2s)
          + 0.5 * np.einsum("ijab,ia,jb->", g[Oo, Oo, Vv, Vv], t1s, t1s))
    assert es == pytest.approx(out["energy"][0] - eref, abs=1e-12)
    e_tb, e4, e5 = triples.textbook_triples(C, G, h, o, t1, t2)
    e_cs = triples.closed_shell_triples(C, G, np.diag(F), o, t1, t2)
    e_ref, c1, c2, c3 = triples.spin_triples(C, G, h, o, t1, t2)
    assert e_cs == pytest.approx(e_tb, rel=1e-11, abs=1e-15)
    assert e_tb < 0 < e_ref
    assert c1 == pytest.approx(-e4, rel=1e-11) and c2 == pytest.approx(-e5, rel=1e-9, abs=1e-15)
    assert abs(c3) < 1e-13                                         # canonical RHF: F_kc = 0
    assert e_ref == pytest.approx(-e_cs, rel=1e-11)
