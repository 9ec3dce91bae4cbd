"""Host logic of the LR-CCSD driver (helios_gb300.lrccsd), no GPU.

The driver's spin-adapted algebra is checked against the spin-orbital sums
of the reference, and the whole driver runs on a CPU stand-in for the engine
(tests/fake_engine.py, built on the oracle): its sigma must equal the
Jacobian of the closed-shell residual, and every state it returns must be an
eigenpair of the reference's own spin-orbital sigma equations with the r0 and
excitation level of energyLR; the Davidson solver must find the lowest roots.
"""
import numpy as np
import pytest

from fake_engine import FakeCoupledCluster
from helios_gb300 import api, lrccsd, molecules
from oracle import ccsd_fact
from oracle import lrccsd as olr
from oracle.ppp import build_model, gamma_matrix
from oracle.rhf import mo_fock, rhf
from oracle.triples import spin_amplitudes


def _random_singlet(rng, o, v):
    r1 = rng.normal(size=(o, v))
    r2 = rng.normal(size=(o, o, v, v))
    return r1, 0.5 * (r2 + r2.transpose(1, 0, 3, 2))


def test_spin_adapted_sums_are_the_spin_orbital_sums():
    rng = np.random.default_rng(11)
    o, v = 3, 4
    x, y = _random_singlet(rng, o, v), _random_singlet(rng, o, v)
    xs, ys = spin_amplitudes(*x), spin_amplitudes(*y)
    no, nv = 2 * o, 2 * v
    up = (np.arange(no)[:, None] < np.arange(no)[None, :])[:, :, None, None] & \
         (np.arange(nv)[:, None] < np.arange(nv)[None, :])[None, None, :, :]
    unique = float((xs[0] * ys[0]).sum()) + float((xs[1][up] * ys[1][up]).sum())
    full = float((xs[0] * ys[0]).sum()) + float((xs[1] * ys[1]).sum())
    assert lrccsd.inner(x, y) == pytest.approx(unique, rel=1e-13)
    assert lrccsd.inner_full(x, y) == pytest.approx(full, rel=1e-13)
    assert lrccsd.max_abs(x) == (float(np.abs(xs[0]).max()), float(np.abs(xs[1]).max()))


@pytest.mark.parametrize("kind", ["ohno-klopman", "mataga-nishimoto", "hubbard"])
def test_coulomb_matrix_is_the_models(kind):
    for mol in (molecules.polyene(10), molecules.ladder(12), molecules.random_molecule(4, 8, 20)):
        G = lrccsd.coulomb_matrix(mol, kind)
        assert np.abs(G - gamma_matrix(mol.coords, np.asarray(mol.gamma), kind)).max() < 1e-13


def _problem(mol):
    model = build_model(mol, alternation=0.1)
    scf = rhf(model)
    F, eref = mo_fock(model, scf["V"], scf["D"])
    o = model["nel"] // 2
    out = ccsd_fact.ccsd(F, scf["V"], model["G"], eref, o, eps=1e-12)
    return model, scf, F, o, out


def test_guess_vectors_are_the_oracles():
    model, scf, F, o, _ = _problem(molecules.polyene(8))
    I = lrccsd.MOIntegrals(scf["V"], model["G"], o)
    got, w = lrccsd.guess_vectors(F, I, 3)
    want, w_ref = olr.cis_guess(F, scf["V"], model["G"], o, 3)
    assert np.allclose(w, w_ref, rtol=1e-12)
    for g, r in zip(got, want):
        assert [(i, a) for i, a, _ in g] == [(i, a) for i, a, _ in r]
        assert np.allclose([c for *_, c in g], [c for *_, c in r], atol=1e-12)
    sel, w_rpa = lrccsd.guess_vectors(F, I, 2, kind="rpa")
    assert len(sel[0]) >= 1 and w_rpa[0] <= w[0] + 1e-12


def test_fake_engine_sigma_is_the_closed_shell_jacobian():
    mol = molecules.polyene(6)
    model, scf, F, o, out = _problem(mol)
    kw = api.Keywords(bond_alternation=0.1, accuracy=12)
    sig = lrccsd.DeviceSigma(mol, kw, out["t1"], out["t2"], scf["V"], nvec=2, engine=FakeCoupledCluster)
    v = F.shape[0] - o
    J = olr.closed_shell_jacobian(F, scf["V"], model["G"], o, out["t1"], out["t2"])
    rng = np.random.default_rng(5)
    vecs = [_random_singlet(rng, o, v) for _ in range(2)]
    for (s1, s2), r in zip(sig(vecs), vecs):
        want1, want2 = olr.closed_shell_unpack(J @ olr.closed_shell_pack(*r), o, v)
        assert np.abs(s1 - want1).max() < 1e-10 and np.abs(s2 - want2).max() < 1e-10
        # the Davidson basis stores rows of flattened vectors: the sigma hands back row-major arrays
        assert s1.flags.c_contiguous and s2.flags.c_contiguous


def test_sigma_in_flipped_orbital_signs():
    """Amplitudes and vectors given in orbitals some of whose signs differ from the
    evaluator's own SCF: the sigma carries them across and is the Jacobian in the caller's
    signs (S J S for the diagonal +-1 sign change S)."""
    mol = molecules.polyene(6)
    model, scf, F, o, out = _problem(mol)
    kw = api.Keywords(bond_alternation=0.1, accuracy=12)
    n = F.shape[0]
    v = n - o
    sg = np.ones(n)
    sg[[0, 2, o + 1]] = -1.0
    so, sv = sg[:o], sg[o:]
    S1 = so[:, None] * sv[None, :]
    S2 = so[:, None, None, None] * so[None, :, None, None] * sv[None, None, :, None] * sv[None, None, None, :]
    sig = lrccsd.DeviceSigma(mol, kw, out["t1"] * S1, out["t2"] * S2, scf["V"] * sg[None, :], nvec=2,
                             engine=FakeCoupledCluster)
    assert any(sig._sign_tensors[k] is not None for k in sig.signs)
    J = olr.closed_shell_jacobian(F, scf["V"], model["G"], o, out["t1"], out["t2"])
    rng = np.random.default_rng(8)
    vecs = [_random_singlet(rng, o, v)]                           # one vector: the second copy set idles
    for (s1, s2), (r1, r2) in zip(sig(vecs), vecs):
        want1, want2 = olr.closed_shell_unpack(J @ olr.closed_shell_pack(r1 * S1, r2 * S2), o, v)
        assert np.abs(s1 - want1 * S1).max() < 1e-10 and np.abs(s2 - want2 * S2).max() < 1e-10


def test_stacked_basis_is_the_inner_metric():
    """The Davidson basis keeps V and W as rows of stacked arrays; its projections, projected
    matrix and Gram-Schmidt must be the ones the pairwise ``inner`` gives."""
    o, v = 3, 4
    rng = np.random.default_rng(11)
    B = lrccsd._Basis(o, v, 6)
    kept = []
    for _ in range(4):
        y = B.orthonormal(_random_singlet(rng, o, v))
        assert y is not None
        kept.append(y)
        B.set_sigma(B.add(y), _random_singlet(rng, o, v))
    G = np.array([[lrccsd.inner(a, b) for b in kept] for a in kept])
    assert np.abs(G - np.eye(4)).max() < 1e-12
    x = _random_singlet(rng, o, v)
    assert np.allclose(B.coeffs(x), [lrccsd.inner(y, x) for y in kept], rtol=0, atol=1e-12)
    W = [(B.W1[j].reshape(o, v), B.W2[j].reshape(o, o, v, v)) for j in range(4)]
    want = np.array([[lrccsd.inner(kept[i], W[j]) for j in range(4)] for i in range(4)])
    assert np.allclose(B.projected(slice(0, 4), slice(0, 4)), want, rtol=0, atol=1e-12)
    assert np.allclose(B.projected([1, 3], [0, 2]), want[np.ix_([1, 3], [0, 2])], rtol=0, atol=1e-12)
    assert B.orthonormal(kept[2]) is None
    assert B.orthonormal((np.zeros((o, v)), np.zeros((o, o, v, v)))) is None


def _spectrum_and_problem(mol):
    model, scf, F, o, out = _problem(mol)
    J = olr.closed_shell_jacobian(F, scf["V"], model["G"], o, out["t1"], out["t2"])
    P = olr.SpinProblem(scf["V"], model["G"], model["core"], o, out["t1"], out["t2"])
    return np.sort(np.linalg.eigvals(J).real), P, olr.intermediates(P)


MOLS = {"butadiene": molecules.polyene(4), "hexatriene": molecules.polyene(6), "rnd7": molecules.random_molecule(7, 6, 8)}


@pytest.mark.parametrize("solver", ["reference", "davidson"])
@pytest.mark.parametrize("name", list(MOLS))
def test_driver_on_the_fake_engine_finds_eigenpairs(name, solver):
    # the reference's iteration settles on rounding-dependent states, each an eigenpair;
    # the Davidson solver finds the lowest roots
    mol = MOLS[name]
    spec, P, X = _spectrum_and_problem(mol)
    kw = api.Keywords(bond_alternation=0.1, accuracy=12)
    lr = lrccsd.LRKeywords(excited_states_number=3, accuracy=8)
    got = lrccsd.linear_response(mol, kw, lr, engine=FakeCoupledCluster, solver=solver)
    assert got["ccsd_status"] == 1 and list(got["status"]) == [1, 1, 1]
    assert np.all(np.diff(got["omega"]) >= 0)
    for k in range(3):
        w = got["omega"][k]
        assert np.min(np.abs(spec - w)) < 1e-8
        r1s, r2s = spin_amplitudes(got["r1"][k], got["r2"][k])
        d1, d2 = olr.sigma(P, X, r1s, r2s)                        # the reference's own sigma equations
        assert max(np.abs(d1 - w * r1s).max(), np.abs(d2 - w * r2s).max()) < 1e-7 * 2 ** k
        _, r0, ael = olr.lr_energy(P, X, r1s, r2s, w)               # energyLR on the spin-orbital vector
        assert got["r0"][k] == pytest.approx(r0, abs=1e-9) and got["ael"][k] == pytest.approx(ael, rel=1e-12)
    if solver == "davidson":
        assert np.abs(got["omega"] - spec[:3]).max() < 1e-8
    assert np.allclose(got["E_total"], got["energy"] + got["omega"])


def test_orthogonalization_runs_the_states_in_turn():
    mol = molecules.polyene(4)
    model, scf, F, o, out = _problem(mol)
    kw = api.Keywords(bond_alternation=0.1, accuracy=12)
    lr = lrccsd.LRKeywords(excited_states_number=2, accuracy=8, orthogonalization=True)
    got = lrccsd.linear_response(mol, kw, lr, engine=FakeCoupledCluster)
    spec, _, _ = _spectrum_and_problem(mol)
    assert list(got["status"]) == [1, 1]
    assert all(np.min(np.abs(spec - w)) < 1e-8 for w in got["omega"])
    assert got["omega"][1] - got["omega"][0] > 1e-3                       # two different states


def test_stored_seeds_restart_at_the_solution():
    mol = molecules.polyene(4)
    kw = api.Keywords(bond_alternation=0.1, accuracy=12)
    lr = lrccsd.LRKeywords(excited_states_number=2, accuracy=8)
    first = lrccsd.linear_response(mol, kw, lr, engine=FakeCoupledCluster)
    again = lrccsd.linear_response(mol, kw, lr, seeds=lrccsd.stored_seeds(first, lr), engine=FakeCoupledCluster)
    assert np.abs(again["omega"] - first["omega"]).max() < 1e-8
    assert np.all(again["iterations"] < first["iterations"])


def test_triplets_and_bad_state_counts_are_refused():
    mol = molecules.polyene(4)
    with pytest.raises(NotImplementedError):
        lrccsd.linear_response(mol, lr=lrccsd.LRKeywords(spin=1), engine=FakeCoupledCluster)
    with pytest.raises(ValueError):
        lrccsd.linear_response(mol, lr=lrccsd.LRKeywords(excited_states_number=0), engine=FakeCoupledCluster)


def test_excited_state_polarizability_on_the_fake_engine(tmp_path):
    from helios_gb300 import properties
    from oracle.polariz import alpha
    mol, step = molecules.polyene(4), 0.05
    kw = api.Keywords(bond_alternation=0.1, accuracy=12)
    lr = lrccsd.LRKeywords(excited_states_number=2, accuracy=9)
    path = str(tmp_path / "states.hrv")
    res, report = properties.polarizability_job(mol, kw, "x", 3, step, harvest_file=path, lr=lr,
                                                lr_solver="davidson", engine=FakeCoupledCluster)
    E = {0: [], 1: [], 2: []}
    for p in (-1, 0, 1):                     # the oracle: E_CCSD and its lowest Jacobian roots per field
        model = build_model(mol, alternation=0.1, field=(p * step, 0.0, 0.0))
        scf = rhf(model)
        F, eref = mo_fock(model, scf["V"], scf["D"])
        o = model["nel"] // 2
        out = ccsd_fact.ccsd(F, scf["V"], model["G"], eref, o, eps=1e-12)
        w = np.sort(np.linalg.eigvals(olr.closed_shell_jacobian(F, scf["V"], model["G"], o, out["t1"], out["t2"])).real)
        E[0].append(out["energy"][0]); E[1].append(out["energy"][0] + w[0]); E[2].append(out["energy"][0] + w[1])
    assert res["stencils"][3]["alpha"]["xx"] == pytest.approx(alpha(E[0], step), rel=1e-6)
    for k in (1, 2):
        assert res["states"][k - 1]["stencils"][3]["alpha"]["xx"] == pytest.approx(alpha(E[k], step), rel=1e-5)
    assert "State #1" in report and "State #2" in report
    recs = properties.read_harvester(path)
    assert [r["state"] for r in recs] == [0, 1, 2]
