"""CPU tests of the oracle: golden values, three-way agreement, invariants.

The oracle is the checker of the GPU engine; these tests pin it before it is
trusted. Golden values: tests/golden/golden.json (tests/golden/make_golden.py).
"""
import json
import math
import os

import numpy as np
import pytest

from helios_gb300 import molecules
from oracle import ccsd_fact, literal, spin_ccsd
from oracle.ppp import TR_CONST, build_model
from oracle.rhf import mo_fock, rhf

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))


def _mol(case):
    if case["kind"] == "polyene":
        return molecules.polyene(case["n"])
    if case["kind"] == "dodecahexaene":
        return molecules.dodecahexaene()
    if case["kind"] == "ladder":
        return molecules.ladder(case["n"])
    return molecules.random_molecule(case["seed"], 8, 14)


def test_gamma_ohno_klopman_formula():
    # two sites 1.4 Angstrom apart: gamma = U / sqrt(1 + (trConst U r)^2)
    m = molecules.polyene(2, 1.4, 1.4)
    model = build_model(m)
    U = molecules.HUBBARD_U
    assert model["G"][0, 0] == pytest.approx(U, abs=1e-15)
    assert model["G"][0, 1] == pytest.approx(U / math.sqrt(1 + (TR_CONST * U * 1.4) ** 2), rel=1e-15)
    assert TR_CONST == pytest.approx(1 / 14.39964535, rel=1e-8)


def test_core_and_alternation():
    m = molecules.polyene(4)
    model = build_model(m, alternation=0.1)
    C = model["connect"]
    assert C[0, 1] == pytest.approx(-2.4 * 1.1)      # double bond
    assert C[1, 2] == pytest.approx(-2.4 * 0.9)      # single bond
    G = model["G"]
    for k in range(4):
        assert model["core"][k, k] == pytest.approx(-(G[k].sum() - G[k, k]))
    assert np.allclose(model["coords"].sum(0), 0.0, atol=1e-12)


def test_field_perturbation_is_diagonal_x():
    m = molecules.polyene(6)
    model = build_model(m, alternation=0.1, field=(0.02, 0.0, 0.0))
    pert = model["core"] - build_model(m, alternation=0.1)["core"]
    assert np.allclose(np.diag(pert), 0.02 * model["coords"][:, 0])
    assert np.allclose(pert - np.diag(np.diag(pert)), 0.0)


@pytest.mark.parametrize("case", GOLD["cases"], ids=[c["name"] for c in GOLD["cases"]])
def test_literal_oracle_matches_golden(case):
    mol = _mol(case)
    r = literal.solve_literal(mol, alternation=0.1, eps=1e-10)
    assert r["status"] == 1
    assert r["eref"] == pytest.approx(case["eref"], abs=1e-10)
    assert r["ecorr"] == pytest.approx(case["ecorr_1e10"], abs=1e-9)
    assert np.allclose(r["scf"]["E"], case["orbital_energies"], atol=1e-9)
    if mol.n_sites >= 12:
        assert abs(r["iterations"] - case["iterations_1e10"]) <= 2


@pytest.mark.parametrize("case", [c for c in GOLD["cases"] if "ecorr_spin_orbital" in c],
                         ids=[c["name"] for c in GOLD["cases"] if "ecorr_spin_orbital" in c])
def test_spin_adapted_equals_spin_orbital(case):
    # the reference's "2-1" closed-shell equations vs textbook spin-orbital CCSD
    assert abs(case["ecorr_1e12"] - case["ecorr_spin_orbital"]) < 1e-10


def test_literal_and_factorised_residuals_agree():
    rc = GOLD["residual_case"]
    mol = molecules.polyene(6)
    model = build_model(mol, alternation=0.1)
    C, F = np.array(rc["C"]), np.array(rc["F"])
    t1, t2 = np.array(rc["t1"]), np.array(rc["t2"])
    o = t1.shape[0]
    I = ccsd_fact.Integrals(C, model["G"], o)
    d1, d2 = ccsd_fact.residuals(F, I, t1, t2)
    assert np.abs(d1 - np.array(rc["d1"])).max() < 1e-12
    assert np.abs(d2 - np.array(rc["d2"])).max() < 1e-12
    # and the literal C code on the same inputs
    R = literal.integrals(C, model["G"])
    l1, l2 = literal.residuals(F, R, t1, t2)
    assert np.abs(l1 - np.array(rc["d1"])).max() < 1e-12
    assert np.abs(l2 - np.array(rc["d2"])).max() < 1e-12


def test_factorised_solver_matches_literal():
    mol = molecules.ladder(10)
    r = literal.solve_literal(mol, alternation=0.1, eps=1e-10)
    f = ccsd_fact.ccsd(r["F"], r["scf"]["V"], r["model"]["G"], r["eref"], r["o"], eps=1e-10)
    assert f["status"] == 1
    assert abs(f["ecorr"] - r["ecorr"]) < 1e-10
    assert abs(f["iterations"] - r["iterations"]) <= 1


def test_doubles_pair_symmetry_and_mirror():
    rc = GOLD["residual_case"]
    d2 = np.array(rc["d2"])
    assert np.abs(d2 - d2.transpose(1, 0, 3, 2)).max() < 1e-14


def test_two_electron_ccsd_is_fci():
    # ethylene: 2 sites, 2 electrons -> CCSD is exact (FCI of the singlet space)
    mol = molecules.polyene(2, 1.34, 1.34)
    r = literal.solve_literal(mol, alternation=0.1, eps=1e-12)
    model = build_model(mol, alternation=0.1)
    C = r["scf"]["V"]
    h = C.T @ model["core"] @ C
    B = np.einsum("mp,mq->mpq", C, C)
    eri = np.einsum("mpq,mn,nrs->pqrs", B, model["G"], B)
    # singlet CSFs |11>, |22>, (|12>+|21>)/sqrt2 in the MO basis
    E0 = 2 * h[0, 0] + eri[0, 0, 0, 0]
    E1 = 2 * h[1, 1] + eri[1, 1, 1, 1]
    Es = h[0, 0] + h[1, 1] + eri[0, 0, 1, 1] + eri[0, 1, 1, 0]
    H = np.array([[E0, eri[0, 1, 0, 1], math.sqrt(2) * (h[0, 1] + eri[0, 0, 0, 1])],
                  [eri[0, 1, 0, 1], E1, math.sqrt(2) * (h[0, 1] + eri[1, 1, 1, 0])],
                  [math.sqrt(2) * (h[0, 1] + eri[0, 0, 0, 1]), math.sqrt(2) * (h[0, 1] + eri[1, 1, 1, 0]), Es]])
    efci = np.linalg.eigvalsh(H)[0]
    enuc = model["G"][0, 1]
    assert r["status"] == 1
    assert abs((efci + enuc) - r["energy"][0]) < 1e-10


def test_size_consistency_two_far_ethylenes():
    e1 = molecules.polyene(2, 1.34, 1.34)
    r1 = literal.solve_literal(e1, alternation=0.1, eps=1e-12)
    two = molecules.Molecule("2xethylene", np.vstack([e1.coords, e1.coords + [0.0, 1.0e7, 0.0]]),
                             np.zeros(4), np.full(4, molecules.HUBBARD_U), np.ones(4, dtype=np.int32),
                             [(0, 1, -2.4, "double"), (2, 3, -2.4, "double")])
    r2 = literal.solve_literal(two, alternation=0.1, eps=1e-12)
    assert abs(r2["ecorr"] - 2 * r1["ecorr"]) < 1e-8


def test_field_energy_is_even_for_centrosymmetric_chain():
    mol = molecules.polyene(8)
    ep = literal.solve_literal(mol, alternation=0.1, field=(0.05, 0, 0), eps=1e-11)["energy"][0]
    em = literal.solve_literal(mol, alternation=0.1, field=(-0.05, 0, 0), eps=1e-11)["energy"][0]
    assert abs(ep - em) < 1e-9


def test_reference_diis_route_reaches_same_energy():
    # the reference solves DIIS through an eigen-decomposition; same energy
    mol = molecules.polyene(8)
    a = literal.solve_literal(mol, alternation=0.1, eps=1e-9, diis_solver=0)
    b = literal.solve_literal(mol, alternation=0.1, eps=1e-9, diis_solver=1)
    assert a["status"] == 1 and b["status"] == 1
    assert abs(a["ecorr"] - b["ecorr"]) < 1e-8


def test_stop_rules_maxiter_and_divergence():
    mol = molecules.polyene(6)
    r = literal.solve_literal(mol, alternation=0.1, eps=1e-10, maxiter=3)
    assert r["status"] == -1 and r["iterations"] == 3
    # without DIIS the 3x Jacobi step of the "2-1" projection diverges
    r = literal.solve_literal(mol, alternation=0.1, eps=1e-10, diis=False)
    assert r["status"] == -2


def test_rhf_reference_scheme_converges():
    for mol in (molecules.polyene(30), molecules.ladder(30)):
        model = build_model(mol, alternation=0.1)
        scf = rhf(model)
        assert scf["status"] == 1
        F, eref = mo_fock(model, scf["V"], scf["D"])
        assert abs(eref - scf["energy"]) < 1e-10
        assert np.abs(F - np.diag(np.diag(F))).max() < 1e-9
        o = model["nel"] // 2
        assert scf["E"][o] - scf["E"][o - 1] > 1.0     # aufbau gap


# ---------------------------------------------------------------- learned-guess network oracle
def test_mlp_oracle_backward_matches_finite_differences():
    from oracle import mlp
    rng = np.random.default_rng(0)
    X = rng.normal(size=(64, 8))
    T = rng.normal(size=64) * 0.01
    p = mlp.init(rng, X.mean(0), 1 / X.std(0), 0.01)
    p["w4"] = rng.normal(size=256) * 0.2
    _, g = mlp.loss_and_grads(p, X, T, rounding=False)
    for name, idx in [("W1", (3, 2)), ("b1", (5,)), ("W2", (4, 4)), ("b2", (9,)), ("W3", (1, 2)),
                      ("b3", (7,)), ("w4", (7,)), ("b4", (0,))]:
        h = 1e-6
        pp = {k: v.copy() for k, v in p.items()}
        pm = {k: v.copy() for k, v in p.items()}
        pp[name][idx] += h
        pm[name][idx] -= h
        fd = (mlp.loss_and_grads(pp, X, T, False)[0] - mlp.loss_and_grads(pm, X, T, False)[0]) / (2 * h)
        assert abs(fd - g[name][idx]) <= 1e-5 * abs(g[name][idx]) + 1e-12, name


def test_mlp_oracle_pack_round_trip_and_bf16_rounding():
    from oracle import mlp
    rng = np.random.default_rng(1)
    p = mlp.init(rng, np.zeros(8), np.ones(8), 1.0)
    blob = mlp.pack(p)
    assert blob.size == mlp.NPARAM == 134162
    q = mlp.unpack(blob)
    assert all(np.array_equal(np.float32(p[k]), np.float32(q[k])) for k in p)
    # ties to even: 1 + 2^-8 is halfway between bf16 neighbours 1 and 1 + 2^-7
    assert mlp.bf16(np.float32(1 + 2 ** -8)) == 1.0
    assert mlp.bf16(np.float32(1 + 3 * 2 ** -8)) == 1 + 2 ** -6


def test_mlp_features_restate_the_guess():
    from oracle import mlp
    mol = molecules.polyene(8)
    model = build_model(mol, alternation=0.1)
    scf = rhf(model)
    F, _ = mo_fock(model, scf["V"], scf["D"])
    o = model["nel"] // 2
    I = ccsd_fact.Integrals(scf["V"], model["G"], o)
    v = F.shape[0] - o
    ov = o * v
    gov = I.coulomb("ovov").reshape(ov, ov)
    rows = np.arange(ov * (ov + 1) // 2)
    X, guess = mlp.features(F, gov, o, rows)
    _, t2 = ccsd_fact.guess(F, I, o)                  # t2[i, j, a, b]
    t2p = t2.transpose(0, 2, 1, 3).reshape(ov, ov)    # rows (ia), columns (jb)
    iu = np.triu_indices(ov)
    assert np.allclose(guess, t2p[iu], rtol=1e-12, atol=1e-15)
    assert np.allclose(X[:, 7], 1.0)                  # 8 / N with N = 8
