"""GPU parity tests: the CUDA engine against the CPU oracle, through the C ABI.

Tolerances: FP64 path |dE| <= 1e-8 eV against the literal restatement of the
reference (the path computes in FP64, so agreement is ~1e-12 in practice);
mixed path (split-BF16 tensor cores + FP64 finishing iterations) |dE| <= 1e-6 eV.
"""
import json
import os
import threading

import numpy as np
import pytest

from helios_gb300 import molecules

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))


@pytest.fixture(scope="module")
def api():
    from helios_gb300 import build
    build.build()
    from helios_gb300 import api as a
    return a


def _kw(api, **k):
    base = dict(bond_alternation=0.1, accuracy=10)
    base.update(k)
    return api.Keywords(**base)


def _mol(case):
    if case["kind"] == "polyene":
        return molecules.polyene(case["n"])
    if case["kind"] == "dodecahexaene":
        return molecules.dodecahexaene()
    if case["kind"] == "ladder":
        return molecules.ladder(case["n"])
    return molecules.random_molecule(case["seed"], 8, 14)


@pytest.mark.parametrize("case", GOLD["cases"], ids=[c["name"] for c in GOLD["cases"]])
def test_fp64_energy_matches_golden(api, case):
    out = api.get_energy(_mol(case), _kw(api))
    assert out["status"] == 1
    assert abs(out["energy"][1] - case["eref"]) < 1e-9
    assert abs(out["ecorr"] - case["ecorr_1e10"]) < 1e-8
    assert np.allclose(out["scf"]["eps"], case["orbital_energies"], atol=1e-8)
    if case["n"] >= 12:
        assert abs(out["iterations"] - case["iterations_1e10"]) <= 2


def test_one_iteration_matches_oracle_residuals(api):
    from oracle import ccsd_fact
    from oracle.ppp import build_model
    mol = molecules.ladder(10)
    cc = api.CoupledCluster(mol, _kw(api))
    cc.initCC()
    s = cc.scf(0)
    o = cc.dims[0][1]
    I = ccsd_fact.Integrals(s["C"], build_model(mol, alternation=0.1)["G"], o)
    t1r, t2r = ccsd_fact.guess(s["F"], I, o)
    t1g, t2g = cc.amplitudes(0)
    assert np.abs(t1g - t1r).max() < 1e-12 and np.abs(t2g - t2r).max() < 1e-12
    acc = cc.iterationCC(1, 1e-10)
    d1, d2 = ccsd_fact.residuals(s["F"], I, t1r, t2r)
    assert abs(acc[0] - np.abs(d1).max()) < 1e-12 and abs(acc[1] - np.abs(d2).max()) < 1e-12
    # after one step (no DIIS mixing on iteration 1) the amplitudes follow stepCC
    eo, ev = np.diag(s["F"])[:o], np.diag(s["F"])[o:]
    D1 = eo[:, None] - ev[None, :]
    D2 = eo[:, None, None, None] + eo[None, :, None, None] - ev[None, None, :, None] - ev[None, None, None, :]
    t1n = t1r + d1 / D1
    t2n = t2r + (2 * d2 + d2.transpose(0, 1, 3, 2)) / D2
    a1, a2 = cc.amplitudes(0)
    assert np.abs(a1 - t1n).max() < 1e-12 and np.abs(a2 - t2n).max() < 1e-12
    cc.finalizeCC()


@pytest.mark.parametrize("coulomb", ["mataga-nishimoto", "hubbard"])
def test_other_coulomb_models(api, coulomb):
    from oracle.literal import solve_literal
    mol = molecules.polyene(8)
    out = api.get_energy(mol, _kw(api, coulomb_integrals=coulomb))
    ref = solve_literal(mol, alternation=0.1, coulomb=coulomb, eps=1e-10)
    assert out["status"] == ref["status"] == 1
    assert abs(out["ecorr"] - ref["ecorr"]) < 1e-8


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_projection_type_1_matches_literal_oracle(api, precision):
    # coupled-cluster:projection-type = 1: stepCC divides d2(ijab) itself by the
    # denominator and DIIS mixes d2 (mod_cc.f90:1007, :1417); same fixed point as "2-1"
    from oracle.literal import solve_literal
    for mol in (molecules.dodecahexaene(), molecules.random_molecule(11, 8, 14)):
        ref = solve_literal(mol, alternation=0.1, eps=1e-10, projtype=1)
        out = api.get_energy(mol, _kw(api, projection_type="1", precision=precision))
        assert ref["status"] == 1 and out["status"] == 1
        assert abs(out["ecorr"] - ref["ecorr"]) < (1e-8 if precision == "fp64" else 1e-6)
        if precision == "fp64":
            assert abs(out["iterations"] - ref["iterations"]) <= 1


def test_batch_matches_individual_oracle(api):
    from oracle.literal import solve_literal
    mols = [molecules.random_molecule(s, 8, 14) for s in (11, 12, 13, 14, 15)] + [molecules.polyene(4)]
    cc = api.CoupledCluster(mols, _kw(api))
    cc.initCC()
    out = cc.solve_batch()
    cc.finalizeCC()
    for k, m in enumerate(mols):
        ref = solve_literal(m, alternation=0.1, eps=1e-10)
        assert out["status"][k] == 1
        assert abs((out["energy"][k, 0] - out["energy"][k, 1]) - ref["ecorr"]) < 1e-8


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_smallest_molecule_and_a_ragged_batch(api, precision):
    """Ethylene (two sites, o = v = 1: the smallest problem, where two-electron CCSD is exact)
    alone and in one batch with molecules of 4 and 14 sites, against the literal oracle."""
    from oracle.literal import solve_literal
    tol = 1e-8 if precision == "fp64" else 1e-6
    mols = [molecules.polyene(2), molecules.polyene(4), molecules.random_molecule(12, 14, 14)]
    refs = [solve_literal(m, alternation=0.1, eps=1e-10)["ecorr"] for m in mols]
    cc = api.CoupledCluster(mols[0], _kw(api, precision=precision))
    cc.initCC()
    out = cc.iterate()
    cc.finalizeCC()
    assert out["status"] == 1 and abs((out["energy"][0] - out["energy"][1]) - refs[0]) < tol
    cc = api.CoupledCluster(mols, _kw(api, precision=precision))
    cc.initCC()
    out = cc.solve_batch()
    cc.finalizeCC()
    for k in range(len(mols)):
        assert out["status"][k] == 1
        assert abs((out["energy"][k, 0] - out["energy"][k, 1]) - refs[k]) < tol


def test_larger_molecule_against_factorised_oracle(api):
    from oracle import ccsd_fact
    from oracle.ppp import build_model
    from oracle.rhf import mo_fock, rhf
    mol = molecules.ladder(24)
    out = api.get_energy(mol, _kw(api))
    model = build_model(mol, alternation=0.1)
    scf = rhf(model)
    F, eref = mo_fock(model, scf["V"], scf["D"])
    f = ccsd_fact.ccsd(F, scf["V"], model["G"], eref, model["nel"] // 2, eps=1e-10)
    assert out["status"] == 1 and f["status"] == 1
    assert abs(out["energy"][1] - eref) < 1e-9
    assert abs(out["ecorr"] - f["ecorr"]) < 1e-8


@pytest.mark.parametrize("accuracy", [10, 12])
def test_mixed_precision_reaches_fp64_energy(api, accuracy):
    # 12 is the reference's default threshold: below the 5-slice floor, so the
    # molecule finishes with 7-slice (emulated FP64) iterations
    for mol in (molecules.polyene(20), molecules.ladder(24)):
        e64 = api.get_energy(mol, _kw(api, accuracy=accuracy))
        mx = api.get_energy(mol, _kw(api, precision="mixed", accuracy=accuracy))
        assert mx["status"] == 1
        assert abs(mx["energy"][0] - e64["energy"][0]) < 1e-6


def test_exact_precision_follows_the_fp64_iteration(api):
    """precision "exact": every iteration on the 7-slice GEMM, whose error is below the
    FP64 GEMM's, so the solve follows the FP64 one: same iteration count, same energy."""
    for mol in (molecules.polyene(20), molecules.ladder(24)):
        e64 = api.get_energy(mol, _kw(api, accuracy=12))
        cc = api.CoupledCluster(mol, _kw(api, precision="exact", accuracy=12))
        cc.initCC()
        r = cc.iterate()
        tr = cc.trace(0)
        cc.finalizeCC()
        assert r["status"] == 1 and np.all(tr[:, 4] == 1.0)
        assert abs(r["iterations"] - e64["iterations"]) <= 1
        assert abs(r["energy"][0] - e64["energy"][0]) < 1e-9


def test_mixed_trace_starts_on_tensor_cores(api):
    cc = api.CoupledCluster(molecules.polyene(24), _kw(api, precision="mixed"))
    cc.initCC()
    r = cc.iterate()
    tr = cc.trace(0)
    cc.finalizeCC()
    assert r["status"] == 1
    # 3-slice tensor cores first; the last iteration is a check (7-slice
    # emulated FP64 by default)
    assert tr[0, 4] == 4.0 and tr[-1, 4] == 1.0
    d = np.diff(tr[:, 4])
    # phases only move down the ladder, except that a check which does not
    # confirm convergence sends the molecule back to 5-slice iterations
    assert np.all((d <= 0) | ((tr[1:, 4] == 2) & (tr[:-1, 4] <= 1)))
    assert np.all(np.diff(tr[:, 3]) >= 0)


def test_tensor_core_gemm_accuracy(api):
    rng = np.random.default_rng(3)
    # partial tiles, one-row / one-column problems and K far below the k-block
    for (M, N, K) in ((130, 70, 200), (512, 384, 1000), (5, 1, 3), (1, 7, 64), (200, 3, 17), (37, 250, 9)):
        A = rng.normal(size=(M, K))
        B = rng.normal(size=(N, K))
        ref = A @ B.T
        C, _ = api.gemm(A, B, "mixed")
        assert np.abs(C - ref).max() / np.abs(ref).max() < 1e-6
        C, _ = api.gemm(A, B, "mid")
        assert np.abs(C - ref).max() / np.abs(ref).max() < 1e-8
        C, _ = api.gemm(A, B, "high")
        assert np.abs(C - ref).max() / np.abs(ref).max() < 1e-10
        C64, _ = api.gemm(A, B, "fp64")
        assert np.abs(C64 - ref).max() / np.abs(ref).max() < 1e-13
        CX, _ = api.gemm(A, B, "exact")
        assert np.abs(CX - ref).max() / np.abs(ref).max() < 1e-14


def test_exact_gemm_is_as_accurate_as_fp64(api):
    # the 7-slice mode against an extended-precision product: its error is
    # that of an FP64 GEMM (rows of very different scales included)
    rng = np.random.default_rng(5)
    for (M, N, K) in ((130, 70, 200), (64, 48, 3000)):
        A = rng.normal(size=(M, K)) * np.exp(2 * rng.normal(size=(M, 1)))
        B = rng.normal(size=(N, K))
        ref = (A.astype(np.longdouble) @ B.T.astype(np.longdouble))
        scale = np.abs(ref).max(axis=1, keepdims=True)
        CX, _ = api.gemm(A, B, "exact")
        C64, _ = api.gemm(A, B, "fp64")
        ex = float((np.abs(CX - ref) / scale).max())
        e64 = float((np.abs(C64 - ref) / scale).max())
        assert ex < 4 * e64 + 1e-16, (ex, e64)


def test_status_codes(api):
    mol = molecules.polyene(6)
    out = api.CoupledCluster(mol, _kw(api))
    out.initCC()
    assert out.iterate(maxiter=2)["status"] == -1
    out.finalizeCC()
    # the "2-1" step is 3x a Newton step: without DIIS it diverges, as in the reference
    out = api.get_energy(mol, _kw(api, diis_enabled=False))
    assert out["status"] == -2


def test_cancel_interrupts(api):
    cc = api.CoupledCluster(molecules.polyene(30), _kw(api, accuracy=14))
    cc.initCC()
    t = threading.Timer(0.05, cc.cancel)
    t.start()
    r = cc.iterate()
    t.join()
    assert r["status"] in (-4, 1, -3)
    cc.finalizeCC()


def test_bad_arguments_are_errors(api):
    bad = molecules.polyene(6)
    bad.nels = bad.nels.copy()
    bad.nels[0] = 2                        # 7 electrons: not closed shell
    with pytest.raises(api.HxError) as e:
        api.CoupledCluster(bad, _kw(api))
    assert e.value.code == -100


def test_amplitudes_round_trip(api):
    cc = api.CoupledCluster(molecules.polyene(10), _kw(api))
    cc.initCC()
    cc.iterate(maxiter=3)
    t1, t2 = cc.amplitudes(0)
    cc.set_guess(0, t1, t2)
    b1, b2 = cc.amplitudes(0)
    assert np.array_equal(t1, b1) and np.array_equal(t2, b2)
    assert np.abs(t2 - t2.transpose(1, 0, 3, 2)).max() == 0.0      # pair symmetry
    cc.finalizeCC()


def test_polarizability_matches_oracle(api):
    from helios_gb300 import polariz
    from oracle.polariz import polarizability as ref_pol
    mol = molecules.polyene(8)
    out = polariz.polarizability(mol, _kw(api, accuracy=11), step=0.02)
    ref, _ = ref_pol(mol, step=0.02)
    assert np.all(out["status"] == 1)
    assert abs(out["alpha"] - ref) / abs(ref) < 1e-6


def test_full_size_polyene_properties(api):
    # N = 160: two FP64 iterations; the device energy must equal the energy
    # functional evaluated on the host from the exported amplitudes and
    # orbitals, and t2 must keep its pair symmetry exactly.
    from oracle import ccsd_fact
    from oracle.ppp import build_model
    mol = molecules.polyene(160)
    cc = api.CoupledCluster(mol, _kw(api))
    cc.initCC()
    r = cc.iterate(maxiter=2)
    t1, t2 = cc.amplitudes(0)
    s = cc.scf(0)
    cc.finalizeCC()
    assert np.abs(t2 - t2.transpose(1, 0, 3, 2)).max() == 0.0
    o = t1.shape[0]
    I = ccsd_fact.Integrals(s["C"], build_model(mol, alternation=0.1)["G"], o)
    e = ccsd_fact.energy(s["F"], I, t1, t2, r["energy"][1])
    assert abs(e[0] - r["energy"][0]) < 1e-8


def test_full_size_polyene_mixed_energy_matches_oracle(api):
    # N = 160 (o = v = 80): the mixed-precision solve, learned guess and the
    # 7-slice (emulated FP64) check included, must land within 1e-6 eV of the
    # FP64 oracle's converged energy (tests/golden/polyene160.json, residual
    # 1e-8), and its SCF must reproduce the oracle's reference energy.
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "polyene160.json")))
    cc = api.CoupledCluster(molecules.polyene(160), _kw(api, accuracy=7, precision="mixed", guess="learned"))
    cc.initCC()
    r = cc.iterate()
    tr = cc.trace(0)
    cc.finalizeCC()
    assert r["status"] == 1 and tr[-1, 4] == 1.0
    assert abs(r["energy"][1] - gold["eref"]) < 1e-9
    assert abs(r["energy"][0] - gold["energy"][0]) < 1e-6
