"""The LR-CCSD oracle (oracle/lrccsd.py), no GPU.

The reference's spin-orbital sigma equations (proj-lrccsd-spin-hf-*.f90) are
pinned element by element against e^{-T} H e^{T} - E_cc built exactly in the
determinant space; the Jacobian of the closed-shell r-ccsd residual has the
singlet part of that spectrum; the reference's iteration (stepLR + DIIS,
mod_lrccsd.f90:216-326, 1081-1225) converges to eigenvalues of it, with the
reference weight r0 of energyLR equal to <HF|H-bar|R> / omega.
"""
import numpy as np
import pytest

from helios_gb300 import molecules
from oracle import ccsd_fact, lrccsd
from oracle.ppp import build_model
from oracle.rhf import mo_fock, rhf
from oracle.triples import spin_amplitudes

MOLS = {"butadiene": molecules.polyene(4), "rnd5-ladder-4": molecules.random_molecule(5, 4, 6),
        "hexatriene": molecules.polyene(6)}


@pytest.fixture(scope="module", params=list(MOLS))
def case(request):
    mol = MOLS[request.param]
    model = build_model(mol, alternation=0.1)
    scf = rhf(model)
    F, eref = mo_fock(model, scf["V"], scf["D"])
    o = model["nel"] // 2
    out = ccsd_fact.ccsd(F, scf["V"], model["G"], eref, o, eps=1e-13)
    assert out["status"] == 1
    C, G, h = scf["V"], model["G"], model["core"]
    A, singles, doubles, e_cc, top = lrccsd.hbar_block(C, G, h, o, out["t1"], out["t2"])
    return {"C": C, "G": G, "h": h, "F": F, "o": o, "t1": out["t1"], "t2": out["t2"], "A": A,
            "singles": singles, "doubles": doubles, "top": top, "eA": np.linalg.eigvals(A).real,
            "ecorr": out["energy"][0] - eref, "e_cc": e_cc, "eref": eref, "enuc": scf["enuc"]}


def _flat(c, r1, r2):
    return np.concatenate([[r1[i, a] for i, a in c["singles"]], [r2[i, j, a, b] for i, j, a, b in c["doubles"]]])


def test_hbar_reference_energy_is_the_ccsd_energy(case):
    # <HF|H-bar|HF> = E_ref + E_corr without the site-site repulsion constant
    assert case["e_cc"] + case["enuc"] == pytest.approx(case["eref"] + case["ecorr"], abs=1e-10)


def test_sigma_equals_the_determinant_space_hbar(case):
    c = case
    P = lrccsd.SpinProblem(c["C"], c["G"], c["h"], c["o"], c["t1"], c["t2"])
    X = lrccsd.intermediates(P)
    rng = np.random.default_rng(3)
    so, sv = np.arange(P.no) % 2, np.arange(P.nv) % 2
    sz = (so[:, None, None, None] + so[None, :, None, None]) == (sv[None, None, :, None] + sv[None, None, None, :])
    for part in ("singles", "doubles", "both"):
        r1 = rng.normal(size=(P.no, P.nv)) * P.same1 * (part != "doubles")
        r2 = lrccsd.antisym_from_upper(P, rng.normal(size=(P.no, P.no, P.nv, P.nv)) * sz) * (part != "singles")
        d1, d2 = lrccsd.sigma(P, X, r1, r2)
        want = c["A"] @ _flat(c, r1, r2)
        got = _flat(c, d1, d2)
        assert np.abs(got - want).max() < 1e-12 * np.abs(want).max(), part


def test_closed_shell_jacobian_has_the_singlet_spectrum(case):
    c = case
    o, v = c["t1"].shape
    J = lrccsd.closed_shell_jacobian(c["F"], c["C"], c["G"], o, c["t1"], c["t2"])
    w, U = np.linalg.eig(J)
    assert np.abs(w.imag).max() < 1e-9
    w, U = w.real, U.real
    for k in np.argsort(w)[:4]:
        assert np.min(np.abs(c["eA"] - w[k])) < 1e-9
        # the eigenvector, made spin-orbital by the amplitude rules, is a sigma eigenvector
        r1, r2 = lrccsd.closed_shell_unpack(U[:, k], o, v)
        s1, s2 = spin_amplitudes(r1, r2)
        x = _flat(c, s1, s2)
        assert np.abs(c["A"] @ x - w[k] * x).max() < 1e-9 * np.abs(x).max()


@pytest.mark.parametrize("spin", [0, 1], ids=["singlet", "triplet"])
def test_reference_iteration_converges_to_eigenpairs(case, spin):
    c = case
    r = lrccsd.lr_solve(c["C"], c["G"], c["h"], c["F"], c["o"], c["t1"], c["t2"], nstates=2, spin=spin, eps=1e-8)
    assert list(r["status"]) == [1, 1] and np.all(np.diff(r["omega"]) >= 0)
    P = lrccsd.SpinProblem(c["C"], c["G"], c["h"], c["o"], c["t1"], c["t2"])
    for k in range(2):
        w, r1, r2 = r["omega"][k], r["r1"][k], r["r2"][k]
        assert np.min(np.abs(c["eA"] - w)) < 1e-8
        s1, s2 = float((r1 ** 2).sum()), float((r2[P.upper] ** 2).sum())
        assert s1 + s2 == pytest.approx(1.0, abs=1e-12)                        # normalize
        ra, rb = r1[0::2, 0::2], r1[1::2, 1::2]
        assert np.abs(ra - (rb if spin == 0 else -rb)).max() < 1e-14            # spin symmetry of r1
        x = _flat(c, r1, r2)
        assert r["r0"][k] == pytest.approx(float(c["top"] @ x) / w, abs=1e-8)   # energyLR r0
        assert r["ael"][k] == pytest.approx((s1 + 2 * s2) / (s1 + s2))
        if spin == 1:
            assert abs(r["r0"][k]) < 1e-10                                       # no overlap with a singlet


def test_cis_guess_is_the_cis_spectrum():
    mol = molecules.polyene(6)
    model = build_model(mol, alternation=0.1)
    scf = rhf(model)
    F, _ = mo_fock(model, scf["V"], scf["D"])
    o = model["nel"] // 2
    sel, w = lrccsd.cis_guess(F, scf["V"], model["G"], o, 3)
    assert np.all(np.diff(w) >= 0) and w[0] > 0
    assert all(len(s) >= 1 and all(abs(c) >= 0.1 for _, _, c in s) for s in sel)
    # HOMO -> LUMO dominates the lowest CIS root of a polyene
    i, a, _ = max(sel[0], key=lambda x: abs(x[2]))
    assert (i, a) == (o - 1, 0)
