"""Regenerate tests/golden/golden.json from the CPU oracle.

    python tests/golden/make_golden.py

The reference (Fortran, Intel-only extensions, no build files) cannot be built
here and ships no test data, so the pinned values come from the literal C
restatement of its algorithm (oracle/cc_literal.c), cross-checked against an
independent textbook spin-orbital CCSD (oracle/spin_ccsd.py) and the
factorised restatement (oracle/ccsd_fact.py).
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from helios_gb300 import molecules                     # noqa: E402
from oracle import ccsd_fact, literal, spin_ccsd       # noqa: E402

CASES = [
    ("polyene", 4, {}),
    ("polyene", 6, {}),
    ("dodecahexaene", 12, {}),
    ("ladder", 8, {}),
    ("ladder", 12, {}),
    ("random", 14, {"seed": 1234}),
]


def make(kind, n, extra):
    if kind == "polyene":
        return molecules.polyene(n)
    if kind == "dodecahexaene":
        return molecules.dodecahexaene()
    if kind == "ladder":
        return molecules.ladder(n)
    return molecules.random_molecule(extra["seed"], 8, 14)


def main():
    out = {"alternation": 0.1, "coulomb": "ohno-klopman", "cases": []}
    for kind, n, extra in CASES:
        mol = make(kind, n, extra)
        r10 = literal.solve_literal(mol, alternation=0.1, eps=1e-10)
        r12 = literal.solve_literal(mol, alternation=0.1, eps=1e-12)
        case = {"kind": kind, "n": mol.n_sites, "name": mol.name, **extra,
                "eref": r10["eref"], "scf_iterations": r10["scf"]["iterations"],
                "ecorr_1e10": r10["ecorr"], "iterations_1e10": r10["iterations"],
                "ecorr_1e12": r12["ecorr"], "iterations_1e12": r12["iterations"],
                "orbital_energies": r10["scf"]["E"].tolist()}
        if mol.n_sites <= 12:
            e, _ = spin_ccsd.ccsd(r12["scf"]["V"], r12["model"]["G"], r12["model"]["core"], r12["o"], eps=1e-12)
            case["ecorr_spin_orbital"] = e
        out["cases"].append(case)
        print(case["name"], case["ecorr_1e10"], case["iterations_1e10"])
    # residuals of one molecule at seeded amplitudes, with the orbitals used
    mol = molecules.polyene(6)
    r = literal.solve_literal(mol, alternation=0.1, eps=1e-10, maxiter=1)
    o = r["o"]
    v = mol.n_sites - o
    rng = np.random.default_rng(20261203)
    t1 = rng.normal(size=(o, v)) * 0.1
    t2 = rng.normal(size=(o, o, v, v)) * 0.05
    t2 = 0.5 * (t2 + t2.transpose(1, 0, 3, 2))
    d1, d2 = literal.residuals(r["F"], r["R"], t1, t2)
    out["residual_case"] = {"name": mol.name, "C": r["scf"]["V"].tolist(), "F": r["F"].tolist(),
                            "t1": t1.tolist(), "t2": t2.tolist(), "d1": d1.tolist(), "d2": d2.tolist(),
                            "energy": literal.energy(r["F"], r["R"], t1, t2, r["eref"]).tolist()}
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
