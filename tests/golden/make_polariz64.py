"""Regenerate tests/golden/polariz64.json: the FP64 oracle's finite-field alpha_xx
of the 2 x 32 acene-like ladder (64 sites).

    python tests/golden/make_polariz64.py

Five field points F = 0, +-1e-4, +-2e-4 a.u. along the long axis, added as
site energies -F x_i (helios's getPolarizability perturbation,
src/modules/mod_property.f90:405-506); each point is solved by the reference
SCF (oracle/rhf.py) and the factorised FP64 restatement of r-ccsd
(oracle/ccsd_fact.py) to residual 1e-10; alpha_xx comes from the Lagrange
second derivative (oracle/polariz.py). A few minutes on 8 cores.

A step of 1e-3 a.u. (about 1 eV across the 38 Angstrom ladder at the first
point, 2 eV at the second) drives the reference SCF into stagnation (status
-3, a fully charge-separated density): every point's SCF status is checked.
"""
from __future__ import annotations

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from helios_gb300 import molecules               # noqa: E402
from oracle import ccsd_fact                     # noqa: E402
from oracle.polariz import alpha                 # noqa: E402
from oracle.ppp import build_model               # noqa: E402
from oracle.rhf import mo_fock, rhf              # noqa: E402

BOHR_RADIUS = 0.52917721067
HARTREE_ENERGY = 27.21138602
AU_FIELD = HARTREE_ENERGY / BOHR_RADIUS          # V/Angstrom per atomic unit of field


def main(n=64, f_au=1e-4, eps=1e-10):
    mol = molecules.ladder(n)
    step = f_au * AU_FIELD
    energies, iters = [], []
    for p in (-2, -1, 0, 1, 2):
        model = build_model(mol, alternation=0.1, field=(p * step, 0.0, 0.0))
        scf = rhf(model)
        assert scf["status"] == 1, (p, scf["status"], scf["iterations"])
        F, eref = mo_fock(model, scf["V"], scf["D"])
        out = ccsd_fact.ccsd(F, scf["V"], model["G"], eref, model["nel"] // 2, eps=eps)
        energies.append(float(out["energy"][0]))
        iters.append(int(out["iterations"]))
        print(p, out["status"], out["iterations"], energies[-1], flush=True)
    a = float(alpha(energies, step))
    res = {"molecule": mol.name, "n": n, "alternation": 0.1, "field_au": f_au, "step_V_per_A": step,
           "eps": eps, "energies": energies, "iterations": iters, "alpha_xx": a}
    with open(os.path.join(HERE, f"polariz{n}.json"), "w") as f:
        json.dump(res, f, indent=1)
    print("alpha_xx", a)


if __name__ == "__main__":
    main()
