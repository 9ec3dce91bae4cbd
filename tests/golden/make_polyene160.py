"""Regenerate tests/golden/polyene160.json: the FP64 oracle on the 160-site polyene.

    python tests/golden/make_polyene160.py

Runs the reference SCF (oracle/rhf.py) and the factorised FP64 restatement of
the reference's r-ccsd (oracle/ccsd_fact.py, "2-1" projection, DIIS 20,
residual threshold 1e-8) on polyene(160) with bond-alternation 0.1 and
records E_ref, E_corr and the per-iteration trace (max|d1|, max|d2|, E).
Takes about two hours on 8 cores (27 iterations of about 4 minutes). At a
1e-8 residual the energy is settled well below 1e-6 eV: the last five
iterations of the trace move it by at most 3e-7 eV.
"""
from __future__ import annotations

import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from helios_gb300 import molecules                 # noqa: E402
from oracle import ccsd_fact                       # noqa: E402
from oracle.ppp import build_model                 # noqa: E402
from oracle.rhf import mo_fock, rhf                # noqa: E402


def main(n=160, eps=1e-8):
    mol = molecules.polyene(n)
    model = build_model(mol, alternation=0.1)
    scf = rhf(model)
    F, eref = mo_fock(model, scf["V"], scf["D"])
    o = model["nel"] // 2
    t0 = time.time()
    trace = []

    def cb(it, acc, e):
        trace.append([acc[0], acc[1], float(e[0]), time.time() - t0])
        print(it, acc, e[0] - eref, f"{time.time() - t0:.0f}s", flush=True)

    out = ccsd_fact.ccsd(F, scf["V"], model["G"], eref, o, eps=eps, callback=cb)
    res = {"molecule": mol.name, "n": n, "alternation": 0.1, "eps": eps, "eref": eref,
           "scf_iterations": scf["iterations"], "status": out["status"], "iterations": out["iterations"],
           "ecorr": out["ecorr"], "energy": out["energy"].tolist(), "trace": trace,
           "orbital_energies": scf["E"].tolist()}
    with open(os.path.join(HERE, f"polyene{n}.json"), "w") as f:
        json.dump(res, f, indent=1)


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 160)
