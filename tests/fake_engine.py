"""A CPU stand-in for helios_gb300.api.CoupledCluster, built on the oracle.

Test infrastructure only: it lets the host logic that drives the engine
(helios_gb300.lrccsd) run on a machine without a GPU. It keeps the engine's
calling conventions: one handle holds a batch of molecules, ``initCC`` runs
the SCF and the reference guess for each, ``iterationCC`` takes one stepCC of
every molecule with the handle's t-steps and no DIIS mixing after
``set_guess``, ``iterate`` solves molecule 0.
"""
import numpy as np

from oracle import ccsd_fact
from oracle.ppp import build_model
from oracle.rhf import mo_fock, rhf


class FakeCoupledCluster:
    def __init__(self, molecules, keywords):
        from helios_gb300.molecules import Molecule
        self.molecules = [molecules] if isinstance(molecules, Molecule) else list(molecules)
        self.keywords = keywords
        self.iterations = 0

    def initCC(self):
        kw = self.keywords
        self.state = []
        for mol in self.molecules:
            model = build_model(mol, coulomb=kw.coulomb_integrals, alternation=kw.bond_alternation, field=kw.field)
            scf = rhf(model, eps=10.0 ** (-kw.scf_accuracy))
            F, eref = mo_fock(model, scf["V"], scf["D"])
            o = model["nel"] // 2
            I = ccsd_fact.Integrals(scf["V"], model["G"], o)
            t1, t2 = ccsd_fact.guess(F, I, o)
            self.state.append({"C": scf["V"], "G": model["G"], "F": F, "eref": eref, "o": o, "I": I,
                               "t1": t1, "t2": t2, "scf": scf})
        self.dims = [(s["C"].shape[0], s["o"], s["C"].shape[0] - s["o"], 0) for s in self.state]

    def iterate(self):
        s = self.state[0]
        out = ccsd_fact.ccsd(s["F"], s["C"], s["G"], s["eref"], s["o"], eps=10.0 ** (-self.keywords.accuracy))
        s["t1"], s["t2"] = out["t1"], out["t2"]
        return {"status": out["status"], "iterations": out["iterations"], "energy": out["energy"]}

    def iterationCC(self, iteration, epsilon):
        kw = self.keywords
        self.iterations += 1
        for s in self.state:
            d1, d2 = ccsd_fact.residuals(s["F"], s["I"], s["t1"], s["t2"])
            eo, ev = np.diag(s["F"])[:s["o"]], np.diag(s["F"])[s["o"]:]
            D1 = eo[:, None] - ev[None, :]
            D2 = eo[:, None, None, None] + eo[None, :, None, None] - ev[None, None, :, None] - ev[None, None, None, :]
            s["t1"] = s["t1"] + kw.t1_step * d1 / D1
            s["t2"] = s["t2"] + kw.t2_step * (2 * d2 + d2.transpose(0, 1, 3, 2)) / D2
        return np.zeros(5)

    def set_guess(self, mol, t1, t2):
        self.state[mol]["t1"] = np.array(t1, dtype=np.float64)
        self.state[mol]["t2"] = np.array(t2, dtype=np.float64)

    def amplitudes(self, mol=0):
        return self.state[mol]["t1"].copy(), self.state[mol]["t2"].copy()

    def scf(self, mol=0):
        s = self.state[mol]
        return {"C": s["C"], "F": s["F"], "eps": np.diag(s["F"]), "energy": s["scf"]["energy"]}

    def finalizeCC(self):
        self.state = []
