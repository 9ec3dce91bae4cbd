"""ORACLE (test infrastructure only) -- closed-shell PPP RHF.

Restates ``src/methods/mod_scf.f90`` (helios SCF 1.100):
  * guess: eigenvectors of ``huckelCore``, aufbau half density
    ``D = sum_{i<=nocc} C_mu,i C_nu,i``                      (``:351-413``)
  * Fock: ``F = core - G o D + 2 diag(G . diag D)``         (``:417-442``)
  * gradient ``Fmin = (F R - R F) R`` with ``R = 2D - 1``    (``:446-494``)
  * iteration: ``D -= (iter-step + variation) Fmin``; rebuild F; diagonalise F;
    aufbau D; rebuild F; accuracy = max|Fmin| before the step (``:106-136``)
  * energy: ``Eel = sum D (core + F)``, ``Enuc = sum_{mu<nu} G``  (``:166-200``)
and the stop rules of the generic iterator (``src/calculation/gIterator.f90:88-210``):
converged when accuracy < eps, diverged when accuracy > divergence threshold,
failed when the next iteration would exceed ``maxiter``, stagnated when after
``stagnation-check-after`` iterations at most ``stagnation-threshold`` percent
of iterations improved.

The reference diagonalises with its own Householder/QL routine (``tred4``,
``src/modules/mod_math.f90:31-230``); any FP64 symmetric eigensolver with
ascending eigenvalues gives the same density, so numpy's is used here.
"""
from __future__ import annotations

import numpy as np

STATUS_CONVERGED = 1
STATUS_MAXITER = -1
STATUS_DIVERGED = -2
STATUS_STAGNATED = -3
STATUS_INTERRUPTED = -4


def fock(core, G, D):
    F = core - G * D
    F[np.diag_indices_from(F)] += 2.0 * (G @ np.diag(D))
    return F


def density(V, nocc):
    Vo = V[:, :nocc]
    return Vo @ Vo.T


def fmin(F, D):
    n = F.shape[0]
    R = 2.0 * D - np.eye(n)
    comm = F @ R - R @ F
    return comm @ R


def energy(core, G, D, F):
    eel = float((D * (core + F)).sum())
    enuc = float(G[np.triu_indices_from(G, 1)].sum())
    return eel + enuc, eel, enuc


class IteratorRules:
    """Stop rules of gIterator.f90 (defaults from src/input/definebd.f90:53-60)."""

    def __init__(self, maxiter, eps, divergence=1e3, stagnation_percent=60.0,
                 stagnation_after=200, check_divergence=True, check_stagnation=True):
        self.maxiter, self.eps = maxiter, eps
        self.divergence, self.stag_pct, self.stag_after = divergence, stagnation_percent, stagnation_after
        self.check_div, self.check_stag = check_divergence, check_stagnation
        self.iteration = 0
        self.successful = 1
        self.current = 0.0

    def update(self, accuracy):
        """Feed max(accuracy) of one iteration; return a status or None to continue."""
        self.iteration += 1
        previous, self.current = self.current, accuracy
        if self.current < previous:
            self.successful += 1
        if self.current < self.eps:
            return STATUS_CONVERGED
        if self.check_div and self.current > self.divergence:
            return STATUS_DIVERGED
        if self.iteration + 1 > self.maxiter:
            return STATUS_MAXITER
        if self.check_stag and self.iteration > self.stag_after:
            if 100.0 * self.successful / self.iteration <= self.stag_pct:
                return STATUS_STAGNATED
        return None


def rhf(model, nocc=None, maxiter=400, eps=1e-12, step=0.05, D0=None):
    """Run the reference SCF. Returns dict(V, E, D, F, energy, status, iterations)."""
    core, G = model["core"], model["G"]
    n = model["n"]
    nocc = model["nel"] // 2 if nocc is None else nocc
    if D0 is None:
        e, V = np.linalg.eigh(model["huckelCore"])
        D = density(V, nocc)
    else:
        D = D0.copy()
    F = fock(core, G, D)
    rules = IteratorRules(maxiter, eps)
    status = None
    E = None
    V = None
    while status is None:
        Fm = fmin(F, D)
        acc = float(np.abs(Fm).max())
        D = D - step * Fm
        F = fock(core, G, D)
        E, V = np.linalg.eigh(F)
        D = density(V, nocc)
        F = fock(core, G, D)
        status = rules.update(acc)
    etot, eel, enuc = energy(core, G, D, F)
    return {"V": V, "E": E, "D": D, "F": F, "energy": etot, "eel": eel, "enuc": enuc,
            "status": status, "iterations": rules.iteration, "nocc": nocc, "n": n}


def mo_fock(model, V, D):
    """MO Fock matrix of prepareFock('spatial') (mod_cc.f90:2336-2396) and the
    reference energy of referenceEnergy (mod_cc.f90:2474-2504)."""
    X = fock(model["core"], model["G"], D)
    eref, _, _ = energy(model["core"], model["G"], D, X)
    return V.T @ X @ V, eref
