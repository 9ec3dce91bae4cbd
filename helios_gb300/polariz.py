"""Finite-field static polarizability on the GB300 CCSD engine.

helios's ``getPolarizability`` (src/modules/mod_property.f90:405-506) solves
the method at field points p = -(n-1)/2 .. (n-1)/2 along one axis, with the
diagonal perturbation ``perturbation(mu,mu) = p * derive-step * x_mu``
(``setCore`` :467-486; x re-centred on the centroid), and
``showPolarizability`` (src/calculation/showPolarizability.f90:47-51,90-96)
turns the energies into ``alpha = deLagDeriv(n, 'xx') * (-E_h / a0^2)``, the
second derivative of the Lagrange interpolating polynomial through the
points (src/modules/mod_math.f90:505-568) divided by ``derive-step^2``.

Here the field points are one batch of the engine (the field enters as site
energies: alpha_mu + p h x_mu is exactly core + perturbation), so the n
solves share every launch. Perturbed points can start from the zero-field
amplitudes (``seed=True``): their orbitals are first matched to the
zero-field ones by sign, and the amplitudes are transformed accordingly.
"""
from __future__ import annotations

import math
from dataclasses import replace

import numpy as np

from . import api
from .molecules import Molecule

BOHR_RADIUS = 0.52917721067     # Angstrom (src/modules/mod_helios.f90:42)
HARTREE_ENERGY = 27.21138602    # eV       (src/modules/mod_helios.f90:43)
AU_FIELD = HARTREE_ENERGY / BOHR_RADIUS   # V/Angstrom per atomic unit of field


def lagrange_weights(npoints: int, order: int) -> np.ndarray:
    """Weights w_p with f^(order)(0) ~ sum_p w_p f(p) on the integer grid -(n-1)/2..(n-1)/2.

    Derived from the Lagrange interpolating polynomial through the points:
    the weights are the unique solution of sum_p w_p p^q = order! delta_{q,order}
    for q = 0..n-1 (exact for polynomials of degree < n).
    """
    if npoints % 2 == 0 or npoints < order + 1:
        raise ValueError("need an odd number of points > derivative order")
    half = (npoints - 1) // 2
    pts = np.arange(-half, half + 1, dtype=np.float64)
    V = np.vander(pts, npoints, increasing=True).T        # V[q, p] = p^q
    rhs = np.zeros(npoints)
    rhs[order] = math.factorial(order)
    return np.linalg.solve(V, rhs)


def alpha_from_energies(energies, step: float) -> float:
    """alpha (a.u.) from total energies (eV) at fields p*step (V/Angstrom), p centred."""
    e = np.asarray(energies, dtype=np.float64)
    w = lagrange_weights(len(e), 2)
    d2 = float(w @ e) / step ** 2
    return d2 * (-HARTREE_ENERGY / BOHR_RADIUS ** 2)


def field_molecule(mol: Molecule, strength: float, axis: int = 0) -> Molecule:
    """The molecule with the diagonal field perturbation folded into its site energies."""
    c = np.asarray(mol.coords, dtype=np.float64)
    x = c[:, axis] - c[:, axis].mean()
    return replace(mol, alpha=np.asarray(mol.alpha, dtype=np.float64) + strength * x,
                   name=f"{mol.name}@F{strength:+.6g}")


def _align(C_ref, C):
    """Signs s_p with s_p C[:, p] closest to C_ref[:, p]."""
    s = np.sign(np.einsum("mp,mp->p", C_ref, C))
    s[s == 0] = 1.0
    return s


def polarizability(mol: Molecule, keywords: api.Keywords | None = None, points: int = 5,
                   step: float = 0.02, axis: int = 0, seed: bool = True):
    """alpha_axis,axis of one molecule; returns dict(alpha, energies, iterations, status)."""
    kw = keywords or api.Keywords()
    half = (points - 1) // 2
    ps = list(range(-half, half + 1))
    mols = [field_molecule(mol, p * step, axis) for p in ps]
    if not seed:
        cc = api.CoupledCluster(mols, kw)
        cc.initCC()
        out = cc.solve_batch()
        cc.finalizeCC()
        energies = out["energy"][:, 0]
        return {"alpha": alpha_from_energies(energies, step), "energies": energies,
                "iterations": out["iterations"], "status": out["status"], "points": ps}
    # zero field first, then the others seeded from its amplitudes
    c0 = api.CoupledCluster(mols[half], kw)
    c0.initCC()
    r0 = c0.iterate()
    t1, t2 = c0.amplitudes(0)
    C0 = c0.scf(0)["C"]
    c0.finalizeCC()
    rest = [m for k, m in enumerate(mols) if k != half]
    cc = api.CoupledCluster(rest, kw)
    cc.initCC()
    o = t1.shape[0]
    for k in range(len(rest)):
        s = _align(C0, cc.scf(k)["C"])
        so, sv = s[:o], s[o:]
        a1 = t1 * so[:, None] * sv[None, :]
        a2 = t2 * so[:, None, None, None] * so[None, :, None, None] * sv[None, None, :, None] * sv[None, None, None, :]
        cc.set_guess(k, a1, a2)
    out = cc.solve_batch()
    cc.finalizeCC()
    energies = np.insert(out["energy"][:, 0], half, r0["energy"][0])
    iters = np.insert(out["iterations"], half, r0["iterations"])
    status = np.insert(out["status"], half, r0["status"])
    return {"alpha": alpha_from_energies(energies, step), "energies": energies, "iterations": iters,
            "status": status, "points": ps}
