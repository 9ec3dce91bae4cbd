"""ORACLE (test infrastructure only) -- finite-field polarizability of helios.

Restates ``LagrangeDerivative`` (src/modules/mod_math.f90:505-568): the
power-th derivative at 0 of the Lagrange polynomial through the integer grid
-(n-1)/2..(n-1)/2 has weights
  w_j = power! * [x^power] prod_{k != j} (x - k) / prod_{k != j} (j - k),
and ``showPolarizability`` (src/calculation/showPolarizability.f90:47-51,90-96):
alpha = deLagDeriv(n, 'xx') * transition(2), transition(2) = -E_h / a0^2,
deLagDeriv dividing by derive-step^power.
"""
from __future__ import annotations

import math

import numpy as np

from .literal import solve_literal
from .ppp import BOHR_RADIUS, HARTREE_ENERGY


def lagrange_derivative_weights(npoints, power):
    half = (npoints - 1) // 2
    grid = list(range(-half, half + 1))
    w = []
    for j in grid:
        others = [k for k in grid if k != j]
        coeffs = np.poly(others)[::-1]          # ascending powers of prod (x - k)
        denom = np.prod([j - k for k in others])
        w.append(math.factorial(power) * coeffs[power] / denom)
    return np.array(w)


def alpha(energies, step):
    w = lagrange_derivative_weights(len(energies), 2)
    return float(np.dot(w, energies)) / step ** 2 * (-HARTREE_ENERGY / BOHR_RADIUS ** 2)


def polarizability(mol, step=0.02, points=5, alternation=0.1, eps=1e-11):
    half = (points - 1) // 2
    energies = [solve_literal(mol, alternation=alternation, field=(p * step, 0.0, 0.0), eps=eps)["energy"][0]
                for p in range(-half, half + 1)]
    return alpha(energies, step), np.array(energies)
