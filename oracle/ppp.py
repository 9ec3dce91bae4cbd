"""ORACLE (test infrastructure only) -- PPP Hamiltonian of a pi-system.

CPU restatement of helios's molecule set-up. Only ``tests/``, the smoke check and
the CPU-baseline leg of ``bench.py`` use this package, and only as the checker.

Follows ``src/input/readMoleculeInformation.f90``:
  * coordinates re-centred on their centroid              (``:381-397``)
  * interatomic distances                                  (``:67-79``)
  * Coulomb integrals gamma (Ohno-Klopman, Mataga-Nishimoto, Hubbard) with
    ``trConst = 1/(BohrRadius*HartreeEnergy)``             (``:216-264``)
  * ``connect``: site energies on the diagonal, beta on bonded pairs, scaled by
    (1-delta) for ``single`` and (1+delta) for ``double`` bonds (``:108-138``)
  * ``core(k,k) = connect(k,k) - sum_{l!=k} nels_l * G(k,l)`` (``:140-159``)
and ``perturbate`` (``src/modules/mod_helios.f90:577-601``):
``core = coreImage + perturbation``, ``huckelCore = connect + perturbation``;
the finite field of ``setCore`` (``src/modules/mod_property.f90:467-486``)
puts ``p * h * x_mu`` on the diagonal of ``perturbation``.
"""
from __future__ import annotations

import numpy as np

# src/modules/mod_helios.f90:42-43 (CODATA 2014 values used by helios)
BOHR_RADIUS = 0.52917721067     # Angstrom
HARTREE_ENERGY = 27.21138602    # eV
TR_CONST = 1.0 / (BOHR_RADIUS * HARTREE_ENERGY)


def centred(coords):
    c = np.asarray(coords, dtype=np.float64)
    return c - c.sum(axis=0) / c.shape[0]


def gamma_matrix(coords, gamma_site, kind="ohno-klopman"):
    """Two-centre Coulomb integrals (readMoleculeInformation.f90:216-264)."""
    c = centred(coords)
    n = c.shape[0]
    d = np.sqrt(((c[:, None, :] - c[None, :, :]) ** 2).sum(-1))
    g = np.zeros((n, n))
    med = (gamma_site[:, None] + gamma_site[None, :]) / 2.0
    if kind == "ohno-klopman":
        g = med / np.sqrt(1.0 + (TR_CONST * med * d) ** 2)
    elif kind == "mataga-nishimoto":
        g = med / (1.0 + TR_CONST * med * d)
    elif kind == "hubbard":
        g[np.diag_indices(n)] = gamma_site
    else:
        raise ValueError(f"unknown coulomb-integrals type {kind!r}")
    return g


def build_model(mol, coulomb="ohno-klopman", alternation=0.0, field=(0.0, 0.0, 0.0)):
    """Return a dict with centred coords, G, connect, coreImage, core, huckelCore.

    ``field`` is the per-axis diagonal perturbation strength (eV per Angstrom),
    i.e. ``p * derive-step`` for polarizability point p, or ``field:along-*``.
    """
    coords = centred(mol.coords)
    n = coords.shape[0]
    G = gamma_matrix(mol.coords, np.asarray(mol.gamma, dtype=np.float64), coulomb)
    connect = np.diag(np.asarray(mol.alpha, dtype=np.float64)).copy()
    for (i, j, beta, kind) in mol.bonds:
        connect[i, j] = connect[j, i] = beta
    if alternation != 0.0:
        for (i, j, beta, kind) in mol.bonds:
            if kind == "single":
                connect[i, j] = connect[j, i] = beta * (1.0 - alternation)
            elif kind == "double":
                connect[i, j] = connect[j, i] = beta * (1.0 + alternation)
            else:
                raise ValueError("bond alternation needs single/double bond labels")
    nels = np.asarray(mol.nels, dtype=np.float64)
    core_image = connect.copy()
    for k in range(n):
        s = 0.0
        for l in range(n):
            if l != k:
                s += nels[l] * G[k, l]
        core_image[k, k] -= s
    pert = np.zeros((n, n))
    for ax in range(3):
        if field[ax] != 0.0:
            pert[np.diag_indices(n)] += field[ax] * coords[:, ax]
    return {
        "n": n,
        "nel": int(nels.sum()),
        "coords": coords,
        "G": G,
        "connect": connect,
        "coreImage": core_image,
        "core": core_image + pert,
        "huckelCore": connect + pert,
        "perturbation": pert,
    }
