"""Finite-field electric properties on the GB300 CCSD engine: the polarizability job.

helios's ``getPolarizability`` (src/modules/mod_property.f90:405-506) solves
the method at every point of a field grid, ``showPolarizability``
(src/calculation/showPolarizability.f90) turns the grid energies into the
dipole moment, polarizability and first and second hyperpolarizabilities, and
the harvester (src/modules/mod_harvester.f90:18-159) appends them to a binary
record file. This module is that job for the engine:

* ``field_points``: the grid of ``symmertySettings.f90:30-140`` -- a line for
  one axis ("x"), the full plane for two ("xy"), the three coordinate planes
  for "xyz" (points with all three indices non-zero are never needed);
* ``energy_grid``: every grid point is one molecule of ONE engine batch (the
  field enters as site energies, ``setCore`` :467-486), the non-zero points
  seeded from the zero-field amplitudes;
* ``grid_derivative``: ``deLagDeriv`` (src/modules/mod_derivative.f90:41-125),
  nested Lagrange derivatives over the central k x k (x k) sub-grid, zero when
  the total order exceeds k - 1;
* ``show_polarizability``: the components and averages of
  ``showPolarizability`` for every odd stencil size 3..Np (hyperpolarizabilities
  from 5), in its units, with its thresholds (``purifyValues``) and the text
  report laid out like its output;
* ``harvester_record`` / ``store_harvester``: the ``hpolariz`` record.

The least-squares inset of showPolarizability (``lsmInterpolation``) runs only
in the reference's quadruple-precision build and is not provided.
"""
from __future__ import annotations

import datetime
import os
import struct
from dataclasses import dataclass, field, replace

import numpy as np

from . import api
from .molecules import Molecule
from .polariz import BOHR_RADIUS, HARTREE_ENERGY, _align, lagrange_weights

DIPOLE_TO_DEBYE = 4.8031          # src/modules/mod_helios.f90:50 (e*Angstrom -> Debye)
GAMMA_TO_ESU = 5.036238e-4        # src/modules/mod_helios.f90:51 (times 1e-36)
SIGMA_BOND_ALPHA = 3.48           # au per C-C and C-H bond (showPolarizability.f90:17)
CC_SIGMA_BOND_GAMMA = 220.0       # au per C-C bond
CH_SIGMA_BOND_GAMMA = 240.0       # au per C-H bond
DERIV_THRESHOLD = (0.001, 0.01, 0.1, 1.0)   # purifyValues thresholds: dipole, alpha, beta, gamma
AXES = "xyz"
HARVEST_VERSION = "1.000"
SYMMETRY_THRESHOLD = 1e-10        # geometry:symmetry-threshold (definebd.f90:66, 10 -> 10^-10)


def transition(order: int) -> float:
    """Unit factor of the order-th field derivative of E (eV, V/Angstrom): Debye, then au."""
    if order == 0:
        return 1.0
    if order == 1:
        return -DIPOLE_TO_DEBYE
    return -HARTREE_ENERGY ** (order - 1) / BOHR_RADIUS ** order


def scale_axes(scales: str) -> list[int]:
    s = scales.lower()
    if s not in ("x", "y", "z", "xy", "yx", "xz", "zx", "yz", "zy", "xyz"):
        raise ValueError(f"polarizability scales {scales!r}: one of x, y, z, xy, xz, yz, xyz")
    return sorted(AXES.index(c) for c in s)


def field_points(scales: str, npoints: int) -> list[tuple[int, int, int]]:
    """Grid points (px, py, pz) to solve, the zero point first."""
    if npoints < 1 or npoints % 2 == 0:
        raise ValueError("the number of points must be odd")
    axes = scale_axes(scales)
    half = (npoints - 1) // 2
    rng = range(-half, half + 1)
    pts = [(0, 0, 0)]
    if len(axes) == 1:
        for i in rng:
            if i:
                p = [0, 0, 0]; p[axes[0]] = i; pts.append(tuple(p))
    elif len(axes) == 2:
        for i in rng:
            for j in rng:
                if i or j:
                    p = [0, 0, 0]; p[axes[0]] = i; p[axes[1]] = j; pts.append(tuple(p))
    else:
        for i in rng:
            for j in rng:
                for k in rng:
                    if (i and j and k) or not (i or j or k):
                        continue
                    pts.append((i, j, k))
    return pts


def field_molecule(mol: Molecule, fvec) -> Molecule:
    """The molecule with F . r (coordinates re-centred on their centroid) added to its site energies."""
    c = np.asarray(mol.coords, dtype=np.float64)
    c = c - c.mean(axis=0)
    shift = c @ np.asarray(fvec, dtype=np.float64)
    return replace(mol, alpha=np.asarray(mol.alpha, dtype=np.float64) + shift,
                   name=f"{mol.name}@F({fvec[0]:+.6g},{fvec[1]:+.6g},{fvec[2]:+.6g})")


@dataclass
class EnergyGrid:
    npoints: int
    step: float                                  # V/Angstrom per grid unit (derive-step)
    scales: str
    energies: dict = field(default_factory=dict)  # (px, py, pz) -> E_total (eV)
    iterations: dict = field(default_factory=dict)
    status: dict = field(default_factory=dict)

    def cube(self) -> np.ndarray:
        """E on the full (Np)^3 cube indexed [px+h, py+h, pz+h]; points not solved are 0."""
        h = (self.npoints - 1) // 2
        out = np.zeros((self.npoints,) * 3)
        for (i, j, k), e in self.energies.items():
            out[i + h, j + h, k + h] = e
        return out


def energy_grid(mol: Molecule, keywords: api.Keywords | None = None, scales: str = "x", npoints: int = 5,
                step: float = 0.02, seed: bool = True) -> EnergyGrid:
    """Solve every point of the grid in one batch of the engine."""
    kw = keywords or api.Keywords()
    pts = field_points(scales, npoints)
    mols = [field_molecule(mol, [p * step for p in pt]) for pt in pts]
    grid = EnergyGrid(npoints, step, scales)
    if not seed or len(pts) == 1:
        cc = api.CoupledCluster(mols, kw)
        cc.initCC()
        out = cc.solve_batch()
        cc.finalizeCC()
        energies, iters, status = out["energy"][:, 0], out["iterations"], out["status"]
    else:
        c0 = api.CoupledCluster(mols[0], kw)
        c0.initCC()
        r0 = c0.iterate()
        t1, t2 = c0.amplitudes(0)
        C0 = c0.scf(0)["C"]
        c0.finalizeCC()
        cc = api.CoupledCluster(mols[1:], kw)
        cc.initCC()
        o = t1.shape[0]
        for k in range(len(mols) - 1):
            s = _align(C0, cc.scf(k)["C"])
            so, sv = s[:o], s[o:]
            cc.set_guess(k, t1 * so[:, None] * sv[None, :],
                         t2 * so[:, None, None, None] * so[None, :, None, None] * sv[None, None, :, None]
                         * sv[None, None, None, :])
        out = cc.solve_batch()
        cc.finalizeCC()
        energies = np.concatenate([[r0["energy"][0]], out["energy"][:, 0]])
        iters = np.concatenate([[r0["iterations"]], out["iterations"]])
        status = np.concatenate([[r0["status"]], out["status"]])
    for pt, e, it, st in zip(pts, energies, iters, status):
        grid.energies[pt] = float(e)
        grid.iterations[pt] = int(it)
        grid.status[pt] = int(st)
    return grid


def lagrange_derivative(values, order: int, step: float) -> float:
    """order-th derivative at 0 of the Lagrange polynomial through values on the centred grid."""
    v = np.asarray(values, dtype=np.float64)
    if order == 0:
        return float(v[(len(v) - 1) // 2])
    if order > len(v) - 1:
        return 0.0
    return float(lagrange_weights(len(v), order) @ v) / step ** order


def grid_derivative(cube: np.ndarray, npoints: int, component: str, step: float) -> float:
    """deLagDeriv: d^|component| E / dF_a dF_b ... from the central npoints sub-grid of cube."""
    counts = [component.lower().count(c) for c in AXES]
    if sum(counts) > npoints - 1:
        return 0.0
    full = cube.shape[0]
    lo = (full - npoints) // 2
    sub = cube[lo:lo + npoints, lo:lo + npoints, lo:lo + npoints]
    c = (npoints - 1) // 2
    idx = [slice(None) if counts[a] else c for a in range(3)]
    arr = sub[tuple(idx)]                               # the present axes only, in x, y, z order
    present = [counts[a] for a in range(3) if counts[a]]
    # innermost axis first, as deLagDeriv nests them
    for order in reversed(present):
        arr = np.apply_along_axis(lambda col: lagrange_derivative(col, order, step), -1, arr)
    return float(arr)


def _purify(threshold: float, *vals):
    return [0.0 if abs(v) < threshold else v for v in vals]


def bond_counts(mol: Molecule) -> tuple[int, int]:
    """(unique C-C bonds, C-H bonds) as readMoleculeInformation.f90:313-371 counts them."""
    c = np.asarray(mol.coords, dtype=np.float64)
    N = len(c)
    unique = np.ones(N, dtype=bool)
    for i in range(N - 1):
        for j in range(i + 1, N):
            if np.all(np.abs(c[i] - c[j]) < SYMMETRY_THRESHOLD):
                unique[j] = False
    na = int(unique.sum())
    connect = np.asarray(mol.nels, dtype=np.int64).copy()
    nbcc = len(mol.bonds)
    for b in mol.bonds:
        i, j = b[0], b[1]
        if not (unique[i] and unique[j]):
            nbcc -= 1
        else:
            connect[i] += 1
            connect[j] += 1
    nbch = int(sum(4 - connect[i] for i in range(N) if unique[i])) - (N - na)
    return nbcc, nbch


def show_polarizability(grid: EnergyGrid, mol: Molecule, method: str = "r-ccsd", state: int = 0):
    """Components per stencil size and the text report; returns (results, report, harvest)."""
    np_ = grid.npoints
    h = grid.step
    cube = grid.cube()
    axes = scale_axes(grid.scales)
    names = [AXES[a] for a in axes]
    nel = int(np.sum(mol.nels))
    nat = mol.n_sites
    nbcc, nbch = bond_counts(mol)
    sig_a = SIGMA_BOND_ALPHA * (nbcc + nbch)
    sig_g = CC_SIGMA_BOND_GAMMA * nbcc + CH_SIGMA_BOND_GAMMA * nbch
    esu = GAMMA_TO_ESU * 1e-36
    P = [transition(k) for k in range(5)]

    def d(k, comp):
        return grid_derivative(cube, k, comp, h)

    harvest = {"m": np.zeros(4), "a": np.zeros(4), "b": np.zeros(10), "g": np.zeros(10),
               "sigma_alpha": sig_a, "sigma_gamma": sig_g}
    res = {"stencils": {}, "sigma_alpha": sig_a, "sigma_gamma": sig_g}
    lines = []
    title = f" Polarizability results for {method} " + (f"State #{state} " if state else "")
    lines += ["", title.center(100, "#"), ""]
    hp = (np_ - 1) // 2
    if len(axes) == 1:
        a = names[0]
        for i in range(-hp, hp + 1):
            pt = [0, 0, 0]; pt[axes[0]] = i
            lines.append(f"    Field {i:2d} {grid.energies[tuple(pt)]:25.16f}")
        lines += ["", "", "", f"    ~~~~~~~~~~ Axis {a.upper()} ~~~~~~~~~~", ""]
        ks = list(range(3, np_ + 1, 2))
        lines.append("  " + " " * 24 + "".join(f"      {k:2d} points" for k in ks))
        dip = [d(k, a) * P[1] for k in ks]
        pol = [d(k, a * 2) * P[2] for k in ks]
        b1 = [d(k, a * 3) * P[3] for k in ks if k >= 5]
        g2 = [d(k, a * 4) * P[4] for k in ks if k >= 5]
        fmt = lambda xs: "".join(f" {x:14.7E}" for x in xs)
        lines.append("  Dipole moment           deby" + fmt(dip))
        lines.append("  Polarizability          au  " + fmt(pol))
        lines.append("  1st hyperpolarizability au   " + " " * 14 + fmt(b1))
        lines.append("  2nd hyperpolarizability au   " + " " * 14 + fmt(g2))
        lines.append("  2nd hyperpolarizability esu  " + " " * 14 + fmt([g * esu for g in g2]))
        for n, k in enumerate(ks):
            res["stencils"][k] = {"dipole": {a: dip[n]}, "alpha": {a * 2: pol[n]}}
            if k >= 5:
                res["stencils"][k].update({"beta": {a * 3: b1[n - 1]}, "gamma": {a * 4: g2[n - 1]}})
        aNp = d(np_, a * 2) * P[2]
        lines += ["", f"         Average polarizability                = {aNp / 3:13.4f} au",
                  f"Specific average polarizability (per electron) = {aNp / (3 * nel):13.4f} au"]
        i = axes[0]
        harvest["m"][i] = d(np_, a) * P[1]
        harvest["a"][i] = aNp
        if np_ > 3:
            gNp = d(np_, a * 4) * P[4]
            if nat != nel:
                lines.append(f"Specific average polarizability (per atom)     = {aNp / (3 * nat):13.4f} au")
            lines += ["", f"  Sigma contribution to average polarizability = {sig_a:11.2f}",
                      f"  {SIGMA_BOND_ALPHA:5.3f} au per C-C and C-H bonds [1]",
                      "", f"         Average 2nd hyperpolarizability                = {gNp / 5:14.7E} au",
                      f"Specific average 2nd hyperpolarizability (per electron) = {gNp / (5 * nel):14.7E} au"]
            if nat != nel:
                lines.append(f"Specific average 2nd hyperpolarizability (per atom)     = {gNp / (5 * nat):14.7E} au")
            lines += ["", f"  Sigma contribution to average 2nd hyperpolarizability = {sig_g:10.3E}",
                      f"  {CC_SIGMA_BOND_GAMMA:5.0f} au per C-C bond [2]", f"  {CH_SIGMA_BOND_GAMMA:5.0f} au per C-H bond [2]"]
            harvest["b"][i] = d(np_, a * 3) * P[3]
            harvest["g"][i] = gNp
    else:
        res.update(_multi_axis(grid, cube, axes, names, P, nel, nat, sig_a, sig_g, esu, lines, harvest, d))
    if np_ >= 3:
        lines += ["", "  ________________________________________________________",
                  "  [1] Yu.B. Visotski and B.C. Briantsev, Quantum Chemistry",
                  "      of Radicals and Ion-Radicals with Conjugated Bonds",
                  "      (Donetsk, DonGuet, 2004), p. 207, in Russian."]
    if np_ >= 5:
        lines.append("  [2] B.M. Pierce, J. Chem. Phys. 91, 791 (1989).")
    lines += ["", "#" * 100]
    return res, "\n".join(lines) + "\n", harvest


def _cont(arr):
    a = np.abs(np.asarray(arr, dtype=np.float64))
    return 100.0 * a.max() / a.sum() if a.sum() else 0.0


# harvester slots of the two-axis components (showPolarizability.f90:238-290)
_HARV2 = {"xy": ((0, 1), (3, 4)), "xz": ((0, 2), (5, 6)), "yz": ((1, 2), (7, 8))}


def _multi_axis(grid, cube, axes, names, P, nel, nat, sig_a, sig_g, esu, lines, harvest, d):
    np_ = grid.npoints
    hp = (np_ - 1) // 2
    res = {"stencils": {}}
    three = len(axes) == 3
    if not three:
        for i in range(-hp, hp + 1):
            for j in range(-hp, hp + 1):
                pt = [0, 0, 0]; pt[axes[0]] = i; pt[axes[1]] = j
                lines.append(f"    Field {i:2d} {j:2d} {grid.energies[tuple(pt)]:25.16f}")
            lines.append("")
    else:
        for k in range(-hp, hp + 1):
            for i in range(-hp, hp + 1):
                for j in range(-hp, hp + 1):
                    if i and j and k:
                        continue
                    lines.append(f"    Field {i:2d} {j:2d} {k:2d} {grid.energies[(i, j, k)]:25.16f}")
        lines += ["", "    ~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~", ""]
    ax = names
    if three:
        beta_c = ["xxx", "yyy", "zzz", "xyy", "yxx", "xzz", "zxx", "yzz", "zyy"]
        gamma_c = ["xxxx", "yyyy", "zzzz", "xxyy", "yyxx", "xxzz", "zzxx", "yyzz", "zzyy"]
    else:
        x, y = ax
        beta_c = [x * 3, y * 3, x + y * 2, y + x * 2]
        gamma_c = [x * 4, y * 4, x * 2 + y * 2, y * 2 + x * 2]
    last = {}
    if np_ >= 3:
        lines += ["", "       Dipole moment (deby)", ""]
        for k in range(3, np_ + 1, 2):
            dm = [d(k, a) * P[1] for a in ax]
            mod = float(np.sqrt(sum(v * v for v in dm)))
            vals = _purify(DERIV_THRESHOLD[0], *dm, mod)
            res["stencils"].setdefault(k, {})["dipole"] = dict(zip(ax, vals[:-1])) | {"|D|": vals[-1]}
            lines.append(f"  {k:2d} points   " + "    ".join(f"{a.upper()} = {v:7.3f}" for a, v in zip(ax, vals))
                         + f"    |D| = {vals[-1]:7.3f}")
            last["m"] = vals
        lines += ["", "       Polarizability (au)", ""]
        for k in range(3, np_ + 1, 2):
            al = [d(k, a * 2) * P[2] for a in ax]
            vals = _purify(DERIV_THRESHOLD[1], *al, sum(al) / 3)
            res["stencils"][k]["alpha"] = dict(zip([a * 2 for a in ax], vals[:-1])) | {"<A>": vals[-1]}
            lines.append(f"  {k:2d} points  " + "  ".join(f"{(a * 2).upper()} = {v:14.7E}" for a, v in zip(ax, vals))
                         + f"  <A> = {vals[-1]:14.7E}")
            last["a"] = vals
        avA = last["a"][-1]
        if nel != nat:
            lines.append(f"\n  Specific average polarizability (per atom)     = {avA / nat:14.7E} au")
        lines += [f"\n  Specific average polarizability (per electron) = {avA / nel:14.7E} au",
                  f"  Contribution of general component =   {_cont(last['a'][:-1]):6.2f}%",
                  "", f"  Sigma contribution to average polarizability = {sig_a:11.2f}",
                  f"  {SIGMA_BOND_ALPHA:5.3f} au per C-C and C-H bonds [1]"]
    if np_ >= 5:
        lines += ["", "", "       1st hyperpolarizability (au)"]
        for k in range(5, np_ + 1, 2):
            bs = [d(k, c) * P[3] for c in beta_c]
            if three:
                bx, by, bz, bxyy, byxx, bxzz, bzxx, byzz, bzyy = bs
                mod = float(np.sqrt((bx + bxyy + bxzz) ** 2 + (by + byxx + byzz) ** 2 + (bz + bzxx + bzyy) ** 2))
            else:
                bx, by, bxyy, byxx = bs
                mod = float(np.sqrt((bx + bxyy) ** 2 + (by + byxx) ** 2))
            vals = _purify(DERIV_THRESHOLD[2], *bs, mod)
            res["stencils"][k]["beta"] = dict(zip(beta_c, vals[:-1])) | {"|B|": vals[-1]}
            lines.append(f"\n  {k:2d} points  " + "   ".join(f"{c.upper()} = {v:14.7E}" for c, v in zip(beta_c, vals[:-1]))
                         + f"   |B| = {vals[-1]:14.7E}")
            last["b"] = vals
        lines += ["", "", "       2nd hyperpolarizability (au)"]
        for k in range(5, np_ + 1, 2):
            gs = [d(k, c) * P[4] for c in gamma_c]
            vals = _purify(DERIV_THRESHOLD[3], *gs, sum(gs) / 5)
            res["stencils"][k]["gamma"] = dict(zip(gamma_c, vals[:-1])) | {"<G>": vals[-1]}
            lines.append(f"\n  {k:2d} points  " + "     ".join(f"{c.upper()} = {v:14.7E}" for c, v in zip(gamma_c, vals[:-1]))
                         + f"\n               <G> = {vals[-1]:14.7E}          = {vals[-1] * esu:14.7E} esu")
            last["g"] = vals
        avG = last["g"][-1]
        if nel != nat:
            lines.append(f"\n  Specific average 2nd hyperpolarizability (per atom)     =         {avG / nat:14.7E} au")
        lines += [f"\n  Specific average 2nd hyperpolarizability (per electron) =         {avG / nel:14.7E} au",
                  f"  Contribution of general component =   {_cont(last['g'][:-1]):6.2f}%",
                  "", f"  Sigma contribution to average 2nd hyperpolarizability = {sig_g:10.3E}",
                  f"  {CC_SIGMA_BOND_GAMMA:5.0f} au per C-C bond [2]", f"  {CH_SIGMA_BOND_GAMMA:5.0f} au per C-H bond [2]"]
    # harvester: the full stencil's values
    if "m" in last:
        m, a = last["m"], last["a"]
        if three:
            harvest["m"][:] = m
            harvest["a"][:] = a
        else:
            (i, j), _ = _HARV2[grid.scales.lower() if grid.scales.lower() in _HARV2 else grid.scales.lower()[::-1]]
            harvest["m"][i], harvest["m"][j], harvest["m"][3] = m
            harvest["a"][i], harvest["a"][j], harvest["a"][3] = a
    if "b" in last:
        b, g = last["b"], last["g"]
        if three:
            harvest["b"][:] = b
            harvest["g"][:] = g
        else:
            key = grid.scales.lower() if grid.scales.lower() in _HARV2 else grid.scales.lower()[::-1]
            (i, j), (p, q) = _HARV2[key]
            harvest["b"][[i, j, p, q, 9]] = b
            harvest["g"][[i, j, p, q, 9]] = g
    return res


def _fixed(text: str, n: int) -> bytes:
    return text.encode("ascii", "replace")[:n].ljust(n, b" ")


def harvester_record(grid: EnergyGrid, mol: Molecule, harvest: dict, method: str = "r-ccsd", state: int = 0,
                     date: str | None = None) -> bytes:
    """One hpolariz record as store_harvester_polariz writes it (stream, native little-endian)."""
    np_ = grid.npoints
    energies = grid.cube()
    date = date or datetime.datetime.now().strftime("%Y-%m-%d %H:%M:%S")
    body = b"".join([
        _fixed(date, 25), _fixed(HARVEST_VERSION, 10),
        _fixed(method, 15), struct.pack("<iii", state, mol.n_sites, int(np.sum(mol.nels))),
        _fixed(grid.scales, 3), struct.pack("<i", np_), struct.pack("<d", grid.step),
        np.asarray(energies, dtype="<f8").tobytes(order="F"),       # Energies(sta:sto, sta:sto, sta:sto)
        np.asarray(harvest["m"], dtype="<f8").tobytes(), np.asarray(harvest["a"], dtype="<f8").tobytes(),
        np.asarray(harvest["b"], dtype="<f8").tobytes(), np.asarray(harvest["g"], dtype="<f8").tobytes(),
        struct.pack("<dd", harvest["sigma_alpha"], harvest["sigma_gamma"]),
    ])
    ln = 25 + 10 + 15 + 4 * 4 + 3 + 3 * 8 + energies.size * 8 + (4 + 4 + 10 + 10) * 8
    assert ln == len(body)
    return struct.pack("<ii", 100, ln) + body


def store_harvester(path: str, record: bytes) -> None:
    """Append a record; a new file starts with the 3-byte tag 'hrv'."""
    new = not os.path.exists(path) or os.path.getsize(path) == 0
    with open(path, "ab") as f:
        if new:
            f.write(b"hrv")
        f.write(record)


def read_harvester(path: str) -> list[dict]:
    """Records of a harvester file (for tools and tests)."""
    data = open(path, "rb").read()
    if data[:3] != b"hrv":
        raise ValueError("not a harvester file")
    pos, out = 3, []
    while pos < len(data):
        kind, ln = struct.unpack_from("<ii", data, pos)
        pos += 8
        b = data[pos:pos + ln]
        pos += ln
        rec = {"kind": kind, "date": b[:25].decode().strip(), "version": b[25:35].decode().strip(),
               "method": b[35:50].decode().strip()}
        rec["state"], rec["n_atoms"], rec["n_electrons"] = struct.unpack_from("<iii", b, 50)
        rec["scales"] = b[62:65].decode().strip()
        (rec["points"],) = struct.unpack_from("<i", b, 65)
        (rec["field"],) = struct.unpack_from("<d", b, 69)
        n = rec["points"]
        off = 77
        rec["energies"] = np.frombuffer(b, dtype="<f8", count=n ** 3, offset=off).reshape((n, n, n), order="F")
        off += 8 * n ** 3
        for key, cnt in (("m", 4), ("a", 4), ("b", 10), ("g", 10), ("sigma", 2)):
            rec[key] = np.frombuffer(b, dtype="<f8", count=cnt, offset=off).copy()
            off += 8 * cnt
        out.append(rec)
    return out


def state_energy_grids(mol: Molecule, keywords: api.Keywords | None = None, lr=None, scales: str = "x",
                       npoints: int = 5, step: float = 0.02, solver: str = "reference", engine=None):
    """getPolarizability with excited states (mod_property.f90:426-443): at every grid point the
    r-ccsd ground state and its LR-CCSD states (getEnergy(method, nStates)), one grid per state
    0..nStates. With linear-response:store-solution (the default) each point starts from the
    previous point's states (dumpSolution / loadSolution, mod_lrccsd.f90:593-734), so a state
    keeps its identity along the grid; the points run one after another for that reason."""
    from . import lrccsd
    kw = keywords or api.Keywords()
    n = lr.excited_states_number
    grids = [EnergyGrid(npoints, step, scales) for _ in range(n + 1)]
    seeds = seed_C = None
    for pt in field_points(scales, npoints):
        r = lrccsd.linear_response(field_molecule(mol, [p * step for p in pt]), kw, lr, seeds=seeds,
                                   seed_orbitals=seed_C, engine=engine, solver=solver)
        grids[0].energies[pt] = r["energy"]
        grids[0].iterations[pt], grids[0].status[pt] = r["ccsd_iterations"], r["ccsd_status"]
        for k in range(n):
            grids[k + 1].energies[pt] = float(r["E_total"][k])
            grids[k + 1].iterations[pt], grids[k + 1].status[pt] = int(r["iterations"][k]), int(r["status"][k])
        if lr.store_solution:
            seeds, seed_C = lrccsd.stored_seeds(r, lr), r["scf"]["C"]
    return grids


def polarizability_job(mol: Molecule, keywords: api.Keywords | None = None, scales: str = "x", npoints: int = 5,
                       step: float = 0.02, seed: bool = True, harvest_file: str | None = None,
                       method: str = "r-ccsd", lr=None, lr_solver: str = "reference", engine=None):
    """getPolarizability + showPolarizability (+ the harvester) for one molecule.

    With ``lr`` (LRKeywords with excited_states_number > 0) every state 0..n gets its grid, its
    report section ("State #k") and its harvester record; ``res["states"]`` holds the results of
    states 1..n."""
    if lr is not None and lr.excited_states_number > 0:
        grids = state_energy_grids(mol, keywords, lr, scales, npoints, step, lr_solver, engine)
    else:
        grids = [energy_grid(mol, keywords, scales, npoints, step, seed)]
    results, reports = [], []
    for state, grid in enumerate(grids):
        res, report, harvest = show_polarizability(grid, mol, method, state)
        if harvest_file:
            store_harvester(harvest_file, harvester_record(grid, mol, harvest, method, state))
        res["grid"] = grid
        results.append(res)
        reports.append(report)
    out = results[0]
    if len(results) > 1:
        out["states"] = results[1:]
    return out, "\n".join(reports)
