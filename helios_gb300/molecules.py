"""Synthetic PPP pi-systems: the molecule descriptions the CCSD path is run on.

A molecule is what a helios ``molecule`` input block holds (reference
``src/input/readMoleculeInformation.f90:20-117``): per site a symbol, Cartesian
coordinates in Angstrom, the site energy ``alpha`` (eV), the one-centre
repulsion ``gamma`` (eV) and the number of pi electrons the site donates; per
bond the two sites, the resonance integral ``beta`` (eV) and its Kekule label
(``double``/``single``), which ``parametrization:bond-alternation`` scales by
``1 +/- delta``.

Generators:
  * ``polyene(n)``  -- all-trans zigzag chain in the XY plane, 120 degree angles,
    bonds alternating double/single starting with a double bond.
  * ``ladder(n)``   -- two-row acene-like ladder of ``n`` sites (two zigzag rows
    of ``n/2`` sites joined by rungs at every other column, i.e. fused
    hexagons), with a valid Kekule labelling for any row length.
  * ``random_molecule(seed)`` -- the seeded ensemble used for batched solves:
    polyene or ladder with probability 1/2, ``n`` even and uniform in 8..64,
    bond-length alternation ``delta ~ U(0, 0.1)`` Angstrom about 1.40 Angstrom
    (polyenes), site energies ``alpha_i ~ N(0, 0.5)`` eV.

Every generated molecule is planar in the XY plane, so the reference's
planarity check (``src/input/planarityCheck.f90:151-179``) leaves it untouched.
"""
from __future__ import annotations

from dataclasses import dataclass, field
import math
import numpy as np

HUBBARD_U = 11.13      # eV, one-centre repulsion of a carbon pi site
BETA = -2.4            # eV, nearest-neighbour resonance integral
ALTERNATION = 0.1      # parametrization:bond-alternation used by every workload


@dataclass
class Molecule:
    """One PPP molecule: sites and bonds exactly as a helios input block lists them."""
    name: str
    coords: np.ndarray                 # (n, 3) Angstrom
    alpha: np.ndarray                  # (n,) eV
    gamma: np.ndarray                  # (n,) eV
    nels: np.ndarray                   # (n,) pi electrons per site
    bonds: list = field(default_factory=list)   # (i, j, beta, kind), 0-based sites

    @property
    def n_sites(self) -> int:
        return int(self.coords.shape[0])

    @property
    def n_electrons(self) -> int:
        return int(self.nels.sum())

    def bond_arrays(self):
        """Bonds as flat arrays (i, j, beta, kind) with kind 1=double, 0=single."""
        i = np.array([b[0] for b in self.bonds], dtype=np.int32)
        j = np.array([b[1] for b in self.bonds], dtype=np.int32)
        beta = np.array([b[2] for b in self.bonds], dtype=np.float64)
        kind = np.array([1 if b[3] == "double" else 0 for b in self.bonds], dtype=np.int32)
        return i, j, beta, kind


def _sites(n, alpha=None, gamma=HUBBARD_U):
    a = np.zeros(n) if alpha is None else np.asarray(alpha, dtype=np.float64)
    return a, np.full(n, float(gamma)), np.ones(n, dtype=np.int32)


def polyene(n: int, r_double: float = 1.35, r_single: float = 1.46, alpha=None,
            beta: float = BETA, gamma: float = HUBBARD_U, name: str | None = None) -> Molecule:
    """All-trans zigzag polyene with ``n`` sites; bond k joins sites k and k+1.

    Even-numbered bonds are ``double`` (length ``r_double``), odd ones ``single``.
    Successive bond directions alternate between +30 and -30 degrees from the
    x axis, which gives 120 degree C-C-C angles.
    """
    if n < 2:
        raise ValueError("a polyene needs at least two sites")
    xyz = np.zeros((n, 3))
    bonds = []
    for k in range(n - 1):
        dbl = (k % 2 == 0)
        r = r_double if dbl else r_single
        ang = math.radians(30.0 if k % 2 == 0 else -30.0)
        xyz[k + 1, 0] = xyz[k, 0] + r * math.cos(ang)
        xyz[k + 1, 1] = xyz[k, 1] + r * math.sin(ang)
        bonds.append((k, k + 1, beta, "double" if dbl else "single"))
    a, g, ne = _sites(n, alpha, gamma)
    return Molecule(name or f"polyene-{n}", xyz, a, g, ne, bonds)


def ladder(n: int, r: float = 1.40, alpha=None, beta: float = BETA,
           gamma: float = HUBBARD_U, name: str | None = None) -> Molecule:
    """Two-row acene-like ladder of ``n`` sites (``n`` even, rows of ``m = n/2``).

    Top row site k sits at x = k*r*sqrt(3)/2, y = +r/2 (k even) or +r (k odd);
    the bottom row is its mirror image in y = 0. Rails join neighbours in each
    row, rungs join the two rows at even columns, so every closed cell is a
    hexagon of side ``r``. Kekule labels: with ``m`` even the rail pairs
    (0,1),(2,3),... of both rows are double; with ``m`` odd the first rung and
    the rail pairs (1,2),(3,4),... are double. Everything else is single.
    Sites 0..m-1 are the top row, m..2m-1 the bottom row.
    """
    if n < 4 or n % 2:
        raise ValueError("a ladder needs an even number of sites >= 4")
    m = n // 2
    xyz = np.zeros((n, 3))
    for k in range(m):
        x = k * r * math.sqrt(3.0) / 2.0
        y = r / 2.0 if k % 2 == 0 else r
        xyz[k] = (x, y, 0.0)
        xyz[m + k] = (x, -y, 0.0)
    doubles = set()
    if m % 2 == 0:
        for k in range(0, m - 1, 2):
            doubles.add((k, k + 1)); doubles.add((m + k, m + k + 1))
    else:
        doubles.add((0, m))
        for k in range(1, m - 1, 2):
            doubles.add((k, k + 1)); doubles.add((m + k, m + k + 1))
    bonds = []
    for k in range(m - 1):
        for (i, j) in ((k, k + 1), (m + k, m + k + 1)):
            bonds.append((i, j, beta, "double" if (i, j) in doubles else "single"))
    for k in range(0, m, 2):
        bonds.append((k, m + k, beta, "double" if (k, m + k) in doubles else "single"))
    a, g, ne = _sites(n, alpha, gamma)
    return Molecule(name or f"ladder-2x{m}", xyz, a, g, ne, bonds)


def dodecahexaene() -> Molecule:
    """All-trans dodecahexaene: 12 sites, bonds 1.35/1.46 Angstrom, alpha = 0."""
    return polyene(12, 1.35, 1.46, name="dodecahexaene")


def random_molecule(seed: int, n_min: int = 8, n_max: int = 64) -> Molecule:
    """One member of the seeded random ensemble (see module docstring)."""
    rng = np.random.default_rng(seed)
    kind = "polyene" if rng.random() < 0.5 else "ladder"
    n = 2 * int(rng.integers(n_min // 2, n_max // 2 + 1))
    delta = float(rng.uniform(0.0, 0.1))
    alpha = rng.normal(0.0, 0.5, size=n)
    if kind == "polyene":
        return polyene(n, 1.40 - delta, 1.40 + delta, alpha=alpha, name=f"rnd{seed}-polyene-{n}")
    return ladder(n, 1.40, alpha=alpha, name=f"rnd{seed}-ladder-{n}")


def ensemble(base_seed: int, count: int, n_min: int = 8, n_max: int = 64) -> list[Molecule]:
    """``count`` molecules with seeds ``base_seed + k``."""
    return [random_molecule(base_seed + k, n_min, n_max) for k in range(count)]
