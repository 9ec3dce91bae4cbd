"""Host logic of the polarizability job (helios_gb300/properties.py), no GPU.

Grids follow symmertySettings.f90:30-140, derivatives deLagDeriv
(mod_derivative.f90:41-125), units and thresholds showPolarizability.f90, and
the record store_harvester_polariz (mod_harvester.f90:110-159). Derivatives
are checked on polynomial energy surfaces (exact for stencils with more points
than the degree) against the oracle's independently built Lagrange weights,
and on oracle CCSD energies of butadiene for the reference's physics
invariants (centrosymmetric: no dipole, no first hyperpolarizability).
"""
import os

import numpy as np
import pytest

from helios_gb300 import molecules, polariz, properties as P
from oracle import polariz as opol


def test_field_points_follow_the_reference_grids():
    assert P.field_points("x", 5) == [(0, 0, 0), (-2, 0, 0), (-1, 0, 0), (1, 0, 0), (2, 0, 0)]
    xy = P.field_points("xy", 5)
    assert len(xy) == 25 and len(set(xy)) == 25 and all(p[2] == 0 for p in xy)
    xyz = P.field_points("xyz", 5)
    assert len(xyz) == 5 ** 3 - 4 ** 3                           # the three coordinate planes
    assert all(0 in p for p in xyz)
    assert P.field_points("z", 3) == [(0, 0, 0), (0, 0, -1), (0, 0, 1)]
    with pytest.raises(ValueError):
        P.field_points("xy", 4)
    with pytest.raises(ValueError):
        P.field_points("w", 5)


@pytest.mark.parametrize("n,order", [(3, 1), (3, 2), (5, 1), (5, 2), (5, 3), (5, 4), (7, 2), (9, 4)])
def test_lagrange_weights_match_the_oracle(n, order):
    assert np.allclose(polariz.lagrange_weights(n, order), opol.lagrange_derivative_weights(n, order),
                       rtol=1e-12, atol=1e-12)


def _poly_grid(scales, npoints, step, coef):
    grid = P.EnergyGrid(npoints, step, scales)
    for pt in P.field_points(scales, npoints):
        F = np.array(pt, dtype=float) * step
        grid.energies[pt] = sum(c * F[0] ** a * F[1] ** b * F[2] ** d for (a, b, d), c in coef.items())
    return grid


COEF = {(0, 0, 0): -50.0, (1, 0, 0): 0.3, (0, 1, 0): -0.2, (0, 0, 1): 0.1, (2, 0, 0): -4.0, (0, 2, 0): -2.5,
        (0, 0, 2): -1.5, (3, 0, 0): 0.7, (0, 3, 0): -0.4, (1, 2, 0): 0.9, (2, 1, 0): -0.6, (1, 0, 2): 0.2,
        (2, 0, 1): 0.35, (0, 1, 2): -0.15, (0, 2, 1): 0.45, (4, 0, 0): -11.0, (0, 4, 0): -6.0, (0, 0, 4): -3.0,
        (2, 2, 0): -1.7, (2, 0, 2): -0.8, (0, 2, 2): -0.9}


@pytest.mark.parametrize("scales", ["x", "xy", "yz", "xyz"])
def test_grid_derivatives_are_exact_on_quartic_surfaces(scales):
    step = 0.05
    grid = _poly_grid(scales, 5, step, COEF)
    cube = grid.cube()
    fact = {0: 1, 1: 1, 2: 2, 3: 6, 4: 24}
    axes = P.scale_axes(scales)
    for comp in ["x", "y", "z", "xx", "yy", "zz", "xxx", "yyy", "xyy", "yxx", "xzz", "zxx", "yzz", "zyy",
                 "xxxx", "yyyy", "zzzz", "xxyy", "xxzz", "yyzz"]:
        cnt = tuple(comp.count(c) for c in "xyz")
        if any(cnt[a] and a not in axes for a in range(3)):
            continue
        want = COEF.get(cnt, 0.0) * np.prod([fact[c] for c in cnt])
        got = P.grid_derivative(cube, 5, comp, step)
        assert got == pytest.approx(want, rel=1e-7, abs=1e-7), comp
    # a 3-point stencil has no third derivative (deLagDeriv returns 0)
    a = "xyz"[axes[0]]
    assert P.grid_derivative(cube, 3, a * 3, step) == 0.0
    two = tuple(2 if k == axes[0] else 0 for k in range(3))
    assert P.grid_derivative(cube, 3, a * 2, step) == pytest.approx(2 * COEF[two], rel=1e-2)


def test_report_units_and_averages():
    step = 0.05
    grid = _poly_grid("xy", 5, step, COEF)
    mol = molecules.polyene(6)
    res, report, harv = P.show_polarizability(grid, mol)
    s5 = res["stencils"][5]
    axx = 2 * COEF[(2, 0, 0)] * P.transition(2)
    ayy = 2 * COEF[(0, 2, 0)] * P.transition(2)
    assert s5["alpha"]["xx"] == pytest.approx(axx, rel=1e-7)
    assert s5["alpha"]["<A>"] == pytest.approx((axx + ayy) / 3, rel=1e-7)
    assert s5["dipole"]["x"] == pytest.approx(COEF[(1, 0, 0)] * P.transition(1), rel=1e-7)
    g = [24 * COEF[(4, 0, 0)], 24 * COEF[(0, 4, 0)], 4 * COEF[(2, 2, 0)], 4 * COEF[(2, 2, 0)]]
    assert s5["gamma"]["<G>"] == pytest.approx(sum(g) * P.transition(4) / 5, rel=1e-6)
    assert harv["a"][3] == pytest.approx(s5["alpha"]["<A>"])
    assert harv["b"][9] == pytest.approx(s5["beta"]["|B|"])
    assert "Polarizability results for r-ccsd" in report and "2nd hyperpolarizability (au)" in report


def test_bond_counts_of_a_polyene():
    for n in (4, 10, 30):
        assert P.bond_counts(molecules.polyene(n)) == (n - 1, n + 2)   # terminal CH2, interior CH


def test_harvester_record_round_trip(tmp_path):
    grid = _poly_grid("xyz", 5, 0.02, COEF)
    mol = molecules.polyene(6)
    res, _, harv = P.show_polarizability(grid, mol)
    path = os.path.join(tmp_path, "run.hrv")
    for _ in range(2):
        P.store_harvester(path, P.harvester_record(grid, mol, harv, date="2026-12-03 12:00:00"))
    data = open(path, "rb").read()
    assert data[:3] == b"hrv" and data.count(b"hrv") == 1
    recs = P.read_harvester(path)
    assert len(recs) == 2
    r = recs[0]
    assert (r["kind"], r["method"], r["scales"], r["points"], r["n_atoms"], r["n_electrons"]) == \
        (100, "r-ccsd", "xyz", 5, 6, 6)
    assert r["field"] == 0.02 and r["version"] == "1.000"
    assert np.array_equal(r["energies"], grid.cube())
    assert np.array_equal(r["a"], harv["a"]) and np.array_equal(r["g"], harv["g"])
    assert np.array_equal(r["sigma"], [harv["sigma_alpha"], harv["sigma_gamma"]])


def test_oracle_energies_of_butadiene_give_the_reference_invariants():
    # literal-oracle CCSD at every point of the xy grid: a centrosymmetric
    # molecule has no dipole and no first hyperpolarizability, and the x-line
    # alpha equals the oracle's own 5-point alpha
    mol = molecules.polyene(4)
    step = 0.05
    grid = P.EnergyGrid(5, step, "xy")
    for pt in P.field_points("xy", 5):
        F = tuple(p * step for p in pt)
        grid.energies[pt] = opol.solve_literal(mol, alternation=0.1, field=F, eps=1e-11)["energy"][0]
    res, report, _ = P.show_polarizability(grid, mol)
    s5 = res["stencils"][5]
    assert s5["dipole"]["|D|"] == 0.0                       # below the 0.001 D threshold
    assert s5["beta"]["|B|"] == 0.0                          # below the 0.1 au threshold
    line = [grid.energies[(p, 0, 0)] for p in range(-2, 3)]
    assert s5["alpha"]["xx"] == pytest.approx(opol.alpha(line, step), rel=1e-10)
    assert s5["alpha"]["xx"] > s5["alpha"]["yy"] > 0                  # along the chain
    assert s5["gamma"]["xxxx"] > 0
