"""The polarizability job on the GPU against the oracle (getPolarizability,
mod_property.f90:405-506; showPolarizability.f90; mod_harvester.f90).

Octatetraene on the 5 x 5 "xy" grid: the 25 field points are one engine
batch; every energy must equal the literal oracle's CCSD energy at the same
field, and the dipole, polarizability and hyperpolarizabilities derived from
the two grids must agree. The harvester file written by the job must hold
the same numbers.
"""
import os

import numpy as np
import pytest

from helios_gb300 import molecules, properties as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    from helios_gb300 import build
    build.build()
    from helios_gb300 import api as a
    return a


@pytest.mark.parametrize("precision,seed", [("fp64", False), ("mixed", True)])
def test_xy_grid_matches_the_oracle(api, tmp_path, precision, seed):
    from oracle.literal import solve_literal
    mol = molecules.polyene(8)
    step = 0.05
    kw = api.Keywords(bond_alternation=0.1, accuracy=11, precision=precision)
    path = os.path.join(tmp_path, "octatetraene.hrv")
    res, report = P.polarizability_job(mol, kw, scales="xy", npoints=5, step=step, seed=seed, harvest_file=path)
    grid = res["grid"]
    assert set(grid.status.values()) == {1}
    ref = P.EnergyGrid(5, step, "xy")
    for pt in P.field_points("xy", 5):
        ref.energies[pt] = solve_literal(mol, alternation=0.1, field=tuple(p * step for p in pt),
                                         eps=1e-11)["energy"][0]
    dE = max(abs(grid.energies[p] - ref.energies[p]) for p in ref.energies)
    assert dE < 1e-8, dE
    want, _, _ = P.show_polarizability(ref, mol)
    for k in (3, 5):
        for prop, tol in (("alpha", 1e-6), ("gamma", 1e-3)):
            if prop not in want["stencils"][k]:
                continue
            for comp, v in want["stencils"][k][prop].items():
                got = res["stencils"][k][prop][comp]
                assert got == pytest.approx(v, rel=tol, abs=tol * abs(want["stencils"][k][prop]["xx" if prop == "alpha"
                                                                                             else "xxxx"])), (k, comp)
    rec = P.read_harvester(path)[0]
    assert rec["points"] == 5 and rec["scales"] == "xy" and rec["field"] == step
    assert rec["a"][0] == pytest.approx(res["stencils"][5]["alpha"]["xx"])
    assert np.allclose(rec["energies"], grid.cube())
    assert "Polarizability (au)" in report
