"""Finite-field alpha_xx of the 2 x 32 acene-like ladder (64 sites) on the GPU
against the FP64 oracle (tests/golden/polariz64.json, make_polariz64.py).

Tolerances: the FP64 path reproduces the oracle's alpha to 1e-6 relative (the
energies agree to ~1e-10 eV and alpha is their second difference divided by
a small step squared); the mixed path, seeded from the zero-field amplitudes,
to 1e-4 relative, the accuracy the polarizability is quoted to.
"""
import json
import os

import numpy as np
import pytest

from helios_gb300 import molecules

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "polariz64.json")


@pytest.fixture(scope="module")
def api():
    from helios_gb300 import build
    build.build()
    from helios_gb300 import api as a
    return a


@pytest.mark.skipif(not os.path.exists(GOLD), reason="no oracle fixture")
@pytest.mark.parametrize("precision,seed,tol", [("fp64", False, 1e-6), ("mixed", True, 1e-4)])
def test_ladder64_alpha_matches_oracle(api, precision, seed, tol):
    from helios_gb300 import polariz
    g = json.load(open(GOLD))
    kw = api.Keywords(bond_alternation=0.1, accuracy=10, precision=precision)
    out = polariz.polarizability(molecules.ladder(64), kw, points=5, step=g["step_V_per_A"], seed=seed)
    assert np.all(out["status"] == 1)
    assert np.abs(out["energies"] - np.array(g["energies"])).max() < 1e-7
    assert abs(out["alpha"] - g["alpha_xx"]) <= tol * abs(g["alpha_xx"])
