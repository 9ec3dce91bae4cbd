"""Tile autotuner on the GPU: every tile candidate forms the same sums.

The candidates of a precision mode differ only in the output tile width;
slices, slice pairs, exact classes and chunking are the mode's own. So a
mixed-precision solve of one molecule gives the same iterations and, to
rounding, the same residuals and energies whichever candidate runs.
Contractions with a long K and few output tiles are cut into K slices whose
FP64 results are added with atomics; the order of those additions, and so the
last bits, changes from run to run (of one candidate too), and in a batch the
phase switches of the mixed ladder can turn that into a few iterations more
or less. There the converged energies must agree. A handle created with tile_tuning = "tune" must record a valid
choice for every contraction group and reproduce the default energies.
"""
import numpy as np
import pytest

from helios_gb300 import molecules

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    from helios_gb300 import build
    build.build()
    from helios_gb300 import api as a
    return a


def _solve(api, mols, **kw):
    base = dict(bond_alternation=0.1, accuracy=10, precision="mixed")
    base.update(kw)
    cc = api.CoupledCluster(mols, api.Keywords(**base))
    cc.initCC()
    out = cc.solve_batch()
    trace = cc.trace(0)
    choices, ms = cc.tile_choices()
    cc.finalizeCC()
    return out, trace, choices, ms


@pytest.mark.parametrize("mols", [[molecules.polyene(24)], molecules.ensemble(4242, 6)], ids=["polyene-24", "ensemble-6"])
def test_every_tile_candidate_gives_the_same_solve(api, mols):
    ref, tref, ch0, _ = _solve(api, mols, tile_force=0)
    assert list(ref["status"]) == [1] * len(mols)
    assert (ch0 == 0).all()
    ncand = max(len(api.tile_variants(m)) for m in range(4))
    for k in range(1, ncand):
        got, tr, ch, _ = _solve(api, mols, tile_force=k)
        for m in range(4):
            assert (ch[m] == min(k, len(api.tile_variants(m)) - 1)).all()
        assert list(got["status"]) == [1] * len(mols)
        assert np.abs(got["energy"][:, 0] - ref["energy"][:, 0]).max() < 1e-9
        if len(mols) == 1:
            # one molecule: the same iterations, and the residual history to rounding
            assert list(got["iterations"]) == list(ref["iterations"])
            assert tr.shape == tref.shape and np.abs(tr[:, :3] - tref[:, :3]).max() <= 1e-9 * np.abs(tref[:, :3]).max()


def test_tuning_at_creation_records_valid_choices(api):
    mols = molecules.ensemble(4343, 5)
    ref, _, _, _ = _solve(api, mols, tile_tuning="default")
    n_before = len(api.tile_table())
    got, _, ch, ms = _solve(api, mols, tile_tuning="tune")
    assert ms > 0.0 or len(api.tile_table()) == n_before      # timed, or every size class was in the table
    for m in range(4):
        assert ((ch[m] >= 0) & (ch[m] < len(api.tile_variants(m)))).all()
    keys = {(e[0], e[1]) for e in api.tile_table()}
    assert all((m, g) in keys for m in range(4) for g in range(ch.shape[1]) if ch[m, g] != 0)
    assert list(got["status"]) == [1] * len(mols)
    assert np.abs(got["energy"][:, 0] - ref["energy"][:, 0]).max() < 1e-9
