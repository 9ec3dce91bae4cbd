"""The mixed-precision ensemble (many PPP molecules of 8-64 sites in one batch) against FP64.

The batched mixed path is where the molecule-size-dependent parts of the
engine live: the MO-basis ladder of molecules with at most 32 virtual
orbitals, the per-molecule phase masks and DIIS gates of a batch whose members
switch precision at different iterations, and the learned guess. Every member
must reach the FP64 path's energy to 1e-6 eV, and the members small enough for
the literal restatement of the reference (oracle/literal.py) its energy to
1e-8 eV.
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


@pytest.fixture(scope="module")
def members():
    from helios_gb300 import learned
    # 48 held-out members: 8..62 sites, both kinds, five of at most 14 sites
    return molecules.ensemble(learned.HELD_OUT_SEED, 48)


def _solve(api, mols, **kw):
    base = dict(bond_alternation=0.1, accuracy=10)
    base.update(kw)
    cc = api.CoupledCluster(mols, api.Keywords(**base))
    cc.initCC()
    out = cc.solve_batch()
    cc.finalizeCC()
    return out


@pytest.fixture(scope="module")
def fp64(api, members):
    out = _solve(api, members)
    assert list(out["status"]) == [1] * len(members)
    return out


@pytest.mark.parametrize("guess", ["reference", "learned"])
def test_mixed_ensemble_matches_fp64(api, members, fp64, guess):
    from oracle.literal import solve_literal
    mx = _solve(api, members, precision="mixed", guess=guess)
    assert list(mx["status"]) == [1] * len(members)
    dE = np.abs(mx["energy"][:, 0] - fp64["energy"][:, 0])
    assert dE.max() <= 1e-6, f"worst member {int(dE.argmax())}: {dE.max():.3e} eV"
    # same reference energies: the SCF does not depend on the precision mode
    assert np.abs(mx["energy"][:, 1] - fp64["energy"][:, 1]).max() < 1e-9
    small = [k for k, m in enumerate(members) if m.n_sites <= 14]
    assert len(small) >= 3
    for k in small:
        ref = solve_literal(members[k], alternation=0.1, eps=1e-10)
        assert ref["status"] == 1
        assert abs((mx["energy"][k, 0] - mx["energy"][k, 1]) - ref["ecorr"]) <= 1e-8
