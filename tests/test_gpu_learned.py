"""Learned T2 guess on the GPU: kernels against the CPU oracle, and what the
trained network gains.

Tolerances: the GPU computes in FP32 with the bf16 roundings of the oracle
(oracle/mlp.py, float64); a rounding that lands on the other side of a bf16
boundary moves one activation by 2^-8 of itself, so gradients are compared
by relative Frobenius norm per parameter group (<= 2e-3) and predictions
relative to the largest one (<= 2e-3).
"""
import os

import numpy as np
import pytest

from helios_gb300 import molecules

pytestmark = pytest.mark.gpu

GROUPS = ["W1", "b1", "W2", "b2", "W3", "b3", "w4", "b4"]


@pytest.fixture(scope="module")
def api():
    from helios_gb300 import build
    build.build()
    from helios_gb300 import api as a
    return a


def _rows_of(api, mols, nrows=None, seed=0):
    """Inputs and targets of solved molecules (converged amplitudes)."""
    cc = api.CoupledCluster(mols, api.Keywords(bond_alternation=0.1, accuracy=9))
    cc.initCC()
    out = cc.solve_batch()
    rng = np.random.default_rng(seed)
    Xs, Ts = [], []
    for k in range(len(mols)):
        assert out["status"][k] == 1
        _, o, v, _ = cc.dims[k]
        npairs = (o * v) * (o * v + 1) // 2
        rows = np.arange(npairs) if nrows is None else rng.choice(npairs, min(nrows, npairs), replace=False)
        X, T = cc.training_rows(k, rows)
        Xs.append(X)
        Ts.append(T)
    cc.finalizeCC()
    return np.concatenate(Xs), np.concatenate(Ts)


def _blob(api, X, T, seed=1):
    from helios_gb300 import learned
    P = learned.init_params(X, T, seed)
    # make the output layer non-trivial so that every gradient group is exercised
    rng = np.random.default_rng(seed)
    from oracle import mlp
    p = mlp.unpack(P)
    p["w4"] = rng.normal(size=256) * 0.2
    p["b4"] = np.array([0.05])
    return mlp.pack(p)


def test_training_rows_match_oracle_features(api):
    from oracle import ccsd_fact, mlp
    from oracle.ppp import build_model
    mol = molecules.polyene(10)
    cc = api.CoupledCluster(mol, api.Keywords(bond_alternation=0.1, accuracy=10))
    cc.initCC()
    s = cc.scf(0)
    _, o, v, _ = cc.dims[0]
    ov = o * v
    rows = np.arange(ov * (ov + 1) // 2)
    X, T = cc.training_rows(0, rows)
    # before any iteration t2 is the reference guess: the target is zero
    assert np.abs(T).max() < 1e-7 * np.abs(X[:, 0]).max()
    I = ccsd_fact.Integrals(s["C"], build_model(mol, alternation=0.1)["G"], o)
    gov = I.coulomb("ovov").reshape(ov, ov)                      # (ia|jb), rows i*v + a
    Xr, _ = mlp.features(s["F"], gov, o, rows)
    assert np.allclose(X, Xr, rtol=1e-6, atol=1e-7 * np.abs(Xr).max())
    cc.finalizeCC()


def test_gradients_match_oracle(api):
    from oracle import mlp
    X, T = _rows_of(api, [molecules.random_molecule(s, 8, 20) for s in (101, 102, 103)], nrows=400)
    P = _blob(api, X, T)
    loss, G = api.mlp_grad(P, X, T)
    lr, gr = mlp.loss_and_grads(mlp.unpack(P), X, T)
    assert abs(loss - lr) <= 1e-4 * lr
    g = mlp.unpack(G)
    for name in GROUPS:
        ref = gr[name]
        err = np.linalg.norm(g[name] - ref) / max(np.linalg.norm(ref), 1e-30)
        assert err < 2e-3, (name, err)
    assert np.all(G[mlp.NPARAM - 17:] == 0.0)          # normalisation constants are not trained


def test_tensor_core_inference_matches_oracle(api):
    from oracle import mlp
    X, T = _rows_of(api, [molecules.random_molecule(7, 8, 24)], nrows=None)
    P = _blob(api, X, T, seed=3)
    Y = api.mlp_predict(P, X)
    Yr, _ = mlp.forward(mlp.unpack(P), X)
    assert np.abs(Y - Yr).max() <= 2e-3 * np.abs(Yr).max()
    # ragged tile counts: a single row and a partial last tile
    assert np.array_equal(api.mlp_predict(P, X[:1]), Y[:1])
    assert np.array_equal(api.mlp_predict(P, X[:300]), Y[:300])


def test_training_lowers_the_loss(api):
    X, T = _rows_of(api, [molecules.random_molecule(s, 8, 24) for s in range(200, 216)], nrows=2048)
    from helios_gb300 import learned
    P, L = learned.fit(X, T, epochs=6, batch=1024, lr=2e-3)
    assert np.all(np.isfinite(L))
    assert L[-1] < 0.5 * L[0]
    assert learned.mse(P, X, T) < np.mean(T.astype(np.float64) ** 2)


def test_engine_guess_is_guess_plus_prediction(api):
    from helios_gb300 import learned
    X, T = _rows_of(api, [molecules.random_molecule(5, 8, 20)], nrows=None)
    P = _blob(api, X, T, seed=9)
    mol = molecules.ladder(12)
    cr = api.CoupledCluster(mol, api.Keywords(bond_alternation=0.1, accuracy=10))
    cr.initCC()
    _, o, v, _ = cr.dims[0]
    ov = o * v
    rows = np.arange(ov * (ov + 1) // 2)
    X0, _ = cr.training_rows(0, rows)
    cr.finalizeCC()
    # an untrained network: scale its output (linear in y_scale) to corrections of at most 1e-3
    P[-1] *= 1e-3 / np.abs(api.mlp_predict(P, X0)).max()
    cc = api.CoupledCluster(mol, api.Keywords(bond_alternation=0.1, accuracy=10, guess="learned", model=P))
    cc.initCC()
    Xg, Tg = cc.training_rows(0, rows)          # T = t2 - guess = the prediction
    assert np.array_equal(Xg, X0)
    Y = api.mlp_predict(P, Xg)
    assert np.allclose(Tg, Y, rtol=1e-6, atol=1e-9)
    t1, t2 = cc.amplitudes(0)
    assert np.abs(t2 - t2.transpose(1, 0, 3, 2)).max() == 0.0
    r = cc.iterate()
    cc.finalizeCC()
    ref = api.get_energy(mol, api.Keywords(bond_alternation=0.1, accuracy=10))
    assert r["status"] == 1
    assert abs(r["energy"][0] - ref["energy"][0]) < 1e-8          # the guess never changes the answer


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(__file__), "..", "helios_gb300", "data",
                                                    "t2_guess.npy")), reason="no trained model shipped")
def test_shipped_model_gain_on_held_out_molecules(api):
    """What the trained network gains over guessCC on molecules it never saw
    (seeds outside its training range): a starting t2 several times closer to
    the converged one, the same converged energies, and no more iterations.
    (Measured on 512 held-out molecules, the closer start saves almost no
    iterations: the singles, which start at zero either way, and the DIIS
    history set the pace; helios_gb300/data/t2_guess.json has the numbers.)"""
    from helios_gb300 import learned
    mols = molecules.ensemble(learned.HELD_OUT_SEED + 1000, 16)
    model = learned.default_model()
    kw = dict(bond_alternation=0.1, accuracy=8)
    ref = api.CoupledCluster(mols, api.Keywords(**kw))
    ref.initCC()
    start_ref = [ref.amplitudes(k)[1] for k in range(len(mols))]
    out_ref = ref.solve_batch()
    conv = [ref.amplitudes(k)[1] for k in range(len(mols))]
    ref.finalizeCC()
    lrn = api.CoupledCluster(mols, api.Keywords(guess="learned", model=model, **kw))
    lrn.initCC()
    start_lrn = [lrn.amplitudes(k)[1] for k in range(len(mols))]
    out_lrn = lrn.solve_batch()
    lrn.finalizeCC()
    assert np.all(out_ref["status"] == 1) and np.all(out_lrn["status"] == 1)
    assert np.abs(out_ref["energy"][:, 0] - out_lrn["energy"][:, 0]).max() < 1e-7
    err_ref = np.sqrt(sum(np.sum((a - c) ** 2) for a, c in zip(start_ref, conv)))
    err_lrn = np.sqrt(sum(np.sum((a - c) ** 2) for a, c in zip(start_lrn, conv)))
    assert err_lrn < 0.4 * err_ref
    assert out_lrn["iterations"].mean() <= out_ref["iterations"].mean() + 1.0
