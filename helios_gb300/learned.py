"""Learned T2 initial guess: data generation, training and evaluation.

The network (8 -> 256 -> 256 -> 256 -> 1, SiLU; bf16 weights in the two
256 x 256 layers, FP32 accumulation) predicts per amplitude the difference
between the converged t2 and the reference's MP2-like guess (guessCC,
src/methods/coupledCluster/mod_cc.f90:634-650). Every step runs on the GPU
through the C ABI:

* ``generate``: batched mixed-precision solves of seeded random PPP molecules
  (``molecules.random_molecule``: zigzag polyenes and acene-like ladders of
  8-64 sites) and, per converged molecule, a random sample of canonical
  amplitude pairs with their inputs and targets (``hx_ccsd_training_rows``);
* ``fit``: training by the engine's own forward/backward kernels and Adam
  (``hx_mlp_train``);
* ``evaluate``: iteration counts and solve times of held-out molecules with
  the reference guess and with the learned guess, to the same residual.

Training molecules use seeds ``TRAIN_SEED + k``; held-out molecules come
from other seeds, so the split is by seed. The shipped model is
``data/t2_guess.npy`` with its training report ``data/t2_guess.json``.

    python -m helios_gb300.learned --molecules 20480 --out helios_gb300/data
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from . import api, molecules

H, F = 256, 8
TRAIN_SEED = 1_000_000
HELD_OUT_SEED = 20261203
_HERE = os.path.dirname(os.path.abspath(__file__))
MODEL_PATH = os.path.join(_HERE, "data", "t2_guess.npy")
FEATURES = ["guess", "e_i", "e_j", "e_a", "e_b", "(ia|jb)", "(ib|ja)", "8/N"]


def default_model() -> np.ndarray:
    if not os.path.exists(MODEL_PATH):
        raise FileNotFoundError(f"{MODEL_PATH} is missing: train one with `python -m helios_gb300.learned`")
    return np.load(MODEL_PATH).astype(np.float32)


def init_params(X, T, seed=0) -> np.ndarray:
    """He-initialised blob with input/output normalisation taken from the data."""
    rng = np.random.default_rng(seed)
    shift = X.mean(0)
    scale = 1.0 / np.maximum(X.std(0), 1e-12)
    ys = max(float(np.sqrt(np.mean(T.astype(np.float64) ** 2))), 1e-12)
    parts = [rng.normal(size=(H, F)) * np.sqrt(2.0 / F), np.zeros(H),
             rng.normal(size=(H, H)) * np.sqrt(2.0 / H), np.zeros(H),
             rng.normal(size=(H, H)) * np.sqrt(2.0 / H), np.zeros(H),
             rng.normal(size=H) * np.sqrt(1.0 / H) * 0.1, np.zeros(1),
             shift, scale, np.array([ys])]
    blob = np.concatenate([np.asarray(p, dtype=np.float32).ravel() for p in parts])
    assert blob.size == api.mlp_nparam()
    return blob


def _keywords(accuracy, precision="mixed", guess="reference", model=None):
    return api.Keywords(bond_alternation=0.1, accuracy=accuracy, precision=precision, guess=guess, model=model)


def generate(count, rows_per_mol=256, batch=512, accuracy=8, seed0=TRAIN_SEED, sample_seed=0, log=None):
    """Training rows from `count` solved molecules (seeds seed0 .. seed0 + count - 1)."""
    rng = np.random.default_rng(sample_seed)
    Xs, Ts, used = [], [], 0
    t0 = time.perf_counter()
    for start in range(0, count, batch):
        mols = molecules.ensemble(seed0 + start, min(batch, count - start))
        cc = api.CoupledCluster(mols, _keywords(accuracy))
        cc.initCC()
        out = cc.solve_batch()
        for k in range(len(mols)):
            if out["status"][k] != 1:
                continue
            _, o, v, _ = cc.dims[k]
            ov = o * v
            npairs = ov * (ov + 1) // 2
            rows = np.arange(npairs) if npairs <= rows_per_mol else rng.choice(npairs, rows_per_mol, replace=False)
            X, T = cc.training_rows(k, rows)
            Xs.append(X)
            Ts.append(T)
            used += 1
        cc.finalizeCC()
        if log:
            log(f"generate: {start + len(mols)}/{count} molecules, {time.perf_counter() - t0:.1f} s")
    return np.concatenate(Xs), np.concatenate(Ts), used


def fit(X, T, epochs=20, batch=4096, lr=2e-3, seed=0):
    """Train a fresh network on (X, T) on the GPU; returns (params, per-epoch loss)."""
    P0 = init_params(X, T, seed)
    return api.mlp_train(P0, X, T, epochs=epochs, batch=batch, lr=lr, seed=seed)


def mse(params, X, T):
    """Mean squared error of the prediction (amplitude units) on (X, T)."""
    Y = api.mlp_predict(params, X)
    return float(np.mean((Y.astype(np.float64) - T) ** 2))


def evaluate(mols, params, accuracy=8, precision="mixed"):
    """Iterations, energies and device solve time with the reference and the learned guess."""
    res = {}
    for guess in ("reference", "learned"):
        cc = api.CoupledCluster(mols, _keywords(accuracy, precision, guess, params if guess == "learned" else None))
        cc.initCC()
        out = cc.solve_batch()
        tm = cc.timing()
        cc.finalizeCC()
        res[guess] = {"iterations": out["iterations"].astype(int), "status": out["status"].astype(int),
                      "energy": out["energy"][:, 0].copy(), "init_s": tm["init_ms"] / 1e3,
                      "solve_s": tm["solve_ms"] / 1e3}
    return res


def main():
    ap = argparse.ArgumentParser(description="train the learned T2 guess on the GPU")
    ap.add_argument("--molecules", type=int, default=20480)
    ap.add_argument("--rows", type=int, default=256, help="amplitude pairs sampled per molecule")
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--held-out", type=int, default=512)
    ap.add_argument("--out", default=os.path.dirname(MODEL_PATH))
    ap.add_argument("--data", help="reuse rows saved by --save-data instead of generating them")
    ap.add_argument("--save-data", help="write the generated rows (X, T) to this .npz")
    ap.add_argument("--save-rows", type=int, default=1_000_000, help="rows written by --save-data")
    args = ap.parse_args()
    log = lambda m: print(m, flush=True)
    t0 = time.perf_counter()
    if args.data:
        d = np.load(args.data)
        X, T, used = d["X"], d["T"], int(d["molecules"])
    else:
        X, T, used = generate(args.molecules, args.rows, log=log)
    t_gen = time.perf_counter() - t0
    if args.save_data:
        keep = np.random.default_rng(1).permutation(len(T))[:args.save_rows]
        np.savez_compressed(args.save_data, X=X[keep], T=T[keep], molecules=used)
    n_test = max(1, len(T) // 20)
    Xtr, Ttr, Xte, Tte = X[n_test:], T[n_test:], X[:n_test], T[:n_test]
    t1 = time.perf_counter()
    P, L = fit(Xtr, Ttr, args.epochs, args.batch, args.lr)
    t_fit = time.perf_counter() - t1
    log(f"fit: {args.epochs} epochs in {t_fit:.1f} s, loss {L[0]:.4g} -> {L[-1]:.4g}")
    zero = float(np.mean(Tte.astype(np.float64) ** 2))
    os.makedirs(args.out, exist_ok=True)
    np.save(os.path.join(args.out, "t2_guess.npy"), P)
    report = {"molecules": used, "rows": int(len(T)), "train_seeds": [TRAIN_SEED, TRAIN_SEED + args.molecules - 1],
              "generate_s": t_gen, "fit_s": t_fit, "epochs": args.epochs, "batch": args.batch, "lr": args.lr,
              "epoch_loss": [float(x) for x in L],
              "rows_mse_reference_guess": zero, "rows_mse_learned_guess": mse(P, Xte, Tte),
              "features": FEATURES}
    if args.held_out > 0:
        mols = molecules.ensemble(HELD_OUT_SEED, args.held_out)
        report["held_out"] = {"molecules": args.held_out, "seeds": [HELD_OUT_SEED, HELD_OUT_SEED + args.held_out - 1],
                              "accuracy": 8}
        for prec in ("fp64", "mixed"):
            ev = evaluate(mols, P, accuracy=8, precision=prec)
            r, l = ev["reference"], ev["learned"]
            ok = (r["status"] == 1) & (l["status"] == 1)
            report["held_out"][prec] = {
                "mean_iterations_reference": float(r["iterations"][ok].mean()),
                "mean_iterations_learned": float(l["iterations"][ok].mean()),
                "fewer_iterations": int((l["iterations"] < r["iterations"])[ok].sum()),
                "more_iterations": int((l["iterations"] > r["iterations"])[ok].sum()),
                "solve_s_reference": r["solve_s"], "solve_s_learned": l["solve_s"],
                "init_s_reference": r["init_s"], "init_s_learned": l["init_s"],
                "converged_both": int(ok.sum()),
                "max_abs_dE_eV": float(np.abs(r["energy"][ok] - l["energy"][ok]).max())}
            log(prec + " " + json.dumps(report["held_out"][prec]))
    json.dump(report, open(os.path.join(args.out, "t2_guess.json"), "w"), indent=1)


if __name__ == "__main__":
    main()
