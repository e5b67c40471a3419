"""Learned SCC starting charges.

The reference starts every SCC loop from the neutral charges
(withSP2_deltaH.cpp:1725-1740).  Here a per-atom MLP (tb_mlp_*, 32 radial
features -> 64 -> 64 -> 1, SiLU, BF16 weights) trained on converged charges
of randomly distorted beta-cristobalite cells predicts q - q0; the
prediction, shifted to conserve the electron count, seeds tb_scc_solve,
which alone decides convergence (|dq| < tol) -- a poor prediction costs
iterations, never accuracy.

  dataset()    converged charges of seeded cells from the batched solver
  train()      minibatch Adam on the GPU (the library's own kernels)
  save()/load()  parameters + feature normalisation as .npz
  warm_start() q_init for a model

``python -m largetb_gb300.learned OUT.npz`` builds the dataset (2000 3x3x3
cells, sigma uniform in [0.02, 0.15] A), trains, and writes the weights.
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

from . import api as T

BOHR_PER_ANG = 1.88973
DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "charge_mlp.npz")


def cell_box(dims, a_ang=7.16):
    return np.array(dims, float) * a_ang * BOHR_PER_ANG


def dataset(n_cells=2000, dims=(3, 3, 3), sigma=(0.02, 0.15), seed=5005, M=200, batch=64, device=0):
    """Features and net charges of n_cells seeded cells (cell i: noise seed
    seed * 1000 + i, sigma uniform in the range)."""
    rng = np.random.default_rng(seed)
    X, Y, iters = [], [], []
    for b0 in range(0, n_cells, batch):
        models = []
        for i in range(b0, min(n_cells, b0 + batch)):
            sig = float(rng.uniform(*sigma))
            models.append(T.model_cristobalite(*dims, sigma_ang=sig, seed=seed * 1000 + i))
        with T.Batch(models, M=M, device=device) as B:
            r = B.scc_solve()
        iters.extend(int(x) for x in r["iters"])
        for m, q in zip(models, r["q"]):
            X.append(T.mlp_features(m.xyz, m.species, cell_box(dims)))
            Y.append(q - m.q0)
    return np.concatenate(X), np.concatenate(Y).astype(np.float32), iters


def train(X, Y, epochs=40, batch=2048, lr=2e-3, seed=1, device=0):
    mlp = T.MLP(device=device, seed=seed)
    loss = mlp.train(X, Y, epochs=epochs, batch=batch, lr=lr, seed=seed)
    return mlp, loss


def save(mlp, path, meta=None):
    p, nrm = mlp.get()
    np.savez_compressed(path, params=p, norm=nrm, meta=json.dumps(meta or {}))


def load(path=DEFAULT_WEIGHTS, device=0):
    d = np.load(path)
    mlp = T.MLP(device=device)
    mlp.set(d["params"], d["norm"])
    return mlp


# Anderson mixing parameter for solves started from the prediction: closer to
# the fixed point than q0, they converge fastest with a smaller step (sweep
# over 6x6x6, sigma 0.05 A and 4x4x4, sigma 0.12 A cristobalite).
MIX_BETA = 0.1


def warm_start(mlp, model, box):
    """q_init = q0 + predicted q - q0, shifted to keep sum(q) = sum(q0)."""
    dq = mlp.predict(T.mlp_features(model.xyz, model.species, box)).astype(np.float64)
    dq -= dq.mean()
    return model.q0 + dq


def main(out, n_cells=2000, epochs=40):
    t0 = time.time()
    X, Y, it = dataset(n_cells=n_cells)
    t1 = time.time()
    mlp, loss = train(X, Y, epochs=epochs)
    t2 = time.time()
    meta = {"cells": n_cells, "dims": [3, 3, 3], "sigma_ang": [0.02, 0.15], "seed": 5005, "M": 200,
            "samples": int(Y.shape[0]), "epochs": epochs, "final_loss": float(loss[-1]),
            "rmse_e": float(np.sqrt(loss[-1])), "dataset_s": t1 - t0, "train_s": t2 - t1,
            "scc_iters_zero_start_mean": float(np.mean(it))}
    save(mlp, out, meta)
    print(json.dumps(meta))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else DEFAULT_WEIGHTS)
