"""Training data and fitting for the learned warm start.

The network learns the step's solution from solves that the FP64 Newton
kernel produces: cells are drawn from the workload's seeded distribution,
their features are taken before the step, the plain solve runs, and the
converged free-ion molalities of the converged cells are the targets.
"""
from __future__ import annotations

import time


def generate(step, make_cells, n, seed, dt, chunk=2_097_152):
    """(X [M,16] float32, molal [N,M] float64) device tensors from `n` cells
    drawn by make_cells(count, seed) -> host CellBatch, solved by `step`."""
    import torch
    Xs, Ms = [], []
    done = 0
    k = 0
    while done < n:
        m = min(chunk, n - done)
        cells = make_cells(m, seed + 1000 * k)
        d = cells.to_device()
        X = step.surrogate_features(d)
        step.react(d, dt)
        ok = d.status == 0
        N = step.network.N
        molal = d.pri_molal.view(N, m)[:, ok]
        Xs.append(X[ok])
        Ms.append(molal)
        done += m
        k += 1
    return torch.cat(Xs), torch.cat(Ms, dim=1).contiguous()


def fit(step, X, molal, epochs=8, batch=8192, lr=2e-3, weight_decay=1e-4, seed=7):
    t0 = time.perf_counter()
    rep = step.surrogate_fit(X, molal, epochs=epochs, batch=batch, lr=lr, weight_decay=weight_decay, seed=seed)
    return rep, time.perf_counter() - t0
