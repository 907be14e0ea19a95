"""The 12-species workload's Newton iteration counts are predictable from
the pre-step state (CPU, oracle): the premise for ordering the persistent
kernel's work queue hardest-first, so that the cells that run to the
200-iteration cap start first instead of forming the straggler tail."""
import os

import numpy as np
import pytest

pytest.importorskip("sklearn")


def test_iteration_counts_are_predictable_from_the_pre_step_state(oracle):
    from scipy.stats import spearmanr
    from sklearn.ensemble import HistGradientBoostingRegressor
    from pflotran_gb300 import workloads
    net = workloads.synthetic_network()
    n = 60_000
    _, opt, cells, dt = workloads.synthetic_cells(n, seed=2024, net=net)
    N = net.N
    X = np.concatenate([np.arcsinh(cells.total.reshape(N, n) * 1e12), np.log(cells.pri_molal.reshape(N, n)),
                        np.log10(cells.ionic_strength)[None], cells.temperature[None]]).T
    b = cells.copy()
    b.sec_molal = np.zeros(net.Nc * n)
    oracle.react(net.as_struct(), opt, dt, b, 0, os.cpu_count() or 1)
    its = b.iterations.astype(float)
    train = np.arange(n) < n // 2
    model = HistGradientBoostingRegressor(max_iter=200, random_state=0).fit(X[train], np.log(its[train]))
    pred, true = model.predict(X[~train]), its[~train]
    assert spearmanr(pred, true).correlation > 0.8
    capped = true >= 200
    assert capped.sum() >= 30
    top = np.argsort(-pred)[:int(0.02 * len(true))]
    assert capped[top].sum() / capped.sum() > 0.8  # the hardest 2 % hold most of the capped cells
