"""The FP64 MLP restatement used to check the GPU training kernels: its
analytic gradients against central finite differences (no BF16 emulation)."""
import numpy as np

from oracle import mlp_oracle as mo

DIMS = (16, 8, 8, 8, 16)


def test_analytic_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    p = mo.init_params(1, DIMS).astype(np.float64)
    X = rng.standard_normal((7, 16))
    T = rng.standard_normal((7, 12))
    _, g = mo.loss_and_grads(p, X, T, 12, emulate_bf16=False, dims=DIMS)
    idx = rng.choice(p.size, 40, replace=False)
    for i in idx:
        e = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[i] += e
        pm[i] -= e
        lp, _ = mo.loss_and_grads(pp, X, T, 12, emulate_bf16=False, dims=DIMS)
        lm, _ = mo.loss_and_grads(pm, X, T, 12, emulate_bf16=False, dims=DIMS)
        fd = (lp - lm) / (2 * e) / (7 * 12)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.001953125, -3.14159265, 1e-30], np.float32)
    r = mo.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0  # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: rounds to even
    assert r[2] == 1.0
    assert r[3] == -3.140625
