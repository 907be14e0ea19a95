"""The warm-start MLP on the tcgen05 tensor-core path (tensor-memory
accumulators, weights resident in shared memory) against the mma.sync path
and the FP64 gradient oracle."""
import numpy as np
import pytest

from oracle import mlp_oracle as mo
from oracle import parity
from pflotran_gb300 import abi, workloads
from pflotran_gb300.lib import ReactionStep
from pflotran_gb300.surrogate import fit, generate

pytestmark = pytest.mark.gpu


def _data(step, n, seed):
    net = step.network
    return generate(step, lambda m, s: workloads.synthetic_cells(m, seed=s, net=net)[2], n, seed, 86400.0,
                    chunk=n)


def test_tcgen05_layers_match_mma_sync_layers():
    """Same weights, same inputs: the two tensor-core paths compute the same
    products in a different FP32 summation order, so the predicted ln m
    agree to BF16 rounding of the hidden activations."""
    net = workloads.synthetic_network()
    _, opt, _, _ = workloads.synthetic_cells(8, seed=1, net=net)
    step = ReactionStep(net, opt)
    step.surrogate_backend(abi.MLP_MMA_SYNC)
    X, molal = _data(step, 65536, 43)
    fit(step, X, molal, epochs=2, batch=4096)
    _, _, cells, _ = workloads.synthetic_cells(50001, seed=44, net=net)
    d = cells.to_device()
    a = step.surrogate_predict_layers(d).cpu().numpy()
    step.surrogate_backend(abi.MLP_TCGEN05)
    b = step.surrogate_predict_layers(d).cpu().numpy()
    c = step.surrogate_predict(d).cpu().numpy()
    assert np.isfinite(b).all()
    np.testing.assert_array_equal(b, c)  # the tcgen05 backend's inference is the layer path
    dl = np.abs(np.log(a) - np.log(b))
    print(f"ln m difference mma.sync vs tcgen05: max {dl.max():.3e}, rms {np.sqrt(np.mean(dl ** 2)):.3e}")
    assert np.sqrt(np.mean(dl ** 2)) < 2e-3 and dl.max() < 0.1


def test_tcgen05_gradients_match_fp64_oracle():
    net = workloads.synthetic_network()
    _, opt, _, _ = workloads.synthetic_cells(8, seed=1, net=net)
    step = ReactionStep(net, opt)
    step.surrogate_backend(abi.MLP_TCGEN05)
    X, molal = _data(step, 1024, 31)
    Xh = X.cpu().numpy().astype(np.float64)
    fm = Xh.mean(0)
    fs = 1.0 / np.maximum(Xh.std(0), 1e-6)
    lm = np.log(molal.cpu().numpy()).T
    tm, ts = lm.mean(0), np.maximum(lm.std(0), 1e-6)
    step.surrogate_normalization((fm, fs, tm, ts))
    p = mo.init_params(5)
    step.surrogate_params(p)
    g_gpu, loss_gpu = step.surrogate_gradients(X, molal)
    Xs = (Xh - fm.astype(np.float32)) * fs.astype(np.float32)
    Ts = ((lm - tm.astype(np.float32)) / ts.astype(np.float32))
    loss_ref, g_ref = mo.loss_and_grads(p, Xs.astype(np.float32), Ts, net.N)
    assert abs(loss_gpu - loss_ref) <= 1e-3 * loss_ref
    off = 0
    for l in range(4):
        k, n = mo.DIMS[l], mo.DIMS[l + 1]
        for size in (k * n, n):
            a, b = g_gpu[off:off + size], g_ref[off:off + size]
            off += size
            if np.linalg.norm(b) == 0:
                continue
            rel = np.linalg.norm(a - b) / np.linalg.norm(b)
            print(f"tcgen05 layer {l} {'weights' if size == k * n else 'bias'}: relative L2 error {rel:.3e}")
            assert rel < 2e-3, (l, size, rel)


def test_tcgen05_trained_warm_start_parity(oracle):
    """Trained and run on the tcgen05 path: fewer iterations than the plain
    guess, and the warm-started GPU solves meet the per-cell bar against the
    oracle started from the same learned guess."""
    net = workloads.synthetic_network()
    _, opt, _, dt = workloads.synthetic_cells(8, seed=1, net=net)
    step = ReactionStep(net, opt)
    step.surrogate_backend(abi.MLP_TCGEN05)
    X, molal = _data(step, 262144, 41)
    rep, _ = fit(step, X, molal, epochs=6, batch=4096, lr=2e-3)
    assert rep.final_loss < 0.2 * rep.first_loss
    _, _, cells, _ = workloads.synthetic_cells(16384, seed=97, net=net)
    plain = cells.to_device()
    step.react(plain, dt)
    it_plain = step.stats().sum_iterations / cells.ncells
    warm = cells.to_device()
    pred = step.surrogate_predict(warm).cpu().numpy()
    step.surrogate_enable(True)
    step.react(warm, dt)
    it_warm = step.stats().sum_iterations / cells.ncells
    assert it_warm < 0.9 * it_plain, (it_plain, it_warm)
    gw = warm.to_host()
    idx = np.arange(4096)
    sub = cells.subset(idx, net)
    ref = parity.solve(net, opt, dt, sub, alt_guess=np.ascontiguousarray(pred.reshape(net.N, -1)[:, idx]).ravel())
    g = gw.subset(idx, net)
    assert ((ref.status == 0) & (g.status == 0)).mean() > 0.999
    plain_ref = parity.solve(net, opt, dt, sub)
    truth = parity.truth_solve(net, opt, dt, sub, plain_ref)
    ok = (ref.status == 0) & (g.status == 0) & (truth.status == 0)
    bar = parity.per_cell_bar(net, g, ref, truth, mask=ok, alt=plain_ref)
    fails = parity.bar_failures(net, g, ref, truth, bar, plain_ref)
    assert not fails, fails
