"""Learned warm start: the GPU training kernels against the FP64 oracle, and
what the trained network gains over the plain previous-step guess."""
import numpy as np
import pytest

from oracle import mlp_oracle as mo
from oracle import parity
from pflotran_gb300 import abi, workloads
from pflotran_gb300.lib import ReactionStep
from pflotran_gb300.surrogate import fit, generate

from helpers import compare

pytestmark = pytest.mark.gpu


def _data(step, n, seed):
    net = step.network
    return generate(step, lambda m, s: workloads.synthetic_cells(m, seed=s, net=net)[2], n, seed, 86400.0,
                    chunk=n)


def test_gradients_match_fp64_oracle():
    net = workloads.synthetic_network()
    _, opt, _, _ = workloads.synthetic_cells(8, seed=1, net=net)
    step = ReactionStep(net, opt)
    step.surrogate_backend(abi.MLP_MMA_SYNC)  # the tcgen05 path has its own gradient test
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
            print(f"layer {l} {'weights' if size == k * n else 'bias'}: relative L2 error {rel:.3e}")
            # measured on GB300: at most 1.5e-4 (layer 0 weights); bar 2e-3
            assert rel < 2e-3, (l, size, rel)


def test_fused_inference_equals_layer_by_layer():
    """The one-kernel inference (activations in registers, packed weight
    fragments) computes the same products in the same order as the
    GEMM-per-layer path: the guesses agree bit for bit, over a batch whose
    size is not a multiple of the kernel's 64-row tile."""
    net = workloads.synthetic_network()
    _, opt, _, _ = workloads.synthetic_cells(8, seed=1, net=net)
    step = ReactionStep(net, opt)
    step.surrogate_backend(abi.MLP_MMA_SYNC)
    X, molal = _data(step, 65536, 43)
    fit(step, X, molal, epochs=2, batch=4096)
    _, _, cells, _ = workloads.synthetic_cells(50001, seed=44, net=net)
    d = cells.to_device()
    a = step.surrogate_predict(d).cpu().numpy()
    b = step.surrogate_predict_layers(d).cpu().numpy()
    assert np.isfinite(a).all()
    np.testing.assert_array_equal(a, b)


def test_trained_warm_start_reduces_iterations_with_identical_results(oracle):
    net = workloads.synthetic_network()
    _, opt, _, dt = workloads.synthetic_cells(8, seed=1, net=net)
    step = ReactionStep(net, opt)
    X, molal = _data(step, 262144, 41)
    rep, _ = fit(step, X, molal, epochs=10, batch=4096, lr=2e-3)
    assert rep.final_loss < 0.2 * rep.first_loss
    # a fresh draw: plain previous-step guess versus the learned warm start
    _, _, cells, _ = workloads.synthetic_cells(65536, seed=97, net=net)
    plain = cells.to_device()
    step.surrogate_enable(False)
    step.react(plain, dt)
    st_plain = step.stats()
    warm = cells.to_device()
    pred = step.surrogate_predict(warm).cpu().numpy()
    step.surrogate_enable(True)
    step.react(warm, dt)
    st_warm = step.stats()
    gw = warm.to_host()
    mean_plain = st_plain.sum_iterations / cells.ncells
    mean_warm = st_warm.sum_iterations / cells.ncells
    assert st_warm.alt_guess_used > 0.5 * cells.ncells
    assert mean_warm < 0.9 * mean_plain, (mean_plain, mean_warm)
    # the warm-started path against the oracle given the same two guesses
    # (the oracle applies the same choice, residual norm at both, and
    # Newton), on 4096 cells; bar per cell at 1e-10: within 1e-10 of that
    # oracle solution, or no farther than it from the root of the cell's
    # equations (long double, 1e-16 relative residual).  A cell whose last
    # residual lands next to the 1e-12 threshold may stop one iteration apart
    # on the two machines; the second branch covers it.
    sub_idx = np.arange(4096)
    sub = cells.subset(sub_idx, net)
    ref = parity.solve(net, opt, dt, sub, alt_guess=np.ascontiguousarray(pred.reshape(net.N, -1)[:, sub_idx]).ravel())
    g_sub = gw.subset(sub_idx, net)
    ok = (ref.status == 0) & (g_sub.status == 0)
    assert ok.all()
    same = ref.iterations == g_sub.iterations
    assert same.mean() > 0.98
    errs = compare(net, g_sub, ref, mask=same)
    assert all(v <= 1e-10 for v in errs.values()), errs
    plain_ref = parity.solve(net, opt, dt, sub)
    truth = parity.truth_solve(net, opt, dt, sub, plain_ref)
    assert (truth.status == 0).all()
    bar = parity.per_cell_bar(net, g_sub, ref, truth, alt=plain_ref)
    fails = parity.bar_failures(net, g_sub, ref, truth, bar, plain_ref)
    assert not fails, fails
