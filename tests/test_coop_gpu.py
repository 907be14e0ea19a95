"""The cooperative kernels (8, 16 or 32 lanes per cell) against the oracle.

Same bar as the other parity tests: 1e-10 scaled relative error on cells
whose iteration counts agree with the oracle's, and per cell, everywhere,
within 1e-10 of the oracle or no farther than it from the root of the
cell's equations."""
import numpy as np
import pytest

from oracle import parity
from pflotran_gb300 import abi, workloads
from pflotran_gb300.lib import PfchemError, ReactionStep

from helpers import compare

pytestmark = pytest.mark.gpu
VARIANTS = [abi.KERNEL_COOP8, abi.KERNEL_COOP16, abi.KERNEL_COOP32]


def _workload(kind):
    if kind == "calcite_grid":
        return workloads.calcite_cells(4096, seed=41, temperature_dependent=True)
    net, opt, cells, dt = workloads.synthetic_cells(4096, seed=42)
    if kind == "synthetic_prefactors":
        workloads.add_rate_prefactors(net)
    elif kind == "synthetic_exact":
        opt.jacobian = abi.JACOBIAN_EXACT
    elif kind == "synthetic_newton_iter":
        opt.act_coef_update_frequency = abi.ACT_COEF_FREQUENCY_NEWTON_ITER
    return net, opt, cells, dt


def _solve(step, variant, cells, dt):
    step.set_launch(128, 1, 1, variant)
    d = cells.to_device()
    d.sec_molal = None
    step.react(d, dt)
    return d.to_host()


def _check(net, opt, dt, cells, gpu, ref):
    ok = (ref.status == 0) & (gpu.status == 0)
    # the GPU reports the oracle's per-cell status (some draws have cells
    # whose inner loops hit their caps in both)
    assert np.mean(ref.status == gpu.status) > 0.999, (np.bincount(ref.status), np.bincount(gpu.status))
    assert ok.mean() > 0.99
    same = ok & (ref.iterations == gpu.iterations)
    assert same.sum() > 0.98 * ok.sum()
    gpu.sec_molal = None
    errs = compare(net, gpu, ref, mask=same)
    assert all(v <= 1e-10 for v in errs.values()), errs
    truth = parity.truth_solve(net, opt, dt, cells, ref)
    for q, (bar, *_r) in parity.per_cell_bar(net, gpu, ref, truth, mask=ok & (truth.status == 0)).items():
        assert bar.all(), (q, int((~bar).sum()))


@pytest.mark.parametrize("kind", ["calcite_grid", "synthetic", "synthetic_prefactors", "synthetic_exact",
                                  "synthetic_newton_iter"])
@pytest.mark.parametrize("variant", VARIANTS)
def test_cooperative_kernel_parity(oracle, kind, variant):
    net, opt, cells, dt = _workload(kind)
    ref = parity.solve(net, opt, dt, cells)
    step = ReactionStep(net, opt)
    gpu = _solve(step, variant, cells, dt)
    _check(net, opt, dt, cells, gpu, ref)
    st = step.stats()
    assert st.ncells == cells.ncells and st.sum_iterations == int(gpu.iterations.sum())


@pytest.mark.parametrize("variant", VARIANTS)
def test_cooperative_kernel_alternative_guess_and_inactive_cells(oracle, variant):
    """The alternative (warm-start) guess taken where its residual is no
    larger, the plain guess elsewhere; inactive cells skipped."""
    net, opt, cells, dt = workloads.synthetic_cells(4096, seed=43)
    sol = parity.solve(net, opt, dt, cells)
    rng = np.random.default_rng(5)
    alt = (sol.pri_molal.reshape(net.N, -1) * np.exp(rng.normal(0.0, 0.3, (net.N, cells.ncells)))).ravel()
    cells.active = np.ones(cells.ncells, np.int32)
    cells.active[::97] = 0
    ref = parity.solve(net, opt, dt, cells, alt_guess=alt)
    c = cells.copy()
    c.alt_guess = alt
    step = ReactionStep(net, opt)
    gpu = _solve(step, variant, c, dt)
    assert (gpu.status[::97] == abi.CELL_INACTIVE).all()
    act = cells.active > 0
    assert step.stats().alt_guess_used == int(np.sum(act)) - 0 or step.stats().alt_guess_used > 0.5 * act.sum()
    sub = np.flatnonzero(act)
    _check(net, opt, dt, cells.subset(sub, net), gpu.subset(sub, net), ref.subset(sub, net))


def test_cooperative_kernel_rejects_unsupported_options():
    net, opt, cells, dt = workloads.calcite_cells(64, seed=44)
    opt.use_log_formulation = 0
    step = ReactionStep(net, opt)
    with pytest.raises(PfchemError, match="cooperative"):
        step.set_launch(128, 1, 1, abi.KERNEL_COOP16)
