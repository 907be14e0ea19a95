"""Cells that RReact's Newton converges slowly, on the oracle (CPU).

RReact damps every update after iteration 50 and loops until converged
(reaction.F90:3478-3496; the "> 500" stop is unreachable).  On the
synthetic 12-species network about 2 % of cells pass iteration 50, where
the reference Jacobian (which lacks the free-site and capped-QK terms)
converges only linearly and the damping slows it tenfold.  These tests pin
what the library option exact_jacobian_after does for them and what the
200-iteration cap without it leaves unconverged."""
import numpy as np

from pflotran_gb300 import abi, workloads

from helpers import cell_errors, per_cell_bar, truth_solve

NCELLS = 20000


def _opts(opt, **kw):
    o = abi.Options.from_buffer_copy(opt)
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def _run(oracle, net, o, cells, dt):
    c = cells.copy()
    c.sec_molal = np.zeros(net.Nc * c.ncells)
    c.iterations = np.zeros(c.ncells, np.int32)
    c.status = np.zeros(c.ncells, np.int32)
    oracle.react(net.as_struct(), o, dt, c, 0, 8)
    return c


def test_capped_cells_converge_slowly_without_the_cap(oracle):
    """The cells the 200-iteration cap stops are slow, not oscillating:
    without the cap every one converges (RReact's own behaviour), and the
    capped answer is their iterate at 200."""
    net, opt, cells, dt = workloads.synthetic_cells(NCELLS, seed=2024)
    capped = _run(oracle, net, _opts(opt, exact_jacobian_after=0), cells, dt)
    stuck = np.flatnonzero(capped.status != 0)
    assert 0.002 * NCELLS < len(stuck) < 0.02 * NCELLS
    assert (capped.status[stuck] == abi.CELL_MAXITER).all()
    free = _run(oracle, net, _opts(opt, exact_jacobian_after=0, max_iterations=100000), cells, dt)
    assert (free.status == 0).all()
    its = free.iterations[stuck]
    assert its.min() > 200 and np.median(its) < 1000, np.percentile(its, [0, 50, 100])
    # the capped iterate is still far (in the scaled metric) from the converged answer
    e = cell_errors(net, capped.subset(stuck, net), free.subset(stuck, net))["total"]
    assert np.median(e) > 1e-10


def test_exact_jacobian_after_50_converges_every_cell_as_accurately_as_rreact(oracle):
    """exact_jacobian_after = 50: iterations 1-50 are RReact's, the few cells
    still unconverged then finish in a handful of exact-Newton iterations.
    Every cell converges; each answer is within 1e-10 of the uncapped RReact
    answer or no farther than it from the root (long-double solve to a 1e-16
    relative residual); and fewer cells than RReact's own answers lie more
    than 1e-10 from the root."""
    net, opt, cells, dt = workloads.synthetic_cells(NCELLS, seed=2024)
    rescued = _run(oracle, net, _opts(opt, exact_jacobian_after=50), cells, dt)
    rreact = _run(oracle, net, _opts(opt, exact_jacobian_after=0, max_iterations=100000), cells, dt)
    assert (rescued.status == 0).all()
    assert rescued.iterations.max() <= 60
    assert rescued.iterations.mean() < rreact.iterations.mean()
    late = rreact.iterations > 50
    assert (rescued.iterations[~late] == rreact.iterations[~late]).all()
    truth = truth_solve(oracle, net, opt, cells, dt, start=rreact)
    assert (truth.status == 0).all() and truth.iterations.max() <= 8
    for q, (ok, exr, ext, ert) in per_cell_bar(net, rescued, rreact, truth).items():
        assert ok.all(), (q, int((~ok).sum()))
        assert (ext > 1e-10).sum() <= (ert > 1e-10).sum(), q
