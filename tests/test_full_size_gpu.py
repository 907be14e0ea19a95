"""Parity at the headline size: 2,097,152 cells of the synthetic 12-species
network through the GPU library, plain and with the learned warm start,
4000 randomly sampled cells re-solved by the oracle.

Bar, per sampled cell and quantity (totals, mineral rates and volume
fractions, scaled relative error): within 1e-10 of the oracle, or no
farther than the oracle from the root of the cell's equations (the oracle
in long double, exact undamped Newton to a 1e-16 relative residual), or --
for the warm start -- no farther from the oracle than the oracle's own
answers from the two starting guesses are from each other.  The last two
branches are for ill-conditioned cells, where two Newton paths that both
pass the 1e-12 relative-residual test land up to the tolerance x the
conditioning apart."""
import numpy as np
import pytest

from oracle import parity
from pflotran_gb300 import workloads
from pflotran_gb300.lib import ReactionStep
from pflotran_gb300.surrogate import fit, generate

pytestmark = pytest.mark.gpu
NCELLS = 2_097_152
SAMPLE = 4000


def _check(net, gpu_sub, ref, truth, alt=None):
    both = (ref.status == 0) & (gpu_sub.status == 0) & (truth.status == 0)
    assert both.mean() > 0.999
    bar = parity.per_cell_bar(net, gpu_sub, ref, truth, 1e-10, both, alt=alt)
    report = {q: (int((~ok).sum()), float(exr[both].max()), float(np.percentile(exr[both], 99)))
              for q, (ok, exr, ext, ert) in bar.items()}
    print(report)
    fails = parity.bar_failures(net, gpu_sub, ref, truth, bar, alt)
    assert not fails, fails
    return report


def test_synthetic_network_full_size_sampled_plain_and_warm(oracle):
    net, opt, cells, dt = workloads.synthetic_cells(NCELLS, seed=2024, device="cuda")
    step = ReactionStep(net, opt)
    rng = np.random.default_rng(7)
    idx = np.sort(rng.choice(NCELLS, SAMPLE, replace=False))
    sub = cells.subset(idx, net)
    ref = parity.solve(net, opt, dt, sub)
    truth = parity.truth_solve(net, opt, dt, sub, ref)
    # plain Newton from the previous-step guess: every cell converges
    d = cells.to_device()
    bad = step.react(d, dt)
    assert bad == 0
    gp = d.to_host()
    assert (gp.status == 0).all() and gp.iterations.max() <= 60
    _check(net, gp.subset(idx, net), ref, truth)
    del d
    # learned warm start (a small training set: parity does not depend on
    # how good the guess is)
    X, molal = generate(step, lambda m, s: workloads.synthetic_cells(m, seed=s, net=net, device="cuda")[2],
                        262144, 41, dt)
    fit(step, X, molal, epochs=4, batch=4096)
    del X, molal
    w = cells.to_device()
    pred = step.surrogate_predict(w).view(net.N, NCELLS)[:, idx.tolist()].cpu().numpy()
    step.surrogate_enable(True)
    # a few cells of 2M may start from a learned guess whose residual is
    # lower but from which Newton does not converge in the cap (reported,
    # not counted as converged)
    assert step.react(w, dt) <= 20
    st = step.stats()
    assert st.alt_guess_used > 0.5 * NCELLS
    gw = w.to_host()
    gsub = gw.subset(idx, net)
    # against the oracle started from the same learned guess (same choice
    # rule); the oracle's own answer from the previous-step guess measures
    # how far RReact's stop lets two starting points land apart
    ref_w = parity.solve(net, opt, dt, sub, alt_guess=np.ascontiguousarray(pred).ravel())
    _check(net, gsub, ref_w, truth, alt=ref)
