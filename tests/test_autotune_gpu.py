"""The launch autotuner on a 32,768-cell draw of the 12-species workload:
the launch it keeps is no slower than the library's default launch, and the
answers do not depend on the launch."""
import numpy as np
import pytest

from pflotran_gb300 import abi, workloads
from pflotran_gb300.lib import ReactionStep

from helpers import compare

pytestmark = pytest.mark.gpu


def _timed(step, cells, dt, reps=3):
    best, out = 1e30, None
    for _ in range(reps):
        d = cells.to_device()
        step.react(d, dt)
        best = min(best, step.stats().kernel_ms)
        out = d.to_host()
    return best, out


def test_autotuned_launch_is_no_slower_and_bit_identical():
    net, opt, cells, dt = workloads.synthetic_cells(32768, seed=77)
    step = ReactionStep(net, opt)
    default = step.launch()
    t_default, a = _timed(step, cells, dt)
    _, _, trial, _ = workloads.synthetic_cells(32768, seed=78, net=net)
    tuned = step.autotune(trial.to_device(), dt)
    t_tuned, b = _timed(step, cells, dt)
    print(f"default {default.block_threads}/{default.blocks_per_sm}/{default.refill_min_idle}/{default.variant} "
          f"{t_default:.3f} ms, tuned {tuned.block_threads}/{tuned.blocks_per_sm}/{tuned.refill_min_idle}/"
          f"{tuned.variant} {t_tuned:.3f} ms")
    assert t_tuned <= 1.10 * t_default, (t_tuned, t_default)
    if tuned.variant in (abi.KERNEL_SPECIALIZED, abi.KERNEL_SPECIALIZED_COMPACT):
        # the specialized candidates do the same operations per cell
        for f in ("pri_molal", "total_out", "mnrl_rate", "mnrl_volfrac", "total_sorb_eq", "iterations", "status"):
            np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f)
    else:
        ok = (a.status == 0) & (b.status == 0) & (a.iterations == b.iterations)
        assert ok.mean() > 0.98
        errs = compare(net, b, a, mask=ok)
        assert all(v <= 1e-10 for v in errs.values()), errs


@pytest.mark.parametrize("kind", ["calcite", "synthetic"])
def test_shared_memory_layouts_are_bit_identical(kind):
    """The specialized kernel's two shared-memory layouts (the augmented
    [J | F], and the compact J with the right-hand side in registers and the
    pivot-column loop of the elimination rolled) and block sizes of 32 and
    64 threads do the same operations per cell: every output agrees bit for
    bit."""
    if kind == "calcite":
        net, opt, cells, dt = workloads.calcite_cells(8192, seed=79, temperature_dependent=True)
    else:
        net, opt, cells, dt = workloads.synthetic_cells(8192, seed=80)
    step = ReactionStep(net, opt)
    outs = []
    for block, variant in ((32, abi.KERNEL_SPECIALIZED), (32, abi.KERNEL_SPECIALIZED_COMPACT),
                           (64, abi.KERNEL_SPECIALIZED_COMPACT)):
        step.set_launch(block, 1, 1, variant)
        d = cells.to_device()
        step.react(d, dt)
        outs.append(d.to_host())
    for o in outs[1:]:
        for f in ("pri_molal", "total_out", "mnrl_rate", "mnrl_volfrac", "total_sorb_eq", "ionic_strength",
                  "iterations", "status"):
            if getattr(o, f) is not None:
                np.testing.assert_array_equal(getattr(outs[0], f), getattr(o, f), err_msg=f)
