"""GPU parity: the CUDA library against the oracle on identical seeded inputs.

Tolerance: 1e-10 scaled relative error (|x - y| / max(|y|, s), with s the
magnitude of the terms that make up the quantity) on free-ion molalities,
aqueous totals, mineral rates and volume fractions, sorbed totals and ionic
strength, at the headline convergence test (relative residual < 1e-12).
"""
import numpy as np
import pytest

from pflotran_gb300 import abi, workloads
from pflotran_gb300.lib import PfchemError, ReactionStep
from pflotran_gb300.network import default_options

from helpers import compare

pytestmark = pytest.mark.gpu
TOL = 1e-10


def run_both(oracle, net, opt, cells, dt, device=True, nthreads=8):
    ref = cells.copy()
    if ref.sec_molal is None:
        ref.sec_molal = np.zeros(max(net.Nc, 1) * cells.ncells)
    gpu = ref.copy()
    oracle.react(net.as_struct(), opt, dt, ref, 0, nthreads)
    step = ReactionStep(net, opt)
    if device:
        d = gpu.to_device()
        step.react(d, dt)
        gpu = d.to_host()
    else:
        step.react(gpu, dt)
    return ref, gpu, step


def assert_parity(net, gpu, ref, tol=TOL, mask=None):
    errs = compare(net, gpu, ref, mask=mask)
    bad = {k: v for k, v in errs.items() if not v <= tol}
    assert not bad, errs
    return errs


def test_calcite_column(oracle):
    net, opt, cells, dt = workloads.calcite_cells(100, seed=0)
    ref, gpu, _ = run_both(oracle, net, opt, cells, dt)
    assert (ref.status == 0).all() and (gpu.status == 0).all()
    assert_parity(net, gpu, ref)
    assert np.mean(gpu.iterations == ref.iterations) > 0.95


def test_calcite_grid_temperature_dependent(oracle):
    net, opt, cells, dt = workloads.calcite_cells(4096, seed=1, temperature_dependent=True)
    ref, gpu, _ = run_both(oracle, net, opt, cells, dt)
    assert (gpu.status == 0).all()
    assert_parity(net, gpu, ref)


def test_synthetic_network(oracle):
    net, opt, cells, dt = workloads.synthetic_cells(4096, seed=11)
    ref, gpu, step = run_both(oracle, net, opt, cells, dt)
    ok = (ref.status == 0) & (gpu.status == 0)
    assert ok.mean() > 0.99, (np.bincount(ref.status), np.bincount(gpu.status))
    assert_parity(net, gpu, ref, mask=ok)
    st = step.stats()
    assert st.ncells == 4096 and st.max_iterations == gpu.iterations.max()
    assert st.sum_iterations == gpu.iterations.sum()


def test_host_pointer_path(oracle):
    net, opt, cells, dt = workloads.calcite_cells(300, seed=2)
    ref, gpu, _ = run_both(oracle, net, opt, cells, dt, device=False)
    assert_parity(net, gpu, ref)


def test_interleaved_tran_xx_adapter(oracle):
    net, opt, cells, dt = workloads.calcite_cells(257, seed=3)
    ref = cells.copy()
    ref.sec_molal = np.zeros(net.Nc * cells.ncells)
    oracle.react(net.as_struct(), opt, dt, ref, 0, 4)
    ncomp = net.N + 2  # RTReact's tran_xx may carry immobile dofs after the aqueous ones
    tran = np.zeros((cells.ncells, ncomp))
    tran[:, :net.N] = cells.total.reshape(net.N, -1).T
    tran[:, net.N:] = 7.0
    gpu = cells.copy()
    gpu.total = None
    step = ReactionStep(net, opt)
    d = gpu.to_device()
    import torch
    t = torch.from_numpy(tran.ravel().copy()).cuda()
    step.react_interleaved(t, ncomp, d, dt)
    out = t.cpu().numpy().reshape(cells.ncells, ncomp)
    g = d.to_host()
    assert np.allclose(out[:, :net.N].T.ravel(), g.pri_molal, rtol=0, atol=0)
    assert (out[:, net.N:] == 7.0).all()
    ref.total = cells.total
    g.total = cells.total
    assert_parity(net, g, ref)


def test_reference_convergence_tests_literal_mode(oracle):
    """RReact's own tests: absolute 1e-12 residual and 1e-6 relative change
    (the last update discarded), literal accumulation.  RReact's literal
    residual is not divided by dt while its Jacobian is, so for dt != 1 s the
    Newton step is dt times too long and the clamped iteration is chaotic;
    at dt = 1 s the two agree and the path is well defined.  Cells whose
    iteration counts agree match."""
    net, opt, cells, _ = workloads.calcite_cells(512, seed=4)
    dt = 1.0
    opt = default_options(use_isothermal=1, residual_tol_kind=abi.RESIDUAL_ABSOLUTE,
                          accum_mode=abi.ACCUM_LITERAL, max_relative_change_tolerance=1e-6)
    ref, gpu, _ = run_both(oracle, net, opt, cells, dt)
    same = gpu.iterations == ref.iterations
    assert same.mean() > 0.98
    assert_parity(net, gpu, ref, mask=same)


def test_linear_formulation(oracle):
    net, opt, cells, dt = workloads.calcite_cells(256, seed=5)
    opt.use_log_formulation = 0
    ref, gpu, _ = run_both(oracle, net, opt, cells, dt)
    ok = (ref.status == 0) & (gpu.status == 0)
    assert ok.mean() > 0.98
    assert_parity(net, gpu, ref, mask=ok)


def test_newton_iteration_activity_update(oracle):
    net, opt, cells, dt = workloads.calcite_cells(256, seed=6)
    opt.act_coef_update_frequency = abi.ACT_COEF_FREQUENCY_NEWTON_ITER
    ref, gpu, _ = run_both(oracle, net, opt, cells, dt)
    assert_parity(net, gpu, ref)


def test_inactive_cells_are_skipped(oracle):
    net, opt, cells, dt = workloads.calcite_cells(200, seed=7)
    cells.active = (np.arange(200) % 3 != 0).astype(np.int32)
    before = cells.pri_molal.copy()
    ref, gpu, _ = run_both(oracle, net, opt, cells, dt)
    act = cells.active > 0
    assert (gpu.status[~act] == abi.CELL_INACTIVE).all()
    assert np.array_equal(gpu.pri_molal.reshape(3, -1)[:, ~act], before.reshape(3, -1)[:, ~act])
    assert_parity(net, gpu, ref, mask=act)


@pytest.mark.parametrize("ncells", [0, 1, 33])
def test_small_and_ragged_batches(oracle, ncells):
    """Batches of 0, 1 and 33 cells (not a multiple of a warp or a block):
    an empty batch (a rank without local cells: no arrays at all, or empty
    device arrays) returns 0; the others match the oracle on every cell."""
    from pflotran_gb300.cells import CellBatch
    net, opt, cells, dt = workloads.synthetic_cells(max(ncells, 1), seed=48)
    step = ReactionStep(net, opt)
    if ncells == 0:
        assert step.react(CellBatch(0), dt) == 0
        assert step.stats().ncells == 0
        assert step.react(CellBatch.allocate(net, 0).to_device(), dt) == 0
        return
    ref, gpu, _ = run_both(oracle, net, opt, cells, dt)
    assert np.array_equal(ref.status, gpu.status)
    ok = ref.status == 0
    assert_parity(net, gpu, ref, mask=ok & (ref.iterations == gpu.iterations))


def test_nonfinite_and_all_inactive_cells(oracle):
    """A cell whose totals are NaN stops with a non-converged status (the
    kernels' finiteness checks and capped inner loops) while every other
    cell of the batch matches the oracle; a batch with no active cell
    returns every cell INACTIVE and unchanged."""
    net, opt, cells, dt = workloads.calcite_cells(64, seed=49)
    tot = cells.total.reshape(net.N, -1)
    tot[:, 5] = np.nan
    ref, gpu, _ = run_both(oracle, net, opt, cells, dt)
    assert gpu.status[5] != 0 and ref.status[5] != 0
    rest = np.arange(64) != 5
    assert (gpu.status[rest] == 0).all()
    assert_parity(net, gpu, ref, mask=rest)
    net, opt, cells, dt = workloads.calcite_cells(64, seed=50)
    cells.active = np.zeros(64, np.int32)
    before = cells.pri_molal.copy()
    step = ReactionStep(net, opt)
    d = cells.to_device()
    assert step.react(d, dt) == 0
    g = d.to_host()
    assert (g.status == abi.CELL_INACTIVE).all()
    assert np.array_equal(g.pri_molal, before)


def test_alternative_guess_and_fallback(oracle):
    net, opt, cells, dt = workloads.synthetic_cells(2048, seed=8)
    ref, gpu, _ = run_both(oracle, net, opt, cells, dt)
    ok = (ref.status == 0)
    # a perfect alternative guess is taken and converges at the first residual
    c2 = cells.copy()
    c2.alt_guess = ref.pri_molal.copy()
    step = ReactionStep(net, opt)
    d = c2.to_device()
    step.react(d, dt)
    g2 = d.to_host()
    assert step.stats().alt_guess_used >= int(0.99 * ok.sum())
    assert (g2.iterations[ok] <= 2).mean() > 0.99
    assert_parity(net, g2, ref, mask=ok & (g2.status == 0))
    # a bad alternative guess is rejected and the plain path's answer results
    c3 = cells.copy()
    c3.alt_guess = cells.pri_molal * 1e3
    d = c3.to_device()
    step.react(d, dt)
    g3 = d.to_host()
    assert step.stats().alt_guess_used < 0.05 * cells.ncells
    assert_parity(net, g3, ref, mask=ok & (g3.status == 0))


def test_update_kinetic_state_entry_point(oracle):
    net, opt, cells, dt = workloads.calcite_cells(128, seed=9)
    opt.update_kinetic_state = 0
    ref, gpu, step = run_both(oracle, net, opt, cells, dt)
    before = gpu.mnrl_volfrac.copy()
    d = gpu.to_device()
    step.update_kinetic_state(d, dt)
    g = d.to_host()
    exp = np.maximum(before + g.mnrl_rate * net.minerals[0].extra["Vm"] * dt, 0.0)
    assert np.allclose(g.mnrl_volfrac, exp, rtol=1e-14, atol=0)


def test_rejects_unsupported_networks():
    from pflotran_gb300.network import ReactionNetwork
    net = ReactionNetwork([(f"P{i}", 1.0, 4.0) for i in range(17)])
    net.build()
    with pytest.raises(PfchemError, match="naqcomp"):
        ReactionStep(net, default_options())
    net = workloads.calcite_network()
    net.minerals[0].extra["pref"] = [dict(rate=1e-9, species=[("H+", 1.0, 0.0, -1.0)])]
    net.build()
    with pytest.raises(PfchemError, match="attenuation"):
        ReactionStep(net, default_options())


@pytest.mark.parametrize("kind", ["calcite_grid", "synthetic"])
@pytest.mark.parametrize("jacobian", [abi.JACOBIAN_REFERENCE, abi.JACOBIAN_EXACT])
@pytest.mark.parametrize("variant", [abi.KERNEL_SPECIALIZED, abi.KERNEL_GENERIC])
def test_mineral_rate_prefactors(oracle, kind, jacobian, variant):
    """Minerals with rate prefactors (reaction_mineral.F90:743-782 rate,
    :897-997 Jacobian): Monod terms in primaries and in an aqueous complex,
    parallel prefactors, a prefactor with its own activation energy (the
    calcite grid is temperature-dependent).  Both kernels, both Jacobians,
    against the oracle: 1e-10 on cells whose iteration counts agree, the
    per-cell bar against the root elsewhere."""
    from oracle import parity
    if kind == "calcite_grid":
        net, opt, cells, dt = workloads.calcite_cells(4096, seed=31, temperature_dependent=True)
    else:
        net, opt, cells, dt = workloads.synthetic_cells(4096, seed=32)
    workloads.add_rate_prefactors(net)
    opt.jacobian = jacobian
    ref = parity.solve(net, opt, dt, cells)
    step = ReactionStep(net, opt)
    if variant == abi.KERNEL_GENERIC:
        step.set_launch(64, 1, 8, abi.KERNEL_GENERIC)
    d = cells.to_device()
    d.sec_molal = None
    step.react(d, dt)
    gpu = d.to_host()
    ok = (ref.status == 0) & (gpu.status == 0)
    # the GPU reports the oracle's per-cell status (with the reference
    # Jacobian a couple of cells of the synthetic draw reach the cap in both)
    assert np.mean(ref.status == gpu.status) > 0.999, (np.bincount(ref.status), np.bincount(gpu.status))
    assert ok.mean() > 0.99
    same = ok & (ref.iterations == gpu.iterations)
    assert same.sum() > 0.98 * ok.sum()
    gpu.sec_molal = None
    assert_parity(net, gpu, ref, mask=same)
    rates = ref.mnrl_rate.reshape(-1, cells.ncells)[:net.Nm]
    assert (np.abs(rates) > 0).any()
    truth = parity.truth_solve(net, opt, dt, cells, ref)
    for q, (bar, *_r) in parity.per_cell_bar(net, gpu, ref, truth, mask=ok & (truth.status == 0)).items():
        assert bar.all(), (q, int((~bar).sum()))


def test_calcite_grid_full_size_sampled(oracle):
    """100^3 cells on the GPU; a seeded sample of 4000 cells re-solved by the oracle."""
    net, opt, cells, dt = workloads.calcite_cells(1_000_000, seed=10, temperature_dependent=True)
    step = ReactionStep(net, opt)
    d = cells.to_device()
    d.sec_molal = None
    import torch
    d.sec_molal = torch.zeros(net.Nc * cells.ncells, dtype=torch.float64, device="cuda")
    assert step.react(d, dt) == 0
    g = d.to_host()
    idx = np.sort(np.random.default_rng(0).choice(cells.ncells, 4000, replace=False))
    sub = cells.subset(idx, net)
    sub.sec_molal = np.zeros(net.Nc * len(idx))
    oracle.react(net.as_struct(), opt, dt, sub, 0, 8)
    assert_parity(net, g.subset(idx, net), sub)


@pytest.mark.parametrize("kind", ["calcite", "synthetic"])
def test_generic_table_driven_kernel(oracle, kind):
    """The library's built-in table-driven kernel (used when the specialized
    kernel is not selected, and by the allocation-free entry point)."""
    if kind == "calcite":
        net, opt, cells, dt = workloads.calcite_cells(2048, seed=12, temperature_dependent=True)
    else:
        net, opt, cells, dt = workloads.synthetic_cells(2048, seed=13)
    ref = cells.copy()
    ref.sec_molal = np.zeros(max(net.Nc, 1) * cells.ncells)
    oracle.react(net.as_struct(), opt, dt, ref, 0, 8)
    step = ReactionStep(net, opt)
    step.set_launch(64, 1, 8, variant=abi.KERNEL_GENERIC)
    gpu = cells.copy()
    gpu.sec_molal = np.zeros(max(net.Nc, 1) * cells.ncells)
    d = gpu.to_device()
    step.react(d, dt)
    g = d.to_host()
    ok = (ref.status == 0) & (g.status == 0)
    assert ok.mean() > 0.99
    assert_parity(net, g, ref, mask=ok)


def test_specialized_kernel_is_default():
    net, opt, cells, dt = workloads.calcite_cells(16, seed=14)
    step = ReactionStep(net, opt)
    assert step.launch().variant in (abi.KERNEL_SPECIALIZED, abi.KERNEL_SPECIALIZED_COMPACT)


@pytest.mark.parametrize("jac", [abi.JACOBIAN_REFERENCE, abi.JACOBIAN_EXACT])
def test_compact_layout_equals_augmented_layout(jac):
    """The compact shared-memory layout (right-hand side in registers) does
    the same operations in the same order: bit-identical results."""
    net, opt, cells, dt = workloads.synthetic_cells(8192, seed=61)
    opt.jacobian = jac
    out = {}
    for variant in (abi.KERNEL_SPECIALIZED, abi.KERNEL_SPECIALIZED_COMPACT):
        step = ReactionStep(net, opt)
        step.set_launch(32, 1, 8, variant=variant)
        d = cells.to_device()
        step.react(d, dt)
        out[variant] = d.to_host()
    a, b = out[abi.KERNEL_SPECIALIZED], out[abi.KERNEL_SPECIALIZED_COMPACT]
    for f in ("pri_molal", "total_out", "mnrl_rate", "mnrl_volfrac", "total_sorb_eq", "iterations", "status"):
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f)


@pytest.mark.parametrize("variant", [abi.KERNEL_SPECIALIZED, abi.KERNEL_GENERIC])
def test_exact_jacobian(oracle, variant):
    """The exact-Jacobian option against the oracle with the same option (same
    Newton path), and against the reference Jacobian (same equations and
    root): the answers agree to what the 1e-12 relative residual allows and
    the exact Jacobian needs fewer iterations."""
    net, opt, cells, dt = workloads.synthetic_cells(4096, seed=17)
    opt.jacobian = abi.JACOBIAN_EXACT
    ref = cells.copy()
    ref.sec_molal = np.zeros(net.Nc * cells.ncells)
    d = ref.copy().to_device()
    oracle.react(net.as_struct(), opt, dt, ref, 0, 8)
    step = ReactionStep(net, opt)
    if variant == abi.KERNEL_GENERIC:
        step.set_launch(64, 1, 8, variant=abi.KERNEL_GENERIC)
    step.react(d, dt)
    g = d.to_host()
    ok = (ref.status == 0) & (g.status == 0)
    assert ok.mean() > 0.999
    assert_parity(net, g, ref, mask=ok)
    assert np.mean(g.iterations == ref.iterations) > 0.98
    # against the reference Jacobian
    opt_ref = default_options(use_isothermal=1)
    base = cells.copy()
    base.sec_molal = np.zeros(net.Nc * cells.ncells)
    oracle.react(net.as_struct(), opt_ref, dt, base, 0, 8)
    # two Newton paths stop at different points inside the 1e-12 relative
    # residual ball; on this draw the worst cell differs by 1.8e-10
    both = ok & (base.status == 0)
    errs = compare(net, g, base, mask=both)
    assert errs["total"] <= 1e-9 and errs["mnrl_rate"] <= 1e-9 and errs["mnrl_volfrac"] <= 1e-9, errs
    assert errs["pri_molal"] <= 1e-8, errs
    assert g.iterations[both].mean() < 0.8 * base.iterations[both].mean()


@pytest.mark.parametrize("kind,jac", [("synthetic", abi.JACOBIAN_REFERENCE), ("synthetic", abi.JACOBIAN_EXACT),
                                      ("calcite", abi.JACOBIAN_REFERENCE)])
def test_reaction_blocks(oracle, kind, jac):
    """Global-implicit per-cell blocks (residual, Jacobian, totals and their
    derivatives) against the oracle at the same state; each block compared
    with its own largest entry as the scale."""
    if kind == "calcite":
        net, opt, cells, dt = workloads.calcite_cells(2048, seed=31, temperature_dependent=True)
    else:
        net, opt, cells, dt = workloads.synthetic_cells(2048, seed=32)
    opt.jacobian = jac
    cells.sec_molal = np.zeros(max(net.Nc, 1) * cells.ncells)
    ref = cells.copy()
    d = cells.copy().to_device()
    bo = oracle.reaction_blocks(net.as_struct(), opt, ref)
    step = ReactionStep(net, opt)
    bg = {k: v.cpu().numpy() for k, v in step.reaction_blocks(d).items()}
    g = d.to_host()
    ok = (ref.status == 0) & (g.status == 0)
    assert ok.mean() > 0.99
    for k in ("jac", "dtotal", "dtotal_sorb"):
        scale = np.abs(bo[k]).max(axis=(1, 2), keepdims=True) + 1e-300
        err = (np.abs(bg[k] - bo[k]) / scale)[ok].max()
        assert err <= 1e-10, (k, err)
    for k in ("res", "total", "total_sorb"):
        scale = np.abs(bo[k]).max(axis=0, keepdims=True) + 1e-300
        err = (np.abs(bg[k] - bo[k]) / scale)[:, ok].max()
        assert err <= 1e-10, (k, err)
    rate_scale = np.abs(ref.mnrl_rate).reshape(-1, cells.ncells).max(axis=0) + 1e-300
    err = (np.abs(g.mnrl_rate - ref.mnrl_rate).reshape(-1, cells.ncells) / rate_scale)[:, ok].max()
    assert err <= 1e-10


def test_mineral_property_update(oracle):
    """Porosity and mineral surface area from the volume fractions, GPU vs oracle."""
    import torch
    net, opt, cells, dt = workloads.synthetic_cells(4096, seed=33)
    n, Nm = cells.ncells, net.Nm
    rng = np.random.default_rng(3)
    cells.mnrl_volfrac = rng.uniform(0.0, 0.05, Nm * n)
    vf0 = rng.uniform(0.0, 0.05, Nm * n)
    vf0[::5] = 0.0
    host = {"surf_area_vol_frac_pwr": np.full(Nm, 2.0 / 3.0), "surf_area_porosity_pwr": np.linspace(0.5, 1.5, Nm),
            "mnrl_volfrac0": vf0, "mnrl_area0": rng.uniform(0.5, 2.0, Nm * n), "porosity0": np.full(n, 0.3),
            "porosity": np.zeros(n)}
    dev = {k: torch.as_tensor(v, device="cuda") for k, v in host.items()}
    ref = cells.copy()
    oracle.update_mineral_properties(net.as_struct(), ref,
                                     abi.mineral_update(host, surface_area_with_porosity=1, minimum_porosity=0.76))
    step = ReactionStep(net, opt)
    d = cells.to_device()
    step.update_mineral_properties(d, abi.mineral_update(dev, surface_area_with_porosity=1, minimum_porosity=0.76))
    g = d.to_host()
    np.testing.assert_array_equal(dev["porosity"].cpu().numpy(), host["porosity"])
    np.testing.assert_allclose(g.mnrl_area, ref.mnrl_area, rtol=1e-14, atol=0)


def test_constraint_speciation(oracle):
    """Batched constraint speciation (pH, log-free, mineral and total rows),
    GPU vs oracle on identical inputs."""
    import torch
    from helpers import constraint_problem
    net, _, cells, dt = workloads.synthetic_cells(4096, seed=42)
    copt = default_options(use_isothermal=1, residual_tol_kind=abi.RESIDUAL_ABSOLUTE,
                           max_relative_change_tolerance=1e-6, max_residual_tolerance=1e-12)
    types, minerals, values = constraint_problem(oracle, net, copt, cells, {0: "ph", 5: "log", 3: "mineral:4"})
    ref = cells.copy()
    ref.sec_molal = np.zeros(net.Nc * cells.ncells)
    d = ref.copy().to_device()
    bad_ref = oracle.equilibrate_constraints(net.as_struct(), copt, ref, types, values, minerals)
    step = ReactionStep(net, copt)
    bad = step.equilibrate_constraints(d, types, torch.as_tensor(values, device="cuda"), minerals)
    g = d.to_host()
    # a few cells of this draw cannot reach saturation of the constraining
    # mineral with the other rows held (the reference's iteration fails too)
    assert bad <= 0.01 * cells.ncells and bad_ref <= 0.01 * cells.ncells
    ok = (g.status == 0) & (ref.status == 0)
    assert ok.sum() >= cells.ncells - max(bad, bad_ref) - 2
    assert np.mean(g.iterations[ok] == ref.iterations[ok]) > 0.98
    assert_parity(net, g, ref, mask=ok)


def test_constraint_gas_and_sorbed_rows(oracle):
    """GAS rows (reaction.F90:1720-1751; one in log10 form) and a TOTAL_SORB
    row (:1608-1614) in the batched constraint speciation, GPU vs oracle on
    identical inputs; invalid rows are rejected."""
    import torch
    from helpers import constraint_problem, gas_sorb_rows
    net, _, cells, dt = workloads.synthetic_cells(4096, seed=45)
    workloads.add_passive_gases(net)
    copt = default_options(use_isothermal=1, residual_tol_kind=abi.RESIDUAL_ABSOLUTE,
                           max_relative_change_tolerance=1e-6, max_residual_tolerance=1e-12)
    types, spec, values = constraint_problem(oracle, net, copt, cells, gas_sorb_rows(net))
    ref = cells.copy()
    ref.sec_molal = np.zeros(net.Nc * cells.ncells)
    d = ref.copy().to_device()
    bad_ref = oracle.equilibrate_constraints(net.as_struct(), copt, ref, types, values, spec, gases=net.gas_table())
    step = ReactionStep(net, copt)
    bad = step.equilibrate_constraints(d, types, torch.as_tensor(values, device="cuda"), spec)
    g = d.to_host()
    # a few cells of the draw do not converge in the reference's iteration
    # (non-positive molality after a linear update); the GPU reports the
    # oracle's status per cell
    assert bad <= 0.01 * cells.ncells and bad_ref <= 0.01 * cells.ncells
    assert np.mean(g.status == ref.status) > 0.995, (np.bincount(g.status), np.bincount(ref.status))
    ok = (g.status == 0) & (ref.status == 0)
    same = ok & (g.iterations == ref.iterations)
    assert same.sum() > 0.98 * ok.sum()
    assert_parity(net, g, ref, mask=same)
    sorb_g = g.total_sorb_eq.reshape(net.N, -1)
    sorb_r = ref.total_sorb_eq.reshape(net.N, -1)
    js = int(np.flatnonzero(types == abi.CONSTRAINT_TOTAL_SORB)[0])
    np.testing.assert_allclose(sorb_g[js][ok], values[js][ok], rtol=1e-10)
    np.testing.assert_allclose(sorb_g[js][ok], sorb_r[js][ok], rtol=1e-10)
    # invalid rows
    t2 = types.copy()
    s2 = spec.copy()
    s2[np.flatnonzero(types == abi.CONSTRAINT_GAS)[0]] = 3
    with pytest.raises(PfchemError, match="passive gas id"):
        step.equilibrate_constraints(d, t2, torch.as_tensor(values, device="cuda"), s2)
    cnet, _, ccells, _ = workloads.calcite_cells(64, seed=46)
    cstep = ReactionStep(cnet, copt)
    with pytest.raises(PfchemError, match="without sorption"):
        cstep.equilibrate_constraints(ccells.to_device(), [1, 8, 1], torch.zeros((3, 64), dtype=torch.float64,
                                                                                   device="cuda"))


def test_constraint_gas_row_temperature_dependent(oracle):
    """A column's initial water (free H+, HCO3- from 1e-3 bar CO2(g), Ca++ at
    calcite saturation) on the temperature-dependent calcite grid: log K(T)
    of the gas from its fit, GPU vs oracle."""
    import torch
    net, _, cells, dt = workloads.calcite_cells(4096, seed=47, temperature_dependent=True)
    workloads.add_passive_gases(net)
    copt = default_options(use_isothermal=0, residual_tol_kind=abi.RESIDUAL_ABSOLUTE,
                           max_relative_change_tolerance=1e-6, max_residual_tolerance=1e-12)
    n = cells.ncells
    types = np.array([abi.CONSTRAINT_FREE, abi.CONSTRAINT_GAS, abi.CONSTRAINT_MINERAL], np.int32)
    spec = np.array([0, 1, 1], np.int32)
    rng = np.random.default_rng(5)
    values = np.ascontiguousarray(np.stack([10.0 ** rng.uniform(-8.5, -7.5, n), -rng.uniform(2.5, 3.5, n),
                                            np.full(n, 5e-4)]))
    ref = cells.copy()
    ref.sec_molal = np.zeros(net.Nc * n)
    d = ref.copy().to_device()
    assert oracle.equilibrate_constraints(net.as_struct(), copt, ref, types, values, spec, gases=net.gas_table()) == 0
    step = ReactionStep(net, copt)
    assert step.equilibrate_constraints(d, types, torch.as_tensor(values, device="cuda"), spec) == 0
    g = d.to_host()
    same = g.iterations == ref.iterations
    assert same.mean() > 0.98
    assert_parity(net, g, ref, mask=same)


@pytest.mark.parametrize("warm", [False, True])
def test_large_host_batch_equals_device_batch(warm):
    """A host-pointer batch of 2^20 cells (staged through the device) gives
    every cell the device batch's result, bit for bit, with and without the
    warm start."""
    from pflotran_gb300.surrogate import fit, generate
    net = workloads.synthetic_network()
    _, opt, cells, dt = workloads.synthetic_cells(1 << 20, seed=51, net=net, device="cuda")
    step = ReactionStep(net, opt)
    if warm:
        X, molal = generate(step, lambda m, s: workloads.synthetic_cells(m, seed=s, net=net, device="cuda")[2],
                            131072, 52, dt, chunk=131072)
        fit(step, X, molal, epochs=2, batch=4096)
        step.surrogate_enable(True)
    d = cells.to_device()
    step.react(d, dt)
    st_dev = step.stats()
    g_dev = d.to_host()
    h = cells.copy()
    step.react(h, dt)
    st_host = step.stats()
    for f in ("pri_molal", "total_out", "mnrl_rate", "mnrl_volfrac", "total_sorb_eq", "ionic_strength",
              "eqionx_ref_cation_sorbed_conc", "srfcplxrxn_free_site_conc", "iterations", "status"):
        np.testing.assert_array_equal(getattr(h, f), getattr(g_dev, f), err_msg=f)
    assert st_host.sum_iterations == st_dev.sum_iterations
    assert st_host.nonconverged == st_dev.nonconverged
    assert st_host.alt_guess_used == st_dev.alt_guess_used


@pytest.mark.parametrize("kind", ["calcite", "synthetic"])
def test_error_statement_against_extended_precision(oracle, kind):
    """GPU vs the double oracle (the parity bar) and both against the
    oracle's long-double instantiation (binary128 on aarch64, 80-bit
    extended on x86-64), max and 99th percentile, on totals, mineral volume
    fractions and rates.  The extended-precision solve stops at the same
    1e-12 relative residual, so its distance to either double solve is the
    convergence tolerance times the cell's conditioning.  Bar, per cell and
    quantity: within 1e-10 of the double oracle, or, on a cell where the
    double oracle itself is further than 1e-10 from the extended-precision
    solution (an ill-conditioned cell whose double Newton path the
    platform's libm rounding moves), within 1e-10 of the latter; and the
    GPU's p99 distance to the extended solution no worse than the double
    oracle's beyond the 1e-12 level.  The report goes to the path in
    PFCHEM_ERROR_STATEMENT when it is set."""
    import json
    import os
    if kind == "calcite":
        net, opt, cells, dt = workloads.calcite_cells(4096, seed=21, temperature_dependent=True)
    else:
        net, opt, cells, dt = workloads.synthetic_cells(2048, seed=21)
    ref, gpu, _ = run_both(oracle, net, opt, cells, dt)
    ext = cells.copy()
    if ext.sec_molal is None:
        ext.sec_molal = np.zeros(max(net.Nc, 1) * cells.ncells)
    oracle.react(net.as_struct(), opt, dt, ext, 1, os.cpu_count() or 1)
    ok = (ref.status == 0) & (gpu.status == 0) & (ext.status == 0)
    assert ok.mean() > 0.99
    from helpers import cell_errors, error_statement
    gd, ge, de = cell_errors(net, gpu, ref), cell_errors(net, gpu, ext), cell_errors(net, ref, ext)
    ill = {q: ok & (de[q] > TOL) for q in gd}
    rep = {"gpu_vs_double": error_statement(net, gpu, ref, ok),
           "gpu_vs_extended": error_statement(net, gpu, ext, ok),
           "double_vs_extended": error_statement(net, ref, ext, ok),
           "double_further_than_bar_from_extended": {q: int(m.sum()) for q, m in ill.items()},
           "cells": int(ok.sum()), "long_double_digits": int(np.finfo(np.longdouble).precision)}
    print(kind, json.dumps(rep))
    path = os.environ.get("PFCHEM_ERROR_STATEMENT")
    if path:
        old = json.load(open(path)) if os.path.exists(path) else {}
        old[kind] = rep
        with open(path, "w") as f:
            json.dump(old, f, indent=1)
    for q in gd:
        good = np.where(ill[q], ge[q] <= TOL, gd[q] <= TOL)
        assert good[ok].all(), (q, rep)
    for q, e in rep["gpu_vs_extended"].items():
        d = rep["double_vs_extended"][q]
        assert e["max"] <= 1e-8, (q, e)
        assert e["p99"] <= 4 * d["p99"] + 1e-12, (q, e, d)


def test_network_from_database_in_a_swapped_basis(oracle, tmp_path):
    """A network read from a PFLOTRAN-format database with CO2(aq) primary
    instead of HCO3- (basis swap) through the GPU library: parity with the
    oracle in that basis at the usual bar."""
    import kat
    db, a, b = kat.calcite_networks_two_bases(tmp_path / "calcite.dat")
    _, opt, ca, dt = workloads.calcite_cells(4096, seed=9, net=a)
    ca.sec_molal = np.zeros(a.Nc * ca.ncells)
    cb = kat.cells_in_basis(oracle, a, b, ca)
    ref, gpu, _ = run_both(oracle, b, opt, cb, dt)
    assert (ref.status == 0).all() and (gpu.status == 0).all()
    assert_parity(b, gpu, ref)


@pytest.mark.parametrize("kind", ["calcite_grid", "synthetic"])
@pytest.mark.parametrize("mode", ["timestep_specialized", "timestep_generic", "newton_iter"])
def test_newton_activity_algorithm(oracle, kind, mode):
    """ACT_COEF_ALGORITHM_NEWTON (reaction.F90:3846-3990): the ionic
    strength iterated with the primaries' entry activities held, at step
    start (TIMESTEP: network-specialized and table-driven kernels) or at
    every Newton iteration (NEWTON_ITER: the table-driven kernel, which the
    library selects for it).  Against the oracle at 1e-10 on cells whose
    iteration counts agree, the per-cell bar against the root elsewhere;
    cells whose activity loop exceeds its 50 passes report the same status."""
    from oracle import parity
    if kind == "calcite_grid":
        net, opt, cells, dt = workloads.calcite_cells(4096, seed=33, temperature_dependent=True)
    else:
        net, opt, cells, dt = workloads.synthetic_cells(4096, seed=34)
    opt.act_coef_update_algorithm = abi.ACT_COEF_ALGORITHM_NEWTON
    opt.act_coef_update_frequency = (abi.ACT_COEF_FREQUENCY_NEWTON_ITER if mode == "newton_iter"
                                     else abi.ACT_COEF_FREQUENCY_TIMESTEP)
    ref = parity.solve(net, opt, dt, cells)
    step = ReactionStep(net, opt)
    if mode == "timestep_generic":
        step.set_launch(64, 1, 8, abi.KERNEL_GENERIC)
    if mode == "newton_iter":
        assert step.launch().variant == abi.KERNEL_GENERIC
        with pytest.raises(PfchemError, match="NEWTON activity"):
            step.set_launch(32, 1, 1, abi.KERNEL_SPECIALIZED)
    d = cells.to_device()
    d.sec_molal = None
    step.react(d, dt)
    gpu = d.to_host()
    ok = (ref.status == 0) & (gpu.status == 0)
    assert np.mean(ref.status == gpu.status) > 0.999, (np.bincount(ref.status), np.bincount(gpu.status))
    assert ok.mean() > 0.97
    same = ok & (ref.iterations == gpu.iterations)
    assert same.sum() > 0.98 * ok.sum()
    gpu.sec_molal = None
    assert_parity(net, gpu, ref, mask=same)
    truth = parity.truth_solve(net, opt, dt, cells, ref)
    for q, (bar, *_r) in parity.per_cell_bar(net, gpu, ref, truth, mask=ok & (truth.status == 0)).items():
        assert bar.all(), (q, int((~bar).sum()))


@pytest.mark.parametrize("flag_in", [0, 1])
def test_mineral_armoring(oracle, flag_in):
    """Mineral armoring (realization_subsurface.F90:1737-1765): two minerals
    armored by others, the flag carried across cells; GPU vs the oracle's
    serial restatement, area and the flag after the last cell."""
    import torch
    net, opt, cells, dt = workloads.synthetic_cells(4096, seed=35)
    n, Nm = cells.ncells, net.Nm
    rng = np.random.default_rng(4)
    cells.mnrl_volfrac = rng.uniform(0.0, 0.05, Nm * n)
    crit = np.zeros(Nm)
    crit[0], crit[2] = 0.03, 0.02
    armor = np.arange(1, Nm + 1, dtype=np.int32)
    armor[0], armor[2] = 2, 4
    host = {"surf_area_vol_frac_pwr": np.full(Nm, 2.0 / 3.0), "mnrl_volfrac0": rng.uniform(0.0, 0.05, Nm * n),
            "mnrl_area0": rng.uniform(0.5, 2.0, Nm * n), "armor_crit_vol_frac": crit, "armor_mineral": armor}
    out_ref = np.full(1, -1, np.int32)
    ref = cells.copy()
    oracle.update_mineral_properties(net.as_struct(), ref, abi.mineral_update(
        dict(host, armor_flag_out=out_ref), update_porosity=0, armor_flag=flag_in))
    dev = {k: torch.as_tensor(v, device="cuda") for k, v in host.items()}
    out_gpu = np.full(1, -1, np.int32)
    step = ReactionStep(net, opt)
    d = cells.to_device()
    step.update_mineral_properties(d, abi.mineral_update(dict(dev, armor_flag_out=out_gpu), update_porosity=0,
                                                         armor_flag=flag_in))
    g = d.to_host()
    np.testing.assert_allclose(g.mnrl_area, ref.mnrl_area, rtol=1e-14, atol=0)
    area = ref.mnrl_area.reshape(Nm, n)
    assert (area[0] == 0).any() and (area[0] > 0).any() and (area[2] == 0).any()
    assert out_gpu[0] == out_ref[0] in (0, 1)
