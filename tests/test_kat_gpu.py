"""PFLOTRAN's own known answers through the GPU path: constraint speciation
and reaction steps on the device (fixtures from tests/golden/, tolerances
of the regression harness, regression_tests/ascem/batch/batch.cfg:15-19)."""
import math

import numpy as np
import pytest

import kat
from pflotran_gb300 import abi
from pflotran_gb300.lib import ReactionStep
from pflotran_gb300.network import default_options

pytestmark = pytest.mark.gpu


def _constraint_on_gpu(net, copt, b, fx, ncopies=64):
    """The deck's constraint solved for `ncopies` identical cells on the GPU."""
    import torch
    from pflotran_gb300.cells import CellBatch
    idx = np.zeros(ncopies, np.int64)
    many = b.subset(idx, net)
    many.iterations = np.zeros(ncopies, np.int32)
    many.status = np.zeros(ncopies, np.int32)
    many.total_out = np.zeros(net.N * ncopies)
    d = many.to_device()
    step = ReactionStep(net, copt)
    conc = np.repeat(np.asarray(fx["constraint"]["conc"], np.float64)[:, None], ncopies, axis=1)
    bad = step.equilibrate_constraints(d, fx["constraint"]["types"], torch.as_tensor(conc, device="cuda"))
    assert bad == 0
    return d.to_host()


def test_ion_exchange_valocchi_gold_gpu(oracle):
    fx = kat.load("kat_ion_exchange_valocchi.json")
    net = kat.build_network(fx, oracle)
    copt = default_options(use_isothermal=1, act_coef_update_frequency=abi.ACT_COEF_FREQUENCY_OFF,
                           residual_tol_kind=abi.RESIDUAL_ABSOLUTE,
                           max_relative_change_tolerance=1e-6, max_residual_tolerance=1e-12)
    g = _constraint_on_gpu(net, copt, kat.one_cell(net, fx, oracle), fx)
    names = [p["name"] for p in fx["primaries"]]
    n = g.ncells
    for i, nm in enumerate(names):
        for key, arr in ((f"Total {nm}", g.total_out), (f"Total Sorbed {nm}", g.total_sorb_eq)):
            v = arr.reshape(net.N, n)[i]
            assert np.abs(v - fx["gold"][key]).max() <= 1e-12, (key, v[0], fx["gold"][key])


@pytest.mark.parametrize("fixture,tol_total,tol_ph", [
    ("kat_calcite_kinetics.json", 1e-12, 1e-12),
    # the gold run's own Newton tolerance and step sequence (see the oracle test)
    ("kat_calcite_kinetics_volume_fractions.json", 1e-11, 1e-9)])
def test_calcite_kinetics_gold_gpu(oracle, fixture, tol_total, tol_ph):
    """Constraint speciation on the GPU, the reference's initialisation of
    the cell, then the deck's reaction steps on the GPU."""
    fx = kat.load(fixture)
    net = kat.build_network(fx, oracle)
    copt = default_options(use_isothermal=1, residual_tol_kind=abi.RESIDUAL_ABSOLUTE,
                           max_relative_change_tolerance=1e-6, max_residual_tolerance=1e-12)
    g = _constraint_on_gpu(net, copt, kat.one_cell(net, fx, oracle), fx, ncopies=32)
    kat.start_from_initial_condition(oracle, net, g)
    d = g.to_device()
    sopt = default_options(use_isothermal=1, residual_tol_kind=abi.RESIDUAL_RELATIVE, max_residual_tolerance=1e-15,
                           max_relative_change_tolerance=0.0, max_iterations=100, update_kinetic_state=1)
    step = ReactionStep(net, sopt)
    I_prev = None
    for dt in kat.step_sizes(fx):
        d.total.copy_(d.total_out)
        I_prev = float(d.ionic_strength[0])
        assert step.react(d, dt) == 0
    h = d.to_host()
    gp, _ = oracle.activity_lag(net.as_struct(), I_prev, net.N, net.Nc)
    n = h.ncells
    tot = h.total_out.reshape(net.N, n)
    for key, v, tol in (("Total H+", tot[0], tol_total), ("Total HCO3-", tot[1], tol_total),
                        ("Total Ca++", tot[2], tol_total), ("Calcite VF", h.mnrl_volfrac.reshape(-1, n)[0], 1e-12),
                        ("Calcite Rate", h.mnrl_rate.reshape(-1, n)[0], 1e-12)):
        assert np.abs(v - fx["gold"][key]).max() <= tol, (key, v[0], fx["gold"][key])
    ph = -math.log10(h.pri_molal[0] * gp[0])
    assert abs(ph - fx["gold"]["pH"]) <= tol_ph


def test_surface_complexation_1_gold_gpu(oracle):
    """surface-complexation-1 at time 0 (pH and charge-balance rows, one
    equilibrium surface-complexation site) solved on the GPU: aqueous totals
    within 1e-12 absolute, free sites and sorbed totals (up to 7.6e4
    mol/m^3, 14 printed digits) within 1e-12 relative."""
    fx = kat.load("kat_surface_complexation_1.json")
    net = kat.build_network(fx, oracle)
    copt = default_options(use_isothermal=1, residual_tol_kind=abi.RESIDUAL_ABSOLUTE,
                           max_relative_change_tolerance=1e-6, max_residual_tolerance=1e-12)
    g = _constraint_on_gpu(net, copt, kat.one_cell(net, fx, oracle), fx)
    names = [p["name"] for p in fx["primaries"]]
    n = g.ncells
    gold = fx["gold"]
    for i, nm in enumerate(names):
        v = g.total_out.reshape(net.N, n)[i]
        assert np.abs(v - gold[f"Total {nm}"]).max() <= 1e-12, (nm, v[0], gold[f"Total {nm}"])
        v = g.total_sorb_eq.reshape(net.N, n)[i]
        ref = gold[f"Total Sorbed {nm}"]
        assert np.abs(v - ref).max() <= 1e-12 * max(abs(ref), 1.0), (nm, v[0], ref)
    free = g.srfcplxrxn_free_site_conc.reshape(-1, n)[0]
    assert np.abs(free - gold["Free >FeOH_w"]).max() <= 1e-12 * gold["Free >FeOH_w"]
