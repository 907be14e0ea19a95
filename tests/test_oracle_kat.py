"""The oracle against PFLOTRAN's own known answers.

Fixtures: tests/golden/*.json, written from the reference's regression decks
and gold files by tests/golden/make_kat_fixtures.py.  The tolerances are the
regression harness's (regression_tests/ascem/batch/batch.cfg:15-19: 1e-12
absolute for concentrations, rates and volume fractions) unless stated.
"""
import numpy as np
import pytest

import kat


def test_ifc67_density_matches_pfunit_value(oracle):
    # src/pflotran/unittests/test_eos_water.pf:131-157 pins 998.32340486329440 kg/m^3 at 20 C
    assert abs(oracle.ifc67_density(20.0, 101325.0) - 998.32340486329440) <= 1e-12


def test_ion_exchange_valocchi_gold(oracle):
    """ion-exchange-valocchi: constraint speciation + RTotalSorbEqIonx (Z != Z inner Newton)."""
    out, gold = kat.run_ion_exchange_valocchi(oracle)
    for key in ("Total Na+", "Total Ca++", "Total Mg++", "Total Cl-", "Total Sorbed Na+",
                "Total Sorbed Ca++", "Total Sorbed Mg++", "Total Sorbed Cl-"):
        assert abs(out[key] - gold[key]) <= 1e-12, (key, out[key], gold[key])


@pytest.mark.parametrize("precision", [0, 1])
def test_calcite_kinetics_gold(oracle, precision):
    """calcite-kinetics: the initialised constraint state, then 500 steps of
    0.5 s of RTotal + LAG activity (TIMESTEP) + RKineticMineral +
    RUpdateKineticState.  Totals, calcite volume fraction, rate and pH meet
    the harness's 1e-12 absolute."""
    out, gold = kat.run_calcite_kinetics(oracle, precision)
    for key in ("Total H+", "Total HCO3-", "Total Ca++", "Calcite VF", "Calcite Rate", "pH"):
        assert abs(out[key] - gold[key]) <= 1e-12, (key, out[key], gold[key])


def test_rsolve_matches_dense_solve(oracle):
    rng = np.random.default_rng(0)
    for n in (3, 7, 12):
        A = rng.standard_normal((n, n)) + n * np.eye(n)
        r = rng.standard_normal(n)
        conc = np.exp(rng.uniform(-5, 0, n))
        u = np.zeros(n)
        Ac = A.copy()
        assert oracle.lib().pfo_rsolve(n, r.copy().ctypes.data, Ac.ctypes.data, conc.ctypes.data, 1, u.ctypes.data) == 0
        ref = np.linalg.solve(A * conc[None, :], r)
        assert np.allclose(u, ref, rtol=1e-10, atol=1e-12)


def test_rsolve_reports_singular_row(oracle):
    A = np.eye(3)
    A[1, :] = 0.0
    u = np.zeros(3)
    r = np.ones(3)
    c = np.ones(3)
    assert oracle.lib().pfo_rsolve(3, r.ctypes.data, A.ctypes.data, c.ctypes.data, 0, u.ctypes.data) == 1


def test_alternative_guess_choice(oracle):
    """The two-guess start: the converged solution offered as the second
    guess is taken and needs one iteration; an invalid second guess leaves
    the plain solve unchanged bit for bit."""
    from pflotran_gb300 import workloads
    net, opt, cells, dt = workloads.calcite_cells(64, seed=3)
    plain = cells.copy()
    oracle.react(net.as_struct(), opt, dt, plain, 0, 4)
    assert (plain.status == 0).all()
    warm = cells.copy()
    warm.alt_guess = plain.pri_molal.copy()
    oracle.react(net.as_struct(), opt, dt, warm, 0, 4)
    assert (warm.status == 0).all()
    assert (warm.iterations == 1).all()
    assert np.array_equal(warm.pri_molal, plain.pri_molal)
    bad = cells.copy()
    bad.alt_guess = -np.ones_like(cells.pri_molal)
    oracle.react(net.as_struct(), opt, dt, bad, 0, 4)
    assert np.array_equal(bad.pri_molal, plain.pri_molal)
    assert np.array_equal(bad.iterations, plain.iterations)


def test_mineral_property_update(oracle):
    """Porosity = max(1 - sum phi_m, min) and area = area0 (phi/phi0)^p_vf
    (por/por0)^p_por, with phi0 = 0 keeping the volume-fraction factor at 1."""
    from pflotran_gb300 import abi, workloads
    net, opt, cells, dt = workloads.synthetic_cells(64, seed=5)
    n, Nm = cells.ncells, net.Nm
    rng = np.random.default_rng(1)
    cells.mnrl_volfrac = rng.uniform(0.0, 0.05, Nm * n)
    vf0 = rng.uniform(0.0, 0.05, Nm * n)
    vf0[::7] = 0.0
    arrays = {"surf_area_vol_frac_pwr": np.full(Nm, 2.0 / 3.0), "surf_area_porosity_pwr": np.linspace(0.5, 1.5, Nm),
              "mnrl_volfrac0": vf0, "mnrl_area0": rng.uniform(0.5, 2.0, Nm * n), "porosity0": np.full(n, 0.3),
              "porosity": np.zeros(n)}
    mu = abi.mineral_update(arrays, surface_area_with_porosity=1, minimum_porosity=0.75)
    oracle.update_mineral_properties(net.as_struct(), cells, mu)
    vf = cells.mnrl_volfrac.reshape(Nm, n)
    por = np.maximum(1.0 - vf.sum(0), 0.75)
    assert np.array_equal(arrays["porosity"], por)
    v0 = vf0.reshape(Nm, n)
    vs = np.where(v0 > 0, (vf / np.where(v0 > 0, v0, 1.0)) ** (2.0 / 3.0), 1.0)
    ps = (por / 0.3)[None, :] ** arrays["surf_area_porosity_pwr"][:, None]
    want = arrays["mnrl_area0"].reshape(Nm, n) * ps * vs
    np.testing.assert_allclose(cells.mnrl_area.reshape(Nm, n), want, rtol=1e-14)


def test_constraint_rows_are_satisfied(oracle):
    """Batched constraint speciation with pH, log-free, mineral and total rows:
    the solution meets every row (pH of the final activity, saturation of the
    constraining mineral, totals)."""
    from pflotran_gb300 import abi, workloads
    from helpers import constraint_problem
    net, _, cells, dt = workloads.synthetic_cells(64, seed=41)
    copt = workloads.default_options(use_isothermal=1, residual_tol_kind=abi.RESIDUAL_ABSOLUTE,
                                     max_relative_change_tolerance=1e-6, max_residual_tolerance=1e-12)
    rows = {0: "ph", 5: "log", 3: "mineral:4"}
    types, minerals, values = constraint_problem(oracle, net, copt, cells, rows)
    out = cells.copy()
    out.sec_molal = np.zeros(net.Nc * cells.ncells)
    bad = oracle.equilibrate_constraints(net.as_struct(), copt, out, types, values, minerals)
    assert bad == 0, np.bincount(out.status)
    N, n = net.N, cells.ncells
    m = out.pri_molal.reshape(N, n)
    tot = out.total_out.reshape(N, n)
    for j in range(N):
        if types[j] == abi.CONSTRAINT_TOTAL:
            assert np.abs(tot[j] - values[j]).max() <= 1e-10 * np.abs(values[j]).max()
    np.testing.assert_allclose(np.log10(m[5] * cells.den_kg * 1e-3), values[5], rtol=0, atol=1e-12)
    # mineral 4 (P2 + P3) at saturation with the final activity coefficients
    gp = np.array([oracle.activity_lag(net.as_struct(), float(I), N, net.Nc)[0] for I in out.ionic_strength]).T
    mn = net.minerals[3]
    lnQK = -mn.logK * 2.30258509299 + sum(nu * np.log(m[net.idx(s)] * gp[net.idx(s)])
                                         for s, nu in zip(mn.species, mn.stoich))
    assert np.abs(lnQK).max() < 1e-6


def test_constraint_gas_and_sorbed_rows_are_satisfied(oracle):
    """GAS rows (reaction.F90:1720-1751: the gas reaction's ln QK equals the
    log of the partial pressure; a value <= 0 is log10 of it) and a
    TOTAL_SORB row (:1608-1614): the solution meets every row and is the
    cells' own state; log10 and plain partial pressures give the same answer."""
    from pflotran_gb300 import abi, workloads
    from helpers import constraint_problem, gas_sorb_rows
    net, _, cells, dt = workloads.synthetic_cells(64, seed=43)
    workloads.add_passive_gases(net)
    copt = workloads.default_options(use_isothermal=1, residual_tol_kind=abi.RESIDUAL_ABSOLUTE,
                                     max_relative_change_tolerance=1e-6, max_residual_tolerance=1e-12)
    rows = gas_sorb_rows(net)
    types, spec, values = constraint_problem(oracle, net, copt, cells, rows)
    assert (types == abi.CONSTRAINT_GAS).sum() == 2 and (types == abi.CONSTRAINT_TOTAL_SORB).sum() == 1
    out = cells.copy()
    out.sec_molal = np.zeros(net.Nc * cells.ncells)
    gases = net.gas_table()
    bad = oracle.equilibrate_constraints(net.as_struct(), copt, out, types, values, spec, gases=gases)
    assert bad == 0, np.bincount(out.status)
    N, n = net.N, cells.ncells
    m = out.pri_molal.reshape(N, n)
    tot = out.total_out.reshape(N, n)
    sorb = out.total_sorb_eq.reshape(N, n)
    for j in range(N):
        if types[j] == abi.CONSTRAINT_TOTAL:
            assert np.abs(tot[j] - values[j]).max() <= 1e-10 * np.abs(values[j]).max()
        if types[j] == abi.CONSTRAINT_TOTAL_SORB:
            np.testing.assert_allclose(sorb[j], values[j], rtol=1e-10)
    gp = np.array([oracle.activity_lag(net.as_struct(), float(I), N, net.Nc)[0] for I in out.ionic_strength]).T
    for j in np.flatnonzero(types == abi.CONSTRAINT_GAS):
        rx = net.gases[spec[j] - 1]
        lnQK = -rx.logK * 2.30258509299 + sum(nu * np.log(m[net.idx(q)] * gp[net.idx(q)])
                                             for q, nu in zip(rx.species, rx.stoich))
        p = values[j] if values[j].max() > 0 else 10.0 ** values[j]
        assert np.abs(lnQK - np.log(p)).max() < 1e-8
    # the rows describe each cell's own equilibrium state
    np.testing.assert_allclose(m, cells.pri_molal.reshape(N, n), rtol=1e-6)
    # the log10 form of a partial pressure
    j2 = next(j for j in np.flatnonzero(types == abi.CONSTRAINT_GAS) if values[j].max() <= 0)
    v2 = values.copy()
    v2[j2] = 10.0 ** values[j2]
    out2 = cells.copy()
    out2.sec_molal = np.zeros(net.Nc * cells.ncells)
    assert oracle.equilibrate_constraints(net.as_struct(), copt, out2, types, v2, spec, gases=gases) == 0
    np.testing.assert_allclose(out2.pri_molal, out.pri_molal, rtol=1e-12)


def test_constraint_gas_row_with_database_gas(oracle):
    """CO2(g) read from a database's gas block and rewritten in the
    primaries (H+ + HCO3- - H2O): the calcite water of a column's initial
    condition (free H+, HCO3- from 1e-3 bar CO2(g), Ca++ at calcite
    saturation) converges and meets its gas row."""
    from pflotran_gb300 import abi, workloads
    net, _, cells, dt = workloads.calcite_cells(4, seed=44)
    workloads.add_passive_gases(net)
    assert net.gases[0].extra["name"] == "CO2(g)" and net.gases[0].h2o == -1.0
    copt = workloads.default_options(use_isothermal=1, residual_tol_kind=abi.RESIDUAL_ABSOLUTE,
                                     max_relative_change_tolerance=1e-6, max_residual_tolerance=1e-12)
    n = cells.ncells
    types = np.array([abi.CONSTRAINT_FREE, abi.CONSTRAINT_GAS, abi.CONSTRAINT_MINERAL], np.int32)
    spec = np.array([0, 1, 1], np.int32)
    values = np.array([[1e-8] * n, [1e-3] * n, [5e-4] * n])
    out = cells.copy()
    out.sec_molal = np.zeros(net.Nc * n)
    assert oracle.equilibrate_constraints(net.as_struct(), copt, out, types, values, spec,
                                          gases=net.gas_table()) == 0
    m = out.pri_molal.reshape(3, n)
    gp = np.array([oracle.activity_lag(net.as_struct(), float(I), 3, net.Nc)[0] for I in out.ionic_strength]).T
    lnQK = 7.8136 * 2.30258509299 + np.log(m[0] * gp[0]) + np.log(m[1] * gp[1])
    assert np.abs(lnQK - np.log(1e-3)).max() < 1e-8
    np.testing.assert_allclose(m[0] * cells.den_kg[:n] * 1e-3, 1e-8, rtol=1e-12)


def test_surface_complexation_1_gold(oracle):
    """surface-complexation-1 (time 0): constraint speciation with pH and
    charge-balance rows + one equilibrium surface-complexation site
    (7.6355e4 mol/m^3, three complexes).  The harness's 1e-12 absolute is
    met on the aqueous totals; the sorbed quantities (up to 7.6e4 mol/m^3,
    printed to 14 digits) are held to 1e-12 relative."""
    out, gold = kat.run_surface_complexation_1(oracle)
    for key in ("Total H+", "Total Na+", "Total NO3-", "Total Zn++"):
        assert abs(out[key] - gold[key]) <= 1e-12, (key, out[key], gold[key])
    for key in ("Free >FeOH_w", ">FeOH2+_w", ">FeO-_w", ">FeOHZn+_w", "Total Sorbed H+", "Total Sorbed Na+",
                "Total Sorbed NO3-", "Total Sorbed Zn++"):
        assert abs(out[key] - gold[key]) <= 1e-12 * max(abs(gold[key]), 1.0), (key, out[key], gold[key])
    assert abs(out["pH"] - gold["pH"]) <= 1e-8


@pytest.mark.parametrize("deck", ["carbonate-unit-activity", "carbonate-debye-huckel-activity",
                                  "ca-carbonate-unit-activity", "ca-carbonate-debye-huckel-activity"])
def test_carbonate_speciation_gold(oracle, deck):
    """The carbonate speciation decks at time 0 (constraint speciation with
    TOTAL rows, unit or Debye-Hueckel activity, then the reference's
    initialisation of the cell): pH, totals and activity coefficients
    within the harness's 1e-12 absolute."""
    out, gold = kat.run_carbonate_speciation(oracle, deck)
    for key, v in out.items():
        assert abs(v - gold[key]) <= 1e-12, (key, v, gold[key])


def test_calcite_kinetics_volume_fractions_gold(oracle):
    """calcite-kinetics-volume-fractions: 1825 days in steps of 30 days to
    near equilibrium (5 years of calcite dissolution).  Volume fraction and
    rate meet the harness's 1e-12 absolute; totals are held to 1e-11 and pH
    to 1e-9: the gold run's global-implicit Newton stops at its solver
    tolerance each step (its final Ca++ and HCO3- totals differ by 3.3e-12
    more than the carbonate the calcite released, which a converged step
    conserves exactly), and its 62-step sequence is not the 61 steps the
    deck's 30-day maximum gives here."""
    out, gold = kat.run_calcite_kinetics(oracle, 0, "kat_calcite_kinetics_volume_fractions.json")
    for key in ("Calcite VF", "Calcite Rate"):
        assert abs(out[key] - gold[key]) <= 1e-12, (key, out[key], gold[key])
    for key in ("Total H+", "Total HCO3-", "Total Ca++"):
        assert abs(out[key] - gold[key]) <= 1e-11, (key, out[key], gold[key])
    assert abs(out["pH"] - gold["pH"]) <= 1e-9


def test_single_cell_constraint_rejects_rows_it_cannot_take(oracle):
    """The single-cell constraint entry has no mineral ids: a MINERAL or an
    unknown row type is an error, not a read through a null table."""
    fx = kat.load("kat_calcite_kinetics.json")
    net = kat.build_network(fx, oracle)
    from pflotran_gb300.network import default_options
    b = kat.one_cell(net, fx, oracle)
    for bad in ([1, 1, 6], [1, 0, 1], [7, 1, 1]):
        with pytest.raises(RuntimeError):
            oracle.equilibrate_constraint(net.as_struct(), default_options(use_isothermal=1), b, bad, [1e-5] * 3)


def test_armoring_flag_is_set_by_the_previous_armored_item(oracle):
    """The reference carries the armoring flag from item to item (cells, then
    minerals); every armored item sets it from its own test, so the serial
    loop equals the data-parallel rule the GPU kernel uses: an item's incoming
    flag is the test of the previous armored item.  Checked on the oracle's
    serial restatement against that rule written out here."""
    from pflotran_gb300 import abi, workloads
    net, opt, cells, dt = workloads.synthetic_cells(257, seed=36)
    n, Nm = cells.ncells, net.Nm
    rng = np.random.default_rng(5)
    vf = rng.uniform(0.0, 0.05, (Nm, n))
    cells.mnrl_volfrac = vf.ravel().copy()
    crit = np.zeros(Nm)
    crit[1], crit[3], crit[4] = 0.025, 0.03, 0.01
    armor = np.arange(1, Nm + 1, dtype=np.int32)
    armor[1], armor[3] = 1, 6
    area0 = rng.uniform(0.5, 2.0, (Nm, n))
    vf0 = rng.uniform(0.01, 0.05, (Nm, n))
    pw = np.full(Nm, 2.0 / 3.0)
    for flag_in in (0, 1):
        out = np.full(1, -1, np.int32)
        c = cells.copy()
        oracle.update_mineral_properties(net.as_struct(), c, abi.mineral_update(
            {"surf_area_vol_frac_pwr": pw, "mnrl_volfrac0": vf0.ravel(), "mnrl_area0": area0.ravel(),
             "armor_crit_vol_frac": crit, "armor_mineral": armor, "armor_flag_out": out},
            update_porosity=0, armor_flag=flag_in))
        expect = area0 * (vf / vf0) ** pw[:, None]
        items = [m for m in range(Nm) if crit[m] > 0]
        test = lambda m, k: crit[m] > vf[armor[m] - 1, k]
        for k in range(n):
            for i, m in enumerate(items):
                prev = (items[i - 1], k) if i > 0 else ((items[-1], k - 1) if k > 0 else None)
                flag = flag_in if prev is None else (0 if test(*prev) else 1)
                if test(m, k):
                    fa = ((crit[m] - vf[armor[m] - 1, k]) / crit[m]) ** pw[m]
                    expect[m, k] = expect[m, k] * fa if flag == 0 else area0[m, k]
                else:
                    expect[m, k] = 0.0
        np.testing.assert_allclose(c.mnrl_area.reshape(Nm, n), expect, rtol=1e-14, atol=0)
        assert out[0] == (0 if test(items[-1], n - 1) else 1)
