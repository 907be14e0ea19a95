"""Database reader and network assembly (CPU)."""
import os

import numpy as np
import pytest

import kat
from pflotran_gb300 import database

# the reference tree is located by PFLOTRAN_SOURCE_DIR (the test is skipped without it)
REF_DB = os.path.join(os.environ.get("PFLOTRAN_SOURCE_DIR", ""), "database", "hanford.dat")


def test_network_from_database_matches_fixture_network(oracle, tmp_path):
    path = tmp_path / "calcite.dat"
    fx = kat.write_calcite_db(path)
    db = database.read_database(path)
    prim = [p["name"] for p in fx["primaries"]]
    net = database.network_from_database(
        db, prim, kinetic_minerals={m["name"]: dict(rate_constant=fx["rate_constant"]) for m in fx["minerals"]},
        debye=kat.debye_25C())
    ref = kat.build_network(fx, oracle)
    a, b = net.build(), ref.build()
    for key in ("eqcplxspecid", "eqcplxstoich", "eqcplx_logK", "eqcplx_Z", "kinmnrlspecid", "kinmnrl_logK",
                "kinmnrl_molar_vol"):
        np.testing.assert_array_equal(np.asarray(a[key]), np.asarray(b[key]), err_msg=key)
    # the Maier-Kelly fit against the oracle's restatement of ReactionFitLogKCoef:
    # the normal equations are ill-conditioned, so compare log K(T), not the coefficients
    ca = np.asarray(a["eqcplx_logKcoef"]).reshape(-1, 5)
    cb = np.asarray(b["eqcplx_logKcoef"]).reshape(-1, 5)
    fitted = [i for i, c in enumerate(fx["complexes"]) if sum(abs(k - 500.0) > 1e-10 for k in c["logK"]) >= 5]
    assert fitted
    for t in (10.0, 25.0, 60.0, 100.0):
        np.testing.assert_allclose([oracle.interpolate_logK(ca[i], t) for i in fitted],
                                   [oracle.interpolate_logK(cb[i], t) for i in fitted], rtol=0, atol=1e-7)


def test_fit_logK_skips_missing_temperatures(oracle):
    temps = [0.0, 25.0, 60.0, 100.0, 150.0, 200.0, 250.0, 300.0]
    logK = [14.9, 13.99, 13.0, 12.25, 11.6, 11.3, 11.2, 500.0]
    c = database.fit_logK(temps, logK)
    ref = oracle.fit_logK(temps, logK)
    for t in temps[:-1] + [37.0]:
        assert abs(oracle.interpolate_logK(np.asarray(c), t) - oracle.interpolate_logK(np.asarray(ref), t)) < 1e-7
    assert database.fit_logK(temps, [500.0] * 4 + [1.0] * 4) is None


@pytest.mark.skipif(not os.path.exists(REF_DB), reason="reference database not present")
def test_reads_reference_database():
    db = database.read_database(REF_DB)
    assert len(db.temperatures) == 8 and db.temperatures[1] == 25.0
    assert {"H+", "Ca++", "HCO3-"} <= set(db.primaries)
    assert "CaCO3(aq)" in db.secondary and "Calcite" in db.minerals
    net = database.network_from_database(db, ["H+", "Ca++", "HCO3-"],
                                         kinetic_minerals={"Calcite": dict(rate_constant=1e-9)})
    names = [c.extra["name"] for c in net.complexes]
    assert "OH-" in names and "CO2(aq)" in names and "CaCO3(aq)" in names
    # a swapped basis on the full database: CO2(aq) primary, HCO3- secondary
    sec = ["OH-", "CO3--", "HCO3-", "CaOH+", "CaHCO3+", "CaCO3(aq)"]
    net2 = database.network_from_database(db, ["H+", "CO2(aq)", "Ca++"], secondary=sec,
                                          kinetic_minerals={"Calcite": dict(rate_constant=1e-9)})
    calcite = net2.minerals[0]
    assert dict(zip(calcite.species, calcite.stoich)) == {"H+": -2.0, "Ca++": 1.0, "CO2(aq)": 1.0}
    # redox couples written with O2(g): gases are not supported
    with pytest.raises(ValueError, match="gases"):
        database.network_from_database(db, ["H+", "SO4--"], secondary=["HS-"])


LN10 = np.log(10.0)


def _ln_activities(net, lna_pri):
    """ln activity of every species at unit activity coefficients: the
    primaries' given values and each complex from its mass action."""
    out = dict(zip(net.pri_names, lna_pri))
    for c in net.complexes:
        out[c.extra["name"]] = -c.logK * LN10 + sum(v * out[s] for s, v in zip(c.species, c.stoich))
    return out


def _ln_QK(net, ln_a):
    return {m.extra["name"]: -m.logK * LN10 + sum(v * ln_a[s] for s, v in zip(m.species, m.stoich))
            for m in net.minerals}


def _calcite_networks(tmp_path):
    path = tmp_path / "calcite.dat"
    fx = kat.write_calcite_db(path)
    db = database.read_database(path)
    sec = [c["name"] for c in fx["complexes"]]
    kin = {"Calcite": dict(rate_constant=1e-9)}
    a = database.network_from_database(db, ["H+", "HCO3-", "Ca++"], secondary=sec, kinetic_minerals=kin)
    # CO2(aq) as a primary instead of HCO3- (a database secondary species)
    sec_b = [s for s in sec if s != "CO2(aq)"] + ["HCO3-"]
    b = database.network_from_database(db, ["H+", "CO2(aq)", "Ca++"], secondary=sec_b, kinetic_minerals=kin)
    return db, a, b


def test_basis_swap_preserves_mass_action(tmp_path):
    """The same solution described in two bases: every species' activity and
    the calcite saturation agree whichever species are primary."""
    db, a, b = _calcite_networks(tmp_path)
    co2 = next(c for c in b.complexes if c.extra["name"] == "HCO3-")
    # HCO3- = CO2(aq) + H2O - H+ with log K = -log K(CO2(aq)) in the database's direction
    assert dict(zip(co2.species, co2.stoich)) == {"CO2(aq)": 1.0, "H+": -1.0} and co2.h2o == 1.0
    assert abs(co2.logK + db.secondary["CO2(aq)"].logK[1]) < 1e-12
    rng = np.random.default_rng(5)
    for _ in range(20):
        la = _ln_activities(a, rng.uniform(-12.0, -1.0, 3))
        lb = _ln_activities(b, np.array([la["H+"], la["CO2(aq)"], la["Ca++"]]))
        for name, v in la.items():
            assert abs(lb[name] - v) < 1e-11, name
        qa, qb = _ln_QK(a, la), _ln_QK(b, lb)
        assert abs(qa["Calcite"] - qb["Calcite"]) < 1e-11


def test_basis_swap_through_the_oracle(oracle, tmp_path):
    """Free-ion constraint speciation in both bases from the same free-ion
    state, through the oracle's tables: the same species concentrations.
    (Unit activity coefficients: the constraint's lagged activity update
    stops after two updates, so with Debye-Hueckel the two bases would
    stop at different points of the same fixed-point iteration.)"""
    from pflotran_gb300 import abi
    from pflotran_gb300.network import default_options
    db, a, b = _calcite_networks(tmp_path)
    fx = kat.load("kat_calcite_kinetics.json")
    opt = default_options(use_isothermal=1, act_coef_update_frequency=abi.ACT_COEF_FREQUENCY_OFF,
                          residual_tol_kind=abi.RESIDUAL_ABSOLUTE,
                          max_relative_change_tolerance=1e-12, max_residual_tolerance=1e-14)
    ca = kat.one_cell(a, fx, oracle)
    molar = [1e-7, 2e-3, 1e-3]  # H+, HCO3-, Ca++ free (mol/L)
    oracle.equilibrate_constraint(a.as_struct(), opt, ca, [2, 2, 2], molar)
    conc_a = dict(zip(a.pri_names, ca.pri_molal[:3]))
    conc_a.update({c.extra["name"]: ca.sec_molal[i] for i, c in enumerate(a.complexes)})
    den = float(ca.den_kg[0]) * 1e-3
    cb = kat.one_cell(b, fx, oracle)
    oracle.equilibrate_constraint(b.as_struct(), opt, cb, [2, 2, 2],
                                  [conc_a["H+"] * den, conc_a["CO2(aq)"] * den, conc_a["Ca++"] * den])
    conc_b = dict(zip(b.pri_names, cb.pri_molal[:3]))
    conc_b.update({c.extra["name"]: cb.sec_molal[i] for i, c in enumerate(b.complexes)})
    for name, v in conc_a.items():
        assert abs(conc_b[name] - v) <= 1e-12 * v, (name, conc_b[name], v)


def test_basis_swap_rejects_inconsistent_bases(tmp_path):
    path = tmp_path / "calcite.dat"
    fx = kat.write_calcite_db(path)
    db = database.read_database(path)
    sec = [c["name"] for c in fx["complexes"]]
    with pytest.raises(ValueError, match="secondary species listed"):
        database.network_from_database(db, ["H+", "CO2(aq)", "Ca++"])
    with pytest.raises(ValueError, match="span the same components"):
        # CO2(aq) primary but HCO3- missing from the secondaries: one reaction too many
        database.network_from_database(db, ["H+", "CO2(aq)", "Ca++"], secondary=[s for s in sec if s != "CO2(aq)"])
    with pytest.raises(ValueError, match="both a primary and a secondary"):
        database.network_from_database(db, ["H+", "HCO3-", "Ca++"], secondary=sec + ["HCO3-"])


def test_reaction_step_is_the_same_in_a_swapped_basis(oracle, tmp_path):
    """The calcite workload stepped by the oracle in the database's basis
    and, re-expressed, with CO2(aq) primary: after the step every species'
    molality agrees to 1e-9 (measured 2e-11: each basis converges its own
    component residuals to 1e-12), the volume fractions to 1e-12 and the
    calcite rate to 5e-9 of k x area (measured 9e-10: near equilibrium the
    affinity 1 - Q/K turns the species' 1e-11 into ~1e-9)."""
    from pflotran_gb300 import workloads
    db, a, b = kat.calcite_networks_two_bases(tmp_path / "calcite.dat")
    _, opt, ca, dt = workloads.calcite_cells(256, seed=9, net=a)
    ca.sec_molal = np.zeros(a.Nc * ca.ncells)
    cb = kat.cells_in_basis(oracle, a, b, ca)
    ra, rb = ca.copy(), cb.copy()
    assert oracle.react(a.as_struct(), opt, dt, ra, 0, 4) == 0
    assert oracle.react(b.as_struct(), opt, dt, rb, 0, 4) == 0
    n = ra.ncells
    sa = dict(zip(a.pri_names, ra.pri_molal.reshape(a.N, n)))
    sa.update({c.extra["name"]: ra.sec_molal.reshape(-1, n)[i] for i, c in enumerate(a.complexes)})
    sb = dict(zip(b.pri_names, rb.pri_molal.reshape(b.N, n)))
    sb.update({c.extra["name"]: rb.sec_molal.reshape(-1, n)[i] for i, c in enumerate(b.complexes)})
    for name, x in sa.items():
        err = np.abs(sb[name] - x) / np.maximum(np.abs(x), 1e-300)
        assert err.max() <= 1e-9, (name, err.max())
    k_area = 1e-9 * ra.mnrl_area
    assert (np.abs(rb.mnrl_rate - ra.mnrl_rate) / k_area).max() <= 5e-9
    assert (np.abs(rb.mnrl_volfrac - ra.mnrl_volfrac) / ra.mnrl_volfrac).max() <= 1e-12
