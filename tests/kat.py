"""Known-answer replays of PFLOTRAN's batch chemistry regression tests
through the oracle (fixtures from tests/golden/make_kat_fixtures.py).

For a one-cell, zero-flux deck the global-implicit time step solves exactly
the dt-consistent per-cell equation F(m) = (psv*T(m) - psv*T_old)/dt + R(m) = 0,
so the oracle's RReact in that mode, converged tightly and stepped with the
deck's time steps, must land on the gold values.
"""
import json
import math
import os

import numpy as np

from pflotran_gb300 import abi
from pflotran_gb300.cells import CellBatch
from pflotran_gb300.network import ReactionNetwork, default_options

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
LOG_TO_LN = 2.30258509299


def load(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def debye_25C():
    """reaction_database.F90:897-915 at the reference temperature 25 C via
    utility.F90:677-701 Interpolate (weight 1 on the 25 C values)."""
    def interp(xh, xl, x, yh, yl):
        w = (x - xl) / (xh - xl)
        return yl + w * (yh - yl)
    return (interp(25.0, 0.0, 25.0, 0.5114, 0.4939), interp(25.0, 0.0, 25.0, 0.3288, 0.3253),
            interp(25.0, 0.0, 25.0, 0.0410, 0.0374))


def build_network(fx, oracle):
    temps = fx["temperatures"]
    prim = [(p["name"], p["Z"], p["a0"]) for p in fx["primaries"]]
    net = ReactionNetwork(prim, debye=debye_25C())
    def fit(logK):
        # reaction_aux.F90:1336-1408; entries with log K at one temperature
        # only (500 elsewhere) have no fit and keep their 25 C value
        return tuple(oracle.fit_logK(temps, logK)) if sum(abs(k - 500.0) > 1e-10 for k in logK) >= 5 else None

    for c in fx.get("complexes", []):
        st = {s: v for s, v in c["stoich"] if s != "H2O"}
        h2o = sum(v for s, v in c["stoich"] if s == "H2O")
        coef = fit(c["logK"])
        # transport-only runs are isothermal (factory_subsurface.F90:368-374): log K is the
        # database value at the 25 C reference temperature (reaction_aux.F90:1412-1457)
        net.add_complex(c["name"], st, logK=c["logK"][temps.index(25.0)], Z=c["Z"], a0=c["a0"],
                        logKcoef=coef, h2o=h2o)
    for m in fx.get("minerals", []):
        st = {s: v for s, v in m["stoich"] if s != "H2O"}
        coef = tuple(oracle.fit_logK(temps, m["logK"]))
        net.add_kinetic_mineral(m["name"], st, logK=m["logK"][temps.index(25.0)],
                                rate_constant=fx["rate_constant"], molar_vol=m["molar_vol_cm3"] * 1e-6,
                                logKcoef=coef)
    if "ionx" in fx:
        net.add_ion_exchange([(c, k) for c, k in fx["ionx"]["cations"]], fx["ionx"]["CEC"])
    if "surface" in fx:
        sf = fx["surface"]
        cx = []
        for c in sf["complexes"]:
            rest = {s: v for s, v in c["stoich"] if s != sf["site"] and s != "H2O"}
            fs = sum(v for s, v in c["stoich"] if s == sf["site"])
            cx.append((rest, fs, c["logK"][temps.index(25.0)]))
        net.add_surface_complexation(sf["site_density"], cx)
    net.build()
    return net


def one_cell(net, fx, oracle):
    b = CellBatch.allocate(net, 1, sec_molal=True)
    b.temperature[:] = 25.0
    b.saturation[:] = 1.0
    b.den_kg[:] = oracle.ifc67_density(25.0, 101325.0)
    b.porosity[:] = fx["porosity"]
    b.volume[:] = fx["volume"]
    b.soil_particle_density[:] = 2650.0
    if net.Nm:
        b.mnrl_volfrac[:] = fx.get("volfrac", 1e-5)
        b.mnrl_area[:] = fx.get("area", 1.0)
    if net.Nix:
        b.eqionx_ref_cation_sorbed_conc[:] = 1e-9  # reactive_transport_aux.F90 initial value
    if net.Nsr:
        b.srfcplxrxn_free_site_conc[:] = 1e-9      # likewise
    return b


def step_sizes(fx):
    """The deck's time steps: `nsteps` of `dt`, or steps of `dt` up to
    `final_time` with the last one shortened to land on it."""
    if fx.get("nsteps"):
        return [fx["dt"]] * fx["nsteps"]
    out, t = [], 0.0
    while fx["final_time"] - t > 1e-6 * fx["dt"]:
        out.append(min(fx["dt"], fx["final_time"] - t))
        t += out[-1]
    return out


def run_calcite_kinetics(oracle, precision=0, fixture="kat_calcite_kinetics.json"):
    fx = load(fixture)
    net = build_network(fx, oracle)
    ns = net.as_struct()
    # constraint speciation (relative-change and residual tolerances of the deck: defaults)
    copt = default_options(use_isothermal=1, residual_tol_kind=abi.RESIDUAL_ABSOLUTE,
                           max_relative_change_tolerance=1e-6, max_residual_tolerance=1e-12)
    b = one_cell(net, fx, oracle)
    oracle.equilibrate_constraint(ns, copt, b, fx["constraint"]["types"], fx["constraint"]["conc"])
    start_from_initial_condition(oracle, net, b)
    # GI steps: the totals at the start of each step are the previous state's totals
    sopt = default_options(use_isothermal=1, residual_tol_kind=abi.RESIDUAL_RELATIVE,
                           max_residual_tolerance=1e-15, max_relative_change_tolerance=0.0,
                           max_iterations=100, update_kinetic_state=1)
    I_prev = float(b.ionic_strength[0])
    for dt in step_sizes(fx):
        b.total[:] = b.total_out
        I_prev = float(b.ionic_strength[0])
        bad = oracle.react(ns, sopt, dt, b, precision, 1)
        assert bad == 0, b.status
    gp, _ = oracle.activity_lag(ns, I_prev, net.N, net.Nc)
    out = {
        "pH": -math.log10(b.pri_molal[0] * gp[0]),
        "Total H+": b.total_out[0], "Total HCO3-": b.total_out[1], "Total Ca++": b.total_out[2],
        "Calcite VF": b.mnrl_volfrac[0], "Calcite Rate": b.mnrl_rate[0],
    }
    return out, fx["gold"]


def run_ion_exchange_valocchi(oracle):
    fx = load("kat_ion_exchange_valocchi.json")
    net = build_network(fx, oracle)
    ns = net.as_struct()
    copt = default_options(use_isothermal=1, act_coef_update_frequency=abi.ACT_COEF_FREQUENCY_OFF,
                           residual_tol_kind=abi.RESIDUAL_ABSOLUTE,
                           max_relative_change_tolerance=1e-6, max_residual_tolerance=1e-12)
    b = one_cell(net, fx, oracle)
    oracle.equilibrate_constraint(ns, copt, b, fx["constraint"]["types"], fx["constraint"]["conc"])
    names = [p["name"] for p in fx["primaries"]]
    out = {}
    for i, nm in enumerate(names):
        out[f"Total {nm}"] = b.total_out[i]
        out[f"Total Sorbed {nm}"] = b.total_sorb_eq[i]
    return out, fx["gold"]


def run_surface_complexation_1(oracle):
    """surface-complexation-1 at time 0: constraint speciation (pH, charge
    balance, totals) and the equilibrium surface complexes of one site
    (RTotalSorbEqSurfCplx1, closed form: every complex binds one free site)."""
    fx = load("kat_surface_complexation_1.json")
    net = build_network(fx, oracle)
    ns = net.as_struct()
    copt = default_options(use_isothermal=1, residual_tol_kind=abi.RESIDUAL_ABSOLUTE,
                           max_relative_change_tolerance=1e-6, max_residual_tolerance=1e-12)
    b = one_cell(net, fx, oracle)
    oracle.equilibrate_constraint(ns, copt, b, fx["constraint"]["types"], fx["constraint"]["conc"])
    names = [p["name"] for p in fx["primaries"]]
    gp, _ = oracle.activity_lag(ns, float(b.ionic_strength[0]), net.N, net.Nc)
    act = b.pri_molal[:net.N] * gp
    out = {"pH": -math.log10(act[0])}
    for i, nm in enumerate(names):
        out[f"Total {nm}"] = b.total_out[i]
        out[f"Total Sorbed {nm}"] = b.total_sorb_eq[i]
    sf = fx["surface"]
    free = float(b.srfcplxrxn_free_site_conc[0])
    out[f"Free {sf['site']}"] = free
    for c in sf["complexes"]:
        lnQK = -c["logK"][fx["temperatures"].index(25.0)] * LOG_TO_LN
        for s_, v in c["stoich"]:
            if s_ in names:
                lnQK += v * math.log(act[names.index(s_)])
        out[c["name"]] = free * math.exp(lnQK)
    return out, fx["gold"]


def _rtotal(net, m, gp, gs):
    """RTotal (reaction.F90:4057-4158) for one cell in numpy: complex
    molalities, component totals (mol/kg) and the ionic strength."""
    lna = np.log(m) + np.log(gp)
    C = np.zeros(net.Nc)
    psi = m.copy()
    for i, c in enumerate(net.complexes):
        lnQK = -c.logK * LOG_TO_LN
        for s_, v in zip(c.species, c.stoich):
            lnQK += v * lna[net.idx(s_)]
        C[i] = math.exp(lnQK) / gs[i]
        for s_, v in zip(c.species, c.stoich):
            psi[net.idx(s_)] += v * C[i]
    zp = np.array(net.pri_Z)
    zs = np.array([c.extra["Z"] for c in net.complexes])
    I = 0.5 * (np.sum(zp * zp * m) + np.sum(zs * zs * C))
    return C, psi, I


def initial_condition_state(oracle, net, m, den_kg, act_coef_on):
    """The state the reference reports at time 0 for a cell initialised from
    a constraint when the constraint is equilibrated once and copied
    (isothermal runs, condition_control.F90:600-700): the cell's own
    activity coefficients start at 1, its auxiliary variables are computed
    once without and, with activity coefficients on, twice with an activity
    update (condition_control.F90:933-944).  Returns (gamma_pri, totals in
    mol/L, ionic strength of the final complexes)."""
    ns = net.as_struct()
    gp, gs = np.ones(net.N), np.ones(net.Nc)
    C, psi, I = _rtotal(net, m, gp, gs)
    if act_coef_on:
        for _ in range(2):
            gp, gs = oracle.activity_lag(ns, I, net.N, net.Nc)
            C, psi, I = _rtotal(net, m, gp, gs)
    return gp, psi * den_kg * 1e-3, I


def start_from_initial_condition(oracle, net, b):
    """Replaces the constraint's final totals and ionic strength in the
    host CellBatch `b` (cell 0) by the initialised cell's
    (`initial_condition_state` with activity coefficients on): the state
    the first time step starts from."""
    m = b.pri_molal.reshape(net.N, -1)[:, 0].copy()
    _, tot, I = initial_condition_state(oracle, net, m, float(b.den_kg[0]), True)
    n = b.ncells
    b.total_out.reshape(net.N, n)[:] = tot[:, None]
    b.ionic_strength[:] = I


def run_carbonate_speciation(oracle, deck):
    """One of the carbonate speciation decks at time 0: constraint
    speciation with TOTAL rows, unit or Debye-Hueckel activity."""
    fx = load("kat_carbonate_speciation.json")[deck]
    net = build_network(fx, oracle)
    ns = net.as_struct()
    freq = abi.ACT_COEF_FREQUENCY_OFF if fx["act_coef"] == "OFF" else abi.ACT_COEF_FREQUENCY_TIMESTEP
    copt = default_options(use_isothermal=1, act_coef_update_frequency=freq, residual_tol_kind=abi.RESIDUAL_ABSOLUTE,
                           max_relative_change_tolerance=1e-6, max_residual_tolerance=1e-12)
    b = one_cell(net, fx, oracle)
    oracle.equilibrate_constraint(ns, copt, b, fx["constraint"]["types"], fx["constraint"]["conc"])
    names = [p["name"] for p in fx["primaries"]]
    m = b.pri_molal[:net.N].copy()
    gp, tot, _ = initial_condition_state(oracle, net, m, float(b.den_kg[0]), fx["act_coef"] != "OFF")
    out = {"pH": -math.log10(m[names.index("H+")] * gp[names.index("H+")])}
    for i, nm in enumerate(names):
        out[f"Total {nm}"] = tot[i]
        out[f"Gamma {nm}"] = gp[i]
    return out, fx["gold"]


def write_calcite_db(path):
    """A database in PFLOTRAN's format with the calcite system's rows as the
    known-answer fixture records them."""
    fx = load("kat_calcite_kinetics.json")
    temps = fx["temperatures"]
    q = lambda s: f"'{s}'"
    lines = [f"'temperature points' {len(temps)} " + " ".join(str(t) for t in temps)]
    for p in fx["primaries"]:
        lines.append(f"{q(p['name'])} {p['a0']} {p['Z']} 1.0")
    lines.append("'null' 0 0 0")
    for c in fx["complexes"]:
        st = " ".join(f"{v} {q(s)}" for s, v in c["stoich"])
        lines.append(f"{q(c['name'])} {len(c['stoich'])} {st} " + " ".join(str(k) for k in c["logK"]) +
                     f" {c['a0']} {c['Z']} 1.0")
    lines.append("'null' 1 0. '0' " + " ".join("0." for _ in temps))
    lines.append("'null' 0. 1 0. '0' " + " ".join("0." for _ in temps))
    for m in fx["minerals"]:
        st = " ".join(f"{v} {q(s)}" for s, v in m["stoich"])
        lines.append(f"{q(m['name'])} {m['molar_vol_cm3']} {len(m['stoich'])} {st} " +
                     " ".join(str(k) for k in m["logK"]) + " 100.0")
    lines.append("'null' 0. 1 0. '0' " + " ".join("0." for _ in temps))
    lines.append("'null' 1 0. '0' " + " ".join("0." for _ in temps))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return fx


def calcite_networks_two_bases(db_path):
    """The calcite system from the database written by write_calcite_db in
    its own basis (H+, HCO3-, Ca++) and with CO2(aq) primary instead of
    HCO3- (basis swap), kinetic calcite in both."""
    from pflotran_gb300 import database
    fx = write_calcite_db(db_path)
    db = database.read_database(db_path)
    sec = [c["name"] for c in fx["complexes"]]
    kin = {"Calcite": dict(rate_constant=1e-9)}
    a = database.network_from_database(db, ["H+", "HCO3-", "Ca++"], secondary=sec, kinetic_minerals=kin,
                                       debye=debye_25C())
    sec_b = [s for s in sec if s != "CO2(aq)"] + ["HCO3-"]
    b = database.network_from_database(db, ["H+", "CO2(aq)", "Ca++"], secondary=sec_b, kinetic_minerals=kin,
                                       debye=debye_25C())
    return db, a, b


def species_molalities(oracle, net, cells):
    """Molality of every species of each cell (primaries: the state's free
    ions; complexes: mass action with LAG activity coefficients at the
    cell's ionic strength): {name: array over cells}."""
    n = cells.ncells
    m = cells.pri_molal.reshape(net.N, n)
    out = {nm: m[j].copy() for j, nm in enumerate(net.pri_names)}
    for c in net.complexes:
        out[c.extra["name"]] = np.zeros(n)
    ns = net.as_struct()
    for k in range(n):
        gp, gs = oracle.activity_lag(ns, float(cells.ionic_strength[k]), net.N, net.Nc)
        lna = np.log(m[:, k]) + np.log(gp)
        for i, c in enumerate(net.complexes):
            ln = -c.logK * LOG_TO_LN + sum(v * lna[net.idx(s)] for s, v in zip(c.species, c.stoich))
            out[c.extra["name"]][k] = math.exp(ln) / gs[i]
    return out


def cells_in_basis(oracle, net_a, net_b, cells_a):
    """The cells of `net_a` described in the basis of `net_b` (same species,
    other primaries).  Every species is the same combination of either
    basis's components, so the component totals map linearly: net_b's total
    of component k = sum_j (net_b composition of net_a's primary j)_k x
    net_a's total j.  The free-ion guess is the species' molalities."""
    n = cells_a.ncells
    conc = species_molalities(oracle, net_a, cells_a)
    comp = {nm: {nm: 1.0} for nm in net_b.pri_names}
    for c in net_b.complexes:
        comp[c.extra["name"]] = dict(zip(c.species, c.stoich))
    conv = np.zeros((net_b.N, net_a.N))
    for j, nm in enumerate(net_a.pri_names):
        for s, v in comp[nm].items():
            conv[net_b.idx(s), j] += v
    b = cells_a.copy()
    b.total = np.ascontiguousarray((conv @ cells_a.total.reshape(net_a.N, n)).ravel())
    b.pri_molal = np.ascontiguousarray(np.stack([conc[nm] for nm in net_b.pri_names]).ravel())
    b.sec_molal = np.zeros(max(net_b.Nc, 1) * n)
    return b
