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
    for c in fx.get("complexes", []):
        st = {s: v for s, v in c["stoich"] if s != "H2O"}
        h2o = sum(v for s, v in c["stoich"] if s == "H2O")
        coef = tuple(oracle.fit_logK(temps, c["logK"]))  # reaction_aux.F90:1336-1408
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
    return b


def run_calcite_kinetics(oracle, precision=0):
    fx = load("kat_calcite_kinetics.json")
    net = build_network(fx, oracle)
    ns = net.as_struct()
    # constraint speciation (relative-change and residual tolerances of the deck: defaults)
    copt = default_options(use_isothermal=1, residual_tol_kind=abi.RESIDUAL_ABSOLUTE,
                           max_relative_change_tolerance=1e-6, max_residual_tolerance=1e-12)
    b = one_cell(net, fx, oracle)
    oracle.equilibrate_constraint(ns, copt, b, fx["constraint"]["types"], fx["constraint"]["conc"])
    # GI steps: the totals at the start of each step are the previous state's totals
    sopt = default_options(use_isothermal=1, residual_tol_kind=abi.RESIDUAL_RELATIVE,
                           max_residual_tolerance=1e-15, max_relative_change_tolerance=0.0,
                           max_iterations=100, update_kinetic_state=1)
    I_prev = float(b.ionic_strength[0])
    for step in range(fx["nsteps"]):
        b.total[:] = b.total_out
        I_prev = float(b.ionic_strength[0])
        bad = oracle.react(ns, sopt, fx["dt"], b, precision, 1)
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
