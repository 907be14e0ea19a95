"""Writes the known-answer fixtures of PFLOTRAN's batch chemistry regression
tests into tests/golden/*.json.

Run in a checkout that has the PFLOTRAN source tree (argument: its root):

    python tests/golden/make_kat_fixtures.py /path/to/pflotran

It reads, as text, the database rows and the regression gold values of

  regression_tests/ascem/batch/calcite-kinetics.{in,regression.gold} + calcite.dat
  regression_tests/ascem/batch/ion-exchange-valocchi.{in,regression.gold} + hanford.dat

and records them with the deck parameters the tests need (cited per deck
line below).  Nothing of PFLOTRAN is executed.
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def read_dat(path, names):
    """database rows of `names` (species, complexes, minerals) in a .dat file."""
    rows = {}
    temps = None
    with open(path) as f:
        for line in f:
            line = line.strip()
            if not line:
                continue
            toks = re.findall(r"'[^']*'|\S+", line)
            head = toks[0].strip("'")
            if head == "temperature points":
                temps = [float(x) for x in toks[2:2 + int(toks[1])]]
                continue
            if head in names and head not in rows:
                rows[head] = toks[1:]
    return temps, rows


def parse_primary(toks):
    # 'name' a0 Z molar_weight
    return dict(a0=float(toks[0]), Z=float(toks[1]))


def parse_rxn(toks, ntemp, mineral=False):
    i = 0
    out = {}
    if mineral:
        out["molar_vol_cm3"] = float(toks[0])
        i = 1
    nsp = int(toks[i]); i += 1
    st = []
    for _ in range(nsp):
        st.append((toks[i + 1].strip("'"), float(toks[i])))
        i += 2
    out["stoich"] = st
    out["logK"] = [float(x) for x in toks[i:i + ntemp]]
    i += ntemp
    if not mineral:
        out["a0"] = float(toks[i])
        out["Z"] = float(toks[i + 1])
    return out


def read_gold(path):
    gold = {}
    key = None
    with open(path) as f:
        for line in f:
            m = re.match(r"-- (\w+): (.*) --", line.strip())
            if m:
                key = m.group(2)
                continue
            m = re.match(r"\s*1:\s+(\S+)", line)
            if m and key is not None:
                gold[key] = float(m.group(1))
                key = None
    return gold


def main(root):
    batch = os.path.join(root, "regression_tests", "ascem", "batch")
    # --- calcite-kinetics ----------------------------------------------------
    pri = ["H+", "HCO3-", "Ca++"]                                         # .in PRIMARY_SPECIES
    sec = ["OH-", "CO3--", "CO2(aq)", "CaOH+", "CaHCO3+", "CaCO3(aq)"]    # .in SECONDARY_SPECIES
    temps, rows = read_dat(os.path.join(batch, "calcite.dat"), set(pri + sec + ["Calcite"]))
    fx = dict(
        source="regression_tests/ascem/batch/calcite-kinetics.in + calcite.dat + .regression.gold",
        temperatures=temps,
        primaries=[dict(name=p, **parse_primary(rows[p])) for p in pri],
        complexes=[dict(name=s, **parse_rxn(rows[s], len(temps))) for s in sec],
        minerals=[dict(name="Calcite", **parse_rxn(rows["Calcite"], len(temps), mineral=True))],
        rate_constant=1e-13 * 1e4,   # RATE_CONSTANT 1.d-13 mol/cm^2-sec -> mol/m^2/s
        volfrac=0.2, area=1.0 * 100.0,  # MINERALS Calcite 0.2 1.0 cm^2/cm^3 -> m^2/m^3
        porosity=0.5, volume=1.0, dt=0.5, nsteps=500,  # POROSITY 0.5; 1 m^3 cell; 0.5 s x 250 s
        constraint=dict(types=[1, 1, 1], conc=[-1e-5, 1e-5, 1e-5]),  # CONSTRAINT initial, T rows
        log_formulation=True, act_coef="TIMESTEP",
        gold=read_gold(os.path.join(batch, "calcite-kinetics.regression.gold")),
    )
    with open(os.path.join(HERE, "kat_calcite_kinetics.json"), "w") as f:
        json.dump(fx, f, indent=1)
    # --- ion-exchange-valocchi ----------------------------------------------
    pri = ["Na+", "Ca++", "Mg++", "Cl-"]
    temps, rows = read_dat(os.path.join(batch, "hanford.dat"), set(pri + ["Halite"]))
    fx = dict(
        source="regression_tests/ascem/batch/ion-exchange-valocchi.in + hanford.dat + .regression.gold",
        temperatures=temps,
        primaries=[dict(name=p, **parse_primary(rows[p])) for p in pri],
        # ION_EXCHANGE_RXN: CEC 750 eq/m^3; cations Ca++ 3.386..., Na+ 1 REFERENCE, Mg++ 6.002...
        ionx=dict(CEC=750.0, cations=[["Na+", 1.0], ["Ca++", 3.38638672536], ["Mg++", 6.00240096038]]),
        porosity=0.25, volume=1.0,
        constraint=dict(types=[1, 1, 1, 3], conc=[8.65e-2, 1.82e-2, 1.11e-2, 2e-3]),  # T T T Z
        log_formulation=True, act_coef="OFF",
        gold=read_gold(os.path.join(batch, "ion-exchange-valocchi.regression.gold")),
    )
    with open(os.path.join(HERE, "kat_ion_exchange_valocchi.json"), "w") as f:
        json.dump(fx, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
