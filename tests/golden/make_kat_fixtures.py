"""Writes the known-answer fixtures of PFLOTRAN's batch chemistry regression
tests into tests/golden/*.json.

Run in a checkout that has the PFLOTRAN source tree (argument: its root):

    python tests/golden/make_kat_fixtures.py /path/to/pflotran

It reads, as text, the database rows and the regression gold values of

  regression_tests/ascem/batch/calcite-kinetics.{in,regression.gold} + calcite.dat
  regression_tests/ascem/batch/calcite-kinetics-volume-fractions.{in,regression.gold}
  regression_tests/ascem/batch/ion-exchange-valocchi.{in,regression.gold} + hanford.dat
  regression_tests/ascem/batch/surface-complexation-1.{in,regression.gold}
      + surface-complexation.dat
  regression_tests/ascem/batch/{carbonate,ca-carbonate}-{unit,debye-huckel}-activity
      .{in,regression.gold} + carbonate.dat / ca-carbonate.dat

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


def parse_srfcplx(toks, ntemp):
    # 'name' n (nu 'species') x n  logK x ntemp  Z molar_weight
    nsp = int(toks[0])
    st = [(toks[2 + 2 * k].strip("'"), float(toks[1 + 2 * k])) for k in range(nsp)]
    i = 1 + 2 * nsp
    return dict(stoich=st, logK=[float(x) for x in toks[i:i + ntemp]], Z=float(toks[i + ntemp]))


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
    # calcite-kinetics-volume-fractions: the same deck but for the time
    # card (FINAL_TIME 60 mo = 60 x 365/12 d, units.F90:445-446; initial and
    # maximum step 30 d) and the constraint (H+ 1e-2, HCO3- 1e-2, Ca++ 1e-19 T)
    vf = dict(fx)
    vf.update(source="regression_tests/ascem/batch/calcite-kinetics-volume-fractions.in + calcite.dat "
                     "+ .regression.gold",
              final_time=60 * 365.0 / 12.0 * 86400.0, dt=30.0 * 86400.0, nsteps=None,
              constraint=dict(types=[1, 1, 1], conc=[1e-2, 1e-2, 1e-19]),
              gold=read_gold(os.path.join(batch, "calcite-kinetics-volume-fractions.regression.gold")))
    with open(os.path.join(HERE, "kat_calcite_kinetics_volume_fractions.json"), "w") as f:
        json.dump(vf, f, indent=1)
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
    # --- surface-complexation-1 ---------------------------------------------
    pri = ["H+", "Na+", "NO3-", "Zn++"]                                        # .in PRIMARY_SPECIES
    sec = ["OH-", "Zn(OH)2(aq)", "Zn(OH)3-", "Zn(OH)4--", "ZnOH+"]              # .in SECONDARY_SPECIES
    srf = [">FeOH2+_w", ">FeO-_w", ">FeOHZn+_w"]                               # .in COMPLEXES
    temps, rows = read_dat(os.path.join(batch, "surface-complexation.dat"), set(pri + sec + srf))
    fx = dict(
        source="regression_tests/ascem/batch/surface-complexation-1.in + surface-complexation.dat "
               "+ .regression.gold (time 0: the gold is the initial constraint state)",
        temperatures=temps,
        primaries=[dict(name=p, **parse_primary(rows[p])) for p in pri],
        complexes=[dict(name=s, **parse_rxn(rows[s], len(temps))) for s in sec],
        # SORPTION SURFACE_COMPLEXATION_RXN EQUILIBRIUM SITE >FeOH_w 7.6355e4 (mol/m^3 bulk)
        surface=dict(site=">FeOH_w", site_density=7.6355e4,
                     complexes=[dict(name=s, **parse_srfcplx(rows[s], len(temps))) for s in srf]),
        porosity=0.9, volume=1.0,                                  # POROSITY 0.9d0; 1 m^3 cell
        # CONSTRAINT initial: H+ 5.0 P, Na+ 1.0e-5 Z, NO3- 1.0e-1 T, Zn++ 1.0e-7 T
        constraint=dict(types=[4, 3, 1, 1], conc=[5.0, 1e-5, 1e-1, 1e-7]),
        log_formulation=True, act_coef="TIMESTEP",
        gold=read_gold(os.path.join(batch, "surface-complexation-1.regression.gold")),
    )
    with open(os.path.join(HERE, "kat_surface_complexation_1.json"), "w") as f:
        json.dump(fx, f, indent=1)
    # --- carbonate speciation decks (all at time 0: the constraint state) ----
    decks = {}
    for deck, dat, pri, sec, conc in (
            ("carbonate", "carbonate.dat", ["H+", "HCO3-"], ["OH-", "CO3--", "CO2(aq)"], [1e-3, 1e-3]),
            ("ca-carbonate", "ca-carbonate.dat", ["HCO3-", "Ca++", "H+"],
             ["OH-", "CO2(aq)", "CO3--", "CaOH+", "CaHCO3+", "CaCO3(aq)"], [3e-3, 1e-3, 1e-3])):
        temps, rows = read_dat(os.path.join(batch, dat), set(pri + sec))
        for act in ("unit", "debye-huckel"):
            name = f"{deck}-{act}-activity"
            decks[name] = dict(
                source=f"regression_tests/ascem/batch/{name}.in + {dat} + .regression.gold (time 0)",
                temperatures=temps,
                primaries=[dict(name=p, **parse_primary(rows[p])) for p in pri],
                complexes=[dict(name=s, **parse_rxn(rows[s], len(temps))) for s in sec],
                porosity=0.25, volume=1.0,                      # POROSITY 0.25d0; 1 m^3 cell
                constraint=dict(types=[1] * len(pri), conc=conc),  # CONSTRAINT initial: T rows
                # ACTIVITY_COEFFICIENTS TIMESTEP in the debye-huckel decks, absent (off) in the others
                log_formulation=True, act_coef="TIMESTEP" if act == "debye-huckel" else "OFF",
                gold=read_gold(os.path.join(batch, f"{name}.regression.gold")),
            )
    with open(os.path.join(HERE, "kat_carbonate_speciation.json"), "w") as f:
        json.dump(decks, f, indent=1)


if __name__ == "__main__":
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PFLOTRAN_SOURCE_DIR")
    if not src:
        sys.exit("usage: make_kat_fixtures.py <pflotran source tree> (or set PFLOTRAN_SOURCE_DIR)")
    main(src)
