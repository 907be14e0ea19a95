"""Reader for PFLOTRAN thermodynamic databases (the `.dat` format of
database/hanford.dat) and assembly of a ReactionNetwork from it.

The format (read by DatabaseRead, src/pflotran/reaction_database.F90:25-768)
is whitespace-separated records with quoted names, in five blocks each
closed by a record named 'null':

  'temperature points' ntemp T1 ... Tn
  primary species:   'name' a0 Z molar_weight
  secondary species: 'name' n (nu 'species') x n  logK x ntemp  a0 Z molar_weight
  gases:             'name' molar_volume n (nu 'species') x n  logK x ntemp  molar_weight
  minerals:          'name' molar_volume n (nu 'species') x n  logK x ntemp  molar_weight
  surface complexes: 'name' n (nu 'species') x n  logK x ntemp  Z molar_weight

log K = 500 marks a temperature without data.  `fit_logK` restates
ReactionFitLogKCoef (reaction_aux.F90:1336-1408): a least-squares fit of
log K(T) = c1 ln T_K + c2 + c3 T_K + c4 / T_K + c5 / T_K^2 over the
temperatures with data.

`network_from_database` builds a ReactionNetwork for a chosen set of primary
species in the database's own basis: every secondary species, mineral and
surface complex must be written in terms of the chosen primaries (and
H2O).  PFLOTRAN's basis swap (reaction_database.F90:772-, which rewrites
reactions for a different basis) is not done: a species whose reaction
uses a component that is not among the primaries (e.g. redox couples
written with O2(g)) is rejected with a message naming it.
"""
from __future__ import annotations

import math
import re
from dataclasses import dataclass, field

import numpy as np

NO_DATA = 500.0


@dataclass
class Reaction:
    name: str
    stoich: list           # [(species, nu)]
    logK: list             # per database temperature
    a0: float = 0.0
    Z: float = 0.0
    molar_vol_cm3: float = 0.0


class _Block(dict):
    """Records of one block, parsed when first used: as in DatabaseRead, only
    the entries a network needs have to be well formed (some databases carry
    entries whose counts do not match their tokens)."""

    def __init__(self, kind, ntemp):
        super().__init__()
        self.kind, self.ntemp, self.raw = kind, ntemp, {}

    def __contains__(self, name):
        return name in self.raw

    def __iter__(self):
        return iter(self.raw)

    def __len__(self):
        return len(self.raw)

    def __getitem__(self, name):
        if not dict.__contains__(self, name):
            dict.__setitem__(self, name, _reaction(self.raw[name], self.ntemp, self.kind))
        return dict.__getitem__(self, name)

    def items(self):
        return ((n, self[n]) for n in self.raw)

    def parsable(self):
        """(name, Reaction) of the entries that parse."""
        for n in self.raw:
            try:
                yield n, self[n]
            except (ValueError, IndexError):
                continue


@dataclass
class Database:
    temperatures: list
    primaries: dict = field(default_factory=dict)     # name -> (a0, Z)
    secondary: dict = None                            # name -> Reaction
    gases: dict = None
    minerals: dict = None
    surface_complexes: dict = None


def _tokens(line):
    return re.findall(r"'[^']*'|\S+", line)


def _name(tok):
    return tok.strip("'")


def _num(tok):
    """A Fortran real (1.5d0 / 1.5D-3 exponents allowed)."""
    return float(tok.replace("d", "e").replace("D", "e"))


def _reaction(toks, ntemp, kind):
    i = 0
    out = Reaction(name=_name(toks[0]), stoich=[], logK=[])
    i = 1
    if kind in ("gas", "mineral"):
        out.molar_vol_cm3 = _num(toks[i])
        i += 1
    n = int(_num(toks[i]))
    i += 1
    for _ in range(n):
        out.stoich.append((_name(toks[i + 1]), _num(toks[i])))
        i += 2
    out.logK = [_num(x) for x in toks[i:i + ntemp]]
    i += ntemp
    if kind == "secondary":
        out.a0, out.Z = _num(toks[i]), _num(toks[i + 1])
    elif kind == "surface":
        out.Z = _num(toks[i])
    return out


def read_database(path):
    """Parses a PFLOTRAN .dat database."""
    blocks = ("primaries", "secondary", "gases", "minerals", "surface_complexes")
    kinds = (None, "secondary", "gas", "mineral", "surface")
    db = None
    b = 0
    with open(path) as f:
        for raw in f:
            line = raw.strip()
            if not line or line.startswith("!"):
                continue
            toks = _tokens(line)
            head = _name(toks[0])
            if head == "temperature points":
                nt = int(toks[1])
                db = Database(temperatures=[_num(x) for x in toks[2:2 + nt]])
                for blk, kind in zip(blocks[1:], kinds[1:]):
                    setattr(db, blk, _Block(kind, nt))
                continue
            if db is None:
                raise ValueError(f"{path}: no 'temperature points' record before the species")
            if head == "null":
                b += 1
                if b >= len(blocks):
                    break
                continue
            if b == 0:
                db.primaries[head] = (_num(toks[1]), _num(toks[2]))
            else:
                getattr(db, blocks[b]).raw.setdefault(head, toks)
    if db is None:
        raise ValueError(f"{path}: empty database")
    return db


def fit_logK(temperatures, logK):
    """Maier-Kelly coefficients (c1..c5) of log K(T) from the database
    temperatures with data; None with fewer than five of them."""
    rows, vals = [], []
    for t, k in zip(temperatures, logK):
        if abs(k - NO_DATA) < 1e-10:
            continue
        tk = t + 273.15
        rows.append((math.log(tk), 1.0, tk, 1.0 / tk, 1.0 / (tk * tk)))
        vals.append(k)
    if len(rows) < 5:
        return None
    A = np.array(rows)
    y = np.array(vals)
    return tuple(np.linalg.solve(A.T @ A, A.T @ y))


def logK_at_25(db, rx):
    if 25.0 not in db.temperatures:
        raise ValueError("the database has no 25 C column")
    k = rx.logK[db.temperatures.index(25.0)]
    if abs(k - NO_DATA) < 1e-10:
        raise ValueError(f"{rx.name}: no log K at 25 C")
    return k


def network_from_database(db, primaries, secondary=None, kinetic_minerals=None, ion_exchange=None,
                          surface_complexation=None, debye=None):
    """ReactionNetwork for `primaries` (names in the database's basis).

    secondary: names of the aqueous complexes, or None for every secondary
      species whose reaction uses only the primaries and H2O (PFLOTRAN lists
      them in the input deck; this is the usual "all that apply");
    kinetic_minerals: {name: dict(rate_constant=mol/m^2/s, ...)} with the
      other add_kinetic_mineral keywords;
    ion_exchange: [(cations with selectivities [(name, k)], CEC)];
    surface_complexation: [(site_density, [complex names], keywords)].
    Log K is the 25 C value; the temperature fit is attached when the
    database has five or more temperatures with data."""
    from .network import ReactionNetwork
    prim = [(p, db.primaries[p][1], db.primaries[p][0]) for p in primaries]
    net = ReactionNetwork(prim, **({} if debye is None else {"debye": debye}))
    allowed = set(primaries) | {"H2O"}

    def check(rx, what):
        bad = [s for s, _ in rx.stoich if s not in allowed]
        if bad:
            raise ValueError(f"{what} {rx.name}: reaction uses {bad}, not among the primaries "
                             f"(a basis swap is not supported)")

    if secondary is None:
        names = [n for n, rx in db.secondary.parsable()
                 if n not in allowed and all(s in allowed for s, _ in rx.stoich) and
                 abs(rx.logK[db.temperatures.index(25.0)] - NO_DATA) > 1e-10]
    else:
        names = list(secondary)
    for n in names:
        rx = db.secondary[n]
        check(rx, "secondary species")
        st = {s: v for s, v in rx.stoich if s != "H2O"}
        h2o = sum(v for s, v in rx.stoich if s == "H2O")
        net.add_complex(n, st, logK=logK_at_25(db, rx), Z=rx.Z, a0=rx.a0,
                        logKcoef=fit_logK(db.temperatures, rx.logK), h2o=h2o)
    for n, kw in (kinetic_minerals or {}).items():
        rx = db.minerals[n]
        check(rx, "mineral")
        st = {s: v for s, v in rx.stoich if s != "H2O"}
        kw = dict(kw)
        kw.setdefault("molar_vol", rx.molar_vol_cm3 * 1e-6)
        net.add_kinetic_mineral(n, st, logK=logK_at_25(db, rx), logKcoef=fit_logK(db.temperatures, rx.logK), **kw)
    for cations, cec in (ion_exchange or []):
        net.add_ion_exchange(cations, cec)
    for site_density, complexes, kw in (surface_complexation or []):
        cplx = []
        for n in complexes:
            rx = db.surface_complexes[n]
            sites = [s for s, _ in rx.stoich if s.startswith(">")]
            rest = {s: v for s, v in rx.stoich if not s.startswith(">") and s != "H2O"}
            bad = [s for s in rest if s not in allowed]
            if bad:
                raise ValueError(f"surface complex {n}: reaction uses {bad}, not among the primaries")
            if len(set(sites)) != 1:
                raise ValueError(f"surface complex {n}: expected one surface site, found {sites}")
            fs = sum(v for s, v in rx.stoich if s.startswith(">"))
            cplx.append((rest, fs, logK_at_25(db, rx)))
        net.add_surface_complexation(site_density, cplx, **kw)
    net.build()
    return net
