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
species.  When that set is not the database's own basis (a primary that the
database lists as a secondary species, e.g. CO2(aq) instead of HCO3-), the
reactions are rewritten for the new basis as BasisInit does
(reaction_database.F90:772-1560): every reaction of a chosen primary or
secondary species that the database defines is a row of
  pri . P + sec . S = log K
over the basis P (H2O and the primaries) and the secondary species S; with
the secondary block inverted, each secondary species becomes
S = -sec^-1 pri . P with log K = -sec^-1 . log K, and every secondary species
left in a mineral or surface-complex reaction is replaced by its rewritten
reaction, scaled by its coefficient there, log K likewise
(BasisSubSpeciesInMineralRxn / BasisSubSpeciesInGasOrSecRxn,
reaction_database_aux.F90:355-545).  Differences, deliberate: the secondary
block is solved with numpy instead of ludcmp/lubksb (log K agrees to
rounding); a rewritten log K at a temperature where any reaction it combines
has no data is marked as no data (500) instead of being combined; and
rewritten coefficients within 1e-12 of an integer are snapped to it, so
that a swap does not leave 1e-16 coefficients in the kinetic tables.  Gas
species are not supported: a reaction that needs one (e.g. redox couples
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


def _has_data(k):
    return abs(k - NO_DATA) > 1e-10


def _combine(terms, ntemp):
    """sum of scale * logK vectors over (scale, logK) terms, per temperature;
    no data where any term with a nonzero scale has none."""
    out = []
    for t in range(ntemp):
        if any(abs(c) > 0 and not _has_data(k[t]) for c, k in terms):
            out.append(NO_DATA)
        else:
            out.append(sum(c * k[t] for c, k in terms))
    return out


def _snap(v):
    r = round(v)
    return float(r) if abs(v - r) <= 1e-12 else float(v)


def swap_basis(db, primaries, secondary):
    """Reactions of the `secondary` species written in the basis H2O +
    `primaries` (the BasisInit rewrite): {name: (stoich {species: nu},
    logK per database temperature, a0, Z)}."""
    basis = ["H2O"] + list(primaries)
    bidx = {n: i for i, n in enumerate(basis)}
    sidx = {n: i for i, n in enumerate(secondary)}
    for n in primaries:
        if n in sidx:
            raise ValueError(f"{n} is listed as both a primary and a secondary species")
    rows = []   # (self name, database reaction)
    for n in primaries:
        if n not in db.primaries:
            if n not in db.secondary:
                raise ValueError(f"primary species {n} is in neither the database's primary nor secondary species")
            rows.append((n, db.secondary[n]))
    for n in secondary:
        if n in db.secondary:
            rows.append((n, db.secondary[n]))
        elif n not in db.primaries:
            raise ValueError(f"secondary species {n} is not in the database")
    ns = len(secondary)
    if len(rows) != ns:
        raise ValueError(f"{len(rows)} reactions from the database for {ns} secondary species: the primaries "
                         f"and secondaries do not span the same components as the database's basis")
    pri = np.zeros((ns, len(basis)))
    sec = np.zeros((ns, ns))
    nt = len(db.temperatures)
    logK = np.zeros((ns, nt))
    for r, (n, rx) in enumerate(rows):
        if n in bidx:
            pri[r, bidx[n]] = -1.0
        else:
            sec[r, sidx[n]] = -1.0
        for sp, nu in rx.stoich:
            if sp in bidx:
                pri[r, bidx[sp]] += nu
            elif sp in sidx:
                sec[r, sidx[sp]] += nu
            else:
                raise ValueError(f"species {sp} in the reaction of {n} is not among the primary or secondary "
                                 f"species (gases and basis swaps through them are not supported)")
        logK[r] = rx.logK
    try:
        inv = np.linalg.inv(sec)
    except np.linalg.LinAlgError:
        raise ValueError("the secondary species' reactions are not independent in this basis") from None
    stoich = -inv @ pri
    own = {n: rx for n, rx in rows}
    out = {}
    for k, n in enumerate(secondary):
        st = {basis[j]: _snap(v) for j, v in enumerate(stoich[k]) if abs(v) > 1e-10}
        if n in own:  # keep the database's species order, then the basis order
            first = [sp for sp, _ in own[n].stoich if sp in st]
            st = {sp: st[sp] for sp in first + [sp for sp in st if sp not in first]}
        lk = _combine([(-inv[k, r], logK[r]) for r in range(ns)], nt)
        if n in db.primaries:
            a0, Z = db.primaries[n]
        else:
            a0, Z = db.secondary[n].a0, db.secondary[n].Z
        out[n] = (st, lk, a0, Z)
    return out


def rewrite_in_basis(rx_stoich, rx_logK, swapped, basis, what):
    """A mineral or surface-complex reaction with every secondary species in
    it replaced by its rewritten reaction (scaled by its coefficient), log K
    likewise; species whose coefficients cancel (|nu| <= 1e-10) are dropped.
    Raises when a species is left that is not in `basis` (plus surface
    sites, names starting with '>')."""
    st = dict()
    for sp, nu in rx_stoich:
        st[sp] = st.get(sp, 0.0) + nu
    terms = [(1.0, list(rx_logK))]
    for sp in list(st):
        if sp in swapped and sp not in basis:
            scale = st.pop(sp)
            s2, lk2, _, _ = swapped[sp]
            for q, v in s2.items():
                st[q] = st.get(q, 0.0) + scale * v
            terms.append((scale, lk2))
    st = {q: _snap(v) for q, v in st.items() if abs(v) > 1e-10}
    bad = [q for q in st if q not in basis and not q.startswith(">")]
    if bad:
        raise ValueError(f"{what}: reaction uses {bad}, not among the primaries or the secondary species")
    return [(q, v) for q, v in st.items()], _combine(terms, len(rx_logK))


def network_from_database(db, primaries, secondary=None, kinetic_minerals=None, ion_exchange=None,
                          surface_complexation=None, debye=None, gases=None):
    """ReactionNetwork for `primaries` (the database's basis or another one,
    rewritten as the module notes describe).

    secondary: names of the aqueous complexes, or, in the database's own
      basis, None for every secondary species whose reaction uses only the
      primaries and H2O (PFLOTRAN lists them in the input deck; this is the
      usual "all that apply");
    kinetic_minerals: {name: dict(rate_constant=mol/m^2/s, ...)} with the
      other add_kinetic_mineral keywords;
    ion_exchange: [(cations with selectivities [(name, k)], CEC)];
    surface_complexation: [(site_density, [complex names], keywords)];
    gases: names of passive gases (GAS constraint rows), their reactions
      rewritten in the primaries like the minerals'.
    Log K is the 25 C value; the temperature fit is attached when the
    database has five or more temperatures with data."""
    from .network import ReactionNetwork

    def primary_params(p):
        if p in db.primaries:
            return db.primaries[p][1], db.primaries[p][0]
        rx = db.secondary[p] if p in db.secondary else None
        if rx is None:
            raise ValueError(f"primary species {p} is not in the database")
        return rx.Z, rx.a0

    prim = [(p, *primary_params(p)) for p in primaries]
    net = ReactionNetwork(prim, **({} if debye is None else {"debye": debye}))
    allowed = set(primaries) | {"H2O"}
    swap = any(p not in db.primaries for p in primaries)
    if secondary is None:
        if swap:
            raise ValueError("a basis other than the database's needs the secondary species listed")
        names = [n for n, rx in db.secondary.parsable()
                 if n not in allowed and all(s in allowed for s, _ in rx.stoich) and
                 _has_data(rx.logK[db.temperatures.index(25.0)])]
    else:
        names = list(secondary)
    swapped = swap_basis(db, primaries, names)
    t25 = db.temperatures.index(25.0)

    def fit(lk):
        return fit_logK(db.temperatures, lk)

    def at25(lk, what):
        if not _has_data(lk[t25]):
            raise ValueError(f"{what}: no log K at 25 C")
        return lk[t25]

    for n in names:
        st, lk, a0, Z = swapped[n]
        net.add_complex(n, {s: v for s, v in st.items() if s != "H2O"}, logK=at25(lk, n), Z=Z, a0=a0,
                        logKcoef=fit(lk), h2o=st.get("H2O", 0.0))
    for n, kw in (kinetic_minerals or {}).items():
        rx = db.minerals[n]
        st, lk = rewrite_in_basis(rx.stoich, rx.logK, swapped, allowed, f"mineral {n}")
        kw = dict(kw)
        kw.setdefault("molar_vol", rx.molar_vol_cm3 * 1e-6)
        net.add_kinetic_mineral(n, {s: v for s, v in st if s != "H2O"}, logK=at25(lk, n), logKcoef=fit(lk), **kw)
    for n in gases or []:
        if not db.gases or n not in db.gases:
            raise ValueError(f"gas {n} is not in the database")
        rx = db.gases[n]
        st, lk = rewrite_in_basis(rx.stoich, rx.logK, swapped, allowed, f"gas {n}")
        net.add_passive_gas(n, {s: v for s, v in st if s != "H2O"}, logK=at25(lk, n), logKcoef=fit(lk),
                            h2o=dict(st).get("H2O", 0.0))
    for cations, cec in (ion_exchange or []):
        net.add_ion_exchange(cations, cec)
    for site_density, complexes, kw in (surface_complexation or []):
        cplx = []
        for n in complexes:
            rx = db.surface_complexes[n]
            sites = [s for s, _ in rx.stoich if s.startswith(">")]
            if len(set(sites)) != 1:
                raise ValueError(f"surface complex {n}: expected one surface site, found {sites}")
            st, lk = rewrite_in_basis(rx.stoich, rx.logK, swapped, allowed, f"surface complex {n}")
            rest = {s: v for s, v in st if not s.startswith(">") and s != "H2O"}
            fs = sum(v for s, v in st if s.startswith(">"))
            cplx.append((rest, fs, at25(lk, n)))
        net.add_surface_complexation(site_density, cplx, **kw)
    net.build()
    return net
