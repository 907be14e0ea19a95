"""Reaction-network tables in PFLOTRAN's own layout.

`ReactionNetwork` collects primary species, aqueous complexes, kinetic
minerals, ion-exchange and surface-complexation reactions and lays them out
exactly as the corresponding fields of PFLOTRAN's reaction_type
(src/pflotran/reaction_aux.F90:142-335, reaction_mineral_aux.F90:76-132,
reaction_surf_complex_aux.F90:68-128): Fortran column-major, 1-based species
ids, id tables (0:ld, n) with the count in row 0.  BasisInit
(src/pflotran/reaction_database.F90:772) fills the same tables from a
database; here they are built directly.  `as_struct()` returns the
`pfchem_network` the C ABI takes.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import abi

# Debye-Hueckel parameters at 25 C (reaction_aux.F90:512-514)
DEBYE_A = 0.5114
DEBYE_B = 0.3288
DEBYE_BDOT = 0.0410


def _f64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def _i32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32))


def _ptr(a, kind):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(kind))


@dataclass
class _Rxn:
    species: list            # primary names
    stoich: list             # coefficients
    logK: float = 0.0
    logKcoef: tuple | None = None
    h2o: float = 0.0
    extra: dict = field(default_factory=dict)


class ReactionNetwork:
    def __init__(self, primaries, debye=(DEBYE_A, DEBYE_B, DEBYE_BDOT)):
        """primaries: list of (name, Z, a0)."""
        self.pri_names = [p[0] for p in primaries]
        self.pri_Z = [float(p[1]) for p in primaries]
        self.pri_a0 = [float(p[2]) for p in primaries]
        self.debye = tuple(float(x) for x in debye)
        self.complexes: list[_Rxn] = []
        self.minerals: list[_Rxn] = []
        self.ionx: list[dict] = []
        self.srfrxn: list[dict] = []
        self.gases: list[_Rxn] = []
        self._tables = None

    # -- builders ---------------------------------------------------------
    def idx(self, name):
        return self.pri_names.index(name)

    def add_complex(self, name, stoich, logK, Z=None, a0=3.0, logKcoef=None, h2o=0.0):
        sp = list(stoich.keys())
        nu = [float(stoich[s]) for s in sp]
        if Z is None:  # charge balance of the dissociation reaction
            Z = sum(n * self.pri_Z[self.idx(s)] for s, n in zip(sp, nu))
        self.complexes.append(_Rxn(sp, nu, float(logK), logKcoef, float(h2o),
                                   dict(name=name, Z=float(Z), a0=float(a0))))

    def add_kinetic_mineral(self, name, stoich, logK, rate_constant, molar_vol,
                            logKcoef=None, activation_energy=0.0, affinity_threshold=0.0,
                            rate_limiter=0.0, h2o=0.0, prefactors=None):
        sp = list(stoich.keys())
        nu = [float(stoich[s]) for s in sp]
        self.minerals.append(_Rxn(sp, nu, float(logK), logKcoef, float(h2o), dict(
            name=name, k=float(rate_constant), Vm=float(molar_vol), Ea=float(activation_energy),
            thr=float(affinity_threshold), lim=float(rate_limiter), pref=prefactors or [])))

    def add_ion_exchange(self, cations, CEC, to_mineral=0):
        """cations: list of (name, k); the first is the reference cation."""
        ids = [self.idx(c[0]) for c in cations]
        zs = [self.pri_Z[i] for i in ids]
        zflag = any(abs(z - zs[0]) > 1e-12 for z in zs)  # reaction_database.F90:2890-2909
        self.ionx.append(dict(ids=ids, k=[float(c[1]) for c in cations], CEC=float(CEC),
                              to_surf=int(to_mineral), zflag=bool(zflag)))

    def add_surface_complexation(self, site_density, complexes, surf_type=abi.NULL_SURFACE, to_mineral=0):
        """complexes: list of (stoich dict, free_site_stoich, logK)."""
        cx = []
        flag = False
        for st, fs, lk in complexes:
            sp = list(st.keys())
            cx.append(_Rxn(sp, [float(st[s]) for s in sp], float(lk), None, 0.0, dict(fs=float(fs))))
            if abs(fs - 1.0) > 1e-12:
                flag = True
        self.srfrxn.append(dict(site_density=float(site_density), complexes=cx,
                                surf_type=int(surf_type), to_surf=int(to_mineral), flag=flag))

    def add_passive_gas(self, name, stoich, logK, logKcoef=None, h2o=0.0):
        """A passive gas (reaction_gas_aux.F90 gas%paseq*): its reaction in the
        primaries, log10 K at 25 C and the optional log K(T) fit.  Used by
        GAS constraint rows only (no gas phase in the reaction step)."""
        sp = list(stoich.keys())
        self.gases.append(_Rxn(sp, [float(stoich[s]) for s in sp], float(logK), logKcoef, float(h2o),
                               dict(name=name)))

    def gas_id(self, name):
        """1-based id of a passive gas (a GAS row's constraint_spec_id)."""
        return [g.extra["name"] for g in self.gases].index(name) + 1

    def gas_table(self):
        """The passive-gas arrays of a pfchem_constraint (abi.constraint's
        `gases`): paseqspecid (0:ld, n), paseqstoich (ld, n), h2o ids and
        stoichiometries, log K and the log K(T) fit (5, n)."""
        n = len(self.gases)
        ld = max([len(g.species) for g in self.gases] + [1])
        if ld > abi.PFCHEM_MAX_NNZ:
            raise ValueError(f"a gas reaction has {ld} species (at most {abi.PFCHEM_MAX_NNZ})")
        ids, nus = self._idtab(self.gases, ld, lambda rx: ([self.idx(q) for q in rx.species], rx.stoich))
        return dict(n=n, ld=ld, specid=ids, stoich=nus,
                    h2oid=_i32([1 if abs(g.h2o) > 0 else 0 for g in self.gases] or [0]),
                    h2ostoich=_f64([g.h2o for g in self.gases] or [0.0]),
                    logK=_f64([g.logK for g in self.gases] or [0.0]), logKcoef=_f64(self._coefs(self.gases)))

    # -- tables -------------------------------------------------------------
    @staticmethod
    def _idtab(rxns, ld, ids_of):
        n = len(rxns)
        t = np.zeros((max(n, 1), ld + 1), dtype=np.int32)  # row r = Fortran column r
        s = np.zeros((max(n, 1), ld), dtype=np.float64)
        for r, rx in enumerate(rxns):
            ids, nus = ids_of(rx)
            t[r, 0] = len(ids)
            for k, (i, nu) in enumerate(zip(ids, nus)):
                t[r, k + 1] = i + 1
                s[r, k] = nu
        return t.ravel(), s.ravel()

    def _coefs(self, rxns):
        out = np.zeros((max(len(rxns), 1), 5))
        for r, rx in enumerate(rxns):
            out[r] = rx.logKcoef if rx.logKcoef is not None else (0.0, rx.logK, 0.0, 0.0, 0.0)
        return out.ravel()

    def build(self):
        N = len(self.pri_names)
        t = {}
        ids_of = lambda rx: ([self.idx(s) for s in rx.species], rx.stoich)
        ld_c = max([len(c.species) for c in self.complexes] + [1])
        ld_m = max([len(m.species) for m in self.minerals] + [1])
        t["eqcplx_ld"], t["kinmnrl_ld"] = ld_c, ld_m
        t["eqcplxspecid"], t["eqcplxstoich"] = self._idtab(self.complexes, ld_c, ids_of)
        t["eqcplxh2oid"] = _i32([1 if c.h2o != 0 else 0 for c in self.complexes] or [0])
        t["eqcplxh2ostoich"] = _f64([c.h2o for c in self.complexes] or [0.0])
        t["eqcplx_Z"] = _f64([c.extra["Z"] for c in self.complexes] or [0.0])
        t["eqcplx_a0"] = _f64([c.extra["a0"] for c in self.complexes] or [0.0])
        t["eqcplx_logK"] = _f64([c.logK for c in self.complexes] or [0.0])
        t["eqcplx_logKcoef"] = _f64(self._coefs(self.complexes))
        t["kinmnrlspecid"], t["kinmnrlstoich"] = self._idtab(self.minerals, ld_m, ids_of)
        t["kinmnrlh2oid"] = _i32([1 if m.h2o != 0 else 0 for m in self.minerals] or [0])
        t["kinmnrlh2ostoich"] = _f64([m.h2o for m in self.minerals] or [0.0])
        t["kinmnrl_logK"] = _f64([m.logK for m in self.minerals] or [0.0])
        t["kinmnrl_logKcoef"] = _f64(self._coefs(self.minerals))
        for key, f in (("kinmnrl_rate_constant", "k"), ("kinmnrl_molar_vol", "Vm"),
                       ("kinmnrl_activation_energy", "Ea"), ("kinmnrl_affinity_threshold", "thr"),
                       ("kinmnrl_rate_limiter", "lim")):
            t[key] = _f64([m.extra[f] for m in self.minerals] or [0.0])
        # rate prefactors (reaction_database.F90:1943-1965 layout)
        maxp = max([len(m.extra["pref"]) for m in self.minerals] + [0])
        maxs = max([len(p["species"]) for m in self.minerals for p in m.extra["pref"]] + [0])
        t["max_num_prefactors"], t["max_num_prefactor_species"] = maxp, maxs
        if maxp > 0:
            Nm = len(self.minerals)
            pid = np.zeros((Nm, maxp, maxs + 1), np.int32)
            alpha = np.zeros((Nm, maxp, maxs))
            beta = np.zeros((Nm, maxp, maxs))
            atten = np.zeros((Nm, maxp, maxs))
            prate = np.zeros((Nm, maxp))
            pEa = np.zeros((Nm, maxp))
            npref = np.zeros(Nm, np.int32)
            for m, mn in enumerate(self.minerals):
                npref[m] = len(mn.extra["pref"])
                for p, pf in enumerate(mn.extra["pref"]):
                    prate[m, p] = pf["rate"]
                    pEa[m, p] = pf.get("Ea", 0.0)
                    pid[m, p, 0] = len(pf["species"])
                    for s, sp in enumerate(pf["species"]):
                        # ("name", alpha, beta, atten); a complex name gives a negative id
                        nm = sp[0]
                        if nm in self.pri_names:
                            pid[m, p, s + 1] = self.idx(nm) + 1
                        else:
                            ci = [c.extra["name"] for c in self.complexes].index(nm)
                            pid[m, p, s + 1] = -(ci + 1)
                        alpha[m, p, s], beta[m, p, s], atten[m, p, s] = sp[1], sp[2], sp[3]
            t["kinmnrl_num_prefactors"] = npref
            t["kinmnrl_pref_rate"] = prate.ravel()
            t["kinmnrl_pref_activation_energy"] = pEa.ravel()
            t["kinmnrl_prefactor_id"] = pid.ravel()
            t["kinmnrl_pref_alpha"] = alpha.ravel()
            t["kinmnrl_pref_beta"] = beta.ravel()
            t["kinmnrl_pref_atten_coef"] = atten.ravel()
        # ion exchange
        ld_x = max([len(x["ids"]) for x in self.ionx] + [1])
        t["eqionx_ld"] = ld_x
        xid = np.zeros((max(len(self.ionx), 1), ld_x + 1), np.int32)
        xk = np.zeros((max(len(self.ionx), 1), ld_x))
        for r, x in enumerate(self.ionx):
            xid[r, 0] = len(x["ids"])
            xid[r, 1:len(x["ids"]) + 1] = np.array(x["ids"]) + 1
            xk[r, :len(x["k"])] = x["k"]
        t["eqionx_rxn_cationid"], t["eqionx_rxn_k"] = xid.ravel(), xk.ravel()
        t["eqionx_rxn_CEC"] = _f64([x["CEC"] for x in self.ionx] or [0.0])
        t["eqionx_rxn_to_surf"] = _i32([x["to_surf"] for x in self.ionx] or [0])
        t["eqionx_rxn_Z_flag"] = _i32([int(x["zflag"]) for x in self.ionx] or [0])
        # surface complexation
        allc = [c for s in self.srfrxn for c in s["complexes"]]
        ld_sr = max([len(s["complexes"]) for s in self.srfrxn] + [1])
        ld_sc = max([len(c.species) for c in allc] + [1])
        t["srfcplxrxn_ld"], t["srfcplx_ld"] = ld_sr, ld_sc
        r2c = np.zeros((max(len(self.srfrxn), 1), ld_sr + 1), np.int32)
        k = 0
        for r, s in enumerate(self.srfrxn):
            r2c[r, 0] = len(s["complexes"])
            for j in range(len(s["complexes"])):
                r2c[r, j + 1] = k + 1
                k += 1
        t["srfcplxrxn_to_complex"] = r2c.ravel()
        t["srfcplxrxn_surf_type"] = _i32([s["surf_type"] for s in self.srfrxn] or [0])
        t["srfcplxrxn_to_surf"] = _i32([s["to_surf"] for s in self.srfrxn] or [0])
        t["srfcplxrxn_site_density"] = _f64([s["site_density"] for s in self.srfrxn] or [0.0])
        t["srfcplxrxn_stoich_flag"] = _i32([int(s["flag"]) for s in self.srfrxn] or [0])
        t["srfcplxspecid"], t["srfcplxstoich"] = self._idtab(allc, ld_sc, ids_of)
        t["srfcplxh2oid"] = _i32([0] * max(len(allc), 1))
        t["srfcplxh2ostoich"] = _f64([0.0] * max(len(allc), 1))
        t["srfcplx_free_site_stoich"] = _f64([c.extra["fs"] for c in allc] or [0.0])
        t["srfcplx_logK"] = _f64([c.logK for c in allc] or [0.0])
        t["srfcplx_logKcoef"] = _f64(self._coefs(allc))
        t["primary_spec_Z"] = _f64(self.pri_Z)
        t["primary_spec_a0"] = _f64(self.pri_a0)
        self._tables = t
        self._nsc = len(allc)
        return t

    @property
    def N(self):
        return len(self.pri_names)

    @property
    def Nc(self):
        return len(self.complexes)

    @property
    def Nm(self):
        return len(self.minerals)

    @property
    def Nix(self):
        return len(self.ionx)

    @property
    def Nsr(self):
        return len(self.srfrxn)

    @property
    def Nsc(self):
        return sum(len(s["complexes"]) for s in self.srfrxn)

    def as_struct(self, temkin=None, min_scale=None, affinity_power=None) -> abi.Network:
        t = self._tables if self._tables is not None else self.build()
        s = abi.Network()
        s.naqcomp, s.neqcplx, s.nkinmnrl = self.N, self.Nc, self.Nm
        s.neqionxrxn, s.nsrfcplxrxn, s.nsrfcplx = self.Nix, self.Nsr, self.Nsc
        for k in ("eqcplx_ld", "kinmnrl_ld", "eqionx_ld", "srfcplxrxn_ld", "srfcplx_ld",
                  "max_num_prefactors", "max_num_prefactor_species"):
            setattr(s, k, int(t[k]))
        s.debyeA, s.debyeB, s.debyeBdot = self.debye
        keep = []
        for name, kind in abi.Network._fields_:
            if name in t and kind in (C.POINTER(C.c_int32), C.POINTER(C.c_double)):
                arr = t[name]
                keep.append(arr)
                setattr(s, name, _ptr(arr, C.c_int32 if kind == C.POINTER(C.c_int32) else C.c_double))
        for name, arr in (("kinmnrl_Temkin_const", temkin), ("kinmnrl_min_scale_factor", min_scale),
                          ("kinmnrl_affinity_power", affinity_power)):
            if arr is not None:
                a = _f64(arr)
                keep.append(a)
                setattr(s, name, _ptr(a, C.c_double))
        s._keep = keep  # keep the numpy buffers alive with the struct
        return s


def default_options(**kw) -> abi.Options:
    """PFLOTRAN's defaults (reaction_aux.F90:418-433, :569-571, option.F90:412)
    with the library's extra fields; keyword arguments override."""
    o = abi.Options()
    o.use_log_formulation = 1
    o.act_coef_update_frequency = abi.ACT_COEF_FREQUENCY_TIMESTEP
    o.act_coef_update_algorithm = abi.ACT_COEF_ALGORITHM_LAG
    o.use_activity_h2o = 0
    o.use_isothermal = 0
    o.residual_tol_kind = abi.RESIDUAL_RELATIVE
    o.accum_mode = abi.ACCUM_DT_CONSISTENT
    o.max_iterations = 200
    o.max_dlnC = 5.0
    o.max_relative_change_tolerance = 0.0
    o.max_residual_tolerance = 1e-12
    o.update_kinetic_state = 1
    o.jacobian = abi.JACOBIAN_REFERENCE
    # RReact's own iterations up to its damping threshold (iteration 50), the
    # exact Jacobian without damping for the few cells still unconverged
    o.exact_jacobian_after = 50
    for k, v in kw.items():
        setattr(o, k, v)
    return o
