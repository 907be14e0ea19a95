"""Seeded synthetic workloads for the per-cell chemistry step.

Three workloads, each a (network, options, cells, dt) tuple:

* calcite column (100 cells, 25 C, dt 3600 s): the calcite system of
  PFLOTRAN's regression tests (regression_tests/ascem/batch/calcite.dat),
  primaries H+, HCO3-, Ca++; complexes OH-, CO3--, CO2(aq), CaCO3(aq),
  CaHCO3+; kinetic calcite (k 1e-9 mol/m^2/s, area 1 m^2/m^3, volume
  fraction 1e-5).  Totals: Ca and carbonate log-uniform in [1e-5, 1e-2] M,
  pH uniform in [5, 9].
* calcite grid (100^3 cells, dt 1 day): the same network with T uniform in
  [10, 60] C and log K linear in T between the 25 C values and 60 C values
  offset by +-0.3 (seeded), i.e. Maier-Kelly coefficients (0, a, b, 0, 0).
* synthetic 12-species network (2M cells, dt 1 day): 40 aqueous complexes, 6
  kinetic minerals, 4 ion-exchange reactions (CEC 5 meq/100 g) and 2
  surface-complexation reactions, stoichiometry in {-2..2} with ~3 nonzeros,
  log K in [-15, 15], rate constants log-uniform in [1e-12, 1e-6].  Cells
  start at an equilibrium state (forward speciation of seeded free-ion
  molalities whose totals lie in [1e-10, 1e-1] M) and take a seeded
  log-normal "transport update" of their totals, which spreads the Newton
  iteration count over ~2-40.

Everything is generated on the host with numpy from numpy.random.Generator
(PCG64) streams, so a seed fixes the inputs on any machine up to the last
ulp of numpy's exp/log.  The forward speciation here is host-side input
generation; it restates RTotal/RTotalSorb only to build consistent states.
"""
from __future__ import annotations

import numpy as np

from . import abi
from .cells import CellBatch
from .network import ReactionNetwork, default_options

LOG_TO_LN = 2.30258509299  # pflotran_constants.F90:48
# IFC67 liquid density at 25 C and 101325 Pa: the reference_water_density a
# transport-only PFLOTRAN run uses (factory_subsurface.F90:995-1000).
DEN_KG_25C = 997.1604062672549


# ---------------------------------------------------------------------------
# networks

def calcite_network(temperature_dependent=False, seed=0, delta=0.3):
    """Calcite network; with temperature_dependent, log K(T) is linear in T_K
    between 25 C and 60 C with a seeded +-delta offset at 60 C."""
    net = ReactionNetwork([("H+", 1.0, 9.0), ("HCO3-", -1.0, 4.0), ("Ca++", 2.0, 6.0)])
    rng = np.random.default_rng(seed + 7919)

    def coef(logK25):
        if not temperature_dependent:
            return None
        d = delta if rng.random() < 0.5 else -delta
        t1, t2 = 298.15, 333.15
        b = d / (t2 - t1)
        a = logK25 - b * t1
        return (0.0, a, b, 0.0, 0.0)

    # calcite.dat rows (stoichiometry, 25 C log K, a0)
    net.add_complex("OH-", {"H+": -1.0}, 13.9951, a0=3.5, h2o=1.0, logKcoef=coef(13.9951))
    net.add_complex("CO3--", {"H+": -1.0, "HCO3-": 1.0}, 10.3288, a0=4.5, logKcoef=coef(10.3288))
    net.add_complex("CO2(aq)", {"H+": 1.0, "HCO3-": 1.0}, -6.3447, a0=3.0, h2o=-1.0, logKcoef=coef(-6.3447))
    net.add_complex("CaCO3(aq)", {"H+": -1.0, "Ca++": 1.0, "HCO3-": 1.0}, 7.0017, a0=3.0, logKcoef=coef(7.0017))
    net.add_complex("CaHCO3+", {"Ca++": 1.0, "HCO3-": 1.0}, -1.0467, a0=4.0, logKcoef=coef(-1.0467))
    net.add_kinetic_mineral("Calcite", {"H+": -1.0, "Ca++": 1.0, "HCO3-": 1.0}, 1.8487,
                            rate_constant=1e-9, molar_vol=36.934e-6, logKcoef=coef(1.8487))
    net.build()
    return net


def synthetic_network(seed=3, N=12, Nc=40, Nm=6, Nix=4, Nsr=2, porosity=0.25, rho_s=2650.0):
    """Seeded synthetic network with the sizes of the 12-species workload
    (other sizes up to 16 primaries for the kernel-mapping comparison)."""
    rng = np.random.default_rng(seed)
    # charges: >= 4 cations (Z > 0) for ion exchange, the rest in {-2..2}
    Z = np.array([1, 2, 1, 2, 1, -1, -2, -1, 0, 1, -1, 2, 1, -1, 0, 2], dtype=float)[:N]
    rng.shuffle(Z)
    # species 0 plays the part of H+: the only species with negative
    # coefficients (deprotonation reactions), so only its total can be < 0
    Z[[0, int(np.flatnonzero(Z == 1)[0])]] = Z[[int(np.flatnonzero(Z == 1)[0]), 0]]
    a0 = rng.uniform(3.0, 9.0, N)
    names = [f"P{i}" for i in range(N)]
    net = ReactionNetwork([(names[i], Z[i], a0[i]) for i in range(N)])
    lm_ref = np.log(1e-5)

    def draw_rxn(nnz_choices=(2, 3, 3, 4), lo=-14.0, hi=-3.0, force_pos=True, max_charge=None):
        for _ in range(100000):
            nnz = int(rng.choice(nnz_choices))
            sp = rng.choice(N, nnz, replace=False)
            nu = rng.choice([1, 2], nnz, p=[0.65, 0.35]).astype(float)
            if 0 in sp and rng.random() < 0.5:
                nu[list(sp).index(0)] *= -1.0
            if force_pos and nu.max() <= 0:
                continue
            if max_charge is not None and abs(float(nu @ Z[sp])) > max_charge:
                continue  # complexes carry charges in {-2..2}
            logK = rng.uniform(-15.0, 15.0)
            # keep reactions whose species concentration at the reference
            # state (all free ions 1e-5 mol/kg) lies in [10^lo, 10^hi]
            log10C = -logK + nu.sum() * lm_ref / LOG_TO_LN
            if lo <= log10C <= hi:
                return sp, nu, logK
        raise RuntimeError("synthetic_network: no admissible reaction drawn")

    for i in range(Nc):
        sp, nu, logK = draw_rxn(lo=-12.0, hi=-6.0, max_charge=2.0)
        net.add_complex(f"C{i}", {names[s]: v for s, v in zip(sp, nu)}, logK, a0=rng.uniform(3.0, 9.0))
    for m in range(Nm):
        sp, nu, logK = draw_rxn(nnz_choices=(2, 3, 3, 4), lo=-2.0, hi=2.0)
        k = 10.0 ** rng.uniform(-12.0, -6.0)
        net.add_kinetic_mineral(f"M{m}", {names[s]: v for s, v in zip(sp, nu)}, logK,
                                rate_constant=k, molar_vol=30e-6)
    cations = [i for i in range(N) if Z[i] > 0]
    # CEC 5 meq/100 g = 0.05 eq/kg solid -> eq/m^3 bulk (reaction.F90:657-660)
    CEC = 0.05 * rho_s * (1.0 - porosity)
    for r in range(Nix):
        sp = list(rng.choice(cations, 3, replace=False))
        # the reference cation (first) has the smallest charge, as in
        # PFLOTRAN's decks (Na+ reference): KDj^(Z_j/Z_ref) then has
        # exponents >= 1 and the KDj Newton is monotone
        sp.sort(key=lambda s: Z[s])
        ks = [1.0] + list(10.0 ** rng.uniform(-1.0, 1.0, 2))
        net.add_ion_exchange([(names[s], k) for s, k in zip(sp, ks)], CEC)
    for r in range(Nsr):
        cx = []
        for j in range(3):
            while True:
                nnz = int(rng.choice([1, 2]))
                sp = rng.choice(N, nnz, replace=False)
                nu = rng.choice([1, 2], nnz, p=[0.7, 0.3]).astype(float)
                if 0 in sp and rng.random() < 0.5:
                    nu[list(sp).index(0)] *= -1.0
                logK = rng.uniform(-15.0, 15.0)
                # surface complex / free site ratio at the reference state in [1e-3, 1e1]
                lr = -logK + nu.sum() * lm_ref / LOG_TO_LN
                if -3.0 <= lr <= 1.0:
                    break
            cx.append(({names[s]: v for s, v in zip(sp, nu)}, 1.0, logK))
        stype = abi.ROCK_SURFACE if r == 0 else abi.NULL_SURFACE
        dens = 1e-3 if stype == abi.ROCK_SURFACE else 1.0  # mol/kg solid (rock) / mol/m^3 (null)
        net.add_surface_complexation(dens, cx, surf_type=stype)
    net.build()
    return net


def add_rate_prefactors(net):
    """Gives the first two kinetic minerals of `net` rate prefactors
    (reaction_mineral.F90:743-782), in place, and rebuilds its tables:
    mineral 0 a Monod term in the first primary (alpha 1, beta 1,
    attenuation 1e4) plus a second parallel prefactor in the first aqueous
    complex (alpha 0.5, beta 1, attenuation 10) and the third primary
    (alpha 1, no attenuation) with its own activation energy; mineral 1 one
    prefactor in the second primary (alpha 0.5, beta 0.5, attenuation 100).
    Returns net."""
    pn = net.pri_names
    cx = net.complexes[0].extra["name"]
    m0, m1 = net.minerals[0], net.minerals[min(1, len(net.minerals) - 1)]
    k0, k1 = m0.extra["k"], m1.extra["k"]
    m0.extra["pref"] = [dict(rate=10.0 * k0, species=[(pn[0], 1.0, 1.0, 1e4)]),
                        dict(rate=k0, Ea=3e4, species=[(cx, 0.5, 1.0, 10.0), (pn[2 % len(pn)], 1.0, 0.0, 0.0)])]
    if m1 is not m0:
        m1.extra["pref"] = [dict(rate=k1, species=[(pn[1 % len(pn)], 0.5, 0.5, 100.0)])]
    net._tables = None
    net.build()
    return net


def add_passive_gases(net, seed=0):
    """Passive gases for GAS constraint rows (reaction.F90:1720-1751), in
    place: CO2(g) = H+ + HCO3- - H2O (log K -7.8136 at 25 C) when the network
    has those primaries, else two seeded gases, each the product of two or
    three primaries with log K in [0, 5].
    log K(T) is linear in T_K with a seeded +-0.3 offset at 60 C.  Returns net."""
    rng = np.random.default_rng(seed + 104729)

    def coef(lk):
        d = 0.3 if rng.random() < 0.5 else -0.3
        b = d / (333.15 - 298.15)
        return (0.0, lk - b * 298.15, b, 0.0, 0.0)

    if "H+" in net.pri_names and "HCO3-" in net.pri_names:
        net.add_passive_gas("CO2(g)", {"H+": 1.0, "HCO3-": 1.0}, -7.8136, logKcoef=coef(-7.8136), h2o=-1.0)
    else:
        pn = net.pri_names
        for g in range(2):
            k = 2 + g
            ids = rng.choice(len(pn), size=min(k, len(pn)), replace=False)
            st = {pn[i]: 1.0 for i in ids}  # partial pressures below 1 bar (activities < 1)
            lk = float(rng.uniform(0.0, 5.0))
            net.add_passive_gas(f"G{g + 1}(g)", st, lk, logKcoef=coef(lk))
    return net


# ---------------------------------------------------------------------------
# forward speciation for input generation (torch, float64, CPU or CUDA)

class Speciator:
    """Vectorised RTotal / RTotalSorb at given free-ion molalities, used to
    build consistent cell states.  Works on torch float64 tensors on any
    device (a CUDA device generates millions of cells in seconds)."""

    def __init__(self, net: ReactionNetwork, device="cpu"):
        import torch
        self.torch = torch
        self.dev = torch.device(device)
        self.net = net
        t = net._tables if net._tables is not None else net.build()
        self.t = t
        N, Nc = net.N, net.Nc
        nu = np.zeros((Nc, N))
        ld = t["eqcplx_ld"]
        ids = t["eqcplxspecid"].reshape(-1, ld + 1)
        st = t["eqcplxstoich"].reshape(-1, ld)
        for i in range(Nc):
            for k in range(ids[i, 0]):
                nu[i, ids[i, k + 1] - 1] = st[i, k]
        self.nu_np = nu
        T = lambda a: torch.as_tensor(np.asarray(a, dtype=np.float64), device=self.dev)
        self.nu = T(nu)
        self.Zp, self.Zc = T(t["primary_spec_Z"]), T(t["eqcplx_Z"][:Nc])
        self.ap, self.ac = T(t["primary_spec_a0"]), T(t["eqcplx_a0"][:Nc])
        self.coef = T(t["eqcplx_logKcoef"].reshape(-1, 5)[:Nc])
        self.logK = T(t["eqcplx_logK"][:Nc])
        self.T = T

    def logK_at(self, temp, isothermal):
        if isothermal:
            return self.logK.expand(len(temp), -1)
        tk = (temp + 273.15)[:, None]
        c = self.coef
        return c[:, 0] * self.torch.log(tk) + c[:, 1] + c[:, 2] * tk + c[:, 3] / tk + c[:, 4] / (tk * tk)

    def ln_gamma(self, I):
        """LAG activity coefficients (reaction.F90:3992-4051) as ln gamma."""
        torch = self.torch
        A, B, Bd = self.net.debye
        s = torch.sqrt(I)[:, None]
        lp = (-self.Zp ** 2 * s * A / (1.0 + self.ap * B * s) + Bd * I[:, None]) * LOG_TO_LN
        lc = (-self.Zc ** 2 * s * A / (1.0 + self.ac * B * s) + Bd * I[:, None]) * LOG_TO_LN
        lp = torch.where(self.Zp.abs() > 1e-10, lp, torch.zeros_like(lp))
        lc = torch.where(self.Zc.abs() > 1e-10, lc, torch.zeros_like(lc))
        return lp, lc

    def aqueous(self, lnm, logK, lngp, lngc):
        """molal totals Psi (n,N), complexes C (n,Nc)."""
        ln_act = lnm + lngp
        lnQK = -logK * LOG_TO_LN + ln_act @ self.nu.T
        Cc = self.torch.exp(lnQK - lngc)
        Psi = self.torch.exp(lnm) + Cc @ self.nu
        return Psi, Cc

    def ionic_strength(self, lnm, Cc):
        return 0.5 * (self.torch.exp(lnm) @ (self.Zp ** 2) + Cc @ (self.Zc ** 2))

    def sorbed(self, m, gp, mnrl_volfrac, porosity, rho_s, ref_sorbed0=1e-9):
        """Equilibrium sorbed totals (mol/m^3 bulk) and the sorption warm
        starts, following RTotalSorbEqIonx (reaction.F90:4305-4535) and
        RTotalSorbEqSurfCplx1 (reaction_surf_complex.F90:658-934) for unit
        free-site stoichiometry."""
        torch = self.torch
        net, t = self.net, self.t
        n, N = m.shape
        S = torch.zeros((n, N), dtype=torch.float64, device=self.dev)
        ref_out = torch.zeros((n, max(net.Nix, 1)), dtype=torch.float64, device=self.dev)
        a = m * gp
        ldx = t["eqionx_ld"]
        xid = t["eqionx_rxn_cationid"].reshape(-1, ldx + 1)
        xk = t["eqionx_rxn_k"].reshape(-1, ldx)
        Zp = t["primary_spec_Z"]
        for r in range(net.Nix):
            nc = int(xid[r, 0])
            ids = [int(x) - 1 for x in xid[r, 1:nc + 1]]
            ks = [float(x) for x in xk[r, :nc]]
            Zs = [float(Zp[i]) for i in ids]
            to = int(t["eqionx_rxn_to_surf"][r])
            omega = float(t["eqionx_rxn_CEC"][r])
            omega = omega * torch.clamp(mnrl_volfrac[:, to - 1], min=1e-40) if to > 0 else \
                torch.full((n,), omega, dtype=torch.float64, device=self.dev)
            if t["eqionx_rxn_Z_flag"][r]:
                ref = ks[0] * a[:, ids[0]]
                KD = (Zs[0] * ref_sorbed0 / omega) / ref
                for _ in range(200):
                    tot = KD * ref
                    d = ref.clone()
                    for j in range(1, nc):
                        x = ks[j] * a[:, ids[j]] * KD ** (Zs[j] / Zs[0])
                        tot = tot + x
                        d = d + x / KD * Zs[j] / Zs[0]
                    step = (1.0 - tot) / d
                    KD = torch.clamp(KD + step, min=1e-40)
                    if bool(torch.all((step / KD).abs() < 1e-13)):
                        break
                X = [KD * ref] + [ks[j] * a[:, ids[j]] * KD ** (Zs[j] / Zs[0]) for j in range(1, nc)]
                ref_out[:, r] = X[0] * omega / Zs[0]
            else:
                X = [ks[j] * a[:, ids[j]] for j in range(nc)]
                ssum = sum(X)
                X = [x / ssum for x in X]
                ref_out[:, r] = ref_sorbed0
            for j in range(nc):
                S[:, ids[j]] += X[j] * omega / Zs[j]
        free_out = torch.zeros((n, max(net.Nsr, 1)), dtype=torch.float64, device=self.dev)
        ldr, lds = t["srfcplxrxn_ld"], t["srfcplx_ld"]
        r2c = t["srfcplxrxn_to_complex"].reshape(-1, ldr + 1)
        sid = t["srfcplxspecid"].reshape(-1, lds + 1)
        sst = t["srfcplxstoich"].reshape(-1, lds)
        lnact = torch.log(a)
        for r in range(net.Nsr):
            stype = int(t["srfcplxrxn_surf_type"][r])
            dens = float(t["srfcplxrxn_site_density"][r])
            if stype == abi.ROCK_SURFACE:
                site = dens * rho_s * (1.0 - porosity)
            elif stype == abi.MINERAL_SURFACE:
                site = dens * mnrl_volfrac[:, int(t["srfcplxrxn_to_surf"][r]) - 1]
            else:
                site = dens
            terms = []
            for j in range(int(r2c[r, 0])):
                ic = int(r2c[r, j + 1]) - 1
                lq = -float(t["srfcplx_logK"][ic]) * LOG_TO_LN
                for k in range(int(sid[ic, 0])):
                    lq = lq + float(sst[ic, k]) * lnact[:, int(sid[ic, k + 1]) - 1]
                terms.append((ic, lq))
            ratio = sum(torch.exp(lq) for _, lq in terms)
            free = site / (1.0 + ratio)
            free_out[:, r] = free
            for ic, lq in terms:
                Sc = torch.exp(lq) * free
                for k in range(int(sid[ic, 0])):
                    S[:, int(sid[ic, k + 1]) - 1] += float(sst[ic, k]) * Sc
        return S, ref_out[:, :net.Nix], free_out[:, :net.Nsr]


def _fill_common(b, n, porosity=0.25, sat=1.0, volume=1.0, den=DEN_KG_25C, rho_s=2650.0):
    b.saturation[:] = sat
    b.porosity[:] = porosity
    b.volume[:] = volume
    b.den_kg[:] = den
    b.soil_particle_density[:] = rho_s


def _np(x):
    return x.detach().cpu().numpy()


def calcite_cells(n=100, seed=0, temperature_dependent=False, net=None, device="cpu"):
    """Calcite column (25 C) or, with temperature_dependent, the calcite grid
    workload with T ~ U[10, 60] C.  Returns (net, opt, cells, dt)."""
    import torch
    rng = np.random.default_rng(seed)
    if net is None:
        net = calcite_network(temperature_dependent=temperature_dependent, seed=seed)
    opt = default_options(use_isothermal=0 if temperature_dependent else 1)
    sp = Speciator(net, device)
    b = CellBatch.allocate(net, n)
    _fill_common(b, n)
    T = rng.uniform(10.0, 60.0, n) if temperature_dependent else np.full(n, 25.0)
    b.temperature[:] = T
    tCa = sp.T(10.0 ** rng.uniform(-5.0, -2.0, n))
    tC = sp.T(10.0 ** rng.uniform(-5.0, -2.0, n))
    pH = sp.T(rng.uniform(5.0, 9.0, n))
    den_L = sp.T(b.den_kg * 1e-3)
    logK = sp.logK_at(sp.T(T), opt.use_isothermal)
    # constraint speciation: pH row for H+, TOTAL rows for HCO3- and Ca++
    lnm = torch.stack([-pH * LOG_TO_LN, torch.log(tC / den_L), torch.log(tCa / den_L)], dim=1)
    I = torch.full((n,), 1e-3, dtype=torch.float64, device=sp.dev)
    eye = torch.eye(3, dtype=torch.float64, device=sp.dev)
    for outer in range(30):
        lngp, lngc = sp.ln_gamma(I)
        lnm[:, 0] = -pH * LOG_TO_LN - lngp[:, 0]
        for it in range(60):
            Psi, Cc = sp.aqueous(lnm, logK, lngp, lngc)
            F = Psi[:, 1:] * den_L[:, None] - torch.stack([tC, tCa], 1)
            # d Psi_j / d ln m_k = m_j delta_jk + sum_i nu_ij nu_ik C_i
            Jf = torch.einsum("ij,ik,ni->njk", sp.nu, sp.nu, Cc) + torch.einsum("jk,nj->njk", eye, torch.exp(lnm))
            J = Jf[:, 1:, 1:] * den_L[:, None, None]
            d = torch.linalg.solve(J, F[..., None])[..., 0]
            d = torch.clamp(d, -2.0, 2.0)
            lnm[:, 1:] -= d
            if float(d.abs().max()) < 1e-14:
                break
        Inew = sp.ionic_strength(lnm, Cc)
        if float(((Inew - I).abs() / Inew).max()) < 1e-15:
            I = Inew
            break
        I = Inew
    lngp, lngc = sp.ln_gamma(I)
    Psi, Cc = sp.aqueous(lnm, logK, lngp, lngc)
    b.view("total", net.N)[:] = _np((Psi * den_L[:, None]).T)
    b.view("pri_molal", net.N)[:] = _np(torch.exp(lnm).T)
    b.ionic_strength[:] = _np(sp.ionic_strength(lnm, Cc))
    b.mnrl_volfrac[:] = 1e-5
    b.mnrl_area[:] = 1.0
    dt = 86400.0 if temperature_dependent else 3600.0
    return net, opt, b, dt


def _forward_state(sp, lnm, iters=12, tol=None):
    """Totals (mol/L), complexes and the self-consistent ionic strength at
    free ions exp(lnm)."""
    torch = sp.torch
    n = lnm.shape[0]
    I = torch.full((n,), 1e-3, dtype=torch.float64, device=sp.dev)
    for _ in range(iters):
        lngp, lngc = sp.ln_gamma(torch.clamp(I, 0.0, 10.0))
        Psi, Cc = sp.aqueous(lnm, sp.logK, lngp, lngc)
        Inew = sp.ionic_strength(lnm, Cc)
        done = tol is not None and bool(torch.all(((Inew - I).abs() <= tol * Inew) | ~torch.isfinite(Inew)))
        I = Inew
        if done:
            break
    return Psi * DEN_KG_25C * 1e-3, Cc, I, lngp


def synthetic_cells(n, seed=5, net=None, sigma_range=(1e-2, 2.0), tot_range=(1e-10, 1e-1), device="cpu"):
    """Cells of the synthetic 12-species workload.  Returns (net, opt, cells, dt).

    Each cell starts from an equilibrium state (free ions drawn log-uniform in
    [1e-7, 3e-4] mol/kg) and receives the totals of a perturbed state, free
    ions scaled by exp(sigma * xi) with xi ~ N(0, 1) per species and sigma
    log-uniform in `sigma_range`: the "transport update".  Both states must
    have all |totals| in `tot_range` (only the H+-like species 0 may have a
    negative total).  The previous-step guess is the equilibrium state.
    Random numbers come from a torch.Generator seeded with `seed` on `device`."""
    import torch
    if net is None:
        net = synthetic_network()
    opt = default_options(use_isothermal=1)
    sp = Speciator(net, device)
    g = torch.Generator(device=sp.dev)
    g.manual_seed(seed)
    N = net.N
    porosity, rho_s = 0.25, 2650.0
    lo, hi = tot_range
    keep_eq, keep_new = [], []
    have = 0
    rounds = 0
    l1, l2 = float(np.log(1e-7)), float(np.log(3e-4))
    s1, s2 = float(np.log10(sigma_range[0])), float(np.log10(sigma_range[1]))
    while have < n:
        rounds += 1
        if rounds > 100:
            raise RuntimeError("synthetic_cells: acceptance too low")
        k = max(2 * (n - have), 4096)
        u = torch.rand((k, N), generator=g, dtype=torch.float64, device=sp.dev)
        lnm = l1 + (l2 - l1) * u
        sig = 10.0 ** (s1 + (s2 - s1) * torch.rand((k,), generator=g, dtype=torch.float64, device=sp.dev))
        xi = torch.randn((k, N), generator=g, dtype=torch.float64, device=sp.dev)
        lnm2 = lnm + sig[:, None] * xi
        t1, _, I1, _ = _forward_state(sp, lnm, iters=6)
        t2, _, I2, _ = _forward_state(sp, lnm2, iters=6)
        a1, a2 = t1.abs(), t2.abs()
        ok = (torch.all((a1 >= lo) & (a1 <= hi), dim=1) & torch.all((a2 >= lo) & (a2 <= hi), dim=1)
              & torch.all(t1[:, 1:] > 0, dim=1) & torch.all(t2[:, 1:] > 0, dim=1) & (I1 < 1.0) & (I2 < 1.0))
        keep_eq.append(lnm[ok])
        keep_new.append(lnm2[ok])
        have += int(ok.sum())
    lnm = torch.cat(keep_eq)[:n]
    lnm2 = torch.cat(keep_new)[:n]
    b = CellBatch.allocate(net, n)
    _fill_common(b, n, porosity=porosity, rho_s=rho_s)
    b.temperature[:] = 25.0
    tot_eq, Cc, I, lngp = _forward_state(sp, lnm, iters=100, tol=1e-15)
    tot_new, _, _, _ = _forward_state(sp, lnm2, iters=100, tol=1e-15)
    m = torch.exp(lnm)
    vf = torch.full((n, max(net.Nm, 1)), 1e-3, dtype=torch.float64, device=sp.dev)
    S, ref, free = sp.sorbed(m, torch.exp(lngp), vf, porosity, rho_s)
    b.view("total", N)[:] = _np(tot_new.T)
    b.view("pri_molal", N)[:] = _np(m.T)
    b.ionic_strength[:] = _np(I)
    b.mnrl_volfrac[:] = 1e-3
    b.mnrl_area[:] = 1.0
    if net.Nix + net.Nsr > 0:
        b.view("total_sorb_eq", N)[:] = _np(S.T)
    if net.Nix > 0:
        b.view("eqionx_ref_cation_sorbed_conc", net.Nix)[:] = _np(ref.T)
    if net.Nsr > 0:
        b.view("srfcplxrxn_free_site_conc", net.Nsr)[:] = _np(free.T)
    return net, opt, b, 86400.0
