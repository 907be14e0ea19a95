// pfchem_oracle.cpp -- CPU oracle for the batched per-cell geochemistry step.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, routine by routine, the
// Fortran that PFLOTRAN runs for one operator-split reaction step of one
// cell.  It is the checker for the GPU library and the timed CPU baseline;
// the library never calls it.  Only tests/, __graft_entry__.smoke() and
// bench.py (cpu_baseline leg and --impl reference) load it.
//
// Every function cites the reference lines it follows (paths relative to the
// PFLOTRAN source tree).  Arithmetic follows the reference's operation order
// so that the `double` instantiation is the parity reference; the `long
// double` instantiation is the higher-precision truth used for error
// statements.  The boundary differences are explicit and listed here:
//   * log K at the cell temperature is computed into a per-cell copy instead
//     of mutating shared tables (reaction.F90:5433-5524 is not thread safe);
//   * the ionic strength that the first activity-coefficient evaluation of a
//     step uses comes from the state field `ionic_strength` (the value at the
//     previous solution) instead of being recomputed from the entry
//     pri_molal/sec_molal (reaction.F90:3407-3409 -> :3992-4004).  Both agree
//     when the guess is the previous solution, which is RTReact's usage;
//   * loops without a cap in the reference (RReact's Newton, surface
//     complexation's free-site Newton) are capped and report a status.
//
// Pinned by known-answer tests against PFLOTRAN's own regression gold files
// (regression_tests/ascem/batch/*.regression.gold) in tests/test_oracle_kat.py.

#include "../include/pfchem.h"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

namespace {

// pflotran_constants.F90:48,53 (LOG_TO_LN is the reference's truncated value)
constexpr double kLOG_TO_LN = 2.30258509299;
constexpr double kIDEAL_GAS_CONSTANT = 8.31446;

constexpr int P = PFCHEM_MAX_PRI;
constexpr int C = PFCHEM_MAX_CPLX;
constexpr int M = PFCHEM_MAX_MNRL;
constexpr int IX = PFCHEM_MAX_IONX;
constexpr int SR = PFCHEM_MAX_SRFRXN;
constexpr int SC = PFCHEM_MAX_SRFCPLX;
constexpr int NZ = PFCHEM_MAX_NNZ;

// Thread-safe view of pfchem_network with 0-based helpers.
struct Net {
  const pfchem_network *n;
  int N, Nc, Nm, Nix, Nsr, Nsc;
  bool exact_jac = false;  // PFCHEM_JACOBIAN_EXACT
  int id(const int32_t *t, int ld, int k, int r) const { return t[(ld + 1) * r + k]; }
  double st(const double *t, int ld, int k, int r) const { return t[ld * (r) + (k - 1)]; }
  // aqueous complex icplx (0-based): count and 0-based species ids
  int cn(int i) const { return id(n->eqcplxspecid, n->eqcplx_ld, 0, i); }
  int cid(int i, int k) const { return id(n->eqcplxspecid, n->eqcplx_ld, k, i) - 1; }
  double cnu(int i, int k) const { return st(n->eqcplxstoich, n->eqcplx_ld, k, i); }
  int mn(int i) const { return id(n->kinmnrlspecid, n->kinmnrl_ld, 0, i); }
  int mid(int i, int k) const { return id(n->kinmnrlspecid, n->kinmnrl_ld, k, i) - 1; }
  double mnu(int i, int k) const { return st(n->kinmnrlstoich, n->kinmnrl_ld, k, i); }
  int xn(int r) const { return id(n->eqionx_rxn_cationid, n->eqionx_ld, 0, r); }
  int xid(int r, int k) const { return id(n->eqionx_rxn_cationid, n->eqionx_ld, k, r) - 1; }
  double xk(int r, int k) const { return st(n->eqionx_rxn_k, n->eqionx_ld, k, r); }
  int srn(int r) const { return id(n->srfcplxrxn_to_complex, n->srfcplxrxn_ld, 0, r); }
  int src(int r, int k) const { return id(n->srfcplxrxn_to_complex, n->srfcplxrxn_ld, k, r) - 1; }
  int sn(int i) const { return id(n->srfcplxspecid, n->srfcplx_ld, 0, i); }
  int sid(int i, int k) const { return id(n->srfcplxspecid, n->srfcplx_ld, k, i) - 1; }
  double snu(int i, int k) const { return st(n->srfcplxstoich, n->srfcplx_ld, k, i); }
};

// Per-cell state: the reactive_transport_auxvar_type fields RReact touches
// (reactive_transport_aux.F90:18-66), global_auxvar (temp, sat, den_kg) and
// material_auxvar (volume, porosity, soil_particle_density).
template <class R>
struct Cell {
  R pri_molal[P], pri_act_coef[P], sec_molal[C], sec_act_coef[C];
  R total[P], dtotal[P][P];
  R total_sorb_eq[P], dtotal_sorb_eq[P][P];
  R eqionx_ref_cation_sorbed_conc[IX], eqionx_conc[NZ][IX];
  R srfcplxrxn_free_site_conc[SR], eqsrfcplx_conc[SC];
  R mnrl_volfrac[M], mnrl_area[M], mnrl_rate[M];
  R ln_act_h2o;
  R temp, sat, den_kg, volume, porosity, soil_particle_density;
  // per-cell copies of the temperature-dependent tables
  R eqcplx_logK[C], kinmnrl_logK[M], srfcplx_logK[SC];
  int inner_fail;
};

template <class R> R rlog(R x) { return std::log(x); }
template <class R> R rexp(R x) { return std::exp(x); }

// ---------------------------------------------------------------------------
// reaction_aux.F90:1461-1488 ReactionInterpolateLogK (Maier-Kelly form)
template <class R>
R interpolate_logK(const double *coef, R temp) {
  R tk = temp + R(273.15);
  return R(coef[0]) * rlog(tk) + R(coef[1]) + R(coef[2]) * tk + R(coef[3]) / tk +
         R(coef[4]) / (tk * tk);
}

// reaction.F90:5433-5524 RUpdateTempDependentCoefs (non-hpt branch) and
// reaction_mineral.F90:1227-1278 MineralUpdateTempDepCoefs, into the cell copy.
template <class R>
void update_temp_dependent_coefs(const Net &w, const pfchem_options &o, Cell<R> &c) {
  const pfchem_network &n = *w.n;
  for (int i = 0; i < w.Nc; ++i)
    c.eqcplx_logK[i] = o.use_isothermal ? R(n.eqcplx_logK[i])
                                        : interpolate_logK(n.eqcplx_logKcoef + 5 * i, c.temp);
  for (int i = 0; i < w.Nm; ++i)
    c.kinmnrl_logK[i] = o.use_isothermal ? R(n.kinmnrl_logK[i])
                                         : interpolate_logK(n.kinmnrl_logKcoef + 5 * i, c.temp);
  for (int i = 0; i < w.Nsc; ++i)
    c.srfcplx_logK[i] = o.use_isothermal ? R(n.srfcplx_logK[i])
                                         : interpolate_logK(n.srfcplx_logKcoef + 5 * i, c.temp);
}

// ---------------------------------------------------------------------------
// reaction.F90:3812-4053 RActivityCoefficients.  `I_start` replaces the
// ionic strength computed from the entry state for the first evaluation of a
// step (see header).  Returns 0, or 1 when the NEWTON algorithm exceeds 50
// iterations (the reference sets NaNs there, reaction.F90:3864-3875).
template <class R>
int activity_coefficients(const Net &w, const pfchem_options &o, Cell<R> &c, bool use_I_start,
                          R I_start) {
  const pfchem_network &n = *w.n;
  const int N = w.N, Nc = w.Nc;
  R sum_pri_molal = 0, sum_sec_molal = 0;
  if (o.use_activity_h2o) {
    for (int j = 0; j < N; ++j) sum_pri_molal += c.pri_molal[j];
  }
  const R A = n.debyeA, B = n.debyeB, Bdot = n.debyeBdot;
  if (o.act_coef_update_algorithm == PFCHEM_ACT_COEF_ALGORITHM_NEWTON) {
    if (use_I_start) {
      // The step's entry state at the library's boundary, which carries the
      // ionic strength rather than the activity coefficients: the primaries'
      // coefficients at that ionic strength and no complexes yet (the first
      // pass of the loop below then keeps I = I_start exactly).
      const R sI = std::sqrt(I_start);
      for (int j = 0; j < N; ++j) {
        const R z = n.primary_spec_Z[j];
        c.pri_act_coef[j] = std::fabs(z) > 0 ? rexp((-z * z * sI * A / (R(1) + R(n.primary_spec_a0[j]) * B * sI) +
                                                      Bdot * I_start) * R(kLOG_TO_LN))
                                             : R(1);
      }
      for (int i = 0; i < Nc; ++i) c.sec_molal[i] = 0;
    }
    R ln_conc[P], ln_act[P];
    for (int j = 0; j < N; ++j) {
      ln_conc[j] = rlog(c.pri_molal[j]);
      ln_act[j] = ln_conc[j] + rlog(c.pri_act_coef[j]);
    }
    R fpri = 0;
    for (int j = 0; j < N; ++j)
      fpri = fpri + c.pri_molal[j] * R(n.primary_spec_Z[j]) * R(n.primary_spec_Z[j]);
    int it = 0;
    R II = 0, I = 0;
    for (;;) {
      ++it;
      if (it > 50) return 1;
      if (it == 1 && use_I_start) {
        I = I_start;
      } else {
        I = fpri;
        for (int i = 0; i < Nc; ++i) I = I + c.sec_molal[i] * R(n.eqcplx_Z[i]) * R(n.eqcplx_Z[i]);
        I = R(0.5) * I;
      }
      R f = I;
      if (std::fabs(I - II) < R(1e-6) * I) break;
      if (Nc > 0) {
        R didi = 0;
        R sqrt_I = std::sqrt(I);
        for (int i = 0; i < Nc; ++i) {
          R zi = n.eqcplx_Z[i];
          if (std::fabs(zi) > 0) {
            R a0 = n.eqcplx_a0[i];
            R t = R(1) + B * a0 * sqrt_I;
            R sum = R(0.5) * A * zi * zi / (sqrt_I * t * t) - Bdot;
            for (int k = 1; k <= w.cn(i); ++k) {
              int j = w.cid(i, k);
              R zj = n.primary_spec_Z[j];
              if (std::fabs(zj) > 0) {
                R tj = R(1) + B * R(n.primary_spec_a0[j]) * sqrt_I;
                R dgamdi = R(-0.5) * A * zj * zj / (sqrt_I * tj * tj) + Bdot;
                sum = sum + R(w.cnu(i, k)) * dgamdi;
              }
            }
            R dcdi = c.sec_molal[i] * R(kLOG_TO_LN) * sum;
            didi = didi + R(0.5) * zi * zi * dcdi;
          }
        }
        R den = R(1) - didi;
        II = (std::fabs(den) > 0) ? (f - I * didi) / den : f;
      } else {
        II = f;
      }
      I = II;
      R sqrt_I = std::sqrt(I);
      for (int j = 0; j < N; ++j) {
        R z = n.primary_spec_Z[j];
        c.pri_act_coef[j] =
            std::fabs(z) > 0
                ? rexp((-z * z * sqrt_I * A / (R(1) + R(n.primary_spec_a0[j]) * B * sqrt_I) + Bdot * I) *
                       R(kLOG_TO_LN))
                : R(1);
      }
      sum_sec_molal = 0;
      for (int i = 0; i < Nc; ++i) {
        R z = n.eqcplx_Z[i];
        c.sec_act_coef[i] =
            std::fabs(z) > 0
                ? rexp((-z * z * sqrt_I * A / (R(1) + R(n.eqcplx_a0[i]) * B * sqrt_I) + Bdot * I) *
                       R(kLOG_TO_LN))
                : R(1);
        R lnQK = -c.eqcplx_logK[i] * R(kLOG_TO_LN);
        if (n.eqcplxh2oid && n.eqcplxh2oid[i] > 0) lnQK = lnQK + R(n.eqcplxh2ostoich[i]) * c.ln_act_h2o;
        for (int k = 1; k <= w.cn(i); ++k) lnQK = lnQK + R(w.cnu(i, k)) * ln_act[w.cid(i, k)];
        c.sec_molal[i] = rexp(lnQK) / c.sec_act_coef[i];
        sum_sec_molal = sum_sec_molal + c.sec_molal[i];
      }
      if (o.use_activity_h2o) {
        R v = R(1) - R(0.017) * (sum_pri_molal + sum_sec_molal);
        c.ln_act_h2o = v > 0 ? rlog(v) : R(0);
      }
    }
    return 0;
  }
  // ACT_COEF_ALGORITHM_LAG (reaction.F90:3992-4051)
  R I;
  if (use_I_start) {
    I = I_start;
  } else {
    I = 0;
    for (int j = 0; j < N; ++j) I = I + c.pri_molal[j] * R(n.primary_spec_Z[j]) * R(n.primary_spec_Z[j]);
    for (int i = 0; i < Nc; ++i) I = I + c.sec_molal[i] * R(n.eqcplx_Z[i]) * R(n.eqcplx_Z[i]);
    I = R(0.5) * I;
  }
  R sqrt_I = std::sqrt(I);
  for (int j = 0; j < N; ++j) {
    R z = n.primary_spec_Z[j];
    c.pri_act_coef[j] =
        std::fabs(z) > R(1e-10)
            ? rexp((-z * z * sqrt_I * A / (R(1) + R(n.primary_spec_a0[j]) * B * sqrt_I) + Bdot * I) *
                   R(kLOG_TO_LN))
            : R(1);
  }
  for (int i = 0; i < Nc; ++i) {
    R z = n.eqcplx_Z[i];
    c.sec_act_coef[i] =
        std::fabs(z) > R(1e-10)
            ? rexp((-z * z * sqrt_I * A / (R(1) + R(n.eqcplx_a0[i]) * B * sqrt_I) + Bdot * I) *
                   R(kLOG_TO_LN))
            : R(1);
    sum_sec_molal = sum_sec_molal + c.sec_molal[i];
  }
  // With the ionic strength taken from the state, ln a_H2O is the state's
  // value too: both were computed at the previous solution.
  if (o.use_activity_h2o && !use_I_start) {
    R v = R(1) - R(0.017) * (sum_pri_molal + sum_sec_molal);
    c.ln_act_h2o = v > 0 ? rlog(v) : R(0);
  }
  return 0;
}

// ---------------------------------------------------------------------------
// reaction.F90:4057-4158 RTotal (aqueous phase; no CO2 modes)
template <class R>
void rtotal(const Net &w, Cell<R> &c) {
  const pfchem_network &n = *w.n;
  const int N = w.N;
  R den_kg_per_L = c.den_kg * R(1e-3);  // xmass = 1
  R ln_conc[P], ln_act[P];
  for (int j = 0; j < N; ++j) {
    ln_conc[j] = rlog(c.pri_molal[j]);
    ln_act[j] = ln_conc[j] + rlog(c.pri_act_coef[j]);
    c.total[j] = c.pri_molal[j];
  }
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) c.dtotal[i][j] = (i == j) ? R(1) : R(0);
  for (int i = 0; i < w.Nc; ++i) {
    R lnQK = -c.eqcplx_logK[i] * R(kLOG_TO_LN);
    if (n.eqcplxh2oid && n.eqcplxh2oid[i] > 0) lnQK = lnQK + R(n.eqcplxh2ostoich[i]) * c.ln_act_h2o;
    const int nc = w.cn(i);
    for (int k = 1; k <= nc; ++k) lnQK = lnQK + R(w.cnu(i, k)) * ln_act[w.cid(i, k)];
    c.sec_molal[i] = rexp(lnQK) / c.sec_act_coef[i];
    for (int k = 1; k <= nc; ++k) {
      int ic = w.cid(i, k);
      c.total[ic] = c.total[ic] + R(w.cnu(i, k)) * c.sec_molal[i];
    }
    for (int kj = 1; kj <= nc; ++kj) {
      int jc = w.cid(i, kj);
      R tempreal = R(w.cnu(i, kj)) * rexp(lnQK - ln_conc[jc]) / c.sec_act_coef[i];
      for (int ki = 1; ki <= nc; ++ki) {
        int ic = w.cid(i, ki);
        c.dtotal[ic][jc] = c.dtotal[ic][jc] + R(w.cnu(i, ki)) * tempreal;
      }
    }
  }
  for (int j = 0; j < N; ++j) c.total[j] = c.total[j] * den_kg_per_L;
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) c.dtotal[i][j] = c.dtotal[i][j] * den_kg_per_L;
}

// ---------------------------------------------------------------------------
// reaction_surf_complex.F90:658-934 RTotalSorbEqSurfCplx1 (immobile sites:
// MINERAL, ROCK and NULL surfaces; colloids are rejected at set-up).
template <class R>
int total_sorb_eq_surfcplx1(const Net &w, Cell<R> &c, int irxn) {
  const pfchem_network &n = *w.n;
  const int N = w.N;
  R ln_conc[P], ln_act[P];
  for (int j = 0; j < N; ++j) {
    ln_conc[j] = rlog(c.pri_molal[j]);
    ln_act[j] = ln_conc[j] + rlog(c.pri_act_coef[j]);
  }
  const int ncplx = w.srn(irxn);
  R free_site_conc = c.srfcplxrxn_free_site_conc[irxn];
  R srfcplx_conc[SC];
  for (int i = 0; i < w.Nsc; ++i) srfcplx_conc[i] = 0;
  R site_density;
  switch (n.srfcplxrxn_surf_type[irxn]) {
    case PFCHEM_MINERAL_SURFACE:
      site_density = R(n.srfcplxrxn_site_density[irxn]) * c.mnrl_volfrac[n.srfcplxrxn_to_surf[irxn] - 1];
      break;
    case PFCHEM_ROCK_SURFACE:
      site_density = R(n.srfcplxrxn_site_density[irxn]) * c.soil_particle_density * (R(1) - c.porosity);
      break;
    default:
      site_density = R(n.srfcplxrxn_site_density[irxn]);
      break;
  }
  if (site_density < R(1e-40)) return 0;
  bool one_more = false;
  int num_iterations = 0;
  R damping_factor = 1;
  for (;;) {
    ++num_iterations;
    if (num_iterations > 2000) return 1;  // capped; the reference damps after 1000 and loops on
    R total = free_site_conc;
    R ln_free_site = rlog(free_site_conc);
    for (int j = 1; j <= ncplx; ++j) {
      int ic = w.src(irxn, j);
      R lnQK = -c.srfcplx_logK[ic] * R(kLOG_TO_LN);
      if (n.srfcplxh2oid && n.srfcplxh2oid[ic] > 0) lnQK = lnQK + R(n.srfcplxh2ostoich[ic]) * c.ln_act_h2o;
      lnQK = lnQK + R(n.srfcplx_free_site_stoich[ic]) * ln_free_site;
      for (int k = 1; k <= w.sn(ic); ++k) lnQK = lnQK + R(w.snu(ic, k)) * ln_act[w.sid(ic, k)];
      srfcplx_conc[ic] = rexp(lnQK);
      total = total + R(n.srfcplx_free_site_stoich[ic]) * srfcplx_conc[ic];
    }
    if (one_more) break;
    if (n.srfcplxrxn_stoich_flag[irxn]) {
      R res = site_density - total;
      R dres_dfree_site = 1;
      for (int j = 1; j <= ncplx; ++j) {
        int ic = w.src(irxn, j);
        dres_dfree_site = dres_dfree_site + R(n.srfcplx_free_site_stoich[ic]) * srfcplx_conc[ic] / free_site_conc;
      }
      R dfree_site_conc = res / dres_dfree_site;
      if (num_iterations > 1000) damping_factor = R(0.5);
      free_site_conc = free_site_conc + damping_factor * dfree_site_conc;
      R rel = std::fabs(dfree_site_conc / free_site_conc);
      if (rel < R(1e-12)) one_more = true;
    } else {
      total = total / free_site_conc;
      free_site_conc = site_density / total;
      one_more = true;
    }
  }
  c.srfcplxrxn_free_site_conc[irxn] = free_site_conc;
  // 2.3-46: derivative of the free-site concentration
  R dSx_dmi[P];
  for (int j = 0; j < N; ++j) dSx_dmi[j] = 0;
  R tempreal = 0;
  for (int j = 1; j <= ncplx; ++j) {
    int ic = w.src(irxn, j);
    for (int k = 1; k <= w.sn(ic); ++k) {
      int icomp = w.sid(ic, k);
      dSx_dmi[icomp] = dSx_dmi[icomp] + R(w.snu(ic, k)) * R(n.srfcplx_free_site_stoich[ic]) * srfcplx_conc[ic];
    }
    tempreal = tempreal + R(n.srfcplx_free_site_stoich[ic]) * R(n.srfcplx_free_site_stoich[ic]) * srfcplx_conc[ic];
  }
  tempreal = tempreal / free_site_conc;
  tempreal = tempreal + R(1);
  for (int j = 0; j < N; ++j) {
    dSx_dmi[j] = -dSx_dmi[j] / tempreal;
    dSx_dmi[j] = dSx_dmi[j] / c.pri_molal[j];
  }
  for (int i = 0; i < w.Nsc; ++i) c.eqsrfcplx_conc[i] = c.eqsrfcplx_conc[i] + srfcplx_conc[i];
  for (int kk = 1; kk <= ncplx; ++kk) {
    int ic = w.src(irxn, kk);
    const int nc = w.sn(ic);
    for (int i = 1; i <= nc; ++i) {
      int icomp = w.sid(ic, i);
      c.total_sorb_eq[icomp] = c.total_sorb_eq[icomp] + R(w.snu(ic, i)) * srfcplx_conc[ic];
    }
    R nui_Si_over_Sx = R(n.srfcplx_free_site_stoich[ic]) * srfcplx_conc[ic] / free_site_conc;
    if (w.exact_jac) {
      // every component of the site moves the free-site concentration
      R t[P];
      for (int j = 0; j < N; ++j) t[j] = nui_Si_over_Sx * dSx_dmi[j];
      for (int j = 1; j <= nc; ++j) {
        int jcomp = w.sid(ic, j);
        t[jcomp] = R(w.snu(ic, j)) * srfcplx_conc[ic] / c.pri_molal[jcomp] + t[jcomp];
      }
      for (int i = 1; i <= nc; ++i) {
        int icomp = w.sid(ic, i);
        for (int j = 0; j < N; ++j) c.dtotal_sorb_eq[icomp][j] = c.dtotal_sorb_eq[icomp][j] + R(w.snu(ic, i)) * t[j];
      }
      continue;
    }
    for (int j = 1; j <= nc; ++j) {
      int jcomp = w.sid(ic, j);
      R t = R(w.snu(ic, j)) * srfcplx_conc[ic] / c.pri_molal[jcomp] + nui_Si_over_Sx * dSx_dmi[jcomp];
      for (int i = 1; i <= nc; ++i) {
        int icomp = w.sid(ic, i);
        c.dtotal_sorb_eq[icomp][jcomp] = c.dtotal_sorb_eq[icomp][jcomp] + R(w.snu(ic, i)) * t;
      }
    }
  }
  return 0;
}

// reaction.F90:4305-4535 RTotalSorbEqIonx (the "#if 1" KDj implementation)
template <class R>
int total_sorb_eq_ionx(const Net &w, Cell<R> &c) {
  const pfchem_network &n = *w.n;
  const int N = w.N;
  R ln_conc[P], ln_act[P];
  for (int j = 0; j < N; ++j) {
    ln_conc[j] = rlog(c.pri_molal[j]);
    ln_act[j] = ln_conc[j] + rlog(c.pri_act_coef[j]);
  }
  (void)ln_act;
  for (int r = 0; r < w.Nix; ++r)
    for (int k = 0; k < NZ; ++k) c.eqionx_conc[k][r] = 0;
  for (int irxn = 0; irxn < w.Nix; ++irxn) {
    const int ncomp = w.xn(irxn);
    R omega;
    if (n.eqionx_rxn_to_surf && n.eqionx_rxn_to_surf[irxn] > 0) {
      omega = std::max(R(n.eqionx_rxn_CEC[irxn]) * c.mnrl_volfrac[n.eqionx_rxn_to_surf[irxn] - 1], R(1e-40));
    } else {
      omega = n.eqionx_rxn_CEC[irxn];
    }
    R cation_X[NZ];
    for (int k = 0; k < NZ; ++k) cation_X[k] = 0;
    if (n.eqionx_rxn_Z_flag[irxn]) {
      int icomp = w.xid(irxn, 1);
      R ref_cation_conc = c.pri_molal[icomp] * c.pri_act_coef[icomp];
      R ref_cation_Z = n.primary_spec_Z[icomp];
      R ref_cation_k = w.xk(irxn, 1);
      R ref_cation_X = ref_cation_Z * c.eqionx_ref_cation_sorbed_conc[irxn] / omega;
      bool one_more = false;
      R KDj = ref_cation_X / (ref_cation_k * ref_cation_conc);
      int it = 0;
      for (;;) {
        ++it;
        if (it > 20000) return 1;  // reference: printErrMsgByRank (reaction.F90:4382-4385)
        ref_cation_X = KDj * (ref_cation_k * ref_cation_conc);
        cation_X[0] = ref_cation_X;
        R total = ref_cation_X;
        R dres_dKDj = 0;
        for (int j = 2; j <= ncomp; ++j) {
          int ic = w.xid(irxn, j);
          R zi = n.primary_spec_Z[ic];
          cation_X[j - 1] = R(w.xk(irxn, j)) * c.pri_molal[ic] * c.pri_act_coef[ic] * std::pow(KDj, zi / ref_cation_Z);
          total = total + cation_X[j - 1];
          dres_dKDj = dres_dKDj + cation_X[j - 1] / KDj * zi;
        }
        dres_dKDj = dres_dKDj / ref_cation_Z + (ref_cation_k * ref_cation_conc);
        R res = R(1) - total;
        if (one_more) break;
        R delta_KDj = res / dres_dKDj;
        KDj = KDj + delta_KDj;
        KDj = std::max(KDj, R(1e-40));
        if (std::fabs(delta_KDj / KDj) < R(1e-12)) one_more = true;
      }
      c.eqionx_ref_cation_sorbed_conc[irxn] = ref_cation_X * omega / ref_cation_Z;
    } else {
      R sumkm = 0;
      for (int j = 1; j <= ncomp; ++j) {
        int ic = w.xid(irxn, j);
        cation_X[j - 1] = c.pri_molal[ic] * c.pri_act_coef[ic] * R(w.xk(irxn, j));
        sumkm = sumkm + cation_X[j - 1];
      }
      for (int j = 0; j < ncomp; ++j) cation_X[j] = cation_X[j] / sumkm;
    }
    R sumZX = 0;
    for (int i = 1; i <= ncomp; ++i) sumZX = sumZX + R(n.primary_spec_Z[w.xid(irxn, i)]) * cation_X[i - 1];
    for (int i = 1; i <= ncomp; ++i) {
      int icomp = w.xid(irxn, i);
      R tempreal1 = cation_X[i - 1] * omega / R(n.primary_spec_Z[icomp]);
      c.eqionx_conc[i - 1][irxn] = c.eqionx_conc[i - 1][irxn] + tempreal1;
      c.total_sorb_eq[icomp] = c.total_sorb_eq[icomp] + tempreal1;
      R tempreal2 = R(n.primary_spec_Z[icomp]) / sumZX;
      for (int j = 1; j <= ncomp; ++j) {
        int jcomp = w.xid(irxn, j);
        if (i == j) {
          c.dtotal_sorb_eq[icomp][jcomp] = c.dtotal_sorb_eq[icomp][jcomp] +
                                           tempreal1 * (R(1) - (tempreal2 * cation_X[j - 1])) / c.pri_molal[jcomp];
        } else {
          c.dtotal_sorb_eq[icomp][jcomp] = c.dtotal_sorb_eq[icomp][jcomp] +
                                           (-tempreal1) * tempreal2 * cation_X[j - 1] / c.pri_molal[jcomp];
        }
      }
    }
  }
  return 0;
}

// reaction.F90:4182-4216 RTotalSorb (+ RZeroSorb :4160-4178)
template <class R>
int total_sorb(const Net &w, Cell<R> &c) {
  for (int i = 0; i < w.N; ++i) {
    c.total_sorb_eq[i] = 0;
    for (int j = 0; j < w.N; ++j) c.dtotal_sorb_eq[i][j] = 0;
  }
  for (int i = 0; i < w.Nsc; ++i) c.eqsrfcplx_conc[i] = 0;
  int fail = 0;
  for (int r = 0; r < w.Nsr; ++r) fail |= total_sorb_eq_surfcplx1(w, c, r);
  if (w.Nix > 0) fail |= total_sorb_eq_ionx(w, c);
  return fail;
}

// reaction.F90:4969-5068 RTAuxVarCompute
template <class R>
int auxvar_compute(const Net &w, Cell<R> &c) {
  rtotal(w, c);
  if (w.Nix + w.Nsr > 0) return total_sorb(w, c);
  return 0;
}

// ---------------------------------------------------------------------------
// reaction_mineral.F90:564-1000 RKineticMineral (non-solid-solution branch)
template <class R>
void kinetic_mineral(const Net &w, Cell<R> &c, R *Res, R (*Jac)[P], bool compute_derivative) {
  const pfchem_network &n = *w.n;
  const int N = w.N;
  R ln_conc[P], ln_act[P], ln_sec[C], ln_sec_act[C];
  for (int j = 0; j < N; ++j) {
    ln_conc[j] = rlog(c.pri_molal[j]);
    ln_act[j] = ln_conc[j] + rlog(c.pri_act_coef[j]);
  }
  for (int i = 0; i < w.Nc; ++i) {
    ln_sec[i] = rlog(c.sec_molal[i]);
    ln_sec_act[i] = ln_sec[i] + rlog(c.sec_act_coef[i]);
  }
  const int maxpref = n.max_num_prefactors, maxsp = n.max_num_prefactor_species;
  for (int m = 0; m < w.Nm; ++m) c.mnrl_rate[m] = 0;
  for (int m = 0; m < w.Nm; ++m) {
    R lnQK = -c.kinmnrl_logK[m] * R(kLOG_TO_LN);
    if (n.kinmnrlh2oid && n.kinmnrlh2oid[m] > 0) lnQK = lnQK + R(n.kinmnrlh2ostoich[m]) * c.ln_act_h2o;
    const int ncomp = w.mn(m);
    for (int i = 1; i <= ncomp; ++i) lnQK = lnQK + R(w.mnu(m, i)) * ln_act[w.mid(m, i)];
    R QK = (lnQK <= R(6.90776)) ? rexp(lnQK) : R(1e3);
    R affinity_factor;
    if (n.kinmnrl_Temkin_const) {
      if (n.kinmnrl_min_scale_factor)
        affinity_factor = R(1) - std::pow(QK, R(1) / (R(n.kinmnrl_min_scale_factor[m]) * R(n.kinmnrl_Temkin_const[m])));
      else
        affinity_factor = R(1) - std::pow(QK, R(1) / R(n.kinmnrl_Temkin_const[m]));
    } else if (n.kinmnrl_min_scale_factor) {
      affinity_factor = R(1) - std::pow(QK, R(1) / R(n.kinmnrl_min_scale_factor[m]));
    } else {
      affinity_factor = R(1) - QK;
    }
    R sign_ = std::signbit((double)affinity_factor) ? R(-1) : R(1);  // Fortran sign(1.d0, x)
    R sum_prefactor_rate, Im, Im_const;
    R prefactor[PFCHEM_MAX_PREF], ln_prefactor_spec[PFCHEM_MAX_PREF_SPEC][PFCHEM_MAX_PREF];
    const int npref = n.kinmnrl_num_prefactors ? n.kinmnrl_num_prefactors[m] : 0;
    if (c.mnrl_volfrac[m] > 0 || sign_ < 0) {
      if (n.kinmnrl_affinity_threshold[m] > 0) {
        if (sign_ < 0 && QK < R(n.kinmnrl_affinity_threshold[m])) continue;
      }
      if (n.kinmnrl_rate_limiter[m] > 0) {
        affinity_factor = affinity_factor / (R(1) + (R(1) - affinity_factor) / R(n.kinmnrl_rate_limiter[m]));
      }
      if (npref > 0) {
        sum_prefactor_rate = 0;
        for (int p = 0; p < PFCHEM_MAX_PREF; ++p) {
          prefactor[p] = 0;
          for (int s = 0; s < PFCHEM_MAX_PREF_SPEC; ++s) ln_prefactor_spec[s][p] = 0;
        }
        for (int p = 0; p < npref; ++p) {
          R ln_prefactor = 0;
          const int base = (maxsp + 1) * (p + maxpref * m);
          const int nsp = n.kinmnrl_prefactor_id[base];
          for (int s = 1; s <= nsp; ++s) {
            int icomp = n.kinmnrl_prefactor_id[base + s];
            R ln_spec_act = icomp > 0 ? ln_act[icomp - 1] : ln_sec_act[-icomp - 1];
            const int q = (s - 1) + maxsp * (p + maxpref * m);
            R ln_numerator = R(n.kinmnrl_pref_alpha[q]) * ln_spec_act;
            R ln_denominator = rlog(R(1) + rexp(rlog(R(n.kinmnrl_pref_atten_coef[q])) + R(n.kinmnrl_pref_beta[q]) * ln_spec_act));
            ln_prefactor = ln_prefactor + ln_numerator;
            ln_prefactor = ln_prefactor - ln_denominator;
            ln_prefactor_spec[s - 1][p] = ln_numerator - ln_denominator;
          }
          prefactor[p] = rexp(ln_prefactor);
          R arrhenius_factor = 1;
          const double Ea = n.kinmnrl_pref_activation_energy[p + maxpref * m];
          if (Ea > 0)
            arrhenius_factor = rexp(R(Ea) / R(kIDEAL_GAS_CONSTANT) *
                                    (R(1) / (R(25) + R(273.15)) - R(1) / (c.temp + R(273.15))));
          sum_prefactor_rate = sum_prefactor_rate + prefactor[p] * R(n.kinmnrl_pref_rate[p + maxpref * m]) * arrhenius_factor;
        }
      } else {
        R arrhenius_factor = 1;
        if (n.kinmnrl_activation_energy[m] > 0)
          arrhenius_factor = rexp(R(n.kinmnrl_activation_energy[m]) / R(kIDEAL_GAS_CONSTANT) *
                                  (R(1) / (R(25) + R(273.15)) - R(1) / (c.temp + R(273.15))));
        sum_prefactor_rate = R(n.kinmnrl_rate_constant[m]) * arrhenius_factor;
      }
      Im_const = -c.mnrl_area[m];
      if (n.kinmnrl_min_scale_factor) Im_const = Im_const / R(n.kinmnrl_min_scale_factor[m]);
      if (n.kinmnrl_affinity_power)
        Im = Im_const * sign_ * std::pow(std::fabs(affinity_factor), R(n.kinmnrl_affinity_power[m])) * sum_prefactor_rate;
      else
        Im = Im_const * sign_ * std::fabs(affinity_factor) * sum_prefactor_rate;
      c.mnrl_rate[m] = Im;
    } else {
      continue;
    }
    Im_const = Im_const * c.volume;
    Im = Im * c.volume;
    for (int i = 1; i <= ncomp; ++i) {
      int ic = w.mid(m, i);
      Res[ic] = Res[ic] + R(w.mnu(m, i)) * Im;
    }
    if (!compute_derivative) continue;
    R dIm_dQK;
    // exact: where QK is capped the rate does not depend on QK (the
    // prefactor terms below still apply)
    const bool qk_terms = !(w.exact_jac && lnQK > R(6.90776));
    if (n.kinmnrl_affinity_power)
      dIm_dQK = -Im * R(n.kinmnrl_affinity_power[m]) / (w.exact_jac ? affinity_factor : std::fabs(affinity_factor));
    else
      dIm_dQK = -Im_const * sum_prefactor_rate;
    if (n.kinmnrl_Temkin_const) {
      if (n.kinmnrl_min_scale_factor)
        dIm_dQK = dIm_dQK * (R(1) / (R(n.kinmnrl_min_scale_factor[m]) * R(n.kinmnrl_Temkin_const[m]))) / QK * (R(1) - affinity_factor);
      else
        dIm_dQK = dIm_dQK * (R(1) / R(n.kinmnrl_Temkin_const[m])) / QK * (R(1) - affinity_factor);
    } else if (n.kinmnrl_min_scale_factor) {
      dIm_dQK = dIm_dQK * (R(1) / R(n.kinmnrl_min_scale_factor[m])) / QK * (R(1) - affinity_factor);
    }
    if (!qk_terms) {
    } else if (n.kinmnrl_rate_limiter[m] <= 0) {
      for (int j = 1; j <= ncomp; ++j) {
        int jc = w.mid(m, j);
        R dQK_dCj = R(w.mnu(m, j)) * QK * rexp(-ln_conc[jc]);
        R dQK_dmj = w.exact_jac ? dQK_dCj : dQK_dCj * c.den_kg * R(1e-3);
        for (int i = 1; i <= ncomp; ++i) {
          int ic = w.mid(m, i);
          Jac[ic][jc] = Jac[ic][jc] + R(w.mnu(m, i)) * dIm_dQK * dQK_dmj;
        }
      }
    } else {
      R rl = n.kinmnrl_rate_limiter[m];
      R den = R(1) + (R(1) - affinity_factor) / rl;
      for (int j = 1; j <= ncomp; ++j) {
        int jc = w.mid(m, j);
        R dQK_dCj = R(w.mnu(m, j)) * QK * rexp(-ln_conc[jc]);
        R dQK_dmj = w.exact_jac ? dQK_dCj : dQK_dCj * c.den_kg * R(1e-3);
        for (int i = 1; i <= ncomp; ++i) {
          int ic = w.mid(m, i);
          Jac[ic][jc] = Jac[ic][jc] + R(w.mnu(m, i)) * dIm_dQK * (R(1) + QK / rl / den) * dQK_dmj / den;
        }
      }
    }
    if (npref > 0) {
      R dIm_dsum_prefactor_rate = Im / sum_prefactor_rate;
      for (int p = 0; p < npref; ++p) {
        R arrhenius_factor = 1;
        const double Ea = n.kinmnrl_pref_activation_energy[p + maxpref * m];
        if (Ea > 0)
          arrhenius_factor = rexp(R(Ea) / R(kIDEAL_GAS_CONSTANT) *
                                  (R(1) / (R(25) + R(273.15)) - R(1) / (c.temp + R(273.15))));
        R ln_prefactor = rlog(prefactor[p]);
        const int base = (maxsp + 1) * (p + maxpref * m);
        const int nsp = n.kinmnrl_prefactor_id[base];
        for (int s = 1; s <= nsp; ++s) {
          const int q = (s - 1) + maxsp * (p + maxpref * m);
          R dprefactor_dprefactor_spec = rexp(ln_prefactor - ln_prefactor_spec[s - 1][p]);
          int icomp = n.kinmnrl_prefactor_id[base + s];
          R ln_spec_act, spec_act_coef;
          if (icomp > 0) {
            ln_spec_act = ln_act[icomp - 1];
            spec_act_coef = c.pri_act_coef[icomp - 1];
          } else {
            ln_spec_act = ln_sec_act[-icomp - 1];
            spec_act_coef = c.sec_act_coef[-icomp - 1];
          }
          R num = R(n.kinmnrl_pref_alpha[q]) * rexp(ln_prefactor_spec[s - 1][p] - ln_spec_act);
          R ln_gam_m_beta = R(n.kinmnrl_pref_beta[q]) * ln_spec_act;
          R denominator = R(1) + rexp(rlog(R(n.kinmnrl_pref_atten_coef[q])) + ln_gam_m_beta);
          R dden = R(-1) * rexp(ln_prefactor_spec[s - 1][p]) / denominator * R(n.kinmnrl_pref_atten_coef[q]) *
                   R(n.kinmnrl_pref_beta[q]) * rexp(ln_gam_m_beta - ln_spec_act);
          R dspec = (num + dden) * spec_act_coef;
          R dIm_dspec = dIm_dsum_prefactor_rate * dprefactor_dprefactor_spec * dspec *
                        R(n.kinmnrl_pref_rate[p + maxpref * m]) * arrhenius_factor;
          if (icomp > 0) {
            for (int i = 1; i <= ncomp; ++i) {
              int jc = w.mid(m, i);
              Jac[jc][icomp - 1] = Jac[jc][icomp - 1] + R(w.mnu(m, i)) * dIm_dspec;
            }
          } else {
            // reaction_mineral.F90:958-991: derivative through a secondary
            // species.  The reference reuses `ncomp` and `icomp` here, so the
            // species loops below run over the complex's own species: the
            // rows are the complex's species with its stoichiometry.  The
            // exact Jacobian puts the same column derivative into the
            // mineral's rows.  (A primary prefactor species listed after a
            // secondary one in the same mineral would, in the reference, loop
            // over the complex's species count; here it uses the mineral's.)
            int icplx = -icomp - 1;
            R lq = -c.eqcplx_logK[icplx] * R(kLOG_TO_LN);
            if (n.eqcplxh2oid && n.eqcplxh2oid[icplx] > 0) lq = lq + R(n.eqcplxh2ostoich[icplx]) * c.ln_act_h2o;
            const int ncx = w.cn(icplx);
            for (int i = 1; i <= ncx; ++i) lq = lq + R(w.cnu(icplx, i)) * ln_act[w.cid(icplx, i)];
            for (int j = 1; j <= ncx; ++j) {
              int jc = w.cid(icplx, j);
              R t = R(w.cnu(icplx, j)) * rexp(lq - ln_conc[jc]) / c.sec_act_coef[icplx];
              if (w.exact_jac) {
                for (int i = 1; i <= ncomp; ++i) {
                  int ic = w.mid(m, i);
                  Jac[ic][jc] = Jac[ic][jc] + R(w.mnu(m, i)) * t * dIm_dspec;
                }
              } else {
                for (int i = 1; i <= ncx; ++i) {
                  int ic = w.cid(icplx, i);
                  Jac[ic][jc] = Jac[ic][jc] + R(w.cnu(icplx, i)) * t * dIm_dspec;
                }
              }
            }
          }
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// utility.F90:393-473 ludcmp (Crout, implicit-scaling partial pivoting)
template <class R>
int ludcmp(R (*A)[P], int N, int *INDX) {
  R VV[P];
  const R tiny = R(1e-20);
  for (int i = 0; i < N; ++i) {
    R aamax = 0;
    for (int j = 0; j < N; ++j)
      if (std::fabs(A[i][j]) > aamax) aamax = std::fabs(A[i][j]);
    if (aamax <= 0) return 1;  // reference: prints and MPI_Abort (utility.F90:423-432)
    VV[i] = R(1) / aamax;
  }
  int imax = 0;
  for (int j = 0; j < N; ++j) {
    for (int i = 0; i < j; ++i) {
      R sum = A[i][j];
      for (int k = 0; k < i; ++k) sum = sum - A[i][k] * A[k][j];
      A[i][j] = sum;
    }
    R aamax = 0;
    for (int i = j; i < N; ++i) {
      R sum = A[i][j];
      for (int k = 0; k < j; ++k) sum = sum - A[i][k] * A[k][j];
      A[i][j] = sum;
      R dum = VV[i] * std::fabs(sum);
      if (dum >= aamax) {
        imax = i;
        aamax = dum;
      }
    }
    if (j != imax) {
      for (int k = 0; k < N; ++k) std::swap(A[imax][k], A[j][k]);
      VV[imax] = VV[j];
    }
    INDX[j] = imax;
    if (A[j][j] == 0) A[j][j] = tiny;
    if (j != N - 1) {
      R dum = R(1) / A[j][j];
      for (int i = j + 1; i < N; ++i) A[i][j] = A[i][j] * dum;
    }
  }
  return 0;
}

// utility.F90:477-523 lubksb
template <class R>
void lubksb(R (*A)[P], int N, const int *INDX, R *B) {
  int ii = -1;
  for (int i = 0; i < N; ++i) {
    int ll = INDX[i];
    R sum = B[ll];
    B[ll] = B[i];
    if (ii >= 0) {
      for (int j = ii; j < i; ++j) sum = sum - A[i][j] * B[j];
    } else if (sum != 0) {
      ii = i;
    }
    B[i] = sum;
  }
  for (int i = N - 1; i >= 0; --i) {
    R sum = B[i];
    for (int j = i + 1; j < N; ++j) sum = sum - A[i][j] * B[j];
    B[i] = sum / A[i][i];
  }
}

// reaction.F90:4835-4880 RSolve
template <class R>
int rsolve(const R *Res, R (*Jac)[P], const R *conc, R *update, int N, bool use_log) {
  R rhs[P];
  for (int i = 0; i < N; ++i) {
    R mx = 0;
    for (int j = 0; j < N; ++j) mx = std::max(mx, std::fabs(Jac[i][j]));
    R norm = std::max(R(1), mx);
    norm = R(1) / norm;
    rhs[i] = Res[i] * norm;
    for (int j = 0; j < N; ++j) Jac[i][j] = Jac[i][j] * norm;
  }
  if (use_log)
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) Jac[i][j] = Jac[i][j] * conc[j];
  int indx[P];
  if (ludcmp(Jac, N, indx)) return 1;
  lubksb(Jac, N, indx, rhs);
  for (int i = 0; i < N; ++i) update[i] = rhs[i];
  return 0;
}

// Magnitude scale S_j of the terms summed into residual component j; the
// relative-residual test is max_j |F_j| / S_j < tol.
template <class R>
void residual_scale(const Net &w, const pfchem_options &o, const Cell<R> &c, const R *fixed_accum,
                    R psv_t, R accum_scale, R *S) {
  const pfchem_network &n = *w.n;
  R den_kg_per_L = c.den_kg * R(1e-3);
  for (int j = 0; j < w.N; ++j) S[j] = c.pri_molal[j];
  for (int i = 0; i < w.Nc; ++i)
    for (int k = 1; k <= w.cn(i); ++k) S[w.cid(i, k)] += std::fabs(R(w.cnu(i, k))) * c.sec_molal[i];
  for (int j = 0; j < w.N; ++j) S[j] = (S[j] * den_kg_per_L * psv_t + std::fabs(fixed_accum[j])) * accum_scale;
  // sorbed terms
  R sorb[P];
  for (int j = 0; j < w.N; ++j) sorb[j] = 0;
  for (int r = 0; r < w.Nix; ++r)
    for (int k = 1; k <= w.xn(r); ++k) sorb[w.xid(r, k)] += std::fabs(c.eqionx_conc[k - 1][r]);
  for (int i = 0; i < w.Nsc; ++i)
    for (int k = 1; k <= w.sn(i); ++k) sorb[w.sid(i, k)] += std::fabs(R(w.snu(i, k)) * c.eqsrfcplx_conc[i]);
  for (int j = 0; j < w.N; ++j) S[j] += sorb[j] * c.volume * accum_scale;
  for (int m = 0; m < w.Nm; ++m)
    for (int k = 1; k <= w.mn(m); ++k) S[w.mid(m, k)] += std::fabs(R(w.mnu(m, k)) * c.mnrl_rate[m]) * c.volume;
  (void)n;
  (void)o;
}

// Residual of the step equations at the cell's current pri_molal, as the
// Newton loop below forms it, and its norm in the units of the convergence
// test (DBL_MAX when not finite).  Returns false when an inner sorption
// iteration failed.  Used only for the choice between two starting guesses,
// an addition of this library with no counterpart in RReact.
template <class R>
bool residual_norm(const Net &w, const pfchem_options &o, Cell<R> &c, const R *fixed_accum, R psv_t, R dt,
                   R accum_scale, R *rnorm) {
  const int N = w.N;
  const bool sorb = (w.Nix + w.Nsr) > 0;
  const bool inner_ok = auxvar_compute(w, c) == 0;
  R residual[P], J[P][P];
  for (int j = 0; j < N; ++j) {
    if (o.accum_mode == PFCHEM_ACCUM_LITERAL) {
      residual[j] = psv_t * c.total[j] - fixed_accum[j];
      if (sorb) residual[j] = residual[j] + c.total_sorb_eq[j] * c.volume;
    } else {
      R acc = psv_t * c.total[j];
      if (sorb) acc = acc + c.total_sorb_eq[j] * c.volume;
      residual[j] = -fixed_accum[j] / dt + acc / dt;
    }
  }
  if (w.Nm > 0) kinetic_mineral(w, c, residual, J, false);
  bool nonfinite = false;
  for (int j = 0; j < N; ++j)
    if (!std::isfinite((double)residual[j])) nonfinite = true;
  if (nonfinite) {
    *rnorm = R(DBL_MAX);
    return inner_ok;
  }
  R r = 0;
  if (o.residual_tol_kind == PFCHEM_RESIDUAL_RELATIVE) {
    R S[P];
    residual_scale(w, o, c, fixed_accum, psv_t, accum_scale, S);
    for (int j = 0; j < N; ++j) r = std::max(r, std::fabs(residual[j]) / S[j]);
  } else {
    for (int j = 0; j < N; ++j) r = std::max(r, std::fabs(residual[j]));
  }
  *rnorm = r;
  return inner_ok;
}

// One Newton system of RReact at the cell's current pri_molal: auxiliary
// variables, residual and Jacobian d residual / d m (reaction.F90:3415-3440).
// Returns non-zero when an inner sorption iteration failed.
template <class R>
int newton_system(const Net &w, const pfchem_options &o, Cell<R> &c, const R *fixed_accum, R psv_t, R dt,
                  R *residual, R (*J)[P]) {
  const int N = w.N;
  const bool sorb = (w.Nix + w.Nsr) > 0;
  const R psvd_t = c.porosity * c.sat * R(1000) * c.volume / dt;
  const R v_t = c.volume / dt;
  if (auxvar_compute(w, c)) return 1;
  // residual: the literal RReact order (reaction.F90:3424-3432), or the
  // global-implicit order r = -accum/dt + (psv*T + V*S)/dt + R
  // (reactive_transport.F90:2541-2564)
  if (o.accum_mode == PFCHEM_ACCUM_LITERAL) {
    for (int j = 0; j < N; ++j) residual[j] = psv_t * c.total[j] - fixed_accum[j];
    if (sorb)
      for (int j = 0; j < N; ++j) residual[j] = residual[j] + c.total_sorb_eq[j] * c.volume;
  } else {
    for (int j = 0; j < N; ++j) {
      R acc = psv_t * c.total[j];
      if (sorb) acc = acc + c.total_sorb_eq[j] * c.volume;
      residual[j] = -fixed_accum[j] / dt + acc / dt;
    }
  }
  // RTAccumulationDerivative (reaction.F90:5152-5232)
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) J[i][j] = c.dtotal[i][j] * psvd_t;
  if (sorb)  // RAccumulationSorbDerivative (reaction.F90:4575-4603)
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) J[i][j] = J[i][j] + c.dtotal_sorb_eq[i][j] * v_t;
  // RReaction -> RKineticMineral (reaction.F90:3515-3584)
  if (w.Nm > 0) kinetic_mineral(w, c, residual, J, true);
  return 0;
}

// ---------------------------------------------------------------------------
// reaction.F90:3322-3511 RReact.  Returns the per-cell status.  `alt`, when
// given, is a second starting guess (the learned warm start): the residual
// is evaluated at both guesses and Newton starts from `alt` when its norm is
// no larger, keeping the ion-exchange warm start of the evaluation it chose
// and the surface free-site state it was given.  With the library option
// exact_jacobian_after = K > 0 (no counterpart in the reference) iterations
// past K use the exact Jacobian and skip the damping of :3478-3496.
template <class R>
int rreact(const Net &w, const pfchem_options &o, Cell<R> &c, const R *tran_xx, R dt, R I_start,
           int *num_iterations_out, const double *alt = nullptr, bool *alt_used = nullptr) {
  const int N = w.N;
  const bool sorb = (w.Nix + w.Nsr) > 0;
  const R one_over_dt = R(1) / dt;
  const R accum_scale = (o.accum_mode == PFCHEM_ACCUM_DT_CONSISTENT) ? one_over_dt : R(1);
  int num_iterations = 0;
  for (int j = 0; j < N; ++j) c.total[j] = tran_xx[j];
  update_temp_dependent_coefs(w, o, c);  // reaction.F90:3394-3396 (isothermal: tables as given)
  // RTAccumulation (reaction.F90:5072-5148): psv*total, no /dt
  const R psv_t = c.porosity * c.sat * R(1000) * c.volume;
  R fixed_accum[P];
  for (int j = 0; j < N; ++j) fixed_accum[j] = psv_t * c.total[j];
  if (sorb)
    for (int j = 0; j < N; ++j) fixed_accum[j] = fixed_accum[j] + c.total_sorb_eq[j] * c.volume;
  if (o.act_coef_update_frequency != PFCHEM_ACT_COEF_FREQUENCY_OFF) {
    if (activity_coefficients(w, o, c, true, I_start)) {
      *num_iterations_out = 0;
      return PFCHEM_CELL_INNER_MAXITER;
    }
  } else {
    for (int j = 0; j < N; ++j) c.pri_act_coef[j] = 1;
    for (int i = 0; i < w.Nc; ++i) c.sec_act_coef[i] = 1;
  }
  if (alt) {
    R srf[SR];
    for (int r = 0; r < w.Nsr; ++r) srf[r] = c.srfcplxrxn_free_site_conc[r];
    R rplain, ralt = R(DBL_MAX);
    residual_norm(w, o, c, fixed_accum, psv_t, dt, accum_scale, &rplain);  // inner status not used here
    const Cell<R> plain = c;
    bool ok = true;
    for (int j = 0; j < N; ++j) {
      const double g = alt[j];
      if (g > 0.0 && g <= DBL_MAX) c.pri_molal[j] = R(g);
      else ok = false;
    }
    if (ok) {
      R r;
      if (residual_norm(w, o, c, fixed_accum, psv_t, dt, accum_scale, &r) && r < R(DBL_MAX)) ralt = r;
    }
    const bool take = ralt <= rplain;
    if (!take) c = plain;
    for (int r = 0; r < w.Nsr; ++r) c.srfcplxrxn_free_site_conc[r] = srf[r];
    if (alt_used) *alt_used = take;
  }
  int status = PFCHEM_CELL_CONVERGED;
  R residual[P], J[P][P], update[P], prev_solution[P], new_solution[P];
  // exact_jacobian_after = K > 0: past iteration K the exact Jacobian, no damping
  Net w_exact = w;
  w_exact.exact_jac = true;
  for (;;) {
    ++num_iterations;
    const bool rescue = o.exact_jacobian_after > 0 && num_iterations > o.exact_jacobian_after;
    const Net &wn = rescue ? w_exact : w;
    if (o.act_coef_update_frequency == PFCHEM_ACT_COEF_FREQUENCY_NEWTON_ITER) {
      if (activity_coefficients(w, o, c, num_iterations == 1, I_start)) {
        status = PFCHEM_CELL_INNER_MAXITER;
        break;
      }
    }
    if (newton_system(wn, o, c, fixed_accum, psv_t, dt, residual, J)) {
      status = PFCHEM_CELL_INNER_MAXITER;
      break;
    }
    bool nonfinite = false;
    R rmax = 0;
    for (int j = 0; j < N; ++j) {
      if (!std::isfinite((double)residual[j])) nonfinite = true;
      rmax = std::max(rmax, std::fabs(residual[j]));
    }
    if (nonfinite) {
      status = PFCHEM_CELL_NONFINITE;
      break;
    }
    if (o.residual_tol_kind == PFCHEM_RESIDUAL_RELATIVE) {
      R S[P];
      residual_scale(w, o, c, fixed_accum, psv_t, accum_scale, S);
      R rr = 0;
      for (int j = 0; j < N; ++j) rr = std::max(rr, std::fabs(residual[j]) / S[j]);
      if (rr < R(o.max_residual_tolerance)) break;
    } else {
      if (rmax < R(o.max_residual_tolerance)) break;
    }
    if (num_iterations >= o.max_iterations) {
      status = PFCHEM_CELL_MAXITER;
      break;
    }
    if (rsolve(residual, J, c.pri_molal, update, N, o.use_log_formulation != 0)) {
      status = PFCHEM_CELL_SINGULAR;
      break;
    }
    for (int j = 0; j < N; ++j) prev_solution[j] = c.pri_molal[j];
    if (o.use_log_formulation) {
      for (int j = 0; j < N; ++j) {
        R s = std::signbit((double)update[j]) ? R(-1) : R(1);
        update[j] = s * std::min(std::fabs(update[j]), R(o.max_dlnC));
        new_solution[j] = prev_solution[j] * rexp(-update[j]);
      }
    } else {
      R min_ratio = R(1e20);
      for (int j = 0; j < N; ++j) {
        if (prev_solution[j] <= update[j]) {
          R ratio = std::fabs(prev_solution[j] / update[j]);
          if (ratio < min_ratio) min_ratio = ratio;
        }
      }
      if (min_ratio < R(1))
        for (int j = 0; j < N; ++j) update[j] = update[j] * min_ratio * R(0.99);
      for (int j = 0; j < N; ++j) new_solution[j] = prev_solution[j] - update[j];
    }
    R maximum_relative_change = 0;
    bool bad = false;
    for (int j = 0; j < N; ++j) {
      R rc = std::fabs((new_solution[j] - prev_solution[j]) / prev_solution[j]);
      if (!std::isfinite((double)new_solution[j])) bad = true;
      maximum_relative_change = std::max(maximum_relative_change, rc);
    }
    if (bad) {
      status = PFCHEM_CELL_NONFINITE;
      break;
    }
    if (o.max_relative_change_tolerance > 0 &&
        maximum_relative_change < R(o.max_relative_change_tolerance))
      break;
    if (num_iterations > 50 && !rescue) {
      R scale = R(0.1);  // reaction.F90:3478-3496: only the first branch is reachable
      for (int j = 0; j < N; ++j) new_solution[j] = scale * (new_solution[j] - prev_solution[j]) + prev_solution[j];
    }
    for (int j = 0; j < N; ++j) c.pri_molal[j] = new_solution[j];
  }
  // one last update (reaction.F90:3507)
  if (status == PFCHEM_CELL_CONVERGED && auxvar_compute(w, c)) status = PFCHEM_CELL_INNER_MAXITER;
  *num_iterations_out = num_iterations;
  return status;
}

// reaction.F90:5320-5365 RUpdateKineticState (mineral part)
template <class R>
void update_kinetic_state(const Net &w, Cell<R> &c, R dt) {
  if (w.Nm == 0) return;
  R res[P], jac[P][P];
  for (int j = 0; j < w.N; ++j) res[j] = 0;
  kinetic_mineral(w, c, res, jac, false);
  for (int m = 0; m < w.Nm; ++m) {
    R delta_volfrac = c.mnrl_rate[m] * R(w.n->kinmnrl_molar_vol[m]) * dt;
    c.mnrl_volfrac[m] = c.mnrl_volfrac[m] + delta_volfrac;
    if (c.mnrl_volfrac[m] < 0) c.mnrl_volfrac[m] = 0;
  }
}

template <class R>
R ionic_strength_of(const Net &w, const Cell<R> &c) {
  R I = 0;
  for (int j = 0; j < w.N; ++j) I = I + c.pri_molal[j] * R(w.n->primary_spec_Z[j]) * R(w.n->primary_spec_Z[j]);
  for (int i = 0; i < w.Nc; ++i) I = I + c.sec_molal[i] * R(w.n->eqcplx_Z[i]) * R(w.n->eqcplx_Z[i]);
  return R(0.5) * I;
}

template <class R>
void load_cell(const Net &w, const pfchem_cells *cl, int64_t k, Cell<R> &c) {
  const int64_t n = cl->ncells;
  std::memset(&c, 0, sizeof(c));
  c.temp = cl->temperature[k];
  c.sat = cl->saturation[k];
  c.den_kg = cl->den_kg[k];
  c.porosity = cl->porosity[k];
  c.volume = cl->volume[k];
  c.soil_particle_density = cl->soil_particle_density ? cl->soil_particle_density[k] : 0.0;
  for (int j = 0; j < w.N; ++j) {
    c.pri_molal[j] = cl->pri_molal[j * n + k];
    c.pri_act_coef[j] = 1;
    c.total_sorb_eq[j] = cl->total_sorb_eq ? cl->total_sorb_eq[j * n + k] : 0.0;
  }
  for (int i = 0; i < w.Nc; ++i) c.sec_act_coef[i] = 1;
  for (int m = 0; m < w.Nm; ++m) {
    c.mnrl_volfrac[m] = cl->mnrl_volfrac[m * n + k];
    c.mnrl_area[m] = cl->mnrl_area[m * n + k];
  }
  for (int r = 0; r < w.Nix; ++r) c.eqionx_ref_cation_sorbed_conc[r] = cl->eqionx_ref_cation_sorbed_conc[r * n + k];
  for (int r = 0; r < w.Nsr; ++r) c.srfcplxrxn_free_site_conc[r] = cl->srfcplxrxn_free_site_conc[r * n + k];
  c.ln_act_h2o = cl->ln_act_h2o ? cl->ln_act_h2o[k] : 0.0;
}

template <class R>
void react_one(const Net &w, const pfchem_options &o, double dt, pfchem_cells *cl, int64_t k) {
  const int64_t n = cl->ncells;
  if (cl->active && cl->active[k] <= 0) {
    if (cl->status) cl->status[k] = PFCHEM_CELL_INACTIVE;
    if (cl->iterations) cl->iterations[k] = 0;
    return;
  }
  Cell<R> c;
  load_cell(w, cl, k, c);
  R tran[P];
  for (int j = 0; j < w.N; ++j) tran[j] = cl->total[j * n + k];
  int iters = 0;
  double alt[P];
  if (cl->alt_guess)
    for (int j = 0; j < w.N; ++j) alt[j] = cl->alt_guess[j * n + k];
  int status = rreact(w, o, c, tran, R(dt), R(cl->ionic_strength[k]), &iters, cl->alt_guess ? alt : nullptr);
  if (status == PFCHEM_CELL_CONVERGED && o.update_kinetic_state) update_kinetic_state(w, c, R(dt));
  for (int j = 0; j < w.N; ++j) {
    cl->pri_molal[j * n + k] = (double)c.pri_molal[j];
    if (cl->total_out) cl->total_out[j * n + k] = (double)c.total[j];
    if (cl->total_sorb_eq) cl->total_sorb_eq[j * n + k] = (double)c.total_sorb_eq[j];
  }
  for (int m = 0; m < w.Nm; ++m) {
    cl->mnrl_volfrac[m * n + k] = (double)c.mnrl_volfrac[m];
    if (cl->mnrl_rate) cl->mnrl_rate[m * n + k] = (double)c.mnrl_rate[m];
  }
  for (int i = 0; i < w.Nc; ++i)
    if (cl->sec_molal) cl->sec_molal[i * n + k] = (double)c.sec_molal[i];
  for (int r = 0; r < w.Nix; ++r) cl->eqionx_ref_cation_sorbed_conc[r * n + k] = (double)c.eqionx_ref_cation_sorbed_conc[r];
  for (int r = 0; r < w.Nsr; ++r) cl->srfcplxrxn_free_site_conc[r * n + k] = (double)c.srfcplxrxn_free_site_conc[r];
  cl->ionic_strength[k] = (double)ionic_strength_of(w, c);
  if (cl->ln_act_h2o) {
    // the value RActivityCoefficients would compute at the solution (reaction.F90:4043-4050)
    if (o.use_activity_h2o) {
      R s = 0;
      for (int j = 0; j < w.N; ++j) s += c.pri_molal[j];
      for (int i = 0; i < w.Nc; ++i) s += c.sec_molal[i];
      R v = R(1) - R(0.017) * s;
      c.ln_act_h2o = v > 0 ? rlog(v) : R(0);
    }
    cl->ln_act_h2o[k] = (double)c.ln_act_h2o;
  }
  if (cl->iterations) cl->iterations[k] = iters;
  if (cl->status) cl->status[k] = status;
}

Net make_net(const pfchem_network *n, const pfchem_options *o = nullptr) {
  Net w;
  w.exact_jac = o && o->jacobian == PFCHEM_JACOBIAN_EXACT;
  w.n = n;
  w.N = n->naqcomp;
  w.Nc = n->neqcplx;
  w.Nm = n->nkinmnrl;
  w.Nix = n->neqionxrxn;
  w.Nsr = n->nsrfcplxrxn;
  w.Nsc = n->nsrfcplx;
  return w;
}

}  // namespace

extern "C" {

// Runs the restated RReact on every cell of `cells` (host pointers) with
// `nthreads` std::threads over static contiguous chunks.  precision 0 =
// double, 1 = long double.  Returns the number of non-converged cells.
int pfo_react_batch(const pfchem_network *net, const pfchem_options *opt, double dt, pfchem_cells *cells,
                    int precision, int nthreads) {
  Net w = make_net(net, opt);
  if (w.N > P || w.Nc > C || w.Nm > M || w.Nix > IX || w.Nsr > SR || w.Nsc > SC) return -1;
  const int64_t n = cells->ncells;
  if (nthreads < 1) nthreads = 1;
  std::vector<std::thread> pool;
  for (int t = 0; t < nthreads; ++t) {
    pool.emplace_back([&, t]() {
      int64_t lo = n * t / nthreads, hi = n * (t + 1) / nthreads;
      for (int64_t k = lo; k < hi; ++k) {
        if (precision == 1)
          react_one<long double>(w, *opt, dt, cells, k);
        else
          react_one<double>(w, *opt, dt, cells, k);
      }
    });
  }
  for (auto &th : pool) th.join();
  int bad = 0;
  if (cells->status)
    for (int64_t k = 0; k < n; ++k)
      if (cells->status[k] != PFCHEM_CELL_CONVERGED && cells->status[k] != PFCHEM_CELL_INACTIVE) ++bad;
  return bad;
}

// Speciation of given free-ion molalities: RTotal (+ RTotalSorb) at `pri_molal`
// with activity coefficients from the LAG formula at ionic strength I
// (freq != OFF) or unity.  Used by the input generators and the KATs.
// Writes total (mol/L), sec_molal, total_sorb_eq, sorption warm starts and
// the self-consistent ionic strength of the speciated state.
// RReact's Newton system for cell k of `cells` at free-ion molalities m:
// residual F (mol/s) and Jacobian J[i*N + j] = dF_i/dm_j as RReact forms
// them, after the step's activity update at the cell's ionic strength.  Test
// support for finite-difference checks of the Jacobian.
int pfo_newton_system(const pfchem_network *net, const pfchem_options *opt, double dt, const pfchem_cells *cells,
                      int64_t k, const double *m, double *F, double *Jout) {
  Net w = make_net(net, opt);
  const pfchem_options &o = *opt;
  Cell<double> c;
  load_cell(w, cells, k, c);
  const int N = w.N;
  const int64_t n = cells->ncells;
  for (int j = 0; j < N; ++j) c.total[j] = cells->total[j * n + k];
  update_temp_dependent_coefs(w, o, c);
  const double psv_t = c.porosity * c.sat * 1000.0 * c.volume;
  double fixed_accum[P];
  for (int j = 0; j < N; ++j) fixed_accum[j] = psv_t * c.total[j];
  if (w.Nix + w.Nsr > 0)
    for (int j = 0; j < N; ++j) fixed_accum[j] += c.total_sorb_eq[j] * c.volume;
  if (o.act_coef_update_frequency != PFCHEM_ACT_COEF_FREQUENCY_OFF) {
    if (activity_coefficients(w, o, c, true, cells->ionic_strength[k])) return 1;
  }
  for (int j = 0; j < N; ++j) c.pri_molal[j] = m[j];
  double res[P], J[P][P];
  if (newton_system(w, o, c, fixed_accum, psv_t, dt, res, J)) return 1;
  for (int i = 0; i < N; ++i) {
    F[i] = res[i];
    for (int j = 0; j < N; ++j) Jout[i * N + j] = J[i][j];
  }
  return 0;
}

// Global-implicit per-cell blocks (RTResidual/RTJacobian reaction terms,
// reactive_transport.F90:2729-2760, :3440-3468): RTAuxVarCompute at the
// cell's pri_molal (totals, sorbed totals and their derivatives,
// reaction.F90:4969-5068) and RReaction with analytical derivative
// (reaction.F90:3515-3584, 3588-3616), log K at the cell temperature, LAG
// activity coefficients at the cell's ionic strength.  Blocks are
// column-major per cell (Fortran Jac(ncomp,ncomp)).
int pfo_reaction_blocks(const pfchem_network *net, const pfchem_options *opt, pfchem_cells *cells,
                        pfchem_reaction_blocks_out *out) {
  Net w = make_net(net, opt);
  const pfchem_options &o = *opt;
  const int N = w.N;
  const int64_t n = cells->ncells, NN = (int64_t)N * N;
  for (int64_t k = 0; k < n; ++k) {
    if (cells->active && cells->active[k] <= 0) {
      for (int j = 0; j < N; ++j) {
        out->res[j * n + k] = 0.0;
        if (out->total) out->total[j * n + k] = 0.0;
        if (out->total_sorb) out->total_sorb[j * n + k] = 0.0;
      }
      for (int64_t q = 0; q < NN; ++q) {
        out->jac[k * NN + q] = 0.0;
        if (out->dtotal) out->dtotal[k * NN + q] = 0.0;
        if (out->dtotal_sorb) out->dtotal_sorb[k * NN + q] = 0.0;
      }
      if (cells->status) cells->status[k] = PFCHEM_CELL_INACTIVE;
      continue;
    }
    Cell<double> c;
    load_cell(w, cells, k, c);
    update_temp_dependent_coefs(w, o, c);
    if (o.act_coef_update_frequency != PFCHEM_ACT_COEF_FREQUENCY_OFF)
      activity_coefficients(w, o, c, true, cells->ionic_strength[k]);
    int status = auxvar_compute(w, c) ? PFCHEM_CELL_INNER_MAXITER : PFCHEM_CELL_CONVERGED;
    double Res[P], Jac[P][P];
    for (int i = 0; i < N; ++i) {
      Res[i] = 0.0;
      for (int j = 0; j < N; ++j) Jac[i][j] = 0.0;
    }
    if (w.Nm > 0) kinetic_mineral(w, c, Res, Jac, true);
    const bool sorb = w.Nix + w.Nsr > 0;
    for (int i = 0; i < N; ++i) {
      out->res[i * n + k] = Res[i];
      if (out->total) out->total[i * n + k] = c.total[i];
      if (out->total_sorb) out->total_sorb[i * n + k] = sorb ? c.total_sorb_eq[i] : 0.0;
      for (int j = 0; j < N; ++j) {
        out->jac[k * NN + j * N + i] = Jac[i][j];
        if (out->dtotal) out->dtotal[k * NN + j * N + i] = c.dtotal[i][j];
        if (out->dtotal_sorb) out->dtotal_sorb[k * NN + j * N + i] = sorb ? c.dtotal_sorb_eq[i][j] : 0.0;
      }
    }
    for (int m = 0; m < w.Nm; ++m)
      if (cells->mnrl_rate) cells->mnrl_rate[m * n + k] = c.mnrl_rate[m];
    for (int i = 0; i < w.Nc; ++i)
      if (cells->sec_molal) cells->sec_molal[i * n + k] = c.sec_molal[i];
    for (int r = 0; r < w.Nix; ++r) cells->eqionx_ref_cation_sorbed_conc[r * n + k] = c.eqionx_ref_cation_sorbed_conc[r];
    for (int r = 0; r < w.Nsr; ++r) cells->srfcplxrxn_free_site_conc[r * n + k] = c.srfcplxrxn_free_site_conc[r];
    if (cells->status) cells->status[k] = status;
  }
  return 0;
}

// realization_subsurface.F90:1686-1735 (mineral surface area) and
// :1946-2001 (RealizationCalcMineralPorosity), over all cells.
int pfo_update_mineral_properties(const pfchem_network *net, pfchem_cells *cells, const pfchem_mineral_update *mu) {
  const int Nm = net->nkinmnrl;
  const int64_t n = cells->ncells;
  int armor_flag = mu->armor_flag;  // reaction%update_armor_mineral_surface_flag
  for (int64_t k = 0; k < n; ++k) {
    double por = cells->porosity[k];
    if (mu->update_porosity && Nm > 0) {
      double sum_volfrac = 0.0;
      for (int m = 0; m < Nm; ++m) sum_volfrac = sum_volfrac + cells->mnrl_volfrac[m * n + k];
      por = std::max(1.0 - sum_volfrac, mu->minimum_porosity);
      mu->porosity[k] = por;
    }
    if (!mu->update_surface_area) continue;
    for (int m = 0; m < Nm; ++m) {
      double porosity_scale = 1.0;
      if (mu->surface_area_with_porosity)
        porosity_scale = std::pow(por / mu->porosity0[k], mu->surf_area_porosity_pwr[m]);
      double volfrac_scale = 1.0;
      if (mu->mnrl_volfrac0[m * n + k] > 0.0)
        volfrac_scale = std::pow(cells->mnrl_volfrac[m * n + k] / mu->mnrl_volfrac0[m * n + k],
                                 mu->surf_area_vol_frac_pwr[m]);
      cells->mnrl_area[m * n + k] = mu->mnrl_area0[m * n + k] * porosity_scale * volfrac_scale;
      // realization_subsurface.F90:1737-1765 mineral armoring, with the flag
      // carried from item to item in loop order
      if (mu->armor_crit_vol_frac && mu->armor_crit_vol_frac[m] > 0.0) {
        const int ma = mu->armor_mineral ? mu->armor_mineral[m] - 1 : m;
        const double crit = mu->armor_crit_vol_frac[m];
        const double vfa = cells->mnrl_volfrac[ma * n + k];
        if (crit > vfa) {
          if (armor_flag == 0)
            cells->mnrl_area[m * n + k] =
                cells->mnrl_area[m * n + k] * std::pow((crit - vfa) / crit, mu->surf_area_vol_frac_pwr[m]);
          else {
            cells->mnrl_area[m * n + k] = mu->mnrl_area0[m * n + k];
            armor_flag = 0;
          }
        } else {
          cells->mnrl_area[m * n + k] = 0.0;
          armor_flag = 1;
        }
      }
    }
  }
  if (mu->armor_flag_out) *mu->armor_flag_out = armor_flag;
  return 0;
}

int pfo_speciate(const pfchem_network *net, const pfchem_options *opt, pfchem_cells *cells) {
  Net w = make_net(net, opt);
  const int64_t n = cells->ncells;
  for (int64_t k = 0; k < n; ++k) {
    Cell<double> c;
    load_cell(w, cells, k, c);
    update_temp_dependent_coefs(w, *opt, c);
    if (opt->act_coef_update_frequency != PFCHEM_ACT_COEF_FREQUENCY_OFF)
      activity_coefficients(w, *opt, c, true, cells->ionic_strength[k]);
    int f = auxvar_compute(w, c);
    for (int j = 0; j < w.N; ++j) {
      if (cells->total_out) cells->total_out[j * n + k] = c.total[j];
      if (cells->total_sorb_eq) cells->total_sorb_eq[j * n + k] = c.total_sorb_eq[j];
    }
    for (int i = 0; i < w.Nc; ++i)
      if (cells->sec_molal) cells->sec_molal[i * n + k] = c.sec_molal[i];
    for (int r = 0; r < w.Nix; ++r) cells->eqionx_ref_cation_sorbed_conc[r * n + k] = c.eqionx_ref_cation_sorbed_conc[r];
    for (int r = 0; r < w.Nsr; ++r) cells->srfcplxrxn_free_site_conc[r * n + k] = c.srfcplxrxn_free_site_conc[r];
    cells->ionic_strength[k] = ionic_strength_of(w, c);
    if (cells->status) cells->status[k] = f ? PFCHEM_CELL_INNER_MAXITER : PFCHEM_CELL_CONVERGED;
  }
  return 0;
}

// Activity coefficients (LAG) at ionic strength I, for KAT outputs (pH).
int pfo_activity_lag(const pfchem_network *net, double I, double *pri_act_coef, double *sec_act_coef) {
  Net w = make_net(net);
  pfchem_options o;
  std::memset(&o, 0, sizeof(o));
  o.act_coef_update_algorithm = PFCHEM_ACT_COEF_ALGORITHM_LAG;
  Cell<double> c;
  std::memset(&c, 0, sizeof(c));
  activity_coefficients(w, o, c, true, I);
  for (int j = 0; j < w.N; ++j) pri_act_coef[j] = c.pri_act_coef[j];
  for (int i = 0; i < w.Nc; ++i) sec_act_coef[i] = c.sec_act_coef[i];
  return 0;
}

// Dense-LU restatement exposed for unit tests: solves RSolve(res, jac) for
// one system (jac row-major N x N, modified in place).  Returns 1 if singular.
int pfo_rsolve(int N, double *res, double *jac, const double *conc, int use_log, double *update) {
  double J[P][P], r[P], u[P];
  for (int i = 0; i < N; ++i) {
    r[i] = res[i];
    for (int j = 0; j < N; ++j) J[i][j] = jac[i * N + j];
  }
  int s = rsolve(r, J, conc, u, N, use_log != 0);
  for (int i = 0; i < N; ++i) update[i] = u[i];
  return s;
}

// reaction_aux.F90:1336-1408 ReactionFitLogKCoef: least-squares fit of the
// 5 Maier-Kelly coefficients to a database log K row (500 = missing point),
// solved with the restated ludcmp/lubksb.
int pfo_fit_logK(int ntemp, const double *temps, const double *logK, double *coefs) {
  double vec[5][16];
  int use[16];
  if (ntemp > 16) return -1;
  for (int i = 0; i < ntemp; ++i) {
    double tk = temps[i] + 273.15;
    vec[0][i] = std::log(tk);
    vec[1][i] = 1.0;
    vec[2][i] = tk;
    vec[3][i] = 1.0 / tk;
    vec[4][i] = 1.0 / (tk * tk);
  }
  double b[P];
  for (int j = 0; j < 5; ++j) {
    b[j] = 0;
    for (int i = 0; i < ntemp; ++i) {
      if (std::fabs(logK[i] - 500.) < 1e-10) {
        use[i] = 0;
      } else {
        b[j] = b[j] + vec[j][i] * logK[i];
        use[i] = 1;
      }
    }
  }
  double a[P][P];
  for (int j = 0; j < 5; ++j)
    for (int k = j; k < 5; ++k) {
      a[j][k] = 0;
      for (int i = 0; i < ntemp; ++i)
        if (use[i]) a[j][k] = a[j][k] + vec[j][i] * vec[k][i];
      if (j != k) a[k][j] = a[j][k];
    }
  int indx[P];
  if (ludcmp(a, 5, indx)) return 1;
  lubksb(a, 5, indx, b);
  for (int j = 0; j < 5; ++j) coefs[j] = b[j];
  return 0;
}

double pfo_interpolate_logK(const double *coefs, double temp) { return interpolate_logK<double>(coefs, temp); }

}  // extern "C"

extern "C" {
// Liquid-water density of the 1967 IFC formulation (region 1), as
// src/pflotran/eos_water.F90:876-1011 EOSWaterDensityIFC67 evaluates it
// (the default EOS, eos_water.F90:240).  t [C], p [Pa] -> kg/m^3.  Used for
// the known-answer tests: transport-only runs take den_kg from it at the
// reference state (factory_subsurface.F90:995-1000, init_subsurface_transport.F90:50).
double pfo_ifc67_density(double t, double p) {
  // IFC-67 region-1 coefficients (published standard; the reference's aa(0:22), a1..a12)
  static const double aa[23] = {6.824687741e03, -5.422063673e02, -2.096666205e04, 3.941286787e04,
                                -6.733277739e04, 9.902381028e04, -1.093911774e05, 8.590841667e04,
                                -4.511168742e04, 1.418138926e04, -2.017271113e03, 7.982692717e00,
                                -2.616571843e-2, 1.522411790e-3, 2.284279054e-2, 2.421647003e02,
                                1.269716088e-10, 2.074838328e-7, 2.174020350e-8, 1.105710498e-9,
                                1.293441934e01, 1.308119072e-5, 6.047626338e-14};
  const double a1 = 8.438375405e-1, a2 = 5.362162162e-4, a3 = 1.720000000e00, a4 = 7.342278489e-2;
  const double a5 = 4.975858870e-2, a6 = 6.537154300e-1, a7 = 1.150000000e-6, a8 = 1.510800000e-5;
  const double a9 = 1.418800000e-1, a10 = 7.002753165e00, a11 = 2.995284926e-4, a12 = 2.040000000e-1;
  const double tc1 = 647.3, pc1 = 22.064e6, vc1 = 0.00317;  // pflotran_constants.F90 critical point
  const double theta = (t + 273.15) * (1.0 / tc1);
  const double theta2x = theta * theta;
  const double theta18 = std::pow(theta, 18.0);
  const double theta20 = theta18 * theta2x;
  const double beta = p * (1.0 / pc1);
  const double beta2x = beta * beta;
  const double yy = 1.0 - a1 * theta2x - a2 * std::pow(theta, -6.0);
  double xx = a3 * yy * yy - 2.0 * (a4 * theta - a5 * beta);
  xx = xx > 0 ? std::sqrt(xx) : 1e-6;
  const double zz = yy + xx;
  const double u0 = -5.0 / 17.0;
  const double u1 = aa[11] * a5 * std::pow(zz, u0);
  const double u2 = 1.0 / (a8 + std::pow(theta, 11.0));
  const double u3 = aa[17] + (2.0 * aa[18] + 3.0 * aa[19] * beta) * beta;
  const double u4 = 1.0 / (a7 + theta18 * theta);
  const double u5 = std::pow(a10 + beta, -4.0);
  const double u6 = a11 - 3.0 * u5;
  const double u7 = aa[20] * theta18 * (a9 + theta2x);
  const double u8 = aa[15] * std::pow(a6 - theta, 9.0);
  const double vr = u1 + aa[12] + theta * (aa[13] + aa[14] * theta) + u8 * (a6 - theta) + aa[16] * u4 - u2 * u3 -
                    u6 * u7 + (3.0 * aa[21] * (a12 - theta) + 4.0 * aa[22] * beta / theta20) * beta2x;
  return 1.0 / (vr * vc1);
}
}

namespace {
// Constraint row types of ReactionEquilibrateConstraint (reaction_aux.F90 CONSTRAINT_*)
enum { kConTotal = 1, kConFree = 2, kConChargeBal = 3, kConPH = 4, kConLog = 5, kConMineral = 6, kConGas = 7,
       kConTotalSorb = 8 };

// reaction.F90:1308-2046 ReactionEquilibrateConstraint with TOTAL [mol/L],
// FREE [mol/L], LOG (log10 free [mol/L]), CHARGE_BAL, pH (H+ as a primary
// species), MINERAL, GAS and TOTAL_SORB rows (no supercritical-CO2 or colloid
// rows); a MINERAL row holds the reaction of kinetic mineral `mineral[i]`
// (1-based) at equilibrium, a GAS row the reaction of passive gas
// `mineral[i]` of `gas`'s tables at partial pressure conc[i] [bar]
// (reaction.F90:1720-1751), a TOTAL_SORB row the sorbed total conc[i]
// [mol/m^3 bulk] (:1608-1614).  Starts from free ions 1e-9 (reaction.F90:1481), alternates
// log/linear updates for iterations 4-8 (:1841-1852) and switches activity
// coefficients on after the first convergence (:1954-1966).  Returns 0,
// 1 (iteration cap), 2 (singular), 3 (non-positive molality, :1876-1894).
template <class R>
int equilibrate_constraint(const Net &w, const pfchem_options &o, Cell<R> &c, const int *type,
                           const double *conc_in, int *iters_out, const int *mineral = nullptr, int max_its = 10000,
                           const pfchem_constraint *gas = nullptr) {
  const int N = w.N;
  const pfchem_network &n = *w.n;
  R convert_molar_to_molal = R(1000) / c.den_kg;
  R total_conc[P], free_conc[P], gas_logK[P];
  double conc[P];
  for (int i = 0; i < N; ++i) {
    conc[i] = conc_in[i];
    free_conc[i] = R(1e-9);
    total_conc[i] = 0;
    if (type[i] == kConTotal || type[i] == kConTotalSorb) total_conc[i] = R(conc[i]);
    else if (type[i] == kConGas) {
      if (conc[i] <= 0.0) conc[i] = std::pow(10.0, conc[i]);  // log10 partial pressure (:1531-1535)
      const int g = mineral[i] - 1;
      gas_logK[i] = o.use_isothermal ? R(gas->paseqlogK[g]) : interpolate_logK(gas->paseqlogKcoef + 5 * g, c.temp);
    } else if (type[i] == kConFree || type[i] == kConChargeBal || type[i] == kConMineral)
      free_conc[i] = R(conc[i]) * convert_molar_to_molal;
    else if (type[i] == kConLog) free_conc[i] = std::pow(R(10), R(conc[i])) * convert_molar_to_molal;
    else if (type[i] == kConPH) free_conc[i] = std::pow(R(10), -R(conc[i]));
  }
  for (int i = 0; i < N; ++i) c.pri_molal[i] = free_conc[i];
  for (int i = 0; i < N; ++i) c.pri_act_coef[i] = 1;
  for (int i = 0; i < w.Nc; ++i) {
    c.sec_act_coef[i] = 1;
    c.sec_molal[i] = 0;
  }
  int num_iterations = 0, num_it_act_coef_turned_on = 0;
  bool compute_activity_coefs = false;
  R Res[P], Jac[P][P], update[P], prev[P];
  for (;;) {
    for (int i = 0; i < N; ++i)
      if (type[i] == kConFree || type[i] == kConLog) c.pri_molal[i] = free_conc[i];
    if (o.act_coef_update_frequency != PFCHEM_ACT_COEF_FREQUENCY_OFF && compute_activity_coefs)
      activity_coefficients(w, o, c, false, R(0));
    rtotal(w, c);
    if (w.Nix + w.Nsr > 0) total_sorb(w, c);
    for (int i = 0; i < N; ++i) {
      for (int j = 0; j < N; ++j) Jac[i][j] = 0;
      if (type[i] == kConTotal) {
        Res[i] = c.total[i] - total_conc[i];
        for (int j = 0; j < N; ++j) Jac[i][j] = c.dtotal[i][j];
      } else if (type[i] == kConFree || type[i] == kConLog) {
        Res[i] = 0;
        Jac[i][i] = 1;
      } else if (type[i] == kConPH) {  // reaction.F90:1653-1661 (H+ primary)
        Res[i] = 0;
        c.pri_molal[i] = std::pow(R(10), -R(conc[i])) / c.pri_act_coef[i];
        Jac[i][i] = 1;
      } else if (type[i] == kConMineral) {  // reaction.F90:1694-1717
        const int m = mineral[i] - 1;
        R lnQK = -c.kinmnrl_logK[m] * R(kLOG_TO_LN);
        if (n.kinmnrlh2oid && n.kinmnrlh2oid[m] > 0) lnQK = lnQK + R(n.kinmnrlh2ostoich[m]) * c.ln_act_h2o;
        for (int k = 1; k <= w.mn(m); ++k) {
          const int j = w.mid(m, k);
          lnQK = lnQK + R(w.mnu(m, k)) * rlog(c.pri_molal[j] * c.pri_act_coef[j]);
        }
        Res[i] = lnQK;
        for (int k = 1; k <= w.mn(m); ++k) {
          const int j = w.mid(m, k);
          Jac[i][j] = R(w.mnu(m, k)) / c.pri_molal[j];
        }
      } else if (type[i] == kConGas) {  // reaction.F90:1720-1751
        const int g = mineral[i] - 1, ld = gas->paseq_ld;
        R lnQK = -gas_logK[i] * R(kLOG_TO_LN);
        if (gas->paseqh2oid && gas->paseqh2oid[g] > 0) lnQK = lnQK + R(gas->paseqh2ostoich[g]) * c.ln_act_h2o;
        const int ns = gas->paseqspecid[g * (ld + 1)];
        for (int k = 1; k <= ns; ++k) {
          const int j = gas->paseqspecid[g * (ld + 1) + k] - 1;
          lnQK = lnQK + R(gas->paseqstoich[g * ld + k - 1]) * rlog(c.pri_molal[j] * c.pri_act_coef[j]);
        }
        Res[i] = lnQK - rlog(R(conc[i]));
        for (int k = 1; k <= ns; ++k) {
          const int j = gas->paseqspecid[g * (ld + 1) + k] - 1;
          Jac[i][j] = R(gas->paseqstoich[g * ld + k - 1]) / c.pri_molal[j];
        }
      } else if (type[i] == kConTotalSorb) {  // reaction.F90:1608-1614
        Res[i] = c.total_sorb_eq[i] - total_conc[i];
        for (int j = 0; j < N; ++j) Jac[i][j] = c.dtotal_sorb_eq[i][j];
      } else {  // charge balance (reaction.F90:1623-1634)
        Res[i] = 0;
        for (int j = 0; j < N; ++j) {
          Res[i] = Res[i] + R(n.primary_spec_Z[j]) * c.total[j];
          for (int k = 0; k < N; ++k) Jac[i][j] = Jac[i][j] + R(n.primary_spec_Z[k]) * c.dtotal[k][j];
        }
      }
    }
    R maximum_residual = 0;
    for (int i = 0; i < N; ++i) maximum_residual = std::max(maximum_residual, std::fabs(Res[i]));
    bool use_log;
    if (o.use_log_formulation) {
      if (num_iterations > 3 && num_iterations < 9) use_log = (num_iterations % 2 == 0);
      else use_log = true;
    } else {
      use_log = false;
    }
    if (rsolve(Res, Jac, c.pri_molal, update, N, use_log)) return 2;
    for (int i = 0; i < N; ++i) prev[i] = c.pri_molal[i];
    if (use_log) {
      for (int i = 0; i < N; ++i) {
        R s = std::signbit((double)update[i]) ? R(-1) : R(1);
        update[i] = s * std::min(std::fabs(update[i]), R(o.max_dlnC));
        c.pri_molal[i] = c.pri_molal[i] * rexp(-update[i]);
      }
    } else {
      R min_ratio = R(1e20);
      for (int i = 0; i < N; ++i)
        if (prev[i] <= update[i]) {
          R ratio = std::fabs(prev[i] / update[i]);
          if (ratio < min_ratio) min_ratio = ratio;
        }
      if (min_ratio <= R(1))
        for (int i = 0; i < N; ++i) update[i] = update[i] * min_ratio * R(0.99);
      for (int i = 0; i < N; ++i) c.pri_molal[i] = prev[i] - update[i];
    }
    for (int i = 0; i < N; ++i)
      if (!(c.pri_molal[i] > 0)) return 3;
    R mrc = 0;
    for (int i = 0; i < N; ++i) mrc = std::max(mrc, std::fabs((c.pri_molal[i] - prev[i]) / prev[i]));
    ++num_iterations;
    if (num_iterations >= max_its) return 1;
    if (maximum_residual < R(o.max_residual_tolerance) && mrc < R(o.max_relative_change_tolerance)) {
      if (compute_activity_coefs && num_iterations - num_it_act_coef_turned_on > 1) break;
      if (!compute_activity_coefs) num_it_act_coef_turned_on = num_iterations;
      compute_activity_coefs = true;
    }
  }
  // The next time step starts from RTAuxVarCompute at the final free ions
  // with the last activity coefficients (RTUpdateFixedAccumulation,
  // reactive_transport.F90:726-790), before any activity update.
  rtotal(w, c);
  if (w.Nix + w.Nsr > 0) total_sorb(w, c);
  *iters_out = num_iterations;
  return 0;
}
}  // namespace

extern "C" {
// Constraint speciation of every cell of `cells` (host pointers): one
// constraint row per component (types and mineral ids shared by the batch,
// values per cell), `nthreads` std::threads.  Writes what the single-cell
// entry below writes, plus iterations and status (0 converged, 1 cap,
// 2 singular, 3 non-positive molality).  Returns the number of failed cells.
int pfo_equilibrate_constraints(const pfchem_network *net, const pfchem_options *opt, pfchem_cells *cells,
                                const pfchem_constraint *con, int nthreads) {
  Net w = make_net(net, opt);
  for (int j = 0; j < w.N; ++j)
    if (con->type[j] == kConGas &&
        (!con->mineral || con->mineral[j] < 1 || con->mineral[j] > con->npassive_gas || !con->paseqspecid ||
         !con->paseqstoich || (opt->use_isothermal ? !con->paseqlogK : !con->paseqlogKcoef)))
      return -1;
  const int64_t n = cells->ncells;
  std::atomic<int> bad{0};
  auto work = [&](int64_t k0, int64_t k1) {
    for (int64_t k = k0; k < k1; ++k) {
      Cell<double> c;
      load_cell(w, cells, k, c);
      update_temp_dependent_coefs(w, *opt, c);
      double conc[P];
      for (int j = 0; j < w.N; ++j) conc[j] = con->value[j * n + k];
      int its = 0;
      const int r = equilibrate_constraint(w, *opt, c, con->type, conc, &its, con->mineral,
                                           con->max_iterations > 0 ? con->max_iterations : 10000, con);
      if (r) bad++;
      for (int j = 0; j < w.N; ++j) {
        cells->pri_molal[j * n + k] = c.pri_molal[j];
        if (cells->total_out) cells->total_out[j * n + k] = c.total[j];
        if (cells->total_sorb_eq) cells->total_sorb_eq[j * n + k] = c.total_sorb_eq[j];
      }
      for (int i = 0; i < w.Nc; ++i)
        if (cells->sec_molal) cells->sec_molal[i * n + k] = c.sec_molal[i];
      for (int q = 0; q < w.Nix; ++q) cells->eqionx_ref_cation_sorbed_conc[q * n + k] = c.eqionx_ref_cation_sorbed_conc[q];
      for (int q = 0; q < w.Nsr; ++q) cells->srfcplxrxn_free_site_conc[q * n + k] = c.srfcplxrxn_free_site_conc[q];
      cells->ionic_strength[k] = ionic_strength_of(w, c);
      if (cells->iterations) cells->iterations[k] = its;
      if (cells->status) cells->status[k] = r;
    }
  };
  if (nthreads < 1) nthreads = 1;
  std::vector<std::thread> pool;
  const int64_t chunk = (n + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; ++t) {
    const int64_t k0 = t * chunk, k1 = std::min(n, k0 + chunk);
    if (k0 < k1) pool.emplace_back(work, k0, k1);
  }
  for (auto &th : pool) th.join();
  return bad.load();
}

// Constraint speciation of one cell given as a 1-cell batch (host pointers).
// type[i]: 1 TOTAL [mol/L], 2 FREE [mol/L], 3 CHARGE_BAL (conc = guess),
// 4 pH, 5 log10 FREE [mol/L] (no mineral rows: those need the batch entry).
// Writes pri_molal, total_out, sec_molal, sorption state and the ionic
// strength (at the final state, recomputed as the next LAG update would).
int pfo_equilibrate_constraint(const pfchem_network *net, const pfchem_options *opt, pfchem_cells *cells,
                               const int *type, const double *conc, int *iters) {
  Net w = make_net(net, opt);
  for (int j = 0; j < w.N; ++j)
    if (type[j] < kConTotal || type[j] >= kConMineral) return -1;  // mineral rows need the batch entry
  Cell<double> c;
  load_cell(w, cells, 0, c);
  update_temp_dependent_coefs(w, *opt, c);
  int r = equilibrate_constraint(w, *opt, c, type, conc, iters);
  const int64_t n = cells->ncells;
  for (int j = 0; j < w.N; ++j) {
    cells->pri_molal[j * n] = c.pri_molal[j];
    if (cells->total_out) cells->total_out[j * n] = c.total[j];
    if (cells->total_sorb_eq) cells->total_sorb_eq[j * n] = c.total_sorb_eq[j];
  }
  for (int i = 0; i < w.Nc; ++i)
    if (cells->sec_molal) cells->sec_molal[i * n] = c.sec_molal[i];
  for (int q = 0; q < w.Nix; ++q) cells->eqionx_ref_cation_sorbed_conc[q * n] = c.eqionx_ref_cation_sorbed_conc[q];
  for (int q = 0; q < w.Nsr; ++q) cells->srfcplxrxn_free_site_conc[q * n] = c.srfcplxrxn_free_site_conc[q];
  cells->ionic_strength[0] = ionic_strength_of(w, c);
  return r;
}
}
