// pfchem_newton.cu -- batched per-cell Newton solve of the operator-split
// reaction step on sm_103a (FP64).
//
// Replaces, for all cells of a batch at once, PFLOTRAN's
//   RReact               src/pflotran/reaction.F90:3322-3511
//   RTotal               reaction.F90:4057-4158
//   RActivityCoefficients (LAG) reaction.F90:3992-4051
//   RTotalSorbEqIonx     reaction.F90:4305-4535
//   RTotalSorbEqSurfCplx1 reaction_surf_complex.F90:658-934
//   RTAccumulation(+Derivative), RAccumulationSorb(+Derivative)
//                        reaction.F90:5072-5232, :4539-4603
//   RKineticMineral      reaction_mineral.F90:564-1000 (no rate prefactors)
//   RSolve/ludcmp/lubksb reaction.F90:4835-4880, utility.F90:393-523
//   RUpdateKineticState  reaction.F90:5320-5365
//   log K(T)             reaction_aux.F90:1461-1488
//
// GB300 design.  On this part the FP64 pipe runs at a small fraction of the
// FP32 rate, so the solve is bound by FP64 instruction issue, not by HBM.
// The formulation therefore removes FP64 work the reference repeats:
//  * one cell per thread; a persistent grid pulls cells from a device work
//    counter, and a warp refills its idle lanes together once at least
//    `refill_min_idle` of them have converged, so cells needing 2 iterations
//    do not hold lanes for cells needing 40;
//  * ln m is carried through the iteration (ln m -= clamped update) instead
//    of four log() calls per species per iteration;
//  * the Jacobian is assembled directly with respect to ln m (the columns
//    RSolve would scale by m), which removes every division by m; the row
//    scaling of RSolve is dropped because implicit-scaling pivoting is
//    invariant to it (both only change rounding);
//  * secondary concentrations are exp(lnQK - ln gamma), with ln gamma fixed
//    for the step under TIMESTEP activity updates;
//  * unit free-site stoichiometry surface complexation uses the closed form
//    Sx = site / (1 + sum_k E_k) with one exp per complex;
//  * KDj^(Z_j/Z_ref) uses x*x / sqrt(x) for the ratios 2 and 1/2.
// The Jacobian lives in shared memory (thread-fastest layout, conflict-free);
// the rest of the per-cell state is thread-private.
#include <cuda_runtime.h>
#include <math.h>

#include "pfchem_device.cuh"

namespace pfchem {

template <int NP_, int NCX_, int NMN_, int NIX_, int NSR_, int NSC_>
struct Sizes {
  static constexpr int NP = NP_, NCX = NCX_, NMN = NMN_, NIX = NIX_, NSR = NSR_, NSC = NSC_;
};
using SizesS = Sizes<4, 8, 2, 1, 1, 4>;
using SizesM = Sizes<12, 48, 8, 4, 2, 8>;
using SizesL = Sizes<PFCHEM_MAX_PRI, PFCHEM_MAX_CPLX, PFCHEM_MAX_MNRL, PFCHEM_MAX_IONX, PFCHEM_MAX_SRFRXN,
                     PFCHEM_MAX_SRFCPLX>;

template <class S>
struct Lane {
  // per-cell constants of the step
  double dt, acc, psv_den, jac_aq, vol, v_t, den_L, den_mnrl, temp, por, rho_s, lnaw;
  double jac_mnrl;  // weight of the mineral terms in the Jacobian (1 in the Newton solve)
  // state
  double m[S::NP], lnm[S::NP], lngp[S::NP], gp[S::NP];
  double fixed[S::NP], absfixed[S::NP];
  double bc[S::NCX], bK[S::NCX], C[S::NCX];
  double bm[S::NMN], rk[S::NMN], vf[S::NMN], area[S::NMN], rate[S::NMN];
  double pk[S::NMN][PFCHEM_MAX_PREF];  // prefactor rate constant x Arrhenius factor
  double bs[S::NSC];
  double ixref[S::NIX], srfree[S::NSR];
  double Psi[S::NP], S_[S::NP], F[S::NP], Sc[S::NP];
  double I;
  int iter;
  bool alt_pending, alt_used;
  bool act_fail;  // the NEWTON activity algorithm did not converge at step start
  double r_plain;
};

__device__ __forceinline__ double sgn1(double x) { return signbit(x) ? -1.0 : 1.0; }
PFCHEM_GLOBALTIMER_FN

// LAG activity coefficients at ionic strength I (reaction.F90:3992-4051), as
// ln gamma; complexes fold theirs into bc = bK - ln gamma.
template <class S>
__device__ void activity(const DevNet &n, Lane<S> &L, double I) {
  const double sI = sqrt(I);
  for (int j = 0; j < n.N; ++j) {
    double lg = 0.0;
    if (n.Z2p[j] > 1e-20)
      lg = (-n.Z2p[j] * sI * n.A / (1.0 + n.ap[j] * n.B * sI) + n.Bdot * I) * kLOG_TO_LN;
    L.lngp[j] = lg;
    L.gp[j] = exp(lg);
  }
  for (int i = 0; i < n.Nc; ++i) {
    double lg = 0.0;
    if (n.cZ2[i] > 1e-20)
      lg = (-n.cZ2[i] * sI * n.A / (1.0 + n.ca[i] * n.B * sI) + n.Bdot * I) * kLOG_TO_LN;
    L.bc[i] = L.bK[i] - lg;
  }
}

// ACT_COEF_ALGORITHM_NEWTON (reaction.F90:3846-3990): the ionic strength is
// iterated to a 1e-6 relative change (at most 50 passes) with the primaries'
// ln activities held at their entry values, the complexes recomputed at each
// pass.  `entry` starts from the step's entry state at the library's
// boundary: the primaries' coefficients at the carried ionic strength I0 and
// no complexes (the first pass keeps I = I0).  Otherwise the entry state is
// the lane's current coefficients and complexes (L.C, from the last
// evaluation), as RActivityCoefficients sees them inside the Newton loop.
// Returns 0, or 1 when the 50 passes did not converge.
template <class S>
__device__ int activity_newton(const DevNet &n, Lane<S> &L, bool entry, double I0) {
  const int N = n.N;
  if (entry) {
    activity(n, L, I0);
    for (int i = 0; i < n.Nc; ++i) L.C[i] = 0.0;
  }
  double lna[S::NP], fpri = 0.0;
  for (int j = 0; j < N; ++j) {
    lna[j] = L.lnm[j] + L.lngp[j];
    fpri += L.m[j] * n.Z2p[j];
  }
  double II = 0.0;
  for (int it = 1;; ++it) {
    if (it > 50) return 1;
    double I;
    if (it == 1 && entry) {
      I = I0;
    } else {
      I = fpri;
      for (int i = 0; i < n.Nc; ++i) I += L.C[i] * n.cZ2[i];
      I = 0.5 * I;
    }
    const double f = I;
    if (fabs(I - II) < 1e-6 * I) break;
    if (n.Nc > 0) {
      double didi = 0.0;
      const double sI = sqrt(I);
      for (int i = 0; i < n.Nc; ++i) {
        if (n.cZ2[i] > 0.0) {
          const double t = 1.0 + n.B * n.ca[i] * sI;
          double sum = 0.5 * n.A * n.cZ2[i] / (sI * t * t) - n.Bdot;
          for (int k = 0; k < n.cn[i]; ++k) {
            const int j = n.cid[i][k];
            if (n.Z2p[j] > 0.0) {
              const double tj = 1.0 + n.B * n.ap[j] * sI;
              sum += n.cnu[i][k] * (-0.5 * n.A * n.Z2p[j] / (sI * tj * tj) + n.Bdot);
            }
          }
          didi += 0.5 * n.cZ2[i] * (L.C[i] * kLOG_TO_LN * sum);
        }
      }
      const double den = 1.0 - didi;
      II = fabs(den) > 0.0 ? (f - I * didi) / den : f;
    } else {
      II = f;
    }
    activity(n, L, II);
    for (int i = 0; i < n.Nc; ++i) {
      double s = L.bc[i];
      for (int k = 0; k < n.cn[i]; ++k) s += n.cnu[i][k] * lna[n.cid[i][k]];
      L.C[i] = exp(s);
    }
  }
  return 0;
}

__device__ __forceinline__ double logK_at(const double *c, double lntk, double tk, double itk) {
  return c[0] * lntk + c[1] + c[2] * tk + c[3] * itk + c[4] * (itk * itk);
}

template <class S>
__device__ void setup(const DevNet &n, const CellArgs &a, int64_t cell, Lane<S> &L, double inv_dt) {
  const int64_t nc = a.ncells;
  const double por = a.por[cell], sat = a.sat[cell], vol = a.vol[cell], den = a.den[cell];
  L.temp = a.temp[cell];
  L.por = por;
  L.vol = vol;
  L.rho_s = a.rho_s ? a.rho_s[cell] : 0.0;
  L.dt = a.dt;
  L.acc = (n.accum_mode == PFCHEM_ACCUM_DT_CONSISTENT) ? inv_dt : 1.0;
  const double psv = por * sat * 1000.0 * vol;
  L.den_L = den * 1e-3;
  L.den_mnrl = den * 1e-3;
  L.psv_den = psv * L.den_L;
  L.jac_aq = psv * inv_dt * L.den_L;
  L.v_t = vol * inv_dt;
  L.lnaw = a.lnaw ? a.lnaw[cell] : 0.0;
  L.jac_mnrl = 1.0;
  const bool sorb = (n.Nix + n.Nsr) > 0;
  for (int j = 0; j < n.N; ++j) {
    const double tot = a.total ? a.total[j * a.total_stride_comp + cell * a.total_stride_cell] : 0.0;
    double f = psv * tot;
    if (sorb) f = f + a.sorb[j * nc + cell] * vol;
    L.fixed[j] = L.acc * f;
    L.absfixed[j] = fabs(L.fixed[j]);
    const double m = a.pri_molal[j * nc + cell];
    L.m[j] = m;
    L.lnm[j] = log(m);
  }
  // log K at the cell temperature (RUpdateTempDependentCoefs, reaction.F90:5433-5524)
  double tk = L.temp + 273.15, lntk = 0.0, itk = 0.0;
  if (!n.isothermal) {
    lntk = log(tk);
    itk = 1.0 / tk;
  }
  for (int i = 0; i < n.Nc; ++i) {
    const double lk = n.isothermal ? n.clogK[i] : logK_at(n.ccoef[i], lntk, tk, itk);
    L.bK[i] = -lk * kLOG_TO_LN + n.ch2o[i] * L.lnaw;
  }
  for (int k = 0; k < n.Nm; ++k) {
    const double lk = n.isothermal ? n.mlogK[k] : logK_at(n.mcoef[k], lntk, tk, itk);
    L.bm[k] = -lk * kLOG_TO_LN + n.mh2o[k] * L.lnaw;
    double af = 1.0;  // Arrhenius factor (reaction_mineral.F90:784-792)
    if (n.mEa[k] > 0.0) af = exp(n.mEa[k] / kIDEAL_GAS_CONSTANT * (1.0 / (25.0 + 273.15) - 1.0 / (L.temp + 273.15)));
    L.rk[k] = n.mk[k] * af;
    for (int p = 0; p < n.mpn[k]; ++p) {
      double pf = 1.0;  // the prefactor's own Arrhenius factor (reaction_mineral.F90:771-778)
      if (n.mpEa[k][p] > 0.0)
        pf = exp(n.mpEa[k][p] / kIDEAL_GAS_CONSTANT * (1.0 / (25.0 + 273.15) - 1.0 / (L.temp + 273.15)));
      L.pk[k][p] = n.mpk[k][p] * pf;
    }
    L.vf[k] = a.vf[k * nc + cell];
    L.area[k] = a.area[k * nc + cell];
    L.rate[k] = 0.0;
  }
  for (int k = 0; k < n.Nsc; ++k) {
    const double lk = n.isothermal ? n.slogK[k] : logK_at(n.scoef[k], lntk, tk, itk);
    L.bs[k] = -lk * kLOG_TO_LN + n.sh2o[k] * L.lnaw;
  }
  for (int r = 0; r < n.Nix; ++r) L.ixref[r] = a.ixref[r * nc + cell];
  for (int r = 0; r < n.Nsr; ++r) L.srfree[r] = a.srfree[r * nc + cell];
  L.I = a.ionic[cell];
  L.act_fail = false;
  if (n.act_freq != PFCHEM_ACT_COEF_FREQUENCY_OFF) {
    if (n.act_newton) L.act_fail = activity_newton(n, L, true, L.I) != 0;
    else activity(n, L, L.I);
  } else {
    for (int j = 0; j < n.N; ++j) {
      L.lngp[j] = 0.0;
      L.gp[j] = 1.0;
    }
    for (int i = 0; i < n.Nc; ++i) L.bc[i] = L.bK[i];
  }
  if (!n.act_newton) for (int i = 0; i < n.Nc; ++i) L.C[i] = 0.0;
  L.iter = 0;
  L.alt_pending = false;
  L.alt_used = false;
}

// ln activity of a rate-prefactor species: a primary (id >= 0) or an aqueous
// complex -(id + 1), whose ln activity is its log K term plus sum nu ln a.
template <class S>
__device__ __forceinline__ double pref_lnact(const DevNet &n, const Lane<S> &L, const double *lna, int id) {
  if (id >= 0) return lna[id];
  const int i = -id - 1;
  double s = L.bK[i];
  for (int k = 0; k < n.cn[i]; ++k) s += n.cnu[i][k] * lna[n.cid[i][k]];
  return s;
}

// Residual F (and, with JAC, the Jacobian dF/dln m into J, stride `js`) at
// the lane's current m.  Returns 0, or a non-converged status when an inner
// loop hit its cap.
template <class S, bool JAC>
__device__ int evaluate(const DevNet &n, Lane<S> &L, double *J, int js, bool exact) {
  const int N = n.N;
  double lna[S::NP], absP[S::NP], absS[S::NP];
  for (int j = 0; j < N; ++j) {
    lna[j] = L.lnm[j] + L.lngp[j];
    L.Psi[j] = L.m[j];
    absP[j] = L.m[j];
    L.S_[j] = 0.0;
    absS[j] = 0.0;
  }
  if (JAC) {
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) J[(i * N + j) * js] = (i == j) ? L.m[j] * L.jac_aq : 0.0;
  }
  // aqueous complexes: mass action and totals (RTotal)
  for (int i = 0; i < n.Nc; ++i) {
    const int nz = n.cn[i];
    double s = L.bc[i];
    for (int k = 0; k < nz; ++k) s += n.cnu[i][k] * lna[n.cid[i][k]];
    const double c = exp(s);
    L.C[i] = c;
    const double cj = c * L.jac_aq;
    for (int k = 0; k < nz; ++k) {
      const int j = n.cid[i][k];
      const double nu = n.cnu[i][k];
      L.Psi[j] += nu * c;
      absP[j] += fabs(nu) * c;
      if (JAC) {
        const double t = nu * cj;
        for (int l = 0; l < nz; ++l) J[(n.cid[i][l] * N + j) * js] += n.cnu[i][l] * t;
      }
    }
  }
  int status = 0;
  // ion exchange (RTotalSorbEqIonx)
  for (int r = 0; r < n.Nix; ++r) {
    const int nz = n.xn[r];
    double omega = n.xCEC[r];
    if (n.xsurf[r] > 0) omega = fmax(n.xCEC[r] * L.vf[n.xsurf[r] - 1], 1e-40);
    double X[PFCHEM_MAX_NNZ];
    const int i1 = n.xid[r][0];
    const double zref = n.Zp[i1];
    if (n.xzflag[r]) {
      const double ref = n.xk[r][0] * (L.m[i1] * L.gp[i1]);
      double KD = (zref * L.ixref[r] / omega) / ref;
      bool one_more = false;
      int it = 0;
      for (;;) {
        if (++it > 20000) {
          status = PFCHEM_CELL_INNER_MAXITER;
          break;
        }
        X[0] = KD * ref;
        double tot = X[0], dsum = 0.0;
        for (int k = 1; k < nz; ++k) {
          const int j = n.xid[r][k];
          double p;
          switch (n.xpow[r][k]) {
            case kPowOne: p = KD; break;
            case kPowTwo: p = KD * KD; break;
            case kPowHalf: p = sqrt(KD); break;
            default: p = pow(KD, n.xzr[r][k]); break;
          }
          X[k] = n.xk[r][k] * (L.m[j] * L.gp[j]) * p;
          tot += X[k];
          dsum += X[k] * n.xzr[r][k];
        }
        if (one_more) break;
        const double d = dsum / KD + ref;
        const double delta = (1.0 - tot) / d;
        KD = fmax(KD + delta, 1e-40);
        if (fabs(delta) < 1e-12 * KD) one_more = true;
      }
      L.ixref[r] = X[0] * omega / zref;
    } else {
      double s = 0.0;
      for (int k = 0; k < nz; ++k) {
        const int j = n.xid[r][k];
        X[k] = (L.m[j] * L.gp[j]) * n.xk[r][k];
        s += X[k];
      }
      const double is = 1.0 / s;
      for (int k = 0; k < nz; ++k) X[k] *= is;
    }
    double sumZX = 0.0;
    for (int k = 0; k < nz; ++k) sumZX += n.Zp[n.xid[r][k]] * X[k];
    const double isz = 1.0 / sumZX;
    for (int k = 0; k < nz; ++k) {
      const int i = n.xid[r][k];
      const double t1 = X[k] * omega / n.Zp[i];
      L.S_[i] += t1;
      absS[i] += fabs(t1);
      if (JAC) {
        const double t2 = n.Zp[i] * isz * t1 * L.v_t;
        for (int q = 0; q < nz; ++q) {
          const int j = n.xid[r][q];
          double v = -t2 * X[q];
          if (q == k) v += t1 * L.v_t;
          J[(i * N + j) * js] += v;
        }
      }
    }
  }
  // surface complexation (RTotalSorbEqSurfCplx1, immobile sites)
  for (int r = 0; r < n.Nsr; ++r) {
    double site;
    if (n.srtype[r] == PFCHEM_MINERAL_SURFACE) site = n.srdens[r] * L.vf[n.srsurf[r] - 1];
    else if (n.srtype[r] == PFCHEM_ROCK_SURFACE) site = n.srdens[r] * L.rho_s * (1.0 - L.por);
    else site = n.srdens[r];
    if (site < 1e-40) continue;
    const int ncx = n.srn[r];
    double Sk[PFCHEM_MAX_NNZ];
    double free = L.srfree[r];
    if (!n.srflag[r]) {
      double sumE = 0.0;
      for (int q = 0; q < ncx; ++q) {
        const int k = n.src[r][q];
        double s = L.bs[k];
        for (int l = 0; l < n.sn[k]; ++l) s += n.snu[k][l] * lna[n.sid[k][l]];
        Sk[q] = exp(s);
        sumE += Sk[q];
      }
      free = site / (1.0 + sumE);
      for (int q = 0; q < ncx; ++q) Sk[q] *= free;
    } else {
      bool one_more = false;
      double damping = 1.0;
      int it = 0;
      for (;;) {
        if (++it > 2000) {
          status = PFCHEM_CELL_INNER_MAXITER;
          break;
        }
        const double lf = log(free);
        double total = free, d = 1.0;
        for (int q = 0; q < ncx; ++q) {
          const int k = n.src[r][q];
          double s = L.bs[k] + n.sfs[k] * lf;
          for (int l = 0; l < n.sn[k]; ++l) s += n.snu[k][l] * lna[n.sid[k][l]];
          Sk[q] = exp(s);
          total += n.sfs[k] * Sk[q];
          d += n.sfs[k] * Sk[q] / free;
        }
        if (one_more) break;
        const double dfree = (site - total) / d;
        if (it > 1000) damping = 0.5;
        free = free + damping * dfree;
        if (fabs(dfree) < 1e-12 * fabs(free)) one_more = true;
      }
    }
    L.srfree[r] = free;
    // dSx/dln m_j = -(sum_k nu_kj fs_k S_k) / (1 + sum_k fs_k^2 S_k / Sx)
    double dSx[S::NP];
    double den = 0.0;
    if (JAC)
      for (int j = 0; j < N; ++j) dSx[j] = 0.0;
    for (int q = 0; q < ncx; ++q) {
      const int k = n.src[r][q];
      if (JAC)
        for (int l = 0; l < n.sn[k]; ++l) dSx[n.sid[k][l]] += n.snu[k][l] * n.sfs[k] * Sk[q];
      den += n.sfs[k] * n.sfs[k] * Sk[q];
    }
    const double iden = -1.0 / (den / free + 1.0);
    const double ifree = 1.0 / free;
    for (int q = 0; q < ncx; ++q) {
      const int k = n.src[r][q];
      const double nuS = n.sfs[k] * Sk[q] * ifree;
      for (int l = 0; l < n.sn[k]; ++l) {
        const int i = n.sid[k][l];
        const double v = n.snu[k][l] * Sk[q];
        L.S_[i] += v;
        absS[i] += fabs(v);
      }
      if (JAC && exact) {
        // the free site couples every component on the site
        double t[S::NP];
        for (int j = 0; j < N; ++j) t[j] = nuS * dSx[j] * iden;
        for (int l = 0; l < n.sn[k]; ++l) t[n.sid[k][l]] += n.snu[k][l] * Sk[q];
        for (int p = 0; p < n.sn[k]; ++p)
          for (int j = 0; j < N; ++j) J[(n.sid[k][p] * N + j) * js] += n.snu[k][p] * (t[j] * L.v_t);
      } else if (JAC) {
        for (int l = 0; l < n.sn[k]; ++l) {
          const int j = n.sid[k][l];
          const double t = (n.snu[k][l] * Sk[q] + nuS * dSx[j] * iden) * L.v_t;
          for (int p = 0; p < n.sn[k]; ++p) J[(n.sid[k][p] * N + j) * js] += n.snu[k][p] * t;
        }
      }
    }
  }
  // accumulation residual and its magnitude scale
  for (int j = 0; j < N; ++j) {
    L.F[j] = L.acc * (L.psv_den * L.Psi[j] + L.vol * L.S_[j]) - L.fixed[j];
    L.Sc[j] = L.acc * (L.psv_den * absP[j] + L.vol * absS[j]) + L.absfixed[j];
  }
  // kinetic minerals (RKineticMineral, TST rate law)
  for (int mm = 0; mm < n.Nm; ++mm) {
    const int nz = n.mn[mm];
    double lnQK = L.bm[mm];
    for (int k = 0; k < nz; ++k) lnQK += n.mnu[mm][k] * lna[n.mid[mm][k]];
    const double QK = (lnQK <= 6.90776) ? exp(lnQK) : 1e3;
    double aff;
    double sig = 1.0;
    if (n.has_temkin) sig = n.mtemkin[mm];
    if (n.has_minscale) sig *= n.mscale[mm];
    aff = (n.has_temkin || n.has_minscale) ? 1.0 - pow(QK, 1.0 / sig) : 1.0 - QK;
    const double sign_ = sgn1(aff);
    L.rate[mm] = 0.0;
    if (!(L.vf[mm] > 0.0 || sign_ < 0.0)) continue;
    if (n.mthr[mm] > 0.0 && sign_ < 0.0 && QK < n.mthr[mm]) continue;
    if (n.mlim[mm] > 0.0) aff = aff / (1.0 + (1.0 - aff) / n.mlim[mm]);
    double kr = L.rk[mm];
    // rate prefactors (reaction_mineral.F90:743-782): a sum over parallel
    // prefactors of products of Monod terms a^alpha / (1 + atten a^beta)
    const int npf = n.mpn[mm];
    double pref[PFCHEM_MAX_PREF], lps[PFCHEM_MAX_PREF][PFCHEM_MAX_PREF_SPEC];
    if (npf > 0) {
      kr = 0.0;
      for (int p = 0; p < npf; ++p) {
        double lp = 0.0;
        for (int q = 0; q < n.mps[mm][p]; ++q) {
          const double lsa = pref_lnact(n, L, lna, n.mpid[mm][p][q]);
          const double lnum = n.mpa[mm][p][q] * lsa;
          const double lden = log(1.0 + exp(log(n.mpatt[mm][p][q]) + n.mpb[mm][p][q] * lsa));
          lp = lp + lnum;
          lp = lp - lden;
          lps[p][q] = lnum - lden;
        }
        pref[p] = exp(lp);
        kr = kr + pref[p] * L.pk[mm][p];
      }
    }
    double Imc = -L.area[mm];
    if (n.has_minscale) Imc = Imc / n.mscale[mm];
    double Im;
    if (n.has_affpow) Im = Imc * sign_ * pow(fabs(aff), n.mpow[mm]) * kr;
    else Im = Imc * sign_ * fabs(aff) * kr;
    L.rate[mm] = Im;
    const double ImV = Im * L.vol;
    for (int k = 0; k < nz; ++k) {
      const int i = n.mid[mm][k];
      const double v = n.mnu[mm][k] * ImV;
      L.F[i] += v;
      L.Sc[i] += fabs(v);
    }
    if (JAC && !(exact && lnQK > 6.90776)) {  // exact: a capped QK does not depend on m
      double dIm_dQK = n.has_affpow ? -ImV * n.mpow[mm] / (exact ? aff : fabs(aff)) : -(Imc * L.vol) * kr;
      if (n.has_temkin || n.has_minscale) dIm_dQK = dIm_dQK * (1.0 / sig) / QK * (1.0 - aff);
      // d/dln m_j of QK is nu_j QK; the reference scales it by den*1e-3
      double g = dIm_dQK * QK * (exact ? 1.0 : L.den_mnrl) * L.jac_mnrl;
      if (n.mlim[mm] > 0.0) {
        const double d2 = 1.0 + (1.0 - aff) / n.mlim[mm];
        g = g * (1.0 + QK / n.mlim[mm] / d2) / d2;
      }
      for (int q = 0; q < nz; ++q) {
        const int j = n.mid[mm][q];
        const double t = g * n.mnu[mm][q];
        for (int k = 0; k < nz; ++k) J[(n.mid[mm][k] * N + j) * js] += n.mnu[mm][k] * t;
      }
    }
    if (JAC && npf > 0) {
      // derivative through the prefactors (reaction_mineral.F90:897-997), per
      // ln m: a primary's column gets the mineral's stoichiometry times
      // dIm/da * gamma * m; a complex's derivative goes through its
      // components (dC/dln m_j = nu_j C) into the rows of the complex's own
      // species as RReact adds it, or (exact) into the mineral's rows
      const double dIm_dsum = ImV / kr;
      for (int p = 0; p < npf; ++p) {
        const double lpf = log(pref[p]);
        for (int q = 0; q < n.mps[mm][p]; ++q) {
          const int id = n.mpid[mm][p][q];
          const double lsa = pref_lnact(n, L, lna, id);
          const double gs = id >= 0 ? L.gp[id] : exp(L.bK[-id - 1] - L.bc[-id - 1]);
          const double a_ = n.mpa[mm][p][q], b_ = n.mpb[mm][p][q], att = n.mpatt[mm][p][q];
          const double dpp = exp(lpf - lps[p][q]);
          const double num = a_ * exp(lps[p][q] - lsa);
          const double lgb = b_ * lsa;
          const double den = 1.0 + exp(log(att) + lgb);
          const double dden = -1.0 * exp(lps[p][q]) / den * att * b_ * exp(lgb - lsa);
          const double dspec = (num + dden) * gs;
          const double dIm = dIm_dsum * dpp * dspec * L.pk[mm][p] * L.jac_mnrl;
          if (id >= 0) {
            const double t = dIm * L.m[id];
            for (int k = 0; k < nz; ++k) J[(n.mid[mm][k] * N + id) * js] += n.mnu[mm][k] * t;
          } else {
            const int ci = -id - 1;
            for (int jj = 0; jj < n.cn[ci]; ++jj) {
              const int j = n.cid[ci][jj];
              const double t = n.cnu[ci][jj] * L.C[ci] * dIm;
              if (exact)
                for (int k = 0; k < nz; ++k) J[(n.mid[mm][k] * N + j) * js] += n.mnu[mm][k] * t;
              else
                for (int k = 0; k < n.cn[ci]; ++k) J[(n.cid[ci][k] * N + j) * js] += n.cnu[ci][k] * t;
            }
          }
        }
      }
    }
  }
  return status;
}

template <class S>
__device__ __forceinline__ bool converged(const DevNet &n, const Lane<S> &L, bool *nonfinite, double *rnorm) {
  bool conv = true;
  bool bad = false;
  double r = 0.0;
  for (int j = 0; j < n.N; ++j) {
    const double f = fabs(L.F[j]);
    if (!(f <= 1.7976931348623157e308)) bad = true;
    if (n.resid_kind == PFCHEM_RESIDUAL_RELATIVE) {
      if (!(f < n.res_tol * L.Sc[j])) conv = false;
      r = fmax(r, f / L.Sc[j]);
    } else {
      if (!(f < n.res_tol)) conv = false;
      r = fmax(r, f);
    }
  }
  *nonfinite = bad;
  *rnorm = r;
  return conv && !bad;
}

// LU with implicit-scaling partial pivoting (utility.F90:393-473, Crout
// order) on the thread's N x N system in J, then the two triangular solves
// (utility.F90:477-523) on rhs.  Returns false for a zero row.
__device__ bool lu_solve(double *J, int js, int N, double *rhs) {
  double vv[PFCHEM_MAX_PRI];
  int indx[PFCHEM_MAX_PRI];
  for (int i = 0; i < N; ++i) {
    double amax = 0.0;
    for (int j = 0; j < N; ++j) amax = fmax(amax, fabs(J[(i * N + j) * js]));
    if (!(amax > 0.0)) return false;
    vv[i] = 1.0 / amax;
  }
  for (int j = 0; j < N; ++j) {
    for (int i = 0; i < j; ++i) {
      double sum = J[(i * N + j) * js];
      for (int k = 0; k < i; ++k) sum -= J[(i * N + k) * js] * J[(k * N + j) * js];
      J[(i * N + j) * js] = sum;
    }
    double amax = 0.0;
    int imax = j;
    for (int i = j; i < N; ++i) {
      double sum = J[(i * N + j) * js];
      for (int k = 0; k < j; ++k) sum -= J[(i * N + k) * js] * J[(k * N + j) * js];
      J[(i * N + j) * js] = sum;
      const double dum = vv[i] * fabs(sum);
      if (dum >= amax) {
        imax = i;
        amax = dum;
      }
    }
    if (j != imax) {
      for (int k = 0; k < N; ++k) {
        const double t = J[(imax * N + k) * js];
        J[(imax * N + k) * js] = J[(j * N + k) * js];
        J[(j * N + k) * js] = t;
      }
      vv[imax] = vv[j];
    }
    indx[j] = imax;
    double piv = J[(j * N + j) * js];
    if (piv == 0.0) {
      piv = 1e-20;
      J[(j * N + j) * js] = piv;
    }
    const double ip = 1.0 / piv;
    vv[j] = ip;  // row j is final: keep 1/pivot for the back substitution
    for (int i = j + 1; i < N; ++i) J[(i * N + j) * js] *= ip;
  }
  int ii = -1;
  for (int i = 0; i < N; ++i) {
    const int ll = indx[i];
    double sum = rhs[ll];
    rhs[ll] = rhs[i];
    if (ii >= 0) {
      for (int j = ii; j < i; ++j) sum -= J[(i * N + j) * js] * rhs[j];
    } else if (sum != 0.0) {
      ii = i;
    }
    rhs[i] = sum;
  }
  for (int i = N - 1; i >= 0; --i) {
    double sum = rhs[i];
    for (int j = i + 1; j < N; ++j) sum -= J[(i * N + j) * js] * rhs[j];
    rhs[i] = sum * vv[i];
  }
  return true;
}

// One Newton iteration of RReact (reaction.F90:3411-3504).  Returns -1 to
// continue, else the cell's final status.
template <class S>
__device__ int newton_step(const DevNet &n, Lane<S> &L, double *J, int js) {
  const int N = n.N;
  L.iter += 1;
  if (L.act_fail) return PFCHEM_CELL_INNER_MAXITER;
  if (n.act_freq == PFCHEM_ACT_COEF_FREQUENCY_NEWTON_ITER && L.iter > 1) {
    if (n.act_newton) {
      if (activity_newton(n, L, false, 0.0)) return PFCHEM_CELL_INNER_MAXITER;
    } else {
      double I = 0.0;
      for (int j = 0; j < N; ++j) I += L.m[j] * n.Z2p[j];
      for (int i = 0; i < n.Nc; ++i) I += L.C[i] * n.cZ2[i];
      I *= 0.5;
      activity(n, L, I);
    }
  }
  // past exact_jacobian_after iterations: the exact Jacobian, no damping
  const bool rescue = n.exact_after > 0 && L.iter > n.exact_after;
  int st = evaluate<S, true>(n, L, J, js, n.jac_exact || rescue);
  if (st) return st;
  bool bad;
  double rn;
  const bool conv = converged(n, L, &bad, &rn);
  if (bad) return PFCHEM_CELL_NONFINITE;
  if (L.alt_pending) {
    // first iteration from the alternative guess: keep it only if its
    // residual is no worse than the plain guess's
    L.alt_pending = false;
    if (rn > L.r_plain) return -2;  // caller restarts from the plain guess
    L.alt_used = true;
  }
  if (conv) return PFCHEM_CELL_CONVERGED;
  if (L.iter >= n.max_iter) return PFCHEM_CELL_MAXITER;
  double upd[S::NP];
  if (!n.use_log) {
    // linear update: RSolve on dF/dm; columns of the ln m Jacobian / m_j
    for (int j = 0; j < N; ++j) {
      const double im = 1.0 / L.m[j];
      for (int i = 0; i < N; ++i) J[(i * N + j) * js] *= im;
    }
  }
  for (int j = 0; j < N; ++j) upd[j] = L.F[j];
  if (!lu_solve(J, js, N, upd)) return PFCHEM_CELL_SINGULAR;
  double mrc = 0.0;
  bool nf = false;
  double mnew[S::NP];
  if (n.use_log) {
    for (int j = 0; j < N; ++j) {
      const double u = sgn1(upd[j]) * fmin(fabs(upd[j]), n.max_dlnC);
      upd[j] = u;
      const double e = exp(-u);
      mnew[j] = L.m[j] * e;
      mrc = fmax(mrc, fabs(e - 1.0));
      if (!(fabs(mnew[j]) <= 1.7976931348623157e308)) nf = true;
    }
  } else {
    double min_ratio = 1e20;
    for (int j = 0; j < N; ++j)
      if (L.m[j] <= upd[j]) min_ratio = fmin(min_ratio, fabs(L.m[j] / upd[j]));
    const double sc = (min_ratio < 1.0) ? min_ratio * 0.99 : 1.0;
    for (int j = 0; j < N; ++j) {
      mnew[j] = L.m[j] - upd[j] * sc;
      mrc = fmax(mrc, fabs((mnew[j] - L.m[j]) / L.m[j]));
      if (!(fabs(mnew[j]) <= 1.7976931348623157e308)) nf = true;
    }
  }
  if (nf) return PFCHEM_CELL_NONFINITE;
  if (n.rel_change_tol > 0.0 && mrc < n.rel_change_tol) return PFCHEM_CELL_CONVERGED;
  if (L.iter > 50 && !rescue) {
    // reaction.F90:3478-3496 (only the 0.1 branch is reachable)
    for (int j = 0; j < N; ++j) {
      mnew[j] = 0.1 * (mnew[j] - L.m[j]) + L.m[j];
      L.m[j] = mnew[j];
      L.lnm[j] = log(mnew[j]);
    }
  } else if (n.use_log) {
    for (int j = 0; j < N; ++j) {
      L.m[j] = mnew[j];
      L.lnm[j] -= upd[j];
    }
  } else {
    for (int j = 0; j < N; ++j) {
      L.m[j] = mnew[j];
      L.lnm[j] = log(mnew[j]);
    }
  }
  return -1;
}

template <class S>
__device__ void finalize(const DevNet &n, const CellArgs &a, int64_t cell, Lane<S> &L, int status) {
  const int64_t nc = a.ncells;
  for (int j = 0; j < n.N; ++j) {
    a.pri_molal[j * nc + cell] = L.m[j];
    if (a.interleaved_out) a.interleaved_out[j * a.total_stride_comp + cell * a.total_stride_cell] = L.m[j];
    if (a.total_out) a.total_out[j * nc + cell] = L.Psi[j] * L.den_L;
    if (a.sorb) a.sorb[j * nc + cell] = L.S_[j];
  }
  double I = 0.0, sum = 0.0;
  for (int j = 0; j < n.N; ++j) {
    I += L.m[j] * n.Z2p[j];
    sum += L.m[j];
  }
  for (int i = 0; i < n.Nc; ++i) {
    I += L.C[i] * n.cZ2[i];
    sum += L.C[i];
    if (a.sec_molal) a.sec_molal[i * nc + cell] = L.C[i];
  }
  a.ionic[cell] = 0.5 * I;
  if (a.lnaw && n.use_h2o) {
    const double v = 1.0 - 0.017 * sum;
    a.lnaw[cell] = v > 0.0 ? log(v) : 0.0;
  }
  for (int k = 0; k < n.Nm; ++k) {
    if (a.rate) a.rate[k * nc + cell] = L.rate[k];
    if (n.update_kin && status == PFCHEM_CELL_CONVERGED) {
      // RUpdateKineticState (reaction.F90:5348-5365)
      double v = L.vf[k] + L.rate[k] * n.mVm[k] * L.dt;
      if (v < 0.0) v = 0.0;
      a.vf[k * nc + cell] = v;
    }
  }
  for (int r = 0; r < n.Nix; ++r) a.ixref[r * nc + cell] = L.ixref[r];
  for (int r = 0; r < n.Nsr; ++r) a.srfree[r * nc + cell] = L.srfree[r];
  if (a.iters) a.iters[cell] = L.iter;
  if (a.status) a.status[cell] = status;
}

// Loads the alternative guess, after evaluating the residual norm at the
// plain guess (the fallback reference).
template <class S>
__device__ void arm_alt_guess(const DevNet &n, const CellArgs &a, int64_t cell, Lane<S> &L) {
  evaluate<S, false>(n, L, nullptr, 0, n.jac_exact);
  bool bad;
  double rn;
  converged(n, L, &bad, &rn);
  L.r_plain = bad ? 1.7976931348623157e308 : rn;
  const int64_t nc = a.ncells;
  for (int j = 0; j < n.N; ++j) {
    const double g = a.alt_guess[j * nc + cell];
    if (g > 0.0 && g <= 1.7976931348623157e308) {
      L.m[j] = g;
      L.lnm[j] = log(g);
    }
  }
  L.alt_pending = true;
}

template <class S>
__global__ void __launch_bounds__(256) react_kernel(const __grid_constant__ DevNet n,
                                                    const __grid_constant__ CellArgs a, Scratch *scr,
                                                    int refill_min_idle, double inv_dt) {
  extern __shared__ double smem[];
  double *J = smem + threadIdx.x;
  const int js = blockDim.x;
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  Lane<S> L;
  int64_t cell = -1;
  bool exhausted = false;
  unsigned long long my_iters = 0, my_alt = 0, my_trips = 0;
  unsigned my_max = 0, my_bad = 0;
  for (;;) {
    const bool want = (cell < 0) && !exhausted;
    const unsigned want_mask = __ballot_sync(full, want);
    const unsigned busy_mask = __ballot_sync(full, cell >= 0);
    const int nwant = __popc(want_mask);
    if (nwant > 0 && (nwant >= refill_min_idle || busy_mask == 0)) {
      const int leader = __ffs(want_mask) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(&scr->next_cell, (unsigned long long)nwant);
      base = __shfl_sync(full, base, leader);
      if (want) {
        const unsigned long long c = base + __popc(want_mask & ((1u << lane) - 1u));
        if (c < (unsigned long long)a.ncells) {
          cell = (int64_t)c;
          if (a.active && a.active[cell] <= 0) {
            if (a.status) a.status[cell] = PFCHEM_CELL_INACTIVE;
            if (a.iters) a.iters[cell] = 0;
            cell = -1;
          } else {
            setup(n, a, cell, L, inv_dt);
            if (a.alt_guess) arm_alt_guess(n, a, cell, L);
          }
        } else {
          if (!exhausted) atomicMax(&scr->t_drain_inv, ~pf_now());
          exhausted = true;
        }
      }
      continue;  // re-vote: inactive cells release their lanes at once
    }
    if (busy_mask == 0) {
      if (__all_sync(full, exhausted)) break;
      continue;
    }
    ++my_trips;
    if (cell >= 0) {
      int st = newton_step(n, L, J, js);
      if (st == -2) {
        // the alternative guess was worse: restart from the plain guess
        for (int j = 0; j < n.N; ++j) {
          L.m[j] = a.pri_molal[j * a.ncells + cell];
          L.lnm[j] = log(L.m[j]);
        }
        L.iter = 0;
        for (int r = 0; r < n.Nix; ++r) L.ixref[r] = a.ixref[r * a.ncells + cell];
        st = -1;
      }
      if (st >= 0) {
        my_alt += L.alt_used ? 1 : 0;
        finalize(n, a, cell, L, st);
        my_iters += L.iter;
        my_max = max(my_max, (unsigned)L.iter);
        if (st != PFCHEM_CELL_CONVERGED) my_bad += 1;
        cell = -1;
      }
    }
  }
  // warp-aggregated statistics
  for (int o = 16; o > 0; o >>= 1) {
    my_iters += __shfl_xor_sync(full, my_iters, o);
    my_alt += __shfl_xor_sync(full, my_alt, o);
    my_max = max(my_max, __shfl_xor_sync(full, my_max, o));
    my_bad += __shfl_xor_sync(full, my_bad, o);
  }
  if (lane == 0) {
    atomicAdd(&scr->sum_iter, my_iters);
    atomicAdd(&scr->newton_trips, my_trips);
    atomicMax(&scr->t_end, pf_now());
    atomicAdd(&scr->alt_used, my_alt);
    atomicMax(&scr->max_iter, my_max);
    atomicAdd(&scr->nonconverged, my_bad);
  }
}

// Variant of react_kernel whose scratch is a caller-supplied block of global
// memory: the work-queue head, then one statistics slot per block (the
// blocks' warps add into their own slot, so the host needs no other buffer).
struct BlockSlot {
  unsigned long long sum_iter, alt_used;
  unsigned int max_iter, nonconverged;
  unsigned long long pad;
};

template <class S>
__global__ void __launch_bounds__(256) react_kernel_slots(const __grid_constant__ DevNet n,
                                                          const __grid_constant__ CellArgs a,
                                                          unsigned long long *queue_head, BlockSlot *slots,
                                                          int refill_min_idle, double inv_dt) {
  extern __shared__ double smem[];
  double *J = smem + threadIdx.x;
  const int js = blockDim.x;
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  Lane<S> L;
  int64_t cell = -1;
  bool exhausted = false;
  unsigned long long my_iters = 0, my_alt = 0;
  unsigned my_max = 0, my_bad = 0;
  for (;;) {
    const bool want = (cell < 0) && !exhausted;
    const unsigned want_mask = __ballot_sync(full, want);
    const unsigned busy_mask = __ballot_sync(full, cell >= 0);
    const int nwant = __popc(want_mask);
    if (nwant > 0 && (nwant >= refill_min_idle || busy_mask == 0)) {
      const int leader = __ffs(want_mask) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(queue_head, (unsigned long long)nwant);
      base = __shfl_sync(full, base, leader);
      if (want) {
        const unsigned long long c = base + __popc(want_mask & ((1u << lane) - 1u));
        if (c < (unsigned long long)a.ncells) {
          cell = (int64_t)c;
          if (a.active && a.active[cell] <= 0) {
            if (a.status) a.status[cell] = PFCHEM_CELL_INACTIVE;
            if (a.iters) a.iters[cell] = 0;
            cell = -1;
          } else {
            setup(n, a, cell, L, inv_dt);
            if (a.alt_guess) arm_alt_guess(n, a, cell, L);
          }
        } else {
          exhausted = true;
        }
      }
      continue;
    }
    if (busy_mask == 0) {
      if (__all_sync(full, exhausted)) break;
      continue;
    }
    if (cell >= 0) {
      int st = newton_step(n, L, J, js);
      if (st == -2) {
        for (int j = 0; j < n.N; ++j) {
          L.m[j] = a.pri_molal[j * a.ncells + cell];
          L.lnm[j] = log(L.m[j]);
        }
        L.iter = 0;
        for (int r = 0; r < n.Nix; ++r) L.ixref[r] = a.ixref[r * a.ncells + cell];
        st = -1;
      }
      if (st >= 0) {
        my_alt += L.alt_used ? 1 : 0;
        finalize(n, a, cell, L, st);
        my_iters += L.iter;
        my_max = max(my_max, (unsigned)L.iter);
        if (st != PFCHEM_CELL_CONVERGED) my_bad += 1;
        cell = -1;
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    my_iters += __shfl_xor_sync(full, my_iters, o);
    my_alt += __shfl_xor_sync(full, my_alt, o);
    my_max = max(my_max, __shfl_xor_sync(full, my_max, o));
    my_bad += __shfl_xor_sync(full, my_bad, o);
  }
  if (lane == 0) {
    BlockSlot *sl = slots + blockIdx.x;
    atomicAdd(&sl->sum_iter, my_iters);
    atomicAdd(&sl->alt_used, my_alt);
    atomicMax(&sl->max_iter, my_max);
    atomicAdd(&sl->nonconverged, my_bad);
  }
}

template <class S>
__global__ void __launch_bounds__(256) kinetic_state_kernel(const __grid_constant__ DevNet n,
                                                            const __grid_constant__ CellArgs a) {
  // RUpdateKineticState at the current state (reaction.F90:5320-5365)
  const int64_t cell = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (cell >= a.ncells) return;
  if (a.active && a.active[cell] <= 0) return;
  Lane<S> L;
  setup(n, a, cell, L, 1.0 / a.dt);
  evaluate<S, false>(n, L, nullptr, 0, n.jac_exact);
  const int64_t nc = a.ncells;
  for (int k = 0; k < n.Nm; ++k) {
    if (a.rate) a.rate[k * nc + cell] = L.rate[k];
    double v = L.vf[k] + L.rate[k] * n.mVm[k] * a.dt;
    a.vf[k * nc + cell] = v < 0.0 ? 0.0 : v;
  }
}

// Global-implicit blocks: three evaluations at the cell's state, each with
// the Jacobian weights of one term (aqueous totals, sorbed totals, minerals),
// written out per cell as column-major d/dm blocks.
struct BlocksOut {
  double *res, *jac, *total, *dtotal, *total_sorb, *dtotal_sorb;
};

template <class S>
__device__ void store_block(const DevNet &n, const Lane<S> &L, const double *J, int js, double *blk, int64_t cell) {
  const int N = n.N;
  double *b = blk + cell * (int64_t)N * N;
  for (int j = 0; j < N; ++j) {
    const double im = 1.0 / L.m[j];  // d/dln m -> d/dm
    for (int i = 0; i < N; ++i) b[j * N + i] = J[(i * N + j) * js] * im;
  }
}

template <class S>
__global__ void __launch_bounds__(32) reaction_blocks_kernel(const __grid_constant__ DevNet n,
                                                             const __grid_constant__ CellArgs a, BlocksOut o) {
  extern __shared__ double smem[];
  const int64_t cell = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (cell >= a.ncells) return;
  const int N = n.N;
  const int64_t nc = a.ncells, NN = (int64_t)N * N;
  double *J = smem + threadIdx.x;
  const int js = blockDim.x;
  if (a.active && a.active[cell] <= 0) {
    for (int j = 0; j < N; ++j) {
      o.res[j * nc + cell] = 0.0;
      if (o.total) o.total[j * nc + cell] = 0.0;
      if (o.total_sorb) o.total_sorb[j * nc + cell] = 0.0;
    }
    for (int64_t q = 0; q < NN; ++q) {
      o.jac[cell * NN + q] = 0.0;
      if (o.dtotal) o.dtotal[cell * NN + q] = 0.0;
      if (o.dtotal_sorb) o.dtotal_sorb[cell * NN + q] = 0.0;
    }
    if (a.status) a.status[cell] = PFCHEM_CELL_INACTIVE;
    return;
  }
  Lane<S> L;
  setup(n, a, cell, L, 1.0);
  L.acc = 0.0;  // no accumulation terms in the residual: F = reaction terms only
  for (int j = 0; j < N; ++j) L.fixed[j] = L.absfixed[j] = 0.0;
  int status = 0;
  // aqueous totals and d total / d ln m (x den/1000, as RTotal returns them)
  L.jac_aq = L.den_L;
  L.v_t = 0.0;
  L.jac_mnrl = 0.0;
  status |= evaluate<S, true>(n, L, J, js, n.jac_exact);
  if (o.total)
    for (int j = 0; j < N; ++j) o.total[j * nc + cell] = L.Psi[j] * L.den_L;
  if (o.dtotal) store_block(n, L, J, js, o.dtotal, cell);
  // sorbed totals and their derivatives
  if (n.Nix + n.Nsr > 0 && (o.total_sorb || o.dtotal_sorb)) {
    L.jac_aq = 0.0;
    L.v_t = 1.0;
    status |= evaluate<S, true>(n, L, J, js, n.jac_exact);
    if (o.total_sorb)
      for (int j = 0; j < N; ++j) o.total_sorb[j * nc + cell] = L.S_[j];
    if (o.dtotal_sorb) store_block(n, L, J, js, o.dtotal_sorb, cell);
  } else {
    if (o.total_sorb)
      for (int j = 0; j < N; ++j) o.total_sorb[j * nc + cell] = 0.0;
    if (o.dtotal_sorb)
      for (int64_t q = 0; q < NN; ++q) o.dtotal_sorb[cell * NN + q] = 0.0;
  }
  // reaction residual (RReaction) and its derivative
  L.jac_aq = 0.0;
  L.v_t = 0.0;
  L.jac_mnrl = 1.0;
  status |= evaluate<S, true>(n, L, J, js, n.jac_exact);
  for (int j = 0; j < N; ++j) o.res[j * nc + cell] = L.F[j];
  store_block(n, L, J, js, o.jac, cell);
  for (int k = 0; k < n.Nm; ++k)
    if (a.rate) a.rate[k * nc + cell] = L.rate[k];
  for (int i = 0; i < n.Nc; ++i)
    if (a.sec_molal) a.sec_molal[i * nc + cell] = L.C[i];
  for (int r = 0; r < n.Nix; ++r) a.ixref[r * nc + cell] = L.ixref[r];
  for (int r = 0; r < n.Nsr; ++r) a.srfree[r * nc + cell] = L.srfree[r];
  if (a.status) a.status[cell] = status ? PFCHEM_CELL_INNER_MAXITER : PFCHEM_CELL_CONVERGED;
}

template <class S>
static cudaError_t launch_blocks_t(const DevNet &n, const CellArgs &a, const BlocksOut &o, cudaStream_t st) {
  const int block = 32;
  const size_t shm = (size_t)n.N * n.N * block * sizeof(double);
  if (shm > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(reaction_blocks_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)shm);
    if (e != cudaSuccess) return e;
  }
  const int64_t grid = (a.ncells + block - 1) / block;
  reaction_blocks_kernel<S><<<(unsigned)grid, block, shm, st>>>(n, a, o);
  return cudaGetLastError();
}

// Batched constraint speciation (ReactionEquilibrateConstraint,
// reaction.F90:1308-2046), one thread per cell: Newton on the constraint
// rows with the aqueous totals and their derivatives from the same
// evaluation the reaction step uses (accumulation and mineral weights zero,
// d total/d ln m in the shared-memory system).
struct ConstraintRows {
  int8_t type[PFCHEM_MAX_PRI];
  int8_t mineral[PFCHEM_MAX_PRI];  // 0-based kinetic mineral of MINERAL rows, gas reaction of GAS rows
  int8_t gn[PFCHEM_MAX_GAS_ROWS];  // GAS reaction g: species count, 0-based primaries, coefficients
  int8_t gid[PFCHEM_MAX_GAS_ROWS][PFCHEM_MAX_NNZ];
  double gnu[PFCHEM_MAX_GAS_ROWS][PFCHEM_MAX_NNZ];
  double gh2o[PFCHEM_MAX_GAS_ROWS];     // H2O coefficient (0 where H2O takes no part)
  double glogK[PFCHEM_MAX_GAS_ROWS];    // log10 K (isothermal)
  double gcoef[PFCHEM_MAX_GAS_ROWS][5]; // log K(T) fit
  int32_t max_its;
  int32_t any_sorb_row;
  const double *value;             // (N, ncells)
};

template <class S>
__global__ void __launch_bounds__(32) constraint_kernel(const __grid_constant__ DevNet n,
                                                        const __grid_constant__ CellArgs a,
                                                        const __grid_constant__ ConstraintRows con, Scratch *scr) {
  extern __shared__ double smem[];
  const int64_t cell = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (cell >= a.ncells) return;
  const int N = n.N;
  const int64_t nc = a.ncells;
  double *J = smem + threadIdx.x;
  const int js = blockDim.x;
  Lane<S> L;
  setup(n, a, cell, L, 1.0);
  // activity coefficients start at 1 (reaction.F90:1308-1478)
  for (int j = 0; j < N; ++j) {
    L.lngp[j] = 0.0;
    L.gp[j] = 1.0;
  }
  for (int i = 0; i < n.Nc; ++i) L.bc[i] = L.bK[i];
  L.acc = 0.0;
  for (int j = 0; j < N; ++j) L.fixed[j] = L.absfixed[j] = 0.0;
  L.jac_aq = L.den_L;  // d(total [mol/L]) / d ln m
  L.v_t = 0.0;
  L.jac_mnrl = 0.0;
  const double molar_to_molal = 1000.0 / a.den[cell];
  double freec[S::NP], totc[S::NP], val[S::NP], res[S::NP], prev[S::NP], gb[S::NP];
  for (int j = 0; j < N; ++j) {
    val[j] = con.value[j * nc + cell];
    freec[j] = 1e-9;
    totc[j] = 0.0;
    gb[j] = 0.0;
    switch (con.type[j]) {
      case PFCHEM_CONSTRAINT_TOTAL:
      case PFCHEM_CONSTRAINT_TOTAL_SORB: totc[j] = val[j]; break;
      case PFCHEM_CONSTRAINT_GAS: {  // log10 partial pressure when <= 0 (reaction.F90:1531-1535)
        if (val[j] <= 0.0) val[j] = pow(10.0, val[j]);
        const int g = con.mineral[j];
        const double tk = L.temp + 273.15;
        const double lk = n.isothermal ? con.glogK[g] : logK_at(con.gcoef[g], log(tk), tk, 1.0 / tk);
        gb[j] = -lk * kLOG_TO_LN;
        break;
      }
      case PFCHEM_CONSTRAINT_FREE:
      case PFCHEM_CONSTRAINT_CHARGE_BAL:
      case PFCHEM_CONSTRAINT_MINERAL: freec[j] = val[j] * molar_to_molal; break;
      case PFCHEM_CONSTRAINT_LOG: freec[j] = pow(10.0, val[j]) * molar_to_molal; break;
      case PFCHEM_CONSTRAINT_PH: freec[j] = pow(10.0, -val[j]); break;
      default: break;
    }
    L.m[j] = freec[j];
  }
  bool act = false;
  int its = 0, its_on = 0, status = 1;
  for (;;) {
    for (int j = 0; j < N; ++j) {
      if (con.type[j] == PFCHEM_CONSTRAINT_FREE || con.type[j] == PFCHEM_CONSTRAINT_LOG) L.m[j] = freec[j];
      L.lnm[j] = log(L.m[j]);
    }
    if (act && n.act_freq != PFCHEM_ACT_COEF_FREQUENCY_OFF) {
      // ionic strength of the current free ions and the last complexes
      double I = 0.0;
      for (int j = 0; j < N; ++j) I += n.Z2p[j] * L.m[j];
      for (int i = 0; i < n.Nc; ++i) I += n.cZ2[i] * L.C[i];
      activity(n, L, 0.5 * I);
    }
    // sorbed totals and d/dm of TOTAL_SORB rows: one evaluation with the
    // sorption weights, the sorption warm starts then put back so that the
    // aqueous evaluation below runs the same inner iterations
    double sres[S::NP], sjac[S::NP][S::NP];
    if (con.any_sorb_row) {
      double ix0[S::NIX], sr0[S::NSR];
      for (int r = 0; r < n.Nix; ++r) ix0[r] = L.ixref[r];
      for (int r = 0; r < n.Nsr; ++r) sr0[r] = L.srfree[r];
      L.jac_aq = 0.0;
      L.v_t = 1.0;
      if (evaluate<S, true>(n, L, J, js, n.jac_exact)) {
        status = 1;
        break;
      }
      for (int i = 0; i < N; ++i)
        if (con.type[i] == PFCHEM_CONSTRAINT_TOTAL_SORB) {
          sres[i] = L.S_[i];
          for (int k = 0; k < N; ++k) sjac[i][k] = J[(i * N + k) * js] / L.m[k];
        }
      for (int r = 0; r < n.Nix; ++r) L.ixref[r] = ix0[r];
      for (int r = 0; r < n.Nsr; ++r) L.srfree[r] = sr0[r];
      L.jac_aq = L.den_L;
      L.v_t = 0.0;
    }
    if (evaluate<S, true>(n, L, J, js, n.jac_exact)) {
      status = 1;
      break;
    }
    // rows in d/dm, as ReactionEquilibrateConstraint forms them (reaction.F90:1597-1717)
    for (int k = 0; k < N; ++k) {
      const double im = 1.0 / L.m[k];
      for (int i = 0; i < N; ++i) J[(i * N + k) * js] *= im;
    }
    double cb[S::NP];
    bool any_cb = false;
    for (int j = 0; j < N; ++j) any_cb |= con.type[j] == PFCHEM_CONSTRAINT_CHARGE_BAL;
    if (any_cb)
      for (int k = 0; k < N; ++k) {
        double s = 0.0;
        for (int i = 0; i < N; ++i) s += n.Zp[i] * J[(i * N + k) * js];
        cb[k] = s;
      }
    double maxres = 0.0;
    for (int i = 0; i < N; ++i) {
      switch (con.type[i]) {
        case PFCHEM_CONSTRAINT_TOTAL: res[i] = L.Psi[i] * L.den_L - totc[i]; break;
        case PFCHEM_CONSTRAINT_CHARGE_BAL: {
          double s = 0.0;
          for (int j = 0; j < N; ++j) s += n.Zp[j] * (L.Psi[j] * L.den_L);
          res[i] = s;
          for (int k = 0; k < N; ++k) J[(i * N + k) * js] = cb[k];
          break;
        }
        case PFCHEM_CONSTRAINT_MINERAL: {
          const int mm = con.mineral[i];
          double lnQK = L.bm[mm];
          for (int k = 0; k < n.mn[mm]; ++k) {
            const int j = n.mid[mm][k];
            lnQK += n.mnu[mm][k] * log(L.m[j] * L.gp[j]);
          }
          res[i] = lnQK;
          for (int k = 0; k < N; ++k) J[(i * N + k) * js] = 0.0;
          for (int k = 0; k < n.mn[mm]; ++k) {
            const int j = n.mid[mm][k];
            J[(i * N + j) * js] = n.mnu[mm][k] / L.m[j];
          }
          break;
        }
        case PFCHEM_CONSTRAINT_GAS: {  // reaction.F90:1720-1751
          const int g = con.mineral[i];
          double lnQK = gb[i] + con.gh2o[g] * L.lnaw;
          for (int k = 0; k < con.gn[g]; ++k) {
            const int j = con.gid[g][k];
            lnQK += con.gnu[g][k] * log(L.m[j] * L.gp[j]);
          }
          res[i] = lnQK - log(val[i]);
          for (int k = 0; k < N; ++k) J[(i * N + k) * js] = 0.0;
          for (int k = 0; k < con.gn[g]; ++k) {
            const int j = con.gid[g][k];
            J[(i * N + j) * js] = con.gnu[g][k] / L.m[j];
          }
          break;
        }
        case PFCHEM_CONSTRAINT_TOTAL_SORB:  // reaction.F90:1608-1614
          res[i] = sres[i] - totc[i];
          for (int k = 0; k < N; ++k) J[(i * N + k) * js] = sjac[i][k];
          break;
        default: {  // FREE, LOG, PH: identity row
          if (con.type[i] == PFCHEM_CONSTRAINT_PH) L.m[i] = pow(10.0, -val[i]) / L.gp[i];
          res[i] = 0.0;
          for (int k = 0; k < N; ++k) J[(i * N + k) * js] = (k == i) ? 1.0 : 0.0;
          break;
        }
      }
      maxres = fmax(maxres, fabs(res[i]));
    }
    bool use_log = false;
    if (n.use_log) use_log = (its > 3 && its < 9) ? (its % 2 == 0) : true;
    if (use_log)  // RSolve's log form scales the columns by the molalities
      for (int k = 0; k < N; ++k)
        for (int i = 0; i < N; ++i) J[(i * N + k) * js] *= L.m[k];
    if (!lu_solve(J, js, N, res)) {
      status = 2;
      break;
    }
    bool nonpos = false;
    double mrc = 0.0;
    if (use_log) {
      for (int j = 0; j < N; ++j) {
        prev[j] = L.m[j];
        const double u = copysign(fmin(fabs(res[j]), n.max_dlnC), res[j]);
        L.m[j] = L.m[j] * exp(-u);
      }
    } else {
      double min_ratio = 1e20;
      for (int j = 0; j < N; ++j) {
        prev[j] = L.m[j];
        if (prev[j] <= res[j]) {
          const double ratio = fabs(prev[j] / res[j]);
          if (ratio < min_ratio) min_ratio = ratio;
        }
      }
      const double sc = (min_ratio <= 1.0) ? min_ratio * 0.99 : 1.0;
      for (int j = 0; j < N; ++j) L.m[j] = prev[j] - (min_ratio <= 1.0 ? res[j] * sc : res[j]);
    }
    for (int j = 0; j < N; ++j) {
      if (!(L.m[j] > 0.0)) nonpos = true;
      mrc = fmax(mrc, fabs((L.m[j] - prev[j]) / prev[j]));
    }
    if (nonpos) {
      status = 3;
      break;
    }
    ++its;
    if (its >= con.max_its) {
      status = 1;
      break;
    }
    if (maxres < n.res_tol && mrc < n.rel_change_tol) {
      if (act && its - its_on > 1) {
        status = 0;
        break;
      }
      if (!act) its_on = its;
      act = true;
    }
  }
  // totals and sorption at the final free ions with the last activity
  // coefficients (what the next step's RTAuxVarCompute sees)
  for (int j = 0; j < N; ++j) L.lnm[j] = log(L.m[j]);
  if (status == 0 && evaluate<S, true>(n, L, J, js, n.jac_exact)) status = 1;
  double I = 0.0;
  for (int j = 0; j < N; ++j) {
    a.pri_molal[j * nc + cell] = L.m[j];
    if (a.total_out) a.total_out[j * nc + cell] = L.Psi[j] * L.den_L;
    if (a.sorb) a.sorb[j * nc + cell] = L.S_[j];
    I += n.Z2p[j] * L.m[j];
  }
  for (int i = 0; i < n.Nc; ++i) {
    if (a.sec_molal) a.sec_molal[i * nc + cell] = L.C[i];
    I += n.cZ2[i] * L.C[i];
  }
  a.ionic[cell] = 0.5 * I;
  for (int r = 0; r < n.Nix; ++r) a.ixref[r * nc + cell] = L.ixref[r];
  for (int r = 0; r < n.Nsr; ++r) a.srfree[r * nc + cell] = L.srfree[r];
  if (a.iters) a.iters[cell] = its;
  if (a.status) a.status[cell] = status;
  if (status != 0) atomicAdd(&scr->nonconverged, 1u);
}

template <class S>
static cudaError_t launch_constraint_t(const DevNet &n, const CellArgs &a, const ConstraintRows &c, Scratch *scr,
                                       cudaStream_t st) {
  const int block = 32;
  const size_t shm = (size_t)n.N * n.N * block * sizeof(double);
  if (shm > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(constraint_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
    if (e != cudaSuccess) return e;
  }
  const int64_t grid = (a.ncells + block - 1) / block;
  constraint_kernel<S><<<(unsigned)grid, block, shm, st>>>(n, a, c, scr);
  return cudaGetLastError();
}

// Mineral-driven porosity and surface area (one thread per cell).
__global__ void __launch_bounds__(128) mineral_properties_kernel(const __grid_constant__ CellArgs a, int Nm,
                                                                 pfchem_mineral_update mu, int *flag_dev) {
  const int64_t cell = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nc = a.ncells;
  if (cell >= nc) return;
  double por = a.por[cell];
  if (mu.update_porosity && Nm > 0) {
    double sum = 0.0;
    for (int k = 0; k < Nm; ++k) sum += a.vf[k * nc + cell];
    por = fmax(1.0 - sum, mu.minimum_porosity);
    mu.porosity[cell] = por;
  }
  if (!mu.update_surface_area) return;
  const double ratio = mu.surface_area_with_porosity ? por / mu.porosity0[cell] : 1.0;
  // armoring: the reference's flag entering this cell is set by the test of
  // the previous cell's last armored mineral (the caller's flag for cell 0)
  int flag = mu.armor_flag;
  int last = -1;
  if (mu.armor_crit_vol_frac) {
    for (int k = 0; k < Nm; ++k)
      if (mu.armor_crit_vol_frac[k] > 0.0) last = k;
    if (last >= 0 && cell > 0) {
      const int ma = mu.armor_mineral ? mu.armor_mineral[last] - 1 : last;
      flag = mu.armor_crit_vol_frac[last] > a.vf[ma * nc + cell - 1] ? 0 : 1;
    }
  }
  for (int k = 0; k < Nm; ++k) {
    double ps = 1.0;
    if (mu.surface_area_with_porosity) ps = pow(ratio, mu.surf_area_porosity_pwr[k]);
    double vs = 1.0;
    const double vf0 = mu.mnrl_volfrac0[k * nc + cell];
    if (vf0 > 0.0) vs = pow(a.vf[k * nc + cell] / vf0, mu.surf_area_vol_frac_pwr[k]);
    double area = mu.mnrl_area0[k * nc + cell] * ps * vs;
    if (mu.armor_crit_vol_frac && mu.armor_crit_vol_frac[k] > 0.0) {
      const int ma = mu.armor_mineral ? mu.armor_mineral[k] - 1 : k;
      const double crit = mu.armor_crit_vol_frac[k];
      const double vfa = a.vf[ma * nc + cell];
      if (crit > vfa) {
        area = flag == 0 ? area * pow((crit - vfa) / crit, mu.surf_area_vol_frac_pwr[k]) : mu.mnrl_area0[k * nc + cell];
        flag = 0;
      } else {
        area = 0.0;
        flag = 1;
      }
    }
    a.area[k * nc + cell] = area;
  }
  // the flag after the last cell (the caller's flag if nothing is armored)
  if (cell == nc - 1 && flag_dev) *flag_dev = flag;
}

cudaError_t launch_mineral_properties(const CellArgs &a, int Nm, const pfchem_mineral_update &mu, int *flag_dev,
                                      cudaStream_t st) {
  const int block = 128;
  const int64_t grid = (a.ncells + block - 1) / block;
  mineral_properties_kernel<<<(unsigned)grid, block, 0, st>>>(a, Nm, mu, flag_dev);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// launch helpers (host)
template <class S>
static cudaError_t launch_react_t(const DevNet &n, const CellArgs &a, Scratch *scr, int grid, int block,
                                  int refill, cudaStream_t st) {
  // the dynamic shared-memory limit was raised by max_active_blocks(), which
  // the host calls outside any stream capture
  const size_t shm = (size_t)n.N * n.N * block * sizeof(double);
  react_kernel<S><<<grid, block, shm, st>>>(n, a, scr, refill, 1.0 / a.dt);
  return cudaGetLastError();
}

template <class S>
static cudaError_t launch_kin_t(const DevNet &n, const CellArgs &a, cudaStream_t st) {
  const int block = 128;
  const int64_t grid = (a.ncells + block - 1) / block;
  kinetic_state_kernel<S><<<(unsigned)grid, block, 0, st>>>(n, a);
  return cudaGetLastError();
}

int size_class(const DevNet &n) {
  if (n.N <= SizesS::NP && n.Nc <= SizesS::NCX && n.Nm <= SizesS::NMN && n.Nix <= SizesS::NIX &&
      n.Nsr <= SizesS::NSR && n.Nsc <= SizesS::NSC)
    return 0;
  if (n.N <= SizesM::NP && n.Nc <= SizesM::NCX && n.Nm <= SizesM::NMN && n.Nix <= SizesM::NIX &&
      n.Nsr <= SizesM::NSR && n.Nsc <= SizesM::NSC)
    return 1;
  return 2;
}

cudaError_t launch_react(const DevNet &n, const CellArgs &a, Scratch *scr, int grid, int block, int refill,
                         cudaStream_t st) {
  switch (size_class(n)) {
    case 0: return launch_react_t<SizesS>(n, a, scr, grid, block, refill, st);
    case 1: return launch_react_t<SizesM>(n, a, scr, grid, block, refill, st);
    default: return launch_react_t<SizesL>(n, a, scr, grid, block, refill, st);
  }
}

cudaError_t launch_reaction_blocks(const DevNet &n, const CellArgs &a, double *res, double *jac, double *total,
                                   double *dtotal, double *total_sorb, double *dtotal_sorb, cudaStream_t st) {
  const BlocksOut o{res, jac, total, dtotal, total_sorb, dtotal_sorb};
  switch (size_class(n)) {
    case 0: return launch_blocks_t<SizesS>(n, a, o, st);
    case 1: return launch_blocks_t<SizesM>(n, a, o, st);
    default: return launch_blocks_t<SizesL>(n, a, o, st);
  }
}

cudaError_t launch_constraint(const DevNet &n, const CellArgs &a, const pfchem_constraint &con, int max_its,
                              Scratch *scr, cudaStream_t st) {
  ConstraintRows c{};
  int ngas = 0;
  for (int j = 0; j < n.N; ++j) {
    c.type[j] = (int8_t)con.type[j];
    c.mineral[j] = (int8_t)(con.mineral && con.mineral[j] > 0 ? con.mineral[j] - 1 : 0);
    if (con.type[j] == PFCHEM_CONSTRAINT_TOTAL_SORB) c.any_sorb_row = 1;
    if (con.type[j] == PFCHEM_CONSTRAINT_GAS) {  // the row's gas reaction, compacted (ids checked by the caller)
      const int g = con.mineral[j] - 1, ld = con.paseq_ld, q = ngas++;
      c.mineral[j] = (int8_t)q;
      c.gn[q] = (int8_t)con.paseqspecid[g * (ld + 1)];
      for (int k = 0; k < c.gn[q]; ++k) {
        c.gid[q][k] = (int8_t)(con.paseqspecid[g * (ld + 1) + 1 + k] - 1);
        c.gnu[q][k] = con.paseqstoich[g * ld + k];
      }
      c.gh2o[q] = (con.paseqh2oid && con.paseqh2oid[g] > 0) ? con.paseqh2ostoich[g] : 0.0;
      c.glogK[q] = con.paseqlogK ? con.paseqlogK[g] : 0.0;
      for (int k = 0; k < 5; ++k) c.gcoef[q][k] = con.paseqlogKcoef ? con.paseqlogKcoef[5 * g + k] : 0.0;
    }
  }
  c.max_its = max_its;
  c.value = con.value;
  switch (size_class(n)) {
    case 0: return launch_constraint_t<SizesS>(n, a, c, scr, st);
    case 1: return launch_constraint_t<SizesM>(n, a, c, scr, st);
    default: return launch_constraint_t<SizesL>(n, a, c, scr, st);
  }
}

cudaError_t launch_kinetic_state(const DevNet &n, const CellArgs &a, cudaStream_t st) {
  switch (size_class(n)) {
    case 0: return launch_kin_t<SizesS>(n, a, st);
    case 1: return launch_kin_t<SizesM>(n, a, st);
    default: return launch_kin_t<SizesL>(n, a, st);
  }
}

template <class S>
static int max_active_blocks_t(int block, size_t shm) {
  int nb = 0;
  constexpr int kMaxDyn = 227 * 1024;
  if (cudaFuncSetAttribute(react_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDyn) != cudaSuccess)
    return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, react_kernel<S>, block, shm) != cudaSuccess) return 0;
  return nb;
}

int max_active_blocks(const DevNet &n, int block) {
  const size_t shm = (size_t)n.N * n.N * block * sizeof(double);
  switch (size_class(n)) {
    case 0: return max_active_blocks_t<SizesS>(block, shm);
    case 1: return max_active_blocks_t<SizesM>(block, shm);
    default: return max_active_blocks_t<SizesL>(block, shm);
  }
}


template <class S>
static int slots_blocks_per_sm_t(int block, size_t shm) {
  int nb = 0;
  if (cudaFuncSetAttribute(react_kernel_slots<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024) !=
      cudaSuccess)
    return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, react_kernel_slots<S>, block, shm) != cudaSuccess) return 0;
  return nb;
}

// Resident blocks per SM of react_kernel_slots for `block` threads (0 if it
// does not fit).  Sets the kernel's dynamic shared-memory limit.
int slots_blocks_per_sm(const DevNet &n, int block) {
  const size_t shm = (size_t)n.N * n.N * block * sizeof(double);
  switch (size_class(n)) {
    case 0: return slots_blocks_per_sm_t<SizesS>(block, shm);
    case 1: return slots_blocks_per_sm_t<SizesM>(block, shm);
    default: return slots_blocks_per_sm_t<SizesL>(block, shm);
  }
}

size_t slots_scratch_bytes(int grid) { return 256 + (size_t)grid * sizeof(BlockSlot); }

template <class S>
static cudaError_t launch_slots_t(const DevNet &n, const CellArgs &a, void *scratch, int grid, int block,
                                  int refill, cudaStream_t st) {
  const size_t shm = (size_t)n.N * n.N * block * sizeof(double);
  unsigned long long *head = (unsigned long long *)scratch;
  BlockSlot *slots = (BlockSlot *)((char *)scratch + 256);
  react_kernel_slots<S><<<grid, block, shm, st>>>(n, a, head, slots, refill, 1.0 / a.dt);
  return cudaGetLastError();
}

// Launches react_kernel_slots with its queue head and statistics slots in
// `scratch` (slots_scratch_bytes(grid) bytes, zeroed by the caller).
cudaError_t launch_react_slots(const DevNet &n, const CellArgs &a, void *scratch, int grid, int block, int refill,
                               cudaStream_t st) {
  switch (size_class(n)) {
    case 0: return launch_slots_t<SizesS>(n, a, scratch, grid, block, refill, st);
    case 1: return launch_slots_t<SizesM>(n, a, scratch, grid, block, refill, st);
    default: return launch_slots_t<SizesL>(n, a, scratch, grid, block, refill, st);
  }
}

// Sums the per-block slots read back to the host.
void sum_slots(const void *host_slots, int grid, unsigned long long *sum_iter, unsigned long long *alt,
               unsigned *max_iter, unsigned *bad) {
  const BlockSlot *sl = (const BlockSlot *)host_slots;
  *sum_iter = 0;
  *alt = 0;
  *max_iter = 0;
  *bad = 0;
  for (int b = 0; b < grid; ++b) {
    *sum_iter += sl[b].sum_iter;
    *alt += sl[b].alt_used;
    *max_iter = sl[b].max_iter > *max_iter ? sl[b].max_iter : *max_iter;
    *bad += sl[b].nonconverged;
  }
}
}  // namespace pfchem
