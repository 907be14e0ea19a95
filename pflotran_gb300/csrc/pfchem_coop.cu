// pfchem_coop.cu -- cooperative Newton kernel: G lanes (8, 16 or 32) solve
// one cell together.
//
// The thread-per-cell kernels keep a cell's N x (N+1) augmented Jacobian in
// shared memory per thread (1.3 KB at N = 12, 8.4 KB at N = 32), which caps
// residency at a few warps per SM for mid-size networks and does not fit at
// all beyond N of about 28.  Here a group of G lanes owns one cell: the
// cell's state, its complexes and its Jacobian live in shared memory once per
// group, and the work of one Newton iteration is spread over the lanes --
// complexes, species, Jacobian entries, ion-exchange sites, surface sites,
// minerals, LU rows and columns.  The per-cell algorithm is that of
// pfchem_newton.cu (RReact, reaction.F90:3322-3511, with the same options:
// reference or exact Jacobian, exact_jacobian_after, rate prefactors, TIMESTEP
// or NEWTON_ITER LAG activity, the learned warm start's alternative guess):
//  * totals and Jacobian entries are gathered per species / per entry from
//    host-built lists (each written by one lane, no atomics);
//  * ion exchange, surface complexation and minerals run one site or
//    mineral per lane and add their terms to the shared residual and
//    Jacobian in a fixed round order (one lane writes per round);
//  * the linear solve is Gaussian elimination on [J | F] with the
//    power-of-two implicit-scaling pivoting of the specialized kernel: rows
//    eliminated by all lanes of the group, the pivot chosen by a shuffle
//    reduction, back substitution by columns.
// Not supported here (the library keeps them on the other kernels): the
// linear update, the NEWTON activity algorithm and the activity of water.
#include <cuda_runtime.h>

#include <climits>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/pfchem.h"
#include "pfchem_device.cuh"

namespace pfchem {

constexpr int kCoopMaxSp = PFCHEM_MAX_CPLX * PFCHEM_MAX_NNZ;
constexpr int kCoopMaxJe = PFCHEM_MAX_CPLX * PFCHEM_MAX_NNZ * PFCHEM_MAX_NNZ;

// Gather lists of the aqueous-complex terms: per species the complexes it is
// in (totals), per Jacobian entry (l, k) the complexes with both species and
// the product of their coefficients.
struct CoopTables {
  int16_t sp_ptr[PFCHEM_MAX_PRI + 1];
  int16_t je_ptr[PFCHEM_MAX_PRI * PFCHEM_MAX_PRI + 1];
  int16_t sp_cplx[kCoopMaxSp];
  int16_t je_cplx[kCoopMaxJe];
  double sp_nu[kCoopMaxSp];
  double je_nu[kCoopMaxJe];
};

// Shared-memory layout of one cell group (offsets in doubles).
struct CoopLayout {
  int m, lm, lg, gam, fx, la, P, aP, Sg, aS, F, Sc, bK, bc, C, bm, rk, vf, ar, rate, pk, bs, ixr, srf, sc, J, E,
      sm, slm, sixr, sfree, total;
};

__host__ __device__ inline CoopLayout coop_layout(const DevNet &n) {
  CoopLayout L;
  int o = 0;
  const int N = n.N, Nc = n.Nc > 0 ? n.Nc : 1, Nm = n.Nm > 0 ? n.Nm : 1;
  L.m = o; o += N; L.lm = o; o += N; L.lg = o; o += N; L.gam = o; o += N; L.fx = o; o += N; L.la = o; o += N;
  L.P = o; o += N; L.aP = o; o += N; L.Sg = o; o += N; L.aS = o; o += N; L.F = o; o += N; L.Sc = o; o += N;
  L.bK = o; o += Nc; L.bc = o; o += Nc; L.C = o; o += Nc;
  L.bm = o; o += Nm; L.rk = o; o += Nm; L.vf = o; o += Nm; L.ar = o; o += Nm; L.rate = o; o += Nm;
  L.pk = o; o += Nm * PFCHEM_MAX_PREF;
  L.bs = o; o += (n.Nsc > 0 ? n.Nsc : 1);
  L.ixr = o; o += (n.Nix > 0 ? n.Nix : 1);
  L.srf = o; o += (n.Nsr > 0 ? n.Nsr : 1);
  L.sc = o; o += 16;
  L.J = o; o += N * (N + 1);
  L.E = o; o += N;
  L.sm = o; o += N; L.slm = o; o += N; L.sixr = o; o += (n.Nix > 0 ? n.Nix : 1);
  L.sfree = o; o += (n.Nsr > 0 ? n.Nsr : 1);
  L.total = o;
  return L;
}

// scalar slots
enum { kAcc = 0, kPsvDen, kJacAq, kVol, kVt, kDenL, kPor, kRhoS, kTk, kIcell, kIacc, kDt };

namespace {

PFCHEM_GLOBALTIMER_FN

__device__ __forceinline__ double csgn1(double x) { return signbit(x) ? -1.0 : 1.0; }
__device__ __forceinline__ long long cabsbits(double x) { return __double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFLL; }

template <int G>
struct Grp {
  unsigned mask;
  int g;
  __device__ __forceinline__ void sync() const { __syncwarp(mask); }
  __device__ __forceinline__ bool any(bool p) const { return (__ballot_sync(mask, p) & mask) != 0u; }
  __device__ __forceinline__ double max(double v) const {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(mask, v, o, G));
    return v;
  }
  __device__ __forceinline__ double sum(double v) const {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o, G);
    return v;
  }
};

// LAG activity coefficients at ionic strength I (reaction.F90:3992-4051):
// ln gamma of the primaries into lg/gam, complexes folded into bc = bK - ln gamma.
template <int G>
__device__ void coop_activity(const DevNet &n, const Grp<G> &q, double *W, const CoopLayout &L, double I) {
  const double sI = sqrt(I);
  for (int j = q.g; j < n.N; j += G) {
    double lg = 0.0;
    if (n.Z2p[j] > 1e-20) lg = (-n.Z2p[j] * sI * n.A / (1.0 + n.ap[j] * n.B * sI) + n.Bdot * I) * kLOG_TO_LN;
    W[L.lg + j] = lg;
    W[L.gam + j] = exp(lg);
  }
  for (int i = q.g; i < n.Nc; i += G) {
    double lg = 0.0;
    if (n.cZ2[i] > 1e-20) lg = (-n.cZ2[i] * sI * n.A / (1.0 + n.ca[i] * n.B * sI) + n.Bdot * I) * kLOG_TO_LN;
    W[L.bc + i] = W[L.bK + i] - lg;
  }
  q.sync();
}

__device__ __forceinline__ double logK_at_c(const double *c, double lntk, double tk, double itk) {
  return c[0] * lntk + c[1] + c[2] * tk + c[3] * itk + c[4] * (itk * itk);
}

// Per-cell constants of the step and the starting guess (RReact's prologue).
template <int G>
__device__ void coop_setup(const DevNet &n, const CellArgs &a, int64_t cell, const Grp<G> &q, double *W,
                           const CoopLayout &L, double inv_dt) {
  const int64_t nc = a.ncells;
  double *sc = W + L.sc;
  const double por = a.por[cell], sat = a.sat[cell], vol = a.vol[cell], den = a.den[cell];
  const double psv = por * sat * 1000.0 * vol;
  const double acc = (n.accum_mode == PFCHEM_ACCUM_DT_CONSISTENT) ? inv_dt : 1.0;
  if (q.g == 0) {
    sc[kAcc] = acc;
    sc[kDenL] = den * 1e-3;
    sc[kPsvDen] = psv * (den * 1e-3);
    sc[kJacAq] = psv * inv_dt * (den * 1e-3);
    sc[kVol] = vol;
    sc[kVt] = vol * inv_dt;
    sc[kPor] = por;
    sc[kRhoS] = a.rho_s ? a.rho_s[cell] : 0.0;
    sc[kTk] = a.temp[cell] + 273.15;
    sc[kIcell] = a.ionic[cell];
    sc[kDt] = a.dt;
  }
  const bool sorb = (n.Nix + n.Nsr) > 0;
  for (int j = q.g; j < n.N; j += G) {
    const double tot = a.total[j * a.total_stride_comp + cell * a.total_stride_cell];
    double f = psv * tot;
    if (sorb) f = f + a.sorb[j * nc + cell] * vol;
    W[L.fx + j] = acc * f;
    const double m = a.pri_molal[j * nc + cell];
    W[L.m + j] = m;
    W[L.lm + j] = log(m);
  }
  const double tk = a.temp[cell] + 273.15;
  double lntk = 0.0, itk = 0.0;
  if (!n.isothermal) {
    lntk = log(tk);
    itk = 1.0 / tk;
  }
  for (int i = q.g; i < n.Nc; i += G) {
    const double lk = n.isothermal ? n.clogK[i] : logK_at_c(n.ccoef[i], lntk, tk, itk);
    W[L.bK + i] = -lk * kLOG_TO_LN;
  }
  for (int k = q.g; k < n.Nm; k += G) {
    const double lk = n.isothermal ? n.mlogK[k] : logK_at_c(n.mcoef[k], lntk, tk, itk);
    W[L.bm + k] = -lk * kLOG_TO_LN;
    double af = 1.0;
    if (n.mEa[k] > 0.0) af = exp(n.mEa[k] / kIDEAL_GAS_CONSTANT * (1.0 / (25.0 + 273.15) - 1.0 / tk));
    W[L.rk + k] = n.mk[k] * af;
    for (int p = 0; p < n.mpn[k]; ++p) {
      double pf = 1.0;
      if (n.mpEa[k][p] > 0.0) pf = exp(n.mpEa[k][p] / kIDEAL_GAS_CONSTANT * (1.0 / (25.0 + 273.15) - 1.0 / tk));
      W[L.pk + k * PFCHEM_MAX_PREF + p] = n.mpk[k][p] * pf;
    }
    W[L.vf + k] = a.vf[k * nc + cell];
    W[L.ar + k] = a.area[k * nc + cell];
    W[L.rate + k] = 0.0;
  }
  for (int k = q.g; k < n.Nsc; k += G) {
    const double lk = n.isothermal ? n.slogK[k] : logK_at_c(n.scoef[k], lntk, tk, itk);
    W[L.bs + k] = -lk * kLOG_TO_LN;
  }
  for (int r = q.g; r < n.Nix; r += G) W[L.ixr + r] = a.ixref[r * nc + cell];
  for (int r = q.g; r < n.Nsr; r += G) W[L.srf + r] = a.srfree[r * nc + cell];
  q.sync();
  if (n.act_freq != PFCHEM_ACT_COEF_FREQUENCY_OFF) {
    coop_activity<G>(n, q, W, L, a.ionic[cell]);
  } else {
    for (int j = q.g; j < n.N; j += G) {
      W[L.lg + j] = 0.0;
      W[L.gam + j] = 1.0;
    }
    for (int i = q.g; i < n.Nc; i += G) W[L.bc + i] = W[L.bK + i];
    q.sync();
  }
}

// ln activity of a rate-prefactor species (>= 0 primary, < 0 complex -(i+1))
__device__ __forceinline__ double coop_pref_lnact(const DevNet &n, const double *W, const CoopLayout &L, int id) {
  if (id >= 0) return W[L.la + id];
  const int i = -id - 1;
  double s = W[L.bK + i];
  for (int k = 0; k < n.cn[i]; ++k) s += n.cnu[i][k] * W[L.la + n.cid[i][k]];
  return s;
}

// Residual F (and with jac the Jacobian d/dln m into J, row stride N + 1) at
// the group's m.  Returns the inner-loop status (0 or INNER_MAXITER).
template <int G>
__device__ int coop_evaluate(const DevNet &n, const CoopTables *__restrict__ t, const Grp<G> &q, double *W,
                             const CoopLayout &L, bool jac, bool exact) {
  const int N = n.N, RS = N + 1;
  double *sc = W + L.sc;
  double *J = W + L.J;
  for (int j = q.g; j < N; j += G) W[L.la + j] = W[L.lm + j] + W[L.lg + j];
  q.sync();
  // aqueous complexes (RTotal): one complex per lane
  double iacc = 0.0;
  for (int i = q.g; i < n.Nc; i += G) {
    double s = W[L.bc + i];
    for (int k = 0; k < n.cn[i]; ++k) s += n.cnu[i][k] * W[L.la + n.cid[i][k]];
    const double c = exp(s);
    W[L.C + i] = c;
    iacc = fma(n.cZ2[i], c, iacc);
  }
  iacc = q.sum(iacc);
  if (q.g == 0) sc[kIacc] = 0.5 * iacc;
  q.sync();
  // totals per species; Jacobian entries per (l, k)
  for (int j = q.g; j < N; j += G) {
    const double m = W[L.m + j];
    double P = m, aP = m;
    for (int e = t->sp_ptr[j]; e < t->sp_ptr[j + 1]; ++e) {
      const double c = W[L.C + t->sp_cplx[e]];
      const double nu = t->sp_nu[e];
      P = fma(nu, c, P);
      aP = fma(fabs(nu), c, aP);
    }
    W[L.P + j] = P;
    W[L.aP + j] = aP;
    W[L.Sg + j] = 0.0;
    W[L.aS + j] = 0.0;
  }
  if (jac) {
    const double jaq = sc[kJacAq];
    for (int e = q.g; e < N * N; e += G) {
      const int l = e / N, k = e % N;
      double v = (l == k) ? W[L.m + l] * jaq : 0.0;
      for (int x = t->je_ptr[e]; x < t->je_ptr[e + 1]; ++x) v = fma(t->je_nu[x], W[L.C + t->je_cplx[x]] * jaq, v);
      J[l * RS + k] = v;
    }
  }
  q.sync();
  int status = 0;
  const double vt = sc[kVt];
  // ion exchange (RTotalSorbEqIonx): one reaction per lane, terms added in reaction order
  {
    double X[PFCHEM_MAX_NNZ];
    double omega = 0.0, isz = 0.0;
    const int r = q.g;
    const bool mine = r < n.Nix;
    if (mine) {
      const int nz = n.xn[r];
      omega = n.xCEC[r];
      if (n.xsurf[r] > 0) omega = fmax(n.xCEC[r] * W[L.vf + n.xsurf[r] - 1], 1e-40);
      const int i1 = n.xid[r][0];
      const double zref = n.Zp[i1];
      if (n.xzflag[r]) {
        const double ref = n.xk[r][0] * (W[L.m + i1] * W[L.gam + i1]);
        double KD = (zref * W[L.ixr + r] / omega) / ref;
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
            X[k] = n.xk[r][k] * (W[L.m + j] * W[L.gam + j]) * p;
            tot += X[k];
            dsum += X[k] * n.xzr[r][k];
          }
          if (one_more) break;
          const double d = dsum / KD + ref;
          const double delta = (1.0 - tot) / d;
          KD = fmax(KD + delta, 1e-40);
          if (fabs(delta) < 1e-12 * KD) one_more = true;
        }
        W[L.ixr + r] = X[0] * omega / zref;
      } else {
        double s = 0.0;
        for (int k = 0; k < nz; ++k) {
          const int j = n.xid[r][k];
          X[k] = (W[L.m + j] * W[L.gam + j]) * n.xk[r][k];
          s += X[k];
        }
        const double is = 1.0 / s;
        for (int k = 0; k < nz; ++k) X[k] *= is;
      }
      double sumZX = 0.0;
      for (int k = 0; k < nz; ++k) sumZX += n.Zp[n.xid[r][k]] * X[k];
      isz = 1.0 / sumZX;
    }
    for (int rr = 0; rr < n.Nix; ++rr) {
      if (mine && rr == r) {
        const int nz = n.xn[r];
        for (int k = 0; k < nz; ++k) {
          const int i = n.xid[r][k];
          const double t1 = X[k] * omega / n.Zp[i];
          W[L.Sg + i] += t1;
          W[L.aS + i] += fabs(t1);
          if (jac) {
            const double t2 = n.Zp[i] * isz * t1 * vt;
            for (int qq = 0; qq < nz; ++qq) {
              const int j = n.xid[r][qq];
              if (qq == k) J[i * RS + j] += t1 * vt - t2 * X[qq];
              else J[i * RS + j] -= t2 * X[qq];
            }
          }
        }
      }
      q.sync();
    }
  }
  // surface complexation (RTotalSorbEqSurfCplx1): one reaction per lane
  {
    double Sk[PFCHEM_MAX_NNZ];
    double free = 0.0, site = 0.0;
    const int r = q.g;
    const bool mine = r < n.Nsr;
    bool present = false;
    if (mine) {
      const int ncx = n.srn[r];
      if (n.srtype[r] == PFCHEM_MINERAL_SURFACE) site = n.srdens[r] * W[L.vf + n.srsurf[r] - 1];
      else if (n.srtype[r] == PFCHEM_ROCK_SURFACE) site = n.srdens[r] * sc[kRhoS] * (1.0 - sc[kPor]);
      else site = n.srdens[r];
      present = site >= 1e-40;
      if (present) {
        free = W[L.srf + r];
        if (!n.srflag[r]) {
          double sumE = 0.0;
          for (int qq = 0; qq < ncx; ++qq) {
            const int k = n.src[r][qq];
            double s = W[L.bs + k];
            for (int l = 0; l < n.sn[k]; ++l) s += n.snu[k][l] * W[L.la + n.sid[k][l]];
            Sk[qq] = exp(s);
            sumE += Sk[qq];
          }
          free = site / (1.0 + sumE);
          for (int qq = 0; qq < ncx; ++qq) Sk[qq] *= free;
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
            for (int qq = 0; qq < ncx; ++qq) {
              const int k = n.src[r][qq];
              double s = W[L.bs + k] + n.sfs[k] * lf;
              for (int l = 0; l < n.sn[k]; ++l) s += n.snu[k][l] * W[L.la + n.sid[k][l]];
              Sk[qq] = exp(s);
              total += n.sfs[k] * Sk[qq];
              d += n.sfs[k] * Sk[qq] / free;
            }
            if (one_more) break;
            const double dfree = (site - total) / d;
            if (it > 1000) damping = 0.5;
            free = free + damping * dfree;
            if (fabs(dfree) < 1e-12 * fabs(free)) one_more = true;
          }
        }
        W[L.srf + r] = free;
      }
    }
    for (int rr = 0; rr < n.Nsr; ++rr) {
      if (mine && rr == r && present) {
        const int ncx = n.srn[r];
        double dSx[PFCHEM_MAX_PRI];
        for (int j = 0; j < N; ++j) dSx[j] = 0.0;
        double den = 0.0;
        for (int qq = 0; qq < ncx; ++qq) {
          const int k = n.src[r][qq];
          if (jac)
            for (int l = 0; l < n.sn[k]; ++l) dSx[n.sid[k][l]] += n.snu[k][l] * n.sfs[k] * Sk[qq];
          den += n.sfs[k] * n.sfs[k] * Sk[qq];
        }
        const double iden = -1.0 / (den / free + 1.0);
        const double ifree = 1.0 / free;
        for (int qq = 0; qq < ncx; ++qq) {
          const int k = n.src[r][qq];
          const double nuS = n.sfs[k] * Sk[qq] * ifree;
          for (int l = 0; l < n.sn[k]; ++l) {
            const int i = n.sid[k][l];
            const double v = n.snu[k][l] * Sk[qq];
            W[L.Sg + i] += v;
            W[L.aS + i] += fabs(v);
          }
          if (jac && exact) {
            double tt[PFCHEM_MAX_PRI];
            for (int j = 0; j < N; ++j) tt[j] = nuS * dSx[j] * iden;
            for (int l = 0; l < n.sn[k]; ++l) tt[n.sid[k][l]] += n.snu[k][l] * Sk[qq];
            for (int p = 0; p < n.sn[k]; ++p)
              for (int j = 0; j < N; ++j) J[n.sid[k][p] * RS + j] += n.snu[k][p] * (tt[j] * vt);
          } else if (jac) {
            for (int l = 0; l < n.sn[k]; ++l) {
              const int j = n.sid[k][l];
              const double tt = (n.snu[k][l] * Sk[qq] + nuS * dSx[j] * iden) * vt;
              for (int p = 0; p < n.sn[k]; ++p) J[n.sid[k][p] * RS + j] += n.snu[k][p] * tt;
            }
          }
        }
      }
      q.sync();
    }
  }
  // accumulation residual and its magnitude scale
  for (int j = q.g; j < N; j += G) {
    W[L.F + j] = sc[kAcc] * (sc[kPsvDen] * W[L.P + j] + sc[kVol] * W[L.Sg + j]) - W[L.fx + j];
    W[L.Sc + j] = sc[kAcc] * (sc[kPsvDen] * W[L.aP + j] + sc[kVol] * W[L.aS + j]) + fabs(W[L.fx + j]);
  }
  q.sync();
  // kinetic minerals (RKineticMineral): one mineral per lane, terms added in mineral order
  for (int base = 0; base < n.Nm; base += G) {
    const int mm = base + q.g;
    const bool mine = mm < n.Nm;
    bool on = false;
    double QK = 0.0, lnQK = 0.0, aff = 0.0, sig = 1.0, Imc = 0.0, kr = 0.0, ImV = 0.0;
    double pref[PFCHEM_MAX_PREF], lps[PFCHEM_MAX_PREF][PFCHEM_MAX_PREF_SPEC];
    if (mine) {
      const int nz = n.mn[mm];
      lnQK = W[L.bm + mm];
      for (int k = 0; k < nz; ++k) lnQK += n.mnu[mm][k] * W[L.la + n.mid[mm][k]];
      QK = (lnQK <= 6.90776) ? exp(lnQK) : 1e3;
      if (n.has_temkin) sig = n.mtemkin[mm];
      if (n.has_minscale) sig *= n.mscale[mm];
      aff = (n.has_temkin || n.has_minscale) ? 1.0 - pow(QK, 1.0 / sig) : 1.0 - QK;
      const double sign_ = csgn1(aff);
      W[L.rate + mm] = 0.0;
      on = (W[L.vf + mm] > 0.0 || sign_ < 0.0);
      if (on && n.mthr[mm] > 0.0 && sign_ < 0.0 && QK < n.mthr[mm]) on = false;
      if (on) {
        if (n.mlim[mm] > 0.0) aff = aff / (1.0 + (1.0 - aff) / n.mlim[mm]);
        kr = W[L.rk + mm];
        if (n.mpn[mm] > 0) {
          kr = 0.0;
          for (int p = 0; p < n.mpn[mm]; ++p) {
            double lp = 0.0;
            for (int s = 0; s < n.mps[mm][p]; ++s) {
              const double lsa = coop_pref_lnact(n, W, L, n.mpid[mm][p][s]);
              const double lnum = n.mpa[mm][p][s] * lsa;
              const double lden = log(1.0 + exp(log(n.mpatt[mm][p][s]) + n.mpb[mm][p][s] * lsa));
              lp = lp + lnum;
              lp = lp - lden;
              lps[p][s] = lnum - lden;
            }
            pref[p] = exp(lp);
            kr = kr + pref[p] * W[L.pk + mm * PFCHEM_MAX_PREF + p];
          }
        }
        Imc = -W[L.ar + mm];
        if (n.has_minscale) Imc = Imc / n.mscale[mm];
        double Im;
        if (n.has_affpow) Im = Imc * sign_ * pow(fabs(aff), n.mpow[mm]) * kr;
        else Im = Imc * sign_ * fabs(aff) * kr;
        W[L.rate + mm] = Im;
        ImV = Im * sc[kVol];
      }
    }
    const int last = min(n.Nm, base + G);
    for (int r = base; r < last; ++r) {
      if (mine && on && r == mm) {
        const int nz = n.mn[mm];
        for (int k = 0; k < nz; ++k) {
          const int i = n.mid[mm][k];
          const double v = n.mnu[mm][k] * ImV;
          W[L.F + i] += v;
          W[L.Sc + i] += fabs(v);
        }
        if (jac && !(exact && lnQK > 6.90776)) {
          double dIm_dQK = n.has_affpow ? -ImV * n.mpow[mm] / (exact ? aff : fabs(aff)) : -(Imc * sc[kVol]) * kr;
          if (n.has_temkin || n.has_minscale) dIm_dQK = dIm_dQK * (1.0 / sig) / QK * (1.0 - aff);
          double gq = dIm_dQK * QK * (exact ? 1.0 : sc[kDenL]);
          if (n.mlim[mm] > 0.0) {
            const double d2 = 1.0 + (1.0 - aff) / n.mlim[mm];
            gq = gq * (1.0 + QK / n.mlim[mm] / d2) / d2;
          }
          for (int qq = 0; qq < nz; ++qq) {
            const int j = n.mid[mm][qq];
            const double tt = gq * n.mnu[mm][qq];
            for (int k = 0; k < nz; ++k) J[n.mid[mm][k] * RS + j] += n.mnu[mm][k] * tt;
          }
        }
        if (jac && n.mpn[mm] > 0) {
          const double dIm_dsum = ImV / kr;
          for (int p = 0; p < n.mpn[mm]; ++p) {
            const double lpf = log(pref[p]);
            for (int s = 0; s < n.mps[mm][p]; ++s) {
              const int id = n.mpid[mm][p][s];
              const double lsa = coop_pref_lnact(n, W, L, id);
              const double gs = id >= 0 ? W[L.gam + id] : exp(W[L.bK - id - 1] - W[L.bc - id - 1]);
              const double a_ = n.mpa[mm][p][s], b_ = n.mpb[mm][p][s], att = n.mpatt[mm][p][s];
              const double dpp = exp(lpf - lps[p][s]);
              const double num = a_ * exp(lps[p][s] - lsa);
              const double lgb = b_ * lsa;
              const double den = 1.0 + exp(log(att) + lgb);
              const double dden = -1.0 * exp(lps[p][s]) / den * att * b_ * exp(lgb - lsa);
              const double dIm = dIm_dsum * dpp * ((num + dden) * gs) * W[L.pk + mm * PFCHEM_MAX_PREF + p];
              if (id >= 0) {
                const double tt = dIm * W[L.m + id];
                for (int k = 0; k < nz; ++k) J[n.mid[mm][k] * RS + id] += n.mnu[mm][k] * tt;
              } else {
                const int ci = -id - 1;
                for (int jj = 0; jj < n.cn[ci]; ++jj) {
                  const int j = n.cid[ci][jj];
                  const double tt = n.cnu[ci][jj] * W[L.C + ci] * dIm;
                  if (exact)
                    for (int k = 0; k < nz; ++k) J[n.mid[mm][k] * RS + j] += n.mnu[mm][k] * tt;
                  else
                    for (int k = 0; k < n.cn[ci]; ++k) J[n.cid[ci][k] * RS + j] += n.cnu[ci][k] * tt;
                }
              }
            }
          }
        }
      }
      q.sync();
    }
  }
  return q.any(status != 0) ? PFCHEM_CELL_INNER_MAXITER : 0;
}

// Convergence test of the group's residual; rn = the residual norm in the
// test's units (alternative-guess choice).
template <int G>
__device__ bool coop_converged(const DevNet &n, const Grp<G> &q, const double *W, const CoopLayout &L, bool *bad,
                               double *rn) {
  bool conv = true, nf = false;
  double r = 0.0;
  for (int j = q.g; j < n.N; j += G) {
    const double f = fabs(W[L.F + j]);
    if (!(f <= 1.7976931348623157e308)) nf = true;
    if (n.resid_kind == PFCHEM_RESIDUAL_RELATIVE) {
      if (!(f < n.res_tol * W[L.Sc + j])) conv = false;
      r = fmax(r, f / W[L.Sc + j]);
    } else {
      if (!(f < n.res_tol)) conv = false;
      r = fmax(r, f);
    }
  }
  *bad = q.any(nf);
  *rn = q.max(r);
  return !q.any(!conv) && !*bad;
}

// Gaussian elimination on [J | F] (row stride N + 1) with the specialized
// kernel's pivoting: |a_ij| / 2^e_i, 2^e_i the power of two of row i's largest
// entry, ties to the later row.  Solution into column N.  False for a zero row.
template <int G>
__device__ bool coop_lu_solve(const DevNet &n, const Grp<G> &q, double *W, const CoopLayout &L) {
  const int N = n.N, RS = N + 1;
  double *J = W + L.J;
  long long *E = reinterpret_cast<long long *>(W + L.E);
  bool zero = false;
  for (int i = q.g; i < N; i += G) {
    long long r = 0;
    for (int k = 0; k < N; ++k) {
      const long long v = cabsbits(J[i * RS + k]);
      r = v > r ? v : r;
    }
    if (r == 0) zero = true;
    E[i] = r & 0x7FF0000000000000LL;
  }
  if (q.any(zero)) return false;
  q.sync();
  for (int j = 0; j < N; ++j) {
    long long best = LLONG_MIN;
    int p = -1;
    for (int i = j + q.g; i < N; i += G) {
      const long long kk = cabsbits(J[i * RS + j]) - E[i];
      if (kk >= best) {
        best = kk;
        p = i;
      }
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
      const long long ob = __shfl_xor_sync(q.mask, best, o, G);
      const int op = __shfl_xor_sync(q.mask, p, o, G);
      if (ob > best || (ob == best && op > p)) {
        best = ob;
        p = op;
      }
    }
    if (p != j) {
      for (int k = j + q.g; k <= N; k += G) {
        const double t = J[p * RS + k];
        J[p * RS + k] = J[j * RS + k];
        J[j * RS + k] = t;
      }
      if (q.g == 0) E[p] = E[j];
    }
    q.sync();
    if (q.g == 0) {
      double piv = J[j * RS + j];
      if (piv == 0.0) piv = 1e-20;
      J[j * RS + j] = 1.0 / piv;
    }
    q.sync();
    const double ip = J[j * RS + j];
    for (int i = j + 1 + q.g; i < N; i += G) J[i * RS + j] = J[i * RS + j] * ip;
    q.sync();
    const int w = N - j;  // columns j+1 .. N
    for (int e = q.g; e < (N - 1 - j) * w; e += G) {
      const int i = j + 1 + e / w, k = j + 1 + e % w;
      J[i * RS + k] = fma(-J[i * RS + j], J[j * RS + k], J[i * RS + k]);
    }
    q.sync();
  }
  for (int i = N - 1; i >= 0; --i) {
    if (q.g == 0) J[i * RS + N] = J[i * RS + N] * J[i * RS + i];
    q.sync();
    const double x = J[i * RS + N];
    for (int r = q.g; r < i; r += G) J[r * RS + N] = fma(-J[r * RS + i], x, J[r * RS + N]);
    q.sync();
  }
  return true;
}

// One Newton iteration (reaction.F90:3411-3504).  Returns -1 to continue,
// else the cell's status.
template <int G>
__device__ int coop_newton_step(const DevNet &n, const CoopTables *t, const Grp<G> &q, double *W,
                                const CoopLayout &L, int iter) {
  const int N = n.N, RS = N + 1;
  if (n.act_freq == PFCHEM_ACT_COEF_FREQUENCY_NEWTON_ITER && iter > 1) {
    double I = 0.0;
    for (int j = q.g; j < N; j += G) I += W[L.m + j] * n.Z2p[j];
    for (int i = q.g; i < n.Nc; i += G) I += W[L.C + i] * n.cZ2[i];
    I = q.sum(I) * 0.5;
    q.sync();
    coop_activity<G>(n, q, W, L, I);
  }
  const bool rescue = n.exact_after > 0 && iter > n.exact_after;
  const int st = coop_evaluate<G>(n, t, q, W, L, true, n.jac_exact || rescue);
  if (st) return st;
  bool bad;
  double rn;
  const bool conv = coop_converged<G>(n, q, W, L, &bad, &rn);
  if (bad) return PFCHEM_CELL_NONFINITE;
  if (conv) return PFCHEM_CELL_CONVERGED;
  if (iter >= n.max_iter) return PFCHEM_CELL_MAXITER;
  double *J = W + L.J;
  for (int j = q.g; j < N; j += G) J[j * RS + N] = W[L.F + j];
  q.sync();
  if (!coop_lu_solve<G>(n, q, W, L)) return PFCHEM_CELL_SINGULAR;
  double mrc = 0.0;
  bool nf = false;
  const bool damp = iter > 50 && !rescue;
  for (int j = q.g; j < N; j += G) {
    const double x = J[j * RS + N];
    const double u = csgn1(x) * fmin(fabs(x), n.max_dlnC);
    const double e = exp(-u);
    double mnew = W[L.m + j] * e;
    mrc = fmax(mrc, fabs(e - 1.0));
    if (!(fabs(mnew) <= 1.7976931348623157e308)) nf = true;
    J[j * RS + N] = u;  // the clamped update
    W[L.sm + j] = mnew;
  }
  if (q.any(nf)) return PFCHEM_CELL_NONFINITE;
  mrc = q.max(mrc);
  if (n.rel_change_tol > 0.0 && mrc < n.rel_change_tol) return PFCHEM_CELL_CONVERGED;
  for (int j = q.g; j < N; j += G) {
    const double m = W[L.m + j];
    double mnew = W[L.sm + j];
    if (damp) {
      // reaction.F90:3478-3496 (only the 0.1 branch is reachable)
      mnew = 0.1 * (mnew - m) + m;
      W[L.m + j] = mnew;
      W[L.lm + j] = log(mnew);
    } else {
      W[L.m + j] = mnew;
      W[L.lm + j] -= J[j * RS + N];
    }
  }
  q.sync();
  return -1;
}

template <int G>
__device__ void coop_finalize(const DevNet &n, const CellArgs &a, int64_t cell, const Grp<G> &q, const double *W,
                              const CoopLayout &L, int status, int iter) {
  const int64_t nc = a.ncells;
  const double *sc = W + L.sc;
  double I = 0.0;
  for (int j = q.g; j < n.N; j += G) {
    const double m = W[L.m + j];
    a.pri_molal[j * nc + cell] = m;
    if (a.interleaved_out) a.interleaved_out[j * a.total_stride_comp + cell * a.total_stride_cell] = m;
    if (a.total_out) a.total_out[j * nc + cell] = W[L.P + j] * sc[kDenL];
    if (a.sorb) a.sorb[j * nc + cell] = W[L.Sg + j];
    I += m * n.Z2p[j];
  }
  for (int i = q.g; i < n.Nc; i += G) {
    I += W[L.C + i] * n.cZ2[i];
    if (a.sec_molal) a.sec_molal[i * nc + cell] = W[L.C + i];
  }
  I = q.sum(I);
  for (int k = q.g; k < n.Nm; k += G) {
    if (a.rate) a.rate[k * nc + cell] = W[L.rate + k];
    if (n.update_kin && status == PFCHEM_CELL_CONVERGED) {
      double v = W[L.vf + k] + W[L.rate + k] * n.mVm[k] * sc[kDt];
      if (v < 0.0) v = 0.0;
      a.vf[k * nc + cell] = v;
    }
  }
  for (int r = q.g; r < n.Nix; r += G) a.ixref[r * nc + cell] = W[L.ixr + r];
  for (int r = q.g; r < n.Nsr; r += G) a.srfree[r * nc + cell] = W[L.srf + r];
  if (q.g == 0) {
    a.ionic[cell] = 0.5 * I;
    if (a.iters) a.iters[cell] = iter;
    if (a.status) a.status[cell] = status;
  }
}

// Persistent grid of groups of G lanes; each group takes cells from the
// work queue one at a time.
template <int G>
__global__ void __launch_bounds__(128) coop_react_kernel(const __grid_constant__ DevNet n,
                                                         const __grid_constant__ CellArgs a,
                                                         const CoopTables *__restrict__ t, Scratch *scr,
                                                         double inv_dt, int group_doubles) {
  extern __shared__ double smem[];
  const int lane = threadIdx.x & 31;
  Grp<G> q;
  q.g = lane % G;
  q.mask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (lane / G * G));
  double *W = smem + (size_t)(threadIdx.x / G) * group_doubles;
  const CoopLayout L = coop_layout(n);
  const int64_t nc = a.ncells;
  unsigned long long my_iters = 0, my_alt = 0;
  unsigned my_max = 0, my_bad = 0;
  for (;;) {
    unsigned long long c = 0;
    if (q.g == 0) c = atomicAdd(&scr->next_cell, 1ull);
    c = __shfl_sync(q.mask, c, 0, G);
    if (c >= (unsigned long long)nc) {
      if (q.g == 0) atomicMax(&scr->t_drain_inv, ~pf_now());
      break;
    }
    const int64_t cell = (int64_t)c;
    if (a.active && a.active[cell] <= 0) {
      if (q.g == 0) {
        if (a.status) a.status[cell] = PFCHEM_CELL_INACTIVE;
        if (a.iters) a.iters[cell] = 0;
      }
      continue;
    }
    coop_setup<G>(n, a, cell, q, W, L, inv_dt);
    bool alt_used = false;
    if (a.alt_guess) {
      // the residual at the plain guess and at the alternative guess; Newton
      // starts from the better one, with the ion-exchange warm starts of the
      // evaluation it chose and the surface free sites as given
      for (int j = q.g; j < n.N; j += G) {
        W[L.sm + j] = W[L.m + j];
        W[L.slm + j] = W[L.lm + j];
      }
      for (int r = q.g; r < n.Nsr; r += G) W[L.sfree + r] = W[L.srf + r];
      q.sync();
      coop_evaluate<G>(n, t, q, W, L, false, n.jac_exact);
      bool bad;
      double rn;
      coop_converged<G>(n, q, W, L, &bad, &rn);
      const double rplain = bad ? 1.7976931348623157e308 : rn;
      for (int r = q.g; r < n.Nix; r += G) W[L.sixr + r] = W[L.ixr + r];
      for (int r = q.g; r < n.Nsr; r += G) W[L.srf + r] = W[L.sfree + r];
      bool ok = true;
      for (int j = q.g; j < n.N; j += G) {
        const double gv = a.alt_guess[j * nc + cell];
        if (gv > 0.0 && gv <= 1.7976931348623157e308) {
          W[L.m + j] = gv;
          W[L.lm + j] = log(gv);
        } else {
          ok = false;
        }
      }
      ok = !q.any(!ok);
      q.sync();
      double ralt = 1.7976931348623157e308;
      if (ok) {
        const int st = coop_evaluate<G>(n, t, q, W, L, false, n.jac_exact);
        coop_converged<G>(n, q, W, L, &bad, &rn);
        if (!bad && st == 0) ralt = rn;
      }
      alt_used = ralt <= rplain;
      if (!alt_used) {
        for (int j = q.g; j < n.N; j += G) {
          W[L.m + j] = W[L.sm + j];
          W[L.lm + j] = W[L.slm + j];
        }
        for (int r = q.g; r < n.Nix; r += G) W[L.ixr + r] = W[L.sixr + r];
      }
      for (int r = q.g; r < n.Nsr; r += G) W[L.srf + r] = W[L.sfree + r];
      q.sync();
    }
    int iter = 0, st = -1;
    while (st < 0) st = coop_newton_step<G>(n, t, q, W, L, ++iter);
    coop_finalize<G>(n, a, cell, q, W, L, st, iter);
    q.sync();
    if (q.g == 0) {
      my_iters += iter;
      my_max = max(my_max, (unsigned)iter);
      my_bad += st != PFCHEM_CELL_CONVERGED;
      my_alt += alt_used;
    }
  }
  if (q.g == 0) {
    atomicAdd(&scr->sum_iter, my_iters);
    atomicAdd(&scr->alt_used, my_alt);
    atomicMax(&scr->max_iter, my_max);
    atomicAdd(&scr->nonconverged, my_bad);
    atomicMax(&scr->t_end, pf_now());
  }
}

}  // namespace

// Host side -------------------------------------------------------------------

// Whether the cooperative kernel computes this network's options.
bool coop_supports(const DevNet &n) {
  return n.use_log && !n.act_newton && !n.use_h2o;
}

// Shared-memory doubles of one cell group.
int coop_group_doubles(const DevNet &n) { return coop_layout(n).total; }

// Builds the gather lists for `n` into host memory `t`.
void coop_build_tables(const DevNet &n, CoopTables *t) {
  std::memset(t, 0, sizeof(*t));
  int e = 0;
  for (int j = 0; j < n.N; ++j) {
    t->sp_ptr[j] = (int16_t)e;
    for (int i = 0; i < n.Nc; ++i)
      for (int k = 0; k < n.cn[i]; ++k)
        if (n.cid[i][k] == j) {
          t->sp_cplx[e] = (int16_t)i;
          t->sp_nu[e] = n.cnu[i][k];
          ++e;
        }
  }
  t->sp_ptr[n.N] = (int16_t)e;
  e = 0;
  for (int l = 0; l < n.N; ++l)
    for (int k = 0; k < n.N; ++k) {
      t->je_ptr[l * n.N + k] = (int16_t)e;
      for (int i = 0; i < n.Nc; ++i)
        for (int p = 0; p < n.cn[i]; ++p)
          for (int r = 0; r < n.cn[i]; ++r)
            if (n.cid[i][p] == l && n.cid[i][r] == k) {
              t->je_cplx[e] = (int16_t)i;
              t->je_nu[e] = n.cnu[i][p] * n.cnu[i][r];
              ++e;
            }
    }
  t->je_ptr[n.N * n.N] = (int16_t)e;
}

size_t coop_tables_bytes() { return sizeof(CoopTables); }

template <int G>
static cudaError_t coop_launch_t(const DevNet &n, const CellArgs &a, const void *t, Scratch *scr, int grid,
                                 int block, cudaStream_t st) {
  // the shared-memory limit was raised by coop_blocks_per_sm (called when the
  // launch was chosen, outside any stream capture)
  const int gd = coop_group_doubles(n);
  const size_t shm = (size_t)(block / G) * gd * sizeof(double);
  if (shm > 227 * 1024) return cudaErrorInvalidValue;
  coop_react_kernel<G><<<grid, block, shm, st>>>(n, a, (const CoopTables *)t, scr, 1.0 / a.dt, gd);
  return cudaGetLastError();
}

cudaError_t coop_launch(int lanes, const DevNet &n, const CellArgs &a, const void *tables, Scratch *scr, int grid,
                        int block, cudaStream_t st) {
  switch (lanes) {
    case 8: return coop_launch_t<8>(n, a, tables, scr, grid, block, st);
    case 16: return coop_launch_t<16>(n, a, tables, scr, grid, block, st);
    case 32: return coop_launch_t<32>(n, a, tables, scr, grid, block, st);
    default: return cudaErrorInvalidValue;
  }
}

template <int G>
static int coop_blocks_per_sm_t(const DevNet &n, int block) {
  const size_t shm = (size_t)(block / G) * coop_group_doubles(n) * sizeof(double);
  if (shm > 227 * 1024) return 0;
  if (cudaFuncSetAttribute(coop_react_kernel<G>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024) !=
      cudaSuccess)
    return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, coop_react_kernel<G>, block, shm) != cudaSuccess) return 0;
  return nb;
}

int coop_blocks_per_sm(int lanes, const DevNet &n, int block) {
  switch (lanes) {
    case 8: return coop_blocks_per_sm_t<8>(n, block);
    case 16: return coop_blocks_per_sm_t<16>(n, block);
    case 32: return coop_blocks_per_sm_t<32>(n, block);
    default: return 0;
  }
}

}  // namespace pfchem
