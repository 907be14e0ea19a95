// pfchem_device.cuh -- device-side network description and kernel arguments.
//
// The host (pfchem_api.cu) flattens a pfchem_network into a DevNet: 0-based
// species ids, stoichiometry with pre-computed |nu|, squared charges, and the
// per-reaction constants the Newton kernel needs.  A DevNet is passed to the
// kernels by value as a __grid_constant__ parameter, so it lives in the
// constant bank (uniform reads broadcast across a warp) and every context
// keeps its own network without global device state.
#pragma once
#include <stdint.h>

#include "../../include/pfchem.h"

namespace pfchem {

constexpr double kLOG_TO_LN = 2.30258509299;    // pflotran_constants.F90:48
constexpr double kIDEAL_GAS_CONSTANT = 8.31446;  // pflotran_constants.F90:53

// Power kinds of KDj^(Z_j / Z_ref) in the ion-exchange inner Newton.
enum : int8_t { kPowOne = 0, kPowTwo = 1, kPowHalf = 2, kPowGeneric = 3 };

struct DevNet {
  int32_t N, Nc, Nm, Nix, Nsr, Nsc;
  // options
  int32_t use_log, act_freq, use_h2o, isothermal, resid_kind, accum_mode, max_iter, update_kin;
  int32_t has_temkin, has_minscale, has_affpow, has_h2o_rxn;
  int32_t jac_exact;  // PFCHEM_JACOBIAN_EXACT
  int32_t exact_after;  // exact_jacobian_after (0: never)
  int32_t act_newton;   // ACT_COEF_ALGORITHM_NEWTON
  double max_dlnC, rel_change_tol, res_tol;
  double A, B, Bdot;
  // primaries
  double Z2p[PFCHEM_MAX_PRI], ap[PFCHEM_MAX_PRI], Zp[PFCHEM_MAX_PRI];
  // aqueous complexes
  int8_t cn[PFCHEM_MAX_CPLX];
  int8_t cid[PFCHEM_MAX_CPLX][PFCHEM_MAX_NNZ];
  double cnu[PFCHEM_MAX_CPLX][PFCHEM_MAX_NNZ];
  double cZ2[PFCHEM_MAX_CPLX], ca[PFCHEM_MAX_CPLX], ch2o[PFCHEM_MAX_CPLX];
  double clogK[PFCHEM_MAX_CPLX];
  double ccoef[PFCHEM_MAX_CPLX][5];
  // kinetic minerals
  int8_t mn[PFCHEM_MAX_MNRL];
  int8_t mid[PFCHEM_MAX_MNRL][PFCHEM_MAX_NNZ];
  double mnu[PFCHEM_MAX_MNRL][PFCHEM_MAX_NNZ];
  double mh2o[PFCHEM_MAX_MNRL], mlogK[PFCHEM_MAX_MNRL], mcoef[PFCHEM_MAX_MNRL][5];
  double mk[PFCHEM_MAX_MNRL], mEa[PFCHEM_MAX_MNRL], mVm[PFCHEM_MAX_MNRL];
  double mthr[PFCHEM_MAX_MNRL], mlim[PFCHEM_MAX_MNRL];
  double mtemkin[PFCHEM_MAX_MNRL], mscale[PFCHEM_MAX_MNRL], mpow[PFCHEM_MAX_MNRL];
  // rate prefactors (reaction_mineral.F90:743-782): per mineral the number of
  // prefactors; per prefactor its species count, rate constant and
  // activation energy; per species its id (>= 0: primary, 0-based; < 0:
  // aqueous complex -(i + 1)), alpha, beta and attenuation coefficient
  int8_t mpn[PFCHEM_MAX_MNRL];
  int8_t mps[PFCHEM_MAX_MNRL][PFCHEM_MAX_PREF];
  int8_t mpid[PFCHEM_MAX_MNRL][PFCHEM_MAX_PREF][PFCHEM_MAX_PREF_SPEC];
  double mpk[PFCHEM_MAX_MNRL][PFCHEM_MAX_PREF], mpEa[PFCHEM_MAX_MNRL][PFCHEM_MAX_PREF];
  double mpa[PFCHEM_MAX_MNRL][PFCHEM_MAX_PREF][PFCHEM_MAX_PREF_SPEC];
  double mpb[PFCHEM_MAX_MNRL][PFCHEM_MAX_PREF][PFCHEM_MAX_PREF_SPEC];
  double mpatt[PFCHEM_MAX_MNRL][PFCHEM_MAX_PREF][PFCHEM_MAX_PREF_SPEC];
  int32_t has_pref;
  // ion exchange
  int8_t xn[PFCHEM_MAX_IONX], xzflag[PFCHEM_MAX_IONX], xsurf[PFCHEM_MAX_IONX];
  int8_t xid[PFCHEM_MAX_IONX][PFCHEM_MAX_NNZ];
  int8_t xpow[PFCHEM_MAX_IONX][PFCHEM_MAX_NNZ];
  double xk[PFCHEM_MAX_IONX][PFCHEM_MAX_NNZ];
  double xzr[PFCHEM_MAX_IONX][PFCHEM_MAX_NNZ];  // Z_j / Z_ref
  double xCEC[PFCHEM_MAX_IONX];
  // surface complexation (reactions, then their complexes)
  int8_t srn[PFCHEM_MAX_SRFRXN], srtype[PFCHEM_MAX_SRFRXN], srsurf[PFCHEM_MAX_SRFRXN], srflag[PFCHEM_MAX_SRFRXN];
  int8_t src[PFCHEM_MAX_SRFRXN][PFCHEM_MAX_NNZ];
  double srdens[PFCHEM_MAX_SRFRXN];
  int8_t sn[PFCHEM_MAX_SRFCPLX];
  int8_t sid[PFCHEM_MAX_SRFCPLX][PFCHEM_MAX_NNZ];
  double snu[PFCHEM_MAX_SRFCPLX][PFCHEM_MAX_NNZ];
  double sfs[PFCHEM_MAX_SRFCPLX], sh2o[PFCHEM_MAX_SRFCPLX], slogK[PFCHEM_MAX_SRFCPLX];
  double scoef[PFCHEM_MAX_SRFCPLX][5];
};

// Per-call pointers (device memory, SoA, field(i, cell) at [i * ncells + cell]).
// The field lists are macros so that the network-specialized kernels, which
// are compiled at run time, declare byte-identical structures.
#define PFCHEM_CELLARGS_FIELDS                                                          \
  int64_t ncells;                                                                     \
  double dt;                                                                          \
  const double *temp, *sat, *den, *por, *vol, *rho_s;                                 \
  const int32_t *active;                                                              \
  const double *total;                                                                \
  int64_t total_stride_cell; /* 1 for SoA; ncomp for RTReact's interleaved tran_xx */ \
  int64_t total_stride_comp; /* ncells for SoA; 1 for interleaved */                  \
  double *pri_molal, *ionic, *lnaw, *vf, *area, *sorb, *ixref, *srfree;               \
  double *total_out, *rate, *sec_molal;                                               \
  int32_t *iters, *status;                                                            \
  const double *alt_guess;                                                            \
  double *interleaved_out; /* RTReact layout write-back of the free ions, or null */

// Work queue and statistics: global memory the solve kernel uses besides its
// inputs and outputs.
#define PFCHEM_SCRATCH_FIELDS                            \
  unsigned long long next_cell; /* work-queue head */ \
  unsigned long long sum_iter;                        \
  unsigned long long alt_used;                        \
  unsigned long long newton_trips; /* warp trips of Newton steps */ \
  unsigned long long t_drain_inv;  /* ~(first time the queue ran dry), ns */ \
  unsigned long long t_end;        /* last warp exit, ns */ \
  unsigned int max_iter;                              \
  unsigned int nonconverged;                          \
  unsigned int armor_flag; /* mineral armoring flag after the last cell */ \
  unsigned int pad_;

struct CellArgs {
  PFCHEM_CELLARGS_FIELDS
};

struct Scratch {
  PFCHEM_SCRATCH_FIELDS
};

// global nanosecond timer (queue-drain statistics only)
#define PFCHEM_GLOBALTIMER_FN \
  __device__ __forceinline__ unsigned long long pf_now() { \
    unsigned long long t; asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t)); return t; }

#define PFCHEM_STR_(...) #__VA_ARGS__
#define PFCHEM_STR(...) PFCHEM_STR_(__VA_ARGS__)

struct LaunchCfg {
  int refill_min_idle;
};

}  // namespace pfchem
