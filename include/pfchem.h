/*
 * pfchem.h -- C ABI of the GB300 (sm_103a) batched per-cell geochemistry library.
 *
 * The library replaces the body of PFLOTRAN's operator-split reaction loop:
 *   RTReact cell loop            src/pflotran/reactive_transport.F90:1697-1724
 *   RReact (per-cell Newton)     src/pflotran/reaction.F90:3322-3511
 *   RTUpdateKineticState loop    src/pflotran/reactive_transport.F90:692-705
 *   RUpdateKineticState          src/pflotran/reaction.F90:5320-5429
 * with one batched call over all cells of a rank, executed on one GPU.
 *
 * Conventions
 *  - Every table in pfchem_network has the shape and meaning of the field of
 *    the same name in PFLOTRAN's reaction_type (src/pflotran/reaction_aux.F90:142-335,
 *    reaction_mineral_aux.F90:76-132, reaction_surf_complex_aux.F90:68-128):
 *    Fortran column-major, species ids 1-based, id tables dimensioned (0:ld, n)
 *    with row 0 holding the count.  A Fortran caller passes c_loc() of its
 *    own arrays; nothing is re-indexed on the caller side.
 *  - Per-cell arrays are structure-of-arrays, cell fastest:
 *    field(i, cell) lives at ptr[i * ncells + cell].
 *  - Return codes: 0 = OK, < 0 = API or CUDA error (see pfchem_last_error),
 *    > 0 = number of cells whose per-cell status is not PFCHEM_CELL_CONVERGED.
 *    The library never aborts the process and never traps on the device.
 *  - One context per host thread.  Calls are stream ordered on the context's
 *    stream and synchronous on return.
 */
#ifndef PFCHEM_H
#define PFCHEM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Compile-time limits of the device kernels (checked by pfchem_set_network). */
#define PFCHEM_MAX_PRI 16       /* primary aqueous species (naqcomp)          */
#define PFCHEM_MAX_CPLX 64      /* aqueous complexes (neqcplx)                */
#define PFCHEM_MAX_MNRL 16      /* kinetic minerals (nkinmnrl)                */
#define PFCHEM_MAX_IONX 8       /* ion-exchange reactions (neqionxrxn)        */
#define PFCHEM_MAX_SRFRXN 8     /* surface-complexation reactions             */
#define PFCHEM_MAX_SRFCPLX 32   /* surface complexes (nsrfcplx)               */
#define PFCHEM_MAX_NNZ 8        /* species per reaction (leading dimensions)  */
#define PFCHEM_MAX_PREF 4       /* rate prefactors per mineral                */
#define PFCHEM_MAX_PREF_SPEC 4  /* species per prefactor                      */

/* reaction_aux.F90:23-27 */
#define PFCHEM_ACT_COEF_FREQUENCY_OFF 0
#define PFCHEM_ACT_COEF_FREQUENCY_TIMESTEP 1
#define PFCHEM_ACT_COEF_FREQUENCY_NEWTON_ITER 2
#define PFCHEM_ACT_COEF_ALGORITHM_LAG 3
#define PFCHEM_ACT_COEF_ALGORITHM_NEWTON 4

/* reaction_surf_complex_aux.F90:19-22 */
#define PFCHEM_NULL_SURFACE 0
#define PFCHEM_COLLOID_SURFACE 1 /* rejected: colloids are not supported      */
#define PFCHEM_MINERAL_SURFACE 2
#define PFCHEM_ROCK_SURFACE 3

/* Residual convergence test (pfchem_options.residual_tol_kind). */
#define PFCHEM_RESIDUAL_ABSOLUTE 0 /* max_j |F_j| < tol, F in mol/s (reaction.F90:3443) */
#define PFCHEM_RESIDUAL_RELATIVE 1 /* max_j |F_j| / S_j < tol, S_j = magnitude of the terms of F_j */

/* Accumulation convention (pfchem_options.accum_mode). */
#define PFCHEM_ACCUM_DT_CONSISTENT 0 /* F = (psv*T(m) + V*S(m) - fixed)/dt + R(m): the global-implicit cell equation */
#define PFCHEM_ACCUM_LITERAL 1       /* F = psv*T(m) + V*S(m) - fixed + R(m): RReact as written (reaction.F90:3424-3426) */

/* Per-cell status codes. */
#define PFCHEM_CELL_CONVERGED 0
#define PFCHEM_CELL_MAXITER 1      /* Newton iteration cap reached            */
#define PFCHEM_CELL_SINGULAR 2     /* a Jacobian row is zero (utility.F90:423) */
#define PFCHEM_CELL_NONFINITE 3    /* NaN/Inf in residual or update           */
#define PFCHEM_CELL_INNER_MAXITER 4 /* ion-exchange / surface-complexation / activity inner loop cap */
#define PFCHEM_CELL_INACTIVE 5     /* skipped (patch%imat <= 0, reactive_transport.F90:1699) */

typedef struct pfchem_network {
  /* counts */
  int32_t naqcomp;       /* reaction%naqcomp                                   */
  int32_t neqcplx;       /* reaction%neqcplx                                   */
  int32_t nkinmnrl;      /* reaction%mineral%nkinmnrl                          */
  int32_t neqionxrxn;    /* reaction%neqionxrxn                                */
  int32_t nsrfcplxrxn;   /* surface_complexation%nsrfcplxrxn (all equilibrium) */
  int32_t nsrfcplx;      /* surface_complexation%nsrfcplx                      */
  /* leading dimensions: id tables are (0:ld, n), stoich tables are (ld, n) */
  int32_t eqcplx_ld;
  int32_t kinmnrl_ld;
  int32_t eqionx_ld;
  int32_t srfcplxrxn_ld; /* srfcplxrxn_to_complex is (0:srfcplxrxn_ld, nsrfcplxrxn) */
  int32_t srfcplx_ld;
  int32_t max_num_prefactors;        /* size(kinmnrl_pref_rate,1); 0 = none  */
  int32_t max_num_prefactor_species; /* size(kinmnrl_pref_alpha,1)            */
  int32_t reserved0;

  /* primary species (reaction_aux.F90 primary_spec_Z/_a0) */
  const double *primary_spec_Z;  /* (naqcomp) */
  const double *primary_spec_a0; /* (naqcomp) ion size [Angstrom] */

  /* aqueous complexes */
  const int32_t *eqcplxspecid;    /* (0:eqcplx_ld, neqcplx) */
  const double *eqcplxstoich;     /* (eqcplx_ld, neqcplx) */
  const int32_t *eqcplxh2oid;     /* (neqcplx) or NULL */
  const double *eqcplxh2ostoich;  /* (neqcplx) or NULL */
  const double *eqcplx_Z;         /* (neqcplx) */
  const double *eqcplx_a0;        /* (neqcplx) */
  const double *eqcplx_logK;      /* (neqcplx): used when use_isothermal */
  const double *eqcplx_logKcoef;  /* (5, neqcplx) Maier-Kelly: used when !use_isothermal */

  /* Debye-Hueckel parameters at the reference temperature (reaction_database.F90:897-990) */
  double debyeA, debyeB, debyeBdot;

  /* kinetic minerals (reaction_mineral_aux.F90) */
  const int32_t *kinmnrlspecid;    /* (0:kinmnrl_ld, nkinmnrl) */
  const double *kinmnrlstoich;     /* (kinmnrl_ld, nkinmnrl) */
  const int32_t *kinmnrlh2oid;     /* (nkinmnrl) or NULL */
  const double *kinmnrlh2ostoich;  /* (nkinmnrl) or NULL */
  const double *kinmnrl_logK;      /* (nkinmnrl) */
  const double *kinmnrl_logKcoef;  /* (5, nkinmnrl) */
  const double *kinmnrl_rate_constant;      /* [mol/m^2/s] */
  const double *kinmnrl_activation_energy;  /* [J/mol]; 0 = no Arrhenius factor */
  const double *kinmnrl_molar_vol;          /* [m^3/mol] */
  const double *kinmnrl_affinity_threshold; /* 0 = off */
  const double *kinmnrl_rate_limiter;       /* 0 = off */
  const double *kinmnrl_Temkin_const;       /* NULL = not associated */
  const double *kinmnrl_min_scale_factor;   /* NULL = not associated */
  const double *kinmnrl_affinity_power;     /* NULL = not associated */
  const int32_t *kinmnrl_num_prefactors;    /* (nkinmnrl) or NULL */
  const double *kinmnrl_pref_rate;              /* (max_pref, nkinmnrl) */
  const double *kinmnrl_pref_activation_energy; /* (max_pref, nkinmnrl) */
  const int32_t *kinmnrl_prefactor_id;          /* (0:max_pref_spec, max_pref, nkinmnrl); <0 = secondary */
  const double *kinmnrl_pref_alpha;             /* (max_pref_spec, max_pref, nkinmnrl) */
  const double *kinmnrl_pref_beta;
  const double *kinmnrl_pref_atten_coef;

  /* equilibrium ion exchange */
  const int32_t *eqionx_rxn_cationid; /* (0:eqionx_ld, neqionxrxn); entry 1 = reference cation */
  const double *eqionx_rxn_k;         /* (eqionx_ld, neqionxrxn) */
  const double *eqionx_rxn_CEC;       /* (neqionxrxn) [eq/m^3 bulk] */
  const int32_t *eqionx_rxn_to_surf;  /* (neqionxrxn) mineral id or 0 */
  const int32_t *eqionx_rxn_Z_flag;   /* (neqionxrxn) logical: charges differ */

  /* equilibrium surface complexation */
  const int32_t *srfcplxrxn_to_complex;   /* (0:srfcplxrxn_ld, nsrfcplxrxn) */
  const int32_t *srfcplxrxn_surf_type;    /* (nsrfcplxrxn) PFCHEM_*_SURFACE */
  const int32_t *srfcplxrxn_to_surf;      /* (nsrfcplxrxn) mineral id for MINERAL_SURFACE */
  const double *srfcplxrxn_site_density;  /* (nsrfcplxrxn) */
  const int32_t *srfcplxrxn_stoich_flag;  /* (nsrfcplxrxn) logical */
  const int32_t *srfcplxspecid;           /* (0:srfcplx_ld, nsrfcplx) */
  const double *srfcplxstoich;            /* (srfcplx_ld, nsrfcplx) */
  const int32_t *srfcplxh2oid;            /* (nsrfcplx) or NULL */
  const double *srfcplxh2ostoich;         /* (nsrfcplx) or NULL */
  const double *srfcplx_free_site_stoich; /* (nsrfcplx) */
  const double *srfcplx_logK;             /* (nsrfcplx) */
  const double *srfcplx_logKcoef;         /* (5, nsrfcplx) */
} pfchem_network;

typedef struct pfchem_options {
  int32_t use_log_formulation;        /* reaction%use_log_formulation */
  int32_t act_coef_update_frequency;  /* PFCHEM_ACT_COEF_FREQUENCY_* */
  int32_t act_coef_update_algorithm;  /* PFCHEM_ACT_COEF_ALGORITHM_* */
  int32_t use_activity_h2o;           /* reaction%use_activity_h2o */
  int32_t use_isothermal;             /* option%use_isothermal: 1 = logK tables as given */
  int32_t residual_tol_kind;          /* PFCHEM_RESIDUAL_* */
  int32_t accum_mode;                 /* PFCHEM_ACCUM_* */
  int32_t max_iterations;             /* Newton cap (the reference has none) */
  double max_dlnC;                    /* reaction%max_dlnC (5) */
  double max_relative_change_tolerance; /* reaction%max_relative_change_tolerance (1e-6); <= 0 disables */
  double max_residual_tolerance;      /* reaction%max_residual_tolerance (1e-12) */
  int32_t update_kinetic_state;       /* 1: fuse RUpdateKineticState after the solve */
  int32_t jacobian;                   /* PFCHEM_JACOBIAN_* (0 = the reference's) */
  int32_t exact_jacobian_after;       /* 0: never; K > 0: see below */
  int32_t reserved3;                  /* 0 */
} pfchem_options;
/* exact_jacobian_after = K > 0: a cell still unconverged after K Newton
 * iterations continues with the EXACT Jacobian and without RReact's x0.1
 * damping.  RReact damps every update after iteration 50 and loops until
 * converged (reaction.F90:3478-3496; its "> 500" stop is unreachable), so a
 * cell whose reference-Jacobian Newton converges slowly crawls for hundreds
 * of iterations (on the synthetic 12-species workload 2 % of cells pass 50
 * iterations; uncapped they need a median 377 and up to ~2200).  With K = 50
 * the first 50 iterations are RReact's and such cells converge 2-4 iterations
 * later to the same root (same residual, same relative-residual test).
 * 0 reproduces RReact's damped path, cut at max_iterations. */
/* Newton Jacobian.  REFERENCE forms it as RReact does, with three
 * inexact terms that make Newton converge linearly:
 *  - RTotalSorbEqSurfCplx1 adds the free-site part of dS_k/dm_j only for the
 *    components j of complex k (reaction_surf_complex.F90:905-931), although
 *    the free-site concentration depends on every component on the site;
 *  - RKineticMineral keeps dQK/dm where QK is capped at 1e3, so a strongly
 *    supersaturated mineral contributes a derivative its rate does not have
 *    (reaction_mineral.F90:699-703, :860-872), scales dQK/dm by den_kg/1000
 *    (:867, :885), and, when kinmnrl_affinity_power is given, divides by
 *    |affinity| where the derivative has the signed affinity (:842-846),
 *    which flips the term's sign for a precipitating mineral.
 * EXACT (no counterpart in the reference) uses the derivatives of the same
 * residual: same equations, same root, fewer iterations; the rate-limiter
 * branch keeps the reference's expression apart from the affinity sign. */
#define PFCHEM_JACOBIAN_REFERENCE 0
#define PFCHEM_JACOBIAN_EXACT 1

/* One batch of cells.  Pointers are all device pointers (on_device = 1) or all
 * host pointers (on_device = 0; the library stages them through the device).
 * Arrays marked "or NULL" may be omitted. */
typedef struct pfchem_cells {
  int64_t ncells;
  int32_t on_device;
  int32_t reserved2;
  /* inputs (ncells) */
  const double *temperature;            /* global_auxvar%temp [C] */
  const double *saturation;             /* global_auxvar%sat(1) */
  const double *den_kg;                 /* global_auxvar%den_kg(1) [kg/m^3] */
  const double *porosity;               /* material_auxvar%porosity */
  const double *volume;                 /* material_auxvar%volume [m^3] */
  const double *soil_particle_density;  /* material_auxvar%soil_particle_density [kg/m^3] or NULL */
  const int32_t *active;                /* patch%imat > 0 per cell, or NULL = all active */
  const double *total;                  /* (naqcomp, ncells) transported totals tran_xx [mol/L] */
  /* state, read and written (the reactive_transport_auxvar_type fields) */
  double *pri_molal;                    /* (naqcomp, ncells) guess in, free-ion molality out */
  double *ionic_strength;               /* (ncells) I of the previous state in (LAG activity), I at the solution out */
  double *ln_act_h2o;                   /* (ncells) or NULL */
  double *mnrl_volfrac;                 /* (nkinmnrl, ncells) */
  double *mnrl_area;                    /* (nkinmnrl, ncells) [m^2/m^3 bulk] */
  double *total_sorb_eq;                /* (naqcomp, ncells) [mol/m^3 bulk] or NULL without sorption */
  double *eqionx_ref_cation_sorbed_conc;/* (neqionxrxn, ncells) or NULL */
  double *srfcplxrxn_free_site_conc;    /* (nsrfcplxrxn, ncells) or NULL */
  /* outputs */
  double *total_out;                    /* (naqcomp, ncells) aqueous totals at the solution [mol/L] or NULL */
  double *mnrl_rate;                    /* (nkinmnrl, ncells) [mol/m^3/s] or NULL */
  double *sec_molal;                    /* (neqcplx, ncells) or NULL */
  int32_t *iterations;                  /* (ncells) Newton iterations, or NULL */
  int32_t *status;                      /* (ncells) PFCHEM_CELL_*, or NULL */
  /* optional second initial guess (e.g. the learned warm start): the kernel
   * evaluates the residual at both guesses and starts from the better one */
  const double *alt_guess;              /* (naqcomp, ncells) or NULL */
} pfchem_cells;

typedef struct pfchem_stats {
  int64_t ncells;          /* cells processed by the last call        */
  int64_t sum_iterations;  /* sum of Newton iterations                */
  int32_t max_iterations;  /* max Newton iterations in a cell         */
  int32_t nonconverged;    /* cells with status != CONVERGED/INACTIVE */
  int64_t alt_guess_used;  /* cells that started from alt_guess       */
  double kernel_ms;        /* device time of the solve kernel         */
  int64_t lane_slots;      /* 32 x warp trips of Newton steps in the persistent
                              kernel: sum_iterations / lane_slots is the share
                              of SIMT lanes doing Newton work (0 if not counted) */
  double drain_ms;         /* time from the work queue running dry to the
                              last warp's exit: the straggler tail (0 if not
                              measured) */
} pfchem_stats;

typedef struct pfchem_ctx pfchem_ctx;

/* Context lifetime.  The context owns its CUDA stream, the device copy of the
 * network tables, the work-queue counters, captured graphs and the autotune
 * cache.  Replaces nothing in the reference (PFLOTRAN keeps this state in
 * reaction_type and the rt_auxvars). */
int pfchem_create(pfchem_ctx **ctx, int device);
void pfchem_destroy(pfchem_ctx *ctx);
const char *pfchem_last_error(const pfchem_ctx *ctx);

/* Copies the reaction tables to the device.  Replaces the reaction_type
 * object that RReact reads (reaction_aux.F90:142-335) and the per-cell
 * RUpdateTempDependentCoefs mutation of it (reaction.F90:5433-5524): the
 * kernels evaluate log K at each cell's temperature privately. */
int pfchem_set_network(pfchem_ctx *ctx, const pfchem_network *net,
                       const pfchem_options *opt);

/* Batched RReact over all cells (reaction.F90:3322-3511), replacing the cell
 * loop of RTReact (reactive_transport.F90:1697-1724); with
 * opt.update_kinetic_state it also applies RUpdateKineticState
 * (reaction.F90:5320-5429) to each cell.  dt = option%tran_dt [s]. */
int pfchem_react_batch(pfchem_ctx *ctx, double dt, pfchem_cells *cells);

/* RTReact's own layout: tran_xx holds ncomp values per cell, interleaved
 * ((cell)*ncomp + i, reactive_transport.F90:1701-1703).  The totals are read
 * from tran_xx (cells->total is ignored); on return the first naqcomp entries
 * of each cell hold the free-ion molalities, as RTReact writes back at
 * reactive_transport.F90:1711.  The guess/state pri_molal and every other
 * per-cell field come from `cells` as in pfchem_react_batch.  tran_xx is a
 * pointer of the same kind (host or device) as the others. */
int pfchem_react_batch_interleaved(pfchem_ctx *ctx, double dt, int32_t ncomp,
                                   double *tran_xx, pfchem_cells *cells);

/* Batched RUpdateKineticState (reaction.F90:5320-5429) at the current state,
 * replacing the cell loop of RTUpdateKineticState (reactive_transport.F90:692-705). */
int pfchem_update_kinetic_state(pfchem_ctx *ctx, double dt, pfchem_cells *cells);

/* Stream-ordered variant for callers that keep the cells on the device and
 * run their own transport update on the GPU (no counterpart in the reference,
 * whose RTReact is synchronous and per cell).  pfchem_react_batch_async
 * enqueues one reaction step -- statistics reset, warm-start inference when
 * enabled, the prologue and the persistent solve -- on `stream` (a
 * cudaStream_t) and returns without waiting.  It allocates nothing and
 * synchronises nothing, so the caller may capture it into a CUDA graph
 * together with its transport kernels and replay that graph step after step.
 * Device pointers only.  The context's buffers must first be reserved for at
 * least cells->ncells cells with pfchem_reserve (outside any capture);
 * otherwise the call fails and enqueues nothing.  One step may be in flight
 * per context: the statistics counters are per context.
 * pfchem_async_stats reads those counters once the caller has synchronised
 * `stream` after the step (kernel_ms is 0: time the step on the caller's
 * stream).  pfchem_reserve also sizes the warm-start buffers when a surrogate
 * exists (fit it before reserving). */
int pfchem_reserve(pfchem_ctx *ctx, int64_t ncells);
int pfchem_react_batch_async(pfchem_ctx *ctx, double dt, pfchem_cells *cells, void *stream);
int pfchem_async_stats(pfchem_ctx *ctx, pfchem_stats *stats);

/* Per-cell blocks of the global-implicit transport system (the path PFLOTRAN
 * runs when operator splitting is off): the reaction residual and its
 * Jacobian that RTResidual and RTJacobian add cell by cell
 * (reactive_transport.F90:2729-2760, :3440-3468) through RReaction /
 * RReactionDerivative (reaction.F90:3515-3686, analytical derivatives), and
 * the auxiliary totals and their derivatives from RTAuxVarCompute
 * (reaction.F90:4969-5068) that the accumulation blocks are built from.
 * Evaluated at each cell's current pri_molal with log K at the cell
 * temperature and LAG activity coefficients at cells->ionic_strength.  Device
 * pointers; cells->total is not read.  Blocks are naqcomp x naqcomp per cell,
 * column-major as the Fortran Jac(ncomp,ncomp) that MatSetValuesBlockedLocal
 * receives: element (i,j) of cell c at [c*N*N + j*N + i].  Inactive cells get
 * zero blocks.  The ion-exchange and surface free-site warm starts are
 * updated; mnrl_rate, sec_molal and status are written when given. */
typedef struct pfchem_reaction_blocks_out {
  double *res;          /* (naqcomp, ncells) RReaction residual [mol/s]                */
  double *jac;          /* blocks: dRes_i/dm_j [kg water/s]                            */
  double *total;        /* (naqcomp, ncells) aqueous totals [mol/L], or NULL            */
  double *dtotal;       /* blocks: d total_i / d m_j [kg water/L], or NULL              */
  double *total_sorb;   /* (naqcomp, ncells) sorbed totals [mol/m^3 bulk], or NULL      */
  double *dtotal_sorb;  /* blocks: d total_sorb_i / d m_j [kg water/m^3 bulk], or NULL  */
} pfchem_reaction_blocks_out;
int pfchem_reaction_blocks(pfchem_ctx *ctx, pfchem_cells *cells, pfchem_reaction_blocks_out *out);

/* Batched constraint speciation (ReactionEquilibrateConstraint,
 * reaction.F90:1308-2046): the free-ion molalities of waters specified by one
 * constraint per primary species -- the initial and boundary waters of a
 * run, and the learned warm start's training waters.  Types (and mineral
 * ids) are shared by the batch, values are per cell.  Rows: TOTAL [mol/L],
 * FREE [mol/L], LOG (log10 of a free concentration [mol/L]), CHARGE_BAL
 * (value: initial guess [mol/L]), PH (the component is H+; value: pH),
 * MINERAL (the reaction of kinetic mineral mineral[i] held at equilibrium;
 * value: initial guess [mol/L]), GAS (reaction.F90:1720-1751: the passive
 * gas mineral[i] of the gas tables below at partial pressure value [bar]; a
 * value <= 0 is log10 of the partial pressure, reaction.F90:1531-1535) and
 * TOTAL_SORB (sorbed total [mol/m^3 bulk], reaction.F90:1608-1614; the
 * component's equilibrium sorption).  Starts from free ions 1e-9, alternates log
 * and linear updates for iterations 4-8, switches activity coefficients on
 * after the first convergence; converged when max|res| <
 * opt.max_residual_tolerance and the relative change <
 * opt.max_relative_change_tolerance.  Device pointers.  Writes pri_molal,
 * total_out, sec_molal, total_sorb_eq, the sorption warm starts,
 * ionic_strength, iterations and status (0 converged, 1 iteration cap,
 * 2 singular, 3 non-positive molality) of every cell; cells->total is not
 * read.  Returns the number of cells that did not converge, or < 0. */
#define PFCHEM_CONSTRAINT_TOTAL 1
#define PFCHEM_CONSTRAINT_FREE 2
#define PFCHEM_CONSTRAINT_CHARGE_BAL 3
#define PFCHEM_CONSTRAINT_PH 4
#define PFCHEM_CONSTRAINT_LOG 5
#define PFCHEM_CONSTRAINT_MINERAL 6
#define PFCHEM_CONSTRAINT_GAS 7
#define PFCHEM_CONSTRAINT_TOTAL_SORB 8
#define PFCHEM_MAX_GAS_ROWS 8    /* GAS rows per constraint */
typedef struct pfchem_constraint {
  const int32_t *type;     /* (naqcomp) PFCHEM_CONSTRAINT_* (host pointer) */
  const int32_t *mineral;  /* (naqcomp) constraint_spec_id: 1-based kinetic mineral of MINERAL rows, 1-based
                              passive gas of GAS rows; or NULL (host pointer) */
  const double *value;     /* (naqcomp, ncells) per-cell values (device pointer) */
  int32_t max_iterations;  /* cap; <= 0 means 10000 */
  int32_t npassive_gas;    /* gases in the tables below (reaction_gas_aux.F90 gas%paseq*), host pointers */
  int32_t paseq_ld;        /* leading dimension of paseqspecid (0:paseq_ld) and paseqstoich */
  int32_t reserved;
  const int32_t *paseqspecid;    /* (0:paseq_ld, npassive_gas): count, then 1-based primary ids */
  const double *paseqstoich;     /* (paseq_ld, npassive_gas) */
  const int32_t *paseqh2oid;     /* (npassive_gas) > 0 where H2O takes part, or NULL */
  const double *paseqh2ostoich;  /* (npassive_gas), or NULL */
  const double *paseqlogK;       /* (npassive_gas) log10 K (use_isothermal) */
  const double *paseqlogKcoef;   /* (5, npassive_gas) log K(T) fit (otherwise) */
} pfchem_constraint;
int pfchem_equilibrate_constraints(pfchem_ctx *ctx, pfchem_cells *cells, const pfchem_constraint *con);

/* Mineral-driven porosity and surface-area update after the kinetic state
 * (RealizationUpdatePropertiesTS, realization_subsurface.F90:1686-1735, and
 * RealizationCalcMineralPorosity, :1946-2001):
 *   porosity = max(1 - sum_m phi_m, minimum_porosity)          (update_porosity)
 *   area_m   = area0_m * (porosity/porosity0)^p_por,m * (phi_m/phi0_m)^p_vf,m
 * with the porosity factor only when surface_area_with_porosity and the
 * volume-fraction factor only where phi0_m > 0.  All cells, active or not,
 * as the reference.  Mineral armoring (:1737-1765): a mineral with a
 * critical volume fraction loses its area (0) where its armoring mineral's
 * volume fraction reaches it; below it the area is scaled by
 * ((crit - phi_armor)/crit)^p_vf,m, or reset to area0_m right after an
 * armored item.  The reference carries that "just armored" flag from item to
 * item in cell-then-mineral order; each armored item sets it from its own
 * test, so an item's incoming flag is the test of the previous armored item
 * (the previous cell's last one for a cell's first), and the update stays
 * data-parallel with the same result.  Device pointers, except armor_flag_out. */
typedef struct pfchem_mineral_update {
  int32_t update_porosity;             /* reaction%update_porosity                       */
  int32_t update_surface_area;         /* reaction%update_mineral_surface_area           */
  int32_t surface_area_with_porosity;  /* reaction%update_mnrl_surf_with_porosity        */
  int32_t reserved;
  double minimum_porosity;             /* reaction%minimum_porosity                      */
  const double *surf_area_vol_frac_pwr;/* (nkinmnrl) kinmnrl_surf_area_vol_frac_pwr      */
  const double *surf_area_porosity_pwr;/* (nkinmnrl) kinmnrl_surf_area_porosity_pwr, or NULL */
  const double *mnrl_volfrac0;         /* (nkinmnrl, ncells) rt_auxvar%mnrl_volfrac0     */
  const double *mnrl_area0;            /* (nkinmnrl, ncells) rt_auxvar%mnrl_area0        */
  const double *porosity0;             /* (ncells) field%porosity0, or NULL without the porosity factor */
  double *porosity;                    /* (ncells) out: porosity_base when update_porosity, else NULL */
  /* mineral armoring (realization_subsurface.F90:1737-1765), with
   * reaction%update_armor_mineral_surface; NULL tables = off */
  const double *armor_crit_vol_frac;   /* (nkinmnrl) kinmnrl_armor_crit_vol_frac; <= 0: not armored */
  const int32_t *armor_mineral;        /* (nkinmnrl) 1-based mineral whose volume fraction armors it
                                          (kinmnrl_armor_min_names matched to kinmnrl_names; itself if none) */
  int32_t armor_flag;                  /* in: reaction%update_armor_mineral_surface_flag before the call */
  int32_t reserved2;
  int32_t *armor_flag_out;             /* host, out: the flag after the last cell, or NULL */
} pfchem_mineral_update;
/* Reads cells->mnrl_volfrac (and cells->porosity when porosity is not
 * updated), writes cells->mnrl_area and mu->porosity. */
int pfchem_update_mineral_properties(pfchem_ctx *ctx, pfchem_cells *cells, const pfchem_mineral_update *mu);

/* Statistics of the last react call: what the OS_STATISTICS block of RTReact
 * accumulates (reactive_transport.F90:1645-1804). */
int pfchem_last_stats(const pfchem_ctx *ctx, pfchem_stats *stats);

/* Kernel mapping chosen by the autotuner or forced by the caller. */
typedef struct pfchem_launch {
  int32_t block_threads;    /* threads per block                         */
  int32_t blocks_per_sm;    /* resident blocks per SM for the persistent grid */
  int32_t refill_min_idle;  /* lanes idle in a warp before they fetch new cells */
  int32_t variant;          /* PFCHEM_KERNEL_* */
} pfchem_launch;
#define PFCHEM_KERNEL_SPECIALIZED 0 /* network-specialized kernel compiled at set_network, [J | F] in
                                       shared memory */
#define PFCHEM_KERNEL_GENERIC 1     /* table-driven kernel compiled into the library */
#define PFCHEM_KERNEL_SPECIALIZED_COMPACT 2 /* specialized, J alone in shared memory (right-hand
                                               side in registers): fits more blocks per SM, same results;
                                               the default wherever it fits as many blocks as variant 0 */
/* Cooperative kernels: 8, 16 or 32 lanes solve one cell together (species,
 * complexes, Jacobian entries, sorption sites, minerals and LU rows spread
 * over the lanes; the cell's system in shared memory once per group).  Not
 * for the linear update, the NEWTON activity algorithm or the activity of
 * water.  block_threads: a multiple of 32 (128 recommended);
 * refill_min_idle: unused. */
#define PFCHEM_KERNEL_COOP8 3
#define PFCHEM_KERNEL_COOP16 4
#define PFCHEM_KERNEL_COOP32 5
int pfchem_get_launch(const pfchem_ctx *ctx, pfchem_launch *launch);
int pfchem_set_launch(pfchem_ctx *ctx, const pfchem_launch *launch);
/* Times candidate mappings on `cells` (device pointers; the state arrays are
 * restored after every trial) and keeps the fastest: 32 or 64 threads per
 * block, the augmented or the compact shared-memory layout of the
 * network-specialized kernel (the candidates compiled concurrently), as many
 * resident blocks per SM as fit or one fewer, and a refill at 1, 2, 4 or 8
 * idle lanes; then the cooperative kernels with 8, 16 and 32 lanes per cell
 * (128-thread blocks, as many or one fewer per SM).  Each candidate runs
 * twice and its faster run counts.  The specialized candidates compute each
 * cell with the same operations (the same answers whichever is chosen); a
 * cooperative kernel sums some terms in another order (answers equal to
 * rounding). */
int pfchem_autotune(pfchem_ctx *ctx, double dt, pfchem_cells *cells);

/* ---------------------------------------------------------------------------
 * Learned warm start (no counterpart in the reference).  A BF16 MLP
 * 16 -> 256 -> 256 -> 256 -> 12 (GELU, FP32 accumulate) maps per-cell features
 * (signed-log conserved totals, pH proxy, T, log ionic strength) to the
 * step's log-molalities.  It is trained on the GPU with the library's own
 * tensor-core kernels on solves produced by pfchem_react_batch itself; when
 * enabled, pfchem_react_batch predicts an alternative guess for every cell
 * and FP64 Newton starts from it only where its first residual is no worse
 * than the previous-step guess's.  All pointers are device pointers. */
#define PFCHEM_SURROGATE_FEATURES 16
/* Tensor-core path of the network's dense layers (training and inference):
 * TCGEN05 (the default) = tcgen05.mma with FP32 accumulators in tensor
 * memory, each layer's weights resident in shared memory, a fused bias/GELU
 * epilogue, layer by layer (the weight gradients stay split-K mma.sync);
 * MMA_SYNC = warp-level mma.sync and the fused one-kernel inference.  Call
 * before training or between steps.  No counterpart in the reference. */
#define PFCHEM_MLP_MMA_SYNC 0
#define PFCHEM_MLP_TCGEN05 1
int pfchem_surrogate_backend(pfchem_ctx *ctx, int backend);
typedef struct pfchem_surrogate_cfg {
  int32_t epochs;       /* passes over the samples                    */
  int32_t batch;        /* rows per optimiser step                    */
  float lr;             /* AdamW learning rate                        */
  float weight_decay;   /* AdamW decoupled weight decay               */
  uint64_t seed;        /* weight initialisation and batch order      */
} pfchem_surrogate_cfg;
typedef struct pfchem_surrogate_report {
  int64_t samples;
  int64_t steps;
  float first_loss;     /* mean squared error (standardised units), first step */
  float final_loss;     /* mean over the last epoch's steps           */
  double train_ms;      /* wall time of the fit                       */
} pfchem_surrogate_report;
/* Features of each cell of `cells` (device) into X [ncells][16] (float). */
int pfchem_surrogate_features(pfchem_ctx *ctx, pfchem_cells *cells, float *X);
/* Trains the context's network on M samples: X [M][16] features taken before
 * the step, molal (SoA [naqcomp][M], double) the converged free-ion
 * molalities of those steps.  Pass converged samples only. */
int pfchem_surrogate_fit(pfchem_ctx *ctx, const float *X, const double *molal, int64_t M,
                         const pfchem_surrogate_cfg *cfg, pfchem_surrogate_report *report);
/* The network's prediction for each cell of `cells` (device) into guess
 * (SoA [naqcomp][ncells] free-ion molalities, device). */
int pfchem_surrogate_predict(pfchem_ctx *ctx, pfchem_cells *cells, double *guess);
/* The same prediction through the layer-by-layer path (one GEMM launch per
 * layer, activations through HBM) that training uses; the warm start itself
 * runs the fused one-kernel inference.  Kept to check one against the other. */
int pfchem_surrogate_predict_layers(pfchem_ctx *ctx, pfchem_cells *cells, double *guess);
/* 1 = predict the alternative guess inside pfchem_react_batch (needs a fit). */
int pfchem_surrogate_enable(pfchem_ctx *ctx, int on);
/* Loss and gradients of the current weights on M samples, without updating
 * them (grad_host[nparam] on the host; returns nparam, or < 0). */
int64_t pfchem_surrogate_gradients(pfchem_ctx *ctx, const float *X, const double *molal, int64_t M,
                                   float *grad_host, float *loss_host);
/* Gets (set = 0) or sets (set = 1) the FP32 master weights, layer by layer
 * W (in x out, row-major) then b; returns the parameter count. */
int64_t pfchem_surrogate_params(pfchem_ctx *ctx, float *host, int set);
/* Gets or sets the standardisation: features (mean, 1/std) [16] each,
 * targets ln m (mean, std) [naqcomp] each. */
int pfchem_surrogate_normalization(pfchem_ctx *ctx, float *feat_mean, float *feat_inv_std, float *tgt_mean,
                                   float *tgt_std, int set);

/* Generates and compiles (NVRTC, sm_103a) the network-specialized solve
 * kernel for `net`/`opt` with `block_threads` threads per block, without
 * loading it; needs no GPU.  Returns 0 or < 0 with the compiler log in
 * log[loglen].  No counterpart in the reference: a build-time check of a
 * network for the specialized path. */
int pfchem_check_specialized(const pfchem_network *net, const pfchem_options *opt, int block_threads,
                             char *log, size_t loglen);

/* Size of the library's static device scratch used by
 * pfchem_react_batch_noalloc: a 256-byte work-queue head plus 32 bytes per
 * thread block of the solve (at most 2040 blocks). */
#define PFCHEM_NOALLOC_SCRATCH_BYTES 65536

/* No counterpart in the reference.  The batched reaction step for callers
 * that may not allocate device memory -- codes whose device memory all comes
 * from their own pool (PETSc/Kokkos pools, a coupling framework's arena) or
 * that cannot afford cudaMalloc's device synchronisation inside a time step.
 * No context is needed: the call flattens `net`/`opt`, solves all cells of
 * `cells` (device pointers only, on_device = 1) on `stream` (a cudaStream_t,
 * NULL = default stream) and waits for it.  It calls no cudaMalloc/cudaFree;
 * its only global scratch is a static device array of
 * PFCHEM_NOALLOC_SCRATCH_BYTES bytes, held by every GPU that loads the
 * library until exit, and launches needing more are rejected (-1, message in
 * err).  The first call on a device looks up that array's address.  Every
 * call copies its statistics to host memory and synchronises `stream`
 * before it returns, so it blocks and can never be captured into a CUDA
 * graph (graph users: pfchem_react_batch_async).  All calls share the array:
 * calls that overlap on one GPU race, so serialise them.  It runs the
 * table-driven solve kernel, about 2.6x slower than pfchem_react_batch's
 * network-specialized kernel on the 12-species network (918 vs 354 ms per
 * step at 2,097,152 cells).  `stats` may be NULL; it is zeroed first and
 * kernel_ms, lane_slots and drain_ms stay 0.  Returns as pfchem_react_batch;
 * error text goes to err[errlen]. */
int pfchem_react_batch_noalloc(const pfchem_network *net, const pfchem_options *opt, double dt,
                               pfchem_cells *cells, void *stream, pfchem_stats *stats, char *err,
                               size_t errlen);

#ifdef __cplusplus
}
#endif
#endif /* PFCHEM_H */
