/* rtreact_harness.c -- a C caller of libpfchem doing what RTReact does around
 * its cell loop (src/pflotran/reactive_transport.F90:1605-1806): the network
 * tables are filled in reaction_type's own layout (Fortran column-major, ids
 * 1-based, id tables (0:ld, n)), the transported totals sit interleaved per
 * cell in tran_xx ((cell)*ncomp + i, :1701-1703), one batched call replaces
 * the cell loop (:1697-1724), and tran_xx holds the free-ion molalities
 * afterwards (:1711).
 *
 * Network: the calcite system (calcite.dat rows at 25 C): primaries H+,
 * HCO3-, Ca++; complexes OH-, CO3--, CO2(aq), CaCO3(aq), CaHCO3+; kinetic
 * calcite (k 1e-9 mol/m^2/s, molar volume 36.934 cm^3/mol).  Options:
 * PFLOTRAN's defaults with isothermal log K, the relative residual test at
 * 1e-12 and the kinetic-state update fused into the step.
 *
 *   rtreact_harness check            compile the network-specialized kernel
 *                                    with NVRTC (no GPU needed)
 *   rtreact_harness run IN OUT       one reaction step on the GPU
 *   rtreact_harness oracle IN OUT    the same step through the oracle's
 *                                    restatement (built with -DWITH_ORACLE;
 *                                    checks these tables and arrays on a CPU)
 *
 * IN: int64 n, double dt, then doubles temperature, saturation, den_kg,
 * porosity, volume (n each), total (3 x n, SoA), pri_molal (3 x n),
 * ionic_strength, mnrl_volfrac, mnrl_area (n each).
 * OUT: int32 return code, then doubles tran_xx (n x 3, interleaved),
 * pri_molal, total_out (3 x n each), mnrl_rate, mnrl_volfrac,
 * ionic_strength (n each), int32 iterations, status (n each).
 * Exit status: 0 ok, 1 usage or I/O, 2 library error, 3 no GPU.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "pfchem.h"

#ifdef WITH_ORACLE
int pfo_react_batch(const pfchem_network *net, const pfchem_options *opt, double dt, pfchem_cells *cells,
                    int precision, int nthreads);
#endif

enum { NCOMP = 3, NCPLX = 5, NMNRL = 1, LD = 3 };

/* primaries: H+ (1), HCO3- (2), Ca++ (3) */
static const double pri_Z[NCOMP] = {1.0, -1.0, 2.0};
static const double pri_a0[NCOMP] = {9.0, 4.0, 6.0};
/* complexes, column i = (count, ids) and (stoichiometry) */
static const int32_t cplx_id[(LD + 1) * NCPLX] = {
    1, 1, 0, 0, /* OH-       = -H+ (+H2O)          */
    2, 1, 2, 0, /* CO3--     = -H+ + HCO3-         */
    2, 1, 2, 0, /* CO2(aq)   = H+ + HCO3- (-H2O)   */
    3, 1, 3, 2, /* CaCO3(aq) = -H+ + Ca++ + HCO3-  */
    2, 3, 2, 0, /* CaHCO3+   = Ca++ + HCO3-        */
};
static const double cplx_nu[LD * NCPLX] = {
    -1, 0, 0, -1, 1, 0, 1, 1, 0, -1, 1, 1, 1, 1, 0,
};
static const int32_t cplx_h2oid[NCPLX] = {1, 0, 1, 0, 0};
static const double cplx_h2onu[NCPLX] = {1.0, 0.0, -1.0, 0.0, 0.0};
static const double cplx_Z[NCPLX] = {-1.0, -2.0, 0.0, 0.0, 1.0};
static const double cplx_a0[NCPLX] = {3.5, 4.5, 3.0, 3.0, 4.0};
static const double cplx_logK[NCPLX] = {13.9951, 10.3288, -6.3447, 7.0017, -1.0467};
/* calcite = -H+ + Ca++ + HCO3- */
static const int32_t mnrl_id[LD + 1] = {3, 1, 3, 2};
static const double mnrl_nu[LD] = {-1.0, 1.0, 1.0};
static const double mnrl_logK[NMNRL] = {1.8487};
static const double mnrl_k[NMNRL] = {1e-9};
static const double mnrl_Ea[NMNRL] = {0.0};
static const double mnrl_Vm[NMNRL] = {36.934e-6};
static const double mnrl_zero[NMNRL] = {0.0};

static double cplx_coef[5 * NCPLX], mnrl_coef[5 * NMNRL];

static void calcite_network(pfchem_network *net, pfchem_options *opt) {
  memset(net, 0, sizeof *net);
  net->naqcomp = NCOMP;
  net->neqcplx = NCPLX;
  net->nkinmnrl = NMNRL;
  net->eqcplx_ld = LD;
  net->kinmnrl_ld = LD;
  net->primary_spec_Z = pri_Z;
  net->primary_spec_a0 = pri_a0;
  net->eqcplxspecid = cplx_id;
  net->eqcplxstoich = cplx_nu;
  net->eqcplxh2oid = cplx_h2oid;
  net->eqcplxh2ostoich = cplx_h2onu;
  net->eqcplx_Z = cplx_Z;
  net->eqcplx_a0 = cplx_a0;
  net->eqcplx_logK = cplx_logK;
  /* Maier-Kelly coefficients of a temperature-independent log K */
  for (int i = 0; i < NCPLX; ++i) cplx_coef[5 * i + 1] = cplx_logK[i];
  for (int m = 0; m < NMNRL; ++m) mnrl_coef[5 * m + 1] = mnrl_logK[m];
  net->eqcplx_logKcoef = cplx_coef;
  net->debyeA = 0.5114; /* reaction_database.F90 values at 25 C */
  net->debyeB = 0.3288;
  net->debyeBdot = 0.0410;
  net->kinmnrlspecid = mnrl_id;
  net->kinmnrlstoich = mnrl_nu;
  net->kinmnrl_logK = mnrl_logK;
  net->kinmnrl_logKcoef = mnrl_coef;
  net->kinmnrl_rate_constant = mnrl_k;
  net->kinmnrl_activation_energy = mnrl_Ea;
  net->kinmnrl_molar_vol = mnrl_Vm;
  net->kinmnrl_affinity_threshold = mnrl_zero;
  net->kinmnrl_rate_limiter = mnrl_zero;

  memset(opt, 0, sizeof *opt);
  opt->use_log_formulation = 1;
  opt->act_coef_update_frequency = PFCHEM_ACT_COEF_FREQUENCY_TIMESTEP;
  opt->act_coef_update_algorithm = PFCHEM_ACT_COEF_ALGORITHM_LAG;
  opt->use_isothermal = 1;
  opt->residual_tol_kind = PFCHEM_RESIDUAL_RELATIVE;
  opt->accum_mode = PFCHEM_ACCUM_DT_CONSISTENT;
  opt->max_iterations = 200;
  opt->max_dlnC = 5.0;
  opt->max_relative_change_tolerance = 0.0;
  opt->max_residual_tolerance = 1e-12;
  opt->update_kinetic_state = 1;
  opt->jacobian = PFCHEM_JACOBIAN_REFERENCE;
}

static double *read_doubles(FILE *f, size_t count) {
  double *p = (double *)malloc(count * sizeof(double));
  if (p && fread(p, sizeof(double), count, f) != count) {
    free(p);
    return NULL;
  }
  return p;
}

static int write_all(FILE *f, const void *p, size_t size, size_t count) {
  return fwrite(p, size, count, f) == count ? 0 : 1;
}

int main(int argc, char **argv) {
  pfchem_network net;
  pfchem_options opt;
  calcite_network(&net, &opt);
  if (argc == 2 && strcmp(argv[1], "check") == 0) {
    char log[8192];
    int rc = pfchem_check_specialized(&net, &opt, 32, log, sizeof log);
    if (rc != 0) {
      fprintf(stderr, "pfchem_check_specialized: %d\n%s\n", rc, log);
      return 2;
    }
    printf("check ok\n");
    return 0;
  }
  if (argc != 4 || (strcmp(argv[1], "run") != 0 && strcmp(argv[1], "oracle") != 0)) {
    fprintf(stderr, "usage: %s check | run IN OUT | oracle IN OUT\n", argv[0]);
    return 1;
  }
  const int use_oracle = strcmp(argv[1], "oracle") == 0;
#ifndef WITH_ORACLE
  if (use_oracle) {
    fprintf(stderr, "built without -DWITH_ORACLE\n");
    return 1;
  }
#endif
  FILE *in = fopen(argv[2], "rb");
  if (!in) return 1;
  int64_t n = 0;
  double dt = 0.0;
  if (fread(&n, sizeof n, 1, in) != 1 || fread(&dt, sizeof dt, 1, in) != 1 || n < 1) return 1;
  const size_t nc = (size_t)n;
  double *temperature = read_doubles(in, nc), *saturation = read_doubles(in, nc), *den = read_doubles(in, nc);
  double *porosity = read_doubles(in, nc), *volume = read_doubles(in, nc);
  double *total = read_doubles(in, NCOMP * nc), *pri_molal = read_doubles(in, NCOMP * nc);
  double *ionic = read_doubles(in, nc), *volfrac = read_doubles(in, NMNRL * nc), *area = read_doubles(in, NMNRL * nc);
  fclose(in);
  if (!temperature || !saturation || !den || !porosity || !volume || !total || !pri_molal || !ionic || !volfrac ||
      !area)
    return 1;

  /* tran_xx as RTReact holds it: the totals of cell k at k*ncomp + i */
  double *tran_xx = (double *)malloc(NCOMP * nc * sizeof(double));
  double *total_out = (double *)calloc(NCOMP * nc, sizeof(double));
  double *rate = (double *)calloc(NMNRL * nc, sizeof(double));
  int32_t *iterations = (int32_t *)calloc(nc, sizeof(int32_t));
  int32_t *status = (int32_t *)calloc(nc, sizeof(int32_t));
  if (!tran_xx || !total_out || !rate || !iterations || !status) return 1;
  for (size_t k = 0; k < nc; ++k)
    for (int i = 0; i < NCOMP; ++i) tran_xx[k * NCOMP + i] = total[i * nc + k];

  pfchem_cells cells;
  memset(&cells, 0, sizeof cells);
  cells.ncells = n;
  cells.on_device = 0; /* host arrays: the library stages them */
  cells.temperature = temperature;
  cells.saturation = saturation;
  cells.den_kg = den;
  cells.porosity = porosity;
  cells.volume = volume;
  cells.pri_molal = pri_molal;
  cells.ionic_strength = ionic;
  cells.mnrl_volfrac = volfrac;
  cells.mnrl_area = area;
  cells.total_out = total_out;
  cells.mnrl_rate = rate;
  cells.iterations = iterations;
  cells.status = status;

  int rc;
  if (use_oracle) {
#ifdef WITH_ORACLE
    /* what the interleaved entry point does around the batch */
    double *soa = (double *)malloc(NCOMP * nc * sizeof(double));
    if (!soa) return 1;
    for (size_t k = 0; k < nc; ++k)
      for (int i = 0; i < NCOMP; ++i) soa[i * nc + k] = tran_xx[k * NCOMP + i];
    cells.total = soa;
    rc = pfo_react_batch(&net, &opt, dt, &cells, 0, 4);
    for (size_t k = 0; k < nc; ++k)
      for (int i = 0; i < NCOMP; ++i) tran_xx[k * NCOMP + i] = pri_molal[i * nc + k];
    free(soa);
#else
    rc = -1;
#endif
  } else {
    pfchem_ctx *ctx = NULL;
    rc = pfchem_create(&ctx, 0);
    if (rc != 0) {
      fprintf(stderr, "pfchem_create: %s\n", ctx ? pfchem_last_error(ctx) : "failed");
      if (ctx) pfchem_destroy(ctx);
      return 3;
    }
    rc = pfchem_set_network(ctx, &net, &opt);
    if (rc == 0) rc = pfchem_react_batch_interleaved(ctx, dt, NCOMP, tran_xx, &cells);
    if (rc < 0) fprintf(stderr, "pfchem: %s\n", pfchem_last_error(ctx));
    pfchem_destroy(ctx);
    if (rc < 0) return 2;
  }

  FILE *out = fopen(argv[3], "wb");
  if (!out) return 1;
  int32_t rc32 = rc;
  int bad = write_all(out, &rc32, sizeof rc32, 1) | write_all(out, tran_xx, sizeof(double), NCOMP * nc) |
            write_all(out, pri_molal, sizeof(double), NCOMP * nc) |
            write_all(out, total_out, sizeof(double), NCOMP * nc) | write_all(out, rate, sizeof(double), NMNRL * nc) |
            write_all(out, volfrac, sizeof(double), NMNRL * nc) | write_all(out, ionic, sizeof(double), nc) |
            write_all(out, iterations, sizeof(int32_t), nc) | write_all(out, status, sizeof(int32_t), nc);
  fclose(out);
  return bad ? 1 : 0;
}
