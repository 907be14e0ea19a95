// pfchem_api.cu -- the C ABI (include/pfchem.h) over the sm_103a kernels.
//
// A context owns a CUDA stream, the flattened network (DevNet), the work
// queue / statistics scratch, device staging buffers for host-pointer calls,
// a captured CUDA graph of the last device-pointer solve, and the launch
// mapping.  Nothing here computes chemistry on the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <random>
#include <utility>
#include <nvrtc.h>

#include "../../include/pfchem.h"
#include "pfchem_device.cuh"

namespace pfchem {
cudaError_t launch_react(const DevNet &n, const CellArgs &a, Scratch *scr, int grid, int block, int refill,
                         cudaStream_t st);
cudaError_t launch_kinetic_state(const DevNet &n, const CellArgs &a, cudaStream_t st);
cudaError_t launch_constraint(const DevNet &n, const CellArgs &a, const pfchem_constraint &con, int max_its,
                              Scratch *scr, cudaStream_t st);
cudaError_t launch_mineral_properties(const CellArgs &a, int Nm, const pfchem_mineral_update &mu, int *flag_dev,
                                      cudaStream_t st);
cudaError_t launch_reaction_blocks(const DevNet &n, const CellArgs &a, double *res, double *jac, double *total,
                                   double *dtotal, double *total_sorb, double *dtotal_sorb, cudaStream_t st);
int max_active_blocks(const DevNet &n, int block);
int gen_kernel(const DevNet &n, int block, bool compact, void **fn_out, void **pro_out, std::string *err);
int gen_kernels_prepare(const DevNet &n, const std::vector<std::pair<int, bool>> &cands, std::string *err);
int gen_prep_fields(const DevNet &n);
int gen_blocks_per_sm(void *fn, const DevNet &n, int block, bool compact);
size_t gen_shared_bytes(const DevNet &n, int block, bool compact);
std::string generate_source(const DevNet &n, int block, bool compact);
cudaError_t gen_launch(void *fn, void *pro, const DevNet &n, const CellArgs &a, Scratch *scr, double *prep, int grid,
                       int block, int refill, cudaStream_t st, bool compact);
bool coop_supports(const DevNet &n);
int coop_group_doubles(const DevNet &n);
size_t coop_tables_bytes();
struct CoopTables;
void coop_build_tables(const DevNet &n, CoopTables *t);
cudaError_t coop_launch(int lanes, const DevNet &n, const CellArgs &a, const void *tables, Scratch *scr, int grid,
                        int block, cudaStream_t st);
int coop_blocks_per_sm(int lanes, const DevNet &n, int block);
struct Surrogate;
Surrogate *surrogate_create(int N, uint64_t seed, std::string *err);
void surrogate_destroy(Surrogate *s);
size_t surrogate_nparam(const Surrogate *s);
cudaError_t surrogate_features(const DevNet &n, const CellArgs &a, float *X, cudaStream_t st);
void surrogate_set_norm(Surrogate *s, const float *fmu, const float *fisd, const float *tmu, const float *tsd);
float surrogate_train_step(Surrogate *s, const float *X, const float *T, long long rows, float lr, float wd,
                           cudaStream_t st, bool sync, cudaError_t *err);
cudaError_t surrogate_gradients(Surrogate *s, const float *X, const float *T, long long rows, float *grad_host,
                                float *loss_host, cudaStream_t st);
cudaError_t surrogate_get_params(Surrogate *s, float *host);
cudaError_t surrogate_set_params(Surrogate *s, const float *host);
cudaError_t surrogate_prepare(Surrogate *s, long long ncells);
double *surrogate_guess_buffer(Surrogate *s);
cudaError_t surrogate_predict(Surrogate *s, const DevNet &n, const CellArgs &a, double *guess, cudaStream_t st,
                              bool pack = true);
cudaError_t surrogate_pack(Surrogate *s, cudaStream_t st);
cudaError_t surrogate_predict_layers(Surrogate *s, const DevNet &n, const CellArgs &a, double *guess,
                                     cudaStream_t st);
cudaError_t surrogate_targets(Surrogate *s, const double *molal, long long M, float *T, cudaStream_t st);
void surrogate_mark_trained(Surrogate *s, bool t);
bool surrogate_trained(const Surrogate *s);
bool surrogate_ready(const Surrogate *s, long long ncells);
void surrogate_set_backend(Surrogate *s, int backend);
cudaError_t surrogate_check(Surrogate *s, bool *timed_out);
}  // namespace pfchem

using namespace pfchem;

struct StageBuf {
  void *ptr = nullptr;
  size_t bytes = 0;
};

struct pfchem_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  DevNet net;
  bool has_net = false;
  pfchem_options opt;
  Scratch *scratch = nullptr;  // device
  pfchem_launch launch{};
  bool launch_forced = false;
  pfchem_stats stats{};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  StageBuf stage[32];
  // graph cache of the last device-pointer solve
  cudaGraphExec_t graph = nullptr;
  CellArgs graph_args{};
  pfchem_launch graph_launch{};
  void *gen_fn = nullptr;  // specialized kernel for gen_block threads per block
  void *gen_pro = nullptr; // its data-parallel prologue
  int gen_block = 0;
  bool gen_compact = false;  // its shared-memory layout (PFCHEM_KERNEL_SPECIALIZED_COMPACT)
  double *prep = nullptr;  // prologue records, gen_prep_fields x prep_cells doubles
  int64_t prep_cells = 0;
  void *coop_tables = nullptr;  // gather lists of the cooperative kernels (device)
  Surrogate *sur = nullptr;  // learned warm start
  bool sur_on = false;
  int64_t async_cells = 0;  // cells of the last pfchem_react_batch_async
  float norm[2 * 16 + 2 * PFCHEM_MAX_PRI] = {};  // host copy of the standardisation
  char err[2048] = {0};
};

namespace {

int fail(pfchem_ctx *c, int code, const char *fmt, ...) {
  if (c) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(c->err, sizeof(c->err), fmt, ap);
    va_end(ap);
  }
  return code;
}

#define CUDA_TRY(ctx, expr)                                                                     \
  do {                                                                                          \
    cudaError_t e_ = (expr);                                                                    \
    if (e_ != cudaSuccess) return fail(ctx, -2, "%s: %s (%s:%d)", #expr, cudaGetErrorString(e_), \
                                       __FILE__, __LINE__);                                     \
  } while (0)

int idtab(const int32_t *t, int ld, int k, int r) { return t[(ld + 1) * r + k]; }
double sttab(const double *t, int ld, int k, int r) { return t[ld * r + (k - 1)]; }

int build_devnet(pfchem_ctx *c, const pfchem_network *w, const pfchem_options *o, DevNet &n) {
  std::memset(&n, 0, sizeof(n));
  if (!w || !o) return fail(c, -1, "null network or options");
  if (w->naqcomp < 1 || w->naqcomp > PFCHEM_MAX_PRI) return fail(c, -1, "naqcomp %d outside [1,%d]", w->naqcomp, PFCHEM_MAX_PRI);
  if (w->neqcplx < 0 || w->neqcplx > PFCHEM_MAX_CPLX) return fail(c, -1, "neqcplx %d > %d", w->neqcplx, PFCHEM_MAX_CPLX);
  if (w->nkinmnrl < 0 || w->nkinmnrl > PFCHEM_MAX_MNRL) return fail(c, -1, "nkinmnrl %d > %d", w->nkinmnrl, PFCHEM_MAX_MNRL);
  if (w->neqionxrxn < 0 || w->neqionxrxn > PFCHEM_MAX_IONX) return fail(c, -1, "neqionxrxn %d > %d", w->neqionxrxn, PFCHEM_MAX_IONX);
  if (w->nsrfcplxrxn < 0 || w->nsrfcplxrxn > PFCHEM_MAX_SRFRXN) return fail(c, -1, "nsrfcplxrxn %d > %d", w->nsrfcplxrxn, PFCHEM_MAX_SRFRXN);
  if (w->nsrfcplx < 0 || w->nsrfcplx > PFCHEM_MAX_SRFCPLX) return fail(c, -1, "nsrfcplx %d > %d", w->nsrfcplx, PFCHEM_MAX_SRFCPLX);
  if (o->act_coef_update_algorithm != PFCHEM_ACT_COEF_ALGORITHM_LAG &&
      o->act_coef_update_algorithm != PFCHEM_ACT_COEF_ALGORITHM_NEWTON)
    return fail(c, -1, "unknown act_coef_update_algorithm %d", o->act_coef_update_algorithm);
  if (o->act_coef_update_algorithm == PFCHEM_ACT_COEF_ALGORITHM_NEWTON && o->use_activity_h2o &&
      o->act_coef_update_frequency != PFCHEM_ACT_COEF_FREQUENCY_OFF)
    return fail(c, -1, "use_activity_h2o with ACT_COEF_ALGORITHM_NEWTON is not supported");
  if (o->use_activity_h2o && o->act_coef_update_frequency == PFCHEM_ACT_COEF_FREQUENCY_NEWTON_ITER)
    return fail(c, -1, "use_activity_h2o with NEWTON_ITER activity updates is not supported");
  if (o->max_iterations < 1) return fail(c, -1, "max_iterations must be >= 1");
  n.N = w->naqcomp;
  n.Nc = w->neqcplx;
  n.Nm = w->nkinmnrl;
  n.Nix = w->neqionxrxn;
  n.Nsr = w->nsrfcplxrxn;
  n.Nsc = w->nsrfcplx;
  n.use_log = o->use_log_formulation != 0;
  n.act_freq = o->act_coef_update_frequency;
  n.act_newton = o->act_coef_update_algorithm == PFCHEM_ACT_COEF_ALGORITHM_NEWTON &&
                 o->act_coef_update_frequency != PFCHEM_ACT_COEF_FREQUENCY_OFF;
  n.use_h2o = o->use_activity_h2o != 0;
  n.isothermal = o->use_isothermal != 0;
  n.resid_kind = o->residual_tol_kind;
  n.accum_mode = o->accum_mode;
  n.max_iter = o->max_iterations;
  n.update_kin = o->update_kinetic_state != 0;
  if (o->jacobian != PFCHEM_JACOBIAN_REFERENCE && o->jacobian != PFCHEM_JACOBIAN_EXACT)
    return fail(c, -1, "unknown jacobian %d", o->jacobian);
  n.jac_exact = o->jacobian == PFCHEM_JACOBIAN_EXACT;
  if (o->exact_jacobian_after < 0) return fail(c, -1, "exact_jacobian_after must be >= 0");
  n.exact_after = o->exact_jacobian_after;
  n.max_dlnC = o->max_dlnC;
  n.rel_change_tol = o->max_relative_change_tolerance;
  n.res_tol = o->max_residual_tolerance;
  n.A = w->debyeA;
  n.B = w->debyeB;
  n.Bdot = w->debyeBdot;
  for (int j = 0; j < n.N; ++j) {
    n.Zp[j] = w->primary_spec_Z[j];
    n.Z2p[j] = std::fabs(n.Zp[j]) > 1e-10 ? n.Zp[j] * n.Zp[j] : 0.0;
    n.ap[j] = w->primary_spec_a0[j];
  }
  auto check_ids = [&](const char *what, const int32_t *t, int ld, int cnt, int maxid) -> int {
    if (cnt > 0 && !t) return fail(c, -1, "%s: table missing", what);
    if (ld > PFCHEM_MAX_NNZ) return fail(c, -1, "%s: leading dimension %d > %d", what, ld, PFCHEM_MAX_NNZ);
    for (int r = 0; r < cnt; ++r) {
      int k = idtab(t, ld, 0, r);
      if (k < 0 || k > ld) return fail(c, -1, "%s %d: count %d outside [0,%d]", what, r + 1, k, ld);
      for (int q = 1; q <= k; ++q) {
        int id = idtab(t, ld, q, r);
        if (id < 1 || id > maxid) return fail(c, -1, "%s %d: species id %d outside [1,%d]", what, r + 1, id, maxid);
      }
    }
    return 0;
  };
  int e;
  if ((e = check_ids("aqueous complex", w->eqcplxspecid, w->eqcplx_ld, n.Nc, n.N))) return e;
  for (int i = 0; i < n.Nc; ++i) {
    n.cn[i] = (int8_t)idtab(w->eqcplxspecid, w->eqcplx_ld, 0, i);
    for (int k = 1; k <= n.cn[i]; ++k) {
      n.cid[i][k - 1] = (int8_t)(idtab(w->eqcplxspecid, w->eqcplx_ld, k, i) - 1);
      n.cnu[i][k - 1] = sttab(w->eqcplxstoich, w->eqcplx_ld, k, i);
    }
    n.cZ2[i] = std::fabs(w->eqcplx_Z[i]) > 1e-10 ? w->eqcplx_Z[i] * w->eqcplx_Z[i] : 0.0;
    n.ca[i] = w->eqcplx_a0[i];
    n.ch2o[i] = (w->eqcplxh2oid && w->eqcplxh2oid[i] > 0) ? w->eqcplxh2ostoich[i] : 0.0;
    n.clogK[i] = w->eqcplx_logK ? w->eqcplx_logK[i] : 0.0;
    for (int q = 0; q < 5; ++q) n.ccoef[i][q] = w->eqcplx_logKcoef ? w->eqcplx_logKcoef[5 * i + q] : 0.0;
  }
  if ((e = check_ids("kinetic mineral", w->kinmnrlspecid, w->kinmnrl_ld, n.Nm, n.N))) return e;
  n.has_temkin = w->kinmnrl_Temkin_const != nullptr;
  n.has_minscale = w->kinmnrl_min_scale_factor != nullptr;
  n.has_affpow = w->kinmnrl_affinity_power != nullptr;
  for (int m = 0; m < n.Nm; ++m) {
    n.mn[m] = (int8_t)idtab(w->kinmnrlspecid, w->kinmnrl_ld, 0, m);
    for (int k = 1; k <= n.mn[m]; ++k) {
      n.mid[m][k - 1] = (int8_t)(idtab(w->kinmnrlspecid, w->kinmnrl_ld, k, m) - 1);
      n.mnu[m][k - 1] = sttab(w->kinmnrlstoich, w->kinmnrl_ld, k, m);
    }
    n.mh2o[m] = (w->kinmnrlh2oid && w->kinmnrlh2oid[m] > 0) ? w->kinmnrlh2ostoich[m] : 0.0;
    n.mlogK[m] = w->kinmnrl_logK ? w->kinmnrl_logK[m] : 0.0;
    for (int q = 0; q < 5; ++q) n.mcoef[m][q] = w->kinmnrl_logKcoef ? w->kinmnrl_logKcoef[5 * m + q] : 0.0;
    n.mk[m] = w->kinmnrl_rate_constant[m];
    n.mEa[m] = w->kinmnrl_activation_energy ? w->kinmnrl_activation_energy[m] : 0.0;
    n.mVm[m] = w->kinmnrl_molar_vol[m];
    n.mthr[m] = w->kinmnrl_affinity_threshold ? w->kinmnrl_affinity_threshold[m] : 0.0;
    n.mlim[m] = w->kinmnrl_rate_limiter ? w->kinmnrl_rate_limiter[m] : 0.0;
    n.mtemkin[m] = n.has_temkin ? w->kinmnrl_Temkin_const[m] : 1.0;
    n.mscale[m] = n.has_minscale ? w->kinmnrl_min_scale_factor[m] : 1.0;
    n.mpow[m] = n.has_affpow ? w->kinmnrl_affinity_power[m] : 1.0;
    // rate prefactors: tables (0:maxsp, maxpref, nkinmnrl) and (maxsp, maxpref, nkinmnrl)
    const int np = (w->max_num_prefactors > 0 && w->kinmnrl_num_prefactors) ? w->kinmnrl_num_prefactors[m] : 0;
    if (np < 0 || np > w->max_num_prefactors || np > PFCHEM_MAX_PREF)
      return fail(c, -1, "mineral %d: %d rate prefactors outside [0, min(max_num_prefactors, %d)]", m + 1, np,
                  PFCHEM_MAX_PREF);
    n.mpn[m] = (int8_t)np;
    if (np > 0) {
      const int maxp = w->max_num_prefactors, maxs = w->max_num_prefactor_species;
      if (!w->kinmnrl_pref_rate || !w->kinmnrl_pref_activation_energy || !w->kinmnrl_prefactor_id ||
          !w->kinmnrl_pref_alpha || !w->kinmnrl_pref_beta || !w->kinmnrl_pref_atten_coef)
        return fail(c, -1, "mineral %d: rate prefactor tables missing", m + 1);
      n.has_pref = 1;
      for (int p = 0; p < np; ++p) {
        const int base = (maxs + 1) * (p + maxp * m);
        const int ns = w->kinmnrl_prefactor_id[base];
        if (ns < 0 || ns > maxs || ns > PFCHEM_MAX_PREF_SPEC)
          return fail(c, -1, "mineral %d prefactor %d: %d species outside [0, min(max_num_prefactor_species, %d)]",
                      m + 1, p + 1, ns, PFCHEM_MAX_PREF_SPEC);
        n.mps[m][p] = (int8_t)ns;
        n.mpk[m][p] = w->kinmnrl_pref_rate[p + maxp * m];
        n.mpEa[m][p] = w->kinmnrl_pref_activation_energy[p + maxp * m];
        for (int q = 0; q < ns; ++q) {
          const int id = w->kinmnrl_prefactor_id[base + 1 + q];
          if (id == 0 || id > n.N || -id > n.Nc)
            return fail(c, -1, "mineral %d prefactor %d: species id %d outside [1,%d] or [-%d,-1]", m + 1, p + 1, id,
                        n.N, n.Nc);
          n.mpid[m][p][q] = (int8_t)(id > 0 ? id - 1 : id);
          const int qq = q + maxs * (p + maxp * m);
          n.mpa[m][p][q] = w->kinmnrl_pref_alpha[qq];
          n.mpb[m][p][q] = w->kinmnrl_pref_beta[qq];
          n.mpatt[m][p][q] = w->kinmnrl_pref_atten_coef[qq];
          if (!(n.mpatt[m][p][q] >= 0.0))
            return fail(c, -1, "mineral %d prefactor %d: negative attenuation coefficient", m + 1, p + 1);
        }
      }
    }
  }
  if ((e = check_ids("ion exchange", w->eqionx_rxn_cationid, w->eqionx_ld, n.Nix, n.N))) return e;
  for (int r = 0; r < n.Nix; ++r) {
    n.xn[r] = (int8_t)idtab(w->eqionx_rxn_cationid, w->eqionx_ld, 0, r);
    if (n.xn[r] < 1) return fail(c, -1, "ion exchange %d has no cations", r + 1);
    n.xzflag[r] = w->eqionx_rxn_Z_flag[r] ? 1 : 0;
    n.xsurf[r] = (int8_t)(w->eqionx_rxn_to_surf ? w->eqionx_rxn_to_surf[r] : 0);
    if (n.xsurf[r] < 0 || n.xsurf[r] > n.Nm) return fail(c, -1, "ion exchange %d: mineral id %d", r + 1, n.xsurf[r]);
    n.xCEC[r] = w->eqionx_rxn_CEC[r];
    const int i1 = idtab(w->eqionx_rxn_cationid, w->eqionx_ld, 1, r) - 1;
    for (int k = 1; k <= n.xn[r]; ++k) {
      const int id = idtab(w->eqionx_rxn_cationid, w->eqionx_ld, k, r) - 1;
      n.xid[r][k - 1] = (int8_t)id;
      n.xk[r][k - 1] = sttab(w->eqionx_rxn_k, w->eqionx_ld, k, r);
      if (std::fabs(n.Zp[id]) < 1e-10) return fail(c, -1, "ion exchange %d: uncharged cation", r + 1);
      const double zr = n.Zp[id] / n.Zp[i1];
      n.xzr[r][k - 1] = zr;
      n.xpow[r][k - 1] = zr == 1.0 ? kPowOne : zr == 2.0 ? kPowTwo : zr == 0.5 ? kPowHalf : kPowGeneric;
    }
  }
  if ((e = check_ids("surface complex", w->srfcplxspecid, w->srfcplx_ld, n.Nsc, n.N))) return e;
  if ((e = check_ids("surface complexation reaction", w->srfcplxrxn_to_complex, w->srfcplxrxn_ld, n.Nsr, n.Nsc)))
    return e;
  for (int r = 0; r < n.Nsr; ++r) {
    n.srn[r] = (int8_t)idtab(w->srfcplxrxn_to_complex, w->srfcplxrxn_ld, 0, r);
    for (int k = 1; k <= n.srn[r]; ++k) n.src[r][k - 1] = (int8_t)(idtab(w->srfcplxrxn_to_complex, w->srfcplxrxn_ld, k, r) - 1);
    n.srtype[r] = (int8_t)w->srfcplxrxn_surf_type[r];
    if (n.srtype[r] == PFCHEM_COLLOID_SURFACE) return fail(c, -1, "surface complexation %d: colloid surfaces are not supported", r + 1);
    n.srsurf[r] = (int8_t)(w->srfcplxrxn_to_surf ? w->srfcplxrxn_to_surf[r] : 0);
    if (n.srtype[r] == PFCHEM_MINERAL_SURFACE && (n.srsurf[r] < 1 || n.srsurf[r] > n.Nm))
      return fail(c, -1, "surface complexation %d: mineral id %d", r + 1, n.srsurf[r]);
    n.srdens[r] = w->srfcplxrxn_site_density[r];
    n.srflag[r] = w->srfcplxrxn_stoich_flag[r] ? 1 : 0;
  }
  for (int k = 0; k < n.Nsc; ++k) {
    n.sn[k] = (int8_t)idtab(w->srfcplxspecid, w->srfcplx_ld, 0, k);
    for (int q = 1; q <= n.sn[k]; ++q) {
      n.sid[k][q - 1] = (int8_t)(idtab(w->srfcplxspecid, w->srfcplx_ld, q, k) - 1);
      n.snu[k][q - 1] = sttab(w->srfcplxstoich, w->srfcplx_ld, q, k);
    }
    n.sfs[k] = w->srfcplx_free_site_stoich[k];
    n.sh2o[k] = (w->srfcplxh2oid && w->srfcplxh2oid[k] > 0) ? w->srfcplxh2ostoich[k] : 0.0;
    n.slogK[k] = w->srfcplx_logK ? w->srfcplx_logK[k] : 0.0;
    for (int q = 0; q < 5; ++q) n.scoef[k][q] = w->srfcplx_logKcoef ? w->srfcplx_logKcoef[5 * k + q] : 0.0;
  }
  return 0;
}

int stage(pfchem_ctx *c, int slot, const void *host, size_t bytes, void **dev, bool upload) {
  *dev = nullptr;
  if (!host) return 0;
  StageBuf &b = c->stage[slot];
  if (b.bytes < bytes) {
    if (b.ptr) cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
    CUDA_TRY(c, cudaMalloc(&b.ptr, bytes));
    b.bytes = bytes;
  }
  if (upload) CUDA_TRY(c, cudaMemcpyAsync(b.ptr, host, bytes, cudaMemcpyHostToDevice, c->stream));
  *dev = b.ptr;
  return 0;
}

// Default mapping: 64 threads per block, as many resident blocks per SM as
// fit, refill when 8 lanes of a warp are idle.
void default_launch(pfchem_ctx *c) {
  c->launch.block_threads = 64;
  int nb = max_active_blocks(c->net, 64);
  c->launch.blocks_per_sm = std::max(1, nb);
  c->launch.refill_min_idle = 8;
  c->launch.variant = PFCHEM_KERNEL_GENERIC;
}

// Compiles (or reuses) the network-specialized kernel for `block` threads per
// block and returns its resident blocks per SM (0 on failure, message in err).
bool is_specialized(int v) { return v == PFCHEM_KERNEL_SPECIALIZED || v == PFCHEM_KERNEL_SPECIALIZED_COMPACT; }
bool is_coop(int v) { return v == PFCHEM_KERNEL_COOP8 || v == PFCHEM_KERNEL_COOP16 || v == PFCHEM_KERNEL_COOP32; }
int coop_lanes(int v) { return v == PFCHEM_KERNEL_COOP8 ? 8 : v == PFCHEM_KERNEL_COOP16 ? 16 : 32; }

// The network-specialized kernel covers every option but the NEWTON activity
// algorithm updated at every Newton iteration, which needs each complex's
// concentration from the previous iteration (the table-driven kernel keeps
// them).
bool specialized_supports(const DevNet &n) {
  return !(n.act_newton && n.act_freq == PFCHEM_ACT_COEF_FREQUENCY_NEWTON_ITER);
}

int ensure_gen(pfchem_ctx *c, int block, bool compact) {
  if (c->gen_fn && c->gen_block == block && c->gen_compact == compact)
    return gen_blocks_per_sm(c->gen_fn, c->net, block, compact);
  std::string e;
  void *fn = nullptr, *pro = nullptr;
  if (gen_kernel(c->net, block, compact, &fn, &pro, &e) != 0) {
    fail(c, -2, "specialized kernel: %s", e.c_str());
    return 0;
  }
  c->gen_fn = fn;
  c->gen_pro = pro;
  c->gen_block = block;
  c->gen_compact = compact;
  int nb = gen_blocks_per_sm(fn, c->net, block, compact);
  if (nb < 1) fail(c, -1, "specialized kernel with %d threads per block does not fit on an SM", block);
  return nb;
}

// Specialized kernel, 32 threads per block, as many blocks per SM as fit,
// refill as soon as one lane of a warp is idle (the prologue leaves a
// refill only loads to do; +5-7% over refilling at 8 idle lanes at 2M cells
// of the 12-species network).  The compact layout (J alone in shared memory,
// the right-hand side in registers) whenever it fits as many blocks per SM
// as the augmented one: for that network 6 blocks against 5, 273 vs 286 ms
// per plain step and 207 vs 218 ms per warm step; 4 % faster at equal
// residency on the calcite and 16-species networks; the same arithmetic in
// the same order.  The autotuner tries both.
int default_specialized_launch(pfchem_ctx *c) {
  const int block = 32;
  {  // both layouts compiled concurrently (NVRTC), then loaded from the cache
    std::vector<std::pair<int, bool>> cands{{block, false}};
    if (gen_shared_bytes(c->net, block, true) <= 227 * 1024) cands.push_back({block, true});
    std::string err;
    if (gen_kernels_prepare(c->net, cands, &err)) return fail(c, -2, "specialized kernel: %s", err.c_str());
  }
  const int nb_aug = ensure_gen(c, block, false);
  if (nb_aug < 1) return -2;
  bool compact = false;
  int nb = nb_aug;
  if (gen_shared_bytes(c->net, block, true) <= 227 * 1024) {
    const int nb_cmp = ensure_gen(c, block, true);
    if (nb_cmp >= nb_aug) {
      compact = true;
      nb = nb_cmp;
    } else if (ensure_gen(c, block, false) < 1) {
      return -2;
    }
  }
  c->launch.block_threads = block;
  c->launch.blocks_per_sm = nb;
  c->launch.refill_min_idle = 1;
  c->launch.variant = compact ? PFCHEM_KERNEL_SPECIALIZED_COMPACT : PFCHEM_KERNEL_SPECIALIZED;
  return 0;
}

double drain_ms(const Scratch &h) {
  const unsigned long long t0 = ~h.t_drain_inv;
  return (h.t_drain_inv && h.t_end > t0) ? (double)(h.t_end - t0) * 1e-6 : 0.0;
}

int check_cells(pfchem_ctx *c, const pfchem_cells *cl) {
  if (!c || !cl) return fail(c, -1, "null argument");
  if (!c->has_net) return fail(c, -1, "pfchem_set_network has not been called");
  if (cl->ncells < 0) return fail(c, -1, "ncells < 0");
  if (cl->ncells == 0) return 0;  // an empty batch (a rank without local cells) names no arrays
  const DevNet &n = c->net;
  if (!cl->temperature || !cl->saturation || !cl->den_kg || !cl->porosity || !cl->volume || !cl->pri_molal ||
      !cl->ionic_strength)
    return fail(c, -1, "a required per-cell array is null");
  if (n.Nm > 0 && (!cl->mnrl_volfrac || !cl->mnrl_area)) return fail(c, -1, "mnrl_volfrac/mnrl_area required");
  if (n.Nix + n.Nsr > 0 && !cl->total_sorb_eq) return fail(c, -1, "total_sorb_eq required with sorption");
  if (n.Nix > 0 && !cl->eqionx_ref_cation_sorbed_conc) return fail(c, -1, "eqionx_ref_cation_sorbed_conc required");
  if (n.Nsr > 0 && !cl->srfcplxrxn_free_site_conc) return fail(c, -1, "srfcplxrxn_free_site_conc required");
  bool rock = false;
  for (int r = 0; r < n.Nsr; ++r) rock |= n.srtype[r] == PFCHEM_ROCK_SURFACE;
  if (rock && !cl->soil_particle_density) return fail(c, -1, "soil_particle_density required for ROCK surfaces");
  if (n.use_h2o && !cl->ln_act_h2o) return fail(c, -1, "ln_act_h2o required with use_activity_h2o");
  return 0;
}

// Fills CellArgs from a pfchem_cells whose pointers are device pointers.
CellArgs device_args(const pfchem_cells *cl, double dt) {
  CellArgs a{};
  a.ncells = cl->ncells;
  a.dt = dt;
  a.temp = cl->temperature;
  a.sat = cl->saturation;
  a.den = cl->den_kg;
  a.por = cl->porosity;
  a.vol = cl->volume;
  a.rho_s = cl->soil_particle_density;
  a.active = cl->active;
  a.total = cl->total;
  a.total_stride_cell = 1;
  a.total_stride_comp = cl->ncells;
  a.pri_molal = cl->pri_molal;
  a.ionic = cl->ionic_strength;
  a.lnaw = cl->ln_act_h2o;
  a.vf = cl->mnrl_volfrac;
  a.area = cl->mnrl_area;
  a.sorb = cl->total_sorb_eq;
  a.ixref = cl->eqionx_ref_cation_sorbed_conc;
  a.srfree = cl->srfcplxrxn_free_site_conc;
  a.total_out = cl->total_out;
  a.rate = cl->mnrl_rate;
  a.sec_molal = cl->sec_molal;
  a.iters = cl->iterations;
  a.status = cl->status;
  a.alt_guess = cl->alt_guess;
  a.interleaved_out = nullptr;
  return a;
}

// Grows the prologue record buffer to `ncells` cells (drops the cached graph,
// whose nodes point at the old buffer).
int reserve_prep(pfchem_ctx *c, int64_t ncells) {
  if (c->prep_cells >= ncells) return 0;
  if (c->prep) cudaFree(c->prep);
  c->prep = nullptr;
  c->prep_cells = 0;
  if (c->graph) {
    cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
  }
  CUDA_TRY(c, cudaMalloc(&c->prep, (size_t)gen_prep_fields(c->net) * ncells * sizeof(double)));
  c->prep_cells = ncells;
  return 0;
}

// Enqueues one reaction step on `st`: statistics reset, warm-start inference
// (when `predict`; a.alt_guess must then point at the surrogate's guess
// buffer), the prologue and the persistent solve.  Allocates nothing.
int enqueue_step(pfchem_ctx *c, const CellArgs &a, bool predict, cudaStream_t st, Scratch *scr = nullptr,
                 double *prep = nullptr, bool pack = true) {
  const DevNet &n = c->net;
  const pfchem_launch &L = c->launch;
  const int grid = std::max(1, c->num_sms * L.blocks_per_sm);
  if (!scr) scr = c->scratch;
  if (!prep) prep = c->prep;
  // the generated kernel is compiled for one block size and shared-memory
  // layout (its per-thread stride and the dynamic shared memory it expects):
  // never launch it with another
  if (is_specialized(L.variant) &&
      (!c->gen_fn || c->gen_block != L.block_threads ||
       c->gen_compact != (L.variant == PFCHEM_KERNEL_SPECIALIZED_COMPACT)))
    return fail(c, -1, "launch (%d threads, %s layout) does not match the loaded specialized kernel",
                L.block_threads, L.variant == PFCHEM_KERNEL_SPECIALIZED_COMPACT ? "compact" : "augmented");
  cudaError_t me = cudaMemsetAsync(scr, 0, sizeof(Scratch), st);
  if (me != cudaSuccess) return fail(c, -2, "statistics reset: %s", cudaGetErrorString(me));
  cudaError_t pe =
      predict ? surrogate_predict(c->sur, n, a, const_cast<double *>(a.alt_guess), st, pack) : cudaSuccess;
  if (pe != cudaSuccess) return fail(c, -2, "surrogate launch: %s", cudaGetErrorString(pe));
  cudaError_t le = is_specialized(L.variant)
                       ? gen_launch(c->gen_fn, c->gen_pro, n, a, scr, prep, grid, L.block_threads,
                                    L.refill_min_idle, st, L.variant == PFCHEM_KERNEL_SPECIALIZED_COMPACT)
                   : is_coop(L.variant)
                       ? coop_launch(coop_lanes(L.variant), n, a, c->coop_tables, scr, grid, L.block_threads, st)
                       : launch_react(n, a, scr, grid, L.block_threads, L.refill_min_idle, st);
  if (le != cudaSuccess) return fail(c, -2, "solve launch: %s", cudaGetErrorString(le));
  return 0;
}

int run_solve(pfchem_ctx *c, const CellArgs &a_in) {
  const DevNet &n = c->net;
  if (a_in.ncells == 0) {
    c->stats = pfchem_stats{};
    return 0;
  }
  CellArgs a = a_in;
  const bool predict = c->sur && c->sur_on && surrogate_trained(c->sur) && !a.alt_guess;
  if (predict) {
    cudaError_t pe = surrogate_prepare(c->sur, a.ncells);
    if (pe != cudaSuccess) return fail(c, -2, "surrogate buffers: %s", cudaGetErrorString(pe));
    a.alt_guess = surrogate_guess_buffer(c->sur);
  }
  const pfchem_launch &L = c->launch;
  if (is_specialized(L.variant)) {
    const int re = reserve_prep(c, a.ncells);
    if (re) return re;
  }
  const bool same = c->graph && std::memcmp(&a, &c->graph_args, sizeof(CellArgs)) == 0 &&
                    std::memcmp(&L, &c->graph_launch, sizeof(pfchem_launch)) == 0;
  if (!same) {
    // capture memset(scratch) + solve into a graph and keep it for replays
    if (c->graph) {
      cudaGraphExecDestroy(c->graph);
      c->graph = nullptr;
    }
    cudaGraph_t g;
    CUDA_TRY(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    const int ee = enqueue_step(c, a, predict, c->stream);
    cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
    if (ee) return ee;
    if (ce != cudaSuccess) return fail(c, -2, "graph capture: %s", cudaGetErrorString(ce));
    cudaError_t ie = cudaGraphInstantiate(&c->graph, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) return fail(c, -2, "graph instantiate: %s", cudaGetErrorString(ie));
    c->graph_args = a;
    c->graph_launch = L;
  }
  CUDA_TRY(c, cudaEventRecord(c->ev0, c->stream));
  CUDA_TRY(c, cudaGraphLaunch(c->graph, c->stream));
  CUDA_TRY(c, cudaEventRecord(c->ev1, c->stream));
  Scratch h;
  CUDA_TRY(c, cudaMemcpyAsync(&h, c->scratch, sizeof(Scratch), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  c->stats.ncells = a.ncells;
  c->stats.sum_iterations = (int64_t)h.sum_iter;
  c->stats.max_iterations = (int32_t)h.max_iter;
  c->stats.nonconverged = (int32_t)h.nonconverged;
  c->stats.alt_guess_used = (int64_t)h.alt_used;
  c->stats.kernel_ms = ms;
  c->stats.lane_slots = 32 * (int64_t)h.newton_trips;
  c->stats.drain_ms = drain_ms(h);
  return (int)h.nonconverged;
}

int react_host(pfchem_ctx *c, double dt, pfchem_cells *cl, double *tran_xx, int32_t ncomp) {
  const DevNet &n = c->net;
  const int64_t nc = cl->ncells;
  const size_t d1 = nc * sizeof(double), dN = n.N * d1, dM = std::max(n.Nm, 1) * d1;
  CellArgs a{};
  void *p;
  int e = 0;
#define ST(slot, ptr, bytes, up)                                 \
  if ((e = stage(c, slot, (ptr), (bytes), &p, (up))) != 0) return e; \
  (void)0
  ST(0, cl->temperature, d1, true); a.temp = (const double *)p;
  ST(1, cl->saturation, d1, true); a.sat = (const double *)p;
  ST(2, cl->den_kg, d1, true); a.den = (const double *)p;
  ST(3, cl->porosity, d1, true); a.por = (const double *)p;
  ST(4, cl->volume, d1, true); a.vol = (const double *)p;
  ST(5, cl->soil_particle_density, d1, true); a.rho_s = (const double *)p;
  ST(6, cl->active, nc * sizeof(int32_t), true); a.active = (const int32_t *)p;
  if (tran_xx) {
    ST(7, tran_xx, (size_t)ncomp * d1, true);
    a.total = (const double *)p;
    a.interleaved_out = (double *)p;
    a.total_stride_cell = ncomp;
    a.total_stride_comp = 1;
  } else {
    ST(7, cl->total, dN, true);
    a.total = (const double *)p;
    a.total_stride_cell = 1;
    a.total_stride_comp = nc;
  }
  ST(8, cl->pri_molal, dN, true); a.pri_molal = (double *)p;
  ST(9, cl->ionic_strength, d1, true); a.ionic = (double *)p;
  ST(10, cl->ln_act_h2o, d1, true); a.lnaw = (double *)p;
  ST(11, cl->mnrl_volfrac, dM, true); a.vf = (double *)p;
  ST(12, cl->mnrl_area, dM, true); a.area = (double *)p;
  ST(13, cl->total_sorb_eq, dN, true); a.sorb = (double *)p;
  ST(14, cl->eqionx_ref_cation_sorbed_conc, std::max(n.Nix, 1) * d1, true); a.ixref = (double *)p;
  ST(15, cl->srfcplxrxn_free_site_conc, std::max(n.Nsr, 1) * d1, true); a.srfree = (double *)p;
  ST(16, cl->total_out, dN, false); a.total_out = (double *)p;
  ST(17, cl->mnrl_rate, dM, false); a.rate = (double *)p;
  ST(18, cl->sec_molal, std::max(n.Nc, 1) * d1, false); a.sec_molal = (double *)p;
  ST(19, cl->iterations, nc * sizeof(int32_t), false); a.iters = (int32_t *)p;
  ST(20, cl->status, nc * sizeof(int32_t), false); a.status = (int32_t *)p;
  ST(21, cl->alt_guess, dN, true); a.alt_guess = (const double *)p;
#undef ST
  a.ncells = nc;
  a.dt = dt;
  int r = run_solve(c, a);
  if (r < 0) return r;
  auto down = [&](void *host, const void *dev, size_t bytes) -> int {
    if (host && dev) CUDA_TRY(c, cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, c->stream));
    return 0;
  };
  if ((e = down(cl->pri_molal, a.pri_molal, dN))) return e;
  if ((e = down(cl->ionic_strength, a.ionic, d1))) return e;
  if ((e = down(cl->ln_act_h2o, a.lnaw, d1))) return e;
  if ((e = down(cl->mnrl_volfrac, a.vf, dM))) return e;
  if ((e = down(cl->total_sorb_eq, a.sorb, dN))) return e;
  if ((e = down(cl->eqionx_ref_cation_sorbed_conc, a.ixref, std::max(n.Nix, 1) * d1))) return e;
  if ((e = down(cl->srfcplxrxn_free_site_conc, a.srfree, std::max(n.Nsr, 1) * d1))) return e;
  if ((e = down(cl->total_out, a.total_out, dN))) return e;
  if ((e = down(cl->mnrl_rate, a.rate, dM))) return e;
  if ((e = down(cl->sec_molal, a.sec_molal, std::max(n.Nc, 1) * d1))) return e;
  if ((e = down(cl->iterations, a.iters, nc * sizeof(int32_t)))) return e;
  if ((e = down(cl->status, a.status, nc * sizeof(int32_t)))) return e;
  if (tran_xx && (e = down(tran_xx, a.total, (size_t)ncomp * d1))) return e;
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return r;
}

}  // namespace

namespace pfchem {
// Flattens and validates a network (used by the allocation-free entry point).
int flatten_network(const pfchem_network *w, const pfchem_options *o, DevNet &n, char *err, size_t errlen) {
  pfchem_ctx tmp;
  int r = build_devnet(&tmp, w, o, n);
  if (r && err && errlen) snprintf(err, errlen, "%s", tmp.err);
  return r;
}
CellArgs cell_args(const pfchem_cells *cl, double dt) { return device_args(cl, dt); }
}  // namespace pfchem

extern "C" {

int pfchem_create(pfchem_ctx **out, int device) {
  if (!out) return -1;
  *out = nullptr;
  pfchem_ctx *c = new pfchem_ctx();
  c->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) {
    delete c;
    return -2;
  }
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&c->scratch, sizeof(Scratch)) != cudaSuccess || cudaEventCreate(&c->ev0) != cudaSuccess ||
      cudaEventCreate(&c->ev1) != cudaSuccess) {
    pfchem_destroy(c);
    return -2;
  }
  *out = c;
  return 0;
}

void pfchem_destroy(pfchem_ctx *c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->graph) cudaGraphExecDestroy(c->graph);
  if (c->sur) surrogate_destroy(c->sur);
  if (c->prep) cudaFree(c->prep);
  if (c->coop_tables) cudaFree(c->coop_tables);
  for (auto &b : c->stage)
    if (b.ptr) cudaFree(b.ptr);
  if (c->scratch) cudaFree(c->scratch);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char *pfchem_last_error(const pfchem_ctx *c) { return c ? c->err : "null context"; }

int pfchem_set_network(pfchem_ctx *c, const pfchem_network *net, const pfchem_options *opt) {
  if (!c) return -1;
  cudaSetDevice(c->device);
  DevNet n;
  int e = build_devnet(c, net, opt, n);
  if (e) return e;
  // gather lists of the cooperative kernels
  {
    std::vector<char> h(coop_tables_bytes());
    coop_build_tables(n, reinterpret_cast<CoopTables *>(h.data()));
    if (!c->coop_tables) CUDA_TRY(c, cudaMalloc(&c->coop_tables, h.size()));
    CUDA_TRY(c, cudaMemcpy(c->coop_tables, h.data(), h.size(), cudaMemcpyHostToDevice));
  }
  c->net = n;
  c->opt = *opt;
  c->has_net = true;
  c->gen_fn = nullptr;
  c->gen_block = 0;
  if (c->graph) {
    cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
  }
  if (!c->launch_forced) {
    // the network-specialized kernel is the default (a compile failure is an
    // error); the table-driven kernel where the specialized one does not apply
    default_launch(c);
    if (specialized_supports(n) && default_specialized_launch(c) != 0) return -2;
  } else if (is_coop(c->launch.variant) && !coop_supports(n)) {
    return fail(c, -1, "the cooperative kernels do not support these options (linear update, NEWTON activity "
                       "algorithm or activity of water); set another launch");
  } else if (is_specialized(c->launch.variant) && !specialized_supports(n)) {
    return fail(c, -1, "the network-specialized kernel does not support the NEWTON activity algorithm at every "
                       "Newton iteration; set a PFCHEM_KERNEL_GENERIC launch");
  } else if (is_specialized(c->launch.variant)) {
    if (ensure_gen(c, c->launch.block_threads, c->launch.variant == PFCHEM_KERNEL_SPECIALIZED_COMPACT) < 1) return -2;
  }
  return 0;
}

int pfchem_react_batch(pfchem_ctx *c, double dt, pfchem_cells *cl) {
  int e = check_cells(c, cl);
  if (e) return e;
  if (!(dt > 0.0)) return fail(c, -1, "dt must be > 0");
  if (cl->ncells == 0) {
    c->stats = pfchem_stats{};
    return 0;
  }
  if (!cl->total) return fail(c, -1, "total is null");
  cudaSetDevice(c->device);
  if (cl->on_device) return run_solve(c, device_args(cl, dt));
  return react_host(c, dt, cl, nullptr, 0);
}

int pfchem_react_batch_interleaved(pfchem_ctx *c, double dt, int32_t ncomp, double *tran_xx, pfchem_cells *cl) {
  int e = check_cells(c, cl);
  if (e) return e;
  if (ncomp < c->net.N) return fail(c, -1, "ncomp %d < naqcomp %d", ncomp, c->net.N);
  if (!(dt > 0.0)) return fail(c, -1, "dt must be > 0");
  if (cl->ncells == 0) {
    c->stats = pfchem_stats{};
    return 0;
  }
  if (!tran_xx) return fail(c, -1, "tran_xx is null");
  cudaSetDevice(c->device);
  if (cl->on_device) {
    CellArgs a = device_args(cl, dt);
    a.total = tran_xx;
    a.interleaved_out = tran_xx;
    a.total_stride_cell = ncomp;
    a.total_stride_comp = 1;
    return run_solve(c, a);
  }
  return react_host(c, dt, cl, tran_xx, ncomp);
}

int pfchem_update_kinetic_state(pfchem_ctx *c, double dt, pfchem_cells *cl) {
  int e = check_cells(c, cl);
  if (e) return e;
  if (cl->ncells == 0) return 0;
  if (!cl->on_device) return fail(c, -1, "pfchem_update_kinetic_state takes device pointers");
  if (!cl->total) return fail(c, -1, "total is null");
  cudaSetDevice(c->device);
  CellArgs a = device_args(cl, dt);
  if (a.ncells == 0) return 0;
  cudaError_t le = launch_kinetic_state(c->net, a, c->stream);
  if (le != cudaSuccess) return fail(c, -2, "kinetic-state launch: %s", cudaGetErrorString(le));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return 0;
}

int pfchem_reserve(pfchem_ctx *c, int64_t ncells) {
  if (!c) return -1;
  if (!c->has_net) return fail(c, -1, "pfchem_set_network must be called first");
  if (ncells < 0) return fail(c, -1, "ncells < 0");
  cudaSetDevice(c->device);
  int e = reserve_prep(c, ncells);
  if (e) return e;
  if (c->sur) {
    cudaError_t pe = surrogate_prepare(c->sur, ncells);
    if (pe != cudaSuccess) return fail(c, -2, "surrogate buffers: %s", cudaGetErrorString(pe));
  }
  return 0;
}

int pfchem_react_batch_async(pfchem_ctx *c, double dt, pfchem_cells *cl, void *stream) {
  int e = check_cells(c, cl);
  if (e) return e;
  if (!cl->on_device && cl->ncells) return fail(c, -1, "pfchem_react_batch_async takes device pointers");
  if (!(dt > 0.0)) return fail(c, -1, "dt must be > 0");
  if (cl->ncells == 0) {
    c->async_cells = 0;
    return 0;
  }
  if (!cl->total) return fail(c, -1, "total is null");
  cudaSetDevice(c->device);
  CellArgs a = device_args(cl, dt);
  c->async_cells = a.ncells;
  if (a.ncells == 0) return 0;
  if (is_specialized(c->launch.variant) && c->prep_cells < a.ncells)
    return fail(c, -1, "%lld cells exceed the reserved %lld: call pfchem_reserve first", (long long)a.ncells,
                (long long)c->prep_cells);
  const bool predict = c->sur && c->sur_on && surrogate_trained(c->sur) && !a.alt_guess;
  if (predict) {
    if (!surrogate_ready(c->sur, a.ncells))
      return fail(c, -1, "warm-start buffers are not reserved for %lld cells: call pfchem_reserve first",
                  (long long)a.ncells);
    a.alt_guess = surrogate_guess_buffer(c->sur);
  }
  return enqueue_step(c, a, predict, (cudaStream_t)stream);
}

int pfchem_async_stats(pfchem_ctx *c, pfchem_stats *s) {
  if (!c || !s) return -1;
  cudaSetDevice(c->device);
  Scratch h;
  CUDA_TRY(c, cudaMemcpyAsync(&h, c->scratch, sizeof(Scratch), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  *s = pfchem_stats{};
  s->ncells = c->async_cells;
  s->sum_iterations = (int64_t)h.sum_iter;
  s->max_iterations = (int32_t)h.max_iter;
  s->nonconverged = (int32_t)h.nonconverged;
  s->alt_guess_used = (int64_t)h.alt_used;
  s->kernel_ms = 0.0;
  s->lane_slots = 32 * (int64_t)h.newton_trips;
  s->drain_ms = drain_ms(h);
  return 0;
}

int pfchem_reaction_blocks(pfchem_ctx *c, pfchem_cells *cl, pfchem_reaction_blocks_out *out) {
  int e = check_cells(c, cl);
  if (e) return e;
  if (cl->ncells == 0) return 0;
  if (!cl->on_device) return fail(c, -1, "pfchem_reaction_blocks takes device pointers");
  if (!out || !out->res || !out->jac) return fail(c, -1, "res and jac are required");
  cudaSetDevice(c->device);
  CellArgs a = device_args(cl, 1.0);
  if (a.ncells == 0) return 0;
  cudaError_t le = launch_reaction_blocks(c->net, a, out->res, out->jac, out->total, out->dtotal, out->total_sorb,
                                          out->dtotal_sorb, c->stream);
  if (le != cudaSuccess) return fail(c, -2, "reaction-blocks launch: %s", cudaGetErrorString(le));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return 0;
}

int pfchem_equilibrate_constraints(pfchem_ctx *c, pfchem_cells *cl, const pfchem_constraint *con) {
  if (!c || !cl || !con || !con->type || !con->value) return fail(c, -1, "null argument");
  if (!c->has_net) return fail(c, -1, "pfchem_set_network has not been called");
  if (!cl->on_device) return fail(c, -1, "pfchem_equilibrate_constraints takes device pointers");
  if (c->net.act_newton) return fail(c, -1, "constraint speciation supports the LAG activity algorithm only");
  const DevNet &n = c->net;
  if (!cl->temperature || !cl->den_kg || !cl->pri_molal || !cl->ionic_strength || !cl->porosity || !cl->saturation ||
      !cl->volume)
    return fail(c, -1, "a required per-cell array is null");
  if (n.Nm > 0 && (!cl->mnrl_volfrac || !cl->mnrl_area)) return fail(c, -1, "mnrl_volfrac/mnrl_area required");
  if (n.Nix + n.Nsr > 0 && (!cl->total_sorb_eq || (n.Nix && !cl->eqionx_ref_cation_sorbed_conc) ||
                            (n.Nsr && !cl->srfcplxrxn_free_site_conc)))
    return fail(c, -1, "sorption state arrays required");
  int ngas_rows = 0;
  for (int j = 0; j < n.N; ++j) {
    const int t = con->type[j];
    if (t < PFCHEM_CONSTRAINT_TOTAL || t > PFCHEM_CONSTRAINT_TOTAL_SORB)
      return fail(c, -1, "component %d: unknown constraint type %d", j + 1, t);
    if (t == PFCHEM_CONSTRAINT_MINERAL && (!con->mineral || con->mineral[j] < 1 || con->mineral[j] > n.Nm))
      return fail(c, -1, "component %d: MINERAL row needs a kinetic mineral id in [1,%d]", j + 1, n.Nm);
    if (t == PFCHEM_CONSTRAINT_TOTAL_SORB && n.Nix + n.Nsr == 0)
      return fail(c, -1, "component %d: TOTAL_SORB row in a network without sorption", j + 1);
    if (t == PFCHEM_CONSTRAINT_GAS) {
      if (!con->mineral || con->mineral[j] < 1 || con->mineral[j] > con->npassive_gas)
        return fail(c, -1, "component %d: GAS row needs a passive gas id in [1,%d]", j + 1, con->npassive_gas);
      if (++ngas_rows > PFCHEM_MAX_GAS_ROWS)
        return fail(c, -1, "more than %d GAS rows", PFCHEM_MAX_GAS_ROWS);
      if (!con->paseqspecid || !con->paseqstoich || (n.isothermal ? !con->paseqlogK : !con->paseqlogKcoef))
        return fail(c, -1, "GAS rows need paseqspecid, paseqstoich and %s",
                    n.isothermal ? "paseqlogK" : "paseqlogKcoef");
      if (con->paseq_ld < 1 || con->paseq_ld > PFCHEM_MAX_NNZ)
        return fail(c, -1, "paseq_ld %d out of [1,%d]", con->paseq_ld, PFCHEM_MAX_NNZ);
      const int g = con->mineral[j] - 1, ns = con->paseqspecid[g * (con->paseq_ld + 1)];
      if (ns < 1 || ns > con->paseq_ld) return fail(c, -1, "gas %d: %d species", g + 1, ns);
      for (int k = 1; k <= ns; ++k) {
        const int id = con->paseqspecid[g * (con->paseq_ld + 1) + k];
        if (id < 1 || id > n.N) return fail(c, -1, "gas %d: species id %d out of [1,%d]", g + 1, id, n.N);
      }
    }
  }
  cudaSetDevice(c->device);
  CellArgs a = device_args(cl, 1.0);
  if (a.ncells == 0) return 0;
  CUDA_TRY(c, cudaMemsetAsync(c->scratch, 0, sizeof(Scratch), c->stream));
  cudaError_t le = launch_constraint(n, a, *con, con->max_iterations > 0 ? con->max_iterations : 10000, c->scratch,
                                     c->stream);
  if (le != cudaSuccess) return fail(c, -2, "constraint launch: %s", cudaGetErrorString(le));
  Scratch h;
  CUDA_TRY(c, cudaMemcpyAsync(&h, c->scratch, sizeof(Scratch), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return (int)h.nonconverged;
}

int pfchem_update_mineral_properties(pfchem_ctx *c, pfchem_cells *cl, const pfchem_mineral_update *mu) {
  if (!c || !cl || !mu) return fail(c, -1, "null argument");
  if (!c->has_net) return fail(c, -1, "pfchem_set_network has not been called");
  if (!cl->on_device) return fail(c, -1, "pfchem_update_mineral_properties takes device pointers");
  const int Nm = c->net.Nm;
  if (Nm > 0 && (!cl->mnrl_volfrac || !cl->mnrl_area)) return fail(c, -1, "mnrl_volfrac/mnrl_area required");
  if (!cl->porosity) return fail(c, -1, "porosity required");
  if (mu->update_porosity && Nm > 0 && !mu->porosity) return fail(c, -1, "porosity output required");
  if (mu->update_surface_area && Nm > 0) {
    if (!mu->surf_area_vol_frac_pwr || !mu->mnrl_volfrac0 || !mu->mnrl_area0)
      return fail(c, -1, "surf_area_vol_frac_pwr, mnrl_volfrac0 and mnrl_area0 required");
    if (mu->surface_area_with_porosity && (!mu->surf_area_porosity_pwr || !mu->porosity0))
      return fail(c, -1, "surf_area_porosity_pwr and porosity0 required with surface_area_with_porosity");
  }
  if (mu->armor_crit_vol_frac && mu->update_surface_area && Nm > 0 && !mu->surf_area_vol_frac_pwr)
    return fail(c, -1, "armoring needs surf_area_vol_frac_pwr");
  cudaSetDevice(c->device);
  CellArgs a = device_args(cl, 1.0);
  if (a.ncells == 0) {
    if (mu->armor_flag_out) *mu->armor_flag_out = mu->armor_flag;
    return 0;
  }
  // the flag after the last cell comes back through the context's scratch
  int *flag_dev = reinterpret_cast<int *>(&c->scratch->armor_flag);
  cudaError_t le = launch_mineral_properties(a, Nm, *mu, flag_dev, c->stream);
  if (le != cudaSuccess) return fail(c, -2, "mineral-properties launch: %s", cudaGetErrorString(le));
  int flag = mu->armor_flag;
  if (mu->armor_flag_out && mu->update_surface_area)
    CUDA_TRY(c, cudaMemcpyAsync(&flag, flag_dev, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (mu->armor_flag_out) *mu->armor_flag_out = flag;
  return 0;
}

int pfchem_last_stats(const pfchem_ctx *c, pfchem_stats *s) {
  if (!c || !s) return -1;
  *s = c->stats;
  return 0;
}

int pfchem_get_launch(const pfchem_ctx *c, pfchem_launch *l) {
  if (!c || !l) return -1;
  *l = c->launch;
  return 0;
}

int pfchem_set_launch(pfchem_ctx *c, const pfchem_launch *l) {
  if (!c || !l) return -1;
  if (l->block_threads < 32 || l->block_threads > 256 || l->block_threads % 32)
    return fail(c, -1, "block_threads must be a multiple of 32 in [32, 256]");
  if (l->refill_min_idle < 1 || l->refill_min_idle > 32) return fail(c, -1, "refill_min_idle must be in [1, 32]");
  if (l->blocks_per_sm < 1) return fail(c, -1, "blocks_per_sm must be >= 1");
  if (!is_specialized(l->variant) && !is_coop(l->variant) && l->variant != PFCHEM_KERNEL_GENERIC)
    return fail(c, -1, "unknown kernel variant %d", l->variant);
  if (c->has_net && is_coop(l->variant)) {
    if (!coop_supports(c->net))
      return fail(c, -1, "the cooperative kernels do not support these options (linear update, NEWTON activity "
                         "algorithm or activity of water)");
    const int nb = coop_blocks_per_sm(coop_lanes(l->variant), c->net, l->block_threads);
    if (nb < 1) return fail(c, -1, "cooperative kernel with %d threads per block does not fit on an SM", l->block_threads);
    if (l->blocks_per_sm > nb) return fail(c, -1, "at most %d blocks of %d threads fit on an SM", nb, l->block_threads);
    c->launch = *l;
    c->launch_forced = true;
    return 0;
  }
  if (c->has_net) {
    if (is_specialized(l->variant) && !specialized_supports(c->net))
      return fail(c, -1, "the network-specialized kernel does not support the NEWTON activity algorithm at every "
                         "Newton iteration");
    if (is_specialized(l->variant)) {
      const bool cmp = l->variant == PFCHEM_KERNEL_SPECIALIZED_COMPACT;
      if (gen_shared_bytes(c->net, l->block_threads, cmp) > 227 * 1024)
        return fail(c, -1, "block_threads %d needs too much shared memory", l->block_threads);
      int nb = ensure_gen(c, l->block_threads, cmp);
      if (nb < 1) return -2;
      if (l->blocks_per_sm > nb) return fail(c, -1, "at most %d blocks of %d threads fit on an SM", nb, l->block_threads);
    } else {
      const size_t shm = (size_t)c->net.N * c->net.N * l->block_threads * sizeof(double);
      if (shm > 227 * 1024) return fail(c, -1, "block_threads %d needs %zu bytes of shared memory", l->block_threads, shm);
      int nb = max_active_blocks(c->net, l->block_threads);
      if (nb < 1) return fail(c, -1, "mapping does not fit on an SM");
      if (l->blocks_per_sm > nb) return fail(c, -1, "at most %d blocks of %d threads fit on an SM", nb, l->block_threads);
    }
  }
  c->launch = *l;
  c->launch_forced = true;
  return 0;
}

int pfchem_autotune(pfchem_ctx *c, double dt, pfchem_cells *cl) {
  int e = check_cells(c, cl);
  if (e) return e;
  if (cl->ncells == 0) return 0;
  if (!cl->on_device) return fail(c, -1, "pfchem_autotune takes device pointers");
  cudaSetDevice(c->device);
  const DevNet &n = c->net;
  if (!specialized_supports(n)) return 0;  // only the table-driven kernel applies: nothing to choose
  const int64_t nc = cl->ncells;
  // back up every array a solve writes, restore after each trial
  struct Arr {
    double *p;
    size_t bytes;
    void *save;
  };
  std::vector<Arr> arrs;
  auto add = [&](double *p, size_t k) {
    if (p) arrs.push_back({p, k * nc * sizeof(double), nullptr});
  };
  add(cl->pri_molal, n.N);
  add(cl->ionic_strength, 1);
  add(cl->ln_act_h2o, 1);
  add(cl->mnrl_volfrac, std::max(n.Nm, 1));
  add(cl->total_sorb_eq, n.N);
  add(cl->eqionx_ref_cation_sorbed_conc, std::max(n.Nix, 1));
  add(cl->srfcplxrxn_free_site_conc, std::max(n.Nsr, 1));
  for (auto &x : arrs) {
    cudaError_t ae = cudaMalloc(&x.save, x.bytes);
    if (ae == cudaSuccess) ae = cudaMemcpyAsync(x.save, x.p, x.bytes, cudaMemcpyDeviceToDevice, c->stream);
    if (ae != cudaSuccess) {  // release the backups made so far
      for (auto &y : arrs)
        if (y.save) cudaFree(y.save);
      return fail(c, -2, "autotune state backup: %s", cudaGetErrorString(ae));
    }
  }
  // candidates: block of 32 or 64 threads, augmented or compact shared-memory
  // layout (compiled concurrently), as many resident blocks per SM as fit or
  // one fewer, refill at 1, 2, 4 or 8 idle lanes; each timed twice (the
  // faster run counts), the state restored after every run; then the three
  // fastest timed three more times each, the fastest of all their runs kept
  // (candidates a few per cent apart are otherwise ordered by noise)
  const int blocks[] = {32, 64};
  const int refills[] = {1, 2, 4, 8};
  std::vector<std::pair<int, bool>> cands;
  for (int variant : {PFCHEM_KERNEL_SPECIALIZED, PFCHEM_KERNEL_SPECIALIZED_COMPACT})
    for (int b : blocks) {
      const bool cmp = variant == PFCHEM_KERNEL_SPECIALIZED_COMPACT;
      if (gen_shared_bytes(n, b, cmp) <= 227 * 1024) cands.push_back({b, cmp});
    }
  {
    std::string err;
    if (gen_kernels_prepare(n, cands, &err)) {
      for (auto &x : arrs) cudaFree(x.save);
      return fail(c, -2, "specialized kernel: %s", err.c_str());
    }
  }
  double best = 1e30;
  pfchem_launch best_l = c->launch;
  std::vector<std::pair<double, pfchem_launch>> timed;
  int rc = 0;
  auto time_launch = [&](const pfchem_launch &l, int reps) {
    double ms = 1e30;
    // load the generated kernel this launch was compiled for
    if (is_specialized(l.variant) &&
        ensure_gen(c, l.block_threads, l.variant == PFCHEM_KERNEL_SPECIALIZED_COMPACT) < 1) {
      rc = -2;
      return ms;
    }
    c->launch = l;
    for (int rep = 0; rep < reps; ++rep) {
      rc = pfchem_react_batch(c, dt, cl);
      if (rc < 0) break;
      ms = std::min(ms, c->stats.kernel_ms);
      for (auto &x : arrs) cudaMemcpyAsync(x.p, x.save, x.bytes, cudaMemcpyDeviceToDevice, c->stream);
    }
    return ms;
  };
  for (const auto &cand : cands) {
    const int b = cand.first;
    const bool cmp = cand.second;
    const int variant = cmp ? PFCHEM_KERNEL_SPECIALIZED_COMPACT : PFCHEM_KERNEL_SPECIALIZED;
    const int nb = ensure_gen(c, b, cmp);
    if (nb < 1) continue;
    for (int bps = nb; bps >= std::max(1, nb - 1) && rc >= 0; --bps) {
      for (int r : refills) {
        const pfchem_launch l{b, bps, r, variant};
        const double ms = time_launch(l, 2);
        if (rc < 0) break;
        timed.push_back({ms, l});
      }
    }
    if (rc < 0) break;
  }
  // cooperative kernels: 8, 16 or 32 lanes per cell, 128-thread blocks
  if (rc >= 0 && coop_supports(n)) {
    for (int variant : {PFCHEM_KERNEL_COOP8, PFCHEM_KERNEL_COOP16, PFCHEM_KERNEL_COOP32}) {
      const int nb = coop_blocks_per_sm(coop_lanes(variant), n, 128);
      for (int bps = nb; bps >= std::max(1, nb - 1) && nb >= 1 && rc >= 0; --bps) {
        const pfchem_launch l{128, bps, 1, variant};
        const double ms = time_launch(l, 2);
        if (rc >= 0) timed.push_back({ms, l});
      }
    }
  }
  if (rc >= 0) {
    std::stable_sort(timed.begin(), timed.end(),
                     [](const std::pair<double, pfchem_launch> &x, const std::pair<double, pfchem_launch> &y) {
                       return x.first < y.first;
                     });
    for (size_t k = 0; k < timed.size() && k < 3 && rc >= 0; ++k) {
      const double ms = std::min(timed[k].first, time_launch(timed[k].second, 3));
      if (rc >= 0 && ms < best) {
        best = ms;
        best_l = timed[k].second;
      }
    }
  }
  for (auto &x : arrs) {
    cudaMemcpyAsync(x.p, x.save, x.bytes, cudaMemcpyDeviceToDevice, c->stream);
  }
  cudaStreamSynchronize(c->stream);
  for (auto &x : arrs) cudaFree(x.save);
  if (rc < 0) return rc;
  c->launch = best_l;
  c->launch_forced = true;
  if (is_specialized(best_l.variant) &&
      ensure_gen(c, best_l.block_threads, best_l.variant == PFCHEM_KERNEL_SPECIALIZED_COMPACT) < 1)
    return -2;
  return 0;
}

static int need_surrogate(pfchem_ctx *c, uint64_t seed) {
  if (!c->has_net) return fail(c, -1, "pfchem_set_network has not been called");
  if (c->sur) return 0;
  std::string e;
  c->sur = surrogate_create(c->net.N, seed, &e);
  if (!c->sur) return fail(c, -2, "surrogate: %s", e.c_str());
  return 0;
}

int pfchem_surrogate_features(pfchem_ctx *c, pfchem_cells *cl, float *X) {
  int e = check_cells(c, cl);
  if (e) return e;
  if (!cl->on_device || !X) return fail(c, -1, "device pointers required");
  cudaSetDevice(c->device);
  CellArgs a = device_args(cl, 1.0);
  if (a.ncells == 0) return 0;
  CUDA_TRY(c, surrogate_features(c->net, a, X, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return 0;
}

// Standardisation from up to 65536 samples copied to the host.
static int fit_norm(pfchem_ctx *c, const float *X, const double *molal, int64_t M) {
  const int N = c->net.N;
  const int64_t S = std::min<int64_t>(M, 65536);
  std::vector<float> xs(S * 16);
  std::vector<double> ms((size_t)N * S);
  CUDA_TRY(c, cudaMemcpy(xs.data(), X, S * 16 * sizeof(float), cudaMemcpyDeviceToHost));
  for (int j = 0; j < N; ++j)
    CUDA_TRY(c, cudaMemcpy(ms.data() + (size_t)j * S, molal + (size_t)j * M, S * sizeof(double),
                           cudaMemcpyDeviceToHost));
  float fmu[16], fisd[16], tmu[PFCHEM_MAX_PRI], tsd[PFCHEM_MAX_PRI];
  for (int f = 0; f < 16; ++f) {
    double s = 0, s2 = 0;
    for (int64_t r = 0; r < S; ++r) {
      s += xs[r * 16 + f];
      s2 += (double)xs[r * 16 + f] * xs[r * 16 + f];
    }
    const double mu = s / S, var = std::max(s2 / S - mu * mu, 0.0);
    fmu[f] = (float)mu;
    fisd[f] = var > 1e-12 ? (float)(1.0 / std::sqrt(var)) : 1.0f;
  }
  for (int j = 0; j < N; ++j) {
    double s = 0, s2 = 0;
    for (int64_t r = 0; r < S; ++r) {
      const double v = std::log(ms[(size_t)j * S + r]);
      s += v;
      s2 += v * v;
    }
    const double mu = s / S, var = std::max(s2 / S - mu * mu, 0.0);
    tmu[j] = (float)mu;
    tsd[j] = var > 1e-12 ? (float)std::sqrt(var) : 1.0f;
  }
  surrogate_set_norm(c->sur, fmu, fisd, tmu, tsd);
  std::memcpy(c->norm, fmu, sizeof(fmu));
  std::memcpy(c->norm + 16, fisd, sizeof(fisd));
  std::memcpy(c->norm + 32, tmu, sizeof(float) * PFCHEM_MAX_PRI);
  std::memcpy(c->norm + 32 + PFCHEM_MAX_PRI, tsd, sizeof(float) * PFCHEM_MAX_PRI);
  return 0;
}

int pfchem_surrogate_fit(pfchem_ctx *c, const float *X, const double *molal, int64_t M,
                         const pfchem_surrogate_cfg *cfg, pfchem_surrogate_report *rep) {
  if (!c || !X || !molal || !cfg) return -1;
  if (M < 1) return fail(c, -1, "no samples");
  if (cfg->batch < 1 || cfg->epochs < 1) return fail(c, -1, "batch and epochs must be >= 1");
  cudaSetDevice(c->device);
  int e = need_surrogate(c, cfg->seed);
  if (e) return e;
  if ((e = fit_norm(c, X, molal, M))) return e;
  const int N = c->net.N;
  float *T = nullptr;
  CUDA_TRY(c, cudaMalloc(&T, (size_t)M * N * sizeof(float)));
  cudaError_t ce = surrogate_targets(c->sur, molal, M, T, c->stream);
  if (ce != cudaSuccess) {
    cudaFree(T);
    return fail(c, -2, "targets: %s", cudaGetErrorString(ce));
  }
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  cudaEventRecord(t0, c->stream);
  const int64_t B = std::min<int64_t>(cfg->batch, M);
  const int64_t nb = M / B;
  std::vector<int64_t> order(nb);
  for (int64_t i = 0; i < nb; ++i) order[i] = i;
  std::mt19937_64 rng(cfg->seed ^ 0x9e3779b97f4a7c15ULL);
  float first = NAN, last_sum = 0.f;
  int64_t last_n = 0, steps = 0;
  for (int ep = 0; ep < cfg->epochs; ++ep) {
    std::shuffle(order.begin(), order.end(), rng);
    const bool last_epoch = ep == cfg->epochs - 1;
    for (int64_t i = 0; i < nb; ++i) {
      const int64_t r0 = order[i] * B;
      const bool sync = (steps == 0) || (last_epoch && (i % 16 == 0));
      // cosine decay of the learning rate over the whole fit
      const double frac = (double)steps / (double)std::max<int64_t>(1, (int64_t)cfg->epochs * nb);
      const float lr = (float)(cfg->lr * (0.02 + 0.98 * 0.5 * (1.0 + std::cos(3.14159265358979 * frac))));
      float l = surrogate_train_step(c->sur, X + r0 * 16, T + r0 * N, B, lr, cfg->weight_decay, c->stream,
                                     sync, &ce);
      if (ce != cudaSuccess) break;
      if (steps == 0) first = l / (float)(B * N);
      if (sync && last_epoch) {
        last_sum += l / (float)(B * N);
        last_n += 1;
      }
      ++steps;
    }
    if (ce != cudaSuccess) break;
  }
  cudaEventRecord(t1, c->stream);
  cudaStreamSynchronize(c->stream);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, t0, t1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  cudaFree(T);
  if (ce != cudaSuccess) return fail(c, -2, "training: %s", cudaGetErrorString(ce));
  {
    bool to = false;
    CUDA_TRY(c, surrogate_check(c->sur, &to));
    if (to) return fail(c, -2, "training: a tensor-core kernel's wait ran out");
  }
  surrogate_mark_trained(c->sur, true);
  if (c->graph) {
    cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
  }
  if (rep) {
    rep->samples = nb * B;
    rep->steps = steps;
    rep->first_loss = first;
    rep->final_loss = last_n ? last_sum / last_n : NAN;
    rep->train_ms = ms;
  }
  return 0;
}

int pfchem_surrogate_predict(pfchem_ctx *c, pfchem_cells *cl, double *guess) {
  int e = check_cells(c, cl);
  if (e) return e;
  if (!cl->on_device || !guess) return fail(c, -1, "device pointers required");
  if (!c->sur || !surrogate_trained(c->sur)) return fail(c, -1, "the surrogate has not been trained");
  cudaSetDevice(c->device);
  CellArgs a = device_args(cl, 1.0);
  if (a.ncells == 0) return 0;
  CUDA_TRY(c, surrogate_prepare(c->sur, a.ncells));
  CUDA_TRY(c, surrogate_predict(c->sur, c->net, a, surrogate_guess_buffer(c->sur), c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(guess, surrogate_guess_buffer(c->sur), (size_t)c->net.N * a.ncells * sizeof(double),
                              cudaMemcpyDeviceToDevice, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  bool to = false;
  CUDA_TRY(c, surrogate_check(c->sur, &to));
  if (to) return fail(c, -2, "prediction: a tensor-core kernel's wait ran out");
  return 0;
}

int pfchem_surrogate_backend(pfchem_ctx *c, int backend) {
  if (!c) return -1;
  if (backend != PFCHEM_MLP_MMA_SYNC && backend != PFCHEM_MLP_TCGEN05) return fail(c, -1, "unknown backend %d", backend);
  cudaSetDevice(c->device);
  int e = need_surrogate(c, 1);
  if (e) return e;
  surrogate_set_backend(c->sur, backend);
  if (c->graph) {
    cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
  }
  return 0;
}

int pfchem_surrogate_predict_layers(pfchem_ctx *c, pfchem_cells *cl, double *guess) {
  int e = check_cells(c, cl);
  if (e) return e;
  if (!cl->on_device || !guess) return fail(c, -1, "device pointers required");
  if (!c->sur || !surrogate_trained(c->sur)) return fail(c, -1, "the surrogate has not been trained");
  cudaSetDevice(c->device);
  CellArgs a = device_args(cl, 1.0);
  if (a.ncells == 0) return 0;
  CUDA_TRY(c, surrogate_prepare(c->sur, a.ncells));
  CUDA_TRY(c, surrogate_predict_layers(c->sur, c->net, a, guess, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return 0;
}

int pfchem_surrogate_enable(pfchem_ctx *c, int on) {
  if (!c) return -1;
  if (on && (!c->sur || !surrogate_trained(c->sur))) return fail(c, -1, "the surrogate has not been trained");
  c->sur_on = on != 0;
  if (c->graph) {
    cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
  }
  return 0;
}

int64_t pfchem_surrogate_gradients(pfchem_ctx *c, const float *X, const double *molal, int64_t M, float *grad_host,
                                   float *loss_host) {
  if (!c || !X || !molal || !grad_host || !loss_host) return -1;
  if (M < 1) return fail(c, -1, "no samples");
  cudaSetDevice(c->device);
  int e = need_surrogate(c, 1);
  if (e) return e;
  const int N = c->net.N;
  float *T = nullptr;
  CUDA_TRY(c, cudaMalloc(&T, (size_t)M * N * sizeof(float)));
  cudaError_t ce = surrogate_targets(c->sur, molal, M, T, c->stream);
  if (ce == cudaSuccess) ce = surrogate_gradients(c->sur, X, T, M, grad_host, loss_host, c->stream);
  cudaFree(T);
  if (ce != cudaSuccess) return fail(c, -2, "gradients: %s", cudaGetErrorString(ce));
  return (int64_t)surrogate_nparam(c->sur);
}

int64_t pfchem_surrogate_params(pfchem_ctx *c, float *host, int set) {
  if (!c) return -1;
  cudaSetDevice(c->device);
  int e = need_surrogate(c, 1);
  if (e) return e;
  if (host) {
    cudaError_t ce = set ? surrogate_set_params(c->sur, host) : surrogate_get_params(c->sur, host);
    if (ce != cudaSuccess) return fail(c, -2, "params: %s", cudaGetErrorString(ce));
    if (set) surrogate_mark_trained(c->sur, true);
  }
  return (int64_t)surrogate_nparam(c->sur);
}

int pfchem_surrogate_normalization(pfchem_ctx *c, float *fmu, float *fisd, float *tmu, float *tsd, int set) {
  if (!c) return -1;
  cudaSetDevice(c->device);
  int e = need_surrogate(c, 1);
  if (e) return e;
  const int N = c->net.N;
  if (set) {
    surrogate_set_norm(c->sur, fmu, fisd, tmu, tsd);
    std::memcpy(c->norm, fmu, 16 * sizeof(float));
    std::memcpy(c->norm + 16, fisd, 16 * sizeof(float));
    std::memcpy(c->norm + 32, tmu, N * sizeof(float));
    std::memcpy(c->norm + 32 + PFCHEM_MAX_PRI, tsd, N * sizeof(float));
  } else {
    std::memcpy(fmu, c->norm, 16 * sizeof(float));
    std::memcpy(fisd, c->norm + 16, 16 * sizeof(float));
    std::memcpy(tmu, c->norm + 32, N * sizeof(float));
    std::memcpy(tsd, c->norm + 32 + PFCHEM_MAX_PRI, N * sizeof(float));
  }
  return 0;
}

int pfchem_check_specialized(const pfchem_network *net, const pfchem_options *opt, int block_threads, char *log,
                             size_t loglen) {
  pfchem_ctx tmp;
  DevNet n;
  int r = build_devnet(&tmp, net, opt, n);
  if (r) {
    if (log && loglen) snprintf(log, loglen, "%s", tmp.err);
    return r;
  }
  // both shared-memory layouts (augmented and compact), logs concatenated
  std::string all;
  int res = 0;
  for (int compact = 0; compact < 2; ++compact) {
    const std::string src = generate_source(n, block_threads, compact != 0);
    nvrtcProgram prog;
    if (nvrtcCreateProgram(&prog, src.c_str(), "pfchem_gen.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS) return -2;
    const char *opts[] = {"--gpu-architecture=sm_103a", "--std=c++17", "-default-device", "--fmad=true",
                          "--ptxas-options=-v"};
    nvrtcResult rc = nvrtcCompileProgram(prog, 5, opts);
    size_t ls = 0;
    nvrtcGetProgramLogSize(prog, &ls);
    std::string lg(ls, '\0');
    nvrtcGetProgramLog(prog, &lg[0]);
    nvrtcDestroyProgram(&prog);
    all += (compact ? "--- compact layout ---\n" : "--- augmented layout ---\n") + std::string(lg.c_str());
    if (rc != NVRTC_SUCCESS) res = -2;
  }
  if (log && loglen) snprintf(log, loglen, "%s", all.c_str());
  return res;
}

}  // extern "C"
