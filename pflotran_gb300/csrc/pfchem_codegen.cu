// pfchem_codegen.cu -- network-specialized Newton kernels, generated as CUDA
// C++ at pfchem_set_network and compiled for sm_103a with NVRTC.
//
// Why: the solve is FP64-issue bound on GB300 (the FP64 pipe runs at a small
// fraction of the FP32 rate), and the table-driven kernel spends about
// twelve non-FP64 instructions (index arithmetic, table and local-memory
// loads) per FP64 instruction.  A reaction network is fixed for a whole run,
// so the kernel is written out for it: species ids, stoichiometric
// coefficients, charges, ion sizes and log K become literals, per-cell state
// is scalarised into registers, unit coefficients cost no multiply, and the
// N x (N+1) augmented Jacobian [J | F] lives in shared memory at
// compile-time offsets (thread-fastest, conflict-free).
//
// The generated code follows the same per-cell algorithm as
// pfchem_newton.cu (the formulation notes there apply) with two further
// changes:
//  * Gaussian elimination on the augmented system [J | F] (row operations
//    applied to F as they happen) instead of a stored LU plus two triangular
//    solves: the same pivots and operation count, no L storage;
//  * partial pivoting compares |a_ij| / 2^e_i, with 2^e_i the power of two
//    of row i's largest |entry| (implicit scaling rounded to a power of two,
//    evaluated on the integer bit patterns, so pivoting costs no FP64 work).
//    The choice differs from ludcmp's 1/max|a_i| scaling only between
//    candidates within a factor of two of each other.
#include <cuda.h>
#include <cuda_runtime.h>
#include <nvrtc.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "pfchem_device.cuh"

namespace pfchem {

namespace {

std::string lit(double v) {
  char b[64];
  snprintf(b, sizeof b, "%.17g", v);
  std::string s(b);
  if (s.find_first_of(".eE") == std::string::npos) s += ".0";
  if (v < 0 || (v == 0.0 && std::signbit(v))) s = "(" + s + ")";
  return s;
}

std::string I(int v) { return std::to_string(v); }

// dst (+)= nu * y with unit coefficients free of multiplies
void acc(std::ostringstream &o, const std::string &dst, double nu, const std::string &y) {
  if (nu == 1.0) o << "  " << dst << " += " << y << ";\n";
  else if (nu == -1.0) o << "  " << dst << " -= " << y << ";\n";
  else o << "  " << dst << " = fma(" << lit(nu) << ", " << y << ", " << dst << ");\n";
}

std::string times(double nu, const std::string &y) {
  if (nu == 1.0) return y;
  if (nu == -1.0) return "(-" + y + ")";
  return "(" + lit(nu) + " * " + y + ")";
}

struct Gen {
  const DevNet &n;
  int js;  // threads per block (shared-memory stride)
  std::ostringstream o;
  bool compact = false;  // J alone in shared memory, the right-hand side in registers
  Gen(const DevNet &net, int block, bool cmp = false) : n(net), js(block), compact(cmp) {}

  int rs() const { return compact ? n.N : n.N + 1; }  // row stride of the shared-memory system
  std::string J(int i, int k) const { return "Jb[" + I((i * rs() + k) * js) + "]"; }
  std::string E(int i) const { return "Eb[" + I(i * js) + "]"; }
  // log K part of the complex constants: kept in the lane only when activity
  // coefficients change during the solve (NEWTON_ITER); else folded into bc
  std::string bK(int i) const {
    return n.act_freq == PFCHEM_ACT_COEF_FREQUENCY_NEWTON_ITER ? "L.bK[" + I(i) + "]" : "L.bc[" + I(i) + "]";
  }
  bool sorb() const { return n.Nix + n.Nsr > 0; }
  // Mass-action products instead of exponentials: with activity
  // coefficients fixed for the step, C_i = exp(bc_i + sum nu ln a) equals
  // K_i * prod a^nu with K_i = exp(bc_i) computed once per cell, so the
  // Newton iterations need multiplications where the log form needs one exp
  // per complex.  Used when every stoichiometric coefficient is an integer
  // in [-4, 4].
  static bool small_int(double v) { return v == std::floor(v) && std::fabs(v) <= 4.0 && v != 0.0; }
  bool prod_cplx() const {
    if (n.act_freq == PFCHEM_ACT_COEF_FREQUENCY_NEWTON_ITER) return false;
    for (int i = 0; i < n.Nc; ++i)
      for (int k = 0; k < n.cn[i]; ++k)
        if (!small_int(n.cnu[i][k])) return false;
    return true;
  }
  // surface complexes of closed-form sites (no free-site inner Newton)
  bool prod_srf(int r) const {
    if (n.srflag[r]) return false;
    for (int q = 0; q < n.srn[r]; ++q) {
      const int k = n.src[r][q];
      for (int l = 0; l < n.sn[k]; ++l)
        if (!small_int(n.snu[k][l])) return false;
    }
    return true;
  }
  bool prod_mnrl() const {
    if (n.act_freq == PFCHEM_ACT_COEF_FREQUENCY_NEWTON_ITER) return false;
    for (int m = 0; m < n.Nm; ++m)
      for (int k = 0; k < n.mn[m]; ++k)
        if (!small_int(n.mnu[m][k])) return false;
    return true;
  }
  bool prod_any() const {
    if (prod_cplx() && n.Nc > 0) return true;
    if (prod_mnrl() && n.Nm > 0) return true;
    for (int r = 0; r < n.Nsr; ++r)
      if (prod_srf(r)) return true;
    return false;
  }
  // product of a^nu over the species of a reaction as a C expression
  std::string prod_expr(const std::string &K, int cnt, const int8_t *ids, const double *nus) const {
    std::string e = K;
    for (int k = 0; k < cnt; ++k) {
      const int j = ids[k];
      const int v = (int)nus[k];
      const std::string b = v > 0 ? "a" + I(j) : "ra" + I(j);
      for (int t = 0; t < std::abs(v); ++t) e += " * " + b;
    }
    return e;
  }
  bool act() const { return n.act_freq != PFCHEM_ACT_COEF_FREQUENCY_OFF; }
  // rate prefactors: flat prefactor index of (mineral, prefactor), and the
  // aqueous complexes some prefactor names (their log K term and activity
  // coefficient are kept per cell)
  int npf_total() const {
    int t = 0;
    for (int m = 0; m < n.Nm; ++m) t += n.mpn[m];
    return t;
  }
  int pf_index(int mm, int p) const {
    int t = 0;
    for (int m = 0; m < mm; ++m) t += n.mpn[m];
    return t + p;
  }
  std::vector<int> pf_complexes() const {
    std::vector<int> v;
    for (int m = 0; m < n.Nm; ++m)
      for (int p = 0; p < n.mpn[m]; ++p)
        for (int q = 0; q < n.mps[m][p]; ++q) {
          const int id = n.mpid[m][p][q];
          if (id < 0 && std::find(v.begin(), v.end(), -id - 1) == v.end()) v.push_back(-id - 1);
        }
    return v;
  }
  int pfc_slot(int i) const {
    const auto v = pf_complexes();
    return (int)(std::find(v.begin(), v.end(), i) - v.begin());
  }
  bool need_bk() const { return n.act_freq == PFCHEM_ACT_COEF_FREQUENCY_NEWTON_ITER; }
  // log K term of complex i (for a prefactor's ln activity)
  std::string pfK(int i) const { return need_bk() ? "L.bK[" + I(i) + "]" : "L.pK[" + I(pfc_slot(i)) + "]"; }
  // activity coefficient of complex i
  std::string pfg(int i) const {
    return need_bk() ? "exp(L.bK[" + I(i) + "] - L.bc[" + I(i) + "])" : "L.pg[" + I(pfc_slot(i)) + "]";
  }
  // ln activity of prefactor species `id` (>= 0 primary, < 0 complex)
  std::string pf_lnact(int id) const {
    if (id >= 0) return "la" + I(id);
    const int i = -id - 1;
    std::string e = "(" + pfK(i);
    for (int k = 0; k < n.cn[i]; ++k) {
      const double nu = n.cnu[i][k];
      e += " + " + (nu == 1.0 ? std::string("") : lit(nu) + " * ") + "la" + I(n.cid[i][k]);
    }
    return e + ")";
  }
  // exact_jacobian_after: the Jacobian's exact terms are selected at run time
  bool rescue() const { return n.exact_after > 0 && !n.jac_exact; }
  // the exact-Jacobian condition as a C expression ("exact" at run time)
  std::string EX() const { return n.jac_exact ? "true" : (rescue() ? "exact" : "false"); }
  bool any_h2o() const {
    for (int i = 0; i < n.Nc; ++i)
      if (n.ch2o[i] != 0.0) return true;
    for (int i = 0; i < n.Nm; ++i)
      if (n.mh2o[i] != 0.0) return true;
    for (int i = 0; i < n.Nsc; ++i)
      if (n.sh2o[i] != 0.0) return true;
    return false;
  }
  bool need_tk() const {
    if (!n.isothermal) return true;
    for (int k = 0; k < n.Nm; ++k) {
      if (n.mEa[k] > 0.0) return true;
      for (int p = 0; p < n.mpn[k]; ++p)
        if (n.mpEa[k][p] > 0.0) return true;
    }
    return false;
  }
  bool need_rho() const {
    for (int r = 0; r < n.Nsr; ++r)
      if (n.srtype[r] == PFCHEM_ROCK_SURFACE) return true;
    return false;
  }

  void header() {
    o << "typedef long long int64_t;\ntypedef int int32_t;\n";
    o << "struct CellArgs { " PFCHEM_STR(PFCHEM_CELLARGS_FIELDS) " };\n";
    o << "struct Scratch { " PFCHEM_STR(PFCHEM_SCRATCH_FIELDS) " };\n";
    o << "__device__ __forceinline__ unsigned long long pf_now() { unsigned long long t; "
         "asm volatile(\"mov.u64 %0, %%globaltimer;\" : \"=l\"(t)); return t; }\n";
    o << "#define NP " << n.N << "\n#define NC " << (n.Nc > 0 ? n.Nc : 1) << "\n#define NM "
      << (n.Nm > 0 ? n.Nm : 1) << "\n#define NIX " << (n.Nix > 0 ? n.Nix : 1) << "\n#define NSR "
      << (n.Nsr > 0 ? n.Nsr : 1) << "\n#define NSC " << (n.Nsc > 0 ? n.Nsc : 1) << "\n#define JS " << js << "\n"
      << "#define NEED_BK " << (n.act_freq == PFCHEM_ACT_COEF_FREQUENCY_NEWTON_ITER ? 1 : 0) << "\n"
      << "#define NPF " << std::max(1, npf_total()) << "\n#define NPC " << std::max(1, (int)pf_complexes().size())
      << "\n";
    o << R"(
struct Lane {
  double m[NP], lm[NP], lg[NP], g[NP], fx[NP];
  double bc[NC];
#if NEED_BK
  double bK[NC];
#endif
  double bm[NM], rk[NM], vf[NM], ar[NM], rate[NM];
  double pk[NPF], pK[NPC], pg[NPC];
  double bs[NSC];
  double ixr[NIX], srf[NSR];
  double P[NP], Sg[NP], F[NP], Sc[NP];
  double acc, psv_den, jac_aq, vol, v_t, den_L, dtc, por, rho_s, lnaw, tk, Icell, rplain, Iacc, Csum;
  int iter;
  bool alt_pending, alt_used, act_fail;
};
__device__ __forceinline__ double sgn1(double x) { return signbit(x) ? -1.0 : 1.0; }
__device__ __forceinline__ long long absbits(double x) { return __double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFLL; }
// one out-of-line copy of each transcendental keeps the kernel inside the
// instruction cache
__device__ __noinline__ double xexp(double x) { return exp(x); }
__device__ __noinline__ double xlog(double x) { return log(x); }
)";
  }

  // LAG activity coefficients at ionic strength `Iv` (reaction.F90:3992-4051);
  // the complex constants are kbase[i] - ln gamma_i (kbase: the log K terms,
  // by default the lane's own)
  void activity(const char *Iv, const char *kbase = nullptr) {
    o << "  {\n  const double sI = sqrt(" << Iv << ");\n";
    bool needg[PFCHEM_MAX_PRI] = {};
    for (int r = 0; r < n.Nix; ++r)
      for (int k = 0; k < n.xn[r]; ++k) needg[n.xid[r][k]] = true;
    if (prod_any())
      for (int j = 0; j < n.N; ++j) needg[j] = true;
    for (int m = 0; m < n.Nm; ++m)
      for (int p = 0; p < n.mpn[m]; ++p)
        for (int q = 0; q < n.mps[m][p]; ++q)
          if (n.mpid[m][p][q] >= 0) needg[n.mpid[m][p][q]] = true;
    for (int j = 0; j < n.N; ++j) {
      if (n.Z2p[j] > 1e-20) {
        o << "  L.lg[" << j << "] = (" << lit(-n.Z2p[j] * n.A) << " * sI / (1.0 + " << lit(n.ap[j] * n.B)
          << " * sI) + " << lit(n.Bdot) << " * " << Iv << ") * " << lit(kLOG_TO_LN) << ";\n";
        if (needg[j]) o << "  L.g[" << j << "] = exp(L.lg[" << j << "]);\n";
      } else {
        o << "  L.lg[" << j << "] = 0.0;\n";
        if (needg[j]) o << "  L.g[" << j << "] = 1.0;\n";
      }
    }
    for (int i = 0; i < n.Nc; ++i) {
      const std::string kb = kbase ? std::string(kbase) + "[" + I(i) + "]" : bK(i);
      if (n.cZ2[i] > 1e-20)
        o << "  L.bc[" << i << "] = " << kb << " - (" << lit(-n.cZ2[i] * n.A) << " * sI / (1.0 + "
          << lit(n.ca[i] * n.B) << " * sI) + " << lit(n.Bdot) << " * " << Iv << ") * " << lit(kLOG_TO_LN) << ";\n";
      else
        o << "  L.bc[" << i << "] = " << kb << ";\n";
    }
    o << "  }\n";
  }

  // ACT_COEF_ALGORITHM_NEWTON at step start (reaction.F90:3846-3990): the
  // ionic strength iterated to a 1e-6 relative change (at most 50 passes)
  // with the primaries' ln activities held at their entry values (the
  // coefficients at the carried ionic strength: the step's entry state at the
  // library's boundary) and the complexes recomputed at every pass.
  void activity_newton() {
    o << "  { // NEWTON activity algorithm\n  double lk[NC];\n";
    for (int i = 0; i < n.Nc; ++i) o << "  lk[" << i << "] = L.bc[" << i << "];\n";
    activity("L.Icell", "lk");
    for (int j = 0; j < n.N; ++j) o << "  const double lae" << j << " = L.lm[" << j << "] + L.lg[" << j << "];\n";
    o << "  double sc[NC];\n  for (int i = 0; i < NC; ++i) sc[i] = 0.0;\n";
    o << "  double fpri = 0.0;\n";
    for (int j = 0; j < n.N; ++j)
      if (n.Z2p[j] > 0) o << "  fpri = fpri + L.m[" << j << "] * " << lit(n.Z2p[j]) << ";\n";
    o << "  double II = 0.0; int it = 0;\n  for (;;) {\n";
    o << "    if (++it > 50) { L.act_fail = true; break; }\n    double I;\n";
    o << "    if (it == 1) { I = L.Icell; } else {\n    I = fpri;\n";
    for (int i = 0; i < n.Nc; ++i)
      if (n.cZ2[i] > 0) o << "    I = I + sc[" << i << "] * " << lit(n.cZ2[i]) << ";\n";
    o << "    I = 0.5 * I; }\n    const double f = I;\n    if (fabs(I - II) < 1e-6 * I) break;\n";
    if (n.Nc > 0) {
      o << "    { const double sI = sqrt(I); double didi = 0.0;\n";
      for (int i = 0; i < n.Nc; ++i) {
        if (!(n.cZ2[i] > 0)) continue;
        o << "    { const double t = 1.0 + " << lit(n.B * n.ca[i]) << " * sI;\n";
        o << "      double sum = " << lit(0.5 * n.A * n.cZ2[i]) << " / (sI * t * t) - " << lit(n.Bdot) << ";\n";
        for (int k = 0; k < n.cn[i]; ++k) {
          const int j = n.cid[i][k];
          if (!(n.Z2p[j] > 0)) continue;
          o << "      { const double tj = 1.0 + " << lit(n.B * n.ap[j]) << " * sI; sum = sum + " << lit(n.cnu[i][k])
            << " * (" << lit(-0.5 * n.A * n.Z2p[j]) << " / (sI * tj * tj) + " << lit(n.Bdot) << "); }\n";
        }
        o << "      didi = didi + " << lit(0.5 * n.cZ2[i]) << " * (sc[" << i << "] * " << lit(kLOG_TO_LN) << " * sum); }\n";
      }
      o << "    const double den = 1.0 - didi;\n    II = fabs(den) > 0.0 ? (f - I * didi) / den : f; }\n";
    } else {
      o << "    II = f;\n";
    }
    activity("II", "lk");
    for (int i = 0; i < n.Nc; ++i) {
      o << "    { double s = L.bc[" << i << "];\n";
      for (int k = 0; k < n.cn[i]; ++k) acc(o, "  s", n.cnu[i][k], "lae" + I(n.cid[i][k]));
      o << "      sc[" << i << "] = exp(s); }\n";
    }
    o << "  }\n  }\n";
  }

  std::string logK(double iso, const double *coef) {
    if (n.isothermal) return lit(-iso * kLOG_TO_LN);
    return "(-(" + lit(coef[0]) + " * lntk + " + lit(coef[1]) + " + " + lit(coef[2]) + " * L.tk + " + lit(coef[3]) +
           " * itk + " + lit(coef[4]) + " * itk2) * " + lit(kLOG_TO_LN) + ")";
  }

  void setup() {
    o << "__device__ __forceinline__ void setup(Lane &L, const CellArgs &a, long long cell, double inv_dt) {\n";
    o << "  const long long nc = a.ncells;\n";
    o << "  const double por = a.por[cell], sat = a.sat[cell], vol = a.vol[cell], den = a.den[cell];\n";
    o << "  L.por = por; L.vol = vol; L.dtc = a.dt;\n";
    if (need_rho()) o << "  L.rho_s = a.rho_s[cell];\n";
    o << "  L.acc = " << (n.accum_mode == PFCHEM_ACCUM_DT_CONSISTENT ? "inv_dt" : "1.0") << ";\n";
    o << "  const double psv = por * sat * 1000.0 * vol;\n";
    o << "  L.den_L = den * 1e-3; L.psv_den = psv * L.den_L; L.jac_aq = psv * inv_dt * L.den_L; L.v_t = vol * inv_dt;\n";
    o << "  L.lnaw = " << (any_h2o() ? "(a.lnaw ? a.lnaw[cell] : 0.0)" : "0.0") << ";\n";
    for (int j = 0; j < n.N; ++j) {
      o << "  { const double t = a.total[" << j << " * a.total_stride_comp + cell * a.total_stride_cell];\n";
      o << "    double f = psv * t;\n";
      if (sorb()) o << "    f = f + a.sorb[" << j << " * nc + cell] * vol;\n";
      o << "    L.fx[" << j << "] = L.acc * f;\n";
      o << "    const double m = a.pri_molal[" << j << " * nc + cell]; L.m[" << j << "] = m; L.lm[" << j
        << "] = xlog(m); }\n";
    }
    if (need_tk()) {
      o << "  L.tk = a.temp[cell] + 273.15;\n";
      if (!n.isothermal) o << "  const double lntk = log(L.tk), itk = 1.0 / L.tk, itk2 = itk * itk;\n";
    }
    for (int i = 0; i < n.Nc; ++i) {
      o << "  " << bK(i) << " = " << logK(n.clogK[i], n.ccoef[i]);
      if (n.ch2o[i] != 0.0) o << " + " << lit(n.ch2o[i]) << " * L.lnaw";
      o << ";\n";
    }
    for (int k = 0; k < n.Nm; ++k) {
      o << "  L.bm[" << k << "] = " << logK(n.mlogK[k], n.mcoef[k]);
      if (n.mh2o[k] != 0.0) o << " + " << lit(n.mh2o[k]) << " * L.lnaw";
      o << ";\n";
      if (n.mEa[k] > 0.0)
        o << "  L.rk[" << k << "] = " << lit(n.mk[k]) << " * exp(" << lit(n.mEa[k] / kIDEAL_GAS_CONSTANT)
          << " * (" << lit(1.0 / (25.0 + 273.15)) << " - 1.0 / L.tk));\n";
      else
        o << "  L.rk[" << k << "] = " << lit(n.mk[k]) << ";\n";
      o << "  L.vf[" << k << "] = a.vf[" << k << " * nc + cell]; L.ar[" << k << "] = a.area[" << k
        << " * nc + cell]; L.rate[" << k << "] = 0.0;\n";
      for (int p = 0; p < n.mpn[k]; ++p) {
        // a prefactor's rate constant with its own Arrhenius factor (reaction_mineral.F90:771-778)
        if (n.mpEa[k][p] > 0.0)
          o << "  L.pk[" << pf_index(k, p) << "] = " << lit(n.mpk[k][p]) << " * exp(" << lit(n.mpEa[k][p] / kIDEAL_GAS_CONSTANT)
            << " * (" << lit(1.0 / (25.0 + 273.15)) << " - 1.0 / L.tk));\n";
        else
          o << "  L.pk[" << pf_index(k, p) << "] = " << lit(n.mpk[k][p]) << ";\n";
      }
    }
    if (!need_bk())
      for (int i : pf_complexes()) o << "  L.pK[" << pfc_slot(i) << "] = L.bc[" << i << "];\n";
    for (int k = 0; k < n.Nsc; ++k) {
      o << "  L.bs[" << k << "] = " << logK(n.slogK[k], n.scoef[k]);
      if (n.sh2o[k] != 0.0) o << " + " << lit(n.sh2o[k]) << " * L.lnaw";
      o << ";\n";
    }
    for (int r = 0; r < n.Nix; ++r) o << "  L.ixr[" << r << "] = a.ixref[" << r << " * nc + cell];\n";
    for (int r = 0; r < n.Nsr; ++r) o << "  L.srf[" << r << "] = a.srfree[" << r << " * nc + cell];\n";
    o << "  L.Icell = a.ionic[cell]; L.act_fail = false;\n";
    if (act()) {
      if (n.act_newton) activity_newton();
      else activity("L.Icell");
    } else {
      for (int j = 0; j < n.N; ++j) o << "  L.lg[" << j << "] = 0.0; L.g[" << j << "] = 1.0;\n";
      for (int i = 0; i < n.Nc; ++i) o << "  L.bc[" << i << "] = " << bK(i) << ";\n";
    }
    if (!need_bk())
      for (int i : pf_complexes())
        o << "  L.pg[" << pfc_slot(i) << "] = exp(L.pK[" << pfc_slot(i) << "] - L.bc[" << i << "]);\n";
    // product-form constants: exp of the log constants, once per cell
    if (prod_mnrl())
      for (int k = 0; k < n.Nm; ++k) o << "  L.bm[" << k << "] = xexp(L.bm[" << k << "]);\n";
    if (prod_cplx())
      for (int i = 0; i < n.Nc; ++i) o << "  L.bc[" << i << "] = xexp(L.bc[" << i << "]);\n";
    for (int r = 0; r < n.Nsr; ++r)
      if (prod_srf(r))
        for (int q = 0; q < n.srn[r]; ++q)
          o << "  L.bs[" << (int)n.src[r][q] << "] = xexp(L.bs[" << (int)n.src[r][q] << "]);\n";
    o << "  L.Iacc = 0.0; L.Csum = 0.0;\n";
    o << "  L.iter = 0; L.alt_pending = false; L.alt_used = false;\n}\n";
  }

  // Residual (and with jac the Jacobian d/dln m into [J | .]) at L.m
  void evaluate(bool jac) {
    const int N = n.N;
    o << "__device__ __forceinline__ int evaluate_" << (jac ? "jac" : "res") << "(Lane &L, double *Jb"
      << (jac && rescue() ? ", bool exact" : "") << ") {\n";
    o << "  int status = 0;\n";
    if (prod_any()) {
      bool neg[PFCHEM_MAX_PRI] = {};
      if (prod_cplx())
        for (int i = 0; i < n.Nc; ++i)
          for (int k = 0; k < n.cn[i]; ++k)
            if (n.cnu[i][k] < 0) neg[n.cid[i][k]] = true;
      for (int r = 0; r < n.Nsr; ++r)
        if (prod_srf(r))
          for (int q = 0; q < n.srn[r]; ++q) {
            const int k = n.src[r][q];
            for (int l = 0; l < n.sn[k]; ++l)
              if (n.snu[k][l] < 0) neg[n.sid[k][l]] = true;
          }
      if (prod_mnrl())
        for (int m = 0; m < n.Nm; ++m)
          for (int k = 0; k < n.mn[m]; ++k)
            if (n.mnu[m][k] < 0) neg[n.mid[m][k]] = true;
      for (int j = 0; j < N; ++j) {
        o << "  const double a" << j << " = L.m[" << j << "]" << (act() ? " * L.g[" + I(j) + "]" : "") << ";\n";
        if (neg[j]) o << "  const double ra" << j << " = 1.0 / a" << j << ";\n";
      }
    }
    for (int j = 0; j < N; ++j) {
      if (act()) o << "  const double la" << j << " = L.lm[" << j << "] + L.lg[" << j << "];\n";
      else o << "  const double la" << j << " = L.lm[" << j << "];\n";
      o << "  L.P[" << j << "] = L.m[" << j << "]; double aP" << j << " = L.m[" << j << "];\n";
      if (sorb()) o << "  L.Sg[" << j << "] = 0.0; double aS" << j << " = 0.0;\n";
    }
    // Jacobian entries touched by some complex: accumulated in registers and
    // stored once (the same additions in the same complex order as a
    // read-modify-write per contribution); the others are stored here
    std::vector<std::vector<int>> contrib((size_t)N * N);
    for (int i = 0; i < n.Nc; ++i)
      for (int k = 0; k < n.cn[i]; ++k)
        for (int l = 0; l < n.cn[i]; ++l) contrib[(size_t)n.cid[i][l] * N + n.cid[i][k]].push_back(i);
    if (jac)
      for (int i = 0; i < N; ++i)
        for (int k = 0; k < N; ++k)
          if (contrib[(size_t)i * N + k].empty())
            o << "  " << J(i, k) << " = " << (i == k ? "L.m[" + I(i) + "] * L.jac_aq" : "0.0") << ";\n";
    // aqueous complexes (RTotal)
    // secondary-species part of the ionic strength (the primary part is added
    // where the ionic strength is used, at the then current molalities)
    o << "  double Iacc = 0.0, Csum = 0.0;\n";
    if (jac && n.Nc > 0) {
      o << "  double cj0";
      for (int i = 1; i < n.Nc; ++i) o << ", cj" << i;
      o << ";\n";
    }
    for (int i = 0; i < n.Nc; ++i) {
      if (prod_cplx()) {
        int8_t ids[PFCHEM_MAX_NNZ];
        for (int k = 0; k < n.cn[i]; ++k) ids[k] = n.cid[i][k];
        o << "  { const double c = " << prod_expr("L.bc[" + I(i) + "]", n.cn[i], ids, n.cnu[i]) << ";\n";
      } else {
        o << "  { double s = L.bc[" << i << "];\n";
        for (int k = 0; k < n.cn[i]; ++k) {
          const double nu = n.cnu[i][k];
          const std::string la = "la" + I(n.cid[i][k]);
          acc(o, "s", nu, la);
        }
        o << "    const double c = xexp(s);\n";
      }
      if (n.cZ2[i] > 0) o << "    Iacc = fma(" << lit(n.cZ2[i]) << ", c, Iacc);\n";
      if (n.use_h2o) o << "    Csum += c;\n";
      for (int k = 0; k < n.cn[i]; ++k) {
        const int j = n.cid[i][k];
        acc(o, "L.P[" + I(j) + "]", n.cnu[i][k], "c");
        acc(o, "aP" + I(j), std::fabs(n.cnu[i][k]), "c");
      }
      if (jac) o << "    cj" << i << " = c * L.jac_aq;\n";
      o << "  }\n";
    }
    o << "  L.Iacc = 0.5 * Iacc; L.Csum = Csum;\n";
    if (jac) {
      for (int l = 0; l < N; ++l)
        for (int k = 0; k < N; ++k) {
          const auto &cs = contrib[(size_t)l * N + k];
          if (cs.empty()) continue;
          o << "  { double v = " << (l == k ? "L.m[" + I(l) + "] * L.jac_aq" : "0.0") << ";\n";
          for (int i : cs) {
            double nuk = 0.0, nul = 0.0;
            for (int q = 0; q < n.cn[i]; ++q) {
              if (n.cid[i][q] == k) nuk = n.cnu[i][q];
              if (n.cid[i][q] == l) nul = n.cnu[i][q];
            }
            o << "    { const double t = " << times(nuk, "cj" + I(i)) << ";";
            acc(o, "v", nul, "t");
            o << "    }\n";
          }
          o << "    " << J(l, k) << " = v; }\n";
        }
    }
    // ion exchange (RTotalSorbEqIonx)
    for (int r = 0; r < n.Nix; ++r) {
      const int nz = n.xn[r];
      const int i1 = n.xid[r][0];
      const double zref = n.Zp[i1];
      o << "  { // ion exchange " << r << "\n";
      if (n.xsurf[r] > 0) o << "  const double omega = fmax(" << lit(n.xCEC[r]) << " * L.vf[" << (n.xsurf[r] - 1) << "], 1e-40);\n";
      else o << "  const double omega = " << lit(n.xCEC[r]) << ";\n";
      for (int k = 0; k < nz; ++k) o << "  double X" << k << ";\n";
      if (n.xzflag[r]) {
        o << "  const double ref = " << lit(n.xk[r][0]) << " * (L.m[" << i1 << "] * L.g[" << i1 << "]);\n";
        o << "  double KD = (" << lit(zref) << " * L.ixr[" << r << "] / omega) / ref;\n";
        o << "  bool one_more = false; int it = 0;\n  for (;;) {\n";
        o << "    if (++it > 20000) { status = " << PFCHEM_CELL_INNER_MAXITER << "; break; }\n";
        o << "    X0 = KD * ref; double tot = X0, dsum = 0.0;\n";
        for (int k = 1; k < nz; ++k) {
          const int j = n.xid[r][k];
          std::string p;
          switch (n.xpow[r][k]) {
            case kPowOne: p = "KD"; break;
            case kPowTwo: p = "(KD * KD)"; break;
            case kPowHalf: p = "sqrt(KD)"; break;
            default: p = "pow(KD, " + lit(n.xzr[r][k]) + ")"; break;
          }
          o << "    X" << k << " = " << lit(n.xk[r][k]) << " * (L.m[" << j << "] * L.g[" << j << "]) * " << p << ";\n";
          o << "    tot += X" << k << ";\n";
          acc(o, "  dsum", n.xzr[r][k], "X" + I(k));
        }
        o << "    if (one_more) break;\n";
        // (1 - tot) / (dsum / KD + ref) with one division: the same Newton
        // step on KD (reaction.F90:4379-4411), converged to the same 1e-12
        o << "    const double delta = (1.0 - tot) * KD / fma(ref, KD, dsum);\n";
        o << "    KD = fmax(KD + delta, 1e-40);\n    if (fabs(delta) < 1e-12 * KD) one_more = true;\n  }\n";
        o << "  L.ixr[" << r << "] = X0 * omega * " << lit(1.0 / zref) << ";\n";
      } else {
        o << "  double s = 0.0;\n";
        for (int k = 0; k < nz; ++k) {
          const int j = n.xid[r][k];
          o << "  X" << k << " = (L.m[" << j << "] * L.g[" << j << "]) * " << lit(n.xk[r][k]) << "; s += X" << k << ";\n";
        }
        o << "  { const double is = 1.0 / s;\n";
        for (int k = 0; k < nz; ++k) o << "  X" << k << " *= is;\n";
        o << "  }\n";
      }
      o << "  double sumZX = 0.0;\n";
      for (int k = 0; k < nz; ++k) acc(o, "sumZX", n.Zp[n.xid[r][k]], "X" + I(k));
      o << "  const double isz = 1.0 / sumZX;\n";
      for (int k = 0; k < nz; ++k) {
        const int i = n.xid[r][k];
        o << "  { const double t1 = X" << k << " * omega * " << lit(1.0 / n.Zp[i]) << ";\n";
        o << "    L.Sg[" << i << "] += t1; aS" << i << " += fabs(t1);\n";
        if (jac) {
          o << "    const double t2 = " << lit(n.Zp[i]) << " * isz * t1 * L.v_t;\n";
          for (int q = 0; q < nz; ++q) {
            const int j = n.xid[r][q];
            if (q == k) o << "    " << J(i, j) << " += t1 * L.v_t - t2 * X" << q << ";\n";
            else o << "    " << J(i, j) << " -= t2 * X" << q << ";\n";
          }
        }
        o << "  }\n";
      }
      o << "  }\n";
    }
    // surface complexation (RTotalSorbEqSurfCplx1, immobile sites)
    for (int r = 0; r < n.Nsr; ++r) {
      const int ncx = n.srn[r];
      o << "  { // surface complexation " << r << "\n";
      if (n.srtype[r] == PFCHEM_MINERAL_SURFACE)
        o << "  const double site = " << lit(n.srdens[r]) << " * L.vf[" << (n.srsurf[r] - 1) << "];\n";
      else if (n.srtype[r] == PFCHEM_ROCK_SURFACE)
        o << "  const double site = " << lit(n.srdens[r]) << " * L.rho_s * (1.0 - L.por);\n";
      else
        o << "  const double site = " << lit(n.srdens[r]) << ";\n";
      o << "  if (site >= 1e-40) {\n";
      for (int q = 0; q < ncx; ++q) o << "  double S" << q << ";\n";
      o << "  double free = L.srf[" << r << "];\n";
      auto lq = [&](int q, bool with_free) {
        const int k = n.src[r][q];
        std::string s = "L.bs[" + I(k) + "]";
        std::ostringstream t;
        t << "  { double s = " << s << ";\n";
        o << t.str();
        if (with_free) acc(o, "s", n.sfs[k], "lf");
        for (int l = 0; l < n.sn[k]; ++l) acc(o, "s", n.snu[k][l], "la" + I(n.sid[k][l]));
      };
      if (prod_srf(r)) {
        o << "  double sumE = 0.0;\n";
        for (int q = 0; q < ncx; ++q) {
          const int k = n.src[r][q];
          o << "  S" << q << " = " << prod_expr("L.bs[" + I(k) + "]", n.sn[k], n.sid[k], n.snu[k])
            << "; sumE += S" << q << ";\n";
        }
        o << "  free = site / (1.0 + sumE);\n";
        for (int q = 0; q < ncx; ++q) o << "  S" << q << " *= free;\n";
      } else if (!n.srflag[r]) {
        o << "  double sumE = 0.0;\n";
        for (int q = 0; q < ncx; ++q) {
          lq(q, false);
          o << "    S" << q << " = xexp(s); sumE += S" << q << "; }\n";
        }
        o << "  free = site / (1.0 + sumE);\n";
        for (int q = 0; q < ncx; ++q) o << "  S" << q << " *= free;\n";
      } else {
        o << "  bool one_more = false; double damping = 1.0; int it = 0;\n  for (;;) {\n";
        o << "    if (++it > 2000) { status = " << PFCHEM_CELL_INNER_MAXITER << "; break; }\n";
        o << "    const double lf = log(free); double total = free, d = 1.0;\n";
        for (int q = 0; q < ncx; ++q) {
          const int k = n.src[r][q];
          lq(q, true);
          o << "    S" << q << " = xexp(s); }\n";
          acc(o, "  total", n.sfs[k], "S" + I(q));
          o << "    d += " << times(n.sfs[k], "S" + I(q)) << " / free;\n";
        }
        o << "    if (one_more) break;\n    const double dfree = (site - total) / d;\n";
        o << "    if (it > 1000) damping = 0.5;\n    free = free + damping * dfree;\n";
        o << "    if (fabs(dfree) < 1e-12 * fabs(free)) one_more = true;\n  }\n";
      }
      o << "  L.srf[" << r << "] = free;\n";
      // components of any complex on the site (those the free site depends on)
      std::vector<int> site_comps;
      for (int q = 0; q < ncx; ++q) {
        const int k = n.src[r][q];
        for (int l = 0; l < n.sn[k]; ++l)
          if (std::find(site_comps.begin(), site_comps.end(), (int)n.sid[k][l]) == site_comps.end())
            site_comps.push_back(n.sid[k][l]);
      }
      o << "  double den = 0.0;\n";
      if (jac) {
        for (int j = 0; j < N; ++j) o << "  double dSx" << j << " = 0.0;\n";
      }
      for (int q = 0; q < ncx; ++q) {
        const int k = n.src[r][q];
        if (jac)
          for (int l = 0; l < n.sn[k]; ++l)
            acc(o, "dSx" + I(n.sid[k][l]), n.snu[k][l] * n.sfs[k], "S" + I(q));
        acc(o, "den", n.sfs[k] * n.sfs[k], "S" + I(q));
      }
      o << "  const double iden = -1.0 / (den / free + 1.0);\n  const double ifree = 1.0 / free;\n";
      for (int q = 0; q < ncx; ++q) {
        const int k = n.src[r][q];
        for (int l = 0; l < n.sn[k]; ++l) {
          const int i = n.sid[k][l];
          o << "  { const double v = " << times(n.snu[k][l], "S" + I(q)) << "; L.Sg[" << i << "] += v; aS" << i
            << " += fabs(v); }\n";
        }
        if (jac) {
          o << "  { const double nuS = " << times(n.sfs[k], "S" + I(q)) << " * ifree;\n";
          // terms of the complex's own components (RReact's Jacobian) ...
          for (int l = 0; l < n.sn[k]; ++l) {
            const int j = n.sid[k][l];
            o << "    { const double t = (" << times(n.snu[k][l], "S" + I(q)) << " + nuS * dSx" << j
              << " * iden) * L.v_t;\n";
            for (int p = 0; p < n.sn[k]; ++p) acc(o, "  " + J(n.sid[k][p], j), n.snu[k][p], "t");
            o << "    }\n";
          }
          // ... and, exact, the free site's coupling to the site's other components
          std::vector<int> others;
          for (int j : site_comps) {
            bool own = false;
            for (int l = 0; l < n.sn[k]; ++l) own |= n.sid[k][l] == j;
            if (!own) others.push_back(j);
          }
          if (!others.empty() && EX() != "false") {
            o << "    if (" << EX() << ") {\n";
            for (int j : others) {
              o << "    { const double t = (nuS * dSx" << j << " * iden) * L.v_t;\n";
              for (int p = 0; p < n.sn[k]; ++p) acc(o, "  " + J(n.sid[k][p], j), n.snu[k][p], "t");
              o << "    }\n";
            }
            o << "    }\n";
          }
          o << "  }\n";
        }
      }
      o << "  }\n  }\n";
    }
    // accumulation residual and magnitude scale
    for (int j = 0; j < N; ++j) {
      if (sorb()) {
        o << "  L.F[" << j << "] = L.acc * (L.psv_den * L.P[" << j << "] + L.vol * L.Sg[" << j << "]) - L.fx[" << j << "];\n";
        o << "  L.Sc[" << j << "] = L.acc * (L.psv_den * aP" << j << " + L.vol * aS" << j << ") + fabs(L.fx[" << j << "]);\n";
      } else {
        o << "  L.F[" << j << "] = L.acc * (L.psv_den * L.P[" << j << "]) - L.fx[" << j << "];\n";
        o << "  L.Sc[" << j << "] = L.acc * (L.psv_den * aP" << j << ") + fabs(L.fx[" << j << "]);\n";
      }
    }
    // kinetic minerals (RKineticMineral)
    for (int mm = 0; mm < n.Nm; ++mm) {
      const int nz = n.mn[mm];
      // the cap of RKineticMineral (QK = 1e3 where ln QK > 6.90776) becomes,
      // in product form, a comparison of QK itself with exp(6.90776)
      const std::string qk_ok = prod_mnrl() ? "(QKp <= " + lit(std::exp(6.90776)) + ")" : "(lnQK <= 6.90776)";
      if (prod_mnrl()) {
        o << "  { // mineral " << mm << "\n  const double QKp = "
          << prod_expr("L.bm[" + I(mm) + "]", nz, n.mid[mm], n.mnu[mm]) << ";\n";
        o << "  const double QK = " << qk_ok << " ? QKp : 1e3;\n";
      } else {
        o << "  { // mineral " << mm << "\n  double lnQK = L.bm[" << mm << "];\n";
        for (int k = 0; k < nz; ++k) acc(o, "lnQK", n.mnu[mm][k], "la" + I(n.mid[mm][k]));
        o << "  const double QK = " << qk_ok << " ? xexp(lnQK) : 1e3;\n";
      }
      double sig = 1.0;
      if (n.has_temkin) sig = n.mtemkin[mm];
      if (n.has_minscale) sig *= n.mscale[mm];
      const bool gen_aff = n.has_temkin || n.has_minscale;
      if (gen_aff) o << "  double aff = 1.0 - pow(QK, " << lit(1.0 / sig) << ");\n";
      else o << "  double aff = 1.0 - QK;\n";
      o << "  const double sign_ = sgn1(aff);\n  L.rate[" << mm << "] = 0.0;\n";
      o << "  bool on = (L.vf[" << mm << "] > 0.0 || sign_ < 0.0);\n";
      if (n.mthr[mm] > 0.0) o << "  if (sign_ < 0.0 && QK < " << lit(n.mthr[mm]) << ") on = false;\n";
      o << "  if (on) {\n";
      if (n.mlim[mm] > 0.0) o << "  aff = aff / (1.0 + (1.0 - aff) * " << lit(1.0 / n.mlim[mm]) << ");\n";
      if (n.mpn[mm] > 0) {
        // rate prefactors (reaction_mineral.F90:743-782): a sum over parallel
        // prefactors of products of Monod terms a^alpha / (1 + atten a^beta)
        o << "  double kr = 0.0;\n";
        for (int p = 0; p < n.mpn[mm]; ++p) {
          o << "  double lp" << p << " = 0.0;\n";
          for (int q = 0; q < n.mps[mm][p]; ++q) {
            const double att = n.mpatt[mm][p][q];
            o << "  double lps" << p << "_" << q << ";\n";
            o << "  { const double lsa = " << pf_lnact(n.mpid[mm][p][q]) << ";\n";
            o << "    const double lnum = " << lit(n.mpa[mm][p][q]) << " * lsa;\n";
            if (att > 0.0)
              o << "    const double lden = xlog(1.0 + xexp(" << lit(std::log(att)) << " + " << lit(n.mpb[mm][p][q])
                << " * lsa));\n";
            else
              o << "    const double lden = 0.0;\n";
            o << "    lp" << p << " = lp" << p << " + lnum; lp" << p << " = lp" << p << " - lden; lps" << p << "_" << q
              << " = lnum - lden; }\n";
          }
          o << "  const double pf" << p << " = xexp(lp" << p << "); kr = kr + pf" << p << " * L.pk["
            << pf_index(mm, p) << "];\n";
        }
      } else {
        o << "  const double kr = L.rk[" << mm << "];\n";
      }
      o << "  const double Imc = -L.ar[" << mm << "]" << (n.has_minscale ? " * " + lit(1.0 / n.mscale[mm]) : "") << ";\n";
      if (n.has_affpow) o << "  const double Im = Imc * sign_ * pow(fabs(aff), " << lit(n.mpow[mm]) << ") * kr;\n";
      else o << "  const double Im = Imc * sign_ * fabs(aff) * kr;\n";
      o << "  L.rate[" << mm << "] = Im;\n  const double ImV = Im * L.vol;\n";
      for (int k = 0; k < nz; ++k) {
        const int i = n.mid[mm][k];
        o << "  { const double v = " << times(n.mnu[mm][k], "ImV") << "; L.F[" << i << "] += v; L.Sc[" << i
          << "] += fabs(v); }\n";
      }
      if (jac) {
        // exact Jacobian: signed affinity, no den/1000 factor, nothing where QK is capped
        const std::string ex = EX();
        if (ex == "true") o << "  if " << qk_ok << " {\n";
        else if (ex != "false") o << "  if (!" << ex << " || " << qk_ok << ") {\n";
        if (n.has_affpow) {
          if (ex == "true") o << "  double dIm_dQK = -ImV * " << lit(n.mpow[mm]) << " / aff;\n";
          else if (ex == "false") o << "  double dIm_dQK = -ImV * " << lit(n.mpow[mm]) << " / fabs(aff);\n";
          else o << "  double dIm_dQK = -ImV * " << lit(n.mpow[mm]) << " / (" << ex << " ? aff : fabs(aff));\n";
        } else o << "  double dIm_dQK = -(Imc * L.vol) * kr;\n";
        if (gen_aff) o << "  dIm_dQK = dIm_dQK * " << lit(1.0 / sig) << " / QK * (1.0 - aff);\n";
        if (ex == "true") o << "  double gq = dIm_dQK * QK;\n";
        else if (ex == "false") o << "  double gq = dIm_dQK * QK * L.den_L;\n";
        else o << "  double gq = dIm_dQK * QK * (" << ex << " ? 1.0 : L.den_L);\n";
        if (n.mlim[mm] > 0.0) {
          o << "  { const double d2 = 1.0 + (1.0 - aff) * " << lit(1.0 / n.mlim[mm]) << ";\n";
          o << "    gq = gq * (1.0 + QK * " << lit(1.0 / n.mlim[mm]) << " / d2) / d2; }\n";
        }
        for (int q = 0; q < nz; ++q) {
          const int j = n.mid[mm][q];
          o << "  { const double t = " << times(n.mnu[mm][q], "gq") << ";\n";
          for (int k = 0; k < nz; ++k) acc(o, "  " + J(n.mid[mm][k], j), n.mnu[mm][k], "t");
          o << "  }\n";
        }
        if (ex != "false") o << "  }\n";
        if (n.mpn[mm] > 0) {
          // derivative through the prefactors (reaction_mineral.F90:897-997)
          // per ln m: a primary's column gets the mineral's stoichiometry times
          // dIm/da * gamma * m; a complex's derivative goes through its
          // components (dC/dln m_j = nu_j C) into the rows of the complex's
          // species as RReact adds it, or (exact) into the mineral's rows
          o << "  { const double dIm_dsum = ImV / kr;\n";
          for (int p = 0; p < n.mpn[mm]; ++p) {
            o << "  const double lpf" << p << " = xlog(pf" << p << ");\n";
            for (int q = 0; q < n.mps[mm][p]; ++q) {
              const int id = n.mpid[mm][p][q];
              const double a_ = n.mpa[mm][p][q], b_ = n.mpb[mm][p][q], att = n.mpatt[mm][p][q];
              const std::string ps = "lps" + I(p) + "_" + I(q);
              o << "  { const double lsa = " << pf_lnact(id) << ";\n";
              o << "    const double gs = " << (id >= 0 ? "L.g[" + I(id) + "]" : pfg(-id - 1)) << ";\n";
              o << "    const double dpp = xexp(lpf" << p << " - " << ps << ");\n";
              o << "    const double num = " << lit(a_) << " * xexp(" << ps << " - lsa);\n";
              if (att > 0.0) {
                o << "    const double lgb = " << lit(b_) << " * lsa;\n";
                o << "    const double den = 1.0 + xexp(" << lit(std::log(att)) << " + lgb);\n";
                o << "    const double dden = -1.0 * xexp(" << ps << ") / den * " << lit(att) << " * " << lit(b_)
                  << " * xexp(lgb - lsa);\n";
              } else {
                o << "    const double dden = 0.0;\n";
              }
              o << "    const double dIm = dIm_dsum * dpp * ((num + dden) * gs) * L.pk[" << pf_index(mm, p) << "];\n";
              if (id >= 0) {
                o << "    { const double t = dIm * L.m[" << id << "];\n";
                for (int k = 0; k < nz; ++k) acc(o, "    " + J(n.mid[mm][k], id), n.mnu[mm][k], "t");
                o << "    }\n";
              } else {
                const int ci = -id - 1;
                o << "    const double Ci = xexp(lsa) / gs;\n";
                for (int jj = 0; jj < n.cn[ci]; ++jj) {
                  const int j = n.cid[ci][jj];
                  o << "    { const double t = " << times(n.cnu[ci][jj], "Ci") << " * dIm;\n";
                  auto mineral_rows = [&]() {
                    for (int k = 0; k < nz; ++k) acc(o, "      " + J(n.mid[mm][k], j), n.mnu[mm][k], "t");
                  };
                  auto complex_rows = [&]() {
                    for (int k = 0; k < n.cn[ci]; ++k) acc(o, "      " + J(n.cid[ci][k], j), n.cnu[ci][k], "t");
                  };
                  if (ex == "true") mineral_rows();
                  else if (ex == "false") complex_rows();
                  else {
                    o << "      if (" << ex << ") {\n";
                    mineral_rows();
                    o << "      } else {\n";
                    complex_rows();
                    o << "      }\n";
                  }
                  o << "    }\n";
                }
              }
              o << "  }\n";
            }
          }
          o << "  }\n";
        }
      }
      o << "  }\n  }\n";
    }
    o << "  return status;\n}\n";
  }

  void converged() {
    o << "__device__ __forceinline__ bool converged(const Lane &L, bool *nonfinite) {\n";
    o << "  bool conv = true, bad = false;\n";
    for (int j = 0; j < n.N; ++j) {
      o << "  { const double f = fabs(L.F[" << j << "]); if (!(f <= 1.7976931348623157e308)) bad = true;\n";
      if (n.resid_kind == PFCHEM_RESIDUAL_RELATIVE)
        o << "    if (!(f < " << lit(n.res_tol) << " * L.Sc[" << j << "])) conv = false; }\n";
      else
        o << "    if (!(f < " << lit(n.res_tol) << ")) conv = false; }\n";
    }
    o << "  *nonfinite = bad; return conv && !bad;\n}\n";
    // residual norm in the units of the convergence test (alternative-guess choice only)
    o << "__device__ __forceinline__ double rnorm(const Lane &L) {\n  double r = 0.0;\n";
    for (int j = 0; j < n.N; ++j) {
      if (n.resid_kind == PFCHEM_RESIDUAL_RELATIVE)
        o << "  r = fmax(r, fabs(L.F[" << j << "]) / L.Sc[" << j << "]);\n";
      else
        o << "  r = fmax(r, fabs(L.F[" << j << "]));\n";
    }
    o << "  return r;\n}\n";
  }

  // Gaussian elimination with power-of-two implicit-scaling pivoting on the
  // augmented [J | F] (column N holds the right-hand side); solution into x.
  void solve() {
    if (compact) {
      // J alone in shared memory: the right-hand side stays in registers
      // (the row loops unrolled under an i > j predicate so every f index is
      // a constant, the pivot column rolled to keep the code small; f[j] and
      // the pivot swap read through unrolled selects), the row exponents are
      // 16-bit.  The same operations in the same order as the augmented form
      // below.
      o << R"(__device__ __forceinline__ bool lu_solve(double *Jb, unsigned short *Eb, double (&f)[NP]) {
#define JA(i, k) Jb[((i) * NP + (k)) * JS]
#pragma unroll 1
  for (int i = 0; i < NP; ++i) {
    long long r = 0;
    for (int k = 0; k < NP; ++k) { const long long v = absbits(JA(i, k)); r = v > r ? v : r; }
    if (r == 0) return false;
    Eb[i * JS] = (unsigned short)((r & 0x7FF0000000000000LL) >> 48);
  }
#pragma unroll 1
  for (int j = 0; j < NP; ++j) {
    int p = j;
    long long best = absbits(JA(j, j)) - ((long long)Eb[j * JS] << 48);
#pragma unroll 1
    for (int i = j + 1; i < NP; ++i) {
      const long long kk = absbits(JA(i, j)) - ((long long)Eb[i * JS] << 48);
      if (kk >= best) { best = kk; p = i; }
    }
    if (p != j) {
#pragma unroll 1
      for (int k = j; k < NP; ++k) { const double t = JA(p, k); JA(p, k) = JA(j, k); JA(j, k) = t; }
      const unsigned short te = Eb[p * JS]; Eb[p * JS] = Eb[j * JS]; Eb[j * JS] = te;
      double fp = f[0], fq = f[0];
#pragma unroll
      for (int q = 1; q < NP; ++q) { if (q == p) fp = f[q]; if (q == j) fq = f[q]; }
#pragma unroll
      for (int q = 0; q < NP; ++q) { if (q == j) f[q] = fp; else if (q == p) f[q] = fq; }
    }
    double piv = JA(j, j);
    if (piv == 0.0) piv = 1e-20;
    const double ip = 1.0 / piv;
    JA(j, j) = ip;
    double fj = f[0];
#pragma unroll
    for (int q = 1; q < NP; ++q) if (q == j) fj = f[q];
#pragma unroll
    for (int i = 1; i < NP; ++i) {
      if (i > j) {
        const double l = JA(i, j) * ip;
#pragma unroll 1
        for (int k = j + 1; k < NP; ++k) JA(i, k) = fma(-l, JA(j, k), JA(i, k));
        f[i] = fma(-l, fj, f[i]);
      }
    }
  }
#pragma unroll
  for (int i = NP - 1; i >= 0; --i) {
    double s = f[i];
#pragma unroll
    for (int k = i + 1; k < NP; ++k) s = fma(-JA(i, k), f[k], s);
    f[i] = s * JA(i, i);
  }
#undef JA
  return true;
}
)";
      return;
    }
    // rolled loops over the shared-memory system keep the code compact; the
    // reciprocal pivots overwrite the diagonal and the solution overwrites
    // the right-hand-side column
    o << R"(__device__ __forceinline__ bool lu_solve(double *Jb, long long *Eb) {
#define JA(i, k) Jb[((i) * (NP + 1) + (k)) * JS]
  for (int i = 0; i < NP; ++i) {
    long long r = 0;
    for (int k = 0; k < NP; ++k) { const long long v = absbits(JA(i, k)); r = v > r ? v : r; }
    if (r == 0) return false;
    Eb[i * JS] = r & 0x7FF0000000000000LL;
  }
#pragma unroll 1
  for (int j = 0; j < NP; ++j) {
    int p = j;
    long long best = absbits(JA(j, j)) - Eb[j * JS];
    for (int i = j + 1; i < NP; ++i) {
      const long long kk = absbits(JA(i, j)) - Eb[i * JS];
      if (kk >= best) { best = kk; p = i; }
    }
    if (p != j) {
      for (int k = j; k <= NP; ++k) { const double t = JA(p, k); JA(p, k) = JA(j, k); JA(j, k) = t; }
      Eb[p * JS] = Eb[j * JS];
    }
    double piv = JA(j, j);
    if (piv == 0.0) piv = 1e-20;
    const double ip = 1.0 / piv;
    JA(j, j) = ip;
    for (int i = j + 1; i < NP; ++i) {
      const double l = JA(i, j) * ip;
      for (int k = j + 1; k <= NP; ++k) JA(i, k) = fma(-l, JA(j, k), JA(i, k));
    }
  }
#pragma unroll 1
  for (int i = NP - 1; i >= 0; --i) {
    double s = JA(i, NP);
    for (int k = i + 1; k < NP; ++k) s = fma(-JA(i, k), JA(k, NP), s);
    JA(i, NP) = s * JA(i, i);
  }
#undef JA
  return true;
}
)";
  }

  void newton_step() {
    const int N = n.N;
    o << "__device__ __forceinline__ int newton_step(Lane &L, double *Jb, " << (compact ? "unsigned short" : "long long")
      << " *Eb) {\n";
    o << "  L.iter += 1;\n";
    if (n.act_newton) o << "  if (L.act_fail) return " << PFCHEM_CELL_INNER_MAXITER << ";\n";
    if (n.act_freq == PFCHEM_ACT_COEF_FREQUENCY_NEWTON_ITER) {
      o << "  if (L.iter > 1) {\n  double Iv = L.Iacc;\n";
      for (int j = 0; j < N; ++j)
        if (n.Z2p[j] > 0) o << "  Iv = fma(" << lit(0.5 * n.Z2p[j]) << ", L.m[" << j << "], Iv);\n";
      activity("Iv");
      o << "  }\n";
    }
    if (rescue()) {
      // past exact_jacobian_after iterations: the exact Jacobian, no damping
      o << "  const bool rescue = L.iter > " << n.exact_after << ";\n";
      o << "  int st = evaluate_jac(L, Jb, rescue); if (st) return st;\n";
    } else {
      o << "  int st = evaluate_jac(L, Jb); if (st) return st;\n";
    }
    o << "  bool bad; const bool conv = converged(L, &bad);\n";
    o << "  if (bad) return " << PFCHEM_CELL_NONFINITE << ";\n";
    o << "  if (conv) return " << PFCHEM_CELL_CONVERGED << ";\n";
    o << "  if (L.iter >= " << n.max_iter << ") return " << PFCHEM_CELL_MAXITER << ";\n";
    if (!n.use_log) {
      for (int j = 0; j < N; ++j) {
        o << "  { const double im = 1.0 / L.m[" << j << "];\n";
        for (int i = 0; i < N; ++i) o << "    " << J(i, j) << " *= im;\n";
        o << "  }\n";
      }
    }
    if (compact) {
      o << "  double x[NP];\n";
      for (int j = 0; j < N; ++j) o << "  x[" << j << "] = L.F[" << j << "];\n";
      o << "  if (!lu_solve(Jb, Eb, x)) return " << PFCHEM_CELL_SINGULAR << ";\n";
    } else {
      for (int j = 0; j < N; ++j) o << "  " << J(j, N) << " = L.F[" << j << "];\n";
      o << "  if (!lu_solve(Jb, Eb)) return " << PFCHEM_CELL_SINGULAR << ";\n  double x[NP];\n";
      for (int j = 0; j < N; ++j) o << "  x[" << j << "] = " << J(j, N) << ";\n";
    }
    o << "  double mrc = 0.0; bool nf = false; double mnew[NP];\n";
    for (int j = 0; j < N; ++j) {
      if (n.use_log) {
        o << "  { const double u = copysign(fmin(fabs(x[" << j << "]), " << lit(n.max_dlnC) << "), x[" << j << "]);\n";
        o << "    x[" << j << "] = u; const double e = xexp(-u); mnew[" << j << "] = L.m[" << j << "] * e;\n";
        if (n.rel_change_tol > 0.0) o << "    mrc = fmax(mrc, fabs(e - 1.0));\n";
        o << "    if (!(fabs(mnew[" << j << "]) <= 1.7976931348623157e308)) nf = true; }\n";
      }
    }
    if (!n.use_log) {
      o << "  double min_ratio = 1e20;\n";
      for (int j = 0; j < N; ++j)
        o << "  if (L.m[" << j << "] <= x[" << j << "]) min_ratio = fmin(min_ratio, fabs(L.m[" << j << "] / x[" << j << "]));\n";
      o << "  const double sc = (min_ratio < 1.0) ? min_ratio * 0.99 : 1.0;\n";
      for (int j = 0; j < N; ++j) {
        o << "  mnew[" << j << "] = L.m[" << j << "] - x[" << j << "] * sc;\n";
        if (n.rel_change_tol > 0.0) o << "  mrc = fmax(mrc, fabs((mnew[" << j << "] - L.m[" << j << "]) / L.m[" << j << "]));\n";
        o << "  if (!(fabs(mnew[" << j << "]) <= 1.7976931348623157e308)) nf = true;\n";
      }
    }
    o << "  if (nf) return " << PFCHEM_CELL_NONFINITE << ";\n";
    if (n.rel_change_tol > 0.0) o << "  if (mrc < " << lit(n.rel_change_tol) << ") return " << PFCHEM_CELL_CONVERGED << ";\n";
    if (n.exact_after > 0)
      o << "  if (L.iter > 50 && L.iter <= " << n.exact_after << ") {\n";
    else
      o << "  if (L.iter > 50) {\n";
    for (int j = 0; j < N; ++j)
      o << "    mnew[" << j << "] = 0.1 * (mnew[" << j << "] - L.m[" << j << "]) + L.m[" << j << "]; L.m[" << j
        << "] = mnew[" << j << "]; L.lm[" << j << "] = log(mnew[" << j << "]);\n";
    o << "  } else {\n";
    for (int j = 0; j < N; ++j) {
      if (n.use_log) o << "    L.m[" << j << "] = mnew[" << j << "]; L.lm[" << j << "] -= x[" << j << "];\n";
      else o << "    L.m[" << j << "] = mnew[" << j << "]; L.lm[" << j << "] = log(mnew[" << j << "]);\n";
    }
    o << "  }\n  return -1;\n}\n";
  }

  void finalize() {
    o << "__device__ __forceinline__ void finalize(Lane &L, const CellArgs &a, long long cell, int status) {\n";
    o << "  const long long nc = a.ncells;\n  double Iv = 0.0, sum = 0.0;\n";
    for (int j = 0; j < n.N; ++j) {
      o << "  a.pri_molal[" << j << " * nc + cell] = L.m[" << j << "];\n";
      o << "  if (a.interleaved_out) a.interleaved_out[" << j << " * a.total_stride_comp + cell * a.total_stride_cell] = L.m[" << j << "];\n";
      o << "  if (a.total_out) a.total_out[" << j << " * nc + cell] = L.P[" << j << "] * L.den_L;\n";
      if (sorb()) o << "  a.sorb[" << j << " * nc + cell] = L.Sg[" << j << "];\n";
      if (n.Z2p[j] > 0) o << "  Iv = fma(" << lit(n.Z2p[j]) << ", L.m[" << j << "], Iv);\n";
      o << "  sum += L.m[" << j << "];\n";
    }
    o << "  if (a.sec_molal) {\n";
    if (prod_cplx()) {
      // L.bc holds the product-form constants
      for (int j = 0; j < n.N; ++j) {
        o << "  const double a" << j << " = L.m[" << j << "]" << (act() ? " * L.g[" + I(j) + "]" : "") << ";\n";
        o << "  const double ra" << j << " = 1.0 / a" << j << ";\n";
      }
      for (int i = 0; i < n.Nc; ++i)
        o << "  a.sec_molal[" << i << " * nc + cell] = " << prod_expr("L.bc[" + I(i) + "]", n.cn[i], n.cid[i], n.cnu[i])
          << ";\n";
    } else {
      for (int j = 0; j < n.N; ++j) {
        if (act()) o << "  const double la" << j << " = L.lm[" << j << "] + L.lg[" << j << "];\n";
        else o << "  const double la" << j << " = L.lm[" << j << "];\n";
      }
      for (int i = 0; i < n.Nc; ++i) {
        o << "  { double s = L.bc[" << i << "];\n";
        for (int k = 0; k < n.cn[i]; ++k) acc(o, "s", n.cnu[i][k], "la" + I(n.cid[i][k]));
        o << "    a.sec_molal[" << i << " * nc + cell] = exp(s); }\n";
      }
    }
    o << "  }\n";
    o << "  sum += L.Csum;\n";
    o << "  a.ionic[cell] = 0.5 * Iv + L.Iacc;\n";
    if (n.use_h2o) o << "  if (a.lnaw) { const double v = 1.0 - 0.017 * sum; a.lnaw[cell] = v > 0.0 ? log(v) : 0.0; }\n";
    for (int k = 0; k < n.Nm; ++k) {
      o << "  if (a.rate) a.rate[" << k << " * nc + cell] = L.rate[" << k << "];\n";
      if (n.update_kin)
        o << "  if (status == 0) { double v = L.vf[" << k << "] + L.rate[" << k << "] * " << lit(n.mVm[k])
          << " * L.dtc; a.vf[" << k << " * nc + cell] = v < 0.0 ? 0.0 : v; }\n";
    }
    for (int r = 0; r < n.Nix; ++r) o << "  a.ixref[" << r << " * nc + cell] = L.ixr[" << r << "];\n";
    for (int r = 0; r < n.Nsr; ++r) o << "  a.srfree[" << r << " * nc + cell] = L.srf[" << r << "];\n";
    o << "  if (a.iters) a.iters[cell] = L.iter;\n  if (a.status) a.status[cell] = status;\n}\n";
  }

  // Per-cell record the prologue writes for the solve kernel (SoA, stride
  // ncells): free-ion molalities and their logs at the chosen starting
  // guess, ln gamma and gamma of the primaries, the fixed accumulation, the
  // complex/mineral/surface constants, the ion-exchange warm starts, and
  // whether the alternative guess was taken.
  int prep_fields() const {
    return 5 * n.N + n.Nc + (n.act_freq == PFCHEM_ACT_COEF_FREQUENCY_NEWTON_ITER ? n.Nc : 0) + 2 * n.Nm + n.Nsc +
           n.Nix + 1 + npf_total() + (need_bk() ? 0 : 2 * (int)pf_complexes().size());
  }
  void prep_io(bool store) {
    int f = 0;
    auto fld = [&](const std::string &lane) {
      if (store) o << "  prep[" << f << " * nc + cell] = " << lane << ";\n";
      else o << "  " << lane << " = prep[" << f << " * nc + cell];\n";
      ++f;
    };
    for (int j = 0; j < n.N; ++j) fld("L.m[" + I(j) + "]");
    for (int j = 0; j < n.N; ++j) fld("L.lm[" + I(j) + "]");
    for (int j = 0; j < n.N; ++j) fld("L.lg[" + I(j) + "]");
    for (int j = 0; j < n.N; ++j) fld("L.g[" + I(j) + "]");
    for (int j = 0; j < n.N; ++j) fld("L.fx[" + I(j) + "]");
    for (int i = 0; i < n.Nc; ++i) fld("L.bc[" + I(i) + "]");
    if (n.act_freq == PFCHEM_ACT_COEF_FREQUENCY_NEWTON_ITER)
      for (int i = 0; i < n.Nc; ++i) fld("L.bK[" + I(i) + "]");
    for (int k = 0; k < n.Nm; ++k) fld("L.bm[" + I(k) + "]");
    for (int k = 0; k < n.Nm; ++k) fld("L.rk[" + I(k) + "]");
    for (int k = 0; k < n.Nsc; ++k) fld("L.bs[" + I(k) + "]");
    for (int r = 0; r < n.Nix; ++r) fld("L.ixr[" + I(r) + "]");
    for (int t = 0; t < npf_total(); ++t) fld("L.pk[" + I(t) + "]");
    if (!need_bk())
      for (size_t q = 0; q < pf_complexes().size(); ++q) {
        fld("L.pK[" + I((int)q) + "]");
        fld("L.pg[" + I((int)q) + "]");
      }
    // flags: 1 = the alternative guess was taken, 2 = the activity algorithm failed
    if (store) o << "  prep[" << f << " * nc + cell] = (L.alt_used ? 1.0 : 0.0) + (L.act_fail ? 2.0 : 0.0);\n";
    else
      o << "  { const double fl = prep[" << f << " * nc + cell]; L.alt_used = fl == 1.0 || fl == 3.0; L.act_fail = fl >= 2.0; }\n";
  }

  // Data-parallel prologue: one thread per cell, every lane busy.  It does
  // all per-cell work that does not iterate -- log K, activity terms, fixed
  // accumulation, logs of the guess -- and, given an alternative guess,
  // evaluates the residual at both guesses and keeps the better one.
  void prologue() {
    o << "extern \"C\" __global__ void __launch_bounds__(128) pfchem_gen_prologue(const __grid_constant__ CellArgs a, "
         "double *prep, double inv_dt, Scratch *scr) {\n";
    o << "  const long long cell = blockIdx.x * (long long)blockDim.x + threadIdx.x;\n";
    o << "  const long long nc = a.ncells;\n  bool used = false;\n";
    o << "  if (cell < nc && !(a.active && a.active[cell] <= 0)) {\n";
    o << "  Lane L;\n  setup(L, a, cell, inv_dt);\n";
    o << "  if (a.alt_guess) {\n";
    o << "    evaluate_res(L, nullptr); bool bad; converged(L, &bad);\n";
    o << "    const double rplain = bad ? 1.7976931348623157e308 : rnorm(L);\n";
    o << "    double pm[NP], plm[NP], pix[NIX];\n";
    o << "    for (int j = 0; j < NP; ++j) { pm[j] = L.m[j]; plm[j] = L.lm[j]; }\n";
    o << "    for (int r = 0; r < NIX; ++r) pix[r] = L.ixr[r];\n";
    o << "    bool ok = true;\n";
    for (int j = 0; j < n.N; ++j)
      o << "    { const double g = a.alt_guess[" << j << " * nc + cell]; if (g > 0.0 && g <= 1.7976931348623157e308) { L.m["
        << j << "] = g; L.lm[" << j << "] = xlog(g); } else ok = false; }\n";
    o << "    double ralt = 1.7976931348623157e308;\n";
    o << "    if (ok) { const int st = evaluate_res(L, nullptr); converged(L, &bad); if (!bad && st == 0) ralt = rnorm(L); }\n";
    o << "    if (ralt <= rplain) { L.alt_used = true; used = true; }\n";
    o << "    else { for (int j = 0; j < NP; ++j) { L.m[j] = pm[j]; L.lm[j] = plm[j]; } for (int r = 0; r < NIX; ++r) L.ixr[r] = pix[r]; }\n";
    o << "  }\n";
    prep_io(true);
    o << "  }\n";
    o << "  const unsigned bal = __ballot_sync(0xffffffffu, used);\n";
    o << "  if ((threadIdx.x & 31) == 0 && bal) atomicAdd(&scr->alt_used, (unsigned long long)__popc(bal));\n";
    o << "}\n";
  }

  // The solve kernel's per-cell start: the prologue's record plus the
  // per-cell scalars that cost no FP64 work worth moving.
  void load_prep() {
    o << "__device__ __forceinline__ void load_prep(Lane &L, const CellArgs &a, long long cell, const double *prep, "
         "double inv_dt) {\n";
    o << "  const long long nc = a.ncells;\n";
    o << "  const double por = a.por[cell], sat = a.sat[cell], vol = a.vol[cell], den = a.den[cell];\n";
    o << "  L.por = por; L.vol = vol; L.dtc = a.dt;\n";
    if (need_rho()) o << "  L.rho_s = a.rho_s[cell];\n";
    o << "  L.acc = " << (n.accum_mode == PFCHEM_ACCUM_DT_CONSISTENT ? "inv_dt" : "1.0") << ";\n";
    o << "  const double psv = por * sat * 1000.0 * vol;\n";
    o << "  L.den_L = den * 1e-3; L.psv_den = psv * L.den_L; L.jac_aq = psv * inv_dt * L.den_L; L.v_t = vol * inv_dt;\n";
    for (int k = 0; k < n.Nm; ++k)
      o << "  L.vf[" << k << "] = a.vf[" << k << " * nc + cell]; L.ar[" << k << "] = a.area[" << k
        << " * nc + cell]; L.rate[" << k << "] = 0.0;\n";
    for (int r = 0; r < n.Nsr; ++r) o << "  L.srf[" << r << "] = a.srfree[" << r << " * nc + cell];\n";
    prep_io(false);
    o << "  L.Icell = a.ionic[cell]; L.Iacc = 0.0; L.Csum = 0.0;\n";
    o << "  L.iter = 0; L.alt_pending = false;\n}\n";
  }

  void kernel() {
    o << "extern \"C\" __global__ void __launch_bounds__(" << js << ") pfchem_gen_react(const __grid_constant__ CellArgs a, "
         "Scratch *scr, int refill_min_idle, double inv_dt, const double *prep) {\n";
    o << "  extern __shared__ double smem[];\n  double *Jb = smem + threadIdx.x;\n";
    if (compact)
      o << "  unsigned short *Eb = (unsigned short *)(smem + " << n.N * n.N * js << ") + threadIdx.x;\n";
    else
      o << "  long long *Eb = (long long *)(smem + " << n.N * (n.N + 1) * js << ") + threadIdx.x;\n";
    o << R"(  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  Lane L;
  long long cell = -1;
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
          cell = (long long)c;
          if (a.active && a.active[cell] <= 0) {
            if (a.status) a.status[cell] = 5;
            if (a.iters) a.iters[cell] = 0;
            cell = -1;
          } else {
            load_prep(L, a, cell, prep, inv_dt);
          }
        } else {
          if (!exhausted) atomicMax(&scr->t_drain_inv, ~pf_now());
          exhausted = true;
        }
      }
      continue;
    }
    if (busy_mask == 0) {
      if (__all_sync(full, exhausted)) break;
      continue;
    }
    ++my_trips;
    if (cell >= 0) {
      int st = newton_step(L, Jb, Eb);
      if (st >= 0) {
        finalize(L, a, cell, st);
        my_iters += L.iter;
        my_max = max(my_max, (unsigned)L.iter);
        if (st != 0) my_bad += 1;
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
    atomicAdd(&scr->sum_iter, my_iters);
    atomicAdd(&scr->newton_trips, my_trips);
    atomicMax(&scr->t_end, pf_now());
    (void)my_alt;
    atomicMax(&scr->max_iter, my_max);
    atomicAdd(&scr->nonconverged, my_bad);
  }
}
)";
  }

  std::string source() {
    header();
    setup();
    evaluate(true);
    evaluate(false);
    converged();
    solve();
    newton_step();
    finalize();
    prologue();
    load_prep();
    kernel();
    return o.str();
  }
};

struct Loaded {
  CUmodule mod = nullptr;
  CUfunction fn = nullptr;   // persistent solve kernel
  CUfunction pro = nullptr;  // data-parallel prologue
};

// Driver-API entry points, resolved through the runtime so that the library
// does not link libcuda (it loads on machines without a driver, e.g. for the
// build-time checks).
struct Driver {
  CUresult (*moduleLoadData)(CUmodule *, const void *) = nullptr;
  CUresult (*moduleGetFunction)(CUfunction *, CUmodule, const char *) = nullptr;
  CUresult (*funcSetAttribute)(CUfunction, CUfunction_attribute, int) = nullptr;
  CUresult (*occupancy)(int *, CUfunction, int, size_t) = nullptr;
  CUresult (*launchKernel)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned,
                           CUstream, void **, void **) = nullptr;
  CUresult (*getErrorString)(CUresult, const char **) = nullptr;
  bool ok = false;
};

const Driver &driver() {
  static Driver d;
  static std::once_flag once;
  std::call_once(once, [] {
    auto get = [](const char *name, void **fn) {
      cudaDriverEntryPointQueryResult q;
      return cudaGetDriverEntryPointByVersion(name, fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
             q == cudaDriverEntryPointSuccess && *fn != nullptr;
    };
    d.ok = get("cuModuleLoadData", (void **)&d.moduleLoadData) &&
           get("cuModuleGetFunction", (void **)&d.moduleGetFunction) &&
           get("cuFuncSetAttribute", (void **)&d.funcSetAttribute) &&
           get("cuOccupancyMaxActiveBlocksPerMultiprocessor", (void **)&d.occupancy) &&
           get("cuLaunchKernel", (void **)&d.launchKernel) && get("cuGetErrorString", (void **)&d.getErrorString);
  });
  return d;
}

std::mutex g_cache_mutex;
std::map<std::string, Loaded> g_cache;  // key: device + block + source

}  // namespace

std::string generate_source(const DevNet &n, int block, bool compact) {
  Gen g(n, block, compact);
  return g.source();
}

// Shared memory of the persistent kernel: per thread the augmented [J | F]
// and 64-bit row exponents, or (compact) J and 16-bit row exponents.
size_t gen_shared_bytes(const DevNet &n, int block, bool compact) {
  if (compact) return (((size_t)n.N * n.N * sizeof(double) + n.N * sizeof(unsigned short) + 7) / 8) * 8 * block;
  return ((size_t)n.N * (n.N + 1) + n.N) * block * sizeof(double);
}

namespace {

// NVRTC compile of one generated source to a cubin (no shared state: runs
// concurrently for several candidates).
int compile_cubin(const std::string &src, std::vector<char> *cubin, std::string *err) {
  nvrtcProgram prog;
  if (nvrtcCreateProgram(&prog, src.c_str(), "pfchem_gen.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS) {
    *err = "nvrtcCreateProgram failed";
    return -2;
  }
  const char *opts[] = {"--gpu-architecture=sm_103a", "--std=c++17", "-default-device", "--fmad=true",
                        "-lineinfo"};
  nvrtcResult rc = nvrtcCompileProgram(prog, 5, opts);
  if (rc != NVRTC_SUCCESS) {
    size_t ls = 0;
    nvrtcGetProgramLogSize(prog, &ls);
    std::string log(ls, '\0');
    nvrtcGetProgramLog(prog, &log[0]);
    nvrtcDestroyProgram(&prog);
    *err = "NVRTC compile failed: " + log.substr(0, 1500);
    return -2;
  }
  size_t cs = 0;
  nvrtcGetCUBINSize(prog, &cs);
  cubin->resize(cs);
  nvrtcGetCUBIN(prog, cubin->data());
  nvrtcDestroyProgram(&prog);
  return 0;
}

// Loads a cubin into the current context and caches it under `key`
// (g_cache_mutex held by the caller).
int load_cubin(const std::string &key, const std::vector<char> &cubin, Loaded *out, std::string *err) {
  const Driver &D = driver();
  if (!D.ok) {
    *err = "CUDA driver entry points unavailable";
    return -2;
  }
  Loaded L;
  CUresult cr = D.moduleLoadData(&L.mod, cubin.data());
  if (cr != CUDA_SUCCESS) {
    const char *s = nullptr;
    D.getErrorString(cr, &s);
    *err = std::string("cuModuleLoadData: ") + (s ? s : "?");
    return -2;
  }
  cr = D.moduleGetFunction(&L.fn, L.mod, "pfchem_gen_react");
  if (cr == CUDA_SUCCESS) cr = D.moduleGetFunction(&L.pro, L.mod, "pfchem_gen_prologue");
  if (cr != CUDA_SUCCESS) {
    *err = "cuModuleGetFunction failed";
    return -2;
  }
  D.funcSetAttribute(L.fn, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, 227 * 1024);
  g_cache[key] = L;
  *out = L;
  return 0;
}

std::string cache_key(int dev, int block, const std::string &src) {
  return std::to_string(dev) + ":" + std::to_string(block) + ":" + src;
}

}  // namespace

// Compiles (or fetches from the per-process cache) the specialized kernel for
// `n` and `block` threads per block on the current device.
int gen_kernel(const DevNet &n, int block, bool compact, void **fn_out, void **pro_out, std::string *err) {
  int dev = 0;
  cudaGetDevice(&dev);
  cudaFree(0);  // make the device's primary context current for the driver API
  const std::string src = generate_source(n, block, compact);
  const std::string key = cache_key(dev, block, src);
  {
    std::lock_guard<std::mutex> lock(g_cache_mutex);
    auto it = g_cache.find(key);
    if (it != g_cache.end()) {
      *fn_out = (void *)it->second.fn;
      *pro_out = (void *)it->second.pro;
      return 0;
    }
  }
  std::vector<char> cubin;
  if (compile_cubin(src, &cubin, err)) return -2;
  std::lock_guard<std::mutex> lock(g_cache_mutex);
  auto it = g_cache.find(key);  // compiled meanwhile by another thread
  Loaded L;
  if (it != g_cache.end()) L = it->second;
  else if (load_cubin(key, cubin, &L, err)) return -2;
  *fn_out = (void *)L.fn;
  *pro_out = (void *)L.pro;
  return 0;
}

// Compiles the specialized kernels of several (block, compact) candidates
// concurrently (one NVRTC program per thread) and caches them; the first
// error, if any, goes to `err`.
int gen_kernels_prepare(const DevNet &n, const std::vector<std::pair<int, bool>> &cands, std::string *err) {
  int dev = 0;
  cudaGetDevice(&dev);
  cudaFree(0);
  std::vector<std::string> keys(cands.size());
  std::vector<std::vector<char>> bins(cands.size());
  std::vector<std::string> errs(cands.size());
  std::vector<int> rcs(cands.size(), 0);
  std::vector<std::thread> pool;
  for (size_t i = 0; i < cands.size(); ++i) {
    const std::string src = generate_source(n, cands[i].first, cands[i].second);
    keys[i] = cache_key(dev, cands[i].first, src);
    {
      std::lock_guard<std::mutex> lock(g_cache_mutex);
      if (g_cache.count(keys[i])) continue;
    }
    pool.emplace_back([&, i, src]() { rcs[i] = compile_cubin(src, &bins[i], &errs[i]); });
  }
  for (auto &t : pool) t.join();
  std::lock_guard<std::mutex> lock(g_cache_mutex);
  int rc = 0;
  for (size_t i = 0; i < cands.size(); ++i) {
    if (rcs[i]) {
      if (!rc) *err = errs[i];
      rc = -2;
      continue;
    }
    if (bins[i].empty() || g_cache.count(keys[i])) continue;
    Loaded L;
    std::string e;
    if (load_cubin(keys[i], bins[i], &L, &e)) {
      if (!rc) *err = e;
      rc = -2;
    }
  }
  return rc;
}

int gen_prep_fields(const DevNet &n) {
  Gen g(n, 32);
  return g.prep_fields();
}

int gen_blocks_per_sm(void *fn, const DevNet &n, int block, bool compact) {
  int nb = 0;
  const Driver &D = driver();
  if (!D.ok || D.occupancy(&nb, (CUfunction)fn, block, gen_shared_bytes(n, block, compact)) != CUDA_SUCCESS) return 0;
  return nb;
}

// Prologue over all cells, then the persistent solve.
cudaError_t gen_launch(void *fn, void *pro, const DevNet &n, const CellArgs &a, Scratch *scr, double *prep, int grid,
                       int block, int refill, cudaStream_t st, bool compact) {
  CellArgs args = a;
  double inv_dt = 1.0 / a.dt;
  const Driver &D = driver();
  if (!D.ok || !fn || !pro) return cudaErrorLaunchFailure;
  void *pparams[] = {&args, &prep, &inv_dt, &scr};
  const unsigned pgrid = (unsigned)((a.ncells + 127) / 128);
  CUresult r = D.launchKernel((CUfunction)pro, pgrid, 1, 1, 128, 1, 1, 0, (CUstream)st, pparams, nullptr);
  if (r != CUDA_SUCCESS) return cudaErrorLaunchFailure;
  void *params[] = {&args, &scr, &refill, &inv_dt, &prep};
  r = D.launchKernel((CUfunction)fn, grid, 1, 1, block, 1, 1, (unsigned)gen_shared_bytes(n, block, compact), (CUstream)st,
                     params, nullptr);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorLaunchFailure;
}

}  // namespace pfchem
