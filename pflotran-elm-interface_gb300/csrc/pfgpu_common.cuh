// pfgpu_common.cuh -- device-side network tables and shared helpers.
//
// A network lives on the device as one packed buffer (see pfgpu_api.cu):
// reaction rows in CSR form (row pointer, species id, stoichiometry), so the
// per-secondary species loops read a contiguous, broadcastable slice that a
// block stages once into shared memory.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/pfgpu.h"

namespace pfgpu {

// pflotran_constants.F90:84 (truncated constant, kept for parity) and :89
constexpr double LOG_TO_LN = 2.30258509299;
constexpr double IDEAL_GAS_CONSTANT = 8.31446;
constexpr double RT_MIN_SATURATION = 1.0e-40;  // reactive_transport_aux.F90:19

enum : int32_t {
  NETF_SEC_LOGKCOEF = 1,
  NETF_MNRL_LOGKCOEF = 2,
  NETF_MSF = 4,
  NETF_TEMKIN = 8,
  NETF_POWER = 16,
  NETF_PREFACTOR = 32,  // some mineral has rate prefactors
  NETF_H2O = 64,        // some complex or mineral has water in its reaction
  NETF_SX_LOGKCOEF = 128,  // surface complexes carry logK temperature fits
};

// Device view of a network.  All pointers index one packed allocation whose
// layout is: [ints: sec_ptr(ns+1) sec_idx(nnz_s) mnrl_ptr(nm+1) mnrl_idx(nnz_m)
// irreversible(nm)] [doubles: sec_nu(nnz_s) sec_logK(ns) sec_logKcoef(5ns)
// pri_Z pri_a0 sec_Z sec_a0 mnrl_nu(nnz_m) mnrl_logK mnrl_logKcoef(5nm)
// rate_constant activation_energy molar_vol affinity_threshold rate_limiter
// msf temkin power]
// Lookup tables of the group-per-cell step kernel (device pointers into one
// allocation): for species i, the secondary complexes sp_s[sp_ptr[i] ..
// sp_ptr[i+1]) that contain it with the CSR slot sp_p of i in each, and the
// same for the kinetic minerals (mp_*).
struct GroupTabs {
  const int32_t* sp_ptr;
  const int32_t* sp_s;
  const int32_t* sp_p;
  const int32_t* mp_ptr;
  const int32_t* mp_m;
  const int32_t* mp_p;
  const double* sp_nu;  // nu of species i in complex sp_s[q] / mineral mp_m[q]
  const double* mp_nu;
  // the complexes in the order a group's lanes take them in the evaluation,
  // longest species list first (the lanes of one round loop alike)
  const int32_t* s_perm;
};

struct DevNet {
  int32_t n, ns, nm;
  int32_t nnz_s, nnz_m;
  int32_t flags;
  int32_t int_words;     // number of int32 words in the int block
  int32_t dbl_words;     // number of doubles in the double block
  int32_t int_words_grp; // the prefixes the group kernel stages (it reads
  int32_t dbl_words_grp; //   no pair table of the one-lane kernel) ...
  int32_t int_words_core, dbl_words_core;  // ... or these, without the per-entry tables
  int32_t ent_staged;    // group launch: the per-entry tables are in shared memory
  const int32_t* ints;   // device: start of int block (16-byte aligned)
  const double* dbls;    // device: start of double block (16-byte aligned)
  // offsets (in elements) into the int block
  int32_t o_sec_ptr, o_sec_idx, o_mnrl_ptr, o_mnrl_idx, o_irrev;
  // offsets into the double block
  int32_t o_sec_nu, o_sec_logK, o_sec_logKcoef, o_pri_Z, o_pri_a0, o_sec_Z, o_sec_a0;
  int32_t o_mnrl_nu, o_mnrl_logK, o_mnrl_logKcoef, o_rate, o_ea, o_molar_vol, o_thresh,
      o_limiter, o_msf, o_temkin, o_power;
  // product-form speciation tables (batched kernel): per CSR entry the index
  // code*n + species into the lane's power table (code 0: a, 1: a^2, 2: 1/a,
  // 3: 1/a^2; -1: other coefficient), and per reaction the (p <= q) species
  // pairs as flat Jacobian index with coefficient nu_p*nu_q (minerals: all
  // ordered pairs)
  int32_t o_sec_pidx, o_spair_ptr, o_spair_idx, o_mnrl_pidx, o_mpair_ptr, o_mpair_idx;
  int32_t o_spair_coef, o_mpair_coef;
  // per-entry assembly of the lower triangle (group kernel): entry e -> flat
  // index i*n+j; CSR over contributing complexes / minerals with nu_i nu_j
  int32_t o_ent_ij, o_ent_ptr, o_ent_sc, o_ent_mptr, o_ent_mm, o_ent_cf, o_ent_mcf;
  int32_t neg_mask;  // bit j: species j carries a negative coefficient somewhere
  // equilibrium sorption (PfSorptionDesc): K_D rows and ion-exchange CSR
  int32_t nkd, nionx, kd_units;
  int32_t o_kd_spec, o_kd_type, o_kd_min, o_ix_ptr, o_ix_cat, o_ix_min, o_ix_zflag;
  int32_t o_kd_coeff, o_kd_b, o_kd_n, o_ix_k, o_ix_cec;
  // equilibrium surface complexation: reactions (sites) and their complexes;
  // ints: complexes of reaction r [sx_ptr(r), sx_ptr(r+1)), surface type,
  // mineral, stoichiometry flag (a complex holds more than one site), the
  // complexes' species CSR; doubles: site density, stoichiometry, free-site
  // stoichiometry, logK, logK fits, water coefficient
  int32_t nsrx, nsrc;
  int32_t o_sx_ptr, o_sx_type, o_sx_min, o_sx_flag, o_sx_cptr, o_sx_spec;
  int32_t o_sx_dens, o_sx_nu, o_sx_nuf, o_sx_logK, o_sx_logKcoef, o_sx_h2o;
  double soil_density;
  // kinetic-mineral rate prefactors (PfPrefactorDesc), dense [nm][MP] and
  // [nm][MP][MS]: counts, species ids (primary j, secondary i as -(i+1));
  // rate, activation energy, alpha, beta, attenuation coefficient
  int32_t o_pf_cnt, o_pf_nsp, o_pf_id;
  int32_t o_pf_rate, o_pf_ea, o_pf_alpha, o_pf_beta, o_pf_atten;
  // water coefficients of the complexes' and minerals' reactions (0: none)
  int32_t o_sec_h2o, o_mnrl_h2o;
  double A, B, Bdot;
  PfOptions o;
  GroupTabs grp;
};

// the network has equilibrium sorption of any kind (the sorbed state
// arrays are required, the sorbed accumulation enters the step)
__host__ __device__ __forceinline__ bool has_sorption(const DevNet& net) {
  return net.nkd + net.nionx + net.nsrx > 0;
}

// Table accessor over either global or shared copies of the packed blocks.
// Water activity in ln Q/K: some reaction has water and the option is on
// (otherwise ln a_H2O stays at RTAuxVarInit's 0 in the reference)
__host__ __device__ __forceinline__ bool water_on(const DevNet& net) {
  return (net.flags & NETF_H2O) && net.o.use_activity_h2o;
}
// the cell's ln a_H2O (0 when the water activity is off or not carried)
__device__ __forceinline__ double cell_lnaw(const DevNet& net, const PfCellState& st, int64_t cell) {
  return (water_on(net) && st.ln_act_h2o) ? st.ln_act_h2o[cell] : 0.0;
}

// ln Q/K's water term: the reaction's water coefficient times ln a_H2O
// (reaction.F90:4715-4717, reaction_mineral.F90:769-772), skipped for a
// reaction without water as the reference skips it
__device__ __forceinline__ double add_h2o(double lnQK, double coef, double ln_act_h2o) {
  return coef != 0.0 ? lnQK + coef * ln_act_h2o : lnQK;
}

// ln a_H2O = ln(1 - 0.017 (sum of molalities)), 0 when the argument is not
// positive (reaction.F90:4539-4547, 4604-4611)
__device__ __forceinline__ double water_activity(double sum_pri_molal, double sum_sec_molal) {
  const double a = 1.0 - 0.017 * (sum_pri_molal + sum_sec_molal);
  return a > 0.0 ? log(a) : 0.0;
}

struct Tables {
  const int32_t* I;
  const double* D;
  const DevNet* net;
  __device__ __forceinline__ int sec_begin(int i) const { return I[net->o_sec_ptr + i]; }
  __device__ __forceinline__ int sec_end(int i) const { return I[net->o_sec_ptr + i + 1]; }
  __device__ __forceinline__ int sec_idx(int p) const { return I[net->o_sec_idx + p]; }
  __device__ __forceinline__ double sec_nu(int p) const { return D[net->o_sec_nu + p]; }
  __device__ __forceinline__ double sec_logK(int i) const { return D[net->o_sec_logK + i]; }
  __device__ __forceinline__ const double* sec_logKcoef(int i) const { return D + net->o_sec_logKcoef + 5 * i; }
  __device__ __forceinline__ double pri_Z(int j) const { return D[net->o_pri_Z + j]; }
  __device__ __forceinline__ double pri_a0(int j) const { return D[net->o_pri_a0 + j]; }
  __device__ __forceinline__ double sec_Z(int i) const { return D[net->o_sec_Z + i]; }
  __device__ __forceinline__ double sec_a0(int i) const { return D[net->o_sec_a0 + i]; }
  __device__ __forceinline__ int mnrl_begin(int m) const { return I[net->o_mnrl_ptr + m]; }
  __device__ __forceinline__ int mnrl_end(int m) const { return I[net->o_mnrl_ptr + m + 1]; }
  __device__ __forceinline__ int mnrl_idx(int p) const { return I[net->o_mnrl_idx + p]; }
  __device__ __forceinline__ double mnrl_nu(int p) const { return D[net->o_mnrl_nu + p]; }
  __device__ __forceinline__ double mnrl_logK(int m) const { return D[net->o_mnrl_logK + m]; }
  __device__ __forceinline__ const double* mnrl_logKcoef(int m) const { return D + net->o_mnrl_logKcoef + 5 * m; }
  __device__ __forceinline__ double rate(int m) const { return D[net->o_rate + m]; }
  __device__ __forceinline__ double ea(int m) const { return D[net->o_ea + m]; }
  __device__ __forceinline__ double molar_vol(int m) const { return D[net->o_molar_vol + m]; }
  __device__ __forceinline__ double thresh(int m) const { return D[net->o_thresh + m]; }
  __device__ __forceinline__ double limiter(int m) const { return D[net->o_limiter + m]; }
  __device__ __forceinline__ int irreversible(int m) const { return I[net->o_irrev + m]; }
  __device__ __forceinline__ double msf(int m) const { return D[net->o_msf + m]; }
  __device__ __forceinline__ double temkin(int m) const { return D[net->o_temkin + m]; }
  __device__ __forceinline__ double power(int m) const { return D[net->o_power + m]; }
  __device__ __forceinline__ int sec_pidx(int p) const { return I[net->o_sec_pidx + p]; }
  __device__ __forceinline__ int spair_begin(int i) const { return I[net->o_spair_ptr + i]; }
  __device__ __forceinline__ int spair_idx(int q) const { return I[net->o_spair_idx + q]; }
  __device__ __forceinline__ double spair_coef(int q) const { return D[net->o_spair_coef + q]; }
  __device__ __forceinline__ int mnrl_pidx(int p) const { return I[net->o_mnrl_pidx + p]; }
  __device__ __forceinline__ int mpair_begin(int m) const { return I[net->o_mpair_ptr + m]; }
  __device__ __forceinline__ int mpair_idx(int q) const { return I[net->o_mpair_idx + q]; }
  __device__ __forceinline__ double mpair_coef(int q) const { return D[net->o_mpair_coef + q]; }
  __device__ __forceinline__ int ent_ij(int e) const { return I[net->o_ent_ij + e]; }
  __device__ __forceinline__ int ent_begin(int e) const { return I[net->o_ent_ptr + e]; }
  __device__ __forceinline__ int ent_end(int e) const { return I[net->o_ent_ptr + e + 1]; }
  __device__ __forceinline__ int ent_sc(int q) const { return I[net->o_ent_sc + q]; }
  __device__ __forceinline__ double ent_cf(int q) const { return D[net->o_ent_cf + q]; }
  __device__ __forceinline__ int ent_mbegin(int e) const { return I[net->o_ent_mptr + e]; }
  __device__ __forceinline__ int ent_mend(int e) const { return I[net->o_ent_mptr + e + 1]; }
  __device__ __forceinline__ int ent_mm(int q) const { return I[net->o_ent_mm + q]; }
  __device__ __forceinline__ double ent_mcf(int q) const { return D[net->o_ent_mcf + q]; }
  __device__ __forceinline__ int kd_spec(int r) const { return I[net->o_kd_spec + r]; }
  __device__ __forceinline__ int kd_type(int r) const { return I[net->o_kd_type + r]; }
  __device__ __forceinline__ int kd_min(int r) const { return I[net->o_kd_min + r]; }
  __device__ __forceinline__ double kd_coeff(int r) const { return D[net->o_kd_coeff + r]; }
  __device__ __forceinline__ double kd_b(int r) const { return D[net->o_kd_b + r]; }
  __device__ __forceinline__ double kd_n(int r) const { return D[net->o_kd_n + r]; }
  __device__ __forceinline__ int ix_begin(int r) const { return I[net->o_ix_ptr + r]; }
  __device__ __forceinline__ int ix_end(int r) const { return I[net->o_ix_ptr + r + 1]; }
  __device__ __forceinline__ int ix_cat(int p) const { return I[net->o_ix_cat + p]; }
  __device__ __forceinline__ double ix_k(int p) const { return D[net->o_ix_k + p]; }
  __device__ __forceinline__ double ix_cec(int r) const { return D[net->o_ix_cec + r]; }
  __device__ __forceinline__ int ix_min(int r) const { return I[net->o_ix_min + r]; }
  __device__ __forceinline__ int ix_zflag(int r) const { return I[net->o_ix_zflag + r]; }
  __device__ __forceinline__ int sx_begin(int r) const { return I[net->o_sx_ptr + r]; }
  __device__ __forceinline__ int sx_end(int r) const { return I[net->o_sx_ptr + r + 1]; }
  __device__ __forceinline__ int sx_type(int r) const { return I[net->o_sx_type + r]; }
  __device__ __forceinline__ int sx_min(int r) const { return I[net->o_sx_min + r]; }
  __device__ __forceinline__ int sx_flag(int r) const { return I[net->o_sx_flag + r]; }
  __device__ __forceinline__ int sx_cbegin(int k) const { return I[net->o_sx_cptr + k]; }
  __device__ __forceinline__ int sx_cend(int k) const { return I[net->o_sx_cptr + k + 1]; }
  __device__ __forceinline__ int sx_spec(int p) const { return I[net->o_sx_spec + p]; }
  __device__ __forceinline__ double sx_dens(int r) const { return D[net->o_sx_dens + r]; }
  __device__ __forceinline__ double sx_nu(int p) const { return D[net->o_sx_nu + p]; }
  __device__ __forceinline__ double sx_nuf(int k) const { return D[net->o_sx_nuf + k]; }
  __device__ __forceinline__ double sx_logK(int k) const { return D[net->o_sx_logK + k]; }
  __device__ __forceinline__ const double* sx_logKcoef(int k) const { return D + net->o_sx_logKcoef + 5 * k; }
  __device__ __forceinline__ double sx_h2o(int k) const { return D[net->o_sx_h2o + k]; }
  __device__ __forceinline__ int pf_cnt(int m) const { return I[net->o_pf_cnt + m]; }
  __device__ __forceinline__ double sec_h2o(int i) const { return D[net->o_sec_h2o + i]; }
  __device__ __forceinline__ double mnrl_h2o(int m) const { return D[net->o_mnrl_h2o + m]; }
  __device__ __forceinline__ int pf_nsp(int m, int p) const { return I[net->o_pf_nsp + m * PF_MAX_PREFACTORS + p]; }
  __device__ __forceinline__ double pf_rate(int m, int p) const {
    return D[net->o_pf_rate + m * PF_MAX_PREFACTORS + p];
  }
  __device__ __forceinline__ double pf_ea(int m, int p) const { return D[net->o_pf_ea + m * PF_MAX_PREFACTORS + p]; }
  // species slot q = (m*MP + p)*MS + s
  __device__ __forceinline__ int pf_id(int q) const { return I[net->o_pf_id + q]; }
  __device__ __forceinline__ double pf_alpha(int q) const { return D[net->o_pf_alpha + q]; }
  __device__ __forceinline__ double pf_beta(int q) const { return D[net->o_pf_beta + q]; }
  __device__ __forceinline__ double pf_atten(int q) const { return D[net->o_pf_atten + q]; }
};

// Fortran SIGN(1.d0, x)
__device__ __forceinline__ double fsign1(double x) { return signbit(x) ? -1.0 : 1.0; }

// ReactionInterpolateLogK, reaction_aux.F90:1285-1312 (one reaction)
__device__ __forceinline__ double interp_logK(const double* c, double temp) {
  double tk = temp + 273.15;
  return c[0] * log(tk) + c[1] + c[2] * tk + c[3] / tk + c[4] / (tk * tk);
}

// interp_logK for many reactions at one temperature: ln T_K, 1/T_K and
// 1/T_K^2 once per cell.  Each quotient c/t is the product q = c (1/t) plus
// one residual correction q + (c - q t)(1/t) (Markstein's correction step,
// one fused multiply-add for the exact residual), which gives the rounded
// quotient but for rare ties -- four FP64 operations instead of a division.
struct LogKAtT {
  double ltk, tk, itk, tk2, itk2;
  __device__ __forceinline__ explicit LogKAtT(double temp) {
    tk = temp + 273.15;
    ltk = log(tk);
    itk = 1.0 / tk;
    tk2 = tk * tk;
    itk2 = 1.0 / tk2;
  }
  __device__ __forceinline__ static double quot(double c, double t, double it) {
    const double q = c * it;
    return fma(fma(-q, t, c), it, q);
  }
  // A zero coefficient contributes an exact zero, so its term is skipped (a
  // branch on the reaction's coefficient, the same in every lane): a fit
  // linear in T costs one multiply-add.
  __device__ __forceinline__ double operator()(const double* c) const {
    double v = c[0] != 0.0 ? c[0] * ltk + c[1] : c[1];
    if (c[2] != 0.0) v = v + c[2] * tk;
    if (c[3] != 0.0) v = v + quot(c[3], tk, itk);
    if (c[4] != 0.0) v = v + quot(c[4], tk2, itk2);
    return v;
  }
};

// Per-cell SoA accessor
struct SoA {
  int64_t N;
  __device__ __forceinline__ int64_t at(int k, int64_t cell) const { return (int64_t)k * N + cell; }
};

}  // namespace pfgpu
