// pfgpu_prefactor.cuh -- kinetic-mineral rate prefactors, shared by the
// kernels that carry them (plain step kernel, global-implicit assembly).
//
// RKineticMineral (src/pflotran/reaction_mineral.F90): the rate of a mineral
// with prefactors is sum_p rate_p Arrhenius_p exp(ln_prefactor_p), each
// ln_prefactor_p a sum over its species of alpha ln a - ln(1 + K a^beta)
// (:820-851); the derivative adds, per prefactor species, dIm/d(species) to
// the Jacobian (:976-1070).  Written as the reference does, including two
// behaviours of its derivative: a secondary species' term goes to the rows of
// the complex's own species with the complex's stoichiometry (:1058-1066),
// and the complex's species count replaces the mineral's for the primary
// species that follow it in the same mineral (:1033-1046; network set-up
// refuses the orderings where that count would exceed the mineral's).
#pragma once

#include "pfgpu_common.cuh"

namespace pfgpu {

__device__ __forceinline__ int pf_slot(int m, int p, int s) {
  return (m * PF_MAX_PREFACTORS + p) * PF_MAX_PREFACTOR_SPECIES + s;
}

__device__ __forceinline__ double pf_arrhenius(double ea, double temp) {
  return ea > 0.0 ? exp(ea / IDEAL_GAS_CONSTANT * (1.0 / (25.0 + 273.15) - 1.0 / (temp + 273.15))) : 1.0;
}

// sum_prefactor_rate of mineral m, and prefactor(p), ln_prefactor_spec(s,p)
// for the derivative.  ln_act(j): ln activity of primary j; ln_sec_act(i):
// ln(m_i gamma_i) of complex i.
template <class LnAct, class LnSecAct>
__device__ double prefactor_rate(const Tables& T, int m, LnAct ln_act, LnSecAct ln_sec_act, double temp,
                                 double* prefactor, double (*lnps)[PF_MAX_PREFACTOR_SPECIES]) {
  double sum = 0.0;
  const int np = T.pf_cnt(m);
  for (int p = 0; p < np; ++p) {
    double ln_prefactor = 0.0;
    const int ns = T.pf_nsp(m, p);
    for (int s = 0; s < ns; ++s) {
      const int q = pf_slot(m, p, s), id = T.pf_id(q);
      const double la = id >= 0 ? ln_act(id) : ln_sec_act(-id - 1);
      const double ln_numerator = T.pf_alpha(q) * la;
      const double ln_denominator = log(1.0 + exp(log(T.pf_atten(q)) + T.pf_beta(q) * la));
      ln_prefactor = ln_prefactor + ln_numerator;
      ln_prefactor = ln_prefactor - ln_denominator;
      lnps[p][s] = ln_numerator - ln_denominator;
    }
    prefactor[p] = exp(ln_prefactor);
    sum = sum + prefactor[p] * T.pf_rate(m, p) * pf_arrhenius(T.pf_ea(m, p), temp);
  }
  return sum;
}

// The prefactor part of the mineral's Jacobian: add(row, col, v) adds v to
// J(row, col).  Im: the rate times the cell volume (mol/s); sum_rate,
// prefactor, lnps: from prefactor_rate.  pri_gam(j), sec_gam(i): activity
// coefficients; ln_conc(j) = ln m_j; sec_lnK(i): the constant part of
// complex i's ln Q/K, -logK ln10 at the cell's temperature plus its water
// term (:1048-1053).
template <class LnAct, class LnSecAct, class PriGam, class SecGam, class LnConc, class SecLnK, class Add>
__device__ void prefactor_derivative(const Tables& T, int m, double Im, double sum_rate, const double* prefactor,
                                     const double (*lnps)[PF_MAX_PREFACTOR_SPECIES], LnAct ln_act,
                                     LnSecAct ln_sec_act, PriGam pri_gam, SecGam sec_gam, LnConc ln_conc,
                                     SecLnK sec_lnK, double temp, Add add) {
  const double dIm_dsum_prefactor_rate = Im / sum_rate;
  const int mb = T.mnrl_begin(m);
  int ncomp = T.mnrl_end(m) - mb;  // the count the primary species below walk
  const int np = T.pf_cnt(m);
  for (int p = 0; p < np; ++p) {
    const double arrhenius_factor = pf_arrhenius(T.pf_ea(m, p), temp);
    const double ln_prefactor = log(prefactor[p]);
    const int ns = T.pf_nsp(m, p);
    for (int s = 0; s < ns; ++s) {
      const int q = pf_slot(m, p, s), id = T.pf_id(q);
      const double dprefactor_dprefactor_spec = exp(ln_prefactor - lnps[p][s]);
      double la, gam;
      if (id >= 0) {
        la = ln_act(id);
        gam = pri_gam(id);
      } else {
        la = ln_sec_act(-id - 1);
        gam = sec_gam(-id - 1);
      }
      const double dnum = T.pf_alpha(q) * exp(lnps[p][s] - la);
      const double ln_gam_m_beta = T.pf_beta(q) * la;
      const double denominator = 1.0 + exp(log(T.pf_atten(q)) + ln_gam_m_beta);
      const double dden =
          -1.0 * exp(lnps[p][s]) / denominator * T.pf_atten(q) * T.pf_beta(q) * exp(ln_gam_m_beta - la);
      double dspec = dnum + dden;
      dspec = dspec * gam;
      const double dIm_dspec =
          dIm_dsum_prefactor_rate * dprefactor_dprefactor_spec * dspec * T.pf_rate(m, p) * arrhenius_factor;
      if (id >= 0) {
        for (int i = 0; i < ncomp; ++i) add(T.mnrl_idx(mb + i), id, T.mnrl_nu(mb + i) * dIm_dspec);
      } else {
        const int icplx = -id - 1, cb = T.sec_begin(icplx);
        double lnQK = sec_lnK(icplx);
        ncomp = T.sec_end(icplx) - cb;
        for (int i = 0; i < ncomp; ++i) lnQK = lnQK + T.sec_nu(cb + i) * ln_act(T.sec_idx(cb + i));
        for (int j = 0; j < ncomp; ++j) {
          const int jc = T.sec_idx(cb + j);
          const double tempreal = T.sec_nu(cb + j) * exp(lnQK - ln_conc(jc)) / sec_gam(icplx);
          for (int i = 0; i < ncomp; ++i) add(T.sec_idx(cb + i), jc, T.sec_nu(cb + i) * tempreal * dIm_dspec);
        }
      }
    }
  }
}

}  // namespace pfgpu
