// rxn_oracle.hpp -- CPU restatement of PFLOTRAN's per-cell geochemistry.
//
// TEST INFRASTRUCTURE ONLY.  This is the oracle the GPU engine is checked
// against; nothing in the product links or calls it.  Only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline and reference legs use it.
//
// Every routine restates one reference subroutine, in the same loop order and
// with the same left-to-right evaluation of each Fortran expression, so that
// rounding follows the reference as closely as a C++ compiler allows
// (built with -ffp-contract=off: no FMA contraction on either host).
// File:line citations are to src/pflotran/ of fmyuan/pflotran-elm-interface.
//
// Pinning: the restatement is checked against the reference's own regression
// gold files (regression_tests/ascem/batch/*.regression.gold, tolerances from
// batch.cfg:20-27) and the pFUnit pin of the water density
// (src/pflotran/unittests/test_eos_water.pf:146-157); see tests/test_oracle_kat.py.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>

#include "../include/pfgpu.h"

namespace oracle {

// pflotran_constants.F90:84 (truncated, not ln 10) and :89
constexpr double LOG_TO_LN = 2.30258509299;
constexpr double IDEAL_GAS_CONSTANT = 8.31446;
// reactive_transport_aux.F90:19
constexpr double rt_min_saturation = 1.0e-40;
// pflotran_constants.F90:76,80
constexpr double H2O_CRITICAL_TEMPERATURE = 647.3;
constexpr double H2O_CRITICAL_PRESSURE = 22.064e6;

constexpr int MAXN = PF_MAX_NCOMP;
constexpr int MAXS = PF_MAX_NSEC;
constexpr int MAXM = PF_MAX_NMNRL;

// Fortran SIGN(1.d0, x): +1 for x >= +0, -1 for x < 0 (and for -0.0).
inline double fsign1(double x) { return std::signbit(x) ? -1.0 : 1.0; }

// Per-cell working copy of rt_auxvar + global_auxvar + material_auxvar
// (reactive_transport_aux.F90:21-74, global_aux.F90:11-35,
//  material_aux.F90:53-77), plus the per-cell logK the reference keeps in the
// shared reaction object (reaction.F90:5976-6069 mutates it per cell).
struct Cell {
  double pri_molal[MAXN];
  double total[MAXN];
  double dtotal[MAXN * MAXN];  // dtotal(i,j) = dtotal[i*MAXN + j]
  double pri_act_coef[MAXN];
  double sec_act_coef[MAXS];
  double sec_molal[MAXS];
  double mnrl_volfrac[MAXM];
  double mnrl_area[MAXM];
  double mnrl_rate[MAXM];
  double porosity, sat, den_kg, volume, temp;
  double ln_act_h2o;
  double sec_logK[MAXS];
  double mnrl_logK[MAXM];
  int ierror;  // option%ierror side channel (activity-coefficient failure)
  // sorption (reactive_transport_aux.F90:21-74: total_sorb_eq, dtotal_sorb_eq,
  // eqionx_ref_cation_sorbed_conc)
  double total_sorb[MAXN];
  double dtotal_sorb[MAXN * MAXN];
  double ionx_ref[PF_MAX_NIONX];
  // surface complexation: srfcplxrxn_free_site_conc, eqsrfcplx_conc
  double srf_free[PF_MAX_NSRFCPLX_RXN];
  double srf_conc[PF_MAX_NSRFCPLX];
};

struct Net {
  const PfNetworkDesc* d;
  PfOptions o;
  int n, ns, nm;
  int sid(int i, int s) const { return d->sec_spec[i * d->sec_stride + s]; }
  double sst(int i, int s) const { return d->sec_stoich[i * d->sec_stride + s]; }
  int mid(int m, int s) const { return d->mnrl_spec[m * d->mnrl_stride + s]; }
  double mst(int m, int s) const { return d->mnrl_stoich[m * d->mnrl_stride + s]; }
  const PfSorptionDesc* sorb;  // null: no sorption
  const PfPrefactorDesc* pref;  // null: no rate prefactors
  explicit Net(const PfNetworkDesc* desc) : d(desc), o(desc->opts), n(desc->ncomp),
      ns(desc->nsec), nm(desc->nmnrl),
      sorb(desc->sorption && (desc->sorption->nkd > 0 || desc->sorption->nionx > 0 || desc->sorption->nsrfcplx_rxn > 0) ? desc->sorption
                                                                                      : nullptr),
      pref(desc->prefactors) {}
  // kinmnrl_num_prefactors, kinmnrl_prefactor_id(0,p,m) and the per-prefactor
  // and per-species arrays (dense [nm][MP] and [nm][MP][MS], 0-based)
  int npref(int m) const { return pref ? pref->num_prefactors[m] : 0; }
  // eqcplxh2ostoich / kinmnrlh2ostoich (0: no water in the reaction)
  double h2o_sec(int i) const { return d->sec_h2o_stoich ? d->sec_h2o_stoich[i] : 0.0; }
  double h2o_mnrl(int m) const { return d->mnrl_h2o_stoich ? d->mnrl_h2o_stoich[m] : 0.0; }
  int pidx(int m, int p) const { return m * PF_MAX_PREFACTORS + p; }
  int psidx(int m, int p, int s) const { return (m * PF_MAX_PREFACTORS + p) * PF_MAX_PREFACTOR_SPECIES + s; }
};

// ReactionInterpolateLogK, reaction_aux.F90:1285-1312 (the coefficient type
// is a parameter so that a counting build can read the network's doubles)
template <class Coef>
inline void interpolate_logK(const Coef* coefs, double* logKs, double temp, int n) {
  double temp_kelvin = temp + 273.15;
  for (int i = 0; i < n; ++i) {
    const Coef* c = coefs + 5 * i;
    logKs[i] = c[0] * std::log(temp_kelvin) + c[1] + c[2] * temp_kelvin +
               c[3] / temp_kelvin + c[4] / (temp_kelvin * temp_kelvin);
  }
}

// Per-cell logK: isothermal -> the network's reference-temperature values;
// otherwise RUpdateTempDependentCoefs (reaction.F90:5976-6069) and
// MineralUpdateTempDepCoefs (reaction_mineral.F90:1306-1357).
inline void set_logK(const Net& net, Cell& c) {
  if (net.o.isothermal || !net.d->sec_logKcoef) {
    for (int i = 0; i < net.ns; ++i) c.sec_logK[i] = net.d->sec_logK[i];
  } else {
    interpolate_logK(net.d->sec_logKcoef, c.sec_logK, c.temp, net.ns);
  }
  if (net.o.isothermal || !net.d->mnrl_logKcoef) {
    for (int m = 0; m < net.nm; ++m) c.mnrl_logK[m] = net.d->mnrl_logK[m];
  } else {
    interpolate_logK(net.d->mnrl_logKcoef, c.mnrl_logK, c.temp, net.nm);
  }
}

// ln a_H2O from the molalities' sum, reaction.F90:4537-4547 and 4604-4611
inline void water_activity(Cell& c, double sum_pri_molal, double sum_sec_molal) {
  c.ln_act_h2o = 1.0 - 0.017 * (sum_pri_molal + sum_sec_molal);
  if (c.ln_act_h2o > 0.0) c.ln_act_h2o = std::log(c.ln_act_h2o);
  else c.ln_act_h2o = 0.0;
}

// RActivityCoefficients, reaction.F90:4368-4614 (no water primary species:
// sum_pri_molal is over all primaries, :4394-4400)
inline void activity_coefficients(const Net& net, Cell& c) {
  const PfNetworkDesc* d = net.d;
  const double A = d->debyeA, B = d->debyeB, Bdot = d->debyeBdot;
  const bool h2o = net.o.use_activity_h2o != 0;
  double sum_pri_molal = 0.0;
  if (h2o)
    for (int j = 0; j < net.n; ++j) sum_pri_molal = sum_pri_molal + c.pri_molal[j];
  if (net.o.act_coef_update_algorithm == PF_ACT_COEF_ALGO_NEWTON) {
    // reaction.F90:4403-4551
    double ln_conc[MAXN], ln_act[MAXN];
    for (int j = 0; j < net.n; ++j) {
      ln_conc[j] = std::log(c.pri_molal[j]);
      ln_act[j] = ln_conc[j] + std::log(c.pri_act_coef[j]);
    }
    double fpri = 0.0;
    for (int j = 0; j < net.n; ++j)
      fpri = fpri + c.pri_molal[j] * d->pri_Z[j] * d->pri_Z[j];
    int it = 0;
    double II = 0.0, I, f, sqrt_I, den = 0.0;
    for (;;) {
      it = it + 1;
      if (it > 50) {
        for (int j = 0; j < net.n; ++j) { c.pri_molal[j] = NAN; c.pri_act_coef[j] = NAN; }
        for (int i = 0; i < net.ns; ++i) c.sec_act_coef[i] = NAN;
        c.ierror = 1;
        return;  // the reference keeps looping on NaN until |I-II| test fails; bounded here
      }
      I = fpri;
      for (int i = 0; i < net.ns; ++i)
        I = I + c.sec_molal[i] * d->sec_Z[i] * d->sec_Z[i];
      I = 0.5 * I;
      f = I;
      if (std::fabs(I - II) < 1.0e-6 * I) break;
      if (net.ns > 0) {
        double didi = 0.0;
        sqrt_I = std::sqrt(I);
        for (int i = 0; i < net.ns; ++i) {
          if (std::fabs(d->sec_Z[i]) > 0.0) {
            double t = 1.0 + B * d->sec_a0[i] * sqrt_I;
            double sum = 0.5 * A * d->sec_Z[i] * d->sec_Z[i] / (sqrt_I * (t * t)) - Bdot;
            int nsp = d->sec_nspec[i];
            for (int s = 0; s < nsp; ++s) {
              int j = net.sid(i, s);
              if (std::fabs(d->pri_Z[j]) > 0.0) {
                double tj = 1.0 + B * d->pri_a0[j] * sqrt_I;
                double dgamdi = -0.5 * A * (d->pri_Z[j] * d->pri_Z[j]) / (sqrt_I * (tj * tj)) + Bdot;
                sum = sum + net.sst(i, s) * dgamdi;
              }
            }
            double dcdi = c.sec_molal[i] * LOG_TO_LN * sum;
            didi = didi + 0.5 * d->sec_Z[i] * d->sec_Z[i] * dcdi;
          }
        }
        den = 1.0 - didi;
        if (std::fabs(den) > 0.0) II = (f - I * didi) / den;
        else II = f;
      } else {
        II = f;
      }
      if (II < 0.0) {
        for (int j = 0; j < net.n; ++j) { c.pri_molal[j] = NAN; c.pri_act_coef[j] = NAN; }
        for (int i = 0; i < net.ns; ++i) c.sec_act_coef[i] = NAN;
        c.ierror = 1;
        return;
      }
      I = II;
      sqrt_I = std::sqrt(I);
      for (int j = 0; j < net.n; ++j) {
        if (std::fabs(d->pri_Z[j]) > 0.0) {
          c.pri_act_coef[j] = std::exp((-d->pri_Z[j] * d->pri_Z[j] * sqrt_I * A /
                                        (1.0 + d->pri_a0[j] * B * sqrt_I) + Bdot * I) * LOG_TO_LN);
        } else {
          c.pri_act_coef[j] = 1.0;
        }
      }
      double sum_sec_molal = 0.0;
      for (int i = 0; i < net.ns; ++i) {
        if (std::fabs(d->sec_Z[i]) > 0.0) {
          c.sec_act_coef[i] = std::exp((-d->sec_Z[i] * d->sec_Z[i] * sqrt_I * A /
                                        (1.0 + d->sec_a0[i] * B * sqrt_I) + Bdot * I) * LOG_TO_LN);
        } else {
          c.sec_act_coef[i] = 1.0;
        }
        double lnQK = -c.sec_logK[i] * LOG_TO_LN;
        if (net.h2o_sec(i) != 0.0) lnQK = lnQK + net.h2o_sec(i) * c.ln_act_h2o;
        int nsp = d->sec_nspec[i];
        for (int s = 0; s < nsp; ++s) lnQK = lnQK + net.sst(i, s) * ln_act[net.sid(i, s)];
        c.sec_molal[i] = std::exp(lnQK) / c.sec_act_coef[i];
        sum_sec_molal = sum_sec_molal + c.sec_molal[i];
      }
      if (h2o) water_activity(c, sum_pri_molal, sum_sec_molal);
    }
    return;
  }
  // LAG algorithm, reaction.F90:4553-4612
  double I = 0.0;
  for (int j = 0; j < net.n; ++j) I = I + c.pri_molal[j] * d->pri_Z[j] * d->pri_Z[j];
  for (int i = 0; i < net.ns; ++i) I = I + c.sec_molal[i] * d->sec_Z[i] * d->sec_Z[i];
  I = 0.5 * I;
  double sqrt_I = std::sqrt(I);
  for (int j = 0; j < net.n; ++j) {
    if (std::fabs(d->pri_Z[j]) > 1.0e-10) {
      c.pri_act_coef[j] = std::exp((-d->pri_Z[j] * d->pri_Z[j] * sqrt_I * A /
                                    (1.0 + d->pri_a0[j] * B * sqrt_I) + Bdot * I) * LOG_TO_LN);
    } else {
      c.pri_act_coef[j] = 1.0;
    }
  }
  double sum_sec_molal = 0.0;
  for (int i = 0; i < net.ns; ++i) {
    if (std::fabs(d->sec_Z[i]) > 1.0e-10) {
      c.sec_act_coef[i] = std::exp((-d->sec_Z[i] * d->sec_Z[i] * sqrt_I * A /
                                    (1.0 + d->sec_a0[i] * B * sqrt_I) + Bdot * I) * LOG_TO_LN);
    } else {
      c.sec_act_coef[i] = 1.0;
    }
    sum_sec_molal = sum_sec_molal + c.sec_molal[i];
  }
  if (h2o) water_activity(c, sum_pri_molal, sum_sec_molal);
}

// RTotalAqueous, reaction.F90:4665-4759 (RTotal :4618 -> aqueous only).
inline void total_aqueous(const Net& net, Cell& c) {
  const PfNetworkDesc* d = net.d;
  const int n = net.n;
  double xmass = 1.0;
  double den_kg_per_L = c.den_kg * xmass * 1.0e-3;
  double ln_conc[MAXN], ln_act[MAXN];
  for (int j = 0; j < n; ++j) {
    ln_conc[j] = std::log(c.pri_molal[j]);
    ln_act[j] = ln_conc[j] + std::log(c.pri_act_coef[j]);
    c.total[j] = c.pri_molal[j];
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) c.dtotal[i * MAXN + j] = (i == j) ? 1.0 : 0.0;
  for (int i = 0; i < net.ns; ++i) {
    double lnQK = -c.sec_logK[i] * LOG_TO_LN;
    if (net.h2o_sec(i) != 0.0) lnQK = lnQK + net.h2o_sec(i) * c.ln_act_h2o;  // :4715-4717
    int nsp = d->sec_nspec[i];
    for (int s = 0; s < nsp; ++s) lnQK = lnQK + net.sst(i, s) * ln_act[net.sid(i, s)];
    c.sec_molal[i] = std::exp(lnQK) / c.sec_act_coef[i];
    for (int s = 0; s < nsp; ++s) {
      int k = net.sid(i, s);
      c.total[k] = c.total[k] + net.sst(i, s) * c.sec_molal[i];
    }
    for (int sj = 0; sj < nsp; ++sj) {
      int jc = net.sid(i, sj);
      double tempreal = net.sst(i, sj) * std::exp(lnQK - ln_conc[jc]) / c.sec_act_coef[i];
      for (int si = 0; si < nsp; ++si) {
        int ic = net.sid(i, si);
        c.dtotal[ic * MAXN + jc] = c.dtotal[ic * MAXN + jc] + net.sst(i, si) * tempreal;
      }
    }
  }
  for (int j = 0; j < n; ++j) c.total[j] = c.total[j] * den_kg_per_L;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) c.dtotal[i * MAXN + j] = c.dtotal[i * MAXN + j] * den_kg_per_L;
}

// RTotalSorbEqIonx, reaction.F90:4906-5140 (the "#if 1" implementation:
// Newton on the reference cation's K_D when the charges differ, :4964-5081;
// the closed form when they are all equal, :5083-5097).  Returns 1 after
// 20000 Newton iterations (the ierror branch, :4983-4986).
inline int total_sorb_eq_ionx(const Net& net, Cell& c) {
  const PfSorptionDesc* sd = net.sorb;
  const auto* Z = net.d->pri_Z;
  const double tol = 1.0e-12;
  for (int irxn = 0; irxn < sd->nionx; ++irxn) {
    const int ncat = sd->ionx_ncation[irxn];
    const int32_t* cat = sd->ionx_cation + irxn * sd->ionx_stride;
    const auto* kk = sd->ionx_k + irxn * sd->ionx_stride;
    const int mi = sd->ionx_mineral ? sd->ionx_mineral[irxn] : -1;
    double omega;
    if (mi >= 0)
      omega = std::max(sd->ionx_cec[irxn] * c.mnrl_volfrac[mi], 1.0e-40);
    else
      omega = sd->ionx_cec[irxn];
    // eqionx_rxn_Z_flag (reaction_database.F90:2905-2919)
    bool zflag = false;
    for (int i = 0; i < ncat && !zflag; ++i)
      for (int j = 0; j < ncat; ++j)
        if (std::fabs(Z[cat[i]] - Z[cat[j]]) > 0.1) { zflag = true; break; }
    double cation_X[PF_MAX_IONX_CATIONS];
    for (int j = 0; j < ncat; ++j) cation_X[j] = 0.0;
    if (zflag) {
      int icomp = cat[0];
      double ref_cation_conc = c.pri_molal[icomp] * c.pri_act_coef[icomp];
      double ref_cation_Z = Z[icomp];
      double ref_cation_k = kk[0];
      double ref_cation_X = ref_cation_Z * c.ionx_ref[irxn] / omega;
      bool one_more = false;
      double KDj = ref_cation_X / (ref_cation_k * ref_cation_conc);
      int it = 0;
      for (;;) {
        it = it + 1;
        if (it > 20000) return 1;
        ref_cation_X = KDj * (ref_cation_k * ref_cation_conc);
        cation_X[0] = ref_cation_X;
        double total = ref_cation_X;
        double dres_dKDj = 0.0;
        for (int j = 1; j < ncat; ++j) {
          icomp = cat[j];
          cation_X[j] = kk[j] * c.pri_molal[icomp] * c.pri_act_coef[icomp] * std::pow(KDj, Z[icomp] / ref_cation_Z);
          total = total + cation_X[j];
          dres_dKDj = dres_dKDj + cation_X[j] / KDj * Z[icomp];
        }
        dres_dKDj = dres_dKDj / ref_cation_Z + (ref_cation_k * ref_cation_conc);
        double res = 1.0 - total;
        if (one_more) break;
        double delta_KDj = res / dres_dKDj;
        KDj = KDj + delta_KDj;
        KDj = std::max(KDj, 1.0e-40);
        if (std::fabs(delta_KDj / KDj) < tol) one_more = true;
      }
      c.ionx_ref[irxn] = ref_cation_X * omega / ref_cation_Z;
    } else {
      double sumkm = 0.0;
      for (int j = 0; j < ncat; ++j) {
        const int icomp = cat[j];
        cation_X[j] = c.pri_molal[icomp] * c.pri_act_coef[icomp] * kk[j];
        sumkm = sumkm + cation_X[j];
      }
      for (int j = 0; j < ncat; ++j) cation_X[j] = cation_X[j] / sumkm;
    }
    double sumZX = 0.0;
    for (int i = 0; i < ncat; ++i) sumZX = sumZX + Z[cat[i]] * cation_X[i];
    for (int i = 0; i < ncat; ++i) {
      const int icomp = cat[i];
      const double tempreal1 = cation_X[i] * omega / Z[icomp];
      c.total_sorb[icomp] = c.total_sorb[icomp] + tempreal1;
      const double tempreal2 = Z[icomp] / sumZX;
      for (int j = 0; j < ncat; ++j) {
        const int jcomp = cat[j];
        if (i == j)
          c.dtotal_sorb[icomp * MAXN + jcomp] =
              c.dtotal_sorb[icomp * MAXN + jcomp] + tempreal1 * (1.0 - (tempreal2 * cation_X[j])) / c.pri_molal[jcomp];
        else
          c.dtotal_sorb[icomp * MAXN + jcomp] =
              c.dtotal_sorb[icomp * MAXN + jcomp] + (-tempreal1) * tempreal2 * cation_X[j] / c.pri_molal[jcomp];
      }
    }
  }
  return 0;
}

// RTotalSorbKD, reaction_isotherm.F90:273-359
inline void total_sorb_kd(const Net& net, Cell& c) {
  const PfSorptionDesc* sd = net.sorb;
  for (int irxn = 0; irxn < sd->nkd; ++irxn) {
    const int icomp = sd->kd_spec[irxn];
    const double molality = c.pri_molal[icomp];
    double kd_kgw_m3b;
    if (sd->kd_units == PF_KD_UNIT_MLW_GSOIL)
      kd_kgw_m3b = sd->kd_coeff[irxn] * c.den_kg * (1.0 - c.porosity) * sd->soil_particle_density * 1.0e-3;
    else
      kd_kgw_m3b = sd->kd_coeff[irxn];
    const int mi = sd->kd_mineral ? sd->kd_mineral[irxn] : -1;
    if (mi >= 0) kd_kgw_m3b = kd_kgw_m3b * (c.mnrl_volfrac[mi]);
    double res, dres_dc;
    switch (sd->kd_type[irxn]) {
      case PF_SORPTION_LINEAR:
        res = kd_kgw_m3b * molality;
        dres_dc = kd_kgw_m3b;
        break;
      case PF_SORPTION_LANGMUIR: {
        const double tempreal = kd_kgw_m3b * molality;
        res = tempreal * sd->kd_langmuir_b[irxn] / (1.0 + tempreal);
        dres_dc = res / molality - res / (1.0 + tempreal) * tempreal / molality;
        break;
      }
      case PF_SORPTION_FREUNDLICH: {
        const double one_over_n = 1.0 / sd->kd_freundlich_n[irxn];
        res = kd_kgw_m3b * std::pow(molality, one_over_n);
        dres_dc = res / molality * one_over_n;
        break;
      }
      default:
        res = 0.0;
        dres_dc = 0.0;
    }
    c.total_sorb[icomp] = c.total_sorb[icomp] + res;
    c.dtotal_sorb[icomp * MAXN + icomp] = c.dtotal_sorb[icomp * MAXN + icomp] + dres_dc;
  }
}

// RTotalSorb, reaction.F90:4783-4832 (RZeroSorb :4763-4779, then ion
// exchange, then K_D; no surface complexation, no dynamic K_D).  Returns the
// ion exchange's ierror.
// RTotalSorbEqSurfCplx1 (reaction_surf_complex.F90:641-900), every
// equilibrium surface complexation reaction in turn (RTotalSorbEqSurfCplx,
// :446-491): the free-site concentration from the site balance (Newton when
// a complex holds more than one site, tolerance 1e-12 on the relative change,
// damping 0.5 after 1000 iterations; otherwise the closed form), the
// complexes' concentrations, the sorbed totals and their derivative with
// respect to the free-ion molalities (the free site's response included).
// The complexes' logK follow the cell temperature like the others
// (RUpdateTempDependentCoefs, reaction.F90:6025-6030).
inline void total_sorb_eq_srfcplx(const Net& net, Cell& c) {
  const PfSorptionDesc* sd = net.sorb;
  const int n = net.n;
  double ln_act[MAXN];
  for (int i = 0; i < n; ++i) ln_act[i] = std::log(c.pri_molal[i]) + std::log(c.pri_act_coef[i]);  // :686-687
  double logK[PF_MAX_NSRFCPLX];
  for (int k = 0; k < sd->nsrfcplx; ++k) logK[k] = sd->srfcplx_logK[k];
  if (!net.o.isothermal && sd->srfcplx_logKcoef) interpolate_logK(sd->srfcplx_logKcoef, logK, c.temp, sd->nsrfcplx);
  for (int irxn = 0; irxn < sd->nsrfcplx_rxn; ++irxn) {
    const int k0 = sd->srfcplx_rxn_ptr[irxn], k1 = sd->srfcplx_rxn_ptr[irxn + 1];
    bool stoich_flag = false;  // srfcplxrxn_stoich_flag, reaction_database.F90:2801-2803
    for (int k = k0; k < k1; ++k) stoich_flag = stoich_flag || sd->srfcplx_free_site_stoich[k] > 1.0;
    double free_site_conc = std::max(c.srf_free[irxn], 1.0e-40);  // :691
    for (int k = k0; k < k1; ++k) c.srf_conc[k] = 0.0;
    double site_density;
    switch (sd->srfcplx_surf_type[irxn]) {
      case PF_SURF_MINERAL:
        site_density = sd->srfcplx_site_density[irxn] * c.mnrl_volfrac[sd->srfcplx_mineral[irxn]];
        break;
      case PF_SURF_ROCK:
        site_density = sd->srfcplx_site_density[irxn] * sd->soil_particle_density * (1.0 - c.porosity);
        break;
      default:
        site_density = sd->srfcplx_site_density[irxn];
    }
    if (site_density < 1.0e-40) {  // :728-737
      c.srf_free[irxn] = 0.0;
      continue;
    }
    bool one_more = false;
    int num_iterations = 0;
    double damping_factor = 1.0;
    for (;;) {  // :743-799
      num_iterations = num_iterations + 1;
      double total = free_site_conc;
      const double ln_free_site = std::log(free_site_conc);
      for (int k = k0; k < k1; ++k) {
        double lnQK = -logK[k] * LOG_TO_LN;
        if (sd->srfcplx_h2o_stoich && sd->srfcplx_h2o_stoich[k] != 0.0)
          lnQK = lnQK + sd->srfcplx_h2o_stoich[k] * c.ln_act_h2o;
        lnQK = lnQK + sd->srfcplx_free_site_stoich[k] * ln_free_site;
        for (int p = 0; p < sd->srfcplx_nspec[k]; ++p)
          lnQK = lnQK + sd->srfcplx_stoich[k * sd->srfcplx_stride + p] * ln_act[sd->srfcplx_spec[k * sd->srfcplx_stride + p]];
        c.srf_conc[k] = std::exp(lnQK);
        total = total + sd->srfcplx_free_site_stoich[k] * c.srf_conc[k];
      }
      if (one_more) break;
      if (stoich_flag) {
        const double res = site_density - total;
        double dres_dfree_site = 1.0;
        for (int k = k0; k < k1; ++k)
          dres_dfree_site = dres_dfree_site + sd->srfcplx_free_site_stoich[k] * c.srf_conc[k] / free_site_conc;
        const double dfree_site_conc = res / dres_dfree_site;
        if (num_iterations > 1000) damping_factor = 0.5;
        free_site_conc = free_site_conc + damping_factor * dfree_site_conc;
        if (std::fabs(dfree_site_conc / free_site_conc) < 1.0e-12) one_more = true;
      } else {
        total = total / free_site_conc;
        free_site_conc = site_density / total;
        one_more = true;
      }
    }
    c.srf_free[irxn] = free_site_conc;
    // derivative of the free site (:803-824)
    double dSx_dmi[MAXN];
    for (int i = 0; i < n; ++i) dSx_dmi[i] = 0.0;
    double tempreal = 0.0;
    for (int k = k0; k < k1; ++k) {
      for (int p = 0; p < sd->srfcplx_nspec[k]; ++p) {
        const int icomp = sd->srfcplx_spec[k * sd->srfcplx_stride + p];
        dSx_dmi[icomp] = dSx_dmi[icomp] +
                         sd->srfcplx_stoich[k * sd->srfcplx_stride + p] * sd->srfcplx_free_site_stoich[k] * c.srf_conc[k];
      }
      tempreal = tempreal + sd->srfcplx_free_site_stoich[k] * sd->srfcplx_free_site_stoich[k] * c.srf_conc[k];
    }
    tempreal = tempreal / free_site_conc;
    tempreal = tempreal + 1.0;
    for (int i = 0; i < n; ++i) dSx_dmi[i] = -dSx_dmi[i] / tempreal;
    for (int i = 0; i < n; ++i) dSx_dmi[i] = dSx_dmi[i] / c.pri_molal[i];
    // sorbed totals and their derivative (:846-893)
    for (int k = k0; k < k1; ++k) {
      const int nc = sd->srfcplx_nspec[k];
      const int* ids = sd->srfcplx_spec + k * sd->srfcplx_stride;
      auto nu = [&](int p) { return sd->srfcplx_stoich[k * sd->srfcplx_stride + p]; };
      for (int p = 0; p < nc; ++p) c.total_sorb[ids[p]] = c.total_sorb[ids[p]] + nu(p) * c.srf_conc[k];
      const double nui_Si_over_Sx = sd->srfcplx_free_site_stoich[k] * c.srf_conc[k] / free_site_conc;
      for (int q = 0; q < nc; ++q) {
        const int jcomp = ids[q];
        const double t = nu(q) * c.srf_conc[k] / c.pri_molal[jcomp] + nui_Si_over_Sx * dSx_dmi[jcomp];
        for (int p = 0; p < nc; ++p)
          c.dtotal_sorb[ids[p] * MAXN + jcomp] = c.dtotal_sorb[ids[p] * MAXN + jcomp] + nu(p) * t;
      }
    }
  }
}

inline int total_sorb(const Net& net, Cell& c) {
  for (int i = 0; i < net.n; ++i) {
    c.total_sorb[i] = 0.0;
    for (int j = 0; j < net.n; ++j) c.dtotal_sorb[i * MAXN + j] = 0.0;
  }
  if (net.sorb->nsrfcplx_rxn > 0) total_sorb_eq_srfcplx(net, c);
  if (net.sorb->nionx > 0 && total_sorb_eq_ionx(net, c) != 0) return 1;
  if (net.sorb->nkd > 0) total_sorb_kd(net, c);
  return 0;
}

// RTotal, reaction.F90:4618-4661: aqueous, then sorbed.  Returns ierror.
inline int total(const Net& net, Cell& c) {
  total_aqueous(net, c);
  return net.sorb ? total_sorb(net, c) : 0;
}

// RAccumulationSorb / RAccumulationSorbDerivative, reaction.F90:5144-5210
inline void accumulation_sorb(const Net& net, const Cell& c, double* res) {
  for (int j = 0; j < net.n; ++j) res[j] = res[j] + c.total_sorb[j] * c.volume;
}
inline void accumulation_sorb_derivative(const Net& net, const Cell& c, double dt, double* J) {
  const double v_t = c.volume / dt;
  for (int i = 0; i < net.n; ++i)
    for (int j = 0; j < net.n; ++j) J[i * MAXN + j] = J[i * MAXN + j] + c.dtotal_sorb[i * MAXN + j] * v_t;
}

// RTAccumulation, reaction.F90:5710-5771 (aqueous, single phase)
inline void accumulation(const Net& net, const Cell& c, double* res) {
  for (int j = 0; j < net.n; ++j) res[j] = 0.0;
  if (c.sat < rt_min_saturation) return;
  double psv_t = c.porosity * c.sat * 1000.0 * c.volume;
  for (int j = 0; j < net.n; ++j) res[j] = psv_t * c.total[j];
}

// RTAccumulationDerivative, reaction.F90:5775-5848. J(i,j) = J[i*MAXN+j]
inline void accumulation_derivative(const Net& net, const Cell& c, double dt, double* J) {
  const int n = net.n;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) J[i * MAXN + j] = 0.0;
  if (c.sat < rt_min_saturation) {
    for (int i = 0; i < n; ++i) J[i * MAXN + i] = 1.0;
    return;
  }
  double psvd_t = c.porosity * c.sat * 1000.0 * c.volume / dt;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) J[i * MAXN + j] = c.dtotal[i * MAXN + j] * psvd_t;
}

// RKineticMineral, reaction_mineral.F90:647-1078 (no solid solution, no water
// activity).  J may be null when !compute_derivative.  Rate prefactors
// (:820-858, derivative :976-1070) as written, two behaviours included:
// a secondary prefactor species' derivative goes to the rows of the
// complex's own species with the complex's stoichiometry (:1058-1066), and
// it reassigns ncomp, the count the later primary prefactor species of the
// same mineral then use for the mineral's species (:1046, :1033-1038; the
// networks where that count exceeds the mineral's are refused at set-up).
// ln_sec_act (:707-710) is formed only when a prefactor uses it.
inline void kinetic_mineral(const Net& net, Cell& c, double* Res, double* J,
                            bool compute_derivative) {
  const PfNetworkDesc* d = net.d;
  const PfPrefactorDesc* pf = net.pref;
  double ln_conc[MAXN], ln_act[MAXN];
  for (int j = 0; j < net.n; ++j) {
    ln_conc[j] = std::log(c.pri_molal[j]);
    ln_act[j] = ln_conc[j] + std::log(c.pri_act_coef[j]);
  }
  auto ln_sec_act = [&](int i) { return std::log(c.sec_molal[i]) + std::log(c.sec_act_coef[i]); };
  double prefactor[PF_MAX_PREFACTORS], ln_prefactor_spec[PF_MAX_PREFACTORS][PF_MAX_PREFACTOR_SPECIES];
  for (int m = 0; m < net.nm; ++m) c.mnrl_rate[m] = 0.0;
  for (int m = 0; m < net.nm; ++m) {
    double lnQK = -c.mnrl_logK[m] * LOG_TO_LN;
    if (net.h2o_mnrl(m) != 0.0) lnQK = lnQK + net.h2o_mnrl(m) * c.ln_act_h2o;  // reaction_mineral.F90:769-772
    int nsp = d->mnrl_nspec[m];
    for (int s = 0; s < nsp; ++s) lnQK = lnQK + net.mst(m, s) * ln_act[net.mid(m, s)];
    double QK = std::exp(lnQK);
    double affinity_factor;
    if (d->mnrl_Temkin_const) {
      if (d->mnrl_min_scale_factor)
        affinity_factor = 1.0 - std::pow(QK, 1.0 / (d->mnrl_min_scale_factor[m] * d->mnrl_Temkin_const[m]));
      else
        affinity_factor = 1.0 - std::pow(QK, 1.0 / d->mnrl_Temkin_const[m]);
    } else if (d->mnrl_min_scale_factor) {
      affinity_factor = 1.0 - std::pow(QK, 1.0 / d->mnrl_min_scale_factor[m]);
    } else {
      affinity_factor = 1.0 - QK;
    }
    double sign_ = fsign1(affinity_factor);
    double Im, Im_const, sum_prefactor_rate;
    if (c.mnrl_volfrac[m] > 0 || sign_ < 0.0) {
      if (d->mnrl_irreversible[m] == 1 && sign_ < 0.0) continue;
      if (d->mnrl_affinity_threshold[m] > 0.0) {
        if (sign_ < 0.0 && QK < d->mnrl_affinity_threshold[m]) continue;
      }
      if (d->mnrl_rate_limiter[m] > 0.0) {
        affinity_factor = affinity_factor / (1.0 + (1.0 - affinity_factor) / d->mnrl_rate_limiter[m]);
      }
      if (net.npref(m) > 0) {
        sum_prefactor_rate = 0.0;
        for (int p = 0; p < net.npref(m); ++p) {
          double ln_prefactor = 0.0;
          for (int s = 0; s < pf->nspec[net.pidx(m, p)]; ++s) {
            const int q = net.psidx(m, p, s), id = pf->spec[q];
            const double ln_spec_act = id >= 0 ? ln_act[id] : ln_sec_act(-id - 1);
            const double ln_numerator = pf->alpha[q] * ln_spec_act;
            const double ln_denominator =
                std::log(1.0 + std::exp(std::log(pf->atten_coef[q]) + pf->beta[q] * ln_spec_act));
            ln_prefactor = ln_prefactor + ln_numerator;
            ln_prefactor = ln_prefactor - ln_denominator;
            ln_prefactor_spec[p][s] = ln_numerator - ln_denominator;
          }
          prefactor[p] = std::exp(ln_prefactor);
          double arrhenius_factor = 1.0;
          if (pf->activation_energy[net.pidx(m, p)] > 0.0) {
            arrhenius_factor = std::exp(pf->activation_energy[net.pidx(m, p)] / IDEAL_GAS_CONSTANT *
                                        (1.0 / (25.0 + 273.15) - 1.0 / (c.temp + 273.15)));
          }
          sum_prefactor_rate = sum_prefactor_rate + prefactor[p] * pf->rate[net.pidx(m, p)] * arrhenius_factor;
        }
      } else {
        double arrhenius_factor = 1.0;
        if (d->mnrl_activation_energy[m] > 0.0) {
          arrhenius_factor = std::exp(d->mnrl_activation_energy[m] / IDEAL_GAS_CONSTANT *
                                      (1.0 / (25.0 + 273.15) - 1.0 / (c.temp + 273.15)));
        }
        sum_prefactor_rate = d->mnrl_rate_constant[m] * arrhenius_factor;
      }
      Im_const = -c.mnrl_area[m];
      if (d->mnrl_min_scale_factor) Im_const = Im_const / d->mnrl_min_scale_factor[m];
      if (d->mnrl_affinity_power) {
        Im = Im_const * sign_ * std::pow(std::fabs(affinity_factor), d->mnrl_affinity_power[m]) *
             sum_prefactor_rate;
      } else {
        Im = Im_const * sign_ * std::fabs(affinity_factor) * sum_prefactor_rate;
      }
      c.mnrl_rate[m] = Im;
    } else {
      continue;
    }
    Im_const = Im_const * c.volume;
    Im = Im * c.volume;
    for (int s = 0; s < nsp; ++s) {
      int k = net.mid(m, s);
      Res[k] = Res[k] + net.mst(m, s) * Im;
    }
    if (!compute_derivative) continue;
    double dIm_dQK;
    if (d->mnrl_affinity_power)
      dIm_dQK = -Im * d->mnrl_affinity_power[m] / std::fabs(affinity_factor);
    else
      dIm_dQK = -Im_const * sum_prefactor_rate;
    if (d->mnrl_Temkin_const) {
      if (d->mnrl_min_scale_factor)
        dIm_dQK = dIm_dQK * (1.0 / (d->mnrl_min_scale_factor[m] * d->mnrl_Temkin_const[m])) / QK *
                  (1.0 - affinity_factor);
      else
        dIm_dQK = dIm_dQK * (1.0 / d->mnrl_Temkin_const[m]) / QK * (1.0 - affinity_factor);
    } else if (d->mnrl_min_scale_factor) {
      dIm_dQK = dIm_dQK * (1.0 / d->mnrl_min_scale_factor[m]) / QK * (1.0 - affinity_factor);
    }
    if (d->mnrl_rate_limiter[m] <= 0.0) {
      for (int sj = 0; sj < nsp; ++sj) {
        int jc = net.mid(m, sj);
        double dQK_dCj = net.mst(m, sj) * QK * std::exp(-ln_conc[jc]);
        double dQK_dmj = dQK_dCj * c.den_kg * 1.0e-3;
        for (int si = 0; si < nsp; ++si) {
          int ic = net.mid(m, si);
          J[ic * MAXN + jc] = J[ic * MAXN + jc] + net.mst(m, si) * dIm_dQK * dQK_dmj;
        }
      }
    } else {
      double rl = d->mnrl_rate_limiter[m];
      double den = 1.0 + (1.0 - affinity_factor) / rl;
      for (int sj = 0; sj < nsp; ++sj) {
        int jc = net.mid(m, sj);
        double dQK_dCj = net.mst(m, sj) * QK * std::exp(-ln_conc[jc]);
        double dQK_dmj = dQK_dCj * c.den_kg * 1.0e-3;
        for (int si = 0; si < nsp; ++si) {
          int ic = net.mid(m, si);
          J[ic * MAXN + jc] = J[ic * MAXN + jc] +
                              net.mst(m, si) * dIm_dQK * (1.0 + QK / rl / den) * dQK_dmj / den;
        }
      }
    }
    if (net.npref(m) > 0) {
      const double dIm_dsum_prefactor_rate = Im / sum_prefactor_rate;
      int ncomp = nsp;  // reassigned by a secondary prefactor species below
      for (int p = 0; p < net.npref(m); ++p) {
        double arrhenius_factor = 1.0;
        if (pf->activation_energy[net.pidx(m, p)] > 0.0) {
          arrhenius_factor = std::exp(pf->activation_energy[net.pidx(m, p)] / IDEAL_GAS_CONSTANT *
                                      (1.0 / (25.0 + 273.15) - 1.0 / (c.temp + 273.15)));
        }
        const double ln_prefactor = std::log(prefactor[p]);
        for (int s = 0; s < pf->nspec[net.pidx(m, p)]; ++s) {
          const int q = net.psidx(m, p, s), id = pf->spec[q];
          const double dprefactor_dprefactor_spec = std::exp(ln_prefactor - ln_prefactor_spec[p][s]);
          double ln_spec_act, spec_act_coef;
          if (id >= 0) {
            ln_spec_act = ln_act[id];
            spec_act_coef = c.pri_act_coef[id];
          } else {
            ln_spec_act = ln_sec_act(-id - 1);
            spec_act_coef = c.sec_act_coef[-id - 1];
          }
          const double dnum = pf->alpha[q] * std::exp(ln_prefactor_spec[p][s] - ln_spec_act);
          const double ln_gam_m_beta = pf->beta[q] * ln_spec_act;
          const double denominator = 1.0 + std::exp(std::log(pf->atten_coef[q]) + ln_gam_m_beta);
          const double dden = -1.0 * std::exp(ln_prefactor_spec[p][s]) / denominator * pf->atten_coef[q] *
                              pf->beta[q] * std::exp(ln_gam_m_beta - ln_spec_act);
          double dprefactor_spec_dspec = dnum + dden;
          dprefactor_spec_dspec = dprefactor_spec_dspec * spec_act_coef;
          const double dIm_dspec = dIm_dsum_prefactor_rate * dprefactor_dprefactor_spec * dprefactor_spec_dspec *
                                   pf->rate[net.pidx(m, p)] * arrhenius_factor;
          if (id >= 0) {
            for (int i = 0; i < ncomp; ++i) {
              const int jc = net.mid(m, i);
              J[jc * MAXN + id] = J[jc * MAXN + id] + net.mst(m, i) * dIm_dspec;
            }
          } else {
            const int icplx = -id - 1;
            double lnQK2 = -c.sec_logK[icplx] * LOG_TO_LN;
            if (net.h2o_sec(icplx) != 0.0) lnQK2 = lnQK2 + net.h2o_sec(icplx) * c.ln_act_h2o;
            ncomp = d->sec_nspec[icplx];
            for (int i = 0; i < ncomp; ++i) lnQK2 = lnQK2 + net.sst(icplx, i) * ln_act[net.sid(icplx, i)];
            for (int j = 0; j < ncomp; ++j) {
              const int jc = net.sid(icplx, j);
              const double tempreal = net.sst(icplx, j) * std::exp(lnQK2 - ln_conc[jc]) / c.sec_act_coef[icplx];
              for (int i = 0; i < ncomp; ++i) {
                const int ic = net.sid(icplx, i);
                J[ic * MAXN + jc] = J[ic * MAXN + jc] + net.sst(icplx, i) * tempreal * dIm_dspec;
              }
            }
          }
        }
      }
    }
  }
}

// RReaction, reaction.F90:4059-4130 (kinetic minerals are the only kind in scope)
inline void reaction(const Net& net, Cell& c, double* Res, double* J, bool derivative) {
  if (c.sat < rt_min_saturation) return;
  if (net.nm > 0) kinetic_mineral(net, c, Res, J, derivative);
}

// RReactionDerivative, reaction.F90:4134-4240: the analytical branch, or with
// numerical = true the forward differences of :4176-4230 (each primary
// molality raised by 1e-5 of itself on a copy of the auxvars, RTotal, then
// RReaction; Res stays zero there, as in the reference)
constexpr double perturbation_tolerance = 1.0e-5;  // reaction.F90:41
inline void reaction_derivative(const Net& net, Cell& c, double* Res, double* J, bool numerical = false) {
  if (c.sat < rt_min_saturation) return;
  for (int i = 0; i < net.n; ++i) {
    Res[i] = 0.0;
    for (int j = 0; j < net.n; ++j) J[i * MAXN + j] = 0.0;
  }
  if (!numerical) {
    reaction(net, c, Res, J, true);
  } else {
    double Res_orig[MAXN], Res_pert[MAXN];
    for (int i = 0; i < net.n; ++i) Res_orig[i] = 0.0;
    reaction(net, c, Res_orig, nullptr, false);
    for (int jc = 0; jc < net.n; ++jc) {
      for (int i = 0; i < net.n; ++i) Res_pert[i] = 0.0;
      Cell cp = c;
      const double pert = cp.pri_molal[jc] * perturbation_tolerance;
      cp.pri_molal[jc] = cp.pri_molal[jc] + pert;
      total(net, cp);
      reaction(net, cp, Res_pert, nullptr, false);
      for (int ic = 0; ic < net.n; ++ic)
        J[ic * MAXN + jc] = J[ic * MAXN + jc] + (Res_pert[ic] - Res_orig[ic]) / pert;
    }
  }
  for (int i = 0; i < net.n; ++i)
    for (int j = 0; j < net.n; ++j)
      if (std::fabs(J[i * MAXN + j]) < 1.0e-40) J[i * MAXN + j] = 0.0;
}

// LUDecomposition1, utility.F90:597-688 (stop_on_error = false). A(i,j) = A[i*MAXN+j]
inline int lu_decomposition(double* A, int N, int* INDX) {
  const double tiny = 1.0e-20;
  double VV[MAXN];
  for (int i = 0; i < N; ++i) {
    double aamax = 0.0;
    for (int j = 0; j < N; ++j)
      if (std::fabs(A[i * MAXN + j]) > aamax) aamax = std::fabs(A[i * MAXN + j]);
    if (aamax <= 0.0) return 1;
    VV[i] = 1.0 / aamax;
  }
  for (int j = 0; j < N; ++j) {
    for (int i = 0; i < j; ++i) {
      double sum = A[i * MAXN + j];
      for (int k = 0; k < i; ++k) sum = sum - A[i * MAXN + k] * A[k * MAXN + j];
      A[i * MAXN + j] = sum;
    }
    double aamax = 0.0;
    int imax = j;  // the reference leaves imax unset if every dum is NaN
    for (int i = j; i < N; ++i) {
      double sum = A[i * MAXN + j];
      for (int k = 0; k < j; ++k) sum = sum - A[i * MAXN + k] * A[k * MAXN + j];
      A[i * MAXN + j] = sum;
      double dum = VV[i] * std::fabs(sum);
      if (dum >= aamax) { imax = i; aamax = dum; }
    }
    if (j != imax) {
      for (int k = 0; k < N; ++k) {
        double dum = A[imax * MAXN + k];
        A[imax * MAXN + k] = A[j * MAXN + k];
        A[j * MAXN + k] = dum;
      }
      VV[imax] = VV[j];
    }
    INDX[j] = imax;
    if (A[j * MAXN + j] == 0.0) A[j * MAXN + j] = tiny;
    if (j != N - 1) {
      double dum = 1.0 / A[j * MAXN + j];
      for (int i = j + 1; i < N; ++i) A[i * MAXN + j] = A[i * MAXN + j] * dum;
    }
  }
  return 0;
}

// LUBackSubstitution, utility.F90:692-735
inline void lu_back_substitution(const double* A, int N, const int* INDX, double* B) {
  int ii = -1;
  for (int i = 0; i < N; ++i) {
    int ll = INDX[i];
    double sum = B[ll];
    B[ll] = B[i];
    if (ii >= 0) {
      for (int j = ii; j < i; ++j) sum = sum - A[i * MAXN + j] * B[j];
    } else if (sum != 0.0) {
      ii = i;
    }
    B[i] = sum;
  }
  for (int i = N - 1; i >= 0; --i) {
    double sum = B[i];
    if (i < N - 1)
      for (int j = i + 1; j < N; ++j) sum = sum - A[i * MAXN + j] * B[j];
    B[i] = sum / A[i * MAXN + i];
  }
}

// RSolve, reaction.F90:5457-5516.  Back-substitutes (the branch at
// :5506-5512); with fork_literal the update is left untouched (the
// solve_error branch at :5501-5504 returns after the decomposition).
inline int rsolve(const double* Res, double* J, const double* conc, double* update, int n,
                  bool use_log_formulation, bool fork_literal) {
  double rhs[MAXN];
  int indices[MAXN];
  for (int i = 0; i < n; ++i) {
    double mx = 0.0;
    for (int j = 0; j < n; ++j) mx = std::max(mx, std::fabs(J[i * MAXN + j]));
    double norm = std::max(1.0, mx);
    norm = 1.0 / norm;
    rhs[i] = Res[i] * norm;
    for (int j = 0; j < n; ++j) J[i * MAXN + j] = J[i * MAXN + j] * norm;
  }
  if (use_log_formulation) {
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) J[i * MAXN + j] = J[i * MAXN + j] * conc[j];
  }
  int ierror = lu_decomposition(J, n, indices);
  if (ierror != 0) return ierror;
  if (fork_literal) return 0;
  lu_back_substitution(J, n, indices, rhs);
  for (int i = 0; i < n; ++i) update[i] = rhs[i];
  return 0;
}

// RUpdateKineticState -> MineralUpdateKineticState,
// reaction.F90:5935-5972, reaction_mineral.F90:1456-1525
inline void update_kinetic_state(const Net& net, Cell& c, double dt) {
  if (net.nm == 0) return;
  double res[MAXN];
  for (int j = 0; j < net.n; ++j) res[j] = 0.0;
  kinetic_mineral(net, c, res, nullptr, false);
  for (int m = 0; m < net.nm; ++m) {
    double delta_volfrac = c.mnrl_rate[m] * net.d->mnrl_molar_vol[m] * dt;
    c.mnrl_volfrac[m] = c.mnrl_volfrac[m] + delta_volfrac;
    if (c.mnrl_volfrac[m] < 0.0) c.mnrl_volfrac[m] = 0.0;
  }
}

// RReact, reaction.F90:3742-4055.  Returns ierror; *num_iterations as the
// reference counts them (the failing evaluation included).
inline int rreact(const Net& net, Cell& c, const double* guess, double dt, int* num_iterations) {
  const int n = net.n;
  const PfOptions& o = net.o;
  int ierror = 0;
  double fixed_accum[MAXN], initial_total[MAXN], residual[MAXN], update[MAXN];
  double J[MAXN * MAXN];
  double prev_solution[MAXN], latest_solution[MAXN], conc[MAXN];
  double two_norm_r0 = 0.0;
  *num_iterations = 0;
  c.ierror = 0;
  set_logK(net, c);
  // the fixed accumulation holds the sorbed total of the last RTotal
  // (:3836-3839), restored or not after a failed RReact
  accumulation(net, c, fixed_accum);
  if (net.sorb) accumulation_sorb(net, c, fixed_accum);
  for (int j = 0; j < n; ++j) initial_total[j] = c.total[j];
  for (int j = 0; j < n; ++j) c.pri_molal[j] = guess[j];
  for (int j = 0; j < n; ++j) update[j] = 0.0;
  for (;;) {
    *num_iterations = *num_iterations + 1;
    if (o.act_coef_update_frequency == PF_ACT_COEF_NEWTON_ITER) activity_coefficients(net, c);
    // RTAuxVarCompute; a failed ion-exchange solve fails RReact (:3861-3865)
    if (total(net, c) != 0) return 1;
    if (*num_iterations > o.maximum_reaction_iterations) {
      ierror = 1;
      for (int j = 0; j < n; ++j) c.total[j] = initial_total[j];
      return ierror;
    }
    accumulation(net, c, residual);
    accumulation_derivative(net, c, dt, J);
    if (net.sorb) {
      accumulation_sorb(net, c, residual);
      accumulation_sorb_derivative(net, c, dt, J);
    }
    for (int j = 0; j < n; ++j) residual[j] = (residual[j] - fixed_accum[j]) / dt;
    reaction(net, c, residual, J, true);
    if (c.ierror != 0) return c.ierror;
    double dot = 0.0;
    for (int j = 0; j < n; ++j) dot = dot + residual[j] * residual[j];
    double two_norm_r = std::sqrt(dot);
    if (*num_iterations == 1) two_norm_r0 = two_norm_r;
    double rel_residual = two_norm_r / two_norm_r0;
    double maxabs = 0.0;
    for (int j = 0; j < n; ++j) maxabs = std::max(maxabs, std::fabs(residual[j]));
    if (maxabs < o.max_residual_tolerance) break;
    if (rel_residual < o.max_rel_residual_tolerance) break;
    for (int j = 0; j < n; ++j) conc[j] = c.pri_molal[j];
    int solve_error = rsolve(residual, J, conc, update, n, o.use_log_formulation != 0,
                             o.fork_literal_rsolve != 0);
    if (solve_error != 0) { ierror = 1; return ierror; }
    for (int j = 0; j < n; ++j) prev_solution[j] = c.pri_molal[j];
    if (o.use_log_formulation) {
      for (int j = 0; j < n; ++j) {
        update[j] = fsign1(update[j]) * std::min(std::fabs(update[j]), o.max_dlnC_rreact);
        latest_solution[j] = prev_solution[j] * std::exp(-update[j]);
      }
    } else {
      double min_ratio = 1.7976931348623157e308;
      for (int j = 0; j < n; ++j) {
        if (prev_solution[j] <= update[j]) {
          double ratio = std::fabs(prev_solution[j] / update[j]);
          if (ratio < min_ratio) min_ratio = ratio;
        }
      }
      if (min_ratio < 1.0)
        for (int j = 0; j < n; ++j) update[j] = update[j] * min_ratio * 0.99;
      for (int j = 0; j < n; ++j) latest_solution[j] = prev_solution[j] - update[j];
    }
    double max_rel = 0.0;
    for (int j = 0; j < n; ++j)
      max_rel = std::max(max_rel, std::fabs((latest_solution[j] - prev_solution[j]) / prev_solution[j]));
    if (max_rel < o.max_relative_change_tolerance) break;
    for (int j = 0; j < n; ++j) c.pri_molal[j] = latest_solution[j];
  }
  total(net, c);  // "one last update", reaction.F90:4051-4052
  return ierror;
}

// Single-cell implicit step as a converged Newton solve: the residual and
// Jacobian of RReact (reaction.F90:3899-3916), the global-implicit log update
// with the dlnC clip of PMRTCheckUpdatePre (pm_rt.F90:857-963), and every
// update applied before the convergence test (the SNES order), iterating until
// the applied relative change is below rel_tol.  Emulates one GIRT step of a
// one-cell problem without transport (the batch regression decks).
inline int implicit_step(const Net& net, Cell& c, double dt, double rel_tol, int max_its,
                         int* num_iterations) {
  const int n = net.n;
  double fixed_accum[MAXN], residual[MAXN], update[MAXN], J[MAXN * MAXN], conc[MAXN];
  set_logK(net, c);
  accumulation(net, c, fixed_accum);
  if (net.sorb) accumulation_sorb(net, c, fixed_accum);
  *num_iterations = 0;
  for (;;) {
    *num_iterations += 1;
    if (net.o.act_coef_update_frequency == PF_ACT_COEF_NEWTON_ITER) activity_coefficients(net, c);
    if (total(net, c) != 0) return 1;
    accumulation(net, c, residual);
    accumulation_derivative(net, c, dt, J);
    if (net.sorb) {
      accumulation_sorb(net, c, residual);
      accumulation_sorb_derivative(net, c, dt, J);
    }
    for (int j = 0; j < n; ++j) residual[j] = (residual[j] - fixed_accum[j]) / dt;
    reaction(net, c, residual, J, true);
    for (int j = 0; j < n; ++j) conc[j] = c.pri_molal[j];
    if (rsolve(residual, J, conc, update, n, true, false) != 0) return 1;
    double max_rel = 0.0;
    for (int j = 0; j < n; ++j) {
      update[j] = fsign1(update[j]) * std::min(std::fabs(update[j]), 5.0);
      double nv = c.pri_molal[j] * std::exp(-update[j]);
      max_rel = std::max(max_rel, std::fabs((nv - c.pri_molal[j]) / c.pri_molal[j]));
      c.pri_molal[j] = nv;
    }
    if (max_rel < rel_tol) break;
    if (*num_iterations >= max_its) return 1;
  }
  total(net, c);
  return 0;
}

struct StepResult {
  int ierror;
  int num_iterations;
  int num_sub_steps;
  int num_kinetic_state_updates;
};

// RStep, reaction.F90:3564-3738 (use_full_geochemistry, no immobile species).
inline StepResult rstep(const Net& net, Cell& c, double* guess, double tran_dt) {
  const int n = net.n;
  StepResult r{0, 0, 0, 0};
  bool small[MAXN];
  double small_val[MAXN];
  for (int i = 0; i < n; ++i) {
    small[i] = false;
    if (c.total[i] <= 1.0e-40) {
      small[i] = true;
      small_val[i] = c.total[i];
      c.total[i] = 1.0e-40;
    }
  }
  if (net.o.use_total_as_guess)
    for (int i = 0; i < n; ++i) guess[i] = c.total[i];
  double target_time = tran_dt;
  double cumulative_time = 0.0;
  double dt = tran_dt;
  int num_constant_timesteps_after_cut = 0;
  int num_cuts = 0;
  for (;;) {
    if (cumulative_time >= target_time) break;
    int inner = 0;
    int ierror = rreact(net, c, guess, dt, &inner);
    r.num_iterations += inner;
    if (ierror != 0) {
      num_cuts = num_cuts + 1;
      if (num_cuts > net.o.maximum_reaction_cuts) {
        r.ierror = 1;
        return r;
      }
      dt = 0.5 * dt;
      num_constant_timesteps_after_cut = 0;
    } else {
      update_kinetic_state(net, c, dt);
      if (net.nm > 0) r.num_kinetic_state_updates += 1;
      cumulative_time = cumulative_time + dt;
      r.num_sub_steps += 1;
      num_constant_timesteps_after_cut += 1;
      for (int i = 0; i < n; ++i) guess[i] = c.pri_molal[i];
      if (num_constant_timesteps_after_cut >= 4) {
        num_cuts = num_cuts - 1;
        dt = std::min(2.0 * dt, target_time - cumulative_time);
      }
    }
  }
  for (int i = 0; i < n; ++i)
    if (small[i]) c.total[i] = small_val[i];
  return r;
}

// EOSWaterDensityIFC67 (density only), eos_water.F90:1583-1748.  The 1967
// IFC industrial formulation; its published coefficients are a table that has
// to be the same as the reference's.
inline double ifc67_density(double t, double p) {
  static const double aa[23] = {
      6.824687741e03, -5.422063673e02, -2.096666205e04, 3.941286787e04,
      -6.733277739e04, 9.902381028e04, -1.093911774e05, 8.590841667e04,
      -4.511168742e04, 1.418138926e04, -2.017271113e03, 7.982692717e00,
      -2.616571843e-2, 1.522411790e-3, 2.284279054e-2, 2.421647003e02,
      1.269716088e-10, 2.074838328e-7, 2.174020350e-8, 1.105710498e-9,
      1.293441934e01, 1.308119072e-5, 6.047626338e-14};
  const double a1 = 8.438375405e-1, a2 = 5.362162162e-4, a3 = 1.720000000e00,
               a4 = 7.342278489e-2, a5 = 4.975858870e-2, a6 = 6.537154300e-1,
               a7 = 1.150000000e-6, a8 = 1.510800000e-5, a9 = 1.418800000e-1,
               a10 = 7.002753165e00, a11 = 2.995284926e-4, a12 = 2.040000000e-1;
  const double tc1 = H2O_CRITICAL_TEMPERATURE, pc1 = H2O_CRITICAL_PRESSURE;
  const double vc1 = 0.00317;
  const double utc1 = 1.0 / tc1, upc1 = 1.0 / pc1;
  double theta = (t + 273.15) * utc1;
  double theta2x = theta * theta;
  double theta18 = std::pow(theta, 18.0);
  double theta20 = theta18 * theta2x;
  double beta = p * upc1;
  double beta2x = beta * beta;
  double yy = 1.0 - a1 * theta2x - a2 * std::pow(theta, -6.0);
  double xx = a3 * yy * yy - 2.0 * (a4 * theta - a5 * beta);
  if (xx > 0.0) xx = std::sqrt(xx);
  else xx = 1.0e-6;
  double zz = yy + xx;
  double u0 = -5.0 / 17.0;
  double u1 = aa[11] * a5 * std::pow(zz, u0);
  double u2 = 1.0 / (a8 + std::pow(theta, 11.0));
  double u3 = aa[17] + (2.0 * aa[18] + 3.0 * aa[19] * beta) * beta;
  double u4 = 1.0 / (a7 + theta18 * theta);
  double u5 = std::pow(a10 + beta, -4.0);
  double u6 = a11 - 3.0 * u5;
  double u7 = aa[20] * theta18 * (a9 + theta2x);
  double u8 = aa[15] * std::pow(a6 - theta, 9.0);
  double vr = u1 + aa[12] + theta * (aa[13] + aa[14] * theta) + u8 * (a6 - theta) +
              aa[16] * u4 - u2 * u3 - u6 * u7 +
              (3.0 * aa[21] * (a12 - theta) + 4.0 * aa[22] * beta / theta20) * beta2x;
  return 1.0 / (vr * vc1);
}

// Constraint types (transport_constraint_rt.F90:22-34 subset)
enum { CON_TOTAL = 1, CON_FREE = 2, CON_PH = 3, CON_CHARGE_BAL = 4, CON_LOG = 5, CON_MINERAL = 6, CON_GAS = 7 };

// ReactionEquilibrateConstraint, reaction.F90:1328-2115, for the
// TOTAL/FREE/LOG/PH/CHARGE_BAL/MINERAL/GAS subset with no sorption
// (initialize_with_molality = false, use_prev_soln_as_guess as given).
// creact[i]: the mineral or gas reaction of a MINERAL/GAS row (:1755-1811);
// its logK follows the cell temperature in non-isothermal runs
// (RUpdateTempDependentCoefs at :1482-1484).
// Returns the iteration count, or -1 when the iteration limit is reached /
// a concentration goes non-positive / the decomposition is singular.
inline int equilibrate_constraint(const Net& net, Cell& c, const int* ctype,
                                  const double* cconc, bool use_prev_soln_as_guess,
                                  const PfConstraintReaction* creact = nullptr,
                                  int max_iterations = 10000) {
  const PfNetworkDesc* d = net.d;
  const int n = net.n;
  double xmass = 1.0;
  double convert_molal_to_molar = 1.0;
  double convert_molar_to_molal = 1000.0 / c.den_kg / xmass;
  set_logK(net, c);
  double free_conc[MAXN], total_conc[MAXN];
  for (int i = 0; i < n; ++i) free_conc[i] = use_prev_soln_as_guess ? c.pri_molal[i] : 1.0e-9;
  for (int i = 0; i < n; ++i) {
    total_conc[i] = 0.0;
    switch (ctype[i]) {
      case CON_TOTAL: total_conc[i] = cconc[i] * convert_molal_to_molar; break;
      case CON_FREE: free_conc[i] = cconc[i] * convert_molar_to_molal; break;
      case CON_LOG: free_conc[i] = std::pow(10.0, cconc[i]) * convert_molar_to_molal; break;
      case CON_CHARGE_BAL:
        if (!use_prev_soln_as_guess) free_conc[i] = cconc[i] * convert_molar_to_molal;
        break;
      case CON_PH: free_conc[i] = std::pow(10.0, -cconc[i]); break;
      case CON_MINERAL:
        if (!use_prev_soln_as_guess) free_conc[i] = cconc[i] * convert_molar_to_molal;  // guess
        break;
      case CON_GAS:  // partial pressure (bar); log10 form when <= 0
        total_conc[i] = cconc[i] <= 0.0 ? std::pow(10.0, cconc[i]) : cconc[i];
        break;
      default: return -1;
    }
  }
  for (int i = 0; i < n; ++i) c.pri_molal[i] = free_conc[i];
  int num_iterations = 0, num_it_act_coef_turned_on = 0;
  bool compute_activity_coefs = use_prev_soln_as_guess;
  bool charge_balance_warning_flag = false;
  double Res[MAXN], J[MAXN * MAXN], update[MAXN], prev_molal[MAXN];
  for (;;) {
    for (int i = 0; i < n; ++i)
      if (ctype[i] == CON_FREE || ctype[i] == CON_LOG) c.pri_molal[i] = free_conc[i];
    if (net.o.act_coef_update_frequency != PF_ACT_COEF_OFF && compute_activity_coefs)
      activity_coefficients(net, c);
    total(net, c);  // RTotal without ierror (:1594): sorbed totals follow the iterate
    for (int i = 0; i < n * MAXN; ++i) J[i] = 0.0;
    for (int i = 0; i < n; ++i) {
      switch (ctype[i]) {
        case CON_TOTAL:
          Res[i] = c.total[i] - total_conc[i];
          for (int j = 0; j < n; ++j) J[i * MAXN + j] = c.dtotal[i * MAXN + j];
          break;
        case CON_FREE:
        case CON_LOG:
          Res[i] = 0.0;
          for (int j = 0; j < n; ++j) J[i * MAXN + j] = 0.0;
          J[i * MAXN + i] = 1.0;
          break;
        case CON_CHARGE_BAL:
          Res[i] = 0.0;
          for (int j = 0; j < n; ++j) J[i * MAXN + j] = 0.0;
          for (int j = 0; j < n; ++j) {
            Res[i] = Res[i] + d->pri_Z[j] * c.total[j];
            for (int k = 0; k < n; ++k)
              J[i * MAXN + j] = J[i * MAXN + j] + d->pri_Z[k] * c.dtotal[k * MAXN + j];
          }
          if (c.pri_molal[i] < 1.0e-20 && !charge_balance_warning_flag) {
            if ((Res[i] > 0.0 && d->pri_Z[i] > 0.0) || (Res[i] < 0.0 && d->pri_Z[i] < 0.0)) {
              charge_balance_warning_flag = true;
              c.pri_molal[i] = (double)1.e-3f;  // the reference writes the single-precision literal 1.e-3
            }
          }
          break;
        case CON_PH:
          Res[i] = 0.0;
          for (int j = 0; j < n; ++j) J[i * MAXN + j] = 0.0;
          c.pri_molal[i] = std::pow(10.0, -cconc[i]) / c.pri_act_coef[i];
          J[i * MAXN + i] = 1.0;
          break;
        case CON_MINERAL:
        case CON_GAS: {
          const PfConstraintReaction& R = creact[i];
          double logK = R.logK;
          if (!net.o.isothermal && R.temperature_dependent) interpolate_logK(R.logKcoef, &logK, c.temp, 1);
          double lnQK = -logK * LOG_TO_LN;
          for (int p = 0; p < R.nspec; ++p)
            lnQK = lnQK + R.stoich[p] * std::log(c.pri_molal[R.spec[p]] * c.pri_act_coef[R.spec[p]]);
          Res[i] = ctype[i] == CON_MINERAL ? lnQK : lnQK - std::log(total_conc[i]);
          for (int j = 0; j < n; ++j) J[i * MAXN + j] = 0.0;
          for (int p = 0; p < R.nspec; ++p) J[i * MAXN + R.spec[p]] = R.stoich[p] / c.pri_molal[R.spec[p]];
          break;
        }
      }
    }
    double maximum_residual = 0.0;
    for (int i = 0; i < n; ++i) maximum_residual = std::max(maximum_residual, std::fabs(Res[i]));
    bool use_log_formulation;
    if (net.o.use_log_formulation) {
      if (num_iterations > 3 && num_iterations < 9)
        use_log_formulation = (num_iterations % 2 == 0);
      else
        use_log_formulation = true;
    } else {
      use_log_formulation = false;
    }
    double conc[MAXN];
    for (int i = 0; i < n; ++i) conc[i] = c.pri_molal[i];
    if (rsolve(Res, J, conc, update, n, use_log_formulation, false) != 0) return -1;
    for (int i = 0; i < n; ++i) prev_molal[i] = c.pri_molal[i];
    if (use_log_formulation) {
      for (int i = 0; i < n; ++i) {
        update[i] = fsign1(update[i]) * std::min(std::fabs(update[i]), 5.0);  // reaction%max_dlnC
        c.pri_molal[i] = c.pri_molal[i] * std::exp(-update[i]);
      }
    } else {
      double min_ratio = 1.7976931348623157e308;
      for (int i = 0; i < n; ++i) {
        if (prev_molal[i] <= update[i]) {
          double ratio = std::fabs(prev_molal[i] / update[i]);
          if (ratio < min_ratio) min_ratio = ratio;
        }
      }
      if (min_ratio <= 1.0)
        for (int i = 0; i < n; ++i) update[i] = update[i] * min_ratio * 0.99;
      for (int i = 0; i < n; ++i) c.pri_molal[i] = prev_molal[i] - update[i];
    }
    double mn = c.pri_molal[0];
    for (int i = 1; i < n; ++i) mn = std::min(mn, c.pri_molal[i]);
    if (!(mn > 0.0)) return -1;
    double maximum_relative_change = 0.0;
    for (int i = 0; i < n; ++i)
      maximum_relative_change =
          std::max(maximum_relative_change, std::fabs((c.pri_molal[i] - prev_molal[i]) / prev_molal[i]));
    num_iterations = num_iterations + 1;
    if (num_iterations >= max_iterations) return -1;
    if (maximum_residual < net.o.max_residual_tolerance &&
        maximum_relative_change < net.o.max_relative_change_tolerance) {
      if (compute_activity_coefs && num_iterations - num_it_act_coef_turned_on > 1) break;
      if (!compute_activity_coefs) num_it_act_coef_turned_on = num_iterations;
      compute_activity_coefs = true;
    }
  }
  return num_iterations;
}

// ---------------------------------------------------------------------------
// Global-implicit residual and Jacobian on a structured grid (config: 7-point
// stencil, zero-flux outer boundary, saturation 1, no dispersion beyond the
// longitudinal term).  Restates
//   RTResidualFlux   reactive_transport.F90:2052-2291 (internal connections)
//   RTResidualNonFlux                     :2293-2669 (accumulation, reaction)
//   RTJacobianFlux                        :2897-3086
//   RTJacobianNonFlux                     :3088-3349 (incl. log scaling :3316-3340,
//                                          MatDiagonalScaleLocal at :2879)
//   TDispersion/TFluxCoef/TFlux/TFluxDerivative transport.F90:52-609
// with the connection order of StructGridComputeInternConnect
// (grid_structured.F90:969-1011): x faces, then y, then z, each with k, j, i
// loops; every block is added in that order (ADD_VALUES), then accumulation,
// then reaction.  Cell index: i + nx*(j + ny*k).  Output BAIJ: block rows in
// cell order, block columns ascending, each bs x bs block column-major
// (PETSc SeqBAIJ storage).
struct GirtGrid {
  int nx, ny, nz;
  double dx, dy, dz;
  const double* qx;   // [nz][ny][nx-1]
  const double* qy;   // [nz][ny-1][nx]
  const double* qz;   // [nz-1][ny][nx]
  double diffusion;   // D_m, m^2/s
  double tortuosity;
  double dispersivity;  // longitudinal
};

// harmonic_tran_coefs_over_dist of TDispersion for one connection
inline double girt_tran_coef(const Cell& up, const Cell& dn, double q, double dist, double dfrac,
                             const GirtGrid& g) {
  double dist_up = dist * dfrac;
  double dist_dn = dist - dist_up;
  if (up.sat < rt_min_saturation || dn.sat < rt_min_saturation) return 0.0;
  double mech_up = g.dispersivity * std::fabs(q);
  double mech_dn = g.dispersivity * std::fabs(q);
  double hd_up = std::max(mech_up + 1.0 * up.sat * up.porosity * g.tortuosity * g.diffusion, 1.0e-40);
  double hd_dn = std::max(mech_dn + 1.0 * dn.sat * dn.porosity * g.tortuosity * g.diffusion, 1.0e-40);
  return (hd_up * hd_dn) / (hd_up * dist_dn + hd_dn * dist_up);
}

// r: [ncells*n] (block interleaved), values: [nnzb*n*n], rowptr/colidx: BAIJ
// pattern, fixed_total: totals at the previous time (accum_k = psv*total_k),
// fixed_sorb: sorbed totals at the previous time (accum_k += S_k*V,
// RTUpdateFixedAccumulation, reactive_transport.F90:1020-1031), used when
// the network has sorption.
inline void girt_assemble(const Net& net, Cell* cells, const GirtGrid& g, const double* fixed_total,
                          const double* fixed_sorb, double dt, const int* rowptr, const int* colidx, double* r,
                          double* values, bool numerical_derivatives = false) {
  const int n = net.n;
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  const long long N = (long long)nx * ny * nz;
  auto idx = [&](int i, int j, int k) { return (long long)i + (long long)nx * (j + (long long)ny * k); };
  for (long long c = 0; c < N; ++c) {
    set_logK(net, cells[c]);
    // RTUpdateAuxVars: RTotal without ierror (a failed ion-exchange solve is
    // reported and the run continues with the last iterate)
    total(net, cells[c]);
  }
  for (long long e = 0; e < N * n; ++e) r[e] = 0.0;
  const long long nnzb = rowptr[N];
  for (long long e = 0; e < nnzb * n * n; ++e) values[e] = 0.0;
  auto block = [&](long long row, long long col) -> double* {
    for (int b = rowptr[row]; b < rowptr[row + 1]; ++b)
      if (colidx[b] == col) return values + (long long)b * n * n;
    return nullptr;
  };
  // J(i,j) in column-major storage: blk[j*n + i]
  auto connection = [&](long long up, long long dn, double q, double area, double dist) {
    const Cell& cu = cells[up];
    const Cell& cd = cells[dn];
    double coef_up[MAXN], coef_dn[MAXN];
    double tran = girt_tran_coef(cu, cd, q, dist, 0.5, g);
    if (cd.sat < rt_min_saturation || cu.sat < rt_min_saturation) {
      for (int k = 0; k < n; ++k) coef_up[k] = coef_dn[k] = 0.0;
    } else {
      for (int k = 0; k < n; ++k) {
        double cup, cdn;
        if (q > 0.0) { cup = tran + q; cdn = -tran; }
        else { cup = tran; cdn = -tran + q; }
        coef_up[k] = cup * area * 1000.0;
        coef_dn[k] = cdn * area * 1000.0;
      }
    }
    double Res[MAXN];
    for (int k = 0; k < n; ++k) Res[k] = coef_up[k] * cu.total[k] + coef_dn[k] * cd.total[k];
    for (int k = 0; k < n; ++k) {
      r[up * n + k] = r[up * n + k] + Res[k];
      r[dn * n + k] = r[dn * n + k] - Res[k];
    }
    double* b_uu = block(up, up);
    double* b_ud = block(up, dn);
    double* b_dd = block(dn, dn);
    double* b_du = block(dn, up);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        double Jup = cu.dtotal[i * MAXN + j] * coef_up[i];
        double Jdn = cd.dtotal[i * MAXN + j] * coef_dn[i];
        b_uu[j * n + i] = b_uu[j * n + i] + Jup;
        b_ud[j * n + i] = b_ud[j * n + i] + Jdn;
        b_dd[j * n + i] = b_dd[j * n + i] + (-Jdn);
        b_du[j * n + i] = b_du[j * n + i] + (-Jup);
      }
  };
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx - 1; ++i)
        connection(idx(i, j, k), idx(i + 1, j, k), g.qx[((long long)k * ny + j) * (nx - 1) + i], g.dy * g.dz, g.dx);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny - 1; ++j)
      for (int i = 0; i < nx; ++i)
        connection(idx(i, j, k), idx(i, j + 1, k), g.qy[((long long)k * (ny - 1) + j) * nx + i], g.dx * g.dz, g.dy);
  for (int k = 0; k < nz - 1; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i)
        connection(idx(i, j, k), idx(i, j, k + 1), g.qz[((long long)k * ny + j) * nx + i], g.dx * g.dy, g.dz);
  // NonFlux: r = r - accum_k/dt; + accumulation/dt; + reaction
  for (long long c = 0; c < N; ++c) {
    Cell& cl = cells[c];
    double psv_t = cl.porosity * cl.sat * 1000.0 * cl.volume;
    for (int k = 0; k < n; ++k) {
      double accum_k = cl.sat < rt_min_saturation ? 0.0 : psv_t * fixed_total[(long long)k * N + c];
      if (net.sorb) accum_k = accum_k + fixed_sorb[(long long)k * N + c] * cl.volume;
      r[c * n + k] = r[c * n + k] - accum_k / dt;
    }
    double Res[MAXN];
    accumulation(net, cl, Res);
    if (net.sorb) accumulation_sorb(net, cl, Res);
    for (int k = 0; k < n; ++k) Res[k] = Res[k] / dt;
    for (int k = 0; k < n; ++k) r[c * n + k] = r[c * n + k] + Res[k];
  }
  for (long long c = 0; c < N; ++c) {
    double J[MAXN * MAXN];
    accumulation_derivative(net, cells[c], dt, J);
    if (net.sorb) accumulation_sorb_derivative(net, cells[c], dt, J);
    double* b = block(c, c);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) b[j * n + i] = b[j * n + i] + J[i * MAXN + j];
  }
  for (long long c = 0; c < N; ++c) {
    double Res[MAXN], J[MAXN * MAXN];
    for (int k = 0; k < n; ++k) Res[k] = 0.0;
    for (int e = 0; e < MAXN * MAXN; ++e) J[e] = 0.0;
    reaction(net, cells[c], Res, J, false);
    for (int k = 0; k < n; ++k) r[c * n + k] = r[c * n + k] + Res[k];
  }
  for (long long c = 0; c < N; ++c) {
    double Res[MAXN], J[MAXN * MAXN];
    for (int k = 0; k < n; ++k) Res[k] = 0.0;
    for (int e = 0; e < MAXN * MAXN; ++e) J[e] = 0.0;
    reaction_derivative(net, cells[c], Res, J, numerical_derivatives);
    double* b = block(c, c);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) b[j * n + i] = b[j * n + i] + J[i * MAXN + j];
  }
  // log formulation: right-scale every block column by the free-ion molality
  if (net.o.use_log_formulation) {
    for (long long row = 0; row < N; ++row)
      for (int b = rowptr[row]; b < rowptr[row + 1]; ++b) {
        const Cell& cc = cells[colidx[b]];
        double* blk = values + (long long)b * n * n;
        for (int j = 0; j < n; ++j)
          for (int i = 0; i < n; ++i) blk[j * n + i] = blk[j * n + i] * cc.pri_molal[j];
      }
  }
}

// The scalar operator-split transport matrix of RTCalculateTransportMatrix
// (reactive_transport.F90:1469-1703) on a structured grid: per internal
// connection (x, then y, then z; k, j, i loops) TFluxCoef's T_up, T_dn
// (transport.F90:495-565; flux only when both saturations reach
// rt_min_saturation) added at (up,up) += T_up, (up,dn) += T_dn, (dn,dn) -= T_dn,
// (dn,up) -= T_up; then psv/dt on the diagonal of every cell.  values follow
// the 7-point pattern rowptr/colidx (block size 1).  The right-hand side of
// the operator-split solve is psv*T_k/dt (RTCalculateRHS_t1 with no
// boundary or source terms).
inline void transport_matrix(const Cell* cells, const GirtGrid& g, double dt, const int* rowptr,
                             const int* colidx, double* values) {
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  const long long N = (long long)nx * ny * nz;
  auto idx = [&](int i, int j, int k) { return (long long)i + (long long)nx * (j + (long long)ny * k); };
  for (long long e = 0; e < rowptr[N]; ++e) values[e] = 0.0;
  auto at = [&](long long row, long long col) -> double& {
    for (int b = rowptr[row]; b < rowptr[row + 1]; ++b)
      if (colidx[b] == col) return values[b];
    return values[rowptr[row]];  // unreachable for the 7-point pattern
  };
  auto connection = [&](long long up, long long dn, double q, double area, double dist) {
    const Cell& cu = cells[up];
    const Cell& cd = cells[dn];
    double T_up = 0.0, T_dn = 0.0;
    if (!(cd.sat < rt_min_saturation) && !(cu.sat < rt_min_saturation)) {
      double tran = girt_tran_coef(cu, cd, q, dist, 0.5, g);
      double coef_up, coef_dn;
      if (q > 0.0) { coef_up = tran + q; coef_dn = -tran; }
      else { coef_up = tran; coef_dn = -tran + q; }
      T_up = coef_up * area * 1000.0;
      T_dn = coef_dn * area * 1000.0;
    }
    at(up, up) = at(up, up) + T_up;
    at(up, dn) = at(up, dn) + T_dn;
    at(dn, dn) = at(dn, dn) + (-T_dn);
    at(dn, up) = at(dn, up) + (-T_up);
  };
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx - 1; ++i)
        connection(idx(i, j, k), idx(i + 1, j, k), g.qx[((long long)k * ny + j) * (nx - 1) + i], g.dy * g.dz, g.dx);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny - 1; ++j)
      for (int i = 0; i < nx; ++i)
        connection(idx(i, j, k), idx(i, j + 1, k), g.qy[((long long)k * (ny - 1) + j) * nx + i], g.dx * g.dz, g.dy);
  for (int k = 0; k < nz - 1; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i)
        connection(idx(i, j, k), idx(i, j, k + 1), g.qz[((long long)k * ny + j) * nx + i], g.dx * g.dy, g.dz);
  for (long long c = 0; c < N; ++c) {
    const Cell& cl = cells[c];
    const double coef = cl.porosity * cl.sat * 1000.0 * cl.volume / dt;
    at(c, c) = at(c, c) + coef;
  }
}

// Boundary connections and sources of the operator-split transport system
// on the structured grid.  Faces in the order x-, x+, y-, y+, z-, z+; a face's
// cells are indexed (j + ny k) on x faces, (i + nx k) on y faces, (i + nx j)
// on z faces.  q: Darcy flux through the face, positive into the domain (the
// boundary is the upstream end of its connection); total: [ncomp][face cells].
struct TransportBC {
  int type[6];  // PF_BC_* of pfgpu.h (0: no boundary connection)
  const double* q[6];
  const double* total[6];
  double sat[6];  // global_auxvars_bc(:)%sat
};
struct TransportSrc {
  int n;
  const int* cell;
  const int* type;      // PF_SRC_*
  const double* q;      // m^3/s, + injection
  const double* total;  // [ncomp][n]
};

// TDispersionBC (transport.F90:236-374) for one boundary connection of a
// structured grid (no transverse dispersion, no Millington-Quirk, no
// secondary continuum: epsilon 1): the hydrodynamic dispersion over
// dist(0) = half the cell's width, with the boundary's saturation.
inline double transport_dispersion_bc(int type, double sat_bc, const Cell& dn, double q, double dist0,
                                      const GirtGrid& g) {
  if (sat_bc < rt_min_saturation || dn.sat < rt_min_saturation) return 0.0;
  const double mechanical = g.dispersivity * std::fabs(q);
  if (type == 1 || type == 2) {  // DIRICHLET_BC, DIRICHLET_ZERO_GRADIENT_BC
    if (type == 2 && q < 0.0) return 0.0;  // outflow: skip
    const double hd = std::max(mechanical + 1.0 * sat_bc * dn.porosity * g.tortuosity * g.diffusion, 1.0e-40);
    return hd / dist0;
  }
  return 0.0;  // ZERO_GRADIENT_BC, NEUMANN_BC, CONCENTRATION_SS
}

// The terms boundary conditions and sources add to the scalar transport
// system: the boundary loop of RTCalculateTransportMatrix
// (reactive_transport.F90:1596-1627: -T_dn on the cell's diagonal) and of
// RTCalculateRHS_t1 (:1337-1370: T_up times the boundary totals on the
// right-hand side), both with TFluxCoefBC (transport.F90:569-609, i.e.
// TFluxCoef without the upwind saturation check); the source/sink loops of
// both (RHS :1372-1418, injection only; matrix :1651-1690, extraction only,
// coefficient > 0) with TSrcSinkCoef (transport.F90:613-673).
// diag_add[N] adds to the diagonal, rhs_add[ncomp][N] to the right-hand side.
inline void transport_bc_terms(const Cell* cells, const GirtGrid& g, int ncomp, const TransportBC& bc,
                               const TransportSrc& src, double* diag_add, double* rhs_add) {
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  const long long N = (long long)nx * ny * nz;
  for (long long c = 0; c < N; ++c) diag_add[c] = 0.0;
  for (long long e = 0; e < N * ncomp; ++e) rhs_add[e] = 0.0;
  for (int f = 0; f < 6; ++f) {
    if (bc.type[f] == 0) continue;
    const int axis = f / 2, plus = f % 2;
    const int na = axis == 0 ? ny : nx, nb = axis == 2 ? ny : nz;  // face cells: a + na*b
    const double area = axis == 0 ? g.dy * g.dz : (axis == 1 ? g.dx * g.dz : g.dx * g.dy);
    const double dist0 = 0.5 * (axis == 0 ? g.dx : (axis == 1 ? g.dy : g.dz));
    for (int b = 0; b < nb; ++b)
      for (int a = 0; a < na; ++a) {
        int i, j, k;
        if (axis == 0) { i = plus ? nx - 1 : 0; j = a; k = b; }
        else if (axis == 1) { i = a; j = plus ? ny - 1 : 0; k = b; }
        else { i = a; j = b; k = plus ? nz - 1 : 0; }
        const long long cell = (long long)i + (long long)nx * (j + (long long)ny * k);
        const long long fi = (long long)a + (long long)na * b, nf = (long long)na * nb;
        const Cell& dn = cells[cell];
        const double q = bc.q[f] ? bc.q[f][fi] : 0.0;
        const double tran = transport_dispersion_bc(bc.type[f], bc.sat[f], dn, q, dist0, g);
        double T_up = 0.0, T_dn = 0.0;
        if (!(dn.sat < rt_min_saturation)) {  // TFluxCoef, check_upwind_saturation false
          double coef_up, coef_dn;
          if (q > 0.0) { coef_up = tran + q; coef_dn = -tran; }
          else { coef_up = tran; coef_dn = -tran + q; }
          T_up = coef_up * area * 1000.0;
          T_dn = coef_dn * area * 1000.0;
        }
        diag_add[cell] = diag_add[cell] + (-T_dn);
        for (int c = 0; c < ncomp; ++c)
          rhs_add[(long long)c * N + cell] = rhs_add[(long long)c * N + cell] + T_up * bc.total[f][c * nf + fi];
      }
  }
  for (int s = 0; s < src.n; ++s) {
    const long long cell = src.cell[s];
    const Cell& cl = cells[cell];
    const double qsrc = src.q[s];
    double T_in = 0.0, T_out = 0.0;
    if (!(cl.sat < rt_min_saturation)) {
      if (src.type[s] == 1) {         // EQUILIBRIUM_SS
        T_in = 1.0e-3;
        T_out = -1.0 * T_in;
      } else if (src.type[s] == 2) {  // MASS_RATE_SS: the "total" is a rate, mol/s
        T_in = 0.0;
        T_out = -1.0;
      } else if (qsrc > 0.0) {        // injection
        T_in = 0.0;
        T_out = -1.0 * qsrc * 1000.0;
      } else {
        T_out = 0.0;
        T_in = -1.0 * qsrc * 1000.0;
      }
    }
    if (!(qsrc > 0.0) && T_in > 0.0) diag_add[cell] = diag_add[cell] + T_in;
    if (!(qsrc < 0.0))
      for (int c = 0; c < ncomp; ++c)
        rhs_add[(long long)c * N + cell] = rhs_add[(long long)c * N + cell] - T_out * src.total[(long long)c * src.n + s];
  }
}

}  // namespace oracle
