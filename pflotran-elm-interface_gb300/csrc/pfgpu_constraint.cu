// pfgpu_constraint.cu -- constraint equilibration, one thread per cell.
//
// ReactionEquilibrateConstraint (src/pflotran/reaction.F90:1328-2115) for the
// constraint types TOTAL, FREE, LOG, PH, CHARGE_BAL, MINERAL and GAS: the
// Newton iteration on free-ion molalities with the log/linear alternation of
// iterations 4-8 (:1902-1913), RSolve (:5457-5516), the dlnC clip
// reaction%max_dlnC (:1932-1935), and activity coefficients switched on after
// the first converged iterate (:2036-2047).  MINERAL rows hold ln(Q/K) of a
// mineral at zero (:1755-1779), GAS rows ln(Q/K) at the log of a partial
// pressure (:1781-1811); their logK follow the cell temperature in
// non-isothermal runs (RUpdateTempDependentCoefs, :1482-1484).  It produces
// the initial conditions of the step kernels; sorption constraints are not
// built.
#include "pfgpu_common.cuh"
#include "pfgpu_kernels.h"
#include "pfgpu_sorb.cuh"

namespace pfgpu {
namespace constraint {

// RActivityCoefficients (LAG), with ln a_H2O (lnaw) when use_activity_h2o
template <int NM>
__device__ void activity_lag(const DevNet& net, const Tables& T, const double* c, const PfCellState& st,
                             const SoA& soa, int64_t cell, double* gam, double& lnaw) {
  double I = 0.0;
  for (int j = 0; j < net.n; ++j) I = I + c[j] * T.pri_Z(j) * T.pri_Z(j);
  for (int i = 0; i < net.ns; ++i) I = I + st.sec_molal[soa.at(i, cell)] * T.sec_Z(i) * T.sec_Z(i);
  I = 0.5 * I;
  const double sI = sqrt(I);
  for (int j = 0; j < net.n; ++j) {
    const double z = T.pri_Z(j);
    gam[j] = fabs(z) > 1.0e-10
                 ? exp((-z * z * sI * net.A / (1.0 + T.pri_a0(j) * net.B * sI) + net.Bdot * I) * LOG_TO_LN)
                 : 1.0;
  }
  double sum_sec_molal = 0.0;
  for (int i = 0; i < net.ns; ++i) {
    const double z = T.sec_Z(i);
    st.sec_act_coef[soa.at(i, cell)] =
        fabs(z) > 1.0e-10
            ? exp((-z * z * sI * net.A / (1.0 + T.sec_a0(i) * net.B * sI) + net.Bdot * I) * LOG_TO_LN)
            : 1.0;
    sum_sec_molal = sum_sec_molal + st.sec_molal[soa.at(i, cell)];
  }
  if (net.o.use_activity_h2o) {
    double sum_pri_molal = 0.0;
    for (int j = 0; j < net.n; ++j) sum_pri_molal = sum_pri_molal + c[j];
    lnaw = water_activity(sum_pri_molal, sum_sec_molal);
  }
}

// per-thread arrays sized for the bucket of ncomp (4, 8, 12, 16, 24), so that
// small networks keep them in registers and L1
template <int NM>
__global__ void __launch_bounds__(128) equilibrate_kernel(DevNet net, PfCellState st, const int32_t* ctype,
                                                          const PfConstraintReaction* creact,
                                                          const double* cconc, int use_prev,
                                                          int32_t* iterations, int max_iterations) {
  const int64_t cell = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= st.ncells) return;
  const Tables T{net.ints, net.dbls, &net};
  const SoA soa{st.ncells};
  const int n = net.n, ns = net.ns;
  const double temp = st.temperature ? st.temperature[cell] : 25.0;
  const double den = st.den_kg[cell];
  const double molar_to_molal = 1000.0 / den / 1.0;
  const bool tsec = !net.o.isothermal && (net.flags & NETF_SEC_LOGKCOEF);
  double c[NM], gam[NM], free_conc[NM], total_conc[NM], tot[NM], lnc[NM], lna[NM];
  double J[NM * NM], Res[NM], prev[NM], VV[NM];
  int indx[NM];
  double lnaw = cell_lnaw(net, st, cell);
  for (int j = 0; j < n; ++j) {
    gam[j] = st.pri_act_coef[soa.at(j, cell)];
    free_conc[j] = use_prev ? st.pri_molal[soa.at(j, cell)] : 1.0e-9;
    total_conc[j] = 0.0;
    const double v = cconc[soa.at(j, cell)];
    switch (ctype[j]) {
      case 1: total_conc[j] = v; break;                                   // TOTAL (mol/L)
      case 2: free_conc[j] = v * molar_to_molal; break;                   // FREE
      case 5: free_conc[j] = pow(10.0, v) * molar_to_molal; break;        // LOG
      case 4: if (!use_prev) free_conc[j] = v * molar_to_molal; break;    // CHARGE_BAL guess
      case 3: free_conc[j] = pow(10.0, -v); break;                        // PH
      case 6: if (!use_prev) free_conc[j] = v * molar_to_molal; break;    // MINERAL guess
      case 7: total_conc[j] = v <= 0.0 ? pow(10.0, v) : v; break;         // GAS partial pressure
      default: break;
    }
    c[j] = free_conc[j];
  }
  // the complexes' logK at the cell's temperature, once (the same values the
  // reference recomputes in every RTotal)
  double logK_sec[PF_MAX_NSEC];
  for (int i = 0; i < ns; ++i) logK_sec[i] = tsec ? interp_logK(T.sec_logKcoef(i), temp) : T.sec_logK(i);
  int its = 0, on_it = 0;
  bool act = use_prev != 0, warned = false;
  int result = -1;
  while (true) {
    for (int j = 0; j < n; ++j)
      if (ctype[j] == 2 || ctype[j] == 5) c[j] = free_conc[j];
    if (net.o.act_coef_update_frequency != PF_ACT_COEF_OFF && act)
      activity_lag<NM>(net, T, c, st, soa, cell, gam, lnaw);
    // RTotalAqueous; d s_i / d m_j = nu_ij s_i / m_j (the reference forms
    // exp(lnQK - ln m_j) / gamma_i, an exp per species of every complex:
    // the same quantity, and the product with 1/m_j rounds within an ulp of it)
    double inv_c[NM];
    for (int j = 0; j < n; ++j) {
      lnc[j] = log(c[j]);
      lna[j] = lnc[j] + log(gam[j]);
      inv_c[j] = 1.0 / c[j];
      tot[j] = c[j];
      for (int k = 0; k < n; ++k) J[j * NM + k] = (j == k) ? 1.0 : 0.0;
    }
    for (int i = 0; i < ns; ++i) {
      double lnQK = add_h2o(-logK_sec[i] * LOG_TO_LN, T.sec_h2o(i), lnaw);
      for (int p = T.sec_begin(i); p < T.sec_end(i); ++p) lnQK = lnQK + T.sec_nu(p) * lna[T.sec_idx(p)];
      const double g = st.sec_act_coef[soa.at(i, cell)];
      const double s = exp(lnQK) / g;
      st.sec_molal[soa.at(i, cell)] = s;
      for (int p = T.sec_begin(i); p < T.sec_end(i); ++p) tot[T.sec_idx(p)] += T.sec_nu(p) * s;
      for (int pj = T.sec_begin(i); pj < T.sec_end(i); ++pj) {
        const int jc = T.sec_idx(pj);
        const double t = T.sec_nu(pj) * s * inv_c[jc];
        for (int pi = T.sec_begin(i); pi < T.sec_end(i); ++pi) J[T.sec_idx(pi) * NM + jc] += T.sec_nu(pi) * t;
      }
    }
    const double den_L = den * 1.0e-3;
    for (int j = 0; j < n; ++j) {
      tot[j] *= den_L;
      for (int k = 0; k < n; ++k) J[j * NM + k] *= den_L;
    }
    if (has_sorption(net)) {
      // the rest of RTotal (:1594, no ierror): sorbed totals follow the
      // iterate; no constraint row here reads them
      for (int j = 0; j < n; ++j) st.total_sorb[soa.at(j, cell)] = 0.0;
      total_sorb(
          net, T, [&](int j) { return c[j]; }, [&](int j) { return gam[j]; },
          [&](int m) { return st.mnrl_volfrac[soa.at(m, cell)]; }, st.porosity[cell], den,
          st.ionx_ref_sorbed ? st.ionx_ref_sorbed + cell : nullptr, st.ncells,
          [&](int j, double v) { st.total_sorb[soa.at(j, cell)] += v; }, [](int, int, double) {},
          surf_cell(net, st, cell));
    }
    // constraint rows (dtotal is J until a row is replaced; charge balance
    // reads dtotal rows of other components, so build it first)
    double cb_row[NM];
    int cb = -1;
    for (int j = 0; j < n; ++j)
      if (ctype[j] == 4) cb = j;
    double cb_res = 0.0;
    if (cb >= 0) {
      for (int k = 0; k < n; ++k) cb_row[k] = 0.0;
      for (int j = 0; j < n; ++j) {
        cb_res = cb_res + T.pri_Z(j) * tot[j];
        for (int k = 0; k < n; ++k) cb_row[j] = cb_row[j] + T.pri_Z(k) * J[k * NM + j];
      }
    }
    for (int j = 0; j < n; ++j) {
      switch (ctype[j]) {
        case 1: Res[j] = tot[j] - total_conc[j]; break;
        case 2: case 5:
          Res[j] = 0.0;
          for (int k = 0; k < n; ++k) J[j * NM + k] = (j == k) ? 1.0 : 0.0;
          break;
        case 4:
          Res[j] = cb_res;
          for (int k = 0; k < n; ++k) J[j * NM + k] = cb_row[k];
          if (c[j] < 1.0e-20 && !warned) {
            if ((Res[j] > 0.0 && T.pri_Z(j) > 0.0) || (Res[j] < 0.0 && T.pri_Z(j) < 0.0)) {
              warned = true;
              c[j] = (double)1.e-3f;
            }
          }
          break;
        case 3:
          Res[j] = 0.0;
          for (int k = 0; k < n; ++k) J[j * NM + k] = (j == k) ? 1.0 : 0.0;
          c[j] = pow(10.0, -cconc[soa.at(j, cell)]) / gam[j];
          break;
        case 6:
        case 7: {
          const PfConstraintReaction& R = creact[j];
          const double logK =
              (!net.o.isothermal && R.temperature_dependent) ? interp_logK(R.logKcoef, temp) : R.logK;
          double lnQK = -logK * LOG_TO_LN;
          for (int p = 0; p < R.nspec; ++p) lnQK = lnQK + R.stoich[p] * log(c[R.spec[p]] * gam[R.spec[p]]);
          Res[j] = ctype[j] == 6 ? lnQK : lnQK - log(total_conc[j]);
          for (int k = 0; k < n; ++k) J[j * NM + k] = 0.0;
          for (int p = 0; p < R.nspec; ++p) J[j * NM + R.spec[p]] = R.stoich[p] / c[R.spec[p]];
          break;
        }
        default: break;
      }
    }
    double maxres = 0.0;
    for (int j = 0; j < n; ++j) maxres = fmax(maxres, fabs(Res[j]));
    bool logf = net.o.use_log_formulation != 0;
    if (logf && its > 3 && its < 9) logf = (its % 2 == 0);
    // RSolve (row scale, log column scale, LU, back-substitution)
    double rhs[NM];
    for (int i = 0; i < n; ++i) {
      double mx = 0.0;
      for (int k = 0; k < n; ++k) mx = fmax(mx, fabs(J[i * NM + k]));
      const double nrm = 1.0 / fmax(1.0, mx);
      rhs[i] = Res[i] * nrm;
      for (int k = 0; k < n; ++k) J[i * NM + k] *= nrm;
    }
    if (logf)
      for (int k = 0; k < n; ++k)
        for (int i = 0; i < n; ++i) J[i * NM + k] *= c[k];
    bool singular = false;
    for (int i = 0; i < n && !singular; ++i) {
      double aamax = 0.0;
      for (int k = 0; k < n; ++k) aamax = fmax(aamax, fabs(J[i * NM + k]));
      if (aamax <= 0.0) singular = true;
      else VV[i] = 1.0 / aamax;
    }
    if (singular) break;
    for (int j = 0; j < n; ++j) {
      for (int i = 0; i < j; ++i) {
        double sum = J[i * NM + j];
        for (int k = 0; k < i; ++k) sum -= J[i * NM + k] * J[k * NM + j];
        J[i * NM + j] = sum;
      }
      double aamax = 0.0;
      int imax = j;
      for (int i = j; i < n; ++i) {
        double sum = J[i * NM + j];
        for (int k = 0; k < j; ++k) sum -= J[i * NM + k] * J[k * NM + j];
        J[i * NM + j] = sum;
        const double dum = VV[i] * fabs(sum);
        if (dum >= aamax) { imax = i; aamax = dum; }
      }
      if (j != imax) {
        for (int k = 0; k < n; ++k) { double d = J[imax * NM + k]; J[imax * NM + k] = J[j * NM + k]; J[j * NM + k] = d; }
        VV[imax] = VV[j];
      }
      indx[j] = imax;
      if (J[j * NM + j] == 0.0) J[j * NM + j] = 1.0e-20;
      if (j != n - 1) {
        const double d = 1.0 / J[j * NM + j];
        for (int i = j + 1; i < n; ++i) J[i * NM + j] *= d;
      }
    }
    for (int i = 0; i < n; ++i) {
      const int ll = indx[i];
      double sum = rhs[ll];
      rhs[ll] = rhs[i];
      for (int k = 0; k < i; ++k) sum -= J[i * NM + k] * rhs[k];
      rhs[i] = sum;
    }
    for (int i = n - 1; i >= 0; --i) {
      double sum = rhs[i];
      for (int k = i + 1; k < n; ++k) sum -= J[i * NM + k] * rhs[k];
      rhs[i] = sum / J[i * NM + i];
    }
    for (int j = 0; j < n; ++j) prev[j] = c[j];
    if (logf) {
      for (int j = 0; j < n; ++j) {
        const double u = fsign1(rhs[j]) * fmin(fabs(rhs[j]), 5.0);  // reaction%max_dlnC
        c[j] = c[j] * exp(-u);
      }
    } else {
      double min_ratio = 1.7976931348623157e308;
      for (int j = 0; j < n; ++j)
        if (prev[j] <= rhs[j]) min_ratio = fmin(min_ratio, fabs(prev[j] / rhs[j]));
      for (int j = 0; j < n; ++j) c[j] = prev[j] - (min_ratio <= 1.0 ? rhs[j] * min_ratio * 0.99 : rhs[j]);
    }
    double mn = c[0];
    for (int j = 1; j < n; ++j) mn = fmin(mn, c[j]);
    if (!(mn > 0.0)) break;
    double maxrel = 0.0;
    for (int j = 0; j < n; ++j) maxrel = fmax(maxrel, fabs((c[j] - prev[j]) / prev[j]));
    its = its + 1;
    if (its >= max_iterations) break;
    if (maxres < net.o.max_residual_tolerance && maxrel < net.o.max_relative_change_tolerance) {
      if (act && its - on_it > 1) { result = its; break; }
      if (!act) on_it = its;
      act = true;
    }
  }
  for (int j = 0; j < n; ++j) {
    st.pri_molal[soa.at(j, cell)] = c[j];
    st.pri_act_coef[soa.at(j, cell)] = gam[j];
    st.total[soa.at(j, cell)] = tot[j];
  }
  if (net.o.use_activity_h2o) st.ln_act_h2o[cell] = lnaw;
  if (iterations) iterations[cell] = result;
}

}  // namespace constraint
}  // namespace pfgpu

using namespace pfgpu;

extern "C" int32_t pf_equilibrate_constraint_impl(const DevNet* net, const PfCellState* st,
                                                  const int32_t* ctype, const PfConstraintReaction* creact,
                                                  const double* cconc, int use_prev, int32_t* iterations,
                                                  int max_iterations, void* stream) {
  const int tpb = 128;
  const int64_t blocks = (st->ncells + tpb - 1) / tpb;
  if (blocks) {
    cudaStream_t s = (cudaStream_t)stream;
#define PF_EQ(NMX) \
  constraint::equilibrate_kernel<NMX><<<blocks, tpb, 0, s>>>(*net, *st, ctype, creact, cconc, use_prev, iterations, \
                                                             max_iterations)
    if (net->n <= 4) PF_EQ(4);
    else if (net->n <= 8) PF_EQ(8);
    else if (net->n <= 12) PF_EQ(12);
    else if (net->n <= 16) PF_EQ(16);
    else PF_EQ(24);
#undef PF_EQ
  }
  return cudaGetLastError() == cudaSuccess ? PF_OK : PF_ERR_CUDA;
}
