// pfgpu_plain.cu -- the plain GPU form of the operator-split reaction step.
//
// One thread per cell, no work queue, no table staging: each thread runs
// RStep (src/pflotran/reaction.F90:3564-3738) exactly as written -- RReact's
// Newton loop (:3742-4055) with RTotalAqueous (:4665-4759), RKineticMineral
// (reaction_mineral.F90:647-1078), RSolve (:5457-5516, back-substituting) and
// the Crout LU (utility.F90:597-735) -- on per-thread arrays sized for the
// largest ncomp of its bucket.  It is the baseline the batched kernel is
// measured against, and a second, independent GPU statement of the algorithm.
// With equilibrium sorption RTAuxVarCompute adds RTotalSorb and the
// accumulation RAccumulationSorb[Derivative] (reaction.F90:3836-3839,
// 3861-3865, 3904-3909), any ncomp; kinetic-mineral rate prefactors
// (reaction_mineral.F90:820-858, 976-1070) and the NEWTON activity
// algorithm at every Newton iteration (:3857-3860, 4403-4551) run here only.
#include "pfgpu_common.cuh"
#include "pfgpu_kernels.h"
#include "pfgpu_prefactor.cuh"
#include "pfgpu_sorb.cuh"

namespace pfgpu {
namespace plain {

template <int NMAX>
struct Work {
  double c[NMAX], total[NMAX], gamma[NMAX], lnc[NMAX], lna[NMAX];
  double dtotal[NMAX * NMAX];
  double J[NMAX * NMAX];
  double res[NMAX], fixed[NMAX], init_total[NMAX], update[NMAX];
  double sorb[NMAX];          // total_sorb of the last evaluation
  double dsorb[NMAX * NMAX];  // dtotal_sorb of the last evaluation
};

struct CellScalars {
  double porosity, sat, den_kg, volume, temp;
  double lnaw;  // ln a_H2O (rt_auxvar%ln_act_h2o)
};

template <int NMAX, bool EXT>
__device__ void total_aqueous(const Tables& T, int n, int ns, const double* sec_logK,
                              const double* sec_gamma, double* sec_molal_out, int64_t cell,
                              const SoA& soa, const CellScalars& cs, Work<NMAX>& w) {
  const double den_kg_per_L = cs.den_kg * 1.0 * 1.0e-3;
  for (int j = 0; j < n; ++j) {
    w.lnc[j] = log(w.c[j]);
    w.lna[j] = w.lnc[j] + log(w.gamma[j]);
    w.total[j] = w.c[j];
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) w.dtotal[i * NMAX + j] = (i == j) ? 1.0 : 0.0;
  for (int i = 0; i < ns; ++i) {
    const int b = T.sec_begin(i), e = T.sec_end(i);
    double lnQK = -sec_logK[i] * LOG_TO_LN;
    if (EXT && water_on(*T.net)) lnQK = add_h2o(lnQK, T.sec_h2o(i), cs.lnaw);
    for (int p = b; p < e; ++p) lnQK = lnQK + T.sec_nu(p) * w.lna[T.sec_idx(p)];
    const double g = sec_gamma[soa.at(i, cell)];
    const double s = exp(lnQK) / g;
    sec_molal_out[soa.at(i, cell)] = s;
    for (int p = b; p < e; ++p) {
      int k = T.sec_idx(p);
      w.total[k] = w.total[k] + T.sec_nu(p) * s;
    }
    for (int pj = b; pj < e; ++pj) {
      int jc = T.sec_idx(pj);
      double tempreal = T.sec_nu(pj) * exp(lnQK - w.lnc[jc]) / g;
      for (int pi = b; pi < e; ++pi) {
        int ic = T.sec_idx(pi);
        w.dtotal[ic * NMAX + jc] = w.dtotal[ic * NMAX + jc] + T.sec_nu(pi) * tempreal;
      }
    }
  }
  for (int j = 0; j < n; ++j) w.total[j] = w.total[j] * den_kg_per_L;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) w.dtotal[i * NMAX + j] = w.dtotal[i * NMAX + j] * den_kg_per_L;
}

// RKineticMineral.  Jac may be null (derivative = false).  sec_logK: the
// complexes' logK at the cell's temperature (prefactor derivative).  PF:
// the extended instantiation (rate prefactors, water activity), separate so
// that the common one keeps its registers.
template <int NMAX, bool PF>
__device__ void kinetic_mineral(const Tables& T, const DevNet& net, int n, const double* mnrl_logK,
                                const double* sec_logK, int64_t cell, const SoA& soa, const PfCellState& st,
                                const CellScalars& cs, Work<NMAX>& w, double* Res, double* Jac) {
  const bool has_msf = net.flags & NETF_MSF, has_tk = net.flags & NETF_TEMKIN,
             has_pw = net.flags & NETF_POWER;
  constexpr bool has_pf = PF;
  double prefactor[PF_MAX_PREFACTORS], lnps[PF_MAX_PREFACTORS][PF_MAX_PREFACTOR_SPECIES];
  auto ln_act = [&](int j) { return w.lna[j]; };
  auto ln_sec_act = [&](int i) { return log(st.sec_molal[soa.at(i, cell)]) + log(st.sec_act_coef[soa.at(i, cell)]); };
  for (int m = 0; m < net.nm; ++m) st.mnrl_rate[soa.at(m, cell)] = 0.0;
  for (int m = 0; m < net.nm; ++m) {
    const int b = T.mnrl_begin(m), e = T.mnrl_end(m);
    double lnQK = -mnrl_logK[m] * LOG_TO_LN;
    if (PF && water_on(net)) lnQK = add_h2o(lnQK, T.mnrl_h2o(m), cs.lnaw);
    for (int p = b; p < e; ++p) lnQK = lnQK + T.mnrl_nu(p) * w.lna[T.mnrl_idx(p)];
    double QK = exp(lnQK);
    double aff;
    if (has_tk) {
      if (has_msf) aff = 1.0 - pow(QK, 1.0 / (T.msf(m) * T.temkin(m)));
      else aff = 1.0 - pow(QK, 1.0 / T.temkin(m));
    } else if (has_msf) {
      aff = 1.0 - pow(QK, 1.0 / T.msf(m));
    } else {
      aff = 1.0 - QK;
    }
    double sign_ = fsign1(aff);
    double Im, Im_const, k;
    const double vf = st.mnrl_volfrac[soa.at(m, cell)];
    if (vf > 0 || sign_ < 0.0) {
      if (T.irreversible(m) == 1 && sign_ < 0.0) continue;
      if (T.thresh(m) > 0.0 && sign_ < 0.0 && QK < T.thresh(m)) continue;
      if (T.limiter(m) > 0.0) aff = aff / (1.0 + (1.0 - aff) / T.limiter(m));
      if (has_pf && T.pf_cnt(m) > 0) {
        k = prefactor_rate(T, m, ln_act, ln_sec_act, cs.temp, prefactor, lnps);
      } else {
        double arr = 1.0;
        if (T.ea(m) > 0.0)
          arr = exp(T.ea(m) / IDEAL_GAS_CONSTANT * (1.0 / (25.0 + 273.15) - 1.0 / (cs.temp + 273.15)));
        k = T.rate(m) * arr;
      }
      Im_const = -st.mnrl_area[soa.at(m, cell)];
      if (has_msf) Im_const = Im_const / T.msf(m);
      if (has_pw) Im = Im_const * sign_ * pow(fabs(aff), T.power(m)) * k;
      else Im = Im_const * sign_ * fabs(aff) * k;
      st.mnrl_rate[soa.at(m, cell)] = Im;
    } else {
      continue;
    }
    Im_const = Im_const * cs.volume;
    Im = Im * cs.volume;
    for (int p = b; p < e; ++p) {
      int ic = T.mnrl_idx(p);
      Res[ic] = Res[ic] + T.mnrl_nu(p) * Im;
    }
    if (!Jac) continue;
    double dIm_dQK;
    if (has_pw) dIm_dQK = -Im * T.power(m) / fabs(aff);
    else dIm_dQK = -Im_const * k;
    if (has_tk) {
      if (has_msf) dIm_dQK = dIm_dQK * (1.0 / (T.msf(m) * T.temkin(m))) / QK * (1.0 - aff);
      else dIm_dQK = dIm_dQK * (1.0 / T.temkin(m)) / QK * (1.0 - aff);
    } else if (has_msf) {
      dIm_dQK = dIm_dQK * (1.0 / T.msf(m)) / QK * (1.0 - aff);
    }
    const double rl = T.limiter(m);
    const double den = 1.0 + (1.0 - aff) / rl;
    for (int pj = b; pj < e; ++pj) {
      int jc = T.mnrl_idx(pj);
      double dQK_dmj = T.mnrl_nu(pj) * QK * exp(-w.lnc[jc]) * cs.den_kg * 1.0e-3;
      for (int pi = b; pi < e; ++pi) {
        int ic = T.mnrl_idx(pi);
        if (rl <= 0.0)
          Jac[ic * NMAX + jc] = Jac[ic * NMAX + jc] + T.mnrl_nu(pi) * dIm_dQK * dQK_dmj;
        else
          Jac[ic * NMAX + jc] = Jac[ic * NMAX + jc] +
                                T.mnrl_nu(pi) * dIm_dQK * (1.0 + QK / rl / den) * dQK_dmj / den;
      }
    }
    if (has_pf && T.pf_cnt(m) > 0)
      prefactor_derivative(
          T, m, Im, k, prefactor, lnps, ln_act, ln_sec_act, [&](int j) { return w.gamma[j]; },
          [&](int i) { return st.sec_act_coef[soa.at(i, cell)]; }, [&](int j) { return w.lnc[j]; },
          [&](int i) { return add_h2o(-sec_logK[i] * LOG_TO_LN, T.sec_h2o(i), cs.lnaw); }, cs.temp,
          [&](int r, int c, double v) { Jac[r * NMAX + c] = Jac[r * NMAX + c] + v; });
  }
}

// RSolve + LUDecomposition1 + LUBackSubstitution (intended branch).
template <int NMAX>
__device__ int rsolve(int n, double* J, const double* conc, const double* Res, double* update,
                      bool log_form, bool fork_literal) {
  double rhs[NMAX], VV[NMAX];
  int indx[NMAX];
  for (int i = 0; i < n; ++i) {
    double mx = 0.0;
    for (int j = 0; j < n; ++j) mx = fmax(mx, fabs(J[i * NMAX + j]));
    double norm = 1.0 / fmax(1.0, mx);
    rhs[i] = Res[i] * norm;
    for (int j = 0; j < n; ++j) J[i * NMAX + j] = J[i * NMAX + j] * norm;
  }
  if (log_form)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) J[i * NMAX + j] = J[i * NMAX + j] * conc[j];
  for (int i = 0; i < n; ++i) {
    double aamax = 0.0;
    for (int j = 0; j < n; ++j)
      if (fabs(J[i * NMAX + j]) > aamax) aamax = fabs(J[i * NMAX + j]);
    if (aamax <= 0.0) return 1;
    VV[i] = 1.0 / aamax;
  }
  for (int j = 0; j < n; ++j) {
    for (int i = 0; i < j; ++i) {
      double sum = J[i * NMAX + j];
      for (int k = 0; k < i; ++k) sum = sum - J[i * NMAX + k] * J[k * NMAX + j];
      J[i * NMAX + j] = sum;
    }
    double aamax = 0.0;
    int imax = j;
    for (int i = j; i < n; ++i) {
      double sum = J[i * NMAX + j];
      for (int k = 0; k < j; ++k) sum = sum - J[i * NMAX + k] * J[k * NMAX + j];
      J[i * NMAX + j] = sum;
      double dum = VV[i] * fabs(sum);
      if (dum >= aamax) { imax = i; aamax = dum; }
    }
    if (j != imax) {
      for (int k = 0; k < n; ++k) {
        double d = J[imax * NMAX + k];
        J[imax * NMAX + k] = J[j * NMAX + k];
        J[j * NMAX + k] = d;
      }
      VV[imax] = VV[j];
    }
    indx[j] = imax;
    if (J[j * NMAX + j] == 0.0) J[j * NMAX + j] = 1.0e-20;
    if (j != n - 1) {
      double dum = 1.0 / J[j * NMAX + j];
      for (int i = j + 1; i < n; ++i) J[i * NMAX + j] = J[i * NMAX + j] * dum;
    }
  }
  if (fork_literal) return 0;
  int ii = -1;
  for (int i = 0; i < n; ++i) {
    int ll = indx[i];
    double sum = rhs[ll];
    rhs[ll] = rhs[i];
    if (ii >= 0) {
      for (int j = ii; j < i; ++j) sum = sum - J[i * NMAX + j] * rhs[j];
    } else if (sum != 0.0) {
      ii = i;
    }
    rhs[i] = sum;
  }
  for (int i = n - 1; i >= 0; --i) {
    double sum = rhs[i];
    for (int j = i + 1; j < n; ++j) sum = sum - J[i * NMAX + j] * rhs[j];
    rhs[i] = sum / J[i * NMAX + i];
  }
  for (int i = 0; i < n; ++i) update[i] = rhs[i];
  return 0;
}

// RActivityCoefficients by the NEWTON algorithm (reaction.F90:4403-4551) at
// the Newton iterate w.c: a Newton iteration on the ionic strength, the
// primaries' activities held at the iterate and the coefficients of the
// last evaluation; each pass rewrites both sets of coefficients, the
// complexes' molalities and (water activity on) ln a_H2O.  Returns false
// where the reference gives up -- more than 50 passes (:4420-4431) or a
// negative ionic strength (:4476-4485) -- after setting the iterate and the
// coefficients to NaN as it does; its option%ierror then fails RReact after
// the residual (:3929-3943).
template <int NMAX>
__device__ bool activity_newton(const Tables& T, const DevNet& net, int n, int ns, const double* sec_logK,
                                int64_t cell, const SoA& soa, const PfCellState& st, CellScalars& cs,
                                Work<NMAX>& w) {
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  auto give_up = [&]() {
    for (int j = 0; j < n; ++j) {
      w.c[j] = nan;
      w.gamma[j] = nan;
    }
    for (int i = 0; i < ns; ++i) st.sec_act_coef[soa.at(i, cell)] = nan;
    return false;
  };
  double sum_pri_molal = 0.0, fpri = 0.0;
  for (int j = 0; j < n; ++j) {
    w.lna[j] = log(w.c[j]) + log(w.gamma[j]);
    sum_pri_molal = sum_pri_molal + w.c[j];
    fpri = fpri + w.c[j] * T.pri_Z(j) * T.pri_Z(j);
  }
  double II = 0.0;
  for (int it = 1;; ++it) {
    if (it > 50) return give_up();
    double I = fpri;
    for (int i = 0; i < ns; ++i) I = I + st.sec_molal[soa.at(i, cell)] * T.sec_Z(i) * T.sec_Z(i);
    I = 0.5 * I;
    const double f = I;
    if (fabs(I - II) < 1.0e-6 * I) return true;
    if (ns > 0) {
      double didi = 0.0;
      const double sqrt_I = sqrt(I);
      for (int i = 0; i < ns; ++i) {
        const double zi = T.sec_Z(i);
        if (fabs(zi) > 0.0) {
          const double t = 1.0 + net.B * T.sec_a0(i) * sqrt_I;
          double sum = 0.5 * net.A * zi * zi / (sqrt_I * (t * t)) - net.Bdot;
          for (int p = T.sec_begin(i); p < T.sec_end(i); ++p) {
            const double zj = T.pri_Z(T.sec_idx(p));
            if (fabs(zj) > 0.0) {
              const double tj = 1.0 + net.B * T.pri_a0(T.sec_idx(p)) * sqrt_I;
              sum = sum + T.sec_nu(p) * (-0.5 * net.A * (zj * zj) / (sqrt_I * (tj * tj)) + net.Bdot);
            }
          }
          didi = didi + 0.5 * zi * zi * (st.sec_molal[soa.at(i, cell)] * LOG_TO_LN * sum);
        }
      }
      const double den = 1.0 - didi;
      II = fabs(den) > 0.0 ? (f - I * didi) / den : f;
    } else {
      II = f;
    }
    if (II < 0.0) return give_up();
    I = II;
    const double sqrt_I = sqrt(I);
    for (int j = 0; j < n; ++j) {
      const double z = T.pri_Z(j);
      w.gamma[j] = fabs(z) > 0.0
                       ? exp((-z * z * sqrt_I * net.A / (1.0 + T.pri_a0(j) * net.B * sqrt_I) + net.Bdot * I) *
                             LOG_TO_LN)
                       : 1.0;
    }
    double sum_sec_molal = 0.0;
    for (int i = 0; i < ns; ++i) {
      const double z = T.sec_Z(i);
      const double g =
          fabs(z) > 0.0
              ? exp((-z * z * sqrt_I * net.A / (1.0 + T.sec_a0(i) * net.B * sqrt_I) + net.Bdot * I) * LOG_TO_LN)
              : 1.0;
      st.sec_act_coef[soa.at(i, cell)] = g;
      double lnQK = -sec_logK[i] * LOG_TO_LN;
      if (water_on(net)) lnQK = add_h2o(lnQK, T.sec_h2o(i), cs.lnaw);
      for (int p = T.sec_begin(i); p < T.sec_end(i); ++p) lnQK = lnQK + T.sec_nu(p) * w.lna[T.sec_idx(p)];
      const double sm = exp(lnQK) / g;
      st.sec_molal[soa.at(i, cell)] = sm;
      sum_sec_molal = sum_sec_molal + sm;
    }
    if (net.o.use_activity_h2o) cs.lnaw = water_activity(sum_pri_molal, sum_sec_molal);
  }
}

template <int NMAX, bool PF>
__global__ void __launch_bounds__(128) rstep_plain_kernel(DevNet net, PfCellState st, double dt_uniform,
                                                          unsigned long long* counters) {
  const int64_t cell = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= st.ncells) return;
  Tables T{net.ints, net.dbls, &net};
  const SoA soa{st.ncells};
  const int n = net.n, ns = net.ns, nm = net.nm;
  const PfOptions& o = net.o;
  Work<NMAX> w;
  CellScalars cs{st.porosity[cell], st.saturation[cell], st.den_kg[cell], st.volume[cell],
                 st.temperature ? st.temperature[cell] : 25.0, PF ? cell_lnaw(net, st, cell) : 0.0};
  // per-cell logK (RUpdateTempDependentCoefs mutates the shared arrays; kept per thread here)
  double sec_logK[PF_MAX_NSEC], mnrl_logK[PF_MAX_NMNRL];
  const bool iso = o.isothermal != 0;
  for (int i = 0; i < ns; ++i)
    sec_logK[i] = (!iso && (net.flags & NETF_SEC_LOGKCOEF)) ? interp_logK(T.sec_logKcoef(i), cs.temp)
                                                            : T.sec_logK(i);
  for (int m = 0; m < nm; ++m)
    mnrl_logK[m] = (!iso && (net.flags & NETF_MNRL_LOGKCOEF)) ? interp_logK(T.mnrl_logKcoef(m), cs.temp)
                                                              : T.mnrl_logK(m);
  for (int j = 0; j < n; ++j) w.gamma[j] = st.pri_act_coef[soa.at(j, cell)];
  double guess[NMAX], small_val[NMAX];
  unsigned small_mask = 0;
  double total_io[NMAX];
  for (int j = 0; j < n; ++j) {
    total_io[j] = st.total[soa.at(j, cell)];
    guess[j] = st.pri_molal[soa.at(j, cell)];
    if (total_io[j] <= 1.0e-40) {  // RStep floor, reaction.F90:3618-3624
      small_mask |= 1u << j;
      small_val[j] = total_io[j];
      total_io[j] = 1.0e-40;
    }
  }
  if (o.use_total_as_guess)
    for (int j = 0; j < n; ++j) guess[j] = total_io[j];
  const double target_time = st.dt_cell ? st.dt_cell[cell] : dt_uniform;
  double cumulative = 0.0, dt = target_time;
  int num_cuts = 0, n_const = 0, nsub = 0, its_total = 0, ierror_step = 0;
  const double psv_t = cs.porosity * cs.sat * 1000.0 * cs.volume;
  const bool dry = cs.sat < RT_MIN_SATURATION;
  const bool has_sorb = has_sorption(net);
  double* ionx_ref = st.ionx_ref_sorbed ? st.ionx_ref_sorbed + cell : nullptr;
  // RTotalSorb (RZeroSorb first) at the current iterate into w.sorb,
  // w.dsorb and the state
  auto sorb_eval = [&]() {
    for (int j = 0; j < n; ++j) {
      w.sorb[j] = 0.0;
      for (int k = 0; k < n; ++k) w.dsorb[j * NMAX + k] = 0.0;
    }
    const bool ok = total_sorb(
        net, T, [&](int j) { return w.c[j]; }, [&](int j) { return w.gamma[j]; },
        [&](int m) { return st.mnrl_volfrac[soa.at(m, cell)]; }, cs.porosity, cs.den_kg, ionx_ref, st.ncells,
        [&](int j, double v) { w.sorb[j] = w.sorb[j] + v; },
        [&](int i, int j, double v) { w.dsorb[i * NMAX + j] = w.dsorb[i * NMAX + j] + v; },
        surf_cell(net, st, cell));
    for (int j = 0; j < n; ++j) st.total_sorb[soa.at(j, cell)] = w.sorb[j];
    return ok;
  };
  if (has_sorb)
    for (int j = 0; j < n; ++j) w.sorb[j] = st.total_sorb[soa.at(j, cell)];
  for (;;) {
    if (cumulative >= target_time) break;
    // ------------------------------------------------------------- RReact
    int ierror = 0, its = 0;
    double r0 = 0.0;
    for (int j = 0; j < n; ++j) {
      w.fixed[j] = dry ? 0.0 : psv_t * total_io[j];
      if (has_sorb) w.fixed[j] = w.fixed[j] + w.sorb[j] * cs.volume;  // RAccumulationSorb
      w.init_total[j] = total_io[j];
      w.c[j] = guess[j];
    }
    for (;;) {
      its = its + 1;
      bool act_failed = false;
      if (PF && o.act_coef_update_frequency == PF_ACT_COEF_NEWTON_ITER &&
          o.act_coef_update_algorithm == PF_ACT_COEF_ALGO_NEWTON) {
        act_failed = !activity_newton<NMAX>(T, net, n, ns, sec_logK, cell, soa, st, cs, w);
      } else if (o.act_coef_update_frequency == PF_ACT_COEF_NEWTON_ITER) {
        // RActivityCoefficients, LAG (reaction.F90:3857-3860, 4553-4612):
        // ionic strength from this iterate and the previous evaluation's
        // complexes
        double I = 0.0;
        for (int j = 0; j < n; ++j) I = I + w.c[j] * T.pri_Z(j) * T.pri_Z(j);
        for (int i = 0; i < ns; ++i) I = I + st.sec_molal[soa.at(i, cell)] * T.sec_Z(i) * T.sec_Z(i);
        I = 0.5 * I;
        const double sI = sqrt(I);
        for (int j = 0; j < n; ++j) {
          const double z = T.pri_Z(j);
          w.gamma[j] = fabs(z) > 1.0e-10
                           ? exp((-z * z * sI * net.A / (1.0 + T.pri_a0(j) * net.B * sI) + net.Bdot * I) * LOG_TO_LN)
                           : 1.0;
        }
        double sum_sec_molal = 0.0;
        for (int i = 0; i < ns; ++i) {
          const double z = T.sec_Z(i);
          st.sec_act_coef[soa.at(i, cell)] =
              fabs(z) > 1.0e-10
                  ? exp((-z * z * sI * net.A / (1.0 + T.sec_a0(i) * net.B * sI) + net.Bdot * I) * LOG_TO_LN)
                  : 1.0;
          sum_sec_molal = sum_sec_molal + st.sec_molal[soa.at(i, cell)];
        }
        if (PF && o.use_activity_h2o) {  // reaction.F90:4604-4611
          double sum_pri_molal = 0.0;
          for (int j = 0; j < n; ++j) sum_pri_molal = sum_pri_molal + w.c[j];
          cs.lnaw = water_activity(sum_pri_molal, sum_sec_molal);
        }
      }
      total_aqueous<NMAX, PF>(T, n, ns, sec_logK, st.sec_act_coef, st.sec_molal, cell, soa, cs, w);
      for (int j = 0; j < n; ++j) total_io[j] = w.total[j];
      // RTotalSorb; a failed ion-exchange solve fails RReact, no restore (:3861-3865)
      if (has_sorb && !sorb_eval()) {
        ierror = 1;
        break;
      }
      if (its > o.maximum_reaction_iterations) {
        ierror = 1;
        for (int j = 0; j < n; ++j) total_io[j] = w.init_total[j];
        break;
      }
      if (dry) {
        for (int j = 0; j < n; ++j) {
          w.res[j] = (0.0 - w.fixed[j]) / dt;
          for (int k = 0; k < n; ++k) w.J[j * NMAX + k] = (j == k) ? 1.0 : 0.0;
        }
      } else {
        const double psvd_t = cs.porosity * cs.sat * 1000.0 * cs.volume / dt;
        for (int j = 0; j < n; ++j) {
          w.res[j] = (psv_t * w.total[j] - w.fixed[j]) / dt;
          for (int k = 0; k < n; ++k) w.J[j * NMAX + k] = w.dtotal[j * NMAX + k] * psvd_t;
        }
        if (nm > 0) kinetic_mineral<NMAX, PF>(T, net, n, mnrl_logK, sec_logK, cell, soa, st, cs, w, w.res, w.J);
      }
      if (has_sorb) {
        // residual with the sorbed accumulation: (psv T + V S - fixed)/dt,
        // Jacobian + dtotal_sorb V/dt; the minerals' terms are already in
        // res, so add V S/dt to it (the same sum up to the order of terms)
        const double v_t = cs.volume / dt;
        for (int j = 0; j < n; ++j) {
          w.res[j] = w.res[j] + w.sorb[j] * cs.volume / dt;
          for (int k = 0; k < n; ++k) w.J[j * NMAX + k] = w.J[j * NMAX + k] + w.dsorb[j * NMAX + k] * v_t;
        }
      }
      if (PF && act_failed) {  // option%ierror of the activity pass: no total restore (:3929-3943)
        ierror = 1;
        break;
      }
      double dot = 0.0, mx = 0.0;
      for (int j = 0; j < n; ++j) {
        dot = dot + w.res[j] * w.res[j];
        mx = fmax(mx, fabs(w.res[j]));
      }
      double two_norm = sqrt(dot);
      if (its == 1) r0 = two_norm;
      if (mx < o.max_residual_tolerance) break;
      if (two_norm / r0 < o.max_rel_residual_tolerance) break;
      if (!o.fork_literal_rsolve || its == 1)
        for (int j = 0; j < n; ++j) w.update[j] = 0.0;
      if (rsolve<NMAX>(n, w.J, w.c, w.res, w.update, o.use_log_formulation != 0,
                       o.fork_literal_rsolve != 0)) {
        ierror = 1;  // solve_error path: no total restore (reaction.F90:3963-3966)
        break;
      }
      double max_rel = 0.0;
      double latest[NMAX];
      if (o.use_log_formulation) {
        for (int j = 0; j < n; ++j) {
          double u = fsign1(w.update[j]) * fmin(fabs(w.update[j]), o.max_dlnC_rreact);
          latest[j] = w.c[j] * exp(-u);
        }
      } else {
        double min_ratio = 1.7976931348623157e308;
        for (int j = 0; j < n; ++j)
          if (w.c[j] <= w.update[j]) min_ratio = fmin(min_ratio, fabs(w.c[j] / w.update[j]));
        for (int j = 0; j < n; ++j) {
          double u = (min_ratio < 1.0) ? w.update[j] * min_ratio * 0.99 : w.update[j];
          latest[j] = w.c[j] - u;
        }
      }
      for (int j = 0; j < n; ++j) max_rel = fmax(max_rel, fabs((latest[j] - w.c[j]) / w.c[j]));
      if (max_rel < o.max_relative_change_tolerance) break;
      for (int j = 0; j < n; ++j) w.c[j] = latest[j];
    }
    if (ierror == 0) {
      // final RTAuxVarCompute (reaction.F90:4052)
      total_aqueous<NMAX, PF>(T, n, ns, sec_logK, st.sec_act_coef, st.sec_molal, cell, soa, cs, w);
      for (int j = 0; j < n; ++j) total_io[j] = w.total[j];
      if (has_sorb) sorb_eval();
    }
    its_total += its;
    // ---------------------------------------------------------- RStep control
    if (ierror != 0) {
      num_cuts = num_cuts + 1;
      if (num_cuts > o.maximum_reaction_cuts) {
        ierror_step = 1;
        break;
      }
      dt = 0.5 * dt;
      n_const = 0;
    } else {
      // RUpdateKineticState -> MineralUpdateKineticState
      if (nm > 0) {
        double dummy[NMAX];
        for (int j = 0; j < n; ++j) dummy[j] = 0.0;
        kinetic_mineral<NMAX, PF>(T, net, n, mnrl_logK, sec_logK, cell, soa, st, cs, w, dummy, nullptr);
        for (int m = 0; m < nm; ++m) {
          double vf = st.mnrl_volfrac[soa.at(m, cell)] + st.mnrl_rate[soa.at(m, cell)] * T.molar_vol(m) * dt;
          st.mnrl_volfrac[soa.at(m, cell)] = vf < 0.0 ? 0.0 : vf;
        }
      }
      cumulative = cumulative + dt;
      nsub += 1;
      n_const += 1;
      for (int j = 0; j < n; ++j) guess[j] = w.c[j];
      if (n_const >= 4) {
        num_cuts = num_cuts - 1;
        dt = fmin(2.0 * dt, target_time - cumulative);
      }
    }
  }
  if (!ierror_step)
    for (int j = 0; j < n; ++j)
      if (small_mask & (1u << j)) total_io[j] = small_val[j];
  for (int j = 0; j < n; ++j) {
    st.total[soa.at(j, cell)] = total_io[j];
    st.pri_molal[soa.at(j, cell)] = w.c[j];
    if (o.act_coef_update_frequency == PF_ACT_COEF_NEWTON_ITER) st.pri_act_coef[soa.at(j, cell)] = w.gamma[j];
  }
  if (PF && o.act_coef_update_frequency == PF_ACT_COEF_NEWTON_ITER && o.use_activity_h2o)
    st.ln_act_h2o[cell] = cs.lnaw;
  const int status = ierror_step ? PF_CELL_TOO_MANY_CUTS : PF_CELL_OK;
  if (st.status) st.status[cell] = status;
  if (st.newton_its) st.newton_its[cell] = its_total;
  if (st.num_substeps) st.num_substeps[cell] = nsub;
  if (counters) {
    atomicAdd(&counters[0], (unsigned long long)its_total);
    if (status) atomicAdd(&counters[1], 1ull);
    atomicMax(&counters[3], (unsigned long long)its_total);
    atomicMax(&counters[4], (unsigned long long)nsub);
  }
}

}  // namespace plain

int launch_rstep_plain(const DevNet& net, const PfCellState& st, double dt,
                       unsigned long long* counters, cudaStream_t stream) {
  const int tpb = 128;
  const int64_t blocks = (st.ncells + tpb - 1) / tpb;
  if (blocks == 0) return 0;
  if ((net.flags & NETF_PREFACTOR) || net.o.use_activity_h2o ||
      (net.o.act_coef_update_frequency == PF_ACT_COEF_NEWTON_ITER &&
       net.o.act_coef_update_algorithm == PF_ACT_COEF_ALGO_NEWTON)) {
    // rate prefactors, water activity or the NEWTON activity algorithm at
    // every Newton iteration: the extended instantiation, three size buckets
    if (net.n <= 8) plain::rstep_plain_kernel<8, true><<<blocks, tpb, 0, stream>>>(net, st, dt, counters);
    else if (net.n <= 12) plain::rstep_plain_kernel<12, true><<<blocks, tpb, 0, stream>>>(net, st, dt, counters);
    else plain::rstep_plain_kernel<24, true><<<blocks, tpb, 0, stream>>>(net, st, dt, counters);
  } else if (net.n <= 4) plain::rstep_plain_kernel<4, false><<<blocks, tpb, 0, stream>>>(net, st, dt, counters);
  else if (net.n <= 8) plain::rstep_plain_kernel<8, false><<<blocks, tpb, 0, stream>>>(net, st, dt, counters);
  else if (net.n <= 12) plain::rstep_plain_kernel<12, false><<<blocks, tpb, 0, stream>>>(net, st, dt, counters);
  else if (net.n <= 16) plain::rstep_plain_kernel<16, false><<<blocks, tpb, 0, stream>>>(net, st, dt, counters);
  else plain::rstep_plain_kernel<24, false><<<blocks, tpb, 0, stream>>>(net, st, dt, counters);
  return (int)cudaGetLastError();
}

}  // namespace pfgpu
