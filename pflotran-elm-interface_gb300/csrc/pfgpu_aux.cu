// pfgpu_aux.cu -- per-cell auxiliary-variable kernels (one thread per cell).
//
//   update_auxvars          RTUpdateAuxVars for cells (reactive_transport.F90:
//                           3625-3660): optional RActivityCoefficients, then
//                           RTotal/RTotalAqueous (reaction.F90:4618-4759) ->
//                           total, sec_molal; with sorption RTotalSorb
//                           (:4783-4832) -> total_sorb, the ion-exchange warm
//                           start.
//   update_activity_coefs   RTUpdateActivityCoefficients (reactive_transport.F90:
//                           3441-3521): RActivityCoefficients only, both the LAG
//                           (reaction.F90:4553-4612) and NEWTON (:4403-4551)
//                           algorithms.
// These are memory-light, exp-dominated kernels; the layout is the same SoA as
// the step kernels, so consecutive threads read consecutive cells.
#include "pfgpu_common.cuh"
#include "pfgpu_kernels.h"
#include "pfgpu_sorb.cuh"

namespace pfgpu {
namespace aux {

__device__ __forceinline__ double dh_lngamma(double z, double a0, double sqrtI, double I, const DevNet& net) {
  // exponent of exp() in RActivityCoefficients: log gamma in natural units
  return (-z * z * sqrtI * net.A / (1.0 + a0 * net.B * sqrtI) + net.Bdot * I) * LOG_TO_LN;
}

__device__ void activity(const DevNet& net, const Tables& T, const PfCellState& st, const SoA& soa,
                         int64_t cell, double temp) {
  const int n = net.n, ns = net.ns;
  const bool h2o = net.o.use_activity_h2o != 0;  // validate_state: st.ln_act_h2o is then present
  double sum_pri_molal = 0.0;
  if (h2o)
    for (int j = 0; j < n; ++j) sum_pri_molal = sum_pri_molal + st.pri_molal[soa.at(j, cell)];
  if (net.o.act_coef_update_algorithm == PF_ACT_COEF_ALGO_NEWTON) {
    double lnaw = cell_lnaw(net, st, cell);
    double ln_act[PF_MAX_NCOMP];
    for (int j = 0; j < n; ++j)
      ln_act[j] = log(st.pri_molal[soa.at(j, cell)]) + log(st.pri_act_coef[soa.at(j, cell)]);
    double fpri = 0.0;
    for (int j = 0; j < n; ++j) fpri = fpri + st.pri_molal[soa.at(j, cell)] * T.pri_Z(j) * T.pri_Z(j);
    const bool tsec = !net.o.isothermal && (net.flags & NETF_SEC_LOGKCOEF);
    double II = 0.0;
    for (int it = 1;; ++it) {
      if (it > 50) {  // reaction.F90:4420-4431: NaN everything, flag the cell
        for (int j = 0; j < n; ++j) {
          st.pri_molal[soa.at(j, cell)] = __longlong_as_double(0x7ff8000000000000ll);
          st.pri_act_coef[soa.at(j, cell)] = __longlong_as_double(0x7ff8000000000000ll);
        }
        for (int i = 0; i < ns; ++i) st.sec_act_coef[soa.at(i, cell)] = __longlong_as_double(0x7ff8000000000000ll);
        if (st.status) st.status[cell] = PF_CELL_NAN;
        return;
      }
      double I = fpri;
      for (int i = 0; i < ns; ++i) I = I + st.sec_molal[soa.at(i, cell)] * T.sec_Z(i) * T.sec_Z(i);
      I = 0.5 * I;
      const double f = I;
      if (fabs(I - II) < 1.0e-6 * I) break;
      if (ns > 0) {
        double didi = 0.0;
        const double sqrt_I = sqrt(I);
        for (int i = 0; i < ns; ++i) {
          const double zi = T.sec_Z(i);
          if (fabs(zi) > 0.0) {
            const double t = 1.0 + net.B * T.sec_a0(i) * sqrt_I;
            double sum = 0.5 * net.A * zi * zi / (sqrt_I * (t * t)) - net.Bdot;
            for (int p = T.sec_begin(i); p < T.sec_end(i); ++p) {
              const int j = T.sec_idx(p);
              const double zj = T.pri_Z(j);
              if (fabs(zj) > 0.0) {
                const double tj = 1.0 + net.B * T.pri_a0(j) * sqrt_I;
                const double dgamdi = -0.5 * net.A * (zj * zj) / (sqrt_I * (tj * tj)) + net.Bdot;
                sum = sum + T.sec_nu(p) * dgamdi;
              }
            }
            const double dcdi = st.sec_molal[soa.at(i, cell)] * LOG_TO_LN * sum;
            didi = didi + 0.5 * zi * zi * dcdi;
          }
        }
        const double den = 1.0 - didi;
        II = fabs(den) > 0.0 ? (f - I * didi) / den : f;
      } else {
        II = f;
      }
      if (II < 0.0) {
        if (st.status) st.status[cell] = PF_CELL_NAN;
        return;
      }
      I = II;
      const double sqrt_I = sqrt(I);
      for (int j = 0; j < n; ++j) {
        const double z = T.pri_Z(j);
        st.pri_act_coef[soa.at(j, cell)] = fabs(z) > 0.0 ? exp(dh_lngamma(z, T.pri_a0(j), sqrt_I, I, net)) : 1.0;
      }
      double sum_sec_molal = 0.0;
      for (int i = 0; i < ns; ++i) {
        const double z = T.sec_Z(i);
        const double g = fabs(z) > 0.0 ? exp(dh_lngamma(z, T.sec_a0(i), sqrt_I, I, net)) : 1.0;
        st.sec_act_coef[soa.at(i, cell)] = g;
        const double logK = tsec ? interp_logK(T.sec_logKcoef(i), temp) : T.sec_logK(i);
        double lnQK = add_h2o(-logK * LOG_TO_LN, T.sec_h2o(i), lnaw);
        for (int p = T.sec_begin(i); p < T.sec_end(i); ++p) lnQK = lnQK + T.sec_nu(p) * ln_act[T.sec_idx(p)];
        const double sm = exp(lnQK) / g;
        st.sec_molal[soa.at(i, cell)] = sm;
        sum_sec_molal = sum_sec_molal + sm;
      }
      if (h2o) {
        lnaw = water_activity(sum_pri_molal, sum_sec_molal);
        st.ln_act_h2o[cell] = lnaw;
      }
    }
    return;
  }
  double I = 0.0;
  for (int j = 0; j < n; ++j) I = I + st.pri_molal[soa.at(j, cell)] * T.pri_Z(j) * T.pri_Z(j);
  for (int i = 0; i < ns; ++i) I = I + st.sec_molal[soa.at(i, cell)] * T.sec_Z(i) * T.sec_Z(i);
  I = 0.5 * I;
  const double sqrt_I = sqrt(I);
  for (int j = 0; j < n; ++j) {
    const double z = T.pri_Z(j);
    st.pri_act_coef[soa.at(j, cell)] = fabs(z) > 1.0e-10 ? exp(dh_lngamma(z, T.pri_a0(j), sqrt_I, I, net)) : 1.0;
  }
  double sum_sec_molal = 0.0;
  for (int i = 0; i < ns; ++i) {
    const double z = T.sec_Z(i);
    st.sec_act_coef[soa.at(i, cell)] = fabs(z) > 1.0e-10 ? exp(dh_lngamma(z, T.sec_a0(i), sqrt_I, I, net)) : 1.0;
    sum_sec_molal = sum_sec_molal + st.sec_molal[soa.at(i, cell)];
  }
  if (h2o) st.ln_act_h2o[cell] = water_activity(sum_pri_molal, sum_sec_molal);
}

__device__ void total(const DevNet& net, const Tables& T, const PfCellState& st, const SoA& soa, int64_t cell,
                      double temp) {
  const int n = net.n, ns = net.ns;
  double lnc[PF_MAX_NCOMP], lna[PF_MAX_NCOMP], tot[PF_MAX_NCOMP];
  for (int j = 0; j < n; ++j) {
    const double m = st.pri_molal[soa.at(j, cell)];
    lnc[j] = log(m);
    lna[j] = lnc[j] + log(st.pri_act_coef[soa.at(j, cell)]);
    tot[j] = m;
  }
  const bool tsec = !net.o.isothermal && (net.flags & NETF_SEC_LOGKCOEF);
  const double lnaw = cell_lnaw(net, st, cell);
  for (int i = 0; i < ns; ++i) {
    const double logK = tsec ? interp_logK(T.sec_logKcoef(i), temp) : T.sec_logK(i);
    double lnQK = add_h2o(-logK * LOG_TO_LN, T.sec_h2o(i), lnaw);
    for (int p = T.sec_begin(i); p < T.sec_end(i); ++p) lnQK = lnQK + T.sec_nu(p) * lna[T.sec_idx(p)];
    const double s = exp(lnQK) / st.sec_act_coef[soa.at(i, cell)];
    st.sec_molal[soa.at(i, cell)] = s;
    for (int p = T.sec_begin(i); p < T.sec_end(i); ++p) tot[T.sec_idx(p)] = tot[T.sec_idx(p)] + T.sec_nu(p) * s;
  }
  const double den_L = st.den_kg[cell] * 1.0e-3;
  for (int j = 0; j < n; ++j) st.total[soa.at(j, cell)] = tot[j] * den_L;
  if (has_sorption(net)) {
    for (int j = 0; j < n; ++j) st.total_sorb[soa.at(j, cell)] = 0.0;
    // RTotal without ierror (RTUpdateAuxVars): a failed ion-exchange solve
    // leaves the last iterate, as the reference's message-and-continue does
    total_sorb(
        net, T, [&](int j) { return st.pri_molal[soa.at(j, cell)]; },
        [&](int j) { return st.pri_act_coef[soa.at(j, cell)]; },
        [&](int m) { return st.mnrl_volfrac[soa.at(m, cell)]; }, st.porosity[cell], st.den_kg[cell],
        st.ionx_ref_sorbed ? st.ionx_ref_sorbed + cell : nullptr, st.ncells,
        [&](int j, double v) { st.total_sorb[soa.at(j, cell)] += v; }, [](int, int, double) {},
        surf_cell(net, st, cell));
  }
}

__global__ void update_auxvars_kernel(DevNet net, PfCellState st, int update_act) {
  const int64_t cell = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= st.ncells) return;
  const Tables T{net.ints, net.dbls, &net};
  const SoA soa{st.ncells};
  const double temp = st.temperature ? st.temperature[cell] : 25.0;
  if (update_act) activity(net, T, st, soa, cell, temp);
  total(net, T, st, soa, cell, temp);
}

__global__ void update_activity_kernel(DevNet net, PfCellState st) {
  const int64_t cell = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= st.ncells) return;
  const Tables T{net.ints, net.dbls, &net};
  const SoA soa{st.ncells};
  activity(net, T, st, soa, cell, st.temperature ? st.temperature[cell] : 25.0);
}

}  // namespace aux

int launch_update_auxvars(const DevNet& net, const PfCellState& st, int update_act, cudaStream_t stream) {
  const int tpb = 128;
  const int64_t blocks = (st.ncells + tpb - 1) / tpb;
  if (blocks) aux::update_auxvars_kernel<<<blocks, tpb, 0, stream>>>(net, st, update_act);
  return (int)cudaGetLastError();
}

int launch_update_activity_coefs(const DevNet& net, const PfCellState& st, cudaStream_t stream) {
  const int tpb = 128;
  const int64_t blocks = (st.ncells + tpb - 1) / tpb;
  if (blocks) aux::update_activity_kernel<<<blocks, tpb, 0, stream>>>(net, st);
  return (int)cudaGetLastError();
}

}  // namespace pfgpu
