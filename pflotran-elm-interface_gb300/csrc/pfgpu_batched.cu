// pfgpu_batched.cu -- dispatch of the batched kernel over the compiled ncomp
// values; each instantiation lives in its own translation unit
// (pfgpu_batched_n*.cu) so they compile in parallel.
#include "pfgpu_common.cuh"
#include "pfgpu_kernels.h"

namespace pfgpu {

#define PF_BATCHED_NCOMPS(X) X(3) X(4) X(6) X(8) X(10) X(12) X(16) X(20) X(24)

#define PF_DECL(N)                                                                               \
  int launch_batched_##N(const DevNet&, const PfCellState&, double, const PfLaunchConfig&, int, \
                         const double*, unsigned long long*, unsigned long long*, const PfAdjointArgs*, \
                         cudaStream_t);
PF_BATCHED_NCOMPS(PF_DECL)
#undef PF_DECL

static size_t lane_doubles(int n, bool js) { return (js ? (size_t)n * n : 0) + 6 * (size_t)n; }

size_t batched_smem_bytes(const DevNet& net, const PfLaunchConfig& cfg) {
  if (cfg.lanes_per_cell > 1) return group_smem_bytes(net, cfg);
  const size_t tables = (size_t)net.int_words * 4 + (size_t)net.dbl_words * 8;
  const size_t lane = lane_doubles(net.n, cfg.jac_in_shared != 0) * 8 + (size_t)net.n * 4;
  return tables + lane * (size_t)cfg.threads_per_block;
}

bool batched_supported(const DevNet& net) {
  if (lane_supported(net)) return true;
  for (int g : {2, 4, 8})
    if (group_supported(net, g)) return true;
  return false;
}

bool lane_supported(const DevNet& net) {
  switch (net.n) {
#define PF_CASE(N) case N:
    PF_BATCHED_NCOMPS(PF_CASE)
#undef PF_CASE
      // rate prefactors add non-symmetric Jacobian terms the factorisation
      // here does not carry: the plain kernel runs those networks
      // water activity moving each Newton iteration: the plain kernel
      return net.ns <= PF_MAX_NSEC && net.nm <= PF_MAX_NMNRL && !(net.flags & NETF_PREFACTOR) &&
             !(net.o.act_coef_update_frequency == PF_ACT_COEF_NEWTON_ITER &&
               net.o.act_coef_update_algorithm == PF_ACT_COEF_ALGO_NEWTON) &&
             !(net.o.act_coef_update_frequency == PF_ACT_COEF_NEWTON_ITER && net.o.use_activity_h2o);
    default:
      return false;
  }
}

// Per-cell setup pre-pass: everything a cell needs once, computed by all
// lanes in step so the persistent kernel's refills are pure loads.
//   scratch[i][cell]        TIMESTEP/OFF: exp(-logK_i(T) ln10) / gamma_i
//                           NEWTON_ITER:  -logK_i(T) ln10
//   scratch[ns+m][cell]     exp(-logK_m(T) ln10)
//   scratch[ns+nm+j][cell]  ln of the initial guess of component j
// (the complexes' and minerals' entries with their reaction's water term,
// coefficient times ln a_H2O, in the exponent)
// logK(T) is ReactionInterpolateLogK (reaction_aux.F90:1285-1312) with ln T,
// 1/T and 1/T^2 formed once per cell.
__global__ void cell_setup_kernel(DevNet net, PfCellState st, double* __restrict__ scratch) {
  const int64_t cell = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= st.ncells) return;
  const Tables T{net.ints, net.dbls, &net};
  const SoA soa{st.ncells};
  const int n = net.n, ns = net.ns, nm = net.nm;
  const bool ni = net.o.act_coef_update_frequency == PF_ACT_COEF_NEWTON_ITER;
  const double temp = st.temperature ? st.temperature[cell] : 25.0;
  const double tk = temp + 273.15, lt = log(tk), it = 1.0 / tk, it2 = it * it;
  const bool tsec = !net.o.isothermal && (net.flags & NETF_SEC_LOGKCOEF);
  const bool tmin = !net.o.isothermal && (net.flags & NETF_MNRL_LOGKCOEF);
  const int64_t N = st.ncells;
  // ln a_H2O is constant over the step here (it follows the activity
  // coefficients, which move each Newton iteration only in a mode these
  // kernels refuse together with the water activity option)
  const bool h2o = water_on(net);
  const double lnaw = cell_lnaw(net, st, cell);
  for (int i = 0; i < ns; ++i) {
    double logK = T.sec_logK(i);
    if (tsec) {
      const double* c = T.sec_logKcoef(i);
      logK = c[0] * lt + c[1] + c[2] * tk + c[3] * it + c[4] * it2;
    }
    double x = -logK * LOG_TO_LN;
    if (h2o) x = add_h2o(x, T.sec_h2o(i), lnaw);
    scratch[(size_t)i * N + cell] = ni ? x : exp(x) / st.sec_act_coef[soa.at(i, cell)];
  }
  for (int m = 0; m < nm; ++m) {
    double logK = T.mnrl_logK(m);
    if (tmin) {
      const double* c = T.mnrl_logKcoef(m);
      logK = c[0] * lt + c[1] + c[2] * tk + c[3] * it + c[4] * it2;
    }
    // K = 10^-logK in every mode: Q/K multiplies it by the activities'
    // powers (only the complexes' constants carry gamma and stay in log
    // form when gamma follows each Newton iteration)
    double x = -logK * LOG_TO_LN;
    if (h2o) x = add_h2o(x, T.mnrl_h2o(m), lnaw);
    scratch[(size_t)(ns + m) * N + cell] = exp(x);
  }
  for (int j = 0; j < n; ++j) {
    double v = net.o.use_total_as_guess ? st.total[soa.at(j, cell)] : st.pri_molal[soa.at(j, cell)];
    if (net.o.use_total_as_guess && v <= 1.0e-40) v = 1.0e-40;
    scratch[(size_t)(ns + nm + j) * N + cell] = log(v);
  }
}

size_t batched_scratch_doubles(const DevNet& net, int64_t ncells) {
  return (size_t)(net.ns + net.nm + net.n) * (size_t)ncells;
}

int launch_cell_setup(const DevNet& net, const PfCellState& st, double* scratch, cudaStream_t stream) {
  const int tpb = 128;
  const int64_t blocks = (st.ncells + tpb - 1) / tpb;
  if (blocks) cell_setup_kernel<<<blocks, tpb, 0, stream>>>(net, st, scratch);
  return (int)cudaGetLastError();
}

int launch_rstep_batched(const DevNet& net, const PfCellState& st, double dt, const PfLaunchConfig& cfg,
                         int num_sms, double* scratch, unsigned long long* queue, unsigned long long* counters,
                         cudaStream_t stream, const PfAdjointArgs* adj, double* adj_store) {
  const bool grp = cfg.lanes_per_cell > 1 && (!adj || adj_store);
  // a group configuration the network's current options rule out (the group
  // kernel reads neither the linear formulation nor the other refused modes)
  if (grp && !group_supported(net, cfg.lanes_per_cell)) return (int)cudaErrorInvalidConfiguration;
  {
    const int e = launch_cell_setup(net, st, scratch, stream);
    if (e) return e;
  }
  if (grp)
    return launch_rstep_group(net, net.grp, st, dt, cfg, num_sms, scratch, queue, counters, stream, adj,
                              adj_store);
  switch (net.n) {
#define PF_CASE(N) \
  case N:          \
    return launch_batched_##N(net, st, dt, cfg, num_sms, scratch, queue, counters, adj, stream);
    PF_BATCHED_NCOMPS(PF_CASE)
#undef PF_CASE
    default:
      return -1;
  }
}

}  // namespace pfgpu
