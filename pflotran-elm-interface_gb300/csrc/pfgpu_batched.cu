// pfgpu_batched.cu -- dispatch of the batched kernel over the compiled ncomp
// values; each instantiation lives in its own translation unit
// (pfgpu_batched_n*.cu) so they compile in parallel.
#include "pfgpu_common.cuh"
#include "pfgpu_kernels.h"

namespace pfgpu {

#define PF_BATCHED_NCOMPS(X) X(3) X(4) X(6) X(8) X(10) X(12) X(16) X(20) X(24)

#define PF_DECL(N)                                                                               \
  int launch_batched_##N(const DevNet&, const PfCellState&, double, const PfLaunchConfig&, int, \
                         unsigned long long*, unsigned long long*, cudaStream_t);
PF_BATCHED_NCOMPS(PF_DECL)
#undef PF_DECL

static size_t lane_doubles(int n, bool js) { return (js ? (size_t)n * n : 0) + 3 * (size_t)n; }

size_t batched_smem_bytes(const DevNet& net, const PfLaunchConfig& cfg) {
  const size_t tables = (size_t)net.int_words * 4 + (size_t)net.dbl_words * 8;
  const size_t lane = lane_doubles(net.n, cfg.jac_in_shared != 0) * 8 + (size_t)net.n * 4;
  return tables + lane * (size_t)cfg.threads_per_block;
}

bool batched_supported(const DevNet& net) {
  switch (net.n) {
#define PF_CASE(N) case N:
    PF_BATCHED_NCOMPS(PF_CASE)
#undef PF_CASE
      return net.ns <= PF_MAX_NSEC && net.nm <= PF_MAX_NMNRL &&
             !(net.o.act_coef_update_frequency == PF_ACT_COEF_NEWTON_ITER &&
               net.o.act_coef_update_algorithm == PF_ACT_COEF_ALGO_NEWTON);
    default:
      return false;
  }
}

int launch_rstep_batched(const DevNet& net, const PfCellState& st, double dt, const PfLaunchConfig& cfg,
                         int num_sms, unsigned long long* queue, unsigned long long* counters,
                         cudaStream_t stream) {
  switch (net.n) {
#define PF_CASE(N) \
  case N:          \
    return launch_batched_##N(net, st, dt, cfg, num_sms, queue, counters, stream);
    PF_BATCHED_NCOMPS(PF_CASE)
#undef PF_CASE
    default:
      return -1;
  }
}

}  // namespace pfgpu
