// pfgpu_batched_n24.cu -- batched kernel, forward variants, ncomp = 24.
#include "pfgpu_batched.cuh"

namespace pfgpu {
int launch_batched_adj_24(const DevNet& net, const PfCellState& st, double dt, const PfLaunchConfig& cfg,
                          int num_sms, const double* scratch, unsigned long long* queue,
                          unsigned long long* counters, const PfAdjointArgs& adj, cudaStream_t stream);

int launch_batched_24(const DevNet& net, const PfCellState& st, double dt, const PfLaunchConfig& cfg,
                      int num_sms, const double* scratch, unsigned long long* queue,
                      unsigned long long* counters, const PfAdjointArgs* adj, cudaStream_t stream) {
  if (adj) return launch_batched_adj_24(net, st, dt, cfg, num_sms, scratch, queue, counters, *adj, stream);
  return launch_batched_fwd<24>(net, st, dt, cfg, num_sms, scratch, queue, counters, stream);
}
}  // namespace pfgpu
