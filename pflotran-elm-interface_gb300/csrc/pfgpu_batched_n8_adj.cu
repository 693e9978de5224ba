// pfgpu_batched_n8_adj.cu -- batched kernel, adjoint variants, ncomp = 8.
#include "pfgpu_batched.cuh"

namespace pfgpu {
int launch_batched_adj_8(const DevNet& net, const PfCellState& st, double dt, const PfLaunchConfig& cfg,
                          int num_sms, const double* scratch, unsigned long long* queue,
                          unsigned long long* counters, const PfAdjointArgs& adj, cudaStream_t stream) {
  return launch_batched_adj<8>(net, st, dt, cfg, num_sms, scratch, queue, counters, adj, stream);
}
}  // namespace pfgpu
