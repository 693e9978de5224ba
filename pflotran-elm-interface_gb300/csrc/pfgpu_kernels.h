// pfgpu_kernels.h -- launchers shared between the C-ABI translation unit and
// the kernel translation units.
#pragma once
#include "pfgpu_common.cuh"

namespace pfgpu {

// K1: one thread per cell, direct form (pfgpu_plain.cu)
int launch_rstep_plain(const DevNet& net, const PfCellState& st, double dt,
                       unsigned long long* counters, cudaStream_t stream);

// K2: persistent lane-refilling kernel (pfgpu_batched.cu).
// queue: device counter zeroed by the caller (cudaMemsetAsync) before launch.
// counters[0] += Newton iterations, counters[1] += failed cells,
// counters[2] = error flags (bit 0: table staging timed out).
int launch_rstep_batched(const DevNet& net, const PfCellState& st, double dt,
                         const PfLaunchConfig& cfg, int num_sms, double* scratch,
                         unsigned long long* queue, unsigned long long* counters,
                         cudaStream_t stream, const PfAdjointArgs* adj = nullptr);
// doubles of per-cell scratch the batched kernel's setup pre-pass writes
size_t batched_scratch_doubles(const DevNet& net, int64_t ncells);
// shared memory bytes a batched launch of this config needs
size_t batched_smem_bytes(const DevNet& net, const PfLaunchConfig& cfg);
bool batched_supported(const DevNet& net);

// auxvar kernels (pfgpu_aux.cu)
int launch_update_auxvars(const DevNet& net, const PfCellState& st, int update_act,
                          cudaStream_t stream);
int launch_update_activity_coefs(const DevNet& net, const PfCellState& st, cudaStream_t stream);

}  // namespace pfgpu
