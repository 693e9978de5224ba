// pfgpu_noalloc.cu -- the batched operator-split step without any device
// allocation in the call.
//
// pf_rstep normally keeps its per-cell scratch (the setup pre-pass output,
// (ncomp + nsec + nmnrl) doubles per cell) in a buffer it grows with
// cudaMalloc.  Some callers cannot allow that: a host model whose GPU memory
// is owned by another framework's pool, or a coupled run that fixes its
// device footprint up front.
// pf_rstep_noalloc runs the same kernels with the scratch in a fixed,
// file-scope device array instead, so the call itself never allocates.
#include <mutex>

#include "pfgpu_common.cuh"
#include "pfgpu_kernels.h"

// 32 MiB of FP64 scratch, resident on every device that loads the library
// until the process exits.  It bounds (ncomp + nsec + nmnrl) * ncells.
#define PF_NOALLOC_SCRATCH_DOUBLES (4u * 1024u * 1024u)

static __device__ __align__(256) double pf_noalloc_scratch[PF_NOALLOC_SCRATCH_DOUBLES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_mutex;
double* g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of the static array on the current device.  The host-side
// symbol is only a stand-in; the address must come from the runtime with that
// device current.  It is looked up afresh on every call outside a stream
// capture (a cudaDeviceReset reloads the module, and the array may move), and
// the last address is used inside one (so a captured call needs one earlier
// call on the device outside the capture).
int scratch_for_current_device(cudaStream_t stream, double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return PF_ERR_CUDA;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(stream, &cap) != cudaSuccess) return PF_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_mutex);
  if (cap == cudaStreamCaptureStatusNone) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, pf_noalloc_scratch) != cudaSuccess || !p) return PF_ERR_CUDA;
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  if (!g_scratch_ptr[dev]) return PF_ERR_CUDA;
  *out = g_scratch_ptr[dev];
  return PF_OK;
}
}  // namespace

// Helpers from pfgpu_api.cu (the network's resident launch state, the
// argument checks of pf_rstep and its read-back of the step counters into the
// network's pinned mirror).
extern "C" int32_t pf_internal_network_view(PfNetwork* net, pfgpu::DevNet* dev, PfLaunchConfig* cfg,
                                            int* num_sms, unsigned long long** counters);
extern "C" int32_t pf_internal_check_rstep(PfNetwork* net, const PfCellState* state, double dt);
extern "C" int32_t pf_internal_read_step_stats(PfNetwork* net, int64_t ncells, void* stream, PfStepStats* stats);

extern "C" int32_t pf_rstep_noalloc(PfNetwork* net, const PfCellState* state, double dt, void* stream,
                                    PfStepStats* stats) {
  using namespace pfgpu;
  int rc = pf_internal_check_rstep(net, state, dt);
  if (rc) return rc;
  DevNet dev;
  PfLaunchConfig cfg;
  int sms = 0;
  unsigned long long* counters = nullptr;
  rc = pf_internal_network_view(net, &dev, &cfg, &sms, &counters);
  if (rc) return rc;
  if (state->ncells == 0) {
    if (stats) *stats = PfStepStats{};
    return PF_OK;
  }
  if (batched_scratch_doubles(dev, state->ncells) > (size_t)PF_NOALLOC_SCRATCH_DOUBLES) return PF_ERR_TOO_LARGE;
  cudaStream_t s = (cudaStream_t)stream;
  double* scratch = nullptr;
  rc = scratch_for_current_device(s, &scratch);
  if (rc) return rc;
  // the work-queue counter and reduction slots must start at zero; the
  // scratch needs no clearing (the setup pre-pass writes every value it reads
  // before the step kernel reads it)
  if (cudaMemsetAsync(counters, 0, 8 * sizeof(unsigned long long), s) != cudaSuccess) return PF_ERR_CUDA;
  // every byte 0xFF: status PF_CELL_NOT_RUN (-1) until the kernel finishes the
  // cell, so a launch that gave up early (a table-staging wait that ran out)
  // shows in the status array even without stats
  if (state->status && cudaMemsetAsync(state->status, 0xFF, (size_t)state->ncells * sizeof(int32_t), s) != cudaSuccess)
    return PF_ERR_CUDA;
  if (launch_rstep_batched(dev, *state, dt, cfg, sms, scratch, counters, counters + 1, s) != 0) return PF_ERR_CUDA;
  if (!stats) return PF_OK;
  return pf_internal_read_step_stats(net, state->ncells, stream, stats);
}
