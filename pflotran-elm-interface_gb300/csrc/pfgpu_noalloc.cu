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
// symbol is only a stand-in; the address must come from the runtime, once per
// device, with that device current (the first call on a device does this; it
// must therefore happen before any stream capture that includes the call).
int scratch_for_current_device(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return PF_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, pf_noalloc_scratch) != cudaSuccess || !p) return PF_ERR_CUDA;
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_ptr[dev];
  return PF_OK;
}
}  // namespace

// Helpers from pfgpu_api.cu (the network's resident launch state).
extern "C" int32_t pf_internal_network_view(PfNetwork* net, pfgpu::DevNet* dev, PfLaunchConfig* cfg,
                                            int* num_sms, unsigned long long** counters);
extern "C" int32_t pf_internal_validate_state(PfNetwork* net, const PfCellState* state);

extern "C" int32_t pf_rstep_noalloc(PfNetwork* net, const PfCellState* state, double dt, void* stream) {
  using namespace pfgpu;
  int rc = pf_internal_validate_state(net, state);
  if (rc) return rc;
  if (!(dt > 0.0) && !state->dt_cell) return PF_ERR_INVALID;
  DevNet dev;
  PfLaunchConfig cfg;
  int sms = 0;
  unsigned long long* counters = nullptr;
  rc = pf_internal_network_view(net, &dev, &cfg, &sms, &counters);
  if (rc) return rc;
  if (!batched_supported(dev)) return PF_ERR_UNSUPPORTED;
  if (state->ncells == 0) return PF_OK;
  if (batched_scratch_doubles(dev, state->ncells) > (size_t)PF_NOALLOC_SCRATCH_DOUBLES) return PF_ERR_TOO_LARGE;
  double* scratch = nullptr;
  rc = scratch_for_current_device(&scratch);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  // the work-queue counter and reduction slots must start at zero; the
  // scratch needs no clearing (the setup pre-pass writes every value it reads)
  if (cudaMemsetAsync(counters, 0, 8 * sizeof(unsigned long long), s) != cudaSuccess) return PF_ERR_CUDA;
  if (launch_rstep_batched(dev, *state, dt, cfg, sms, scratch, counters, counters + 1, s) != 0) return PF_ERR_CUDA;
  return PF_OK;
}
