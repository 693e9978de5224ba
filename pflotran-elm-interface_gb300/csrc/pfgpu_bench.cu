// pfgpu_bench.cu -- FP64 pipe throughput probe (denominator of the FP64
// roofline): independent DFMA chains, no memory traffic in the loop.
#include <cuda_runtime.h>

#include "../../include/pfgpu_bench.h"

namespace {
__global__ void fp64_fma_kernel(double* out, int64_t iters) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = 1.0 + 1.0e-9 * (tid + k);
  const double m = 0.9999999999, c = 1.0e-12;
  for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma(a[k], m, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  out[tid] = s;
}
}  // namespace

extern "C" int32_t pf_bench_fp64_fma(double* out, int64_t iters, int32_t blocks, int32_t threads,
                                     void* stream) {
  if (!out || iters < 1 || blocks < 1 || threads < 32 || threads > 1024) return -1;
  fp64_fma_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(out, iters);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}
