/*
 * pfgpu_bench.h -- measurement helpers shipped with the engine (not part of
 * the reference-facing interface).
 */
#ifndef PFGPU_BENCH_H_
#define PFGPU_BENCH_H_
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
/* FP64 FMA throughput probe: blocks x threads threads, each running 8
 * independent DFMA chains for iters iterations (16*iters flops per thread);
 * out (device, blocks*threads doubles) receives the chain sums so nothing is
 * dead code.  The caller times the launch on the given stream. */
int32_t pf_bench_fp64_fma(double* out, int64_t iters, int32_t blocks, int32_t threads, void* stream);
#ifdef __cplusplus
}
#endif
#endif
