// Entry points of the per-precision factor translation units (factor_f64.cu,
// factor_f32_s1.cu, factor_f32_s2.cu), dispatched from factor.cu.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.h"

namespace sog {
// which: 0 = persistent ready queue, 1 = persistent static order, 2 = per level (items, nitems)
int run_executor_f64(int which, const DevTasks& t, double* tiles, const int32_t* items, int nitems, int grid,
                     cudaStream_t s);
int run_executor_f32_s1(int which, const DevTasks& t, float* tiles, const int32_t* items, int nitems, int grid,
                        cudaStream_t s);
int run_executor_f32_s2(int which, const DevTasks& t, float* tiles, const int32_t* items, int nitems, int grid,
                        cudaStream_t s);
// persistent CTAs per SM
int residency_f64();
int residency_f32_s1();
int residency_f32_s2();
}  // namespace sog
