// Mixed path, two operand stages: the executors of the factor phase instantiated for FP32 tiles with two tcgen05 operand stages
// (one translation unit per precision and operand-stage count, so the build
// compiles them in parallel; the device code is in factor_impl.cuh).
#include "factor_impl.cuh"
#include "factor_units.h"

namespace sog {

int run_executor_f32_s2(int which, const DevTasks& t, float* tiles, const int32_t* items, int nitems, int grid, cudaStream_t s) {
    return run_executor<float, 2>(which, t, tiles, items, nitems, grid, s);
}
int residency_f32_s2() { return persistent_residency<float, 2>(); }

}  // namespace sog
