// FP64 path: the executors of the factor phase instantiated for double tiles (no tensor-memory stages)
// (one translation unit per precision and operand-stage count, so the build
// compiles them in parallel; the device code is in factor_impl.cuh).
#include "factor_impl.cuh"
#include "factor_units.h"

namespace sog {

int run_executor_f64(int which, const DevTasks& t, double* tiles, const int32_t* items, int nitems, int grid, cudaStream_t s) {
    return run_executor<double, 2>(which, t, tiles, items, nitems, grid, s);
}
int residency_f64() { return persistent_residency<double, 2>(); }

}  // namespace sog
