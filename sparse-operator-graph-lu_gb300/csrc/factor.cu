// Factor-phase entry points (kernels.h): dispatch to the executors of the
// per-precision translation units, and the element-wise kernels that move
// input values into tiles and tiles between precisions.
#include <cuda_runtime.h>

#include <stdint.h>

#include "factor_units.h"
#include "kernels.h"

namespace sog {

namespace {

// input tiles from the caller's values; vidx (symmetric input): value index of
// each mirrored triplet
__global__ void scatter_kernel(const double* __restrict__ V, const int32_t* __restrict__ vidx,
                               const int32_t* __restrict__ tile, const int16_t* __restrict__ off, int64_t nnz,
                               const int32_t* __restrict__ pad_tile, const int16_t* __restrict__ pad_off, int64_t npad,
                               double* t64, float* t32) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nnz) {
        const int32_t tl = tile[i];
        if (tl >= 0) {
            const int64_t e = (int64_t)tl * 4096 + off[i];
            const double v = V[vidx ? vidx[i] : i];
            if (t64) t64[e] = v;
            else t32[e] = (float)v;
        }
    } else if (i - nnz < npad) {
        const int64_t k = i - nnz;
        const int64_t e = (int64_t)pad_tile[k] * 4096 + pad_off[k];
        if (t64) t64[e] = 1.0;
        else t32[e] = 1.0f;
    }
}

__global__ void convert_kernel(const double* __restrict__ s, float* __restrict__ d, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        d[i] = (float)s[i];
}
__global__ void widen_kernel(const float* __restrict__ s, double* __restrict__ d, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        d[i] = (double)s[i];
}

}  // namespace

// The FP64 path has no tensor-memory stages (its stage argument is unused).
int factor_queue_launch(const DevTasks& t, double* tiles, int grid, int, cudaStream_t s) {
    return run_executor_f64(0, t, tiles, nullptr, 0, grid, s);
}
int factor_queue_launch(const DevTasks& t, float* tiles, int grid, int stages, cudaStream_t s) {
    return stages == 1 ? run_executor_f32_s1(0, t, tiles, nullptr, 0, grid, s)
                       : run_executor_f32_s2(0, t, tiles, nullptr, 0, grid, s);
}
int factor_ordered_launch(const DevTasks& t, double* tiles, int grid, int, cudaStream_t s) {
    return run_executor_f64(1, t, tiles, nullptr, 0, grid, s);
}
int factor_ordered_launch(const DevTasks& t, float* tiles, int grid, int stages, cudaStream_t s) {
    return stages == 1 ? run_executor_f32_s1(1, t, tiles, nullptr, 0, grid, s)
                       : run_executor_f32_s2(1, t, tiles, nullptr, 0, grid, s);
}
int factor_level_launch(const DevTasks& t, double* tiles, const int32_t* items, int nitems, int, cudaStream_t s) {
    return run_executor_f64(2, t, tiles, items, nitems, 0, s);
}
int factor_level_launch(const DevTasks& t, float* tiles, const int32_t* items, int nitems, int stages,
                        cudaStream_t s) {
    return stages == 1 ? run_executor_f32_s1(2, t, tiles, items, nitems, 0, s)
                       : run_executor_f32_s2(2, t, tiles, items, nitems, 0, s);
}

int factor_persistent_grid(bool fp64, int stages, int num_sms) {
    const int per_sm = fp64 ? residency_f64() : (stages == 1 ? residency_f32_s1() : residency_f32_s2());
    return per_sm * num_sms;
}

void scatter_values_launch(const double* V, const int32_t* vidx, const int32_t* tile, const int16_t* off, int64_t nnz,
                           const int32_t* pad_tile, const int16_t* pad_off, int64_t npad, double* tiles64,
                           float* tiles32, cudaStream_t s) {
    const int64_t n = nnz + npad;
    if (n == 0) return;
    scatter_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(V, vidx, tile, off, nnz, pad_tile, pad_off, npad,
                                                               tiles64, tiles32);
}
void convert_tiles_launch(const double* src, float* dst, int64_t n, cudaStream_t s) {
    if (n > 0) convert_kernel<<<1216, 256, 0, s>>>(src, dst, n);
}
void widen_tiles_launch(const float* src, double* dst, int64_t n, cudaStream_t s) {
    if (n > 0) widen_kernel<<<1216, 256, 0, s>>>(src, dst, n);
}

}  // namespace sog
