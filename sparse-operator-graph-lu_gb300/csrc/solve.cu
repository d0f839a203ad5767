// Solve-phase kernels for sm_103a: block forward (L) and back (U)
// substitution over the resident factor tiles (BlockPlanner::solve,
// BlockPlanner.cpp:652-862), the FP64 residual r = b - A x on the permuted
// matrix for iterative refinement, and the permutation gathers.
//
// Substitution runs as one persistent launch per triangle. Block rows are
// dealt round-robin to co-resident CTAs; a CTA folds in each off-diagonal
// block as soon as the block row it multiplies is published (a per-row
// readiness flag), then solves its diagonal block and publishes its own row.
// Rows only wait on rows dealt earlier, so the smallest unfinished row can
// always proceed; every wait is bounded and reports a timeout status.
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.h"

namespace sog {

namespace {

constexpr int NT = 256;
constexpr int LD = 65;

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ int ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// smem: Ts[64][LD] | Vs[64*nrhs] | Acc[64*nrhs]
template <typename T>
__global__ void __launch_bounds__(NT) trisolve_kernel(DevSolve s, const T* __restrict__ tiles, T* vec, int nrhs,
                                                      int epoch, int lower) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* Ts = reinterpret_cast<T*>(smem_raw);
    T* Vs = Ts + 64 * LD;
    T* Acc = Vs + 64 * nrhs;
    __shared__ int s_stop;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int R = s.block_rows;
    const int nv = 64 * nrhs;
    const int my_epoch = lower ? epoch : epoch + 1;
    const int* ptr = lower ? s.l_ptr : s.u_ptr;
    const int* col = lower ? s.l_col : s.u_col;
    const int* ids = lower ? s.l_id : s.u_id;
    const int* diag = lower ? s.l_diag : s.u_diag;
    if (tid == 0) s_stop = 0;
    for (int k = blockIdx.x; k < R; k += gridDim.x) {
        const int i = lower ? k : R - 1 - k;
        for (int e = tid; e < nv; e += NT) Acc[e] = __ldcg(vec + (size_t)i * nv + e);
        for (int q = ptr[i]; q < ptr[i + 1]; q++) {
            const int j = col[q];
            if (tid == 0) {
                const unsigned long long t0 = globaltimer_ns();
                unsigned ns = 32;
                while (ld_acquire(s.flags + j) != my_epoch) {
                    if (globaltimer_ns() - t0 > s.wait_limit_ns) {
                        atomicOr(&s.status->flags, ST_SOLVE_TIMEOUT);
                        s_stop = 1;
                        break;
                    }
                    __nanosleep(ns);
                    if (ns < 512) ns *= 2;
                }
                __threadfence();
            }
            __syncthreads();
            if (s_stop) return;
            const T* B = tiles + (size_t)ids[q] * 4096;
            const T* vj = vec + (size_t)j * nv;
            if (nrhs == 1) {
                if (tid < 64) Vs[tid] = __ldcg(vj + tid);
                __syncthreads();
                // warp w: rows w*8..w*8+7; lanes stream the row (coalesced)
                for (int r = warp * 8; r < warp * 8 + 8; r++) {
                    T v = __ldcg(B + r * 64 + lane) * Vs[lane] + __ldcg(B + r * 64 + lane + 32) * Vs[lane + 32];
                    v = warp_sum(v);
                    if (lane == 0) Acc[r] -= v;
                }
            } else {
                for (int e = tid; e < 4096; e += NT) Ts[(e >> 6) * LD + (e & 63)] = __ldcg(B + e);
                for (int e = tid; e < nv; e += NT) Vs[e] = __ldcg(vj + e);
                __syncthreads();
                for (int e = tid; e < nv; e += NT) {
                    const int r = e / nrhs, c = e - r * nrhs;
                    T acc = T(0);
#pragma unroll 8
                    for (int kk = 0; kk < 64; kk++) acc += Ts[r * LD + kk] * Vs[kk * nrhs + c];
                    Acc[e] -= acc;
                }
            }
            __syncthreads();
        }
        // diagonal block: row-sequential substitution, one warp per rhs column
        const T* D = tiles + (size_t)diag[i] * 4096;
        for (int e = tid; e < 4096; e += NT) Ts[(e >> 6) * LD + (e & 63)] = __ldcg(D + e);
        __syncthreads();
        for (int c = warp; c < nrhs; c += NT / 32) {
            for (int step = 0; step < 64; step++) {
                const int r = lower ? step : 63 - step;
                T v = T(0);
                if (lower) {
                    if (lane < r) v += Ts[r * LD + lane] * Acc[lane * nrhs + c];
                    if (lane + 32 < r) v += Ts[r * LD + lane + 32] * Acc[(lane + 32) * nrhs + c];
                } else {
                    if (lane > r) v += Ts[r * LD + lane] * Acc[lane * nrhs + c];
                    if (lane + 32 > r) v += Ts[r * LD + lane + 32] * Acc[(lane + 32) * nrhs + c];
                }
                v = warp_sum(v);
                if (lane == 0) Acc[r * nrhs + c] = (Acc[r * nrhs + c] - v) / Ts[r * LD + r];
                __syncwarp();
            }
        }
        __syncthreads();
        for (int e = tid; e < nv; e += NT) vec[(size_t)i * nv + e] = Acc[e];
        __threadfence();
        __syncthreads();
        if (tid == 0) st_release(s.flags + i, my_epoch);
    }
}

template <typename T>
size_t trisolve_smem(int nrhs) {
    return (64 * LD + 2 * 64 * (size_t)nrhs) * sizeof(T);
}

template <typename T>
int trisolve_impl(const DevSolve& s, const T* tiles, T* vec, int nrhs, int epoch, int grid, cudaStream_t st) {
    const size_t smem = trisolve_smem<T>(nrhs);
    cudaFuncSetAttribute(trisolve_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    trisolve_kernel<T><<<grid, NT, smem, st>>>(s, tiles, vec, nrhs, epoch, 1);
    trisolve_kernel<T><<<grid, NT, smem, st>>>(s, tiles, vec, nrhs, epoch, 0);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// r = b - A x over CSR rows; per-rhs reductions red[c*5 + {0..4}] =
// {sum r^2, sum b^2, max|r|, max|x|, max|b|}
__device__ __forceinline__ void atomic_max_nonneg(double* p, double v) {
    atomicMax(reinterpret_cast<unsigned long long*>(p), (unsigned long long)__double_as_longlong(v));
}
__global__ void residual_kernel(DevCSR A, const double* __restrict__ b, const double* __restrict__ x,
                                double* __restrict__ r, int nrhs, double* red, int n_stat) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    double rowabs = 0;
    if (row < n_stat)
        for (int k = A.ptr[row]; k < A.ptr[row + 1]; k++) rowabs += fabs(A.val[k]);
    for (int o = 16; o > 0; o >>= 1) rowabs = fmax(rowabs, __shfl_xor_sync(0xffffffffu, rowabs, o));
    for (int c = 0; c < nrhs; c++) {
        double rr = 0, bb = 0, ar = 0, ax = 0, ab = 0;
        if (row < A.n) {
            double acc = 0;
            for (int k = A.ptr[row]; k < A.ptr[row + 1]; k++) acc += A.val[k] * x[(size_t)A.col[k] * nrhs + c];
            const double bv = b[(size_t)row * nrhs + c];
            const double rv = bv - acc;
            r[(size_t)row * nrhs + c] = rv;
            if (row < n_stat) {
                rr = rv * rv; bb = bv * bv; ar = fabs(rv); ax = fabs(x[(size_t)row * nrhs + c]); ab = fabs(bv);
            }
        }
        rr = warp_sum(rr);
        bb = warp_sum(bb);
        for (int o = 16; o > 0; o >>= 1) {
            ar = fmax(ar, __shfl_xor_sync(0xffffffffu, ar, o));
            ax = fmax(ax, __shfl_xor_sync(0xffffffffu, ax, o));
            ab = fmax(ab, __shfl_xor_sync(0xffffffffu, ab, o));
        }
        if (lane == 0) {
            atomicAdd(red + c * RED + 0, rr);
            atomicAdd(red + c * RED + 1, bb);
            atomic_max_nonneg(red + c * RED + 2, ar);
            atomic_max_nonneg(red + c * RED + 3, ax);
            atomic_max_nonneg(red + c * RED + 4, ab);
            atomic_max_nonneg(red + c * RED + 5, rowabs);
        }
    }
}
__global__ void scatter_csr_kernel(const double* __restrict__ V, const int32_t* __restrict__ pos, int64_t nnz,
                                   double* __restrict__ val) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nnz && pos[k] >= 0) val[pos[k]] = V[k];
}

__global__ void cast_kernel(const double* __restrict__ s, float* __restrict__ d, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        d[i] = (float)s[i];
}
__global__ void axpy_kernel(const float* __restrict__ d, double* __restrict__ x, int64_t n, int assign) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = assign ? (double)d[i] : x[i] + (double)d[i];
}
__global__ void gather_kernel(const double* __restrict__ b, const int32_t* __restrict__ n2o, int n, int n_ext,
                              int nrhs, double* __restrict__ out) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)n_ext * nrhs) return;
    const int i = (int)(e / nrhs), c = (int)(e - (int64_t)i * nrhs);
    out[e] = i < n ? b[(size_t)c * n + n2o[i]] : 1.0;
}
__global__ void scatter_kernel(const double* __restrict__ xe, const int32_t* __restrict__ o2n, int n, int nrhs,
                               double* __restrict__ x) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)n * nrhs) return;
    const int c = (int)(e / n), i = (int)(e - (int64_t)c * n);
    x[e] = xe[(size_t)o2n[i] * nrhs + c];
}
__global__ void nonfinite_kernel(const double* __restrict__ x, int64_t n, unsigned long long* cnt) {
    unsigned long long local = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (!isfinite(x[i])) local++;
    if (local) atomicAdd(cnt, local);
}

}  // namespace

int trisolve_launch(const DevSolve& s, const double* tiles, double* vec, int nrhs, int epoch, int grid,
                    cudaStream_t st) {
    return trisolve_impl<double>(s, tiles, vec, nrhs, epoch, grid, st);
}
int trisolve_launch(const DevSolve& s, const float* tiles, float* vec, int nrhs, int epoch, int grid,
                    cudaStream_t st) {
    return trisolve_impl<float>(s, tiles, vec, nrhs, epoch, grid, st);
}
int trisolve_grid(bool fp64, int nrhs, int num_sms) {
    int per_sm = 0;
    if (fp64) {
        const size_t smem = trisolve_smem<double>(nrhs);
        cudaFuncSetAttribute(trisolve_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, trisolve_kernel<double>, NT, smem);
    } else {
        const size_t smem = trisolve_smem<float>(nrhs);
        cudaFuncSetAttribute(trisolve_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, trisolve_kernel<float>, NT, smem);
    }
    if (per_sm < 1) per_sm = 1;
    return per_sm * num_sms;
}

void residual_launch(const DevCSR& A, const double* b, const double* x, double* r, int nrhs, double* red,
                     int n_stat, cudaStream_t s) {
    cudaMemsetAsync(red, 0, sizeof(double) * RED * nrhs, s);
    residual_kernel<<<(A.n + 255) / 256, 256, 0, s>>>(A, b, x, r, nrhs, red, n_stat);
}
void scatter_csr_launch(const double* V, const int32_t* pos, int64_t nnz, double* csr_val, cudaStream_t s) {
    if (nnz > 0) scatter_csr_kernel<<<(unsigned)((nnz + 255) / 256), 256, 0, s>>>(V, pos, nnz, csr_val);
}
void cast_f64_to_f32_launch(const double* src, float* dst, int64_t n, cudaStream_t s) {
    if (n > 0) cast_kernel<<<608, 256, 0, s>>>(src, dst, n);
}
void axpy_f32_to_f64_launch(const float* d, double* x, int64_t n, int assign, cudaStream_t s) {
    if (n > 0) axpy_kernel<<<608, 256, 0, s>>>(d, x, n, assign);
}
void gather_rhs_launch(const double* b, const int32_t* new_to_old, int n, int n_ext, int nrhs, double* out,
                       cudaStream_t s) {
    const int64_t tot = (int64_t)n_ext * nrhs;
    gather_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(b, new_to_old, n, n_ext, nrhs, out);
}
void scatter_solution_launch(const double* xe, const int32_t* old_to_new, int n, int nrhs, double* x,
                             cudaStream_t s) {
    const int64_t tot = (int64_t)n * nrhs;
    scatter_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(xe, old_to_new, n, nrhs, x);
}
int count_nonfinite_launch(const double* x, int64_t n, unsigned long long* counter, cudaStream_t s) {
    cudaMemsetAsync(counter, 0, sizeof(unsigned long long), s);
    if (n > 0) nonfinite_kernel<<<304, 256, 0, s>>>(x, n, counter);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace sog
