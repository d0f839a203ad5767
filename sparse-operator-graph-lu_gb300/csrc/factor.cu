// Factor-phase kernels for sm_103a: the unit ops of the reference's DAG
// (MatrixStdDouble.cpp) as CTA-wide tile tasks, and two executors that run the
// task graph: a persistent kernel that pulls ready tasks from a device queue
// with atomic dependency counters, and a per-level launch (stage-synchronous,
// as BlockPlanner::calculate runs stages, BlockPlanner.cpp:376-651).
//
// Tiles are dense 64x64 row-major; block id k lives at tiles + k*4096.
// FP64 path: tile products on the FP64 tensor pipe (DMMA, mma.sync m8n8k4).
// Mixed path: FP32 tiles, tile products as split-precision TF32 (3 products:
// hi*hi + hi*lo + lo*hi, FP32 accumulation).
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.h"
#include "tasks.h"

namespace sog {

namespace {

constexpr int NT = 256;  // threads per CTA for every task kind
constexpr int LD = 65;   // padded leading dimension of square smem tiles

// smem footprints (elements of T)
constexpr int F64_GEMM_ELEMS = 32 * 68 + 64 * 40;
constexpr int F32_GEMM_ELEMS = 64 * 68 + 64 * 72;
constexpr int TWO_TILES = 2 * 64 * LD + 64;

template <typename T>
constexpr int smem_elems() {
    return sizeof(T) == 8 ? (F64_GEMM_ELEMS > TWO_TILES ? F64_GEMM_ELEMS : TWO_TILES)
                          : (F32_GEMM_ELEMS > TWO_TILES ? F32_GEMM_ELEMS : TWO_TILES);
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned long long dbits(double x) { return (unsigned long long)__double_as_longlong(x); }

// ---------------------------------------------------------------- tile loads
// Load a 64x64 tile from global (L2, bypassing L1: tiles are produced by other
// SMs during the same launch) into smem with leading dimension LD.
template <typename T>
__device__ __forceinline__ void load_tile(const T* __restrict__ g, T* s) {
    for (int e = threadIdx.x; e < 4096; e += NT) s[(e >> 6) * LD + (e & 63)] = __ldcg(g + e);
}

// ---------------------------------------------------------------- FP64 GEMM (DMMA)
__device__ __forceinline__ void dmma_8x8x4(double (&c)[2], double a, double b) {
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                 : "+d"(c[0]), "+d"(c[1])
                 : "d"(a), "d"(b));
}

// C[quadrant q] = sum_p s_p A_p[rows] * B_p[cols] for one 32x32 output quadrant.
// 8 warps: warp w owns rows (w&3)*8..+8 and columns (w>>2)*16..+16 (two 8x8 MMA tiles).
__device__ void gemm_f64_quadrant(const DevTasks& tk, double* __restrict__ tiles, int task, int q, double* sm) {
    double* sA = sm;            // [32][68]
    double* sB = sm + 32 * 68;  // [64][40]
    const int r0 = (q >> 1) * 32, c0 = (q & 1) * 32;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 2, t = lane & 3, rg = warp & 3, ch = warp >> 2;
    double acc[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
    const int p0 = tk.pair_ptr[task], p1 = tk.pair_ptr[task + 1];
    for (int p = p0; p < p1; p++) {
        const int pa = tk.pair_a[p];
        const int pbs = tk.pair_b[p];
        const double sgn = pbs < 0 ? -1.0 : 1.0;
        const int pb = pbs < 0 ? -pbs : pbs;
        const double* A = tiles + (size_t)pa * 4096 + r0 * 64;
        const double* Bm = tiles + (size_t)pb * 4096 + c0;
        __syncthreads();
        for (int i = tid; i < 1024; i += NT) {
            const int row = i >> 5, c2 = (i & 31) * 2;
            double2 v = __ldcg(reinterpret_cast<const double2*>(A + row * 64 + c2));
            sA[row * 68 + c2] = v.x * sgn;
            sA[row * 68 + c2 + 1] = v.y * sgn;
        }
        for (int i = tid; i < 1024; i += NT) {
            const int row = i >> 4, c2 = (i & 15) * 2;
            double2 v = __ldcg(reinterpret_cast<const double2*>(Bm + row * 64 + c2));
            sB[row * 40 + c2] = v.x;
            sB[row * 40 + c2 + 1] = v.y;
        }
        __syncthreads();
#pragma unroll
        for (int k0 = 0; k0 < 64; k0 += 4) {
            const double a = sA[(rg * 8 + g) * 68 + k0 + t];
#pragma unroll
            for (int nt = 0; nt < 2; nt++) {
                const double b = sB[(k0 + t) * 40 + ch * 16 + nt * 8 + g];
                dmma_8x8x4(acc[nt], a, b);
            }
        }
    }
    double* C = tiles + (size_t)tk.out[task] * 4096;
#pragma unroll
    for (int nt = 0; nt < 2; nt++) {
        const int row = r0 + rg * 8 + g, col = c0 + ch * 16 + nt * 8 + 2 * t;
        *reinterpret_cast<double2*>(C + row * 64 + col) = make_double2(acc[nt][0], acc[nt][1]);
    }
}

// ---------------------------------------------------------------- FP32 GEMM (3xTF32)
__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ void mma_tf32(float (&c)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Full 64x64 output per CTA. 8 warps: warp w owns rows (w&3)*16..+16 and
// columns (w>>2)*32..+32 (four m16n8 tiles).
__device__ void gemm_f32_full(const DevTasks& tk, float* __restrict__ tiles, int task, float* sm) {
    float* sA = sm;            // [64][68]
    float* sB = sm + 64 * 68;  // [64][72]
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 2, t = lane & 3, rt = warp & 3, cg = warp >> 2;
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.f;
    const int p0 = tk.pair_ptr[task], p1 = tk.pair_ptr[task + 1];
    for (int p = p0; p < p1; p++) {
        const int pa = tk.pair_a[p];
        const int pbs = tk.pair_b[p];
        const float sgn = pbs < 0 ? -1.f : 1.f;
        const int pb = pbs < 0 ? -pbs : pbs;
        const float* A = tiles + (size_t)pa * 4096;
        const float* Bm = tiles + (size_t)pb * 4096;
        __syncthreads();
        for (int i = tid; i < 1024; i += NT) {
            const int row = i >> 4, c4 = (i & 15) * 4;
            float4 v = __ldcg(reinterpret_cast<const float4*>(A + row * 64 + c4));
            v.x *= sgn; v.y *= sgn; v.z *= sgn; v.w *= sgn;
            *reinterpret_cast<float4*>(sA + row * 68 + c4) = v;
            float4 w = __ldcg(reinterpret_cast<const float4*>(Bm + row * 64 + c4));
            *reinterpret_cast<float4*>(sB + row * 72 + c4) = w;
        }
        __syncthreads();
#pragma unroll 2
        for (int k0 = 0; k0 < 64; k0 += 8) {
            float af[4] = {sA[(rt * 16 + g) * 68 + k0 + t], sA[(rt * 16 + g + 8) * 68 + k0 + t],
                           sA[(rt * 16 + g) * 68 + k0 + t + 4], sA[(rt * 16 + g + 8) * 68 + k0 + t + 4]};
            uint32_t ahi[4], alo[4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                ahi[i] = to_tf32(af[i]);
                alo[i] = to_tf32(af[i] - __uint_as_float(ahi[i]));
            }
#pragma unroll
            for (int nt = 0; nt < 4; nt++) {
                const int col = cg * 32 + nt * 8 + g;
                float bf[2] = {sB[(k0 + t) * 72 + col], sB[(k0 + t + 4) * 72 + col]};
                uint32_t bhi[2], blo[2];
                bhi[0] = to_tf32(bf[0]);
                bhi[1] = to_tf32(bf[1]);
                blo[0] = to_tf32(bf[0] - __uint_as_float(bhi[0]));
                blo[1] = to_tf32(bf[1] - __uint_as_float(bhi[1]));
                mma_tf32(acc[nt], alo, bhi);
                mma_tf32(acc[nt], ahi, blo);
                mma_tf32(acc[nt], ahi, bhi);
            }
        }
    }
    float* C = tiles + (size_t)tk.out[task] * 4096;
#pragma unroll
    for (int nt = 0; nt < 4; nt++) {
        const int col = cg * 32 + nt * 8 + 2 * t;
        const int row = rt * 16 + g;
        *reinterpret_cast<float2*>(C + row * 64 + col) = make_float2(acc[nt][0], acc[nt][1]);
        *reinterpret_cast<float2*>(C + (row + 8) * 64 + col) = make_float2(acc[nt][2], acc[nt][3]);
    }
}

// ---------------------------------------------------------------- LU of a diagonal block
// Right-looking unpivoted LU; pivots with |u_kk| < 1e-9 are clamped to
// +-1e-9 (sign kept, 0 -> +1e-9) exactly as ludcmpSimple does
// (MatrixStdDouble.cpp:2751-2761). L is unit lower, U upper. The pivot test,
// the clamp and the growth ratio are evaluated in FP64 in both precisions.
template <typename T>
__device__ void lu_task(const DevTasks& tk, T* __restrict__ tiles, int task, T* sm) {
    T* S = sm;                 // [64][LD]
    T* piv = sm + 64 * LD;     // [64]
    __shared__ float s_maxa, s_maxu;
    const int tid = threadIdx.x;
    if (tid == 0) { s_maxa = 0.f; s_maxu = 0.f; }
    const T* A = tiles + (size_t)tk.a[task] * 4096;
    __syncthreads();
    float ma = 0.f;
    for (int e = tid; e < 4096; e += NT) {
        T v = __ldcg(A + e);
        S[(e >> 6) * LD + (e & 63)] = v;
        ma = fmaxf(ma, fabsf((float)v));
    }
    for (int o = 16; o > 0; o >>= 1) ma = fmaxf(ma, __shfl_xor_sync(0xffffffffu, ma, o));
    if ((tid & 31) == 0) atomicMax(reinterpret_cast<int*>(&s_maxa), __float_as_int(ma));
    __syncthreads();
    for (int k = 0; k < 64; k++) {
        double pd = (double)S[k * LD + k];
        const bool clamp = (pd < 1e-9 && pd > -1e-9);
        if (clamp) pd = pd < 0 ? -1e-9 : 1e-9;
        const T p = (T)pd;
        const T rp = T(1) / p;
        for (int i = k + 1 + tid; i < 64; i += NT) S[i * LD + k] *= rp;
        if (tid == 0) {
            piv[k] = p;
            if (clamp) atomicAdd(&tk.status->clamped, 1);
            double ap = fabs((double)S[k * LD + k]);
            atomicMin(&tk.status->min_pivot_bits, dbits(ap));
        }
        __syncthreads();
        const int m = 63 - k;
        for (int idx = tid; idx < m * m; idx += NT) {
            const int i = k + 1 + idx / m, j = k + 1 + idx % m;
            S[i * LD + j] -= S[i * LD + k] * S[k * LD + j];
        }
        __syncthreads();
    }
    T* L = tiles + (size_t)tk.out[task] * 4096;
    T* U = tiles + (size_t)tk.out2[task] * 4096;
    float mu = 0.f;
    for (int e = tid; e < 4096; e += NT) {
        const int i = e >> 6, j = e & 63;
        const T s = S[i * LD + j];
        L[e] = i > j ? s : (i == j ? T(1) : T(0));
        const T u = i < j ? s : (i == j ? piv[i] : T(0));
        U[e] = u;
        mu = fmaxf(mu, fabsf((float)u));
    }
    for (int o = 16; o > 0; o >>= 1) mu = fmaxf(mu, __shfl_xor_sync(0xffffffffu, mu, o));
    if ((tid & 31) == 0) atomicMax(reinterpret_cast<int*>(&s_maxu), __float_as_int(mu));
    __syncthreads();
    if (tid == 0 && s_maxa > 0.f) atomicMax(&tk.status->max_growth_bits, dbits((double)s_maxu / (double)s_maxa));
}

// ---------------------------------------------------------------- triangular inverses
// Column-parallel: 4 threads per column j (tid = 4*j + s) split each inner
// product and combine with shuffles. Y = L^-1 uses only the lower triangle of
// the source including its diagonal (inv_lower, MatrixStdDouble.cpp:2787-2802);
// Y = U^-1 only the upper triangle (inv_upper, MatrixStdDouble.cpp:2829-2866).
template <typename T, bool LOWER>
__device__ void inv_task(const DevTasks& tk, T* __restrict__ tiles, int task, T* sm) {
    T* M = sm;            // source [64][LD]
    T* Y = sm + 64 * LD;  // result [64][LD]
    load_tile(tiles + (size_t)tk.a[task] * 4096, M);
    __syncthreads();
    const int j = threadIdx.x >> 2, s = threadIdx.x & 3;
    for (int step = 0; step < 64; step++) {
        const int i = LOWER ? step : 63 - step;
        T part = T(0);
        if (LOWER) {
            if (i > j)
                for (int k = j + s; k < i; k += 4) part += M[i * LD + k] * Y[k * LD + j];
        } else {
            if (i < j)
                for (int k = i + 1 + s; k <= j; k += 4) part += M[i * LD + k] * Y[k * LD + j];
        }
        part += __shfl_xor_sync(0xffffffffu, part, 1);
        part += __shfl_xor_sync(0xffffffffu, part, 2);
        if (s == 0) {
            const T q = T(1) / M[i * LD + i];
            T y;
            if (i == j) y = q;
            else if (LOWER ? (i > j) : (i < j)) y = -part * q;
            else y = T(0);
            Y[i * LD + j] = y;
        }
        __syncwarp();
    }
    __syncthreads();
    T* out = tiles + (size_t)tk.out[task] * 4096;
    for (int e = threadIdx.x; e < 4096; e += NT) out[e] = Y[(e >> 6) * LD + (e & 63)];
}

// R = A2 - A1; copy / negate when one side is absent (BlockPlanner.cpp:553-572)
template <typename T>
__device__ void sub_task(const DevTasks& tk, T* __restrict__ tiles, int task) {
    const int a2 = tk.a[task], a1 = tk.b[task];
    const T* X = tiles + (size_t)a2 * 4096;
    const T* Z = tiles + (size_t)a1 * 4096;
    T* R = tiles + (size_t)tk.out[task] * 4096;
    for (int e = threadIdx.x; e < 4096; e += NT) {
        T v = a2 > 0 ? __ldcg(X + e) : T(0);
        if (a1 > 0) v -= __ldcg(Z + e);
        R[e] = v;
    }
}

template <typename T>
__device__ __forceinline__ void run_item(const DevTasks& tk, T* tiles, int task, int part, T* sm) {
    switch (tk.kind[task]) {
        case K_GEMM:
            if constexpr (sizeof(T) == 8) {
                if (tk.parts[task] == 4) gemm_f64_quadrant(tk, tiles, task, part, sm);
                else
                    for (int q = 0; q < 4; q++) gemm_f64_quadrant(tk, tiles, task, q, sm);
            } else {
                gemm_f32_full(tk, tiles, task, sm);
            }
            break;
        case K_LU: lu_task<T>(tk, tiles, task, sm); break;
        case K_LINV: inv_task<T, true>(tk, tiles, task, sm); break;
        case K_UINV: inv_task<T, false>(tk, tiles, task, sm); break;
        case K_SUB: sub_task<T>(tk, tiles, task); break;
        default: break;
    }
}

// Mark an item done; the last part of a task releases its successors, and a
// successor whose last dependency this was is appended to the ready queue.
// Called by warp 0 after the CTA's writes are complete.
__device__ void complete_item(const DevTasks& tk, int task) {
    const int lane = threadIdx.x & 31;
    int last = 0;
    if (lane == 0) {
        __threadfence();
        last = (tk.parts[task] == 1) || (atomicSub(&tk.parts_left[task], 1) == 1);
    }
    last = __shfl_sync(0xffffffffu, last, 0);
    if (!last) return;
    __threadfence();
    const int s0 = tk.succ_ptr[task], s1 = tk.succ_ptr[task + 1];
    for (int k = s0 + lane; k < s1; k += 32) {
        const int s = tk.succ[k];
        if (atomicSub(&tk.dep[s], 1) == 1) {
            __threadfence();
            const int np = tk.parts[s];
            const int pos = atomicAdd(tk.tail, np);
            for (int p = 0; p < np; p++) atomicExch(&tk.queue[pos + p], (s << 2) | p);
        }
    }
}

__device__ __forceinline__ int ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Each CTA claims the next queue slot, waits (bounded) until a producer has
// filled it, runs the item and releases successors. Every slot is filled
// exactly once because every task becomes ready exactly once, so the loop
// ends when all slots are claimed; no CTA ever waits inside a task.
template <typename T>
__global__ void __launch_bounds__(NT) factor_persistent_kernel(DevTasks tk, T* tiles) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sm = reinterpret_cast<T*>(smem_raw);
    __shared__ int s_item, s_stop;
    for (;;) {
        if (threadIdx.x == 0) {
            int item = -1;
            const int slot = atomicAdd(tk.head, 1);
            if (slot < tk.total_items) {
                const unsigned long long t0 = globaltimer_ns();
                unsigned ns = 32;
                while ((item = ld_acquire(tk.queue + slot)) < 0) {
                    if (globaltimer_ns() - t0 > tk.wait_limit_ns) {
                        atomicOr(&tk.status->flags, ST_TIMEOUT);
                        tk.status->timeout_where = slot;
                        item = -2;
                        break;
                    }
                    __nanosleep(ns);
                    if (ns < 1024) ns *= 2;
                }
                if (item >= 0 && (item >> 2) >= tk.ntasks) {
                    atomicOr(&tk.status->flags, ST_BAD_ITEM);
                    item = -2;
                }
            }
            __threadfence();
            s_item = item;
        }
        __syncthreads();
        const int item = s_item;
        if (item < 0) break;
        run_item<T>(tk, tiles, item >> 2, item & 3, sm);
        __threadfence();
        __syncthreads();
        if (threadIdx.x < 32) complete_item(tk, item >> 2);
        // a timeout anywhere stops every CTA at its next claim
        if (threadIdx.x == 0) s_stop = (ld_acquire(&tk.status->flags) & ST_TIMEOUT) ? 1 : 0;
        __syncthreads();
        if (s_stop) break;
    }
}

template <typename T>
__global__ void __launch_bounds__(NT) factor_level_kernel(DevTasks tk, T* tiles, const int32_t* items) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sm = reinterpret_cast<T*>(smem_raw);
    const int item = items[blockIdx.x];
    run_item<T>(tk, tiles, item >> 2, item & 3, sm);
}

template <typename T>
int persistent_launch(const DevTasks& t, T* tiles, int grid, cudaStream_t s) {
    const size_t smem = smem_elems<T>() * sizeof(T);
    cudaFuncSetAttribute(factor_persistent_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    factor_persistent_kernel<T><<<grid, NT, smem, s>>>(t, tiles);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <typename T>
int level_launch(const DevTasks& t, T* tiles, const int32_t* items, int nitems, cudaStream_t s) {
    if (nitems <= 0) return 0;
    const size_t smem = smem_elems<T>() * sizeof(T);
    cudaFuncSetAttribute(factor_level_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    factor_level_kernel<T><<<nitems, NT, smem, s>>>(t, tiles, items);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

__global__ void scatter_kernel(const double* __restrict__ V, const int32_t* __restrict__ tile,
                               const int16_t* __restrict__ off, int64_t nnz, const int32_t* __restrict__ pad_tile,
                               const int16_t* __restrict__ pad_off, int64_t npad, double* t64, float* t32) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nnz) {
        const int32_t tl = tile[i];
        if (tl >= 0) {
            const int64_t e = (int64_t)tl * 4096 + off[i];
            if (t64) t64[e] = V[i];
            else t32[e] = (float)V[i];
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

int factor_persistent_launch(const DevTasks& t, double* tiles, int grid, cudaStream_t s) {
    return persistent_launch<double>(t, tiles, grid, s);
}
int factor_persistent_launch(const DevTasks& t, float* tiles, int grid, cudaStream_t s) {
    return persistent_launch<float>(t, tiles, grid, s);
}
int factor_level_launch(const DevTasks& t, double* tiles, const int32_t* items, int nitems, cudaStream_t s) {
    return level_launch<double>(t, tiles, items, nitems, s);
}
int factor_level_launch(const DevTasks& t, float* tiles, const int32_t* items, int nitems, cudaStream_t s) {
    return level_launch<float>(t, tiles, items, nitems, s);
}

size_t factor_smem_bytes(bool fp64) {
    return fp64 ? smem_elems<double>() * sizeof(double) : smem_elems<float>() * sizeof(float);
}

int factor_persistent_grid(bool fp64, int num_sms) {
    int per_sm = 0;
    const size_t smem = factor_smem_bytes(fp64);
    if (fp64) {
        cudaFuncSetAttribute(factor_persistent_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, factor_persistent_kernel<double>, NT, smem);
    } else {
        cudaFuncSetAttribute(factor_persistent_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, factor_persistent_kernel<float>, NT, smem);
    }
    if (per_sm < 1) per_sm = 1;
    return per_sm * num_sms;
}

void scatter_values_launch(const double* V, const int32_t* tile, const int16_t* off, int64_t nnz,
                           const int32_t* pad_tile, const int16_t* pad_off, int64_t npad, double* tiles64,
                           float* tiles32, cudaStream_t s) {
    const int64_t n = nnz + npad;
    if (n == 0) return;
    scatter_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(V, tile, off, nnz, pad_tile, pad_off, npad, tiles64,
                                                               tiles32);
}
void convert_tiles_launch(const double* src, float* dst, int64_t n, cudaStream_t s) {
    if (n > 0) convert_kernel<<<1216, 256, 0, s>>>(src, dst, n);
}
void widen_tiles_launch(const float* src, double* dst, int64_t n, cudaStream_t s) {
    if (n > 0) widen_kernel<<<1216, 256, 0, s>>>(src, dst, n);
}

}  // namespace sog
