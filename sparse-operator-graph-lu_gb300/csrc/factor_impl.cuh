// Factor-phase device code for sm_103a, shared by the per-precision
// translation units (factor_f64.cu, factor_f32_s1.cu, factor_f32_s2.cu, which
// the build compiles in parallel): the unit ops of the reference's DAG
// (MatrixStdDouble.cpp) as CTA-wide tile tasks, and three executors that run
// the task graph with atomic dependency counters: a persistent kernel whose
// CTAs claim tasks in a static order and wait for each to become ready (the
// default), a persistent kernel that pulls ready tasks from a device queue,
// and a per-level launch (stage-synchronous, as BlockPlanner::calculate runs
// stages, BlockPlanner.cpp:376-651).
//
// Hardware notes for sm_103a: the mixed path's tile products use tcgen05 MMAs
// with TMEM accumulators and TMA operand copies (tc_gemm.cuh); LU and
// triangular inverses run on the CUDA cores with rows in registers; FP64
// scalar and DMMA throughput on this part are about 1.2 TFLOP/s, so the FP64
// path is compute-bound and the mixed path latency-bound on the DAG's
// critical path.
//
// Tiles are dense 64x64 row-major; block id k lives at tiles + k*4096.
// FP64 path: tile products on the FP64 tensor pipe (DMMA, mma.sync m8n8k4),
// operand quadrants double-buffered through cp.async. Mixed path: FP32 tiles,
// tile products as split-precision TF32 (hi*hi + hi*lo + lo*hi, FP32
// accumulation in TMEM).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <stdint.h>

#include "kernels.h"
#include "tasks.h"
#include "tc_gemm.cuh"

namespace sog {

namespace {

constexpr int NT = 256;  // threads per CTA for every task kind
constexpr int LD = 65;   // padded leading dimension of square smem tiles
constexpr unsigned FULL = 0xffffffffu;

// smem footprints (elements of T)
constexpr int F64_STAGE = 32 * 68 + 64 * 40;  // A quadrant rows + B quadrant columns
constexpr int F32_STAGE = 64 * 68 + 64 * 72;  // full A and B tiles
constexpr int INV_ELEMS = 64 * LD + 16 * 64 + 64;  // source tile + 2 x 8 finished rows + reciprocals
constexpr int LU_ELEMS = 32 * 64 + 3 * 64;          // 2 x 8 pivot rows of A and of L^-1 + pivot data

template <typename T, int S>
constexpr int smem_elems() {
    // FP64: double-buffered DMMA stages; FP32: the tcgen05 operand area
    // (+128 B: the raw slots start on a 128-byte boundary, as TMA tile copies require)
    constexpr int g =
        sizeof(T) == 8 ? 2 * F64_STAGE : (S * tc::STAGE_BYTES + tc::raw_slots<S>() * tc::RAW_BYTES + 128) / 4;
    constexpr int t = INV_ELEMS > LU_ELEMS ? INV_ELEMS : LU_ELEMS;
    return g > t ? g : t;
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// release/acquire fence at GPU scope: with the CTA barrier before it, it
// orders every thread's earlier writes before the flag or count that follows
// (the fence.sc that __threadfence() issues is stronger than a release needs)
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
__device__ __forceinline__ unsigned long long dbits(double x) { return (unsigned long long)__double_as_longlong(x); }
__device__ __forceinline__ int ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

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

// C[quadrant q] = init[quadrant q] + sum_p s_p A_p[rows] * B_p[cols] for one 32x32
// output quadrant. 8 warps: warp w owns rows (w&3)*8..+8 and columns
// (w>>2)*16..+16 (two 8x8 MMA tiles). Pairs stream through two smem stages.
__device__ void gemm_f64_quadrant(const DevTasks& tk, double* __restrict__ tiles, int task, int q, double* sm) {
    const int r0 = (q >> 1) * 32, c0 = (q & 1) * 32;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 2, t = lane & 3, rg = warp & 3, ch = warp >> 2;
    const int p0 = tk.pair_ptr[task], p1 = tk.pair_ptr[task + 1];
    // stage: sA = A rows r0..r0+31; sB = B[0:64][c0:c0+32] as [k][40], or for
    // a transposed operand X (B = X^T) the rows X[c0:c0+32][0:64] as [n][68]
    auto issue = [&](int p, int s) {
        double* sA = sm + s * F64_STAGE;
        double* sB = sA + 32 * 68;
        const int pbs = tk.pair_b[p], pb = (pbs < 0 ? -pbs : pbs);
        const double* A = tiles + (size_t)tk.pair_a[p] * 4096 + r0 * 64;
        const bool tr = (pb & PAIR_TRANS) != 0;
        const double* X = tiles + (size_t)(pb & ~PAIR_TRANS) * 4096;
        for (int i = tid; i < 1024; i += NT) {
            const int ra = i >> 5, ca = (i & 31) * 2;
            cp_async16(sA + ra * 68 + ca, A + ra * 64 + ca);
            if (tr) cp_async16(sB + ra * 68 + ca, X + (c0 + ra) * 64 + ca);
            else {
                const int rb = i >> 4, cb = (i & 15) * 2;
                cp_async16(sB + rb * 40 + cb, X + rb * 64 + c0 + cb);
            }
        }
        cp_commit();
    };
    double acc[2][2];
    const int init = tk.a[task];
#pragma unroll
    for (int nt = 0; nt < 2; nt++) {
        if (init > 0) {
            const double2 v = __ldcg(reinterpret_cast<const double2*>(
                tiles + (size_t)init * 4096 + (r0 + rg * 8 + g) * 64 + c0 + ch * 16 + nt * 8 + 2 * t));
            acc[nt][0] = v.x;
            acc[nt][1] = v.y;
        } else {
            acc[nt][0] = acc[nt][1] = 0.0;
        }
    }
    if (p0 < p1) issue(p0, 0);
    for (int p = p0; p < p1; p++) {
        const int s = (p - p0) & 1;
        if (p + 1 < p1) {
            issue(p + 1, s ^ 1);
            cp_wait<1>();
        } else {
            cp_wait<0>();
        }
        __syncthreads();
        const double* sA = sm + s * F64_STAGE;
        const double* sB = sA + 32 * 68;
        const double sgn = tk.pair_b[p] < 0 ? -1.0 : 1.0;
        // in-tile sparsity (tk.skip_zero): an 8x4 fragment of A or a 4x8
        // fragment of B that is all zero contributes exact zeros, so its MMA
        // is skipped after one warp vote (a NaN is not zero). The reference
        // skips zero 8x8 sub-tiles by their masks (MatrixStdDouble.cpp:268-289).
        // The votes cost about 5 % on dense tiles, so the autotuner decides.
        const bool tr = ((tk.pair_b[p] < 0 ? -tk.pair_b[p] : tk.pair_b[p]) & PAIR_TRANS) != 0;
        if (tk.skip_zero) {
#pragma unroll
            for (int k0 = 0; k0 < 64; k0 += 4) {
                const double a = sgn * sA[(rg * 8 + g) * 68 + k0 + t];
                if (!__any_sync(FULL, a != 0.0)) continue;
#pragma unroll
                for (int nt = 0; nt < 2; nt++) {
                    const double b = tr ? sB[(ch * 16 + nt * 8 + g) * 68 + k0 + t] : sB[(k0 + t) * 40 + ch * 16 + nt * 8 + g];
                    if (__any_sync(FULL, b != 0.0)) dmma_8x8x4(acc[nt], a, b);
                }
            }
        } else if (tr) {  // B[k][n] = sB[n][k]
#pragma unroll
            for (int k0 = 0; k0 < 64; k0 += 4) {
                const double a = sgn * sA[(rg * 8 + g) * 68 + k0 + t];
#pragma unroll
                for (int nt = 0; nt < 2; nt++) dmma_8x8x4(acc[nt], a, sB[(ch * 16 + nt * 8 + g) * 68 + k0 + t]);
            }
        } else {
#pragma unroll
            for (int k0 = 0; k0 < 64; k0 += 4) {
                const double a = sgn * sA[(rg * 8 + g) * 68 + k0 + t];
#pragma unroll
                for (int nt = 0; nt < 2; nt++) dmma_8x8x4(acc[nt], a, sB[(k0 + t) * 40 + ch * 16 + nt * 8 + g]);
            }
        }
        __syncthreads();
    }
    double* C = tiles + (size_t)tk.out[task] * 4096;
#pragma unroll
    for (int nt = 0; nt < 2; nt++) {
        const int row = r0 + rg * 8 + g, col = c0 + ch * 16 + nt * 8 + 2 * t;
        *reinterpret_cast<double2*>(C + row * 64 + col) = make_double2(acc[nt][0], acc[nt][1]);
    }
}

// ---------------------------------------------------------------- LU of a diagonal block
// Right-looking unpivoted LU held in registers: thread t owns row t>>2,
// columns (t&3) + 4m (m = 0..15). Step k: the four owners of row k scale it by
// the pivot into a shared row buffer (double-buffered, so one barrier per step),
// every lower row applies the rank-1 update, and the owner of column k turns
// its entry into l_ik. Pivots with |u_kk| < 1e-9 are clamped to +-1e-9 (sign
// kept, 0 -> +1e-9) as ludcmpSimple does (MatrixStdDouble.cpp:2751-2761); the
// pivot test, clamp and growth ratio are evaluated in FP64 in both precisions.
//
// Both triangular inverses come out of the same 64 steps, in one register
// array y per row: for c <= r it holds L^-1[r][c] (the multipliers applied to
// the identity beside A, i.e. elimination on [A | I]: lowerInv of this LU's L,
// which the recursion always needs next); for c > r it holds X[r][c] of
// X = (D^-1 U)^-1, built by column operations: at step k every row r <= k
// subtracts X[r][k] times the published scaled pivot row, and U^-1 = X D^-1
// (upperInv of this LU's U). Rows below the pivot touch only columns <= k of
// y, rows at or above it only columns > k, so the halves never collide, and
// the column operations run on rows the elimination leaves idle.
__device__ __forceinline__ float fast_rcp(float x) { return __frcp_rn(x); }
// the hardware reciprocal (within 1 ulp): the FP32 LU's pivot reciprocal is on
// the per-step critical chain, and the factor's accuracy is refined in FP64
// anyway (|pivot| >= 1e-9 after the clamp, far from the flush-to-zero range)
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ double fast_rcp(double x) { return __drcp_rn(x); }

// Pivot statistics of one diagonal-block factorisation, in FP64 off the
// elimination's critical chain (warp 0, after the CTA barrier that also ORs
// `bad` over the block): min |pivot| before the clamp, the clamp count, the
// largest magnitude the task saw (its input block or its factor; LL^T: |L|^2,
// comparable with the input), and, when the task formed U^-1, the check the
// reference makes after every upperInv (inv_check_diag, MatrixStdDouble.cpp:
// 2871-2937, called at BlockPlanner.cpp:575-577): the diagonal of U U^-1
// within 1e-3 of 1 and no NaN. For triangular U and U^-1 that diagonal is
// u_ii (U^-1)_ii, and the entries the reference checks below it are exact
// zeros unless a factor entry is not finite, which `bad` reports. Written to
// the task's system entry of tk.piv.
template <typename T, bool CHOL>
__device__ __forceinline__ void pivot_stats(const DevTasks& tk, int task, const T* raw, const T* piv, const T* rpiv,
                                            bool check_inv, float maxa, float maxu, bool anybad) {
    const int lane = threadIdx.x & 31;
    double mn = 1e300;
    int cl = 0;
    bool off = false;
    for (int k = lane; k < 64; k += 32) {
        const double v = fabs((double)raw[k]);
        mn = fmin(mn, v);
        cl += CHOL ? (double)raw[k] < 1e-20 : v < 1e-9;
        if (check_inv) off = off || !(fabs((double)piv[k] * (double)rpiv[k] - 1.0) <= 1e-3);
    }
    for (int o = 16; o > 0; o >>= 1) {
        mn = fmin(mn, __shfl_xor_sync(FULL, mn, o));
        cl += __shfl_xor_sync(FULL, cl, o);
    }
    off = __any_sync(FULL, off) || (check_inv && anybad);
    if (lane == 0) {
        DevPivot& pv = tk.piv[tk.task_seg ? tk.task_seg[task] : 0];
        if (cl) atomicAdd(&pv.clamped, cl);
        if (off) atomicAdd(&pv.inv_fail, 1);
        atomicMin(&pv.min_pivot_bits, dbits(mn));
        const double mu = CHOL ? (double)maxu * (double)maxu : (double)maxu;
        atomicMax(&pv.max_mag_bits, dbits(fmax((double)maxa, mu)));
    }
}

// LU task (outputs L, U; L^-1 if tk.b, U^-1 if tk.c); with CHOL the LL^T task
// of a symmetric tile (lltdcmpSimple, MatrixStdDouble.cpp:2629-2668): the same
// elimination on the tile symmetrised from its lower triangle, pivots below
// 1e-20 raised to it, and L = L_lu diag(sqrt(pivots)),
// L^-1 = diag(1/sqrt(pivots)) L_lu^-1.
template <typename T, bool CHOL = false>
__device__ void lu_task(const DevTasks& tk, T* __restrict__ tiles, int task, T* sm) {
    T* rowbuf = sm;          // [2][8][64] scaled pivot rows of A for the current block
    T* wbuf = sm + 1024;     // [2][8][64] rows of the running L^-1 for the current block
    T* piv = sm + 2048;      // [64] clamped pivots
    T* rpiv = piv + 64;      // [64] their reciprocals
    T* raw = piv + 128;      // [64] pivots before the clamp
    __shared__ float s_maxa, s_maxu;
    const int tid = threadIdx.x, lane = tid & 31, r = tid >> 2, q = tid & 3;
    if (tid == 0) {
        s_maxa = 0.f;
        s_maxu = 0.f;
    }
    const T* A = tiles + (size_t)tk.a[task] * 4096 + r * 64 + q;
    const T* At = tiles + (size_t)tk.a[task] * 4096 + q * 64 + r;  // column r: A[q + 4m][r]
    T a[16], y[16];
    float ma = 0.f;
#pragma unroll
    for (int m = 0; m < 16; m++) {
        a[m] = (CHOL && q + 4 * m > r) ? __ldcg(At + 4 * m * 64) : __ldcg(A + 4 * m);
        ma = fmaxf(ma, fabsf((float)a[m]));
        y[m] = (q + 4 * m == r) ? T(1) : T(0);
    }
    __syncthreads();
    // One pivot per step: the four owners of row k publish it (scaled by the
    // pivot reciprocal) and their row of L^-1; after one CTA barrier every
    // lower row applies the rank-1 update and every upper row its column
    // operation. Buffers alternate by step so one barrier per step suffices.
    // (A variant factoring 8-row panels inside one warp with 8 CTA barriers
    // measured slower on GB300: the single-warp panel serialises more than the
    // barriers cost.)
#pragma unroll
    for (int k = 0; k < 64; k++) {
        const int km = k >> 2, kq = k & 3;
        T* ub = rowbuf + (k & 1) * 64;
        T* wb = wbuf + (k & 1) * 64;
        const int src = (lane & ~3) | kq;
        const T aik = __shfl_sync(FULL, a[km], src);  // a[r][k] for this thread's row
        const T xrk = CHOL ? T(0) : __shfl_sync(FULL, y[km], src);  // X[r][k] (rows r <= k)
        if (r == k) {
            // LU: clamp |u_kk| < 1e-9 to +-1e-9 (0 -> +1e-9); LL^T: p < 1e-20 -> 1e-20
            const T tiny = T(1e-9);
            const T p = CHOL ? (aik < T(1e-20) ? T(1e-20) : aik)
                             : ((aik < tiny && aik > -tiny) ? (aik < T(0) ? -tiny : tiny) : aik);
            const T rp = fast_rcp(p);
#pragma unroll
            for (int m = 0; m < 16; m++) {
                const int c = q + 4 * m;
                if (c > k) ub[c] = a[m] * rp;
                else wb[c] = y[m];
            }
            if (q == 0) {
                piv[k] = p;
                rpiv[k] = rp;
                raw[k] = aik;
            }
        }
        __syncthreads();
        if (r > k) {
            const T lik = aik * rpiv[k];
#pragma unroll
            for (int m = 0; m < 16; m++) {
                const int c = q + 4 * m;
                if (c > k) a[m] -= aik * ub[c];
                else y[m] -= lik * wb[c];
            }
            if (q == kq) a[km] = lik;
        } else if (!CHOL) {
#pragma unroll
            for (int m = 0; m < 16; m++) {
                const int c = q + 4 * m;
                if (c > k) y[m] -= xrk * ub[c];
            }
        }
    }
    T* L = tiles + (size_t)tk.out[task] * 4096 + r * 64 + q;
    const int32_t linv = tk.b[task], uinv = CHOL ? 0 : tk.c[task];
    float mu = 0.f;
    bool bad = false;
    if (CHOL) {
        T* sq = rowbuf;  // sqrt of the pivots (the pivot-row buffers are free now)
        if (tid < 64) sq[tid] = sqrt(piv[tid]);
        __syncthreads();
        const T sr = sq[r];
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int c = q + 4 * m;
            const T v = r > c ? a[m] * sq[c] : (r == c ? sr : T(0));
            L[4 * m] = v;
            mu = fmaxf(mu, fabsf((float)v));
        }
        if (linv > 0) {
            T* W = tiles + (size_t)linv * 4096 + r * 64 + q;
            const T isr = T(1) / sr;
#pragma unroll
            for (int m = 0; m < 16; m++) W[4 * m] = q + 4 * m <= r ? y[m] * isr : T(0);
        }
    } else {
        T* U = tiles + (size_t)tk.out2[task] * 4096 + r * 64 + q;
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int c = q + 4 * m;
            L[4 * m] = r > c ? a[m] : (r == c ? T(1) : T(0));
            const T u = r < c ? a[m] : (r == c ? piv[r] : T(0));
            U[4 * m] = u;
            mu = fmaxf(mu, fabsf((float)u));
            bad = bad || !isfinite(u);
        }
        if (linv > 0) {
            T* W = tiles + (size_t)linv * 4096 + r * 64 + q;
#pragma unroll
            for (int m = 0; m < 16; m++) W[4 * m] = q + 4 * m <= r ? y[m] : T(0);
        }
        if (uinv > 0) {
            T* V = tiles + (size_t)uinv * 4096 + r * 64 + q;
#pragma unroll
            for (int m = 0; m < 16; m++) {
                const int c = q + 4 * m;
                const T v = c >= r ? y[m] * rpiv[c] : T(0);
                V[4 * m] = v;
                bad = bad || !isfinite(v);
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        ma = fmaxf(ma, __shfl_xor_sync(FULL, ma, o));
        mu = fmaxf(mu, __shfl_xor_sync(FULL, mu, o));
    }
    if (lane == 0) {
        atomicMax(reinterpret_cast<int*>(&s_maxa), __float_as_int(ma));
        atomicMax(reinterpret_cast<int*>(&s_maxu), __float_as_int(mu));
    }
    const bool anybad = __syncthreads_or(bad) != 0;
    if (tid < 32) pivot_stats<T, CHOL>(tk, task, raw, piv, rpiv, !CHOL && uinv > 0, s_maxa, s_maxu, anybad);
}

// FP32 variant of the same elimination with column pairs: thread (r, q) owns
// columns 8m + 2q and 8m + 2q + 1 (m = 0..7) of row r, so the rank-1 update
// and the inverse updates run as paired FMAs (__ffma2_rn, two independent
// round-to-nearest FMAs: bit-identical to the scalar form) on 8-byte shared
// loads; only the pair holding column k needs per-element selection. Half the
// instructions per step of the stride-4 layout above, which the FP64 path keeps
// (there is no paired FP64 FMA).
// blocks: in (source), lo (L), up (U), linv (L^-1, 0 = none), uinv (U^-1, 0 = none)
template <bool CHOL>
__device__ void lu_task_f2(const DevTasks& tk, float* __restrict__ tiles, int task, int32_t in, int32_t lo, int32_t up,
                           int32_t linv, int32_t uinv, float* sm) {
    float* rowbuf = sm;     // [2][64] published rows
    float* piv = sm + 128;  // [64]
    float* rpiv = piv + 64;
    float* raw = piv + 128;
    __shared__ float s_maxa, s_maxu;
    const int tid = threadIdx.x, lane = tid & 31, r = tid >> 2, q = tid & 3;
    if (tid == 0) { s_maxa = 0.f; s_maxu = 0.f; }
    const float* A = tiles + (size_t)in * 4096;
    float2 a2[8], y2[8];
    float ma = 0.f;
#pragma unroll
    for (int m = 0; m < 8; m++) {
        const int c0 = 8 * m + 2 * q;
        if (CHOL) {
            a2[m].x = c0 > r ? __ldcg(A + c0 * 64 + r) : __ldcg(A + r * 64 + c0);
            a2[m].y = c0 + 1 > r ? __ldcg(A + (c0 + 1) * 64 + r) : __ldcg(A + r * 64 + c0 + 1);
        } else {
            a2[m] = __ldcg(reinterpret_cast<const float2*>(A + r * 64 + c0));
        }
        ma = fmaxf(ma, fmaxf(fabsf(a2[m].x), fabsf(a2[m].y)));
        y2[m] = make_float2(c0 == r ? 1.f : 0.f, c0 + 1 == r ? 1.f : 0.f);
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 64; k++) {
        const int km = k >> 3, kq = (k >> 1) & 3, kb = k & 1;
        float2* P2 = reinterpret_cast<float2*>(rowbuf + (k & 1) * 64);
        const int src = (lane & ~3) | kq;
        const float aik = __shfl_sync(FULL, kb ? a2[km].y : a2[km].x, src);
        const float xrk = CHOL ? 0.f : __shfl_sync(FULL, kb ? y2[km].y : y2[km].x, src);
        // columns of pair km right of the pivot: c0 > k, c1 > k
        const bool g0 = q > kq, g1 = q > kq || (q == kq && kb == 0);
        if (r == k) {
            const float tiny = 1e-9f;
            const float p = CHOL ? (aik < 1e-20f ? 1e-20f : aik)
                                 : ((aik < tiny && aik > -tiny) ? (aik < 0.f ? -tiny : tiny) : aik);
            const float rp = rcp_approx(p);
#pragma unroll
            for (int m = 0; m < 8; m++) {
                float2 o;
                if (m > km) o = make_float2(a2[m].x * rp, a2[m].y * rp);
                else if (m < km) o = y2[m];
                else o = make_float2(g0 ? a2[m].x * rp : y2[m].x, g1 ? a2[m].y * rp : y2[m].y);
                P2[4 * m + q] = o;
            }
            if (q == 0) { piv[k] = p; rpiv[k] = rp; raw[k] = aik; }
        }
        __syncthreads();
        if (r > k) {
            const float lik = aik * rpiv[k];
            const float2 na = make_float2(-aik, -aik), nl = make_float2(-lik, -lik);
#pragma unroll
            for (int m = 0; m < 8; m++) {
                const float2 v = P2[4 * m + q];
                if (m > km) a2[m] = __ffma2_rn(na, v, a2[m]);
                else if (m < km) y2[m] = __ffma2_rn(nl, v, y2[m]);
                else {
                    if (g0) a2[m].x = fmaf(-aik, v.x, a2[m].x); else y2[m].x = fmaf(-lik, v.x, y2[m].x);
                    if (g1) a2[m].y = fmaf(-aik, v.y, a2[m].y); else y2[m].y = fmaf(-lik, v.y, y2[m].y);
                }
            }
            if (q == kq) { if (kb) a2[km].y = lik; else a2[km].x = lik; }
        } else if (!CHOL) {
            const float2 nx = make_float2(-xrk, -xrk);
#pragma unroll
            for (int m = 0; m < 8; m++) {
                if (m > km) y2[m] = __ffma2_rn(nx, P2[4 * m + q], y2[m]);
                else if (m == km) {
                    const float2 v = P2[4 * m + q];
                    if (g0) y2[m].x = fmaf(-xrk, v.x, y2[m].x);
                    if (g1) y2[m].y = fmaf(-xrk, v.y, y2[m].y);
                }
            }
        }
    }
    __syncthreads();
    float* L = tiles + (size_t)lo * 4096 + r * 64 + 2 * q;
    float mu = 0.f;
    bool bad = false;
    if (CHOL) {
        float* sq = rowbuf;
        if (tid < 64) sq[tid] = sqrtf(piv[tid]);
        __syncthreads();
        const float sr = sq[r];
#pragma unroll
        for (int m = 0; m < 8; m++) {
            const int c0 = 8 * m + 2 * q, c1 = c0 + 1;
            const float2 v = make_float2(r > c0 ? a2[m].x * sq[c0] : (r == c0 ? sr : 0.f),
                                         r > c1 ? a2[m].y * sq[c1] : (r == c1 ? sr : 0.f));
            *reinterpret_cast<float2*>(L + 8 * m) = v;
            mu = fmaxf(mu, fmaxf(fabsf(v.x), fabsf(v.y)));
        }
        if (linv > 0) {
            float* W = tiles + (size_t)linv * 4096 + r * 64 + 2 * q;
            const float isr = 1.f / sr;
#pragma unroll
            for (int m = 0; m < 8; m++) {
                const int c0 = 8 * m + 2 * q;
                *reinterpret_cast<float2*>(W + 8 * m) =
                    make_float2(c0 <= r ? y2[m].x * isr : 0.f, c0 + 1 <= r ? y2[m].y * isr : 0.f);
            }
        }
    } else {
        float* U = tiles + (size_t)up * 4096 + r * 64 + 2 * q;
#pragma unroll
        for (int m = 0; m < 8; m++) {
            const int c0 = 8 * m + 2 * q, c1 = c0 + 1;
            *reinterpret_cast<float2*>(L + 8 * m) = make_float2(r > c0 ? a2[m].x : (r == c0 ? 1.f : 0.f),
                                                                r > c1 ? a2[m].y : (r == c1 ? 1.f : 0.f));
            const float2 u = make_float2(r < c0 ? a2[m].x : (r == c0 ? piv[r] : 0.f),
                                         r < c1 ? a2[m].y : (r == c1 ? piv[r] : 0.f));
            *reinterpret_cast<float2*>(U + 8 * m) = u;
            mu = fmaxf(mu, fmaxf(fabsf(u.x), fabsf(u.y)));
            bad = bad || !isfinite(u.x) || !isfinite(u.y);
        }
        if (linv > 0) {
            float* W = tiles + (size_t)linv * 4096 + r * 64 + 2 * q;
#pragma unroll
            for (int m = 0; m < 8; m++) {
                const int c0 = 8 * m + 2 * q;
                *reinterpret_cast<float2*>(W + 8 * m) = make_float2(c0 <= r ? y2[m].x : 0.f, c0 + 1 <= r ? y2[m].y : 0.f);
            }
        }
        if (uinv > 0) {
            float* V = tiles + (size_t)uinv * 4096 + r * 64 + 2 * q;
#pragma unroll
            for (int m = 0; m < 8; m++) {
                const int c0 = 8 * m + 2 * q, c1 = c0 + 1;
                const float2 v = make_float2(c0 >= r ? y2[m].x * rpiv[c0] : 0.f, c1 >= r ? y2[m].y * rpiv[c1] : 0.f);
                *reinterpret_cast<float2*>(V + 8 * m) = v;
                bad = bad || !isfinite(v.x) || !isfinite(v.y);
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        ma = fmaxf(ma, __shfl_xor_sync(FULL, ma, o));
        mu = fmaxf(mu, __shfl_xor_sync(FULL, mu, o));
    }
    if (lane == 0) {
        atomicMax(reinterpret_cast<int*>(&s_maxa), __float_as_int(ma));
        atomicMax(reinterpret_cast<int*>(&s_maxu), __float_as_int(mu));
    }
    const bool anybad = __syncthreads_or(bad) != 0;
    if (tid < 32) pivot_stats<float, CHOL>(tk, task, raw, piv, rpiv, !CHOL && uinv > 0, s_maxa, s_maxu, anybad);
}

// ---------------------------------------------------------------- triangular inverses
// Y = L^-1 by forward elimination on the identity, Y = U^-1 by backward
// elimination, the working rows held in registers (thread t owns row t>>2,
// columns (t&3) + 4m) and one barrier per step. Y = L^-1 reads only the lower
// triangle of the source including its diagonal (inv_lower,
// MatrixStdDouble.cpp:2787-2802); Y = U^-1 only the upper triangle (inv_upper,
// MatrixStdDouble.cpp:2829-2866).
template <typename T, bool LOWER>
__device__ void inv_task(const DevTasks& tk, T* __restrict__ tiles, int task, T* sm) {
    T* M = sm;                  // source [64][LD]
    T* rowbuf = sm + 64 * LD;   // [2][8][64] finished rows of Y for the current block
    T* rdiag = rowbuf + 1024;   // [64] reciprocals of the diagonal
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, r = tid >> 2, q = tid & 3;
    load_tile(tiles + (size_t)tk.a[task] * 4096, M);
    T w[16];
#pragma unroll
    for (int m = 0; m < 16; m++) w[m] = (q + 4 * m == r) ? T(1) : T(0);
    __syncthreads();
    if (tid < 64) rdiag[tid] = T(1) / M[tid * LD + tid];
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 64; kk++) {
        const int k = LOWER ? kk : 63 - kk;
        T* rb = rowbuf + (kk & 1) * 64;
        if (r == k) {
            const T d = rdiag[k];
#pragma unroll
            for (int m = 0; m < 16; m++) {
                w[m] *= d;
                rb[q + 4 * m] = w[m];
            }
        }
        __syncthreads();
        if (LOWER ? (r > k) : (r < k)) {
            const T mk = M[r * LD + k];
#pragma unroll
            for (int m = 0; m < 16; m++) {
                const int c = q + 4 * m;
                if (LOWER ? (c <= k) : (c >= k)) w[m] -= mk * rb[c];
            }
        }
    }
    T* out = tiles + (size_t)tk.out[task] * 4096 + r * 64 + q;
    bool bad = false;
#pragma unroll
    for (int m = 0; m < 16; m++) {
        out[4 * m] = w[m];
        bad = bad || !isfinite(w[m]);
    }
    if (!LOWER) {
        // inv_check_diag after upperInv (BlockPlanner.cpp:575-577): the
        // diagonal of U U^-1 is u_kk (U^-1)_kk for triangular factors
        const bool anybad = __syncthreads_or(bad) != 0;
        if (warp == 0) {
            bool off = anybad;
            for (int k = lane; k < 64; k += 32)
                off = off || !(fabs((double)M[k * LD + k] * (double)rdiag[k] - 1.0) <= 1e-3);
            off = __any_sync(FULL, off);
            if (lane == 0 && off) atomicAdd(&tk.piv[tk.task_seg ? tk.task_seg[task] : 0].inv_fail, 1);
        }
    }
}

// R = A2 - A1; copy / negate when one side is absent (BlockPlanner.cpp:553-572)
template <typename T>
__device__ void sub_task(const DevTasks& tk, T* __restrict__ tiles, int task) {
    const int a2 = tk.a[task], a1 = tk.b[task];
    const T* X = tiles + (size_t)a2 * 4096;
    const T* Z = tiles + (size_t)a1 * 4096;
    T* R = tiles + (size_t)tk.out[task] * 4096;
#pragma unroll 4
    for (int e = threadIdx.x; e < 4096; e += NT) {
        T v = a2 > 0 ? __ldcg(X + e) : T(0);
        if (a1 > 0) v -= __ldcg(Z + e);
        R[e] = v;
    }
}

// R = A^T through shared memory (coalesced reads and writes): the upper
// factor L^T of an LL^T plan for the back substitution
template <typename T>
__device__ void trans_task(const DevTasks& tk, T* __restrict__ tiles, int task, T* sm) {
    const T* A = tiles + (size_t)tk.a[task] * 4096;
    T* R = tiles + (size_t)tk.out[task] * 4096;
    for (int e = threadIdx.x; e < 4096; e += NT) sm[(e & 63) * LD + (e >> 6)] = __ldcg(A + e);
    __syncthreads();
    for (int e = threadIdx.x; e < 4096; e += NT) R[e] = sm[(e >> 6) * LD + (e & 63)];
}

// C = init + sum_p s_p A_p B_p on the tcgen05 tensor cores (tc_gemm.cuh).
// Thread 0 keeps up to R operand pairs in flight: the TMA copies the raw FP32
// tiles (contiguous 16 KB each) into a ring of R slots (mbarrier completion).
// Every warp splits its share of the oldest slot into a stage (A heads and
// remainders in interleaved rows, B_hi^T, B_lo^T) and signals the stage's
// `full` barrier; thread
// 0 then issues that stage's MMAs and refills the slot, while the other warps
// already stage the next pair (no CTA barrier per pair). Only the first pair's
// copy latency is exposed. `phase` holds this CTA's mbarrier parities (stages
// free: bits 0-1, stages full: bits 16-17, thread 0 only; raw slots: bits
// 8-10), carried across tasks.
//
// early: the task was claimed before its last producer finished (the ordered
// executor, mixed path). Pairs are ordered by the estimated finish of their
// producers; thread 0 waits, bounded, for a pair's two producers just before
// copying it, so the ready pairs accumulate while the late one is computed
// elsewhere. Warp 0 checks the first 32 pairs' producers at once up front.
constexpr int PAIRS_SMEM = 64;  // operand pairs listed in shared memory per task
template <int S>
__device__ void gemm_f32_tc(const DevTasks& tk, float* __restrict__ tiles, int task, float* sm, tc::State& st,
                            uint32_t& phase, bool early) {
    constexpr int R = tc::raw_slots<S>();
    __shared__ int32_t s_pa[PAIRS_SMEM], s_pb[PAIRS_SMEM], s_wa[PAIRS_SMEM], s_wb[PAIRS_SMEM];
    __shared__ unsigned s_ready;  // pairs 0..31 whose producers had finished at the start
    __shared__ int s_init_ready;
    unsigned char* smb = reinterpret_cast<unsigned char*>(sm);
    unsigned char* raw = smb + S * tc::STAGE_BYTES;
    raw += (128u - (tc::smem_u32(raw) & 127u)) & 127u;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int p0 = tk.pair_ptr[task], p1 = tk.pair_ptr[task + 1];
    const unsigned long long lim = tk.wait_limit_ns;
    const int n = p1 - p0;
    for (int j = tid; j < n && j < PAIRS_SMEM; j += NT) {
        s_pa[j] = tk.pair_a[p0 + j];
        s_pb[j] = tk.pair_b[p0 + j];
        if (early) {
            s_wa[j] = tk.pair_wa[p0 + j];
            s_wb[j] = tk.pair_wb[p0 + j];
        }
    }
    auto pair_a = [&](int i) { return i < PAIRS_SMEM ? s_pa[i] : tk.pair_a[p0 + i]; };
    auto pair_b = [&](int i) { return i < PAIRS_SMEM ? s_pb[i] : tk.pair_b[p0 + i]; };
    const int init = tk.a[task];
    if (early && warp == 0) {
        bool ok = true;
        if (lane < n) {
            const int wa = tk.pair_wa[p0 + lane], wb = tk.pair_wb[p0 + lane];
            ok = (wa < 0 || ld_acquire(tk.task_done + wa) != 0) && (wb < 0 || ld_acquire(tk.task_done + wb) != 0);
        }
        const unsigned m = __ballot_sync(FULL, ok);
        if (lane == 0) {
            s_ready = m;
            const int wi = init > 0 ? tk.init_w[task] : -1;
            s_init_ready = wi < 0 || ld_acquire(tk.task_done + wi) != 0;
        }
    }
    __syncthreads();
    // wait (thread 0, bounded) until tasks ta and tb (-1: none) finished;
    // false on timeout. Both flags are read at once on every probe.
    auto wait_done = [&](int ta, int tb) -> bool {
        bool da = ta < 0, db = tb < 0;
        unsigned long long t0 = 0;
        for (unsigned spins = 0;; spins++) {
            const int va = da ? 1 : ld_acquire(tk.task_done + ta), vb = db ? 1 : ld_acquire(tk.task_done + tb);
            da = da || va != 0;
            db = db || vb != 0;
            if (da && db) return true;
            if (spins == 0) t0 = globaltimer_ns();
            else if (globaltimer_ns() - t0 > lim) return false;
        }
    };
    // the initial tile is read in the epilogue, 16 columns of one row per
    // lane: load it now, under the operand copies and the MMAs (or after its
    // producer, if late)
    const int quad = warp & 3, colh = (warp >> 2) * 32;
    const int erow = 16 * quad + (lane >> 1), ecol = colh + 16 * (lane & 1);  // this lane's output slice
    const bool init_now = !early || s_init_ready;
    float4 u[4];
    auto load_init = [&]() {
        if (init > 0) {
            const float4* I = reinterpret_cast<const float4*>(tiles + (size_t)init * 4096 + erow * 64 + ecol);
#pragma unroll
            for (int i = 0; i < 4; i++) u[i] = __ldcg(I + i);
        }
    };
    if (init_now) load_init();
    auto fetch = [&](int i) {  // thread 0: copies of pair p0 + i into raw slot i % R
        if (early && !(i < 32 && ((s_ready >> i) & 1u))) {
            const int wa = i < PAIRS_SMEM ? s_wa[i] : tk.pair_wa[p0 + i];
            const int wb = i < PAIRS_SMEM ? s_wb[i] : tk.pair_wb[p0 + i];
            if (!wait_done(wa, wb)) st.fail = 1;
            tc::fence_proxy_async_global();
        }
        const int slot = i % R, pbs = pair_b(i), pb = pbs < 0 ? -pbs : pbs, b = pb & ~PAIR_TRANS;
        unsigned char* dst = raw + slot * tc::RAW_BYTES;
        tc::expect_tx(&st.raw[slot], tc::RAW_BYTES);
        tc::bulk_copy(dst, tiles + (size_t)pair_a(i) * 4096, tc::RAW_BYTES / 2, &st.raw[slot]);
        tc::bulk_copy(dst + tc::RAW_BYTES / 2, tiles + (size_t)b * 4096, tc::RAW_BYTES / 2, &st.raw[slot]);
    };
    if (tid == 0 && n > 0) {
        tc::fence_proxy_async_global();  // the acquired producers' writes, then the copies
        for (int i = 0; i < n && i < R; i++) fetch(i);
    }
    for (int i = 0; i < n; i++) {
        const int s = i % S, slot = i % R;
        unsigned char* stg = smb + s * tc::STAGE_BYTES;
        if (i >= S) {  // the MMAs of pair i-S read this stage
            if (!tc::mbar_wait(&st.bar[s], (phase >> s) & 1u, lim)) st.fail = 1;
            phase ^= 1u << s;
        }
        if (!tc::mbar_wait(&st.raw[slot], (phase >> (8 + slot)) & 1u, lim)) st.fail = 1;
        phase ^= 1u << (8 + slot);
        const int pbs = pair_b(i);
        tc::stage_from_raw(stg, raw + slot * tc::RAW_BYTES, ((pbs < 0 ? -pbs : pbs) & PAIR_TRANS) != 0,
                           pbs < 0 ? -1.f : 1.f);
        tc::fence_proxy_async();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&st.full[s]);
        if (tid == 0) {
            if (!tc::mbar_wait(&st.full[s], (phase >> (16 + s)) & 1u, lim)) st.fail = 1;
            phase ^= 1u << (16 + s);
            tc::fence_after_sync();
            tc::issue_pair(stg, st.tmem, i == 0);
            tc::mma_commit(&st.bar[s]);
            if (i + R < n) fetch(i + R);  // every warp has staged from this slot (full barrier)
        }
    }
    if (early && tid == 0 && !init_now && !wait_done(tk.init_w[task], -1)) st.fail = 1;  // a late initial tile
    for (int i = n > S ? n - S : 0; i < n; i++) {  // the commits not yet waited for
        const int s = i % S;
        if (!tc::mbar_wait(&st.bar[s], (phase >> s) & 1u, lim)) st.fail = 1;
        phase ^= 1u << s;
    }
    tc::fence_after_sync();
    // epilogue: C = init + D summed over the split products. Output row r has
    // its head in TMEM lane 2r and its remainder in lane 2r + 1 (one warp);
    // columns 0-63 are x B_hi, 64-127 x B_lo. Each lane adds its two column
    // halves, takes its partner lane's sum by a shuffle, and the pair stores
    // the row's 32 columns of this warp (16 each). No shared memory, no barrier.
    float v[32];
    if (p0 < p1) {
        float w[32];
        const uint32_t tq = st.tmem + ((uint32_t)(32 * quad) << 16) + colh;
        tc::tmem_ld32(tq, v);
        tc::tmem_ld32(tq + 64, w);
#pragma unroll
        for (int i = 0; i < 32; i++) {
            v[i] += w[i];
            v[i] += __shfl_xor_sync(FULL, v[i], 1);
        }
    } else {
#pragma unroll
        for (int i = 0; i < 32; i++) v[i] = 0.f;
    }
    if (!init_now) {
        __syncthreads();  // orders thread 0's acquire of the late initial tile before the loads
        load_init();
    }
    const bool upper = (lane & 1) != 0;
    float o[16];
#pragma unroll
    for (int i = 0; i < 16; i++) o[i] = upper ? v[16 + i] : v[i];
    if (init > 0) {
#pragma unroll
        for (int i = 0; i < 4; i++) {
            o[4 * i] += u[i].x; o[4 * i + 1] += u[i].y; o[4 * i + 2] += u[i].z; o[4 * i + 3] += u[i].w;
        }
    }
    float4* C = reinterpret_cast<float4*>(tiles + (size_t)tk.out[task] * 4096 + erow * 64 + ecol);
#pragma unroll
    for (int i = 0; i < 4; i++) C[i] = make_float4(o[4 * i], o[4 * i + 1], o[4 * i + 2], o[4 * i + 3]);
    tc::fence_before_sync();
    __syncthreads();
}

// Per-CTA tensor-memory set-up / tear-down for the mixed path.
__device__ __forceinline__ void tc_setup(tc::State& st) {
    if ((threadIdx.x >> 5) == 0) tc::tmem_alloc(&st.tmem);
    if (threadIdx.x == 0) {
        for (int s = 0; s < tc::MAX_STAGES; s++) tc::mbar_init(&st.bar[s], 1);
        for (int s = 0; s < tc::MAX_STAGES; s++) tc::mbar_init(&st.full[s], NT / 32);
        for (int s = 0; s < tc::MAX_RAW; s++) tc::mbar_init(&st.raw[s], 1);
        st.fail = 0;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
}
__device__ __forceinline__ void tc_teardown(tc::State& st, const DevTasks& tk) {
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x == 0 && st.fail) atomicOr(&tk.status->flags, ST_TIMEOUT);
    if ((threadIdx.x >> 5) == 0) tc::tmem_dealloc(st.tmem);
}

template <typename T, int S>
__device__ __forceinline__ void run_item(const DevTasks& tk, T* tiles, int task, int part, bool early, T* sm, tc::State& st,
                                         uint32_t& phase) {
    switch (tk.kind[task]) {
        case K_GEMM:
            if constexpr (sizeof(T) == 8) {
                if (tk.parts[task] == 4) {
                    gemm_f64_quadrant(tk, tiles, task, part, sm);
                } else {
                    for (int q = 0; q < 4; q++) {
                        gemm_f64_quadrant(tk, tiles, task, q, sm);
                        __syncthreads();
                    }
                }
            } else {
                gemm_f32_tc<S>(tk, tiles, task, sm, st, phase, early);
            }
            break;
        case K_LU:
            if constexpr (sizeof(T) == 4)
                lu_task_f2<false>(tk, tiles, task, tk.a[task], tk.out[task], tk.out2[task], tk.b[task], tk.c[task], sm);
            else lu_task<T, false>(tk, tiles, task, sm);
            break;
        case K_LLT:
            if constexpr (sizeof(T) == 4)
                lu_task_f2<true>(tk, tiles, task, tk.a[task], tk.out[task], 0, tk.b[task], 0, sm);
            else lu_task<T, true>(tk, tiles, task, sm);
            break;
        case K_GEMM_LU:
        case K_GEMM_LLT:  // the product, then in the same CTA the factorisation of its result
            if constexpr (sizeof(T) == 4) {
                gemm_f32_tc<S>(tk, tiles, task, sm, st, phase, early);  // ends with a CTA barrier
                if (tk.kind[task] == K_GEMM_LU)
                    lu_task_f2<false>(tk, tiles, task, tk.out[task], tk.out3[task], tk.out2[task], tk.b[task],
                                      tk.c[task], sm);
                else
                    lu_task_f2<true>(tk, tiles, task, tk.out[task], tk.out3[task], 0, tk.b[task], 0, sm);
            }
            break;
        case K_LINV: inv_task<T, true>(tk, tiles, task, sm); break;
        case K_UINV: inv_task<T, false>(tk, tiles, task, sm); break;
        case K_SUB: sub_task<T>(tk, tiles, task); break;
        case K_TRANS: trans_task<T>(tk, tiles, task, sm); break;
        default: break;
    }
}

__device__ __forceinline__ void st_relaxed(int* p, int v) {
    asm volatile("st.relaxed.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_release(int* p, int v) {
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void red_release_add(int* p, int v) {
    asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int atom_add_acquire(int* p, int v) {
    int old;
    asm volatile("atom.acquire.gpu.global.add.s32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

// Called by warp 0 once the CTA's writes for an item are complete. The last
// part of a task releases its successors; of those that become ready, the one
// with the longest remaining path is kept to run next on this CTA (no queue
// round trip on the critical chain) and the others are queued. Returns the
// kept item or -1.
__device__ int complete_item(const DevTasks& tk, int task) {
    const int lane = threadIdx.x & 31;
    int last = 0;
    // release: the CTA's writes for this item (ordered before this warp by the
    // CTA barrier) become visible before any counter below moves
    fence_acq_rel_gpu();
    if (lane == 0) last = (tk.parts[task] == 1) || (atom_add_acquire(&tk.parts_left[task], -1) == 1);
    last = __shfl_sync(FULL, last, 0);
    int keep = -1, keep_prio = -1;  // warp-uniform
    if (last) {
        const int s0 = tk.succ_ptr[task], s1 = tk.succ_ptr[task + 1];
        for (int base = s0; base < s1; base += 32) {
            const int k = base + lane;
            int s = -1;
            if (k < s1) {
                s = tk.succ[k];
                // acquire: the lane that sees the count reach zero synchronises
                // with every producer's release of this successor's inputs
                if (atom_add_acquire(&tk.dep[s], -1) != 1) s = -1;
                else if (tk.trace) tk.trace[4 * (size_t)s] = globaltimer_ns();
            }
            if (!__any_sync(FULL, s >= 0)) continue;
            // the highest-priority newly ready task of this batch (ties: lowest lane)
            int best = s >= 0 ? tk.prio[s] : -1, bl = lane;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const int ob = __shfl_xor_sync(FULL, best, o), ol = __shfl_xor_sync(FULL, bl, o);
                if (ob > best || (ob == best && ol < bl)) { best = ob; bl = ol; }
            }
            if (best > keep_prio) {  // keep it; the lane that found it queues the previous keep instead
                const int t = __shfl_sync(FULL, s, bl);
                if (lane == bl) s = keep;
                keep = t;
                keep_prio = best;
            }
            // queue the rest: one tail reservation for the whole batch, then release stores
            const int np = s >= 0 ? tk.parts[s] : 0;
            int incl = np;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(FULL, incl, o);
                if (lane >= o) incl += v;
            }
            const int total = __shfl_sync(FULL, incl, 31);
            if (total) {
                int base_pos = 0;
                if (lane == 0) {
                    fence_acq_rel_gpu();
                    base_pos = atomicAdd(tk.tail, total);
                }
                base_pos = __shfl_sync(FULL, base_pos, 0) + incl - np;
                for (int p = 0; p < np; p++) st_release(&tk.queue[base_pos + p], (s << 4) | p);
            }
        }
        if (keep >= 0) {
            // the kept task's inputs were acquired by the lane that released it;
            // the CTA barrier before the task passes that on to every thread
            const int np = tk.parts[keep];
            if (np > 1) {
                int base_pos = 0;
                if (lane == 0) base_pos = atomicAdd(tk.tail, np - 1);
                base_pos = __shfl_sync(FULL, base_pos, 0);
                if (lane > 0 && lane < np) st_release(&tk.queue[base_pos + lane - 1], (keep << 4) | lane);
            }
        }
    }
    if (lane == 0) red_release_add(tk.done, 1);
    return keep >= 0 ? (keep << 4) : -1;
}

// Ready-queue executor: each CTA runs the item it kept from its last
// completion, else claims the next queue slot and waits (bounded) until a
// producer fills it. The launch ends when every item has completed; no CTA
// ever waits inside a task.
template <typename T, int S>
__global__ void __launch_bounds__(NT, (S == 1 || sizeof(T) == 8) ? 2 : 1) factor_queue_kernel(const __grid_constant__ DevTasks tk, T* tiles) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sm = reinterpret_cast<T*>(smem_raw);
    __shared__ int s_item, s_next, s_stop;
    __shared__ tc::State st;
    uint32_t phase = 0;
    if constexpr (sizeof(T) == 4) tc_setup(st);
    if (threadIdx.x == 0) {
        s_next = -1;
        s_stop = 0;
    }
    unsigned done_here = 0;  // items this CTA completed (thread 0)
    for (;;) {
        if (threadIdx.x == 0) {
            int item = s_next;
            s_next = -1;
            if (item < 0) {
                const int slot = atomicAdd(tk.head, 1);
                if (slot < tk.total_items) {
                    unsigned long long t0 = 0;
                    unsigned spins = 0;
                    while ((item = ld_acquire(tk.queue + slot)) < 0) {
                        if (spins == 0) t0 = globaltimer_ns();  // the clock only once waiting
                        if ((++spins & 15) == 0) {
                            if (ld_acquire(tk.done) >= tk.total_items) { item = -1; break; }
                            if (ld_acquire(&tk.status->flags) & ST_TIMEOUT) { item = -1; break; }
                            if (globaltimer_ns() - t0 > tk.wait_limit_ns) {
                                atomicOr(&tk.status->flags, ST_TIMEOUT);
                                tk.status->timeout_where = slot;
                                item = -1;
                                break;
                            }
                        }
                        __nanosleep(64);
                    }
                    if (item >= 0 && (item >> 4) >= tk.ntasks) {
                        atomicOr(&tk.status->flags, ST_BAD_ITEM);
                        item = -1;
                    }
                }
            }
            if (item >= 0 && tk.trace) {
                unsigned smid;
                asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
                unsigned long long* tr = tk.trace + 4 * (size_t)(item >> 4);
                atomicMax(tr + 1, ~globaltimer_ns());  // start = min over parts, stored inverted
                tr[3] = smid;
            }
            // a claimed item was acquired from its queue slot, a kept one by
            // complete_item; the barrier below extends either to the CTA
            s_item = item;
        }
        __syncthreads();
        const int item = s_item;
        if (item < 0) break;
        run_item<T, S>(tk, tiles, item >> 4, item & 7, false, sm, st, phase);
        __syncthreads();
        if (threadIdx.x < 32) {
            if (tk.trace && threadIdx.x == 0) atomicMax(tk.trace + 4 * (size_t)(item >> 4) + 2, globaltimer_ns());
            const int keep = complete_item(tk, item >> 4);
            if (threadIdx.x == 0) {
                s_next = keep;
                // a timeout anywhere stops every CTA: spinning ones in the claim
                // loop, busy ones here every 8th item (an L2 round trip each)
                if ((++done_here & 7) == 0) s_stop = (ld_acquire(&tk.status->flags) & ST_TIMEOUT) ? 1 : 0;
            }
        }
        __syncthreads();
        if (s_stop) break;
    }
    if constexpr (sizeof(T) == 4) tc_teardown(st, tk);
}

// Warp 0 after the CTA's writes for an item are complete: the last part of a
// task releases its successors with fire-and-forget reductions (no round
// trip): a claimant spinning on a successor's count sees it reach zero.
__device__ void release_item(const DevTasks& tk, int task) {
    const int lane = threadIdx.x & 31;
    fence_acq_rel_gpu();  // release: the CTA's writes (ordered before this warp by the barrier)
    int last = 1;
    if (tk.parts[task] > 1) {
        if (lane == 0) last = atom_add_acquire(&tk.parts_left[task], -1) == 1;
        last = __shfl_sync(FULL, last, 0);
        if (last) fence_acq_rel_gpu();  // the other parts' writes, acquired above, released with ours
    }
    if (last) {
        // completion flag (for products started early and for a forward
        // substitution overlapping the factorisation; ordered after the
        // CTA's writes by the fence above), then the successors' counts
        if (lane == 0) st_relaxed(tk.task_done + task, 1);
        for (int k = tk.succ_ptr[task] + lane; k < tk.succ_ptr[task + 1]; k += 32)
            red_release_add(&tk.dep[tk.succ[k]], -1);
    }
}

// Static list scheduling. Every CTA claims the next position of a fixed item
// order (estimated start time, then longest remaining path) and waits,
// bounded, until that item's task has no unfinished predecessor; then runs it
// and releases its successors. Predecessors always come earlier in the order,
// so the smallest unfinished position can always run: with every CTA
// co-resident the launch cannot deadlock. A critical task is usually claimed
// before it is ready, so its claimant starts as soon as the count drops.
template <typename T, int S>
__global__ void __launch_bounds__(NT, (S == 1 || sizeof(T) == 8) ? 2 : 1) factor_ordered_kernel(const __grid_constant__ DevTasks tk, T* tiles) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sm = reinterpret_cast<T*>(smem_raw);
    __shared__ int s_item;
    __shared__ tc::State st;
    uint32_t phase = 0;
    if constexpr (sizeof(T) == 4) tc_setup(st);
    for (;;) {
        if (threadIdx.x == 0) {
            int item = -1;
            const int pos = atomicAdd(tk.head, 1);
            if (pos < tk.total_items) {
                item = tk.order[pos];
                const int task = item >> 4;
                if (task < 0 || task >= tk.ntasks) {
                    atomicOr(&tk.status->flags, ST_BAD_ITEM);
                    item = -1;
                } else {
                    unsigned long long t0 = 0;
                    unsigned spins = 0;
                    // a product started early waits per operand pair instead
                    const bool early = sizeof(T) == 4 && tk.early && (item & ITEM_EARLY) != 0;
                    while (!early && ld_acquire(tk.dep + task) > 0) {
                        if (spins == 0) t0 = globaltimer_ns();  // the clock only once waiting
                        if ((++spins & 15) == 0) {
                            if (ld_acquire(&tk.status->flags) & (ST_TIMEOUT | ST_BAD_ITEM)) { item = -1; break; }
                            if (globaltimer_ns() - t0 > tk.wait_limit_ns) {
                                atomicOr(&tk.status->flags, ST_TIMEOUT);
                                tk.status->timeout_where = pos;
                                item = -1;
                                break;
                            }
                        }
                        __nanosleep(32);
                    }
                    if (item >= 0 && tk.trace) {
                        unsigned smid;
                        asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
                        unsigned long long* tr = tk.trace + 4 * (size_t)task;
                        const unsigned long long now = globaltimer_ns();
                        atomicMax(tr + 0, now);   // ready: seen by the (last) claimant
                        atomicMax(tr + 1, ~now);  // start = min over parts, stored inverted
                        tr[3] = smid;
                    }
                }
            }
            s_item = item;  // the claimant's acquire passes to the CTA at the barrier
        }
        __syncthreads();
        const int item = s_item;
        if (item < 0) break;
        run_item<T, S>(tk, tiles, item >> 4, item & 7, tk.early && (item & ITEM_EARLY) != 0, sm, st, phase);
        __syncthreads();
        if (threadIdx.x < 32) {
            if (tk.trace && threadIdx.x == 0) atomicMax(tk.trace + 4 * (size_t)(item >> 4) + 2, globaltimer_ns());
            release_item(tk, item >> 4);
        }
    }
    if constexpr (sizeof(T) == 4) tc_teardown(st, tk);
}

template <typename T, int S>
__global__ void __launch_bounds__(NT) factor_level_kernel(const __grid_constant__ DevTasks tk, T* tiles, const int32_t* items) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sm = reinterpret_cast<T*>(smem_raw);
    __shared__ tc::State st;
    uint32_t phase = 0;
    if constexpr (sizeof(T) == 4) tc_setup(st);
    const int item = items[blockIdx.x];
    run_item<T, S>(tk, tiles, item >> 4, item & 7, false, sm, st, phase);
    if constexpr (sizeof(T) == 4) tc_teardown(st, tk);
}

template <typename T, int S>
int queue_launch(const DevTasks& t, T* tiles, int grid, cudaStream_t s) {
    const size_t smem = smem_elems<T, S>() * sizeof(T);
    cudaFuncSetAttribute(factor_queue_kernel<T, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    factor_queue_kernel<T, S><<<grid, NT, smem, s>>>(t, tiles);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <typename T, int S>
int ordered_launch(const DevTasks& t, T* tiles, int grid, cudaStream_t s) {
    const size_t smem = smem_elems<T, S>() * sizeof(T);
    cudaFuncSetAttribute(factor_ordered_kernel<T, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    factor_ordered_kernel<T, S><<<grid, NT, smem, s>>>(t, tiles);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <typename T, int S>
int level_launch(const DevTasks& t, T* tiles, const int32_t* items, int nitems, cudaStream_t s) {
    if (nitems <= 0) return 0;
    const size_t smem = smem_elems<T, S>() * sizeof(T);
    cudaFuncSetAttribute(factor_level_kernel<T, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    factor_level_kernel<T, S><<<nitems, NT, smem, s>>>(t, tiles, items);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace

// CTAs of one kernel co-resident on an SM with `smem` bytes of dynamic shared memory
template <typename K>
int resident_per_sm(K kernel, size_t smem) {
    int per_sm = 0;
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, NT, smem);
    return per_sm < 1 ? 1 : per_sm;
}

// One instantiation set per translation unit: executor `which` (0 ready
// queue, 1 static order, 2 per level) of the kernels for T and S.
template <typename T, int S>
int run_executor(int which, const DevTasks& t, T* tiles, const int32_t* items, int nitems, int grid, cudaStream_t s) {
    switch (which) {
        case 0: return queue_launch<T, S>(t, tiles, grid, s);
        case 1: return ordered_launch<T, S>(t, tiles, grid, s);
        default: return level_launch<T, S>(t, tiles, items, nitems, s);
    }
}
// persistent CTAs per SM: the smaller residency of the two persistent executors
template <typename T, int S>
int persistent_residency() {
    const size_t smem = smem_elems<T, S>() * sizeof(T);
    return std::min(resident_per_sm(factor_queue_kernel<T, S>, smem), resident_per_sm(factor_ordered_kernel<T, S>, smem));
}

}  // namespace sog
