// Solve-phase kernels for sm_103a: block forward (L) and back (U)
// substitution over the resident factor tiles (BlockPlanner::solve,
// BlockPlanner.cpp:652-862), the FP64 residual r = b - A x on the permuted
// matrix for iterative refinement, and the permutation gathers.
//
// Substitution runs as one persistent launch per triangle. Block rows are
// claimed in a fixed dealing order by resident CTAs; a CTA folds in each off-diagonal
// block as soon as the block row it multiplies is published (a per-row
// readiness flag), then solves its diagonal block and publishes its own row.
// Rows only wait on rows dealt earlier, so the smallest unfinished row can
// always proceed; every wait is bounded and reports a timeout status. A plain
// system runs in thread-block clusters that take consecutive rows together and
// hand each solved row to the cluster's later CTAs through distributed shared
// memory. A batch of independent systems deals its rows interleaved (row 0 of
// every system, then row 1, ...), so that neighbouring CTAs work on different
// systems.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <mutex>
#include <string>

#include "api_internal.h"
#include "kernels.h"

namespace sog {

namespace {

constexpr int NT = 256;

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// release/acquire fence at GPU scope: with the CTA barrier before it, it
// orders every thread's earlier writes before the flag or count that follows
// (the fence.sc that __threadfence() issues is stronger than a release needs)
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
__device__ __forceinline__ int ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// 16-byte read-only vector load of consecutive T (factor tiles are written by
// an earlier kernel, so the non-coherent path is safe here)
template <typename T>
struct Vec16 {
    T v[16 / sizeof(T)];
};
template <typename T>
__device__ __forceinline__ Vec16<T> ldg16(const T* p) {
    const int4 r = __ldg(reinterpret_cast<const int4*>(p));
    Vec16<T> o;
    memcpy(&o, &r, 16);
    return o;
}
// the same through L2 only, for tiles a concurrently running factor kernel
// has just written (FW: forward pass overlapping the factorisation)
template <bool FW, typename T>
__device__ __forceinline__ Vec16<T> ldt16(const T* p) {
    if constexpr (!FW) return ldg16(p);
    const int4 r = __ldcg(reinterpret_cast<const int4*>(p));
    Vec16<T> o;
    memcpy(&o, &r, 16);
    return o;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ---- thread-block clusters: distributed shared memory hand-over of solved rows
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
// address of the same shared variable in CTA `rank` of the cluster
__device__ __forceinline__ uint32_t map_rank(uint32_t addr, uint32_t rank) {
    uint32_t d;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(d) : "r"(addr), "r"(rank));
    return d;
}
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ void st_cluster_u32(uint32_t addr, uint32_t v) {
    asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
}
__device__ __forceinline__ void st_cluster_v4(uint32_t addr, int4 v) {
    asm volatile("st.shared::cluster.v4.s32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(v.x), "r"(v.y), "r"(v.z),
                 "r"(v.w)
                 : "memory");
}
__device__ __forceinline__ int ld_cluster_s32(uint32_t addr) {
    int v;
    asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(addr) : "memory");
    return v;
}
__device__ __forceinline__ void mbar_init_cta(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
// one arrival on the mbarrier at cluster address `addr`, releasing at cluster scope
__device__ __forceinline__ void mbar_arrive_remote(uint32_t addr) {
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(addr) : "memory");
}
__device__ __forceinline__ bool mbar_test_cluster(const uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// A row solved by a cluster rank goes through distributed shared memory to
// the next SOLVE_FANOUT ranks of its group; farther ranks, which need it
// several hops later, read it from global memory like rows of earlier groups
constexpr int SOLVE_FANOUT = 7;

// One launch per triangle and per chunk of NR right-hand-side columns
// [c0, c0+NR) of vec (n_ext x ld, row-major). For block row i the warps split
// its off-diagonal blocks: each warp waits (bounded) only for the row its
// block multiplies, stages that row's NR-column slice in shared memory and
// accumulates block * slice in registers (lane l: rows 2l, 2l+1). The warp
// partials and b_i are combined and multiplied by the precomputed inverse of
// the diagonal block. With look-ahead products M_d = Dinv_i * B_{i,j_d} for
// the SOLVE_LOOKAHEAD nearest rows j_d = i -+ d (d = 1, 2, ...), those blocks
// are left out of the sum and y_i = Dinv_i (b_i - sum) - sum_d M_d y_{j_d}
// is finished as the rows j_d are published, the farthest first: after the
// nearest row arrives the critical path is one 64x64 product. A row from
// global memory is staged in the warp's shared buffer before its product.
// The row is then published with a release store.
//
// CL > 1 (a plain system, no dealing order): the CTAs of a thread-block
// cluster take CL consecutive rows of one column chunk together (cluster rank
// r: the r-th row in dealing order). A solved row is also stored straight into
// the shared memory of the next SOLVE_FANOUT ranks of the cluster, with one
// mbarrier arrival per receiving rank, so the hand-over between neighbouring
// rows of a group is a distributed-shared-memory store and an mbarrier wait
// instead of an L2 round trip behind a GPU-scope fence and a polled flag;
// rows of earlier groups come through the global flags as before. The ranks finish a group
// with a cluster barrier (their receive slots are then free), after which
// rank 0's claim of the next group is read by all. Results are bit-identical
// to CL = 1: the same products in the same order, only the source of the
// neighbouring rows' values differs.
// smem: part[8][64*NR] | ybuf[8][NVP] | acc[64*NR] | slot[CL][NVP] (CL > 1).
// A staged row (ybuf, slot) keeps each block row's NR values together, with
// 16 bytes of padding after every 16 rows: the four lanes of a row quad read
// rows 16 apart without bank conflicts, 16 bytes at a time.
//
// FW (forward pass overlapping the factorisation, CL = 1): a row first waits
// (warp 0, bounded) for the factor tasks that produce its tiles, then reads
// them through L2 only, with no L1 prefetch.
template <typename T, int NR, int CL, bool FW = false>
__global__ void __launch_bounds__(NT) trisolve_kernel(DevSolve s, const T* __restrict__ tiles, T* vec, int ld,
                                                      int cbase, int nch, int epoch, int lower) {
    static_assert(!FW || CL == 1, "the overlapped forward pass runs unclustered");
    constexpr int FAN = CL - 1 < SOLVE_FANOUT ? CL - 1 : SOLVE_FANOUT;  // hand-over reach in ranks
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int NV = 64 * NR;
    constexpr int PADE = 16 / (int)sizeof(T);  // elements of 16 bytes
    constexpr int NVP = NV + 4 * PADE;         // a staged row with its padding
    // element (row, r) of a staged row
    auto pidx = [](int row, int r) { return row * NR + r + (row >> 4) * PADE; };
    constexpr int VW = 16 / (int)sizeof(T);  // elements per 16-byte load
    T* part = reinterpret_cast<T*>(smem_raw);
    T* ybuf = part + 8 * NV;
    T* acc = ybuf + 8 * NVP;
    T* slot = acc + NV;  // CL > 1: slot[r] holds the row solved by cluster rank r of this group
    __shared__ int s_stop, s_next;
    __shared__ int s_claim[2], s_cstop;           // CL > 1: rank 0's claims (by group parity), stop flag
    __shared__ __align__(8) uint64_t s_bar[CL];   // CL > 1: s_bar[r]: rank r's row delivered here
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int R = s.block_rows;
    const int* ptr = lower ? s.l_ptr : s.u_ptr;
    const int* col = lower ? s.l_col : s.u_col;
    const int* ids = lower ? s.l_id : s.u_id;
    const int* dinv = lower ? s.l_dinv : s.u_dinv;
    const int32_t* const* lookahead = lower ? s.l_la : s.u_la;
    const int dir = lower ? -1 : 1;  // the rows a row waits on lie on this side
    const int* order = lower ? s.order_l : s.order_u;
    int* claim = s.claim + (lower ? 0 : 1);
    const int rank = CL > 1 ? (int)cluster_rank() : 0;
    const int ngroups = (R + CL - 1) / CL * nch;
    if (tid == 0) {
        s_stop = 0;
        if constexpr (CL > 1) {
            s_cstop = 0;
            if (rank == 0) s_claim[0] = atomicAdd(claim, 1);
        } else {
            s_next = atomicAdd(claim, 1);
        }
    }
    if constexpr (CL > 1) {
        if (tid < CL) mbar_init_cta(&s_bar[tid], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        cluster_sync_all();
        if (tid == 0) s_next = ld_cluster_s32(map_rank(smem_addr(&s_claim[0]), 0));
    }
    __syncthreads();
    T* yw = ybuf + warp * NVP;
    // row j's NR-column slice [c0, c0+NR) of vec into this warp's buffer yw
    // (staged layout); vec is written by other CTAs of the launch: L2 loads
    auto stage_row = [&](int j, int c0, bool vec16) {
        const T* vj = vec + (size_t)j * 64 * ld + c0;
        __syncwarp();  // the warp's earlier reads of yw are done
        if constexpr ((NR * (int)sizeof(T)) % 16 == 0) {
            if (vec16) {
                constexpr int Q = NR * (int)sizeof(T) / 16;  // 16-byte pieces per block row
#pragma unroll
                for (int e = lane; e < 64 * Q; e += 32) {
                    const int row = e / Q, h = e - row * Q;
                    const int4 w4 = __ldcg(reinterpret_cast<const int4*>(vj + (size_t)row * ld) + h);
                    *reinterpret_cast<int4*>(yw + pidx(row, h * PADE)) = w4;
                }
                __syncwarp();
                return;
            }
        }
        for (int e = lane; e < NV; e += 32) yw[pidx(e / NR, e % NR)] = __ldcg(vj + (size_t)(e / NR) * ld + (e % NR));
        __syncwarp();
    };
    // bounded wait of lane 0 for row j's flag; the warp's later reads of row j
    // are ordered after lane 0's acquire by the __syncwarp that follows
    const int* fl = nullptr;  // this position's chunk of the flags
    auto wait_row = [&](int j) -> bool {
        if (lane == 0 && ld_acquire(fl + j) != epoch) {  // the clock only once waiting
            const unsigned long long t0 = globaltimer_ns();
            while (ld_acquire(fl + j) != epoch) {
                if (globaltimer_ns() - t0 > s.wait_limit_ns) {
                    atomicOr(&s.status->flags, ST_SOLVE_TIMEOUT);
                    s_stop = 1;
                    break;
                }
                __nanosleep(32);
            }
        }
        __syncwarp();
        return !*(volatile int*)&s_stop;
    };
    uint32_t gpar = 0;  // CL > 1: phase parity of s_bar for this group
    // bounded wait (every lane) for the row of cluster rank `snd` of this group
    auto wait_rank = [&](int snd) -> bool {
        if (!mbar_test_cluster(&s_bar[snd], gpar)) {
            const unsigned long long t0 = globaltimer_ns();
            while (!mbar_test_cluster(&s_bar[snd], gpar)) {
                if (globaltimer_ns() - t0 > s.wait_limit_ns) {
                    if (lane == 0) atomicOr(&s.status->flags, ST_SOLVE_TIMEOUT);
                    s_stop = 1;
                    break;
                }
            }
        }
        __syncwarp();
        return !*(volatile int*)&s_stop;
    };
    // positions: nch column chunks of each row in turn, rows in dealing order
    // (CL > 1: groups of CL rows), claimed in dealing order (the next one
    // while this one runs): a row only waits on rows dealt earlier, which
    // resident CTAs hold
    for (int k = s_next; k < ngroups; k = s_next) {
        __syncthreads();  // every thread has read s_next
        if (tid == 0) {
            if constexpr (CL > 1) {
                if (rank == 0) s_claim[gpar ^ 1u] = atomicAdd(claim, 1);
            } else {
                s_next = atomicAdd(claim, 1);
            }
        }
        const int kg = k / nch, ch = k - kg * nch, c0 = cbase + ch * NR;
        // this chunk's rows of vec in 16-byte pieces
        const bool vec16 = ((size_t)ld * sizeof(T)) % 16 == 0 && ((size_t)c0 * sizeof(T)) % 16 == 0;
        const int kk = kg * CL + rank, kk0 = kg * CL;
        const bool have = kk < R;  // CL > 1: the last group may be short
        const int i = !have ? 0 : (order ? order[kk] : (lower ? kk : R - 1 - kk));
        // CL > 1: rows of this group lie on the waiting side of row i, up to
        // the group's first row: sender rank of row j, -1 = an earlier group
        auto rank_of = [&](int j) -> int {
            if constexpr (CL == 1) return -1;
            const int d = lower ? j - kk0 : (R - 1 - kk0) - j;
            return d >= 0 && d < rank && rank - d <= FAN ? d : -1;
        };
        fl = s.flags + (size_t)ch * R;
        bool stop = false;
        if (have) {
        if (s.trace && tid == 0) s.trace[4 * (size_t)i + (lower ? 0 : 2)] = globaltimer_ns();
        if constexpr (FW) {
            // the factor tasks producing this row's tiles (acquire by warp 0,
            // passed to the CTA by the barrier)
            if (warp == 0) {
                for (int q = s.fwait_ptr[i] + lane; q < s.fwait_ptr[i + 1]; q += 32) {
                    const int* f = s.task_done + s.fwait[q];
                    if (ld_acquire(f) != 0) continue;
                    const unsigned long long t0 = globaltimer_ns();
                    while (ld_acquire(f) == 0) {
                        // a factorisation that gave up never finishes the task
                        if ((ld_acquire(&s.status->flags) & ST_TIMEOUT) ||
                            globaltimer_ns() - t0 > s.wait_limit_ns) {
                            atomicOr(&s.status->flags, ST_SOLVE_TIMEOUT);
                            s_stop = 1;
                            break;
                        }
                        __nanosleep(64);
                    }
                }
            }
            __syncthreads();
            stop = *(volatile int*)&s_stop != 0;
        }
        const T* Dm = tiles + (size_t)dinv[i] * 4096;
        // this thread's values of b_i (row i of vec is written only by this
        // CTA, at its end): loaded now, used after the products
        constexpr int NB = (NV + NT - 1) / NT;
        T bv[NB];
#pragma unroll
        for (int k = 0; k < NB; k++) {
            const int e = tid + k * NT;
            bv[k] = e < NV ? __ldcg(vec + ((size_t)i * 64 + e / NR) * ld + c0 + (e % NR)) : T(0);
        }
        // look-ahead products of this row by distance (la[d-1]: row i + d*dir)
        int la[SOLVE_LOOKAHEAD], nla = 0;
#pragma unroll
        for (int d = 0; d < SOLVE_LOOKAHEAD; d++) {
            la[d] = lookahead[d] ? lookahead[d][i] : 0;
            nla += la[d] > 0;
        }
        // warm L1 with this lane's slice of the diagonal inverse
        if constexpr (!FW)
            asm volatile("prefetch.global.L1 [%0];" ::"l"(Dm + (warp * 8 + (lane >> 2)) * 64 + (lane & 3) * 16));
        T pa[NR], pb[NR];
#pragma unroll
        for (int r = 0; r < NR; r++) pa[r] = pb[r] = T(0);
        // with look-ahead products the last blocks (the neighbouring rows; the
        // lists run in readiness order) are left out
        const int q1 = ptr[i + 1] - nla;
        for (int q = ptr[i] + warp; q < q1 && !stop; q += 8) {
            const int j = col[q];
            const T* B = tiles + (size_t)ids[q] * 4096 + (2 * lane) * 64;
            // warm L1 with the lane's two block rows (128 contiguous elements) while waiting
            if constexpr (!FW) {
#pragma unroll
                for (int o = 0; o < 128; o += 128 / (int)sizeof(T))
                    asm volatile("prefetch.global.L1 [%0];" ::"l"(B + o));
            }
            const int snd = rank_of(j);
            const T* ys = yw;
            if (snd >= 0) {
                if (!wait_rank(snd)) {
                    stop = true;
                    break;
                }
                ys = slot + snd * NVP;
            } else {
                if (!wait_row(j)) {
                    stop = true;
                    break;
                }
                stage_row(j, c0, vec16);
            }
#pragma unroll 4
            for (int c = 0; c < 64; c += VW) {
                const Vec16<T> b0 = ldt16<FW>(B + c), b1 = ldt16<FW>(B + 64 + c);
#pragma unroll
                for (int v = 0; v < VW; v++)
#pragma unroll
                    for (int r = 0; r < NR; r++) {
                        const T y = ys[pidx(c + v, r)];
                        pa[r] += b0.v[v] * y;
                        pb[r] += b1.v[v] * y;
                    }
            }
            __syncwarp();
        }
        T* pw = part + warp * NV;
#pragma unroll
        for (int r = 0; r < NR; r++) {
            pw[(2 * lane) * NR + r] = pa[r];
            pw[(2 * lane + 1) * NR + r] = pb[r];
        }
        __syncthreads();
        stop = stop || s_stop;
        if (!stop) {
#pragma unroll
        for (int k = 0; k < NB; k++) {
            const int e = tid + k * NT;
            if (e < NV) {
                T v = bv[k];
#pragma unroll
                for (int w = 0; w < 8; w++) v -= part[w * NV + e];
                acc[e] = v;
            }
        }
        }
        __syncthreads();
        // y_i = inv(D_ii) * acc [- M * y_j]: warp w rows 8w..8w+7, four lanes
        // per row, each lane 16 columns; partial sums reduced over the four lanes
        if (!stop) {
            const int row = warp * 8 + (lane >> 2), cb = (lane & 3) * 16;
            Vec16<T> m[16 / VW];
            if (la[0] > 0) {  // the nearest row's look-ahead slice, loaded before the wait
                const T* M = tiles + (size_t)la[0] * 4096 + row * 64 + cb;
#pragma unroll
                for (int c = 0; c < 16 / VW; c++) m[c] = ldt16<FW>(M + c * VW);
            }
            if constexpr (!FW) {
#pragma unroll
                for (int d = 1; d < SOLVE_LOOKAHEAD; d++)
                    if (la[d] > 0)
                        asm volatile("prefetch.global.L1 [%0];" ::"l"(tiles + (size_t)la[d] * 4096 + row * 64 + cb));
            }
            T y[NR];
#pragma unroll
            for (int r = 0; r < NR; r++) y[r] = T(0);
#pragma unroll
            for (int c = 0; c < 16; c += VW) {
                const Vec16<T> d = ldt16<FW>(Dm + row * 64 + cb + c);
#pragma unroll
                for (int v = 0; v < VW; v++)
#pragma unroll
                    for (int r = 0; r < NR; r++) y[r] += d.v[v] * acc[(cb + c + v) * NR + r];
            }
            // y -= M y_j over this lane's 16 columns (all warps: a 64x64 product
            // split over the CTA instead of one warp's block product). Row j
            // comes from this CTA's shared memory: within a cluster group from
            // the sender's slot, otherwise staged from global memory into the
            // warp's buffer first (independent 16-byte L2 loads, one round
            // trip, instead of loads interleaved with the products)
            auto apply = [&](const Vec16<T>* mm, int j, int snd) {
                const T* sj;
                if (CL > 1 && snd >= 0) {
                    sj = slot + snd * NVP;
                } else {
                    stage_row(j, c0, vec16);
                    sj = yw;
                }
#pragma unroll
                for (int c = 0; c < 16 / VW; c++)
#pragma unroll
                    for (int v = 0; v < VW; v++) {
                        T yj[NR];
                        const T* q = sj + pidx(cb + c * VW + v, 0);
                        if constexpr ((NR * (int)sizeof(T)) % 16 == 0) {
#pragma unroll
                            for (int h = 0; h < NR * (int)sizeof(T) / 16; h++) {
                                const int4 w4 = reinterpret_cast<const int4*>(q)[h];
                                memcpy(&yj[h * PADE], &w4, 16);
                            }
                        } else {
#pragma unroll
                            for (int r = 0; r < NR; r++) yj[r] = q[r];
                        }
#pragma unroll
                        for (int r = 0; r < NR; r++) y[r] -= mm[c].v[v] * yj[r];
                    }
            };
            auto wait_any = [&](int j, int snd) { return snd >= 0 ? wait_rank(snd) : wait_row(j); };
            // the farthest look-ahead row first (Md = Dinv_i B_{i,i+d*dir}),
            // the nearest last; a wait that runs out sets s_stop: the CTA
            // publishes nothing
            bool ok = true;
#pragma unroll
            for (int d = SOLVE_LOOKAHEAD - 1; d >= 1; d--) {
                if (ok && la[d] > 0) {
                    const int jd = i + (d + 1) * dir, sndd = rank_of(jd);
                    ok = wait_any(jd, sndd);
                    if (ok) {
                        Vec16<T> md[16 / VW];
                        const T* M = tiles + (size_t)la[d] * 4096 + row * 64 + cb;
#pragma unroll
                        for (int c = 0; c < 16 / VW; c++) md[c] = ldt16<FW>(M + c * VW);
                        apply(md, jd, sndd);
                    }
                }
            }
            if (ok && la[0] > 0) {
                const int j1 = i + dir, snd1 = rank_of(j1);
                if (wait_any(j1, snd1)) apply(m, j1, snd1);
            }
#pragma unroll
            for (int r = 0; r < NR; r++) {
                y[r] += __shfl_xor_sync(0xffffffffu, y[r], 1);
                y[r] += __shfl_xor_sync(0xffffffffu, y[r], 2);
            }
            if ((lane & 3) == 0) {
                if (CL == 1 || rank == CL - 1) {
                    // no later rank: straight to global memory, where the next
                    // group's first rows wait for it
#pragma unroll
                    for (int r = 0; r < NR; r++) vec[((size_t)i * 64 + row) * ld + c0 + r] = y[r];
                } else {
                    // the row into this CTA's own slot (copied to vec below,
                    // once the later ranks have it) and into slot[rank] of
                    // every later rank of the group
                    T* own = slot + rank * NVP + pidx(row, 0);
#pragma unroll
                    for (int r = 0; r < NR; r++) own[r] = y[r];
                    const uint32_t src = smem_addr(own);
                    for (int dst = rank + 1; dst < CL && dst <= rank + FAN; dst++) {
                        const uint32_t a = map_rank(src, (uint32_t)dst);
                        if constexpr ((NR * (int)sizeof(T)) % 16 == 0) {
#pragma unroll
                            for (int q = 0; q < NR * (int)sizeof(T) / 16; q++) {
                                int4 v;
                                memcpy(&v, reinterpret_cast<const char*>(y) + 16 * q, 16);
                                st_cluster_v4(a + 16 * q, v);
                            }
                        } else {
#pragma unroll
                            for (int q = 0; q < NR * (int)sizeof(T) / 4; q++) {
                                uint32_t v;
                                memcpy(&v, reinterpret_cast<const char*>(y) + 4 * q, 4);
                                st_cluster_u32(a + 4 * q, v);
                            }
                        }
                    }
                }
            }
        }
        }  // have
        __syncthreads();
        stop = stop || s_stop;
        if (CL > 1 && rank < CL - 1) {
            // the later ranks first: their hand-over then waits for no global
            // store (a fence waits for the stores issued before it). Every
            // later rank's barrier completes one phase per group (also when
            // this rank has no row or stopped), so that the parities stay in
            // step.
            if (warp == 0) {  // one lane per later rank: the arrivals go out together
                if (lane == 0) asm volatile("fence.acq_rel.cluster;" ::: "memory");
                __syncwarp();
                const int dst = rank + 1 + lane;
                if (dst < CL && dst <= rank + FAN) mbar_arrive_remote(map_rank(smem_addr(&s_bar[rank]), (uint32_t)dst));
                if (lane == 0 && stop) st_cluster_u32(map_rank(smem_addr(&s_cstop), 0), 1u);
            }
            __syncthreads();
            if (have && !stop)
                for (int e = tid; e < NV; e += NT)
                    vec[((size_t)i * 64 + e / NR) * ld + c0 + (e % NR)] = slot[rank * NVP + pidx(e / NR, e % NR)];
            __syncthreads();
        }
        if (CL > 1 && rank == CL - 1 && tid == 0 && stop) st_cluster_u32(map_rank(smem_addr(&s_cstop), 0), 1u);
        if (tid == 0) {
            if (have && !stop) {
                fence_acq_rel_gpu();  // the row written by all threads (ordered by the barrier) before the flag
                st_release(s.flags + (size_t)ch * R + i, epoch);
                if (s.trace) s.trace[4 * (size_t)i + (lower ? 1 : 3)] = globaltimer_ns();
            }
        }
        if constexpr (CL > 1) {
            // the group is done in every rank (its slots are free); rank 0's
            // claim of the next group and any rank's stop are visible
            cluster_sync_all();
            gpar ^= 1u;
            if (tid == 0) {
                const int st0 = ld_cluster_s32(map_rank(smem_addr(&s_cstop), 0));
                s_next = st0 ? ngroups : ld_cluster_s32(map_rank(smem_addr(&s_claim[gpar]), 0));
            }
            __syncthreads();
        } else {
            if (stop) return;
            __syncthreads();  // thread 0's next claim is visible
        }
    }
    if constexpr (CL > 1) cluster_sync_all();  // no rank leaves while another may still store into it
}

template <typename T, int NR, int CL>
size_t trisolve_smem() {
    const size_t nv = 64 * NR, nvp = nv + 4 * (16 / sizeof(T));
    return (9 * nv + (8 + (CL > 1 ? CL : 0)) * nvp) * sizeof(T);
}

// rows per cluster group of the substitution of a plain system
constexpr int SOLVE_CLUSTER = 8;

template <typename T, int NR, int CL>
int trisolve_pair(const DevSolve& s, const T* tiles, T* vec, int ld, int c0, int nch, int epoch, int grid,
                  cudaStream_t st) {
    const size_t smem = trisolve_smem<T, NR, CL>();
    auto kern = trisolve_kernel<T, NR, CL>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (CL > 8) cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaMemsetAsync(s.claim, 0, 8, st);
    if constexpr (CL == 1) {
        kern<<<grid, NT, smem, st>>>(s, tiles, vec, ld, c0, nch, epoch, 1);
        kern<<<grid, NT, smem, st>>>(s, tiles, vec, ld, c0, nch, epoch + 1, 0);
    } else {
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = CL;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3(grid);
        cfg.blockDim = dim3(NT);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = st;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        if (cudaLaunchKernelEx(&cfg, kern, s, tiles, vec, ld, c0, nch, epoch, 1) != cudaSuccess) return -1;
        if (cudaLaunchKernelEx(&cfg, kern, s, tiles, vec, ld, c0, nch, epoch + 1, 0) != cudaSuccess) return -1;
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// resident clusters of CL CTAs of the kernel (0: cannot be launched so)
template <typename T, int NR, int CL>
int resident_clusters() {
    const size_t smem = trisolve_smem<T, NR, CL>();
    auto kern = trisolve_kernel<T, NR, CL>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
        (CL > 8 && cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)) {
        cudaGetLastError();
        return 0;
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = CL;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(CL);
    cfg.blockDim = dim3(NT);
    cfg.dynamicSmemBytes = smem;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

// One launch pair (lower, upper) for nch column chunks of NR columns. A plain
// system (no dealing order) runs in clusters when at least one cluster fits
// the grid bound: at most grid CTAs, a multiple of the cluster size.
template <typename T, int NR>
int trisolve_chunk(const DevSolve& s, const T* tiles, T* vec, int ld, int c0, int nch, int& epoch, int grid,
                   cudaStream_t st) {
    int rc = 1;
    // clusters for full 8-column chunks: with one right-hand side the
    // hand-over saves less than the group barrier costs (48^3: 22.1 against
    // 20.0 ms)
    if constexpr (NR == 8) {
        constexpr int CL = SOLVE_CLUSTER;
        // the kernel's resident clusters, queried once (every GPU this
        // library drives is the same model)
        static std::atomic<int> cached{-1};
        int clusters = cached.load(std::memory_order_relaxed);
        if (clusters < 0) {
            clusters = resident_clusters<T, NR, CL>();
            cached.store(clusters, std::memory_order_relaxed);
        }
        const bool plain = s.order_l == nullptr && s.order_u == nullptr;
        if (plain && clusters > 0 && grid >= CL) {
            const int groups = (s.block_rows + CL - 1) / CL * nch;
            const int ncl = std::max(1, std::min({clusters, groups, grid / CL}));
            rc = trisolve_pair<T, NR, CL>(s, tiles, vec, ld, c0, nch, epoch, ncl * CL, st);
        }
    }
    if (rc == 1) rc = trisolve_pair<T, NR, 1>(s, tiles, vec, ld, c0, nch, epoch, grid, st);
    epoch += 2;
    return rc;
}

template <typename T>
int trisolve_impl(const DevSolve& s, const T* tiles, T* vec, int nrhs, int& epoch, int grid, cudaStream_t st,
                  int& launches) {
    int rc = 0;
    for (int c0 = 0; c0 < nrhs && rc == 0;) {
        const int left = nrhs - c0;
        if (left >= 8) {
            const int nch = std::min(left / 8, TRISOLVE_MAX_CHUNKS);
            rc = trisolve_chunk<T, 8>(s, tiles, vec, nrhs, c0, nch, epoch, grid, st);
            c0 += 8 * nch;
        } else if (left >= 4) { rc = trisolve_chunk<T, 4>(s, tiles, vec, nrhs, c0, 1, epoch, grid, st); c0 += 4; }
        else if (left >= 2) { rc = trisolve_chunk<T, 2>(s, tiles, vec, nrhs, c0, 1, epoch, grid, st); c0 += 2; }
        else { rc = trisolve_chunk<T, 1>(s, tiles, vec, nrhs, c0, 1, epoch, grid, st); c0 += 1; }
        launches += 2;
    }
    return rc;
}

template <typename T, int NR>
int occupancy_grid(int num_sms) {
    int per_sm = 0;
    const size_t smem = trisolve_smem<T, NR, 1>();
    cudaFuncSetAttribute(trisolve_kernel<T, NR, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, trisolve_kernel<T, NR, 1>, NT, smem);
    return (per_sm < 1 ? 1 : per_sm) * num_sms;
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
__global__ void scatter_csr_kernel(const double* __restrict__ V, const int32_t* __restrict__ vidx,
                                   const int32_t* __restrict__ pos, int64_t nnz, double* __restrict__ val) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nnz && pos[k] >= 0) val[pos[k]] = V[vidx ? vidx[k] : k];
}

__global__ void cast_kernel(const double* __restrict__ s, float* __restrict__ d, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        d[i] = (float)s[i];
}
__global__ void axpy_kernel(const float* __restrict__ d, double* __restrict__ x, int64_t n, int assign) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = assign ? (double)d[i] : x[i] + (double)d[i];
}
// one thread per (permuted row, column) of the chunk; systems are whole
// 64-row block rows, so the system lookup is one load per row
__global__ void gather_seg_kernel(const double* __restrict__ b, DevSegs g, int n_ext, int c0, int nc,
                                  double* __restrict__ out) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)n_ext * nc) return;
    const int i = (int)(e / nc), c = (int)(e - (int64_t)i * nc), col = c0 + c;
    const int k = g.of_brow[i >> 6], o = g.n2o[i];
    double v = 1.0;
    if (o >= 0) v = col < g.nrhs[k] ? b[g.voff[k] + (int64_t)col * g.n[k] + o] : 0.0;
    out[e] = v;
}
__global__ void scatter_seg_kernel(const double* __restrict__ xe, DevSegs g, int n_ext, int c0, int nc,
                                   double* __restrict__ x, unsigned long long* cnt) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)n_ext * nc) return;
    const int i = (int)(e / nc), c = (int)(e - (int64_t)i * nc), col = c0 + c;
    const int k = g.of_brow[i >> 6], o = g.n2o[i];
    if (o < 0 || col >= g.nrhs[k]) return;
    const double v = xe[e];
    x[g.voff[k] + (int64_t)col * g.n[k] + o] = v;
    if (!isfinite(v)) atomicAdd(cnt + k, 1ull);
}
// as residual_kernel, reductions per (system, column). Each CTA walks a
// contiguous range of 64-row block rows (a block row belongs to one system).
// Its first nc * (256 / nc) threads each keep one column c = t % nc and rows
// t / nc, t / nc + 256 / nc, ... of every block row, so the lanes of a warp
// read consecutive columns of x and b (coalesced for nc >= 32; several rows
// per warp for fewer columns), and each thread accumulates its column's sums
// and maxima in registers. Partial results leave once per system the range
// touches: shared-memory atomics per column, then one global atomic per
// (column, slot) and CTA, instead of one per (warp, column, slot). r is
// formed exactly as in residual_kernel (same products in the same order).
constexpr int RES_THREADS = 256;
constexpr int RES_CTAS = 4 * 152;  // four per SM of a GB300
__global__ void __launch_bounds__(RES_THREADS) residual_seg_kernel(DevCSR A, const double* __restrict__ b,
                                                                 const double* __restrict__ x, double* __restrict__ r,
                                                                 int c0, int nc, double* red, DevSegs g, int nbr) {
    __shared__ double s_acc[64 * 5];
    __shared__ double s_rowabs;
    const int t = threadIdx.x;
    const int rpp = RES_THREADS / nc;  // rows per pass over a block row
    const bool act = t < rpp * nc;
    const int c = act ? t % nc : 0, roff = act ? t / nc : 0;
    const int br0 = (int)((int64_t)blockIdx.x * nbr / gridDim.x);
    const int br1 = (int)((int64_t)(blockIdx.x + 1) * nbr / gridDim.x);
    for (int i = t; i < 64 * 5; i += RES_THREADS) s_acc[i] = 0.0;
    if (t == 0) s_rowabs = 0.0;
    __syncthreads();
    double rr = 0, bb = 0, ar = 0, ax = 0, ab = 0, rowabs = 0;
    auto smax = [](double* p, double v) {
        atomicMax(reinterpret_cast<unsigned long long*>(p), (unsigned long long)__double_as_longlong(v));
    };
    // this CTA's partial results for system k -> red; uniform across the CTA
    auto flush = [&](int k) {
        const int creal = min(nc, g.nrhs[k] - c0);
        if (act && c < creal) {
            atomicAdd(&s_acc[c * 5 + 0], rr);
            atomicAdd(&s_acc[c * 5 + 1], bb);
            smax(&s_acc[c * 5 + 2], ar);
            smax(&s_acc[c * 5 + 3], ax);
            smax(&s_acc[c * 5 + 4], ab);
            smax(&s_rowabs, rowabs);
        }
        rr = bb = ar = ax = ab = rowabs = 0;
        __syncthreads();
        for (int i = t; i < max(creal, 0) * RED; i += RES_THREADS) {
            const int cc = i / RED, slot = i % RED;
            double* rd = red + ((size_t)k * nc + cc) * RED + slot;
            if (slot < 2) atomicAdd(rd, s_acc[cc * 5 + slot]);
            else atomic_max_nonneg(rd, slot < 5 ? s_acc[cc * 5 + slot] : s_rowabs);
        }
        __syncthreads();
        for (int i = t; i < 64 * 5; i += RES_THREADS) s_acc[i] = 0.0;
        if (t == 0) s_rowabs = 0.0;
        __syncthreads();
    };
    int k = br0 < br1 ? g.of_brow[br0] : 0;
    for (int br = br0; br < br1; br++) {
        const int kb = g.of_brow[br];
        if (kb != k) {
            flush(k);
            k = kb;
        }
        const int creal = min(nc, g.nrhs[k] - c0);
        if (!act) continue;
        for (int rw = roff; rw < 64; rw += rpp) {
            const int row = br * 64 + rw;
            const int q0 = A.ptr[row], q1 = A.ptr[row + 1];
            double acc = 0, ra = 0;
            for (int q = q0; q < q1; q++) {
                const double a = A.val[q];
                acc += a * x[(size_t)A.col[q] * nc + c];
                ra += fabs(a);
            }
            const double bv = b[(size_t)row * nc + c];
            const double rv = bv - acc;
            r[(size_t)row * nc + c] = rv;
            if (c < creal && g.n2o[row] >= 0) {
                rr += rv * rv;
                bb += bv * bv;
                ar = fmax(ar, fabs(rv));
                ax = fmax(ax, fabs(x[(size_t)row * nc + c]));
                ab = fmax(ab, fabs(bv));
                rowabs = fmax(rowabs, ra);
            }
        }
    }
    if (br0 < br1) flush(k);
}
// max |a_ij| per system: one thread per permuted row, a warp's 32 rows lie in
// one 64-row block row (one system); padding rows skipped
__global__ void csr_absmax_seg_kernel(DevCSR A, DevSegs g, unsigned long long* out) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row - (threadIdx.x & 31) >= A.n) return;  // whole warp past the end (A.n is a multiple of 64)
    double m = 0;
    if (row < A.n && g.n2o[row] >= 0)
        for (int q = A.ptr[row]; q < A.ptr[row + 1]; q++) m = fmax(m, fabs(A.val[q]));
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0)
        atomicMax(out + g.of_brow[row >> 6], (unsigned long long)__double_as_longlong(m));
}
__global__ void absmax_kernel(const double* __restrict__ v, int64_t n, unsigned long long* out) {
    double m = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        m = fmax(m, fabs(v[i]));
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}
__global__ void gather_tiles_kernel(const int4* __restrict__ src, int4* __restrict__ dst, const int32_t* ids,
                                    int64_t n, int per_tile) {
    const int64_t tot = n * per_tile;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = e / per_tile, o = e - k * per_tile;
        dst[(k + 1) * per_tile + o] = __ldcg(src + (int64_t)ids[k] * per_tile + o);
    }
}
__global__ void cast_seg_kernel(const double* __restrict__ src, float* __restrict__ dst, int n_ext, int nc,
                                DevSegs g) {
    const int64_t tot = (int64_t)n_ext * nc;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(e / nc);
        dst[e] = g.active[g.of_brow[i >> 6]] ? (float)src[e] : 0.0f;
    }
}

}  // namespace

int trisolve_launch(const DevSolve& s, const double* tiles, double* vec, int nrhs, int& epoch, int grid,
                    cudaStream_t st, int& launches) {
    return trisolve_impl<double>(s, tiles, vec, nrhs, epoch, grid, st, launches);
}
int trisolve_launch(const DevSolve& s, const float* tiles, float* vec, int nrhs, int& epoch, int grid,
                    cudaStream_t st, int& launches) {
    return trisolve_impl<float>(s, tiles, vec, nrhs, epoch, grid, st, launches);
}
int trisolve_lower_overlap_launch(const DevSolve& s, const float* tiles, float* vec, int nrhs, int epoch, int grid,
                                  cudaStream_t st) {
    if (!s.fwait_ptr || !(nrhs == 1 || (nrhs % 8 == 0 && nrhs <= 8 * TRISOLVE_MAX_CHUNKS)) || grid < 1) return -1;
    cudaMemsetAsync(s.claim, 0, 8, st);
    if (nrhs == 1) {
        const size_t smem = trisolve_smem<float, 1, 1>();
        auto kern = trisolve_kernel<float, 1, 1, true>;
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        kern<<<grid, NT, smem, st>>>(s, tiles, vec, nrhs, 0, 1, epoch, 1);
    } else {
        const size_t smem = trisolve_smem<float, 8, 1>();
        auto kern = trisolve_kernel<float, 8, 1, true>;
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        kern<<<grid, NT, smem, st>>>(s, tiles, vec, nrhs, 0, nrhs / 8, epoch, 1);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int trisolve_lower_join_launch(const DevSolve& s, const float* tiles, float* vec, int nrhs, int epoch, int grid,
                               cudaStream_t st) {
    if (!(nrhs == 1 || (nrhs % 8 == 0 && nrhs <= 8 * TRISOLVE_MAX_CHUNKS)) || grid < 1) return -1;
    // the overlapped pass's kernel without its factor waits, on the same
    // claim counter (not zeroed again) and flags
    if (nrhs == 1) {
        const size_t smem = trisolve_smem<float, 1, 1>();
        auto kern = trisolve_kernel<float, 1, 1>;
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        kern<<<grid, NT, smem, st>>>(s, tiles, vec, nrhs, 0, 1, epoch, 1);
    } else {
        const size_t smem = trisolve_smem<float, 8, 1>();
        auto kern = trisolve_kernel<float, 8, 1>;
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        kern<<<grid, NT, smem, st>>>(s, tiles, vec, nrhs, 0, nrhs / 8, epoch, 1);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int trisolve_upper_launch(const DevSolve& s, const float* tiles, float* vec, int nrhs, int epoch1, int grid,
                          cudaStream_t st) {
    if (!(nrhs == 1 || (nrhs % 8 == 0 && nrhs <= 8 * TRISOLVE_MAX_CHUNKS)) || grid < 1) return -1;
    if (nrhs == 1) {
        const size_t smem = trisolve_smem<float, 1, 1>();
        auto kern = trisolve_kernel<float, 1, 1>;
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        kern<<<grid, NT, smem, st>>>(s, tiles, vec, nrhs, 0, 1, epoch1, 0);
        return cudaGetLastError() == cudaSuccess ? 0 : -1;
    }
    // clusters as in trisolve_chunk (the upper counter was zeroed with the lower one)
    constexpr int CL = SOLVE_CLUSTER;
    const int nch = nrhs / 8;
    const int clusters = resident_clusters<float, 8, CL>();
    const bool plain = s.order_l == nullptr && s.order_u == nullptr;
    const size_t smem_cl = trisolve_smem<float, 8, CL>();
    if (plain && clusters > 0 && grid >= CL) {
        const int groups = (s.block_rows + CL - 1) / CL * nch;
        const int ncl = std::max(1, std::min({clusters, groups, grid / CL}));
        auto kern = trisolve_kernel<float, 8, CL>;
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_cl);
        if (CL > 8) cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = CL;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3(ncl * CL);
        cfg.blockDim = dim3(NT);
        cfg.dynamicSmemBytes = smem_cl;
        cfg.stream = st;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        if (cudaLaunchKernelEx(&cfg, kern, s, tiles, vec, nrhs, 0, nch, epoch1, 0) != cudaSuccess) return -1;
    } else {
        const size_t smem = trisolve_smem<float, 8, 1>();
        auto kern = trisolve_kernel<float, 8, 1>;
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        kern<<<grid, NT, smem, st>>>(s, tiles, vec, nrhs, 0, nch, epoch1, 0);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int trisolve_grid(bool fp64, int nrhs, int num_sms) {
    // the smallest occupancy over the chunk widths this nrhs uses
    int g = 1 << 30;
    auto take = [&](int v) { g = v < g ? v : g; };
    if (fp64) {
        if (nrhs >= 8) take(occupancy_grid<double, 8>(num_sms));
        if (nrhs % 8 >= 4) take(occupancy_grid<double, 4>(num_sms));
        if (nrhs % 4 >= 2) take(occupancy_grid<double, 2>(num_sms));
        if (nrhs % 2 == 1) take(occupancy_grid<double, 1>(num_sms));
    } else {
        if (nrhs >= 8) take(occupancy_grid<float, 8>(num_sms));
        if (nrhs % 8 >= 4) take(occupancy_grid<float, 4>(num_sms));
        if (nrhs % 4 >= 2) take(occupancy_grid<float, 2>(num_sms));
        if (nrhs % 2 == 1) take(occupancy_grid<float, 1>(num_sms));
    }
    return g;
}

void residual_launch(const DevCSR& A, const double* b, const double* x, double* r, int nrhs, double* red,
                     int n_stat, cudaStream_t s) {
    cudaMemsetAsync(red, 0, sizeof(double) * RED * nrhs, s);
    residual_kernel<<<(A.n + 255) / 256, 256, 0, s>>>(A, b, x, r, nrhs, red, n_stat);
}
void scatter_csr_launch(const double* V, const int32_t* vidx, const int32_t* pos, int64_t nnz, double* csr_val,
                        cudaStream_t s) {
    if (nnz > 0) scatter_csr_kernel<<<(unsigned)((nnz + 255) / 256), 256, 0, s>>>(V, vidx, pos, nnz, csr_val);
}
void cast_f64_to_f32_launch(const double* src, float* dst, int64_t n, cudaStream_t s) {
    if (n > 0) cast_kernel<<<608, 256, 0, s>>>(src, dst, n);
}
void axpy_f32_to_f64_launch(const float* d, double* x, int64_t n, int assign, cudaStream_t s) {
    if (n > 0) axpy_kernel<<<608, 256, 0, s>>>(d, x, n, assign);
}
void gather_seg_launch(const double* b, const DevSegs& g, int n_ext, int c0, int nc, double* out, cudaStream_t s) {
    const int64_t tot = (int64_t)n_ext * nc;
    if (tot > 0) gather_seg_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(b, g, n_ext, c0, nc, out);
}
void scatter_seg_launch(const double* xe, const DevSegs& g, int n_ext, int c0, int nc, double* x,
                        unsigned long long* cnt, cudaStream_t s) {
    const int64_t tot = (int64_t)n_ext * nc;
    if (tot > 0) scatter_seg_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(xe, g, n_ext, c0, nc, x, cnt);
}
void residual_seg_launch(const DevCSR& A, const double* b, const double* x, double* r, int c0, int nc,
                         double* red, const DevSegs& g, cudaStream_t s) {
    cudaMemsetAsync(red, 0, sizeof(double) * RED * nc * g.nseg, s);
    const int nbr = A.n / 64;  // A.n is a multiple of 64
    if (nbr > 0 && nc > 0 && nc <= 64)
        residual_seg_kernel<<<std::min(nbr, RES_CTAS), RES_THREADS, 0, s>>>(A, b, x, r, c0, nc, red, g, nbr);
}
void cast_seg_launch(const double* src, float* dst, int n_ext, int nc, const DevSegs& g, cudaStream_t s) {
    if ((int64_t)n_ext * nc > 0) cast_seg_kernel<<<608, 256, 0, s>>>(src, dst, n_ext, nc, g);
}
void gather_tiles_launch(const void* src, void* dst, const int32_t* ids, int64_t n, uint64_t tile_bytes,
                         cudaStream_t s) {
    if (n > 0)
        gather_tiles_kernel<<<1216, 256, 0, s>>>(static_cast<const int4*>(src), static_cast<int4*>(dst), ids, n,
                                                 (int)(tile_bytes / 16));
}
void csr_absmax_seg_launch(const DevCSR& A, const DevSegs& g, unsigned long long* out, cudaStream_t s) {
    if (A.n > 0) csr_absmax_seg_kernel<<<(A.n + 255) / 256, 256, 0, s>>>(A, g, out);
}
void absmax_launch(const double* v, int64_t n, unsigned long long* out, cudaStream_t s) {
    if (n > 0) absmax_kernel<<<608, 256, 0, s>>>(v, n, out);
}

// ---------------------------------------------------------------- allocation-free residual check
// The residual kernel's reduction buffer normally comes from the block pool.
// This variant keeps it in a fixed array of device memory that exists for as
// long as the library is loaded, for callers that must not allocate device
// memory themselves: code whose device memory is owned by another allocator
// (a framework's caching allocator, a fixed serving budget) and latency-
// critical loops where cudaMalloc / cudaFree would synchronise the device.
constexpr int NOALLOC_MAX_RHS = 64;  // 6 doubles per right-hand side: 3 KB
static __device__ __align__(256) double g_noalloc_red[RED * NOALLOC_MAX_RHS];

namespace {
std::mutex g_noalloc_mu;
double* g_noalloc_addr[256] = {};  // device address of g_noalloc_red, per device

// Once per device, with that device current: the device address of the
// array (in host code the array's name is only a host-side stand-in).
int noalloc_scratch(int dev, double** out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (dev < 0 || dev >= 256) return SOG_EINVAL;
    if (g_noalloc_addr[dev]) {
        // a device reset (or a released and recreated primary context) reloads
        // the module at another address: look it up again when the cached one
        // is no longer device memory of this context
        cudaPointerAttributes at{};
        if (cudaPointerGetAttributes(&at, g_noalloc_addr[dev]) != cudaSuccess || at.type != cudaMemoryTypeDevice ||
            at.device != dev) {
            cudaGetLastError();
            g_noalloc_addr[dev] = nullptr;
        }
    }
    if (!g_noalloc_addr[dev]) {
        double* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress((void**)&p, g_noalloc_red);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return sog_internal::fail(SOG_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        }
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return SOG_OK;
}
}  // namespace

}  // namespace sog

extern "C" int sog_residual_noalloc(int32_t n, const int32_t* row_ptr, const int32_t* col, const double* val,
                                    int32_t nrhs, const double* b, const double* x, double* r, double* rel_resid,
                                    double* backward_error, void* stream) {
    using namespace sog;
    if (n <= 0 || !row_ptr || !col || !val || !b || !x || !r || !rel_resid || !backward_error)
        return sog_internal::fail(SOG_EINVAL, "sog_residual_noalloc: bad argument");
    if (nrhs < 1 || nrhs > NOALLOC_MAX_RHS)
        return sog_internal::fail(SOG_EINVAL, "sog_residual_noalloc: nrhs must be 1.." +
                                                  std::to_string(NOALLOC_MAX_RHS) + " (fixed scratch size)");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return sog_internal::fail(SOG_ENODEV, "sog_residual_noalloc: no current device");
    }
    double* red = nullptr;
    int rc = noalloc_scratch(dev, &red);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    DevCSR A{n, row_ptr, col, val};
    // the array keeps the previous call's sums: clear the part this call accumulates into
    cudaError_t e = cudaMemsetAsync(red, 0, sizeof(double) * RED * nrhs, s);
    if (e == cudaSuccess) {
        residual_kernel<<<(n + 255) / 256, 256, 0, s>>>(A, b, x, r, nrhs, red, n);
        e = cudaGetLastError();  // a launch that did not start would leave the zeros: a silent perfect residual
    }
    double host[RED * NOALLOC_MAX_RHS];
    if (e == cudaSuccess) e = cudaMemcpyAsync(host, red, sizeof(double) * RED * nrhs, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return sog_internal::fail(SOG_ECUDA, std::string("sog_residual_noalloc: ") + cudaGetErrorString(e));
    }
    for (int c = 0; c < nrhs; c++) {
        const double* q = host + RED * c;
        rel_resid[c] = q[1] > 0 ? std::sqrt(q[0]) / std::sqrt(q[1]) : std::sqrt(q[0]);
        const double den = q[5] * q[3] + q[4];
        backward_error[c] = den > 0 ? q[2] / den : q[2];
    }
    return SOG_OK;
}
