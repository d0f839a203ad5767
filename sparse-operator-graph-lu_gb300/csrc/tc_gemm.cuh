// Split-precision TF32 64x64 tile product on the 5th-generation tensor cores
// (tcgen05, sm_100a family incl. sm_103a), accumulator in tensor memory.
//
//   C = init + sum_p s_p A_p B_p      (A_p, B_p, C: 64x64 FP32, row-major in HBM)
//
// Operand tiles reach shared memory by TMA bulk copies into a ring of raw
// slots (mbarrier completion). Each operand is then split into a TF32 head
// (rounded to nearest) and the FP32 remainder, staged in the canonical
// no-swizzle K-major layout (core matrices of 8 rows x 16 bytes): A as a
// 128-row operand with the head of row r in row 2r and its remainder in row
// 2r + 1, B transposed as the 128-row operand [B_hi^T; B_lo^T]. One M=128,
// N=128 MMA per K=8 step then accumulates all four split products; output row
// r's head and remainder parts sit in TMEM lanes 2r and 2r + 1 (one warp), its
// x B_hi and x B_lo parts in columns c and 64 + c, and the epilogue adds them
// (hi*hi + hi*lo + lo*hi + the negligible lo*lo). The tensor core reads the
// TF32 part of each FP32 word, so the remainder enters truncated to TF32
// (relative error 2^-22 of the element). Two shared-memory stages alternate:
// pair p+1 is staged while pair p's MMAs run. One thread issues the MMAs and
// commits them to the stage's mbarrier; every wait is bounded.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace sog {
namespace tc {

constexpr int ROW_GROUP_BYTES = 8 * 64 * 4;                 // 8 rows x K=64 fp32 = 2048
constexpr int A_BYTES = 128 / 8 * ROW_GROUP_BYTES;         // heads and remainders of A = 32768
constexpr int B_BYTES = 64 / 8 * ROW_GROUP_BYTES;          // 16384 per part
constexpr int STAGE_BYTES = A_BYTES + 2 * B_BYTES;         // 65536
// operand stages per CTA: 2 (the next pair stages while this one's MMAs run,
// 128 KB, one CTA per SM) or 1 (64 KB, two CTAs per SM)
constexpr int MAX_STAGES = 2;
// raw FP32 operand pairs in flight (A and B tiles as copied from global by
// the tensor-memory-access unit), ahead of the conversion into a stage: 3
// with two stages (128 + 96 KB), 1 with one stage (64 + 32 KB)
constexpr int RAW_BYTES = 2 * 64 * 64 * 4;
constexpr int MAX_RAW = 3;
template <int S>
__host__ __device__ constexpr int raw_slots() { return S == 2 ? 3 : 1; }
constexpr uint32_t TMEM_COLS = 128;  // D: 128 lanes x 128 FP32 columns

// byte offset of element (row, k) in the K-major core-matrix layout:
// 8-row groups at ROW_GROUP_BYTES, K-adjacent core matrices at 128 bytes
__device__ __forceinline__ uint32_t kmajor_off(int row, int k) {
    return (uint32_t)((row >> 3) * ROW_GROUP_BYTES + (k >> 2) * 128 + (row & 7) * 16 + (k & 3) * 4);
}

// 64-bit shared-memory matrix descriptor, no swizzle: start address, leading
// byte offset (K-adjacent core matrices) and stride byte offset (8-row groups)
// in 16-byte units, version 1 at bit 46, swizzle mode 0 at bits 61-63
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// instruction descriptor for kind::tf32: D f32, A/B tf32, K-major A and B,
// N = 128 (bits 17-22 hold N >> 3), M = 128 (bits 24-28 hold M >> 4)
__host__ __device__ constexpr uint32_t idesc_tf32_m128_n128() {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((128u >> 3) << 17) | ((128u >> 4) << 24);
}

// TF32 head of x, rounded to nearest (ties away from zero) on the magnitude
__device__ __forceinline__ float tf32_head(float x) {
    return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// bounded wait for the mbarrier phase `parity` to complete; false on timeout
// (the clock is read only once the first probe found the phase open)
__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0;
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, unsigned long long limit_ns) {
    if (mbar_try(bar, parity)) return true;
    unsigned long long t0;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    for (;;) {
        if (mbar_try(bar, parity)) return true;
        unsigned long long t;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        if (t - t0 > limit_ns) return false;
    }
}

// TMEM allocation by one full warp; the address lands in *slot (shared)
__device__ __forceinline__ void tmem_alloc(uint32_t* slot) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(TMEM_COLS) : "memory");
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 32 consecutive fp32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
        "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// Per-CTA state of the tensor-core product (static shared memory). phase
// holds, per stage s, the parity of that stage's next mbarrier phase (bit s);
// pending, per stage, whether a commit on it is not yet waited for.
struct State {
    uint64_t bar[MAX_STAGES];   // MMAs of a stage completed (the stage is free again)
    uint64_t full[MAX_STAGES];  // every warp staged its share of a stage
    uint64_t raw[MAX_RAW];      // copies into a raw slot landed
    uint32_t tmem;
    int32_t fail;
};

// ---- copies by the tensor-memory-access unit (TMA) into shared memory
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
// contiguous copy (16-byte aligned addresses, size a multiple of 16)
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
// orders this thread's earlier (acquired) generic view of global memory
// before its later copies by the async proxy
__device__ __forceinline__ void fence_proxy_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }

// Thread -> chunk mapping: warp w owns the 8-row group 8w..8w+7; in chunk j,
// lane l handles row 8w + (l & 7) and K-quad 4j + (l >> 3). Eight consecutive
// lanes then touch one 128-byte core matrix (conflict-free 16-byte accesses).
__device__ __forceinline__ void chunk_of(int j, int& row, int& k) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    row = 8 * warp + (lane & 7);
    k = 4 * (4 * j + (lane >> 3));
}

__device__ __forceinline__ void split4(const float4& x, float sgn, float4& hi, float4& lo) {
    hi.x = tf32_head(sgn * x.x); lo.x = sgn * x.x - hi.x;
    hi.y = tf32_head(sgn * x.y); lo.y = sgn * x.y - hi.y;
    hi.z = tf32_head(sgn * x.z); lo.z = sgn * x.z - hi.z;
    hi.w = tf32_head(sgn * x.w); lo.w = sgn * x.w - hi.w;
}

// Stage one pair from a raw slot holding the row-major A and B tiles (two
// 1-D copies): A (x sgn) becomes heads and remainders in interleaved rows of
// the K-major core-matrix layout (stage_a_interleaved); B becomes B_hi^T,
// B_lo^T, either from the tile's rows (trans: they
// are the K-major rows of the MMA's B operand) or transposed here. Every
// shared-memory access is conflict-free. Row-major to core-matrix chunks use
// a diagonal assignment: in each group of 8 lanes, lane e takes row 8w + e
// and k-quad (e + c) mod 16, so the 8 lanes read 8 distinct bank quads of
// the raw rows and write 8 distinct rows of one core matrix.
__device__ __forceinline__ void stage_kmajor(unsigned char* hi_dst, unsigned char* lo_dst, const float* src,
                                             float sgn) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, e = lane & 7, ph = lane >> 3;
    const int row = 8 * warp + e;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int k = 4 * ((e + 4 * ph + j) & 15);
        float4 hi, lo;
        split4(*reinterpret_cast<const float4*>(src + row * 64 + k), sgn, hi, lo);
        *reinterpret_cast<float4*>(hi_dst + kmajor_off(row, k)) = hi;
        *reinterpret_cast<float4*>(lo_dst + kmajor_off(row, k)) = lo;
    }
}
// A (x sgn) with the head of row r in operand row 2r and the remainder in
// 2r + 1, so that one output row's two partial products land in adjacent
// TMEM lanes of one warp. In each group of 8 lanes, rows 8w..8w+3 store heads
// while rows 8w+4..8w+7 store remainders and then the other way round: every
// store instruction hits 8 distinct core-matrix rows (conflict-free).
__device__ __forceinline__ void stage_a_interleaved(unsigned char* dst, const float* src, float sgn) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, e = lane & 7, ph = lane >> 3;
    const int row = 8 * warp + e;
    const bool head_first = e < 4;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int k = 4 * ((e + 4 * ph + j) & 15);
        float4 hi, lo;
        split4(*reinterpret_cast<const float4*>(src + row * 64 + k), sgn, hi, lo);
        *reinterpret_cast<float4*>(dst + kmajor_off(2 * row + (head_first ? 0 : 1), k)) = head_first ? hi : lo;
        *reinterpret_cast<float4*>(dst + kmajor_off(2 * row + (head_first ? 1 : 0), k)) = head_first ? lo : hi;
    }
}
__device__ __forceinline__ void stage_from_raw(unsigned char* st, const unsigned char* raw, bool trans, float sgn) {
    const float* A = reinterpret_cast<const float*>(raw);
    const float* B = reinterpret_cast<const float*>(raw + RAW_BYTES / 2);
    stage_a_interleaved(st, A, sgn);
    if (trans) {
        stage_kmajor(st + A_BYTES, st + A_BYTES + B_BYTES, B, 1.f);
    } else {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        const int n = 32 * (warp & 1) + lane;
        float4 hi, lo;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int k = 4 * (4 * (warp >> 1) + j);
            const float4 x = make_float4(B[(k + 0) * 64 + n], B[(k + 1) * 64 + n], B[(k + 2) * 64 + n],
                                         B[(k + 3) * 64 + n]);
            split4(x, 1.f, hi, lo);
            *reinterpret_cast<float4*>(st + A_BYTES + kmajor_off(n, k)) = hi;
            *reinterpret_cast<float4*>(st + A_BYTES + B_BYTES + kmajor_off(n, k)) = lo;
        }
    }
}

// Issue the 8 MMAs of one staged pair (K = 64 in steps of 8): one M = 128,
// N = 128 product per step of the interleaved A heads/remainders against
// [B_hi^T; B_lo^T] (the B halves are adjacent 8-row groups of one K-major
// operand), so D holds all four split products: lanes 2r / 2r + 1 = head /
// remainder of row r, columns c / 64 + c = x B_hi / x B_lo.
__device__ __forceinline__ void issue_pair(const unsigned char* st, uint32_t tmem, bool first) {
    const uint32_t base = smem_u32(st);
    constexpr uint32_t idesc = idesc_tf32_m128_n128();
#pragma unroll
    for (int ks = 0; ks < 8; ks++) {
        const uint32_t koff = ks * 256;  // K = 8 tf32 = two core matrices of 128 bytes
        const uint64_t a = smem_desc(base + koff, 128, ROW_GROUP_BYTES);
        const uint64_t b = smem_desc(base + A_BYTES + koff, 128, ROW_GROUP_BYTES);
        mma_tf32(tmem, a, b, idesc, (first && ks == 0) ? 0u : 1u);
    }
}

}  // namespace tc
}  // namespace sog
