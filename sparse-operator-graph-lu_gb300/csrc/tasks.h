// Device task graph built from the reference-format op DAG.
//
// The reference executes its DAG stage by stage with a barrier per stage and
// serialises all writers of one block in one thread (BlockPlanner.cpp:397-592).
// Here every block is produced by exactly one task:
//   GEMM : C = init + sum_k (+/-) A_k * B_k over all mul/mulneg ops writing C
//   LU   : (L, U) = lu(A)            LINV : Y = L^-1      UINV : Y = U^-1
//   SUB  : R = A2 - A1 (either side may be absent: copy / negate)
// and a task depends only on the tasks producing the blocks it reads, so a
// persistent kernel can run any ready task without stage barriers.
//
// A Schur-complement update S = D - (sum of products) arrives from the planner
// as a product into a temporary block followed by a sub (BlockPlanner.cpp:
// 921-923); when the temporary has no other reader the two are fused into one
// GEMM task with initial tile D and negated products.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "plan.h"

namespace sog {

// K_GEMM_LU / K_GEMM_LLT: a product followed, in the same task, by the LU
// (LL^T) of its result (the diagonal block is read by nothing else)
enum TaskKind : uint8_t {
    K_GEMM = 0, K_LU = 1, K_LINV = 2, K_UINV = 3, K_SUB = 4, K_LLT = 5, K_TRANS = 6, K_GEMM_LU = 7, K_GEMM_LLT = 8
};
constexpr int NUM_KINDS = 9;
// GEMM operand pairs: pair_b = +-(id | PAIR_TRANS): a negative entry subtracts
// the product, PAIR_TRANS multiplies by the transpose of block id (mult ops)
constexpr int32_t PAIR_TRANS = 1 << 30;
// Internal op kind (not in the reference's enum): res = src^T; used to give an
// LL^T plan the upper factor L^T for the back substitution
constexpr int32_t OP_TRANSPOSE = 100;

struct TaskGraph {
    int32_t ntasks = 0;
    int32_t storage_count = 0;
    std::vector<uint8_t> kind, parts;
    std::vector<int32_t> out, out2, a, b, c, out3;  // block ids (see kernels.h DevTasks)
    std::vector<int32_t> pair_ptr;             // ntasks+1; GEMM operand pairs
    std::vector<int32_t> pair_a, pair_b;       // pair_b < 0: subtract A*B(|pair_b|)
    std::vector<int32_t> succ_ptr, succ;       // successor tasks
    std::vector<int32_t> ndep;                 // predecessor task count
    std::vector<int32_t> level;                // dependency level, 0-based
    std::vector<int32_t> prio;                 // longest path (tasks) to a sink
    std::vector<int32_t> level_ptr;            // nlevels+1 offsets into level_items
    std::vector<int32_t> level_items;          // (task << 2 | part), grouped by level
    std::vector<int32_t> ready_items;          // initially ready items, longest path first
    int32_t nlevels = 0;
    int64_t total_items = 0;                   // sum of parts
    int64_t gemm_pairs = 0;
    int64_t fused_subs = 0;
    int64_t fused_inverses = 0;  // lowerInv / upperInv tasks folded into their LU task
    int64_t aliased_copies = 0;  // copy ops (sub with src = 0) replaced by aliasing
    int64_t aliased_inverses = 0;  // repeated lowerInv / upperInv of one block replaced by aliasing
    int64_t count[NUM_KINDS] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    int64_t fused_lu = 0;  // LU / LL^T tasks merged into the product producing their block
    // block -> block whose tile holds its value: identity except the result of
    // a copy, which reads its source's tile (every block is written once, so
    // a copy's source never changes after the copy would have run)
    std::vector<int32_t> alias;
    // block -> task producing it (-1: an input block or none)
    std::vector<int32_t> producer;
};

// The op list a task graph is built from: a plan's ops (not copied) followed
// by the ops appended for the substitution and the LL^T path (diagonal
// inverses, look-ahead products, transposed leaves).
struct OpSeq {
    const Op* base = nullptr;
    int64_t nbase = 0;
    std::vector<Op> extra;
    OpSeq() = default;
    OpSeq(const Op* b, int64_t n) : base(b), nbase(n) {}
    int64_t size() const { return nbase + (int64_t)extra.size(); }
    const Op& operator[](int64_t i) const { return i < nbase ? base[i] : extra[i - nbase]; }
    // sequence number and stage of the last op (0, 0 when empty)
    int32_t last_seq() const { return size() == 0 ? 0 : (*this)[size() - 1].seq; }
    int32_t last_stage() const { return size() == 0 ? 0 : (*this)[size() - 1].stage; }
};

// outputs: block ids that must be materialised (the L/U leaves; a copied
// output is materialised in its source's tile, see TaskGraph::alias). Throws
// std::runtime_error on a block written by ops of different kinds, a read of a
// block nobody produces (and not an input), an id out of range, or a cycle.
// gemm_parts: parts per GEMM task (1 or 4).
// fuse_lu: merge an LU / LL^T task into the single-part product producing its
// input block when nothing else reads that block (the mixed path).
TaskGraph build_tasks(const OpSeq& ops, int32_t storage_count, int32_t n_input,
                      const std::vector<int32_t>& outputs, int gemm_parts, bool fuse_subs = true,
                      bool fuse_lu = false);

// Appends, for every diagonal L (U) block without one already in the DAG, a
// lowerInv (upperInv) op; returns per block row the id of the inverse of the
// diagonal L and U blocks. storage_count grows by the number of new blocks.
void add_diag_inverses(OpSeq& ops, int32_t& storage_count, int block_rows, const std::vector<Leaf>& L,
                       const std::vector<Leaf>& U, std::vector<int32_t>& linv, std::vector<int32_t>& uinv);
// LL^T plans have no U leaves: U = L^T is materialised by one transpose op
// per L leaf (new blocks), so the back substitution runs as for LU.
void add_transposed_leaves(OpSeq& ops, int32_t& storage_count, const std::vector<Leaf>& L,
                           std::vector<Leaf>& U);

// Claim order of the ordered executor: items by estimated start time (longest
// weighted path from a source, single-CTA task latencies as weights), ties by
// longest remaining path. Every task comes after its predecessors.
std::vector<int32_t> static_order(const TaskGraph& g, bool fp64);
// Reorders every product's operand pairs by the estimated finish of their
// producers (stable), so a task that starts before its last producer ends
// accumulates the ready pairs first and the late one last.
void order_pairs_by_ready(TaskGraph& g, bool fp64);

// Look-ahead products for the substitution at distance dist: for every block
// row i with an L block at (i, i-dist), lla[i] = id of a new block Linv_ii *
// L_{i,i-dist}; for every U block at (i, i+dist), ula[i] = id of Uinv_ii *
// U_{i,i+dist} (0 = none). With distances 1..d the substitution forms y_i =
// Linv_ii (b_i - sum_{j<i-d} L_ij y_j) - sum_k lla_k[i] y_{i-k}: each of the
// d nearest rows costs one 64x64 product once it is published, and the rest
// is done before.
void add_lookahead_products(OpSeq& ops, int32_t& storage_count, int block_rows, const std::vector<Leaf>& L,
                            const std::vector<Leaf>& U, const std::vector<int32_t>& linv,
                            const std::vector<int32_t>& uinv, int dist, std::vector<int32_t>& lla,
                            std::vector<int32_t>& ula);
// The forward substitution overlapping the factorisation: per block row i
// the tasks producing the tiles it reads (its off-diagonal L leaves
// lid[lptr[i] .. lptr[i+1]), its diagonal inverse linv[i] and its look-ahead
// products la[d][i]), sorted and unique, as list[ptr[i] .. ptr[i+1]). Block
// ids are the graph's (aliased) ids; tiles no task writes (input blocks) need
// no wait.
void forward_wait_lists(const TaskGraph& g, int block_rows, const std::vector<int32_t>& lptr,
                        const std::vector<int32_t>& lid, const std::vector<int32_t>& linv,
                        const std::vector<const std::vector<int32_t>*>& la, std::vector<int32_t>& ptr,
                        std::vector<int32_t>& list);

}  // namespace sog
