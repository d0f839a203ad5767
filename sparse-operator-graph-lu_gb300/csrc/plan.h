// Host planner: MatrixMarket reading, GPS reordering and the recursive block-LU
// decomposition into a level-scheduled DAG of 64x64 unit operations.
//
// This is the host side that the reference keeps on the CPU (mtx.cpp,
// GPSOrder.cpp, BlockPlanner.cpp:103-374 and :865-1577, config.cpp). It is
// rewritten here so that, on the same input, it emits the same DAG as the
// reference op for op (same op kinds, same block ids, same stages): the
// executor behind the C-ABI is then a drop-in for BlockPlanner::calculate and
// BlockPlanner::solve on exactly the reference's workload.
#pragma once
#include <cstdint>
#include <memory>
#include <new>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

namespace sog {

// Op kinds, numbered as the reference's enum blockOp (operation.h:20).
enum OpKind : int32_t {
    OP_INV = 0, OP_LU = 1, OP_LOWERINV = 2, OP_UPPERINV = 3, OP_SUB = 4, OP_ADD = 5,
    OP_NEG = 6, OP_COPY = 7, OP_MUL = 8, OP_MULNEG = 9, OP_LLT = 10, OP_MULT = 11, OP_NOOP = 12
};

// One unit operation, the fields of the reference's struct operation
// (operation.h:37-48). Block id 0 means "none".
//   lu:        (res, res2) = (L, U) of block src
//   lowerInv:  res = inverse of lower-triangular block src
//   upperInv:  res = inverse of upper-triangular block src
//   sub:       res = src2 - src; src == 0: res = src2 (copy); src2 == 0: res = -src (neg)
//   mul:       res += src * src2;   mulneg: res -= src * src2   (res starts at zero)
//   llt:       res = L with L L^T = src (lower triangle of src read)
//   mult:      res += src * src2^T  (res starts at zero)
struct Op {
    int32_t op, src, src2, res, res2, stage;
    int32_t seq, group;
};

// Allocator that leaves default-constructed elements uninitialised, so that
// sizing an op list of several hundred MB does not zero it first (the
// planner fills it from several threads, which also spreads the page faults).
template <class T>
struct NoInitAlloc : std::allocator<T> {
    template <class U>
    struct rebind { using other = NoInitAlloc<U>; };
    NoInitAlloc() = default;
    template <class U>
    NoInitAlloc(const NoInitAlloc<U>&) noexcept {}
    template <class U>
    void construct(U* p) noexcept(std::is_nothrow_default_constructible<U>::value) { ::new ((void*)p) U; }
    template <class U, class... A>
    void construct(U* p, A&&... a) { ::new ((void*)p) U(std::forward<A>(a)...); }
};
using OpVec = std::vector<Op, NoInitAlloc<Op>>;

struct Config {
    int n = 0;             // matrix dimension
    int block_rows = 0;    // fine 64-row block rows (power of two, config.cpp:30-49)
    int block_rows_l2 = 0; // coarse block rows
    int block_size_l2 = 0; // coarse block size in rows
    int n_ext() const { return block_rows * 64; }
};
Config make_config(int n);

// Row/column permutation: new_to_old[i_new] = i_old; old_to_new[i_old] = i_new.
struct Ordering {
    std::vector<int32_t> new_to_old, old_to_new;
};

// GPS-style bandwidth reordering (GPSOrder.cpp:494-650) followed by the
// in-block diagonal sort (GPSOrder.cpp:55-150). I/J are 0-based triplet
// indices of an n x n matrix; V the values (only diagonal values are read).
Ordering gps_order(int n, const std::vector<int32_t>& I, const std::vector<int32_t>& J,
                   const std::vector<double>& V, int threads = 0);

struct Leaf {
    int32_t bi, bj, id;
};

// One system of a batch plan (merge_plans): its rows occupy permuted rows
// [row0, row0 + 64*R) of the block-diagonal union, of which the first n are
// real (the rest are its unit-diagonal padding); its original rows are
// [noff, noff + n) of the concatenated original ordering, and its triplets
// [trip_off, trip_off + ntrip) of the concatenated triplet values.
struct Segment {
    int32_t row0 = 0, n = 0, R = 0;
    int64_t noff = 0, trip_off = 0, ntrip = 0;
    bool symmetric = false;  // an LL^T system (its L leaves only)
};

// Everything the executor needs, in the reference's terms.
struct Plan {
    Config cfg;
    Ordering ord;
    OpVec ops;                   // fine ops, sorted by stage as the reference executes them
    int32_t storage_count = 0;   // block ids are 1..storage_count-1
    int32_t n_input = 0;         // input tiles carry ids 1..n_input
    std::vector<int32_t> input_bi, input_bj;  // block coordinates of input tiles (index id-1)
    std::vector<Leaf> L, U;      // leaves of the L and U block quadtrees (U empty for LL^T)
    bool symmetric = false;      // LL^T plan: ops llt / mult, A = L L^T
    int32_t stages = 0;
    // Value scatter for (re)factorisation with the same pattern: triplet k goes
    // to input tile scatter_tile[k] (0-based, -1 = superseded duplicate) at
    // element scatter_off[k] (row*64+col). Padded rows carry a unit diagonal.
    std::vector<int32_t> scatter_tile;
    std::vector<int16_t> scatter_off;
    // Symmetric input: the scatter runs over the mirrored triplets; value
    // source of each (index into the caller's triplets), else empty. Callers
    // always pass values in their own triplet order (nval of them).
    std::vector<int32_t> mirror_src;
    int64_t nval = 0;
    std::vector<int32_t> pad_tile;  // tile index of each padded row's diagonal
    std::vector<int16_t> pad_off;
    // Batch plans only: the merged systems in order. Then ord.new_to_old has
    // one entry per permuted row (n_ext): the row's index within its own
    // system's original ordering, -1 for padding; ord.old_to_new is empty.
    std::vector<Segment> segs;
    // statistics
    int64_t coarse_ops_emitted = 0, coarse_ops = 0, fine_ops_emitted = 0;
    double t_order = 0, t_plan = 0;
};

// Full host planning: symmetric mirroring (solver.cpp:132-149), ordering,
// two-level planning (solver.cpp:56-110). Throws std::runtime_error on bad input.
Plan build_plan(int n, int64_t nnz, bool symmetric, const int32_t* I, const int32_t* J, const double* V,
                int threads = 0);

// Block-diagonal union of independent systems' plans (a batch): one DAG whose
// ops from different systems never share a block, so one executor launch
// factors all of them. Block ids are renumbered with every system's input
// tiles first (ids 1..sum n_input, in system order), then every system's
// other blocks; block rows are stacked in system order. Throws on plans that
// cannot be merged (imported plans, batch plans, size overflow).
Plan merge_plans(const std::vector<const Plan*>& ps);

// Dense input tiles (n_input x 64 x 64, row-major) for values V of the
// triplets given to build_plan (mirrored here when symmetric).
void scatter_tiles(const Plan& p, const double* V, double* tiles);

// Triplets after mirroring (what build_plan and scatter_tiles index).
void mirror_triplets(int n, int64_t nnz, bool symmetric, const int32_t* I, const int32_t* J, const double* V,
                     std::vector<int32_t>& Io, std::vector<int32_t>& Jo, std::vector<double>& Vo);

// MatrixMarket reader with the reference's acceptance rules (mtx.cpp:44-117):
// header "symmetric" => lower triangle given; lines of <= 3 chars and lines
// containing '%' are skipped; zero values are dropped; indices are 1-based.
struct MtxData {
    int n = 0;
    bool symmetric = false;
    std::vector<int32_t> I, J;
    std::vector<double> V;
};
bool read_mtx(const std::string& path, MtxData& out, std::string& err);
// read_mtx through a binary cache <path>.sogbin (written after a text parse,
// used while the text file's size and modification time are unchanged)
bool read_mtx_cached(const std::string& path, MtxData& out, std::string& err, bool* from_cache = nullptr);
// Array reader (mtx.cpp:145-181): missing entries are 1.
std::vector<double> read_rhs(const std::string& path, int n);

}  // namespace sog
