// Launch interface between the host runtime (runtime.cpp) and the sm_103a
// kernels (factor*.cu, solve.cu). Plain structs of device pointers.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace sog {

// status word bits (DevStatus::flags)
enum : int32_t {
    ST_TIMEOUT = 1,      // a bounded wait expired
    ST_BAD_ITEM = 2,     // queue delivered an out-of-range item
    ST_SOLVE_TIMEOUT = 4,
};

struct DevStatus {
    int32_t flags;
    int32_t timeout_where;                 // debugging aid: item index at timeout
};

// Pivot statistics of one system's diagonal-block factorisations (one entry
// per system of a batch). Non-negative doubles order as their bit patterns,
// so integer atomics keep the minimum / maximum.
struct DevPivot {
    unsigned long long min_pivot_bits;  // min |u_ii| before the clamp
    unsigned long long max_mag_bits;    // max over diagonal blocks of max(|block entering the LU|, |U|) (LL^T: |L|^2)
    int32_t clamped;                    // pivots raised to the clamp value
    int32_t inv_fail;                   // blocks whose U U^-1 diagonal is off 1 by more than 1e-3 or not finite
};

struct DevTasks {
    int32_t ntasks;
    int64_t total_items;
    const uint8_t* kind;
    const uint8_t* parts;
    // out/out2: result blocks; a: source (LU/inverses), minuend (SUB) or initial
    // tile of a product (GEMM, 0 = zero); b: subtrahend (SUB) or L^-1 of an
    // LU / LL^T task (0 = none); c: U^-1 of an LU task (0 = none). A product
    // with its LU (K_GEMM_LU / K_GEMM_LLT): out = the product, which the LU
    // factors; out3 = L, out2 = U, b = L^-1, c = U^-1.
    const int32_t *out, *out2, *a, *b, *c, *out3;
    const int32_t* prio;  // longest path to a sink, for choosing which ready successor to keep
    const int32_t *pair_ptr, *pair_a, *pair_b;
    const int32_t *succ_ptr, *succ;
    int32_t* dep;         // working dependency counters
    int32_t* parts_left;  // working per-task part counters
    int32_t* queue;       // ready items (task << 2 | part); -1 = not yet filled
    int32_t* head;        // next slot to claim
    int32_t* tail;        // next slot to fill
    int32_t* done;        // completed items
    // static claim order of items (the ordered executor): estimated start
    // time, then longest remaining path; ITEM_EARLY marks a product that may
    // start before its last producer finished
    const int32_t* order;
    // early start (mixed path, ordered executor): producer task of each
    // pair's A and B tile and of each product's initial tile (-1: none), and
    // per-task completion flags (set after the task's writes are released)
    int32_t early;
    const int32_t *pair_wa, *pair_wb, *init_w;
    int32_t* task_done;
    // FP64 products skip MMAs of all-zero operand fragments (in-tile sparsity)
    int32_t skip_zero;
    DevStatus* status;
    // pivot statistics per system; task_seg = system of each task (NULL: one system)
    DevPivot* piv;
    const int32_t* task_seg;
    unsigned long long wait_limit_ns;  // bound on any single queue wait
    // optional per-task trace (4 x u64 per task: ready, start, end, sm id), NULL = off
    unsigned long long* trace;
};

// item = task << 4 | part (parts < 8) | ITEM_EARLY
constexpr int32_t ITEM_EARLY = 8;

// ---- factor (factor.cu dispatching to factor_f64.cu / factor_f32_s1.cu / factor_f32_s2.cu) ----
// tiles: block id -> tiles + id*4096 elements. double => SOG_FP64, float => SOG_MIXED.
// stages: tensor-core operand stages of the mixed path (1 or 2; ignored for FP64).
int factor_queue_launch(const DevTasks& t, double* tiles, int grid, int stages, cudaStream_t s);
int factor_queue_launch(const DevTasks& t, float* tiles, int grid, int stages, cudaStream_t s);
// ordered executor: one persistent launch claiming items in the static order
int factor_ordered_launch(const DevTasks& t, double* tiles, int grid, int stages, cudaStream_t s);
int factor_ordered_launch(const DevTasks& t, float* tiles, int grid, int stages, cudaStream_t s);
int factor_level_launch(const DevTasks& t, double* tiles, const int32_t* items, int nitems, int stages,
                        cudaStream_t s);
int factor_level_launch(const DevTasks& t, float* tiles, const int32_t* items, int nitems, int stages,
                        cudaStream_t s);
// persistent grid size (CTAs co-resident on the device)
int factor_persistent_grid(bool fp64, int stages, int num_sms);

// value scatter into input tiles: tiles[tile[k]*4096 + off[k]] = V[vidx ? vidx[k] : k] (tile < 0: skip)
void scatter_values_launch(const double* V, const int32_t* vidx, const int32_t* tile, const int16_t* off, int64_t nnz,
                           const int32_t* pad_tile, const int16_t* pad_off, int64_t npad, double* tiles64,
                           float* tiles32, cudaStream_t s);
// dst tile k+1 = src tile ids[k] (k < n), tiles of tile_bytes bytes
void gather_tiles_launch(const void* src, void* dst, const int32_t* ids, int64_t n, uint64_t tile_bytes,
                         cudaStream_t s);
// FP64 input tiles -> FP32 input tiles (first n elements)
void convert_tiles_launch(const double* src, float* dst, int64_t n, cudaStream_t s);
void widen_tiles_launch(const float* src, double* dst, int64_t n, cudaStream_t s);

// ---- solve (solve.cu) ----
// Look-ahead distances of the substitution: the blocks of the SOLVE_LOOKAHEAD
// neighbouring rows are applied as products with the diagonal inverse
// folded in, each as soon as its row is published
constexpr int SOLVE_LOOKAHEAD = 3;
struct DevSolve {
    int32_t block_rows;
    // block-row CSR of off-diagonal L (j < i) and U (j > i) leaves; L sorted by
    // ascending j, U by descending j (the order their operands become ready)
    const int32_t *l_ptr, *l_col, *l_id;
    const int32_t *u_ptr, *u_col, *u_id;
    const int32_t *l_diag, *u_diag;  // diagonal block id per block row
    const int32_t *l_dinv, *u_dinv;  // block id of the inverse of each diagonal block
    int32_t* flags;                  // readiness epoch per (column chunk, block row): R x TRISOLVE_MAX_CHUNKS
    DevStatus* status;
    unsigned long long wait_limit_ns;
    // optional trace (4 x u64 per block row: lower start/end, upper start/end), NULL = off
    unsigned long long* trace;
    // optional dealing order of block rows to CTAs (position -> block row) for
    // the lower / upper solve; NULL = ascending / descending rows. Every row's
    // dependencies must come at earlier positions. Batches interleave their
    // systems so that consecutive positions are independent rows.
    const int32_t *order_l, *order_u;
    // optional look-ahead products per block row: l_la[d-1][i] = block id of
    // Dinv_i L_{i,i-d}, u_la[d-1][i] of Dinv_i U_{i,i+d} (d = 1 ..
    // SOLVE_LOOKAHEAD; 0 = none); NULL = none at that distance
    const int32_t* l_la[SOLVE_LOOKAHEAD];
    const int32_t* u_la[SOLVE_LOOKAHEAD];
    // position claim counters of the lower and upper launch (zeroed before
    // each launch pair): CTAs claim positions in dealing order as they become
    // resident, so a launch needs no co-residency of all its CTAs (systems on
    // other streams may hold part of the GPU)
    int32_t* claim;
    // forward substitution overlapped with the factorisation (NULL = off):
    // per block row the factor tasks producing the tiles it reads
    // (fwait[fwait_ptr[i] .. fwait_ptr[i+1]]), and the factor's per-task
    // completion flags; the row starts once all of them are set
    const int32_t *fwait_ptr, *fwait;
    const int32_t* task_done;
};
// Column chunks of 8 right-hand sides solved together in one launch pair
constexpr int TRISOLVE_MAX_CHUNKS = 8;
// In-place block substitution on vec (n_ext x nrhs, row-major), lower then
// upper: full 8-column chunks together in one launch per triangle (their rows
// interleaved), the remaining columns in chunks of 4, 2, 1. epoch: readiness
// tag, advanced by 2 per launch pair (lower publishes epoch, upper epoch+1);
// launches counts kernels.
int trisolve_launch(const DevSolve& s, const double* tiles, double* vec, int nrhs, int& epoch, int grid,
                    cudaStream_t st, int& launches);
int trisolve_launch(const DevSolve& s, const float* tiles, float* vec, int nrhs, int& epoch, int grid,
                    cudaStream_t st, int& launches);
int trisolve_grid(bool fp64, int nrhs, int num_sms);
// The lower (forward) pass alone, for nrhs = 1 or a multiple of 8 up to 64,
// on grid CTAs, with s.fwait_ptr set: each block row waits for the factor
// tasks that produce its tiles, so it runs while the factor kernel is still
// running on other SMs. Uses epoch; the upper pass of the same solve uses
// epoch + 1 (trisolve_upper_launch).
int trisolve_lower_overlap_launch(const DevSolve& s, const float* tiles, float* vec, int nrhs, int epoch, int grid,
                                  cudaStream_t st);
// After the factor kernel has finished: the same lower pass on grid more
// CTAs, without the factor waits, sharing the overlapped launch's claim
// counter and flags, so it takes over every position not yet claimed.
int trisolve_lower_join_launch(const DevSolve& s, const float* tiles, float* vec, int nrhs, int epoch, int grid,
                               cudaStream_t st);
// The upper (backward) pass alone, for the same nrhs as the lower pass
// before it, with epoch + 1 of that pass.
int trisolve_upper_launch(const DevSolve& s, const float* tiles, float* vec, int nrhs, int epoch1, int grid,
                          cudaStream_t st);

// CSR of the permuted, padded matrix for FP64 residuals
struct DevCSR {
    int32_t n;
    const int32_t *ptr, *col;
    const double* val;
};
// r = b - A x (all n x nrhs row-major). Per-rhs reductions over rows < n_stat:
// red[c*6 + {0..5}] = {sum r^2, sum b^2, max|r|, max|x|, max|b|, max row abs sum of A}
constexpr int RED = 6;
void residual_launch(const DevCSR& A, const double* b, const double* x, double* r, int nrhs, double* red,
                     int n_stat, cudaStream_t s);
// csr_val[pos[k]] = V[vidx ? vidx[k] : k] for pos[k] >= 0
void scatter_csr_launch(const double* V, const int32_t* vidx, const int32_t* pos, int64_t nnz, double* csr_val,
                        cudaStream_t s);
void cast_f64_to_f32_launch(const double* src, float* dst, int64_t n, cudaStream_t s);
void axpy_f32_to_f64_launch(const float* d, double* x, int64_t n, int assign, cudaStream_t s);
// The systems of a solve. Permuted row i belongs to system of_brow[i >> 6]
// and is row n2o[i] of that system's original ordering (-1 = padding). The
// caller's b / x hold, per system k, nrhs[k] x n[k] values (rhs-major) at
// offset voff[k]. A plain system is one such system with voff = 0.
struct DevSegs {
    int32_t nseg;
    const int32_t* of_brow;  // per block row
    const int32_t* n2o;      // per permuted row
    const int32_t* n;        // per system
    const int32_t* nrhs;     // per system, this solve
    const int64_t* voff;     // per system, this solve
    const int32_t* active;   // per system: 1 = takes the next refinement correction
};
// caller layout -> permuted padded row-major (n_ext x nc) for columns
// [c0, c0+nc): padding rows get 1 (the reference's b for padded rows,
// solver.cpp:159-161), columns past a system's nrhs get 0
void gather_seg_launch(const double* b, const DevSegs& g, int n_ext, int c0, int nc, double* out, cudaStream_t s);
// the inverse for real rows and columns; per-system non-finite counts into cnt[k]
void scatter_seg_launch(const double* xe, const DevSegs& g, int n_ext, int c0, int nc, double* x,
                        unsigned long long* cnt, cudaStream_t s);
// r = b - A x (n_ext x nc, 1 <= nc <= 64: the solve's column chunk);
// reductions per (system, column) over the system's real rows and columns:
// red[(k*nc + c)*6 + {0..5}] as residual_launch
void residual_seg_launch(const DevCSR& A, const double* b, const double* x, double* r, int c0, int nc,
                         double* red, const DevSegs& g, cudaStream_t s);
// dst = active[system of row] ? (float)src : 0 over n_ext x nc
void cast_seg_launch(const double* src, float* dst, int n_ext, int nc, const DevSegs& g, cudaStream_t s);

// max |a| per system over the real rows of the permuted CSR (padding rows
// skipped) into out[k] as double bits (atomicMax; the caller zeroes out)
void csr_absmax_seg_launch(const DevCSR& A, const DevSegs& g, unsigned long long* out, cudaStream_t s);
// max |v[i]| over n values into *out as double bits (atomicMax; the caller zeroes *out)
void absmax_launch(const double* v, int64_t n, unsigned long long* out, cudaStream_t s);

}  // namespace sog
