/*
 * soglu_gb300 — GB300 (sm_103a) executor for the factor-and-solve path of
 * sparse-operator-graph-LU, behind a plain C ABI (no exceptions, no C++ or
 * torch types; int status codes; opaque handles).
 *
 * The reference solver has no FFI; its executor boundary is internal:
 *   planner  -> BlockPlanner::calculate()           (BlockPlanner.cpp:376)
 *            -> BlockPlanner::solve(bl, bu, b, n)   (BlockPlanner.cpp:834)
 * and its outer API is SOGLU::solveLU (solver.cpp:121, solver.h:24). Each
 * entry point below names the reference interface it replaces.
 *
 * Threading: a context owns one CUDA stream on one device; calls on one
 * context must come from one thread at a time. Systems are independent.
 */
#ifndef SOGLU_GB300_H
#define SOGLU_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define SOG_OK 0
#define SOG_EINVAL 1    /* malformed argument, matrix or DAG */
#define SOG_ENOMEM 2    /* device block pool or device memory exhausted */
#define SOG_EPIVOT 3    /* a diagonal-block pivot was clamped or grew past the limit */
#define SOG_ENAN 4      /* NaN/Inf in the solution */
#define SOG_ETIMEOUT 5  /* a bounded device-side wait expired; the context stays usable */
#define SOG_ECUDA 6     /* CUDA runtime error (message in sog_last_error) */
#define SOG_ENOCONV 7   /* iterative refinement did not reach the tolerance */
#define SOG_ESTATE 8    /* call out of order (e.g. solve before factor) */
#define SOG_ENODEV 9    /* no CUDA device, or the library was built without one */

/* ---- precision and executor modes ---------------------------------------- */
#define SOG_FP64 0      /* plain FP64 factor + solve (DMMA tile products) */
#define SOG_MIXED 1     /* FP32 factors, 3xTF32 tile products, FP64 iterative refinement */

#define SOG_EXEC_PERSISTENT 0 /* one persistent launch claiming tasks in a static order (estimated start
                                 time), each claimant waiting for its task's dependency count to reach zero */
#define SOG_EXEC_LEVELS 1     /* one launch per dependency level (stage-synchronous, like calculate()) */
#define SOG_EXEC_QUEUE 2      /* one persistent launch pulling ready tasks from a device queue, each CTA
                                 keeping the most urgent successor it readied */
#define SOG_EXEC_AUTO 3       /* tuned: the first factorisation times the persistent executors (and, for
                                 SOG_MIXED with pipeline_stages = 0, both stage counts where two CTAs fit
                                 per SM) and keeps the fastest, remembered for task graphs of the same
                                 size and parallelism */

/* One unit operation: the fields of the reference's struct operation
 * (operation.h:37-48); op numbering follows enum blockOp (operation.h:20):
 * 1 lu, 2 lowerInv, 3 upperInv, 4 sub, 8 mul, 9 mulneg. Block id 0 = none. */
typedef struct {
    int32_t op, src, src2, result, result2, stage;
} sog_op;

typedef struct sog_plan sog_plan;     /* host planner output: ordering + op DAG */
typedef struct sog_ctx sog_ctx;       /* device, stream, block pool */
typedef struct sog_system sog_system; /* one system's tiles/factors resident on the device */

typedef struct {
    int32_t n, n_ext, block_rows, block_rows_l2, block_size_l2;
    int32_t storage_count; /* block ids are 1..storage_count-1 */
    int32_t n_input;       /* input tiles carry ids 1..n_input */
    int32_t stages;
    int64_t nops, n_lleaf, n_uleaf, nnz;
    int64_t op_count[13];  /* per enum blockOp */
    int64_t coarse_ops, fine_ops_emitted;
    double t_order, t_plan; /* seconds */
} sog_plan_info;

typedef struct {
    int32_t precision;   /* SOG_FP64 or SOG_MIXED */
    int32_t executor;    /* SOG_EXEC_PERSISTENT, SOG_EXEC_LEVELS, SOG_EXEC_QUEUE or SOG_EXEC_AUTO */
    int32_t max_refine;  /* iterative-refinement steps allowed (SOG_MIXED) */
    double tol;          /* target ||b - A x||_2 / ||b||_2 (SOG_MIXED), e.g. 1e-10 */
    int32_t gemm_split;  /* 0 = auto; FP64 tile products split into 1 or 4 output quadrants */
    int32_t solve_lookahead; /* 0 = on, -1 = off: the factor also forms Dinv_i * L_{i,i-d} for d = 1..3
                                (and the U counterparts) so each substitution row waits on each of its
                                three nearest rows for one 64x64 product only */
    int32_t pipeline_stages; /* SOG_MIXED tensor-core operand stages: 2 (the next product stages while
                                one computes; 128 KB of shared memory), 1 (64 KB), or 0 = 2, tuned with
                                SOG_EXEC_AUTO */
    int32_t max_ctas;        /* 0 = the whole GPU; else at most this many CTAs for the persistent factor and
                                the substitution launches, so that systems running on other streams
                                (sog_system_set_stream) share the SMs */
    double growth_limit;     /* pivot gate (the method does not pivot): the factor call returns SOG_EPIVOT,
                                with the factors resident and usable, when a system had a pivot clamped, a
                                diagonal block whose U U^-1 check failed (the reference's inv_check_diag,
                                MatrixStdDouble.cpp:2871-2937, which it only prints), or a growth
                                (sog_solve_stats.max_growth) above this limit. 0 = default: 1e8 for SOG_FP64,
                                1e4 for SOG_MIXED (FP32 factors lose about growth x 6e-8 of relative accuracy;
                                on SOG_EPIVOT a mixed caller whose refinement does not converge should factor
                                in SOG_FP64); < 0 = no gate, the reference's clamp-and-continue */
    int32_t resident_compact; /* 1 = after each factorisation keep only the tiles the substitution reads
                                 (L/U leaves, diagonal inverses, look-ahead products) and return the rest
                                 of the block pool (the reference frees blocks after their last stage,
                                 BlockPlanner.cpp:597-648); the next factorisation allocates them again.
                                 0 = keep every tile (no reallocation between refactorisations) */
    int32_t reserved;
} sog_options;

typedef struct {
    int32_t status;          /* SOG_* of the solve */
    int32_t iterations;      /* refinement steps taken */
    double rel_resid;        /* ||b - A x||_2 / ||b||_2, worst right-hand side */
    double backward_error;   /* ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf), worst rhs */
    int64_t nan_count;
    double min_pivot;        /* smallest |u_ii| seen by the last factorisation (before the clamp) */
    int32_t clamped_pivots;  /* pivots raised to +-1e-9 (the reference's clamp; LL^T: 1e-20) */
    int32_t inv_check_failures; /* diagonal blocks whose U U^-1 diagonal is off 1 by more than 1e-3 or not
                                   finite (inv_check_diag after upperInv, BlockPlanner.cpp:575-577) */
    double max_growth;       /* max over diagonal blocks of the largest magnitude its factorisation saw
                                (the Schur-updated block entering ludcmpSimple, or its U; LL^T: |L|^2)
                                divided by max |a_ij| of the system: a lower bound on the element
                                growth factor of the unpivoted factorisation */
    int32_t reserved[2];
} sog_solve_stats;

/* Last error message of the calling thread ("" if none). */
const char *sog_last_error(void);
/* Build identification, e.g. "soglu_gb300 sm_103a". */
const char *sog_version(void);

/* ---- host planner ----------------------------------------------------------
 * Replaces the planning half of SOGLU::solveLU (solver.cpp:121-170) and
 * SOGLU::decompose_solveLU (solver.cpp:50-110): GOrder::Reorder +
 * GOrder::sortInBlock (GPSOrder.cpp:55-650), config::set (config.cpp:41),
 * blockMatrixLU + copyOperatorL2 + blockPlan (BlockPlanner.cpp:103-374,
 * 865-1577). I/J are 0-based; symmetric = lower triangle given (mtx.cpp:60,
 * solver.cpp:132-149; the LL^T recursion, BlockPlanner.cpp:941-989, with llt
 * and mult ops and L leaves only).
 * threads = OpenMP threads for the ordering search (0 = default). */
int sog_plan_build(int32_t n, int64_t nnz, int32_t symmetric, const int32_t *I, const int32_t *J,
                   const double *V, int32_t threads, sog_plan **out);
int sog_plan_get_info(const sog_plan *plan, sog_plan_info *info);
/* Copy out the plan: new_to_old[n] (GOrder::newOrder), ops[nops] in the
 * reference's stage order, lleaf/uleaf [n_*leaf][3] = {bi, bj, block id}. Any
 * pointer may be NULL to skip that array. For a batch plan (sog_plan_merge)
 * new_to_old has n_ext entries: per permuted row its row in its own system's
 * original ordering, -1 for padding. */
int sog_plan_export(const sog_plan *plan, int32_t *new_to_old, sog_op *ops, int32_t *lleaf, int32_t *uleaf);
/* Dense input tiles (n_input x 64 x 64, row-major) for values V in the
 * triplet order given to sog_plan_build (BlockPlanner::iniBlockStorage,
 * BlockPlanner.cpp:1491-1539, padded rows get a unit diagonal). */
int sog_plan_input_tiles(const sog_plan *plan, const double *V, double *tiles);
/* Import a DAG produced elsewhere (e.g. the reference planner's data::graph
 * and L/U quadtree leaves) instead of building one; no ordering is attached
 * (identity), input tiles then come through sog_factor_tiles. */
int sog_plan_import(int32_t block_rows, int32_t storage_count, int32_t n_input, const sog_op *ops, int64_t nops,
                    const int32_t *lleaf, int64_t n_lleaf, const int32_t *uleaf, int64_t n_uleaf, sog_plan **out);
void sog_plan_destroy(sog_plan *plan);

/* ---- MatrixMarket input --------------------------------------------------------
 * SOGLU::mtx::readMTX (mtx.cpp:44-117): coordinate file, header "symmetric" =>
 * lower triangle given; lines of <= 3 characters and lines containing '%'
 * skipped; zero values dropped; 1-based indices (returned 0-based). Entry
 * lines are parsed in parallel chunks, in file order. use_cache: read
 * <path>.sogbin when it matches the text file's size and modification time,
 * else parse and write it (no reference counterpart). */
typedef struct sog_mtx sog_mtx;
int sog_mtx_read(const char *path, int32_t use_cache, sog_mtx **out);
int sog_mtx_info(const sog_mtx *m, int32_t *n, int64_t *nnz, int32_t *symmetric);
/* copy the triplets out (arrays of nnz entries; any pointer may be NULL) */
int sog_mtx_copy(const sog_mtx *m, int32_t *I, int32_t *J, double *V);
void sog_mtx_destroy(sog_mtx *m);

/* ---- batches -----------------------------------------------------------------
 * No counterpart in the reference, which factors one system per process
 * (solver.cpp:121). A batch plan is the block-diagonal union of independent
 * systems' plans: every op, stage and leaf of each system as its own planner
 * made it, block ids and block rows shifted, so one executor launch factors
 * all systems and merges ready tile operations of different systems into the
 * same launch. A system built from it (sog_system_create) takes, in system
 * order: V = the systems' triplet values concatenated (sog_factor*), and for
 * solves b / x = per system nrhs_k x n_k values (rhs-major within the system),
 * concatenated. Refinement (SOG_MIXED) stops per system: a system that has
 * converged receives no further corrections while others refine, so its
 * result is the one it gets alone. Imported plans cannot be batched. */
int sog_plan_merge(const sog_plan *const *plans, int32_t count, sog_plan **out);
/* Number of systems in a plan (1 for a plain plan) and, if n is not NULL,
 * each system's dimension. */
int sog_plan_segments(const sog_plan *plan, int32_t *count, int32_t *n);

/* ---- device context ----------------------------------------------------------
 * The device block-pool arena that replaces memutil's per-thread block pools
 * (memutil.cpp:74-113). pool_bytes = 0: 90% of free device memory. */
int sog_ctx_create(int32_t device, uint64_t pool_bytes, sog_ctx **out);
/* Destroy every system and server of the context first: they use its stream
 * and pool. */
void sog_ctx_destroy(sog_ctx *ctx);
/* bytes of the pool in use / total */
int sog_ctx_pool_usage(const sog_ctx *ctx, uint64_t *used, uint64_t *total);
/* The context's CUDA stream (a cudaStream_t) — every kernel of every system
 * on this context is launched on it, so callers can order and time work
 * against it with their own events. */
int sog_ctx_stream(const sog_ctx *ctx, void **stream);
/* Return pool chunks that hold no allocation to the device (after many
 * systems of different sizes came and went). */
int sog_ctx_trim(sog_ctx *ctx);

/* ---- one system --------------------------------------------------------------
 * Upload the plan's DAG and allocate its tiles in the pool (admission: returns
 * SOG_ENOMEM without side effects when the pool cannot hold them). */
int sog_system_create(sog_ctx *ctx, const sog_plan *plan, const sog_options *opt, sog_system **out);
/* bytes of pool this plan needs under opt (for admission decisions) */
int sog_system_bytes(const sog_plan *plan, const sog_options *opt, uint64_t *bytes);
/* BlockPlanner::calculate (BlockPlanner.cpp:376-651) on values V (host, the
 * triplet order of sog_plan_build). Returns after the factors are resident;
 * SOG_EPIVOT (factors resident, usable) when a system fails the pivot gate
 * of sog_options.growth_limit. */
int sog_factor(sog_system *sys, const double *V);
/* Same with V already on the device (device pointer). */
int sog_factor_device(sog_system *sys, const double *V_dev);
/* BlockPlanner::calculate with input tiles given directly (host,
 * n_input x 64 x 64 row-major FP64, block id k+1 at index k). */
int sog_factor_tiles(sog_system *sys, const double *tiles);
/* Run this system's kernels and copies on the caller's stream (a
 * cudaStream_t; NULL = the context's stream again), e.g. several systems of
 * one context factored concurrently from different host threads, each on its
 * own stream (the block pool is shared and locked). Waits for the system's
 * work on its previous stream first. No reference counterpart (one system per
 * process, main.cpp). */
int sog_system_set_stream(sog_system *sys, void *stream);
/* Solve with the resident factors. b and x are host arrays of nrhs right-hand
 * sides, each of length n, in the ORIGINAL ordering (rhs-major: b[r*n + i]).
 * Replaces BlockPlanner::solve + GOrder::reOrderResult (BlockPlanner.cpp:834,
 * GPSOrder.cpp:41). SOG_MIXED refines in FP64 on the original matrix. */
int sog_solve(sog_system *sys, int32_t nrhs, const double *b, double *x, sog_solve_stats *stats);
/* Same with device pointers. */
int sog_solve_device(sog_system *sys, int32_t nrhs, const double *b_dev, double *x_dev, sog_solve_stats *stats);
/* sog_factor then sog_solve in one call (host arrays; the device variant
 * takes device pointers), with the same results and return codes: a pivot-gate
 * failure (SOG_EPIVOT) still solves with the resident factors. A plain
 * SOG_MIXED system factored by the static-order executor, with nrhs = 1 or a
 * multiple of 8 up to 64, runs the first forward substitution while the
 * factorisation runs, each block row starting once the factor tasks that
 * produce its tiles have finished. The reference runs BlockPlanner::calculate
 * and BlockPlanner::solve one after the other (main.cpp). */
int sog_factor_solve(sog_system *sys, const double *V, int32_t nrhs, const double *b, double *x,
                     sog_solve_stats *stats);
int sog_factor_solve_device(sog_system *sys, const double *V_dev, int32_t nrhs, const double *b_dev, double *x_dev,
                            sog_solve_stats *stats);
/* Batch solve with a right-hand-side count per system (nrhs[k] >= 0; a
 * system with 0 right-hand sides is skipped): b / x = per system nrhs[k] x
 * n_k values, concatenated in system order. stats, if not NULL, receives one
 * entry per system (count from sog_plan_segments); the return value is the
 * worst status. On a plain plan this is sog_solve with nrhs[0]. */
int sog_solve_batch(sog_system *sys, const int32_t *nrhs, const double *b, double *x, sog_solve_stats *stats);
/* Same with device pointers. */
int sog_solve_batch_device(sog_system *sys, const int32_t *nrhs, const double *b_dev, double *x_dev,
                           sog_solve_stats *stats);
/* BlockPlanner::solve exactly: b_ext / x_ext are host arrays of length n_ext
 * in the planner's (permuted, padded) ordering; one right-hand side; no
 * refinement. */
int sog_solve_permuted(sog_system *sys, const double *b_ext, double *x_ext);
/* Copy resident L/U leaf tiles (in plan leaf order) to host, FP64 (an LL^T
 * plan has L leaves only). */
int sog_system_export_factors(sog_system *sys, double *ltiles, double *utiles);
/* Device time of the last factor / solve in milliseconds (CUDA events on the
 * context's stream; after sog_factor_solve the solve's time runs from the end
 * of the factor kernel, including any wait for the overlapped forward
 * substitution). */
int sog_system_last_times(const sog_system *sys, double *factor_ms, double *solve_ms);
void sog_system_destroy(sog_system *sys);
/* Build the device task graph of a plan on the host only (no device):
 * counts[15] = {tasks, dependency levels, queue items, tile-product pairs,
 * GEMM, LU, LINV, UINV, SUB tasks, fused Schur subs, added diagonal-inverse
 * blocks, critical-path length in tasks, lower inverses fused into LU, copies
 * replaced by aliasing (a copy's readers read its source's tile), repeated
 * inverses of one block replaced by aliasing}. */
int sog_plan_task_graph_info(const sog_plan *plan, int32_t gemm_split, int64_t *counts);
/* Task-graph summary: counts[11] = {tasks, dependency levels, queue items,
 * tile-product pairs, GEMM, LU, LINV, UINV, SUB tasks, persistent grid,
 * kernel launches issued by this system so far}. */
int sog_system_task_info(const sog_system *sys, int64_t *counts);
/* Pivot statistics of the last factorisation, one entry per system of the
 * plan (sog_plan_segments): min_pivot, clamped_pivots, inv_check_failures,
 * max_growth, and status = SOG_EPIVOT for a system that failed the pivot gate
 * (sog_options.growth_limit), else SOG_OK; the other fields are 0. No
 * reference counterpart: ludcmpSimple clamps silently
 * (MatrixStdDouble.cpp:2751-2761) and inv_check_diag only prints. */
int sog_system_pivots(const sog_system *sys, sog_solve_stats *stats);
/* Executor configuration in use (after autotuning, the chosen one):
 * SOG_EXEC_*, tensor-core operand stages (mixed), and whether products start
 * before their last producer finished (mixed, static order: 1). */
int sog_system_executor(const sog_system *sys, int32_t *executor, int32_t *stages, int32_t *early);

/* ---- profiling (no reference counterpart: the reference prints phase
 * timers only, solver.cpp:53-118) ---------------------------------------------
 * Per-task device timestamps (globaltimer ns) of the next factorisations:
 * task_trace[4*t] = {ready, ~start, end, SM id} (start is stored inverted;
 * ready = 0 for tasks ready at launch), row_trace[4*i] = {lower start, lower
 * end, upper start, upper end} of the last substitution. */
int sog_system_trace_enable(sog_system *sys, int32_t on);
int sog_system_trace_get(sog_system *sys, uint64_t *task_trace, uint64_t *row_trace, int32_t *task_kind);
/* Task graph export: succ_ptr[tasks+1], succ[...], npairs[tasks] (GEMM operand pairs). */
int sog_system_task_graph(const sog_system *sys, int32_t *succ_ptr, int32_t *succ, int32_t *npairs);

/* ---- failure handling (no reference counterpart: the reference has no
 * device waits) ------------------------------------------------------------
 * Bound, in milliseconds, on any single device-side wait (ready-queue slot in
 * the factor, row readiness in the solve; default 10 s). A wait that runs out
 * sets a status bit, the kernel returns, the call returns SOG_ETIMEOUT and the
 * context stays usable. */
int sog_system_set_wait_limit(sog_system *sys, double ms);
/* Testing hook: raise one task's dependency count so it never becomes ready
 * (host-side fault injection); sog_debug_unpoison restores the graph. */
int sog_debug_poison_task(sog_system *sys, int32_t task);
int sog_debug_unpoison(sog_system *sys);
/* Testing hook (FP64 systems): on = 0 runs every DMMA of the FP64 products,
 * on = 1 skips those whose operand fragment is all zero (the default; the
 * autotuner may pick either). Either way the factors are the same: a skipped
 * MMA would only add exact zeros. Overrides a pending autotuning choice. */
int sog_debug_fp64_fragment_skip(sog_system *sys, int32_t on);

/* ---- allocation-free residual check (no counterpart in the reference) ------
 * r = b - A x in FP64 for a CSR matrix on the device, and per right-hand side
 * rel_resid[c] = ||r||_2 / ||b||_2 and backward_error[c] =
 * ||r||_inf / (||A||_inf ||x||_inf + ||b||_inf), the figures sog_solve
 * reports. For callers that cannot call cudaMalloc: code whose device memory
 * is owned by another allocator (a framework's caching allocator, a fixed
 * serving budget) and latency-critical loops where an allocation would
 * synchronise the device. It allocates nothing: its reduction scratch is a
 * fixed 3 KB array of device memory that every GPU loading the library holds
 * until exit, so nrhs is limited to 1..64 (SOG_EINVAL beyond). All calls
 * share that array: calls that overlap on the GPU (different streams or host
 * threads) race and must be serialised by the caller. The first call on a
 * device looks up the array's device address (with that device current);
 * make that first call before any stream capture. Arrays are device pointers;
 * b, x, r are n x nrhs row-major; rel_resid and backward_error are host
 * arrays of nrhs; stream is a cudaStream_t (NULL = default stream); returns
 * after the results are on the host. */
int sog_residual_noalloc(int32_t n, const int32_t *row_ptr, const int32_t *col, const double *val, int32_t nrhs,
                         const double *b, const double *x, double *r, double *rel_resid, double *backward_error,
                         void *stream);

/* ---- outer drop-in --------------------------------------------------------------
 * SOGLU::solveLU (solver.cpp:121-184): plan, factor and solve one system on
 * device 0; x_out receives n values in the original ordering. */
int soglu_solveLU(int32_t dim, int64_t valcount, int32_t symmetric, const int32_t *index_i, const int32_t *index_j,
                  const double *vals, const double *b, double *x_out, int32_t precision);

/* ---- serving -----------------------------------------------------------------
 * No counterpart in the reference (one system per process, main.cpp). A
 * request loop with continuous batching: sog_server_submit copies a request
 * (COO system as for sog_plan_build, nrhs right-hand sides rhs-major) and
 * returns at once; host worker threads plan it; a scheduler thread admits
 * the planned requests that the block pool can hold (first come, first
 * served, sog_system_bytes as the estimate) to the first free lane, merged
 * into one batch plan. A lane (a host thread and a CUDA stream) factors its
 * batch in one executor launch and solves all its right-hand sides together.
 * Lanes run concurrently: a request that arrives while another batch is on
 * the GPU starts at once on a free lane, its kernels beside the other batch's
 * (each batch's persistent grid is sized to its parallelism, at most three
 * quarters of the GPU while there are other lanes). A request larger than the
 * whole pool fails with SOG_ENOMEM; one that fits once others are released
 * waits. A system that fails the pivot gate (sog_options.growth_limit) is
 * answered with SOG_EPIVOT and its solution. Resident factors are compacted
 * (sog_options.resident_compact is set for the server's systems).
 * Factors stay resident after the answer (sog_server_solve for further
 * right-hand sides) until sog_server_release. The context must not be used
 * directly while a server runs on it. */
typedef struct sog_server sog_server;
typedef struct {
    int32_t planner_threads;      /* host planning workers (0 = 2) */
    int32_t planner_omp_threads;  /* OpenMP threads per plan (0 = default) */
    int32_t max_batch;            /* requests merged into one launch at most (0 = 256) */
    int32_t lanes;                /* batches on the GPU at the same time, each on its own stream (0 = 2) */
    double batch_window_ms;       /* once a request is planned, wait up to this long for requests
                                     still being planned to join its launch (0 = launch at once) */
    int32_t reserved[2];
} sog_server_options;
typedef struct {
    int32_t status;       /* SOG_OK, SOG_ENOCONV, SOG_ENAN, or the request's error */
    int32_t batch_size;   /* requests factored in the same launch */
    int64_t batch_id;
    double plan_ms;       /* host planning */
    double queue_ms;      /* planned -> admitted */
    double setup_ms;      /* admitted -> the batch's factor starts: plan merge, task graph, device upload */
    double gpu_ms;        /* the batch's factor + solve, host clock */
    double total_ms;      /* submit -> answer */
    sog_solve_stats stats;
} sog_request_info;
/* opt: the systems' options (NULL = SOG_MIXED, 10 refinement steps, 1e-10) */
int sog_server_create(sog_ctx *ctx, const sog_options *opt, const sog_server_options *sopt, sog_server **out);
/* symmetric: lower triangle given, factored L L^T (as sog_plan_build) */
int sog_server_submit(sog_server *srv, int32_t n, int64_t nnz, const int32_t *I, const int32_t *J, const double *V,
                      int32_t symmetric, int32_t nrhs, const double *b, int64_t *id);
/* Wait for the answer (timeout_ms < 0: no limit; SOG_ETIMEOUT if still
 * running). x (if not NULL) receives nrhs x n values. */
int sog_server_wait(sog_server *srv, int64_t id, double timeout_ms, double *x, sog_request_info *info);
/* Further right-hand sides on a request's resident factors (blocks the caller). */
int sog_server_solve(sog_server *srv, int64_t id, int32_t nrhs, const double *b, double *x, sog_solve_stats *stats);
/* Drop a finished request; its batch's pool memory returns when all of the
 * batch's requests are released. */
int sog_server_release(sog_server *srv, int64_t id);
/* counts[8] = {batches launched, requests admitted, completed, rejected,
 * largest batch, requests resident, planned and waiting, waiting to plan} */
int sog_server_counters(sog_server *srv, int64_t *counts);
void sog_server_destroy(sog_server *srv);

#ifdef __cplusplus
}
#endif
#endif /* SOGLU_GB300_H */
