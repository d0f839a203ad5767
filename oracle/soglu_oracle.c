/*
 * ORACLE — test infrastructure, not the product. Only tests/, the smoke check
 * in __graft_entry__.py and the CPU-baseline leg of bench.py load this code,
 * as the checker or as the timed CPU baseline; the GPU executor never calls it.
 *
 * A plain-C restatement of the reference's executor path for one system:
 *   oracle_calculate : BlockPlanner::calculate (BlockPlanner.cpp:376-651) with
 *                      the unit ops of MatrixStdDouble.cpp (LU and LL^T paths)
 *   oracle_solve     : BlockPlanner::solve (BlockPlanner.cpp:652-862)
 * on dense 64x64 row-major FP64 tiles indexed by block id, and
 *   oracle_solve_lean: the two together with the reference's block lifetime
 *                      (lazy allocation on first write, free after the last
 *                      stage that reads a block, BlockPlanner.cpp:419-445,
 *                      597-648, laststage from BlockPlanner.cpp:355-371), so
 *                      large systems need the reference's memory, not one
 *                      tile per block id; right-hand sides solved in parallel.
 * Like the reference it runs each stage's ops in parallel (OpenMP), serialising ops that write
 * the same block, and skips all-zero 8x8 sub-tiles in the block products
 * (the mask skipping of MatrixStdDouble.cpp:2043-2507).
 *
 * Pinning: tests compare this restatement with the compiled reference
 * (oracle/_ref/ref_solve, built from the reference sources by
 * oracle/build_ref.sh) through golden fixtures under tests/golden/.
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define B 64
#define TILE (B * B)

enum { OP_INV = 0, OP_LU = 1, OP_LOWERINV = 2, OP_UPPERINV = 3, OP_SUB = 4, OP_MUL = 8, OP_MULNEG = 9, OP_LLT = 10,
       OP_MULT = 11 };

/* 8x8 occupancy: bit kb of m[ib] set when sub-tile (ib, kb) has a nonzero. */
static void occupancy(const double *t, uint8_t m[8]) {
    for (int ib = 0; ib < 8; ib++) {
        uint8_t bits = 0;
        for (int r = 0; r < 8; r++) {
            const double *row = t + (ib * 8 + r) * B;
            for (int kb = 0; kb < 8; kb++) {
                if (bits & (1u << kb)) continue;
                for (int c = 0; c < 8; c++)
                    if (row[kb * 8 + c] != 0.0) { bits |= (uint8_t)(1u << kb); break; }
            }
        }
        m[ib] = bits;
    }
}

/* C += sign * A * B over nonzero 8x8 sub-tiles (MatrixStdDouble.cpp:2043 mul, :237 mulneg). */
static void tile_gemm(double *restrict c, const double *restrict a, const double *restrict b, double sign) {
    uint8_t ma[8], mb[8];
    occupancy(a, ma);
    occupancy(b, mb);
    for (int ib = 0; ib < 8; ib++) {
        for (int kb = 0; kb < 8; kb++) {
            if (!(ma[ib] & (1u << kb))) continue;
            for (int jb = 0; jb < 8; jb++) {
                if (!(mb[kb] & (1u << jb))) continue;
                for (int i = ib * 8; i < ib * 8 + 8; i++) {
                    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                    for (int k = kb * 8; k < kb * 8 + 8; k++) {
                        double av = a[i * B + k];
                        const double *brow = b + k * B + jb * 8;
                        for (int j = 0; j < 8; j++) acc[j] += av * brow[j];
                    }
                    double *crow = c + i * B + jb * 8;
                    for (int j = 0; j < 8; j++) crow[j] += sign * acc[j];
                }
            }
        }
    }
}

/* Unpivoted Doolittle LU, unit-diagonal L, pivots |u_ii| < 1e-9 clamped to
 * +-1e-9 (ludcmpSimple, MatrixStdDouble.cpp:2711-2784). */
static void tile_lu(const double *a, double *l, double *u) {
    memset(l, 0, sizeof(double) * TILE);
    memset(u, 0, sizeof(double) * TILE);
    for (int i = 0; i < B; i++) {
        for (int j = i; j < B; j++) {
            double s = 0;
            for (int k = 0; k < i; k++) s += l[i * B + k] * u[k * B + j];
            u[i * B + j] = a[i * B + j] - s;
        }
        double p = u[i * B + i];
        if (p < 1e-9 && p > -1e-9) p = (p < 0) ? -1e-9 : 1e-9;
        u[i * B + i] = p;
        double r = 1.0 / p;
        for (int j = i + 1; j < B; j++) {
            double s = 0;
            for (int k = 0; k < i; k++) s += l[j * B + k] * u[k * B + i];
            l[j * B + i] = r * (a[j * B + i] - s);
        }
        l[i * B + i] = 1.0;
    }
}

/* C += A * B^T (mat_mult, MatrixStdDouble.cpp:704-1555). */
static void tile_mult(double *restrict c, const double *restrict a, const double *restrict b) {
    for (int i = 0; i < B; i++)
        for (int j = 0; j < B; j++) {
            double s = 0;
            for (int k = 0; k < B; k++) s += a[i * B + k] * b[j * B + k];
            c[i * B + j] += s;
        }
}

/* Cholesky L L^T = A from the lower triangle of a, column by column; pivots
 * below 1e-20 (TINY, MatrixStdDouble.cpp:29) are raised to it before the
 * square root (lltdcmpSimple, MatrixStdDouble.cpp:2629-2668). */
static void tile_llt(const double *a, double *l) {
    memset(l, 0, sizeof(double) * TILE);
    for (int j = 0; j < B; j++) {
        double s = 0;
        for (int r = 0; r < j; r++) s += l[j * B + r] * l[j * B + r];
        double p = a[j * B + j] - s;
        if (p < 1e-20) p = 1e-20;
        p = sqrt(p);
        l[j * B + j] = p;
        const double rp = 1.0 / p;
        for (int i = j + 1; i < B; i++) {
            double t = 0;
            for (int r = 0; r < j; r++) t += l[i * B + r] * l[j * B + r];
            l[i * B + j] = rp * (a[i * B + j] - t);
        }
    }
}

/* Y = L^-1, lower triangle of l incl. its diagonal (inv_lower, MatrixStdDouble.cpp:2787-2802). */
static void tile_inv_lower(const double *l, double *y) {
    memset(y, 0, sizeof(double) * TILE);
    for (int i = 0; i < B; i++) {
        double q = 1.0 / l[i * B + i];
        y[i * B + i] = q;
        for (int j = 0; j < i; j++) {
            double s = 0;
            for (int k = j; k < i; k++) s += l[i * B + k] * y[k * B + j];
            y[i * B + j] = -s * q;
        }
    }
}

/* Y = U^-1 by Gauss-Jordan from the bottom row (inv_upper, MatrixStdDouble.cpp:2829-2866). */
static void tile_inv_upper(const double *u, double *y) {
    memset(y, 0, sizeof(double) * TILE);
    for (int i = 0; i < B; i++) y[i * B + i] = 1.0;
    for (int j = B - 1; j >= 0; j--) {
        for (int i = j - 1; i >= 0; i--) {
            double scale = u[i * B + j] / u[j * B + j];
            for (int k = j; k < B; k++) y[i * B + k] -= scale * y[j * B + k];
        }
        double rate = 1.0 / u[j * B + j];
        for (int k = j; k < B; k++) y[j * B + k] *= rate;
    }
}

typedef struct {
    int32_t op, src, src2, res, res2, stage;
} op6;

static int cmp_i64(const void *x, const void *y) {
    int64_t a = *(const int64_t *)x, b = *(const int64_t *)y;
    return (a > b) - (a < b);
}

/*
 * Execute a stage-sorted op list. tiles[id*4096 ...] holds block `id`; input
 * tiles are filled by the caller, every other tile must be zero on entry.
 * Returns 0, or -1 on a malformed DAG.
 */
int oracle_calculate(int64_t nops, const int32_t *ops_flat, int32_t storage_count, double *tiles, int threads) {
    const op6 *ops = (const op6 *)ops_flat;
    if (threads > 0) omp_set_num_threads(threads);
    for (int64_t i = 0; i < nops; i++) {
        const op6 *o = &ops[i];
        if (o->res < 0 || o->res >= storage_count || o->src < 0 || o->src >= storage_count || o->src2 < 0 ||
            o->src2 >= storage_count || o->res2 < 0 || o->res2 >= storage_count)
            return -1;
        if (i > 0 && ops[i - 1].stage > o->stage) return -1;
    }
    /* group ops of a stage by result so that same-result writers run in one
     * thread, in graph order (the reference's streams, BlockPlanner.cpp:402-416) */
    int64_t *perm = (int64_t *)malloc(sizeof(int64_t) * (nops + 1));
    int64_t *heads = (int64_t *)malloc(sizeof(int64_t) * (nops + 1));
    if (!perm || !heads) { free(perm); free(heads); return -2; }
    int64_t s0 = 0;
    while (s0 < nops) {
        int64_t s1 = s0;
        while (s1 < nops && ops[s1].stage == ops[s0].stage) s1++;
        /* gather same-result ops, keeping graph order among them: sort keys
         * (result << 32 | position) */
        int64_t n = s1 - s0;
        for (int64_t k = 0; k < n; k++) perm[k] = ((int64_t)ops[s0 + k].res << 32) | k;
        qsort(perm, (size_t)n, sizeof(int64_t), cmp_i64);
        for (int64_t k = 0; k < n; k++) perm[k] = s0 + (perm[k] & 0xffffffffLL);
        int64_t nh = 0;
        for (int64_t k = 0; k < n; k++)
            if (k == 0 || ops[perm[k]].res != ops[perm[k - 1]].res) heads[nh++] = k;
        heads[nh] = n;
#pragma omp parallel for schedule(dynamic)
        for (int64_t h = 0; h < nh; h++) {
            for (int64_t k = heads[h]; k < heads[h + 1]; k++) {
                const op6 *o = &ops[perm[k]];
                double *r = tiles + (int64_t)o->res * TILE;
                const double *a = tiles + (int64_t)o->src * TILE;
                const double *b2 = tiles + (int64_t)o->src2 * TILE;
                switch (o->op) {
                    case OP_LU: tile_lu(a, r, tiles + (int64_t)o->res2 * TILE); break;
                    case OP_LOWERINV: tile_inv_lower(a, r); break;
                    case OP_UPPERINV: tile_inv_upper(a, r); break;
                    case OP_MUL: tile_gemm(r, a, b2, 1.0); break;
                    case OP_MULNEG: tile_gemm(r, a, b2, -1.0); break;
                    case OP_LLT: tile_llt(a, r); break;
                    case OP_MULT: tile_mult(r, a, b2); break;
                    case OP_SUB: /* r = src2 - src; copy / negate when one is absent (BlockPlanner.cpp:553-572) */
                        for (int e = 0; e < TILE; e++) {
                            double v = 0;
                            if (o->src2 > 0) v = b2[e];
                            if (o->src > 0) v -= a[e];
                            r[e] = v;
                        }
                        break;
                    default: break;
                }
            }
        }
        s0 = s1;
    }
    free(perm);
    free(heads);
    return 0;
}

/*
 * Block forward (unit-L) and back (U) substitution over the L/U leaves
 * (lowerSolver / upperSolver / updateVector, BlockPlanner.cpp:669-832).
 * leaves: {bi, bj, id} triples. b (length block_rows*64) is overwritten with
 * the forward-eliminated right-hand side, as the reference does; x receives
 * the solution (length block_rows*64). Returns the number of NaNs in x.
 */
int64_t oracle_solve(int32_t block_rows, int64_t nl, const int32_t *lleaf, int64_t nu, const int32_t *uleaf,
                     const double *tiles, double *b, double *x) {
    const int R = block_rows;
    int64_t n = (int64_t)R * B;
    double *y = (double *)calloc((size_t)n, sizeof(double));
    int64_t *lp = (int64_t *)calloc((size_t)R + 1, sizeof(int64_t));
    int64_t *up = (int64_t *)calloc((size_t)R + 1, sizeof(int64_t));
    int32_t *ld = (int32_t *)calloc((size_t)R, sizeof(int32_t));
    int32_t *ud = (int32_t *)calloc((size_t)R, sizeof(int32_t));
    int64_t *li = (int64_t *)malloc(sizeof(int64_t) * (nl + 1));
    int64_t *ui = (int64_t *)malloc(sizeof(int64_t) * (nu + 1));
    for (int64_t k = 0; k < nl; k++) if (lleaf[3 * k] != lleaf[3 * k + 1]) lp[lleaf[3 * k] + 1]++;
    for (int64_t k = 0; k < nu; k++) if (uleaf[3 * k] != uleaf[3 * k + 1]) up[uleaf[3 * k] + 1]++;
    for (int i = 0; i < R; i++) { lp[i + 1] += lp[i]; up[i + 1] += up[i]; }
    int64_t *lf = (int64_t *)malloc(sizeof(int64_t) * (R + 1));
    int64_t *uf = (int64_t *)malloc(sizeof(int64_t) * (R + 1));
    memcpy(lf, lp, sizeof(int64_t) * (R + 1));
    memcpy(uf, up, sizeof(int64_t) * (R + 1));
    for (int64_t k = 0; k < nl; k++) {
        if (lleaf[3 * k] == lleaf[3 * k + 1]) ld[lleaf[3 * k]] = lleaf[3 * k + 2];
        else li[lf[lleaf[3 * k]]++] = k;
    }
    for (int64_t k = 0; k < nu; k++) {
        if (uleaf[3 * k] == uleaf[3 * k + 1]) ud[uleaf[3 * k]] = uleaf[3 * k + 2];
        else ui[uf[uleaf[3 * k]]++] = k;
    }
    /* forward: y_i = L_ii^-1 (b_i - sum_j L_ij y_j) */
    for (int i = 0; i < R; i++) {
        double *bi = b + (int64_t)i * B;
        for (int64_t q = lp[i]; q < lp[i + 1]; q++) {
            int64_t k = li[q];
            const double *t = tiles + (int64_t)lleaf[3 * k + 2] * TILE;
            const double *yj = y + (int64_t)lleaf[3 * k + 1] * B;
            for (int r = 0; r < B; r++) {
                double s = 0;
                for (int c = 0; c < B; c++) s += t[r * B + c] * yj[c];
                bi[r] -= s;
            }
        }
        double *yi = y + (int64_t)i * B;
        if (ld[i] > 0) {
            const double *t = tiles + (int64_t)ld[i] * TILE;
            for (int r = 0; r < B; r++) {
                double s = 0;
                for (int c = 0; c < r; c++) s += t[r * B + c] * yi[c];
                bi[r] -= s;
                yi[r] = bi[r] / t[r * B + r];
            }
        }
    }
    /* backward: x_i = U_ii^-1 (y_i - sum_j U_ij x_j) */
    for (int i = R - 1; i >= 0; i--) {
        double *yi = y + (int64_t)i * B;
        for (int64_t q = up[i]; q < up[i + 1]; q++) {
            int64_t k = ui[q];
            const double *t = tiles + (int64_t)uleaf[3 * k + 2] * TILE;
            const double *xj = x + (int64_t)uleaf[3 * k + 1] * B;
            for (int r = 0; r < B; r++) {
                double s = 0;
                for (int c = 0; c < B; c++) s += t[r * B + c] * xj[c];
                yi[r] -= s;
            }
        }
        double *xi = x + (int64_t)i * B;
        if (ud[i] > 0) {
            const double *t = tiles + (int64_t)ud[i] * TILE;
            for (int r = B - 1; r >= 0; r--) {
                double s = 0;
                for (int c = r + 1; c < B; c++) s += t[r * B + c] * xi[c];
                yi[r] -= s;
                xi[r] = yi[r] / t[r * B + r];
            }
        } else {
            for (int r = 0; r < B; r++) xi[r] = 0;
        }
    }
    int64_t nans = 0;
    for (int64_t k = 0; k < n; k++) if (isnan(x[k])) nans++;
    free(y); free(lp); free(up); free(ld); free(ud); free(li); free(ui); free(lf); free(uf);
    return nans;
}

/* ------------------------------------------------------------------------
 * Lean path: block pointers instead of one flat tile array.
 */
static double *blk_new(void) {
    double *t = (double *)aligned_alloc(64, sizeof(double) * TILE);
    if (t) memset(t, 0, sizeof(double) * TILE);
    return t;
}

/* The substitution of oracle_solve over block pointers, for one right-hand
 * side (b overwritten, y scratch of n doubles). */
static void solve_ptrs(int R, const int64_t *lp, const int64_t *li, const int32_t *ld, const int32_t *lleaf,
                       const int64_t *up, const int64_t *ui, const int32_t *ud, const int32_t *uleaf,
                       double *const *blk, double *b, double *y, double *x) {
    for (int i = 0; i < R; i++) {
        double *bi = b + (int64_t)i * B;
        for (int64_t q = lp[i]; q < lp[i + 1]; q++) {
            const int64_t k = li[q];
            const double *t = blk[lleaf[3 * k + 2]];
            const double *yj = y + (int64_t)lleaf[3 * k + 1] * B;
            if (!t) continue;
            for (int r = 0; r < B; r++) {
                double s = 0;
                for (int c = 0; c < B; c++) s += t[r * B + c] * yj[c];
                bi[r] -= s;
            }
        }
        double *yi = y + (int64_t)i * B;
        const double *t = ld[i] > 0 ? blk[ld[i]] : NULL;
        if (t) {
            for (int r = 0; r < B; r++) {
                double s = 0;
                for (int c = 0; c < r; c++) s += t[r * B + c] * yi[c];
                bi[r] -= s;
                yi[r] = bi[r] / t[r * B + r];
            }
        }
    }
    for (int i = R - 1; i >= 0; i--) {
        double *yi = y + (int64_t)i * B;
        for (int64_t q = up[i]; q < up[i + 1]; q++) {
            const int64_t k = ui[q];
            const double *t = blk[uleaf[3 * k + 2]];
            const double *xj = x + (int64_t)uleaf[3 * k + 1] * B;
            if (!t) continue;
            for (int r = 0; r < B; r++) {
                double s = 0;
                for (int c = 0; c < B; c++) s += t[r * B + c] * xj[c];
                yi[r] -= s;
            }
        }
        double *xi = x + (int64_t)i * B;
        const double *t = ud[i] > 0 ? blk[ud[i]] : NULL;
        if (t) {
            for (int r = B - 1; r >= 0; r--) {
                double s = 0;
                for (int c = r + 1; c < B; c++) s += t[r * B + c] * xi[c];
                yi[r] -= s;
                xi[r] = yi[r] / t[r * B + r];
            }
        } else {
            for (int r = 0; r < B; r++) xi[r] = 0;
        }
    }
}

/*
 * Factor and solve one system with the reference's block lifetime. Input
 * tile k (0-based) is block id k+1. Blocks are allocated (zeroed) when first
 * written and freed after the last stage that reads them as src or src2,
 * except the L/U leaves the substitution needs (the reference's outputs carry
 * a laststage past every stage, BlockPlanner.cpp:88-100). An empty U leaf list
 * means an LL^T plan: the back substitution uses transposed copies of the L
 * tiles (upperSolverT, BlockPlanner.cpp:752-797). b_ext / x_ext: nrhs x
 * (block_rows*64), rhs-major, in the planner's ordering; b_ext is not
 * modified. peak (if not NULL) receives the largest number of live blocks.
 * Returns the NaN count of x, or -1 (malformed DAG), -2 (out of memory).
 */
int64_t oracle_solve_lean(int64_t nops, const int32_t *ops_flat, int32_t storage_count, int32_t n_input,
                          const double *input_tiles, int32_t block_rows, int64_t nl, const int32_t *lleaf, int64_t nu,
                          const int32_t *uleaf, int32_t nrhs, const double *b_ext, double *x_ext, int threads,
                          int64_t *peak) {
    const op6 *ops = (const op6 *)ops_flat;
    if (threads > 0) omp_set_num_threads(threads);
    for (int64_t i = 0; i < nops; i++) {
        const op6 *o = &ops[i];
        if (o->res < 0 || o->res >= storage_count || o->src < 0 || o->src >= storage_count || o->src2 < 0 ||
            o->src2 >= storage_count || o->res2 < 0 || o->res2 >= storage_count)
            return -1;
        if (i > 0 && ops[i - 1].stage > o->stage) return -1;
    }
    if (n_input < 0 || n_input >= storage_count) return -1;
    double **blk = (double **)calloc((size_t)storage_count, sizeof(double *));
    int32_t *last = (int32_t *)calloc((size_t)storage_count, sizeof(int32_t));
    uint8_t *pin = (uint8_t *)calloc((size_t)storage_count, 1);
    int64_t *perm = (int64_t *)malloc(sizeof(int64_t) * (nops + 1));
    int64_t *heads = (int64_t *)malloc(sizeof(int64_t) * (nops + 1));
    int32_t *tbd = (int32_t *)malloc(sizeof(int32_t) * (2 * nops + 1));
    int64_t live = 0, top = 0, ret = 0;
    if (!blk || !last || !pin || !perm || !heads || !tbd) { ret = -2; goto out; }
    for (int64_t k = 0; k < nl; k++) if (lleaf[3 * k + 2] > 0 && lleaf[3 * k + 2] < storage_count) pin[lleaf[3 * k + 2]] = 1;
    for (int64_t k = 0; k < nu; k++) if (uleaf[3 * k + 2] > 0 && uleaf[3 * k + 2] < storage_count) pin[uleaf[3 * k + 2]] = 1;
    /* laststage: the last stage reading each block (BlockPlanner.cpp:355-371) */
    for (int64_t i = 0; i < nops; i++) {
        const op6 *o = &ops[i];
        if (o->src > 0 && last[o->src] < o->stage) last[o->src] = o->stage;
        if (o->src2 > 0 && last[o->src2] < o->stage) last[o->src2] = o->stage;
    }
    for (int32_t k = 0; k < n_input; k++) {
        if (!(blk[k + 1] = blk_new())) { ret = -2; goto out; }
        memcpy(blk[k + 1], input_tiles + (int64_t)k * TILE, sizeof(double) * TILE);
    }
    live = top = n_input;
    int64_t s0 = 0;
    while (s0 < nops) {
        int64_t s1 = s0;
        while (s1 < nops && ops[s1].stage == ops[s0].stage) s1++;
        const int64_t n = s1 - s0;
        for (int64_t k = 0; k < n; k++) perm[k] = ((int64_t)ops[s0 + k].res << 32) | k;
        qsort(perm, (size_t)n, sizeof(int64_t), cmp_i64);
        for (int64_t k = 0; k < n; k++) perm[k] = s0 + (perm[k] & 0xffffffffLL);
        int64_t nh = 0;
        for (int64_t k = 0; k < n; k++)
            if (k == 0 || ops[perm[k]].res != ops[perm[k - 1]].res) heads[nh++] = k;
        heads[nh] = n;
        /* lazy allocation of this stage's results (BlockPlanner.cpp:419-445) */
        for (int64_t k = 0; k < n; k++) {
            const op6 *o = &ops[perm[k]];
            if (o->res > 0 && !blk[o->res]) { if (!(blk[o->res] = blk_new())) { ret = -2; goto out; } live++; }
            if (o->op == OP_LU && o->res2 > 0 && !blk[o->res2]) {
                if (!(blk[o->res2] = blk_new())) { ret = -2; goto out; }
                live++;
            }
        }
        if (live > top) top = live;
#pragma omp parallel for schedule(dynamic)
        for (int64_t h = 0; h < nh; h++) {
            for (int64_t k = heads[h]; k < heads[h + 1]; k++) {
                const op6 *o = &ops[perm[k]];
                double *r = blk[o->res];
                const double *a = o->src > 0 ? blk[o->src] : NULL;
                const double *b2 = o->src2 > 0 ? blk[o->src2] : NULL;
                switch (o->op) {
                    case OP_LU: if (a) tile_lu(a, r, blk[o->res2]); break;
                    case OP_LOWERINV: if (a) tile_inv_lower(a, r); break;
                    case OP_UPPERINV: if (a) tile_inv_upper(a, r); break;
                    case OP_MUL: if (a && b2) tile_gemm(r, a, b2, 1.0); break;
                    case OP_MULNEG: if (a && b2) tile_gemm(r, a, b2, -1.0); break;
                    case OP_LLT: if (a) tile_llt(a, r); break;
                    case OP_MULT: if (a && b2) tile_mult(r, a, b2); break;
                    case OP_SUB: /* r = src2 - src; an absent (or freed) side counts as zero */
                        for (int e = 0; e < TILE; e++) {
                            double v = 0;
                            if (b2) v = b2[e];
                            if (a) v -= a[e];
                            r[e] = v;
                        }
                        break;
                    default: break;
                }
            }
        }
        /* free what this stage read for the last time (BlockPlanner.cpp:597-648) */
        int64_t nt = 0;
        for (int64_t i = s0; i < s1; i++) {
            const op6 *o = &ops[i];
            if (o->src > 0 && last[o->src] == o->stage && !pin[o->src]) tbd[nt++] = o->src;
            if (o->src2 > 0 && last[o->src2] == o->stage && !pin[o->src2]) tbd[nt++] = o->src2;
        }
        for (int64_t k = 0; k < nt; k++)
            if (blk[tbd[k]]) { free(blk[tbd[k]]); blk[tbd[k]] = NULL; live--; }
        s0 = s1;
    }
    {
        /* LL^T plan: U leaves = transposed L leaves */
        int32_t *ut = NULL;
        double **ext = blk;
        int32_t ext_count = storage_count;
        if (nu == 0) {
            ext_count = storage_count + (int32_t)nl;
            ext = (double **)calloc((size_t)ext_count, sizeof(double *));
            ut = (int32_t *)malloc(sizeof(int32_t) * 3 * (nl + 1));
            if (!ext || !ut) { free(ext == blk ? NULL : ext); free(ut); ret = -2; goto out; }
            memcpy(ext, blk, sizeof(double *) * storage_count);
            for (int64_t k = 0; k < nl; k++) {
                const double *src = blk[lleaf[3 * k + 2]];
                double *t = blk_new();
                if (!t) { ret = -2; break; }
                if (src)
                    for (int i = 0; i < B; i++)
                        for (int j = 0; j < B; j++) t[j * B + i] = src[i * B + j];
                ext[storage_count + k] = t;
                ut[3 * k] = lleaf[3 * k + 1];
                ut[3 * k + 1] = lleaf[3 * k];
                ut[3 * k + 2] = storage_count + (int32_t)k;
            }
            uleaf = ut;
            nu = nl;
        }
        const int R = block_rows;
        const int64_t nn = (int64_t)R * B;
        int64_t *lp = (int64_t *)calloc((size_t)R + 1, sizeof(int64_t));
        int64_t *up = (int64_t *)calloc((size_t)R + 1, sizeof(int64_t));
        int32_t *ldg = (int32_t *)calloc((size_t)R, sizeof(int32_t));
        int32_t *udg = (int32_t *)calloc((size_t)R, sizeof(int32_t));
        int64_t *li = (int64_t *)malloc(sizeof(int64_t) * (nl + 1));
        int64_t *ui = (int64_t *)malloc(sizeof(int64_t) * (nu + 1));
        int64_t *lf = (int64_t *)malloc(sizeof(int64_t) * (R + 1));
        int64_t *uf = (int64_t *)malloc(sizeof(int64_t) * (R + 1));
        if (ret == 0 && lp && up && ldg && udg && li && ui && lf && uf) {
            for (int64_t k = 0; k < nl; k++) if (lleaf[3 * k] != lleaf[3 * k + 1]) lp[lleaf[3 * k] + 1]++;
            for (int64_t k = 0; k < nu; k++) if (uleaf[3 * k] != uleaf[3 * k + 1]) up[uleaf[3 * k] + 1]++;
            for (int i = 0; i < R; i++) { lp[i + 1] += lp[i]; up[i + 1] += up[i]; }
            memcpy(lf, lp, sizeof(int64_t) * (R + 1));
            memcpy(uf, up, sizeof(int64_t) * (R + 1));
            for (int64_t k = 0; k < nl; k++) {
                if (lleaf[3 * k] == lleaf[3 * k + 1]) ldg[lleaf[3 * k]] = lleaf[3 * k + 2];
                else li[lf[lleaf[3 * k]]++] = k;
            }
            for (int64_t k = 0; k < nu; k++) {
                if (uleaf[3 * k] == uleaf[3 * k + 1]) udg[uleaf[3 * k]] = uleaf[3 * k + 2];
                else ui[uf[uleaf[3 * k]]++] = k;
            }
            int64_t nans = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : nans)
            for (int c = 0; c < nrhs; c++) {
                double *bb = (double *)malloc(sizeof(double) * nn);
                double *yy = (double *)calloc((size_t)nn, sizeof(double));
                double *xx = x_ext + (int64_t)c * nn;
                if (bb && yy) {
                    memcpy(bb, b_ext + (int64_t)c * nn, sizeof(double) * nn);
                    solve_ptrs(R, lp, li, ldg, lleaf, up, ui, udg, uleaf, ext, bb, yy, xx);
                    for (int64_t k = 0; k < nn; k++) if (isnan(xx[k])) nans++;
                } else {
                    nans += nn;
                }
                free(bb);
                free(yy);
            }
            ret = nans;
        } else if (ret == 0) {
            ret = -2;
        }
        free(lp); free(up); free(ldg); free(udg); free(li); free(ui); free(lf); free(uf);
        if (ext != blk) {
            for (int64_t k = 0; k < nl; k++) free(ext[storage_count + k]);
            free(ext);
            free(ut);
        }
    }
out:
    if (peak) *peak = top;
    if (blk) for (int32_t k = 0; k < storage_count; k++) free(blk[k]);
    free(blk); free(last); free(pin); free(perm); free(heads); free(tbd);
    return ret;
}
