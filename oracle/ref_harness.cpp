// Test infrastructure only: a harness around the REFERENCE solver, compiled
// from the reference's own sources by oracle/build_ref.sh into oracle/_ref/.
// It never ships and nothing on the product path links it.
//
// It drives the reference exactly as SOGLU::solveLU (solver.cpp:121-184) and
// SOGLU::decompose_solveLU (solver.cpp:50-119) do, calling the same public
// entry points in the same order, but keeps handles on the intermediate state
// so that tests can pin the oracle and the host planner:
//   perm.i32   final row/column permutation (GOrder::newOrder after sortInBlock)
//   dag.i32    fine op DAG after the last blockPlan: {op,src,src2,result,result2,stage}
//   lblk.i32 / ublk.i32   leaves of the L / U quadtrees: {bi,bj,blockid}
//   x.f64      solution returned in the original ordering (GOrder::reOrderResult)
//   tiles.f64  (optional, --tiles) dense 64x64 L/U tiles in lblk/ublk order
//   stats.txt  key=value summary incl. the reference's own phase timings
//
// usage: ref_solve A.mtx [b.mtx|-] OUTDIR [--tiles] [--threads N]
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <chrono>
#include <map>
#include <omp.h>

#include "operation.h"
#include "matrix.h"
#include "data.h"
#include "memutil.h"
#include "BlockPlanner.h"
#include "GPSOrder.h"
#include "config.h"
#include "mtx.h"
#include "solver.h"
#include "const.h"

using namespace SOGLU;

static double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

static void write_file(const std::string& path, const void* p, size_t bytes) {
    FILE* f = fopen(path.c_str(), "wb");
    if (!f) { perror(path.c_str()); exit(2); }
    if (bytes) fwrite(p, 1, bytes, f);
    fclose(f);
}

struct Leaf { int bi, bj, id; };

// Walk a quadtree (matrix.h:22-44) and collect its level-0 leaves with block
// coordinates; child index = 2*rowbit + colbit (matrix.cpp:41). Coordinates
// come from the span each node covers: the fine L/U trees assembled by
// matrixZoomUpdate (BlockPlanner.cpp:1316-1330) carry coarse `level` values
// on their upper nodes.
static void leaves(matrix* m, int bi, int bj, int span, std::vector<Leaf>& out) {
    if (m == NULL) return;
    if (m->level == 0) {
        if (m->blockindex > 0) out.push_back({bi, bj, (int)m->blockindex});
        return;
    }
    int h = span / 2;
    for (int q = 0; q < 4; q++)
        leaves(m->submatrix[q], bi + (q >> 1) * h, bj + (q & 1) * h, h, out);
}

// Dense copy of a reference tile (64 rows x BLOCKCOL stride), honouring the
// per-row 8-column detail masks (const.h:27-33): entries outside the mask are
// not part of the tile's value (MatrixStdDouble.cpp:161-190 zeroes them).
static void dense_tile(const double* t, double* out) {
    const uint16_t* det = (const uint16_t*)(t + DETAILOFFSET);
    for (int i = 0; i < 64; i++) {
        uint16_t m = det[DETAILSKIPSHORT * (i / 32) + i % 32];
        for (int j = 0; j < 64; j++)
            out[i * 64 + j] = (m & (1u << (j / 8))) ? t[i * BLOCKCOL + j] : 0.0;
    }
}

int main(int argc, char** argv) {
    if (argc < 4) {
        fprintf(stderr, "usage: %s A.mtx [b.mtx|-] OUTDIR [--tiles] [--threads N]\n", argv[0]);
        return 1;
    }
    std::string amtx = argv[1], bmtx = argv[2], outdir = argv[3];
    bool want_tiles = false;
    for (int i = 4; i < argc; i++) {
        if (!strcmp(argv[i], "--tiles")) want_tiles = true;
        else if (!strcmp(argv[i], "--threads") && i + 1 < argc) omp_set_num_threads(atoi(argv[++i]));
    }

    iniData();
    if (mtx::readMTX(amtx) == 0) { fprintf(stderr, "empty matrix\n"); return 3; }
    if (bmtx != "-") mtx::readArray(bmtx, mtx::mSize);
    else {  // missing right-hand side: all ones, as mtx::readArray does for absent entries
        mtx::b = (double*)memutil::getSmallMem(1, sizeof(double) * mtx::mSize);
        for (int i = 0; i < mtx::mSize; i++) mtx::b[i] = 1.0;
    }
    const int dim = mtx::mSize;
    const bool sym = mtx::symmetric;
    double t0 = now_s();

    // ---- solveLU set-up (solver.cpp:125-161) ----
    data::mSize = dim; data::mSize_out = dim; data::symmetric = sym;
    int vc = mtx::valcount;
    int cap = sym ? vc * 2 - dim : vc;
    if (cap < vc) cap = vc;
    data::indexi = (int*)memutil::getSmallMem(1, sizeof(int) * cap);
    data::indexj = (int*)memutil::getSmallMem(1, sizeof(int) * cap);
    data::vals = (double*)memutil::getSmallMem(1, sizeof(double) * cap);
    int ii = 0;
    for (int i = 0; i < vc; i++) {
        data::indexi[ii] = mtx::indexi[i]; data::indexj[ii] = mtx::indexj[i]; data::vals[ii] = mtx::vals[i]; ii++;
        if (sym && mtx::indexi[i] != mtx::indexj[i]) {
            data::indexi[ii] = mtx::indexj[i]; data::indexj[ii] = mtx::indexi[i]; data::vals[ii] = mtx::vals[i]; ii++;
        }
    }
    data::valcount = ii;
    config::set(dim);
    data::blockRows = config::blockRows;
    data::blockSize = config::blockSize;
    const int next = data::blockRows * data::blockSize;
    data::b = (double*)memutil::getSmallMem(1, next * sizeof(double));
    for (int i = 0; i < dim; i++) data::b[i] = mtx::b[i];
    for (int i = dim; i < next; i++) data::b[i] = 1;

    GOrder::Reorder();
    GOrder::sortInBlock();
    double t_reorder = now_s() - t0;
    std::vector<int> perm(GOrder::newOrder, GOrder::newOrder + dim);
    GOrder::clearmost();

    // ---- decompose_solveLU (solver.cpp:50-119) ----
    double tp0 = now_s();
    BlockPlanner::appendBlockStorage(NULL);
    data::PlanL2 = true;
    data::blockSize = config::blockSizeL2;
    data::blockRows = config::blockRowsL2;
    BlockPlanner::checkBlock();
    BlockPlanner::iniBlockStorage();
    int n = data::blockRows;
    int levels = __builtin_popcount(data::blockRows - 1);
    matrix* bl = memutil::newmatrix(0, n, levels);
    matrix* bu = memutil::newmatrix(0, n, levels);
    if (sym) BlockPlanner::blockMatrixLLT(data::blocks, bl, n, NULL);
    else BlockPlanner::blockMatrixLU(data::blocks, bl, bu, n, NULL, NULL);
    long coarse_ops_emitted = (long)data::graph.size();
    if (sym) BlockPlanner::blockPlan(bl, NULL); else BlockPlanner::blockPlan(bl, bu);
    long coarse_ops = (long)data::graph.size();
    data::PlanL2 = false;
    data::blockSize = BLOCK64;
    int levelall = __builtin_popcount(data::blockRows - 1);
    matrix* bl2 = memutil::newmatrix(0, data::blockRows, levelall);
    matrix* bu2 = memutil::newmatrix(0, data::blockRows, levelall);
    if (sym) BlockPlanner::copyOperatorL2(data::blocks, bl, NULL, bl2, bu2, n);
    else BlockPlanner::copyOperatorL2(data::blocks, bl, bu, bl2, bu2, n);
    memutil::freeAllSmallMem(0);
    long fine_ops_emitted = (long)data::graph.size();
    int storage_before_plan = data::storageCount;
    BlockPlanner::blockPlan(bl2, bu2);
    double t_plan = now_s() - tp0;

    // dump DAG (graph order = stage-sorted execution order)
    std::vector<int> dag;
    dag.reserve(data::graph.size() * 6);
    std::map<int, long> hist;
    int maxstage = 0;
    for (operation* o : data::graph) {
        dag.push_back((int)o->op); dag.push_back(o->src); dag.push_back(o->src2);
        dag.push_back(o->result); dag.push_back(o->result2); dag.push_back(o->stage);
        hist[(int)o->op]++;
        if (o->stage > maxstage) maxstage = o->stage;
    }
    std::vector<Leaf> L, U;
    leaves(bl2, 0, 0, data::blockRows, L);
    if (!sym) leaves(bu2, 0, 0, data::blockRows, U);

    long fine_ops = (long)data::graph.size();
    double tk0 = now_s();
    BlockPlanner::calculate();
    double t_kernel = now_s() - tk0;

    std::vector<double> tiles;
    if (want_tiles) {
        tiles.resize((L.size() + U.size()) * 4096);
        size_t k = 0;
        for (auto& lf : L) dense_tile(data::blockstorage[lf.id], &tiles[4096 * k++]);
        for (auto& lf : U) dense_tile(data::blockstorage[lf.id], &tiles[4096 * k++]);
    }
    data::clearOperations();
    double ts0 = now_s();
    BlockPlanner::solve(bl2, bu2, data::b, data::blockRows * data::blockSize);
    double t_solve = now_s() - ts0;
    double* x = GOrder::reOrderResult(data::x);
    double t_total = now_s() - t0;

    // residual in the original ordering (mtx.cpp:183-215)
    double maxres = mtx::checkResult(x);

    write_file(outdir + "/perm.i32", perm.data(), perm.size() * 4);
    write_file(outdir + "/dag.i32", dag.data(), dag.size() * 4);
    write_file(outdir + "/lblk.i32", L.data(), L.size() * sizeof(Leaf));
    write_file(outdir + "/ublk.i32", U.data(), U.size() * sizeof(Leaf));
    write_file(outdir + "/x.f64", x, sizeof(double) * dim);
    if (want_tiles) write_file(outdir + "/tiles.f64", tiles.data(), tiles.size() * 8);

    FILE* f = fopen((outdir + "/stats.txt").c_str(), "w");
    fprintf(f, "n=%d\nblock_rows=%d\nblock_rows_l2=%d\nblock_size_l2=%d\n", dim, config::blockRows,
            config::blockRowsL2, config::blockSizeL2);
    fprintf(f, "coarse_ops_emitted=%ld\ncoarse_ops=%ld\nfine_ops_emitted=%ld\nfine_ops=%ld\n", coarse_ops_emitted,
            coarse_ops, fine_ops_emitted, fine_ops);
    fprintf(f, "storage_count=%d\nstages=%d\nl_blocks=%zu\nu_blocks=%zu\n", storage_before_plan, maxstage, L.size(),
            U.size());
    const char* names[] = {"inv", "lu", "lowerInv", "upperInv", "sub", "add", "neg", "copy",
                           "mul", "mulneg", "llt", "mult", "noop"};
    for (auto& kv : hist) fprintf(f, "op_%s=%ld\n", names[kv.first], kv.second);
    fprintf(f, "threads=%d\nt_reorder=%.6f\nt_plan=%.6f\nt_kernel=%.6f\nt_solve=%.6f\nt_total=%.6f\nmax_resid=%.6e\n",
            omp_get_max_threads(), t_reorder, t_plan, t_kernel, t_solve, t_total, maxres);
    fclose(f);
    return 0;
}
