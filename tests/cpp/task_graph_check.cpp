// Host-side invariants of the device task graph, checked without a GPU.
//
// For a few systems planned through the C ABI, the task graph is built the
// way each precision's system builds it (FP64: four-part products, no LU
// fusion; mixed: products merged with the LU of their result, pairs ordered by
// estimated producer finish) and checked against the plain graph:
//  - every task's dependency count equals the number of distinct tasks that
//    produce the blocks it reads, successors mirror predecessors, and the
//    levels form a topological order;
//  - the fused graph has exactly fused_lu fewer tasks, and each product+LU
//    task writes the same L, U, L^-1 and U^-1 blocks as the LU task it
//    absorbed, whose input block it produces and nothing else reads;
//  - reordering pairs by readiness permutes each product's pairs only;
//  - the static claim order lists every item once, predecessors first;
//  - look-ahead products Dinv_i * L_{i,i-d} (d = 1..3, and the U
//    counterparts) exist exactly for the leaves at that distance, and the
//    forward-wait list of each block row names, sorted and once, the task
//    that writes each non-input tile the row reads, and no other task.
// Prints "ok" and exits 0, or prints the first violation and exits 1.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <string>
#include <vector>

#include "api_internal.h"
#include "tasks.h"

using namespace sog;

static int g_fail = 0;
#define CHECK(cond, ...)                                  \
    do {                                                  \
        if (!(cond)) {                                    \
            std::printf("FAIL %s:%d: ", __FILE__, __LINE__); \
            std::printf(__VA_ARGS__);                     \
            std::printf("\n");                            \
            g_fail = 1;                                   \
            return;                                       \
        }                                                 \
    } while (0)

static int32_t pair_b_block(int32_t pb) { return (pb < 0 ? -pb : pb) & ~PAIR_TRANS; }

// dependency counts, successor lists and levels of one graph
static void check_structure(const TaskGraph& g, int32_t n_input, const char* name) {
    const int32_t nt = g.ntasks;
    CHECK((int32_t)g.kind.size() == nt && (int32_t)g.ndep.size() == nt, "%s: array sizes", name);
    std::vector<std::vector<int32_t>> preds(nt);
    auto add = [&](int32_t t, int32_t block) {
        if (block <= n_input) return;
        const int32_t p = g.producer[block];
        if (p >= 0) preds[t].push_back(p);
    };
    for (int32_t t = 0; t < nt; t++) {
        add(t, g.a[t]);
        if (g.kind[t] == K_SUB) add(t, g.b[t]);
        for (int32_t q = g.pair_ptr[t]; q < g.pair_ptr[t + 1]; q++) {
            add(t, g.pair_a[q]);
            add(t, pair_b_block(g.pair_b[q]));
        }
        std::sort(preds[t].begin(), preds[t].end());
        preds[t].erase(std::unique(preds[t].begin(), preds[t].end()), preds[t].end());
    }
    std::vector<int32_t> indeg(nt, 0);
    for (int32_t t = 0; t < nt; t++) {
        CHECK(g.ndep[t] == (int32_t)preds[t].size(), "%s: task %d has count %d, %zu producers", name, t, g.ndep[t],
              preds[t].size());
        for (int32_t p : preds[t]) {
            CHECK(g.level[p] < g.level[t], "%s: producer %d not at an earlier level than %d", name, p, t);
            bool found = false;
            for (int32_t k = g.succ_ptr[p]; k < g.succ_ptr[p + 1]; k++) found = found || g.succ[k] == t;
            CHECK(found, "%s: %d missing from the successors of %d", name, t, p);
        }
        for (int32_t k = g.succ_ptr[t]; k < g.succ_ptr[t + 1]; k++) indeg[g.succ[k]]++;
    }
    for (int32_t t = 0; t < nt; t++) CHECK(indeg[t] == g.ndep[t], "%s: successor lists disagree at %d", name, t);
}

// the static claim order: each item once, every producer before its consumers
static void check_order(const TaskGraph& g, bool fp64, const char* name) {
    const std::vector<int32_t> order = static_order(g, fp64);
    CHECK((int64_t)order.size() == g.total_items, "%s: order has %zu items of %lld", name, order.size(),
          (long long)g.total_items);
    std::vector<int32_t> first(g.ntasks, -1), seen(g.ntasks, 0);
    for (size_t i = 0; i < order.size(); i++) {
        const int32_t t = order[i] >> 4;
        CHECK(t >= 0 && t < g.ntasks, "%s: bad item", name);
        if (first[t] < 0) first[t] = (int32_t)i;
        seen[t]++;
    }
    for (int32_t t = 0; t < g.ntasks; t++) {
        CHECK(seen[t] == g.parts[t], "%s: task %d listed %d times for %d parts", name, t, seen[t], g.parts[t]);
        for (int32_t k = g.succ_ptr[t]; k < g.succ_ptr[t + 1]; k++)
            CHECK(first[t] < first[g.succ[k]], "%s: successor %d claimed before %d", name, g.succ[k], t);
    }
}

// a product's pairs as a sorted multiset (for "permuted only")
static std::vector<std::pair<int32_t, int32_t>> pairs_of(const TaskGraph& g, int32_t t) {
    std::vector<std::pair<int32_t, int32_t>> v;
    for (int32_t q = g.pair_ptr[t]; q < g.pair_ptr[t + 1]; q++) v.push_back({g.pair_a[q], g.pair_b[q]});
    std::sort(v.begin(), v.end());
    return v;
}

// blocks a task writes
static std::vector<int32_t> writes_of(const TaskGraph& g, int32_t t) {
    std::vector<int32_t> w = {g.out[t]};
    const uint8_t k = g.kind[t];
    if (k == K_LU || k == K_LLT || k == K_GEMM_LU || k == K_GEMM_LLT) {
        w.push_back(g.out2[t]);
        w.push_back(g.b[t]);
        w.push_back(g.c[t]);
    }
    if (k == K_GEMM_LU || k == K_GEMM_LLT) w.push_back(g.out3[t]);
    return w;
}

// look-ahead products and the forward substitution's wait lists (mixed graph)
static void check_lookahead(const char* name, const Plan& p) {
    constexpr int D = 3;
    OpSeq ops(p.ops.data(), (int64_t)p.ops.size());
    int32_t storage = p.storage_count;
    const int R = p.cfg.block_rows;
    std::vector<int32_t> linv, uinv, outputs;
    add_diag_inverses(ops, storage, R, p.L, p.U, linv, uinv);
    std::vector<int32_t> lla[D], ula[D];
    for (int d = 0; d < D; d++) {
        const size_t before = ops.extra.size();
        add_lookahead_products(ops, storage, R, p.L, p.U, linv, uinv, d + 1, lla[d], ula[d]);
        std::map<int32_t, Op> made;  // result block -> op
        for (size_t k = before; k < ops.extra.size(); k++) made[ops.extra[k].res] = ops.extra[k];
        std::vector<int32_t> lwant(R, 0), uwant(R, 0);
        for (const Leaf& lf : p.L)
            if (lf.bj == lf.bi - (d + 1)) lwant[lf.bi] = lf.id;
        for (const Leaf& lf : p.U)
            if (lf.bj == lf.bi + (d + 1)) uwant[lf.bi] = lf.id;
        for (int i = 0; i < R; i++) {
            CHECK((lla[d][i] > 0) == (lwant[i] > 0), "%s: row %d L look-ahead at %d", name, i, d + 1);
            CHECK((ula[d][i] > 0) == (uwant[i] > 0), "%s: row %d U look-ahead at %d", name, i, d + 1);
            if (lla[d][i] > 0) {
                const Op& o = made.at(lla[d][i]);
                CHECK(o.op == OP_MUL && o.src == linv[i] && o.src2 == lwant[i], "%s: L product of row %d", name, i);
            }
            if (ula[d][i] > 0) {
                const Op& o = made.at(ula[d][i]);
                CHECK(o.op == OP_MUL && o.src == uinv[i] && o.src2 == uwant[i], "%s: U product of row %d", name, i);
            }
        }
        CHECK(made.size() == (size_t)(std::count_if(lwant.begin(), lwant.end(), [](int32_t v) { return v > 0; }) +
                                      std::count_if(uwant.begin(), uwant.end(), [](int32_t v) { return v > 0; })),
              "%s: extra look-ahead products at %d", name, d + 1);
    }
    for (const Leaf& lf : p.L) outputs.push_back(lf.id);
    for (const Leaf& lf : p.U) outputs.push_back(lf.id);
    for (int32_t id : linv) outputs.push_back(id);
    for (int32_t id : uinv) outputs.push_back(id);
    for (int d = 0; d < D; d++)
        for (auto* v : {&lla[d], &ula[d]})
            for (int32_t id : *v)
                if (id > 0) outputs.push_back(id);
    const TaskGraph g = build_tasks(ops, storage, p.n_input, outputs, 1, true, true);
    // the substitution's view: aliased ids, off-diagonal L leaves by (row, column)
    std::vector<Leaf> loff;
    for (Leaf lf : p.L) {
        lf.id = g.alias[lf.id];
        if (lf.bj < lf.bi) loff.push_back(lf);
    }
    std::sort(loff.begin(), loff.end(), [](const Leaf& a, const Leaf& b) { return a.bi != b.bi ? a.bi < b.bi : a.bj < b.bj; });
    std::vector<int32_t> lptr(R + 1, 0), lid;
    for (const Leaf& lf : loff) { lptr[lf.bi + 1]++; lid.push_back(lf.id); }
    for (int i = 0; i < R; i++) lptr[i + 1] += lptr[i];
    for (int32_t& id : linv) if (id > 0) id = g.alias[id];
    std::vector<const std::vector<int32_t>*> las;
    for (int d = 0; d < D; d++) {
        for (int32_t& id : lla[d]) if (id > 0) id = g.alias[id];
        las.push_back(&lla[d]);
    }
    std::vector<int32_t> fptr, fw;
    forward_wait_lists(g, R, lptr, lid, linv, las, fptr, fw);
    CHECK((int)fptr.size() == R + 1 && fptr[R] == (int32_t)fw.size(), "%s: wait list offsets", name);
    for (int i = 0; i < R; i++) {
        std::vector<int32_t> tiles(lid.begin() + lptr[i], lid.begin() + lptr[i + 1]);
        tiles.push_back(linv[i]);
        for (int d = 0; d < D; d++) tiles.push_back(lla[d][i]);
        std::vector<int32_t> want;  // writers of the row's non-input tiles, from the tasks' own outputs
        for (int32_t b : tiles) {
            if (b <= p.n_input) continue;
            int32_t writer = -1;
            for (int32_t t = 0; t < g.ntasks && writer < 0; t++) {
                const std::vector<int32_t> w = writes_of(g, t);
                if (std::find(w.begin(), w.end(), b) != w.end()) writer = t;
            }
            CHECK(writer >= 0, "%s: row %d reads block %d that no task writes", name, i, b);
            want.push_back(writer);
        }
        std::sort(want.begin(), want.end());
        want.erase(std::unique(want.begin(), want.end()), want.end());
        const std::vector<int32_t> got(fw.begin() + fptr[i], fw.begin() + fptr[i + 1]);
        CHECK(got == want, "%s: row %d waits on %zu tasks, its tiles have %zu writers", name, i, got.size(),
              want.size());
    }
}

static void check_system(const char* name, int n, const std::vector<int32_t>& I, const std::vector<int32_t>& J,
                         const std::vector<double>& V) {
    sog_plan* plan = nullptr;
    if (sog_plan_build(n, (int64_t)I.size(), 0, I.data(), J.data(), V.data(), 0, &plan) != 0) {
        std::printf("FAIL %s: plan: %s\n", name, sog_last_error());
        g_fail = 1;
        return;
    }
    const Plan& p = plan->p;
    OpSeq ops(p.ops.data(), (int64_t)p.ops.size());
    int32_t storage = p.storage_count;
    std::vector<int32_t> linv, uinv, outputs;
    add_diag_inverses(ops, storage, p.cfg.block_rows, p.L, p.U, linv, uinv);
    for (const Leaf& lf : p.L) outputs.push_back(lf.id);
    for (const Leaf& lf : p.U) outputs.push_back(lf.id);
    for (int32_t id : linv) outputs.push_back(id);
    for (int32_t id : uinv) outputs.push_back(id);
    const TaskGraph plain = build_tasks(ops, storage, p.n_input, outputs, 1, true, false);
    const TaskGraph fp64 = build_tasks(ops, storage, p.n_input, outputs, 4, true, false);
    TaskGraph mixed = build_tasks(ops, storage, p.n_input, outputs, 1, true, true);
    const std::string nm(name);
    check_structure(plain, p.n_input, (nm + " plain").c_str());
    check_structure(fp64, p.n_input, (nm + " fp64").c_str());
    check_structure(mixed, p.n_input, (nm + " mixed").c_str());
    if (g_fail) return;
    CHECK(fp64.total_items == plain.total_items + 3 * plain.count[K_GEMM], "%s: four parts per FP64 product", name);
    // fusion: one task fewer per merged LU, and the same outputs
    CHECK(mixed.fused_lu > 0, "%s: no LU merged into a product", name);
    CHECK(mixed.ntasks == plain.ntasks - mixed.fused_lu, "%s: %d tasks, expected %d - %lld", name, mixed.ntasks,
          plain.ntasks, (long long)mixed.fused_lu);
    CHECK(mixed.count[K_GEMM_LU] + mixed.count[K_GEMM_LLT] == mixed.fused_lu, "%s: fused kinds", name);
    std::map<int32_t, int32_t> lu_by_out;  // L block -> LU task of the plain graph
    for (int32_t t = 0; t < plain.ntasks; t++)
        if (plain.kind[t] == K_LU) lu_by_out[plain.out[t]] = t;
    for (int32_t t = 0; t < mixed.ntasks; t++) {
        if (mixed.kind[t] != K_GEMM_LU) continue;
        auto it = lu_by_out.find(mixed.out3[t]);
        CHECK(it != lu_by_out.end(), "%s: merged task %d writes an L no LU wrote", name, t);
        const int32_t u = it->second;
        CHECK(plain.a[u] == mixed.out[t], "%s: merged task %d factors block %d, the LU read %d", name, t,
              mixed.out[t], plain.a[u]);
        CHECK(plain.out2[u] == mixed.out2[t] && plain.b[u] == mixed.b[t] && plain.c[u] == mixed.c[t],
              "%s: merged task %d outputs differ from its LU's", name, t);
    }
    // readiness order: pairs permuted within each product only
    std::vector<std::vector<std::pair<int32_t, int32_t>>> before(mixed.ntasks);
    for (int32_t t = 0; t < mixed.ntasks; t++) before[t] = pairs_of(mixed, t);
    order_pairs_by_ready(mixed, false);
    for (int32_t t = 0; t < mixed.ntasks; t++)
        CHECK(pairs_of(mixed, t) == before[t], "%s: pairs of task %d changed", name, t);
    check_order(plain, true, (nm + " plain").c_str());
    check_order(fp64, true, (nm + " fp64").c_str());
    check_order(mixed, false, (nm + " mixed").c_str());
    check_lookahead(name, p);
    sog_plan_destroy(plan);
}

static void lap3d(int side, std::vector<int32_t>& I, std::vector<int32_t>& J, std::vector<double>& V) {
    auto id = [&](int x, int y, int z) { return (x * side + y) * side + z; };
    for (int x = 0; x < side; x++)
        for (int y = 0; y < side; y++)
            for (int z = 0; z < side; z++) {
                const int i = id(x, y, z);
                I.push_back(i); J.push_back(i); V.push_back(6.01);
                const int nb[3] = {x + 1 < side ? id(x + 1, y, z) : -1, y + 1 < side ? id(x, y + 1, z) : -1,
                                   z + 1 < side ? id(x, y, z + 1) : -1};
                for (int k : nb)
                    if (k >= 0) {
                        I.push_back(i); J.push_back(k); V.push_back(-1.0);
                        I.push_back(k); J.push_back(i); V.push_back(-1.0);
                    }
            }
}

static void band(int n, unsigned seed, std::vector<int32_t>& I, std::vector<int32_t>& J, std::vector<double>& V) {
    std::srand(seed);
    const int hb = std::max(2, n / 50);
    for (int i = 0; i < n; i++) {
        I.push_back(i); J.push_back(i); V.push_back(100.0);
        const int k = 3 + std::rand() % 25;
        for (int t = 1; t < k; t++) {
            const int j = i + std::rand() % (2 * hb + 1) - hb;
            if (j < 0 || j >= n || j == i) continue;
            I.push_back(i); J.push_back(j); V.push_back(1.0);
        }
    }
}

int main() {
    {
        std::vector<int32_t> I, J; std::vector<double> V;
        lap3d(14, I, J, V);
        check_system("lap3d_14", 14 * 14 * 14, I, J, V);
    }
    {
        std::vector<int32_t> I, J; std::vector<double> V;
        band(9000, 7, I, J, V);
        check_system("band_9000", 9000, I, J, V);
    }
    if (g_fail) return 1;
    std::printf("ok\n");
    return 0;
}
