#include "tasks.h"

#include <algorithm>
#include <stdexcept>
#include <unordered_map>

namespace sog {

// Redundant ops become aliases (every block is written once, so equal inputs
// give equal values): a copy (sub with src = 0: res = src2) reads src2's tile,
// and a second lowerInv / upperInv of the same block reads the first one's
// result (the planner's two levels invert some diagonal blocks twice). Chains
// resolve to the first non-redundant block.
// Marks in skip the ops replaced by aliasing; readers of the other ops then
// read alias[src] (a view, not a copy of the op list).
static void alias_copies(const OpSeq& in, int32_t storage_count, std::vector<int32_t>& alias,
                         std::vector<char>& skip, int64_t& ncopies, int64_t& ndup) {
    alias.resize(storage_count);
    for (int32_t b = 0; b < storage_count; b++) alias[b] = b;
    ncopies = ndup = 0;
    auto find = [&](int32_t b) {
        int32_t r = b;
        while (alias[r] != r) r = alias[r];
        while (alias[b] != r) {
            const int32_t nx = alias[b];
            alias[b] = r;
            b = nx;
        }
        return r;
    };
    auto valid = [&](int32_t b) { return b > 0 && b < storage_count; };
    skip.assign(in.size(), 0);
    std::vector<int32_t> first_inv;  // (source root << 1 | upper) -> result, 0 = none yet
    for (int64_t i = 0; i < in.size(); i++) {
        const Op& o = in[i];
        if (o.op == OP_SUB && o.src == 0 && valid(o.src2) && valid(o.res) && alias[o.res] == o.res) {
            alias[o.res] = o.src2;
            skip[i] = 1;
            ncopies++;
        } else if ((o.op == OP_LOWERINV || o.op == OP_UPPERINV) && valid(o.src) && valid(o.res) &&
                   alias[o.res] == o.res) {
            if (first_inv.empty()) first_inv.assign(2 * (size_t)storage_count, 0);
            const size_t key = ((size_t)find(o.src) << 1) | (o.op == OP_UPPERINV ? 1 : 0);
            if (first_inv[key] == 0) {
                first_inv[key] = o.res;
            } else {
                alias[o.res] = first_inv[key];
                skip[i] = 1;
                ndup++;
            }
        }
    }
    for (int32_t b = 0; b < storage_count; b++) find(b);
}

TaskGraph build_tasks(const OpSeq& ops_in, int32_t storage_count, int32_t n_input,
                      const std::vector<int32_t>& outputs_in, int gemm_parts, bool fuse_subs, bool fuse_lu) {
    if (gemm_parts != 1 && gemm_parts != 4) throw std::runtime_error("gemm_parts must be 1 or 4");
    std::vector<int32_t> alias;
    int64_t ncopies = 0, ndup = 0;
    std::vector<char> skip;
    alias_copies(ops_in, storage_count, alias, skip, ncopies, ndup);
    const OpSeq& ops = ops_in;
    // an op that survives aliasing, with its sources read through the aliases
    auto view = [&](int64_t i) {
        Op q = ops[i];
        if (q.src > 0 && q.src < storage_count) q.src = alias[q.src];
        if (q.src2 > 0 && q.src2 < storage_count) q.src2 = alias[q.src2];
        return q;
    };
    std::vector<int32_t> outputs;
    outputs.reserve(outputs_in.size());
    for (int32_t id : outputs_in) outputs.push_back(id > 0 && id < storage_count ? alias[id] : id);
    const int64_t nops = ops.size();
    std::vector<int32_t> producer(storage_count, -1);  // block -> task
    std::vector<int32_t> readers(storage_count, 0);
    auto check_id = [&](int32_t id) {
        if (id < 0 || id >= storage_count) throw std::runtime_error("block id out of range in DAG");
    };
    // pass 1: one task per produced block (LU: per result pair). Products
    // keep their operand pairs in op order in flat arrays: counted here,
    // placed after the pass.
    struct T0 {
        uint8_t kind;
        int32_t out, out2, a, b, c = 0, out3 = 0;
        int32_t p0 = 0, np = 0;  // this task's range of fpa / fpb
        bool dead = false;
    };
    std::vector<T0> tl;
    tl.reserve(nops / 4 + 16);
    std::vector<int32_t> op_task(nops, -1);  // product op -> its task
    for (int64_t i = 0; i < nops; i++) {
        if (skip[i]) continue;
        const Op o = view(i);
        check_id(o.src); check_id(o.src2); check_id(o.res); check_id(o.res2);
        if ((o.res > 0 && alias[o.res] != o.res) || (o.res2 > 0 && alias[o.res2] != o.res2))
            throw std::runtime_error("block written by a copy and by another op");
        if (o.res <= 0) throw std::runtime_error("op without result");
        if (o.res <= n_input || (o.res2 > 0 && o.res2 <= n_input)) throw std::runtime_error("op writes an input block");
        if (o.src > 0) readers[o.src]++;
        if (o.src2 > 0) readers[o.src2]++;
        uint8_t k;
        switch (o.op) {
            case OP_MUL: case OP_MULNEG: case OP_MULT: k = K_GEMM; break;
            case OP_LU: k = K_LU; break;
            case OP_LLT: k = K_LLT; break;
            case OP_LOWERINV: k = K_LINV; break;
            case OP_UPPERINV: k = K_UINV; break;
            case OP_SUB: k = K_SUB; break;
            case OP_TRANSPOSE: k = K_TRANS; break;
            default: throw std::runtime_error("unsupported op kind " + std::to_string(o.op));
        }
        int32_t t = producer[o.res];
        if (t >= 0 && (k != K_GEMM || tl[t].kind != K_GEMM))
            throw std::runtime_error("block written by more than one non-accumulating op");
        if (t < 0) {
            t = (int32_t)tl.size();
            T0 x;
            x.kind = k;
            x.out = o.res;
            x.out2 = k == K_LU ? o.res2 : 0;
            x.a = k == K_SUB ? o.src2 : (k == K_GEMM ? 0 : o.src);
            x.b = k == K_SUB ? o.src : 0;
            tl.push_back(x);
            producer[o.res] = t;
            if (k == K_LU) {
                if (o.res2 <= 0 || producer[o.res2] >= 0) throw std::runtime_error("bad LU result pair");
                producer[o.res2] = t;
            }
        }
        if (k == K_GEMM) {
            if (o.src <= 0 || o.src2 <= 0) throw std::runtime_error("mul with absent operand");
            op_task[i] = t;
            tl[t].np++;
        }
    }
    int64_t npairs = 0;
    for (T0& x : tl) {
        x.p0 = (int32_t)npairs;
        npairs += x.np;
    }
    std::vector<int32_t> fpa(npairs), fpb(npairs);
    {
        std::vector<int32_t> fill(tl.size(), 0);
        for (int64_t i = 0; i < nops; i++) {
            const int32_t t = op_task[i];
            if (t < 0) continue;
            const Op o = view(i);
            const int32_t q = tl[t].p0 + fill[t]++;
            fpa[q] = o.src;
            const int32_t b = o.op == OP_MULT ? (o.src2 | PAIR_TRANS) : o.src2;
            fpb[q] = o.op == OP_MULNEG ? -b : b;
        }
    }
    // fuse  S = D - X  with  X = GEMM (X read only by S, not an output)
    std::vector<char> is_out(storage_count, 0);
    for (int32_t id : outputs) {
        check_id(id);
        is_out[id] = 1;
    }
    int64_t fused = 0;
    if (fuse_subs) {
        for (size_t s = 0; s < tl.size(); s++) {
            T0& S = tl[s];
            if (S.kind != K_SUB || S.b <= 0) continue;
            const int32_t x = S.b;
            const int32_t g = producer[x];
            if (g < 0 || tl[g].kind != K_GEMM || tl[g].a != 0 || readers[x] != 1 || is_out[x]) continue;
            T0& G = tl[g];
            for (int32_t q = G.p0; q < G.p0 + G.np; q++) fpb[q] = -fpb[q];
            G.a = S.a;  // initial tile D (0: none)
            producer[x] = -1;
            G.out = S.out;
            producer[S.out] = g;
            S.dead = true;
            fused++;
        }
    }
    // fuse  Y = L^-1  into the LU task producing L: the LU sweep on [A | I]
    // yields L^-1 with the same multipliers (LU task field b = Y)
    int64_t fused_inv = 0;
    for (size_t s = 0; s < tl.size(); s++) {
        T0& X = tl[s];
        if (X.dead || X.kind != K_LINV || X.a <= 0) continue;
        const int32_t t = producer[X.a];
        if (t < 0 || (tl[t].kind != K_LU && tl[t].kind != K_LLT) || tl[t].out != X.a || tl[t].b != 0) continue;
        tl[t].b = X.out;
        producer[X.out] = t;
        X.dead = true;
        fused_inv++;
    }
    // fuse  Y = U^-1  into the LU task producing U: the same sweep applies the
    // published pivot rows as column operations to the identity above the
    // diagonal (LU task field c = Y)
    for (size_t s = 0; s < tl.size(); s++) {
        T0& X = tl[s];
        if (X.dead || X.kind != K_UINV || X.a <= 0) continue;
        const int32_t t = producer[X.a];
        if (t < 0 || tl[t].kind != K_LU || tl[t].out2 != X.a || tl[t].c != 0) continue;
        tl[t].c = X.out;
        producer[X.out] = t;
        X.dead = true;
        fused_inv++;
    }
    // fuse  LU(S)  into the product writing S when S is read by nothing else:
    // the factorisation starts in the same CTA right after the product, with
    // no dependency hop (product result S stays in out; the LU's L moves to
    // out3, its U / L^-1 / U^-1 to out2 / b / c)
    int64_t fused_lu = 0;
    if (fuse_lu && gemm_parts == 1) {
        for (size_t s = 0; s < tl.size(); s++) {
            T0& X = tl[s];
            if (X.dead || (X.kind != K_LU && X.kind != K_LLT) || X.a <= 0) continue;
            const int32_t src = X.a;
            const int32_t t = producer[src];
            if (t < 0 || tl[t].kind != K_GEMM || tl[t].out != src || readers[src] != 1 || is_out[src]) continue;
            T0& G = tl[t];
            G.kind = X.kind == K_LU ? K_GEMM_LU : K_GEMM_LLT;
            G.out3 = X.out;
            G.out2 = X.out2;
            G.b = X.b;
            G.c = X.c;
            for (int32_t id : {X.out, X.out2, X.b, X.c})
                if (id > 0) producer[id] = (int32_t)t;
            X.dead = true;
            fused_lu++;
        }
    }
    // renumber live tasks
    std::vector<int32_t> newid(tl.size(), -1);
    TaskGraph g;
    g.storage_count = storage_count;
    g.fused_subs = fused;
    g.fused_inverses = fused_inv;
    g.fused_lu = fused_lu;
    g.aliased_copies = ncopies;
    g.aliased_inverses = ndup;
    g.alias = std::move(alias);
    for (size_t t = 0; t < tl.size(); t++)
        if (!tl[t].dead) newid[t] = g.ntasks++;
    g.pair_ptr.assign(g.ntasks + 1, 0);
    for (auto* v : {&g.out, &g.out2, &g.a, &g.b, &g.c, &g.out3}) v->reserve(g.ntasks);
    g.kind.reserve(g.ntasks);
    g.parts.reserve(g.ntasks);
    g.pair_a.reserve(npairs);
    g.pair_b.reserve(npairs);
    for (size_t t = 0; t < tl.size(); t++) {
        if (tl[t].dead) continue;
        const T0& x = tl[t];
        g.kind.push_back(x.kind);
        g.parts.push_back(x.kind == K_GEMM ? (uint8_t)gemm_parts : 1);
        g.out.push_back(x.out);
        g.out2.push_back(x.out2);
        g.a.push_back(x.a);
        g.b.push_back(x.b);
        g.c.push_back(x.c);
        g.out3.push_back(x.out3);
        g.pair_a.insert(g.pair_a.end(), fpa.begin() + x.p0, fpa.begin() + x.p0 + x.np);
        g.pair_b.insert(g.pair_b.end(), fpb.begin() + x.p0, fpb.begin() + x.p0 + x.np);
        g.pair_ptr[newid[t] + 1] = (int32_t)g.pair_a.size();
    }
    for (int32_t b = 0; b < storage_count; b++)
        if (producer[b] >= 0) producer[b] = newid[producer[b]];
    g.producer = producer;  // copied: the dependency pass below still reads it
    g.gemm_pairs = (int64_t)g.pair_a.size();
    // dependencies from each task's sources: per task its producer tasks
    // (sorted, unique) in one flat array
    auto prod_of = [&](int32_t t, int32_t src) -> int32_t {
        if (src <= 0 || src <= n_input) return -1;
        const int32_t pt = producer[src];
        if (pt < 0) throw std::runtime_error("read of a block that no op produces");
        if (pt == t) throw std::runtime_error("task reads its own result");
        return pt;
    };
    std::vector<int64_t> pptr(g.ntasks + 1, 0);
    for (int32_t t = 0; t < g.ntasks; t++)
        pptr[t + 1] = pptr[t] + 1 + (g.kind[t] == K_SUB ? 1 : 0) + 2 * (g.pair_ptr[t + 1] - g.pair_ptr[t]);
    std::vector<int32_t> preds(pptr[g.ntasks]);
    g.ndep.assign(g.ntasks, 0);
    // tasks are independent here: their predecessor lists in parallel (the
    // first malformed read found is reported after the loop)
    std::string bad;
    int32_t bad_task = -1;  // the smallest task with a malformed input (deterministic report)
#pragma omp parallel for schedule(dynamic, 4096)
    for (int32_t t = 0; t < g.ntasks; t++) {
        int32_t* p = preds.data() + pptr[t];
        int n = 0;
        try {
            auto add = [&](int32_t pt) {
                if (pt >= 0) p[n++] = pt;
            };
            add(prod_of(t, g.a[t]));
            if (g.kind[t] == K_SUB) add(prod_of(t, g.b[t]));
            for (int32_t q = g.pair_ptr[t]; q < g.pair_ptr[t + 1]; q++) {
                add(prod_of(t, g.pair_a[q]));
                add(prod_of(t, (g.pair_b[q] < 0 ? -g.pair_b[q] : g.pair_b[q]) & ~PAIR_TRANS));
            }
        } catch (const std::exception& e) {
#pragma omp critical(sog_tasks_bad)
            if (bad_task < 0 || t < bad_task) {
                bad = e.what();
                bad_task = t;
            }
            n = 0;
        }
        std::sort(p, p + n);
        n = (int)(std::unique(p, p + n) - p);
        g.ndep[t] = n;
    }
    if (!bad.empty()) throw std::runtime_error(bad);
    std::vector<int32_t> scount(g.ntasks + 1, 0);
    for (int32_t t = 0; t < g.ntasks; t++)
        for (int32_t i = 0; i < g.ndep[t]; i++) scount[preds[pptr[t] + i] + 1]++;
    g.succ_ptr.assign(g.ntasks + 1, 0);
    for (int32_t t = 0; t < g.ntasks; t++) g.succ_ptr[t + 1] = g.succ_ptr[t] + scount[t + 1];
    g.succ.resize(g.succ_ptr[g.ntasks]);
    std::vector<int32_t> sf(g.succ_ptr.begin(), g.succ_ptr.end() - 1);
    for (int32_t t = 0; t < g.ntasks; t++)
        for (int32_t i = 0; i < g.ndep[t]; i++) g.succ[sf[preds[pptr[t] + i]]++] = t;
    // topological order (Kahn); levels = longest path from a source
    std::vector<int32_t> indeg(g.ndep), order;
    order.reserve(g.ntasks);
    for (int32_t t = 0; t < g.ntasks; t++)
        if (indeg[t] == 0) order.push_back(t);
    g.level.assign(g.ntasks, 0);
    for (size_t h = 0; h < order.size(); h++) {
        const int32_t t = order[h];
        for (int32_t k = g.succ_ptr[t]; k < g.succ_ptr[t + 1]; k++) {
            const int32_t s = g.succ[k];
            g.level[s] = std::max(g.level[s], g.level[t] + 1);
            if (--indeg[s] == 0) order.push_back(s);
        }
    }
    if ((int32_t)order.size() != g.ntasks) throw std::runtime_error("cycle in the op DAG");
    for (int32_t t = 0; t < g.ntasks; t++) g.nlevels = std::max(g.nlevels, g.level[t] + 1);
    g.prio.assign(g.ntasks, 0);
    for (int32_t h = g.ntasks - 1; h >= 0; h--) {
        const int32_t t = order[h];
        for (int32_t k = g.succ_ptr[t]; k < g.succ_ptr[t + 1]; k++) g.prio[t] = std::max(g.prio[t], g.prio[g.succ[k]] + 1);
    }
    g.level_ptr.assign(g.nlevels + 1, 0);
    for (int32_t t = 0; t < g.ntasks; t++) g.level_ptr[g.level[t] + 1] += g.parts[t];
    for (int32_t l = 0; l < g.nlevels; l++) g.level_ptr[l + 1] += g.level_ptr[l];
    g.level_items.resize(g.level_ptr[g.nlevels]);
    std::vector<int32_t> lf(g.level_ptr.begin(), g.level_ptr.end() - 1);
    for (int32_t t = 0; t < g.ntasks; t++)
        for (int p = 0; p < g.parts[t]; p++) g.level_items[lf[g.level[t]]++] = (t << 4) | p;
    std::vector<int32_t> roots;
    for (int32_t t = 0; t < g.ntasks; t++)
        if (g.ndep[t] == 0) roots.push_back(t);
    std::stable_sort(roots.begin(), roots.end(), [&](int32_t x, int32_t y) { return g.prio[x] > g.prio[y]; });
    for (int32_t t : roots)
        for (int p = 0; p < g.parts[t]; p++) g.ready_items.push_back((t << 4) | p);
    for (int32_t t = 0; t < g.ntasks; t++) {
        g.total_items += g.parts[t];
        g.count[g.kind[t]]++;
    }
    return g;
}

void add_diag_inverses(OpSeq& ops, int32_t& storage_count, int block_rows, const std::vector<Leaf>& L,
                       const std::vector<Leaf>& U, std::vector<int32_t>& linv, std::vector<int32_t>& uinv) {
    // per source block the result of the last lowerInv / upperInv of it (0: none)
    std::vector<int32_t> have_l(storage_count, 0), have_u(storage_count, 0);
    for (int64_t i = 0; i < ops.size(); i++) {
        const Op& o = ops[i];
        if (o.src <= 0 || o.src >= storage_count) continue;
        if (o.op == OP_LOWERINV) have_l[o.src] = o.res;
        if (o.op == OP_UPPERINV) have_u[o.src] = o.res;
    }
    ops.extra.reserve(ops.extra.size() + L.size() + U.size());
    linv.assign(block_rows, 0);
    uinv.assign(block_rows, 0);
    int32_t seq = ops.last_seq();
    int32_t stage = ops.size() == 0 ? 1 : ops.last_stage() + 1;
    for (int side = 0; side < 2; side++) {
        const std::vector<Leaf>& lv = side == 0 ? L : U;
        auto& have = side == 0 ? have_l : have_u;
        auto& dst = side == 0 ? linv : uinv;
        for (const Leaf& lf : lv) {
            if (lf.bi != lf.bj) continue;
            if (lf.id > 0 && lf.id < (int32_t)have.size() && have[lf.id] != 0) {
                dst[lf.bi] = have[lf.id];
                continue;
            }
            const int32_t id = storage_count++;
            ops.extra.push_back({side == 0 ? OP_LOWERINV : OP_UPPERINV, lf.id, 0, id, 0, stage, ++seq, 0});
            dst[lf.bi] = id;
        }
    }
}

void add_transposed_leaves(OpSeq& ops, int32_t& storage_count, const std::vector<Leaf>& L,
                           std::vector<Leaf>& U) {
    U.clear();
    int32_t seq = ops.last_seq();
    const int32_t stage = ops.size() == 0 ? 1 : ops.last_stage() + 1;
    for (const Leaf& lf : L) {
        const int32_t id = storage_count++;
        ops.extra.push_back({OP_TRANSPOSE, lf.id, 0, id, 0, stage, ++seq, 0});
        U.push_back({lf.bj, lf.bi, id});
    }
    std::sort(U.begin(), U.end(), [](const Leaf& a, const Leaf& b) { return a.bi != b.bi ? a.bi < b.bi : a.bj < b.bj; });
}

// single-CTA task latencies on GB300 (us), enough to rank start times
static double task_cost(const TaskGraph& g, int32_t t, bool fp64) {
    const int np = g.pair_ptr[t + 1] - g.pair_ptr[t];
    switch (g.kind[t]) {
        case K_GEMM: return fp64 ? 5.0 + 20.0 * np / g.parts[t] : 2.5 + 1.0 * np;
        case K_GEMM_LU:
        case K_GEMM_LLT: return 2.5 + 1.0 * np + 18.0;
        case K_LU:
        case K_LLT: return fp64 ? 140.0 : 20.0;
        case K_LINV:
        case K_UINV: return fp64 ? 95.0 : 14.0;
        default: return fp64 ? 6.0 : 3.0;
    }
}
static constexpr double HOP_US = 2.4;

// earliest start of every task with unlimited CTAs (longest weighted path
// from a source)
static std::vector<double> estimate_start(const TaskGraph& g, bool fp64) {
    std::vector<double> est(g.ntasks, 0.0);
    // level_items lists every task's parts grouped by level: visiting part 0
    // of each visits the tasks level by level
    for (int32_t it : g.level_items) {
        if (it & 15) continue;
        const int32_t t = it >> 4;
        const double fin = est[t] + task_cost(g, t, fp64) + HOP_US;
        for (int32_t k = g.succ_ptr[t]; k < g.succ_ptr[t + 1]; k++) est[g.succ[k]] = std::max(est[g.succ[k]], fin);
    }
    return est;
}

std::vector<int32_t> static_order(const TaskGraph& g, bool fp64) {
    const std::vector<double> est = estimate_start(g, fp64);
    std::vector<int32_t> tasks(g.ntasks);
    for (int32_t t = 0; t < g.ntasks; t++) tasks[t] = t;
    std::stable_sort(tasks.begin(), tasks.end(), [&](int32_t a, int32_t b) {
        if (est[a] != est[b]) return est[a] < est[b];
        if (g.prio[a] != g.prio[b]) return g.prio[a] > g.prio[b];
        return a < b;
    });
    std::vector<int32_t> items;
    items.reserve(g.total_items);
    for (int32_t t : tasks)
        for (int p = 0; p < g.parts[t]; p++) items.push_back((t << 4) | p);
    return items;
}

void order_pairs_by_ready(TaskGraph& g, bool fp64) {
    const std::vector<double> est = estimate_start(g, fp64);
    auto ready = [&](int32_t block) {
        const int32_t t = block > 0 && block < (int32_t)g.producer.size() ? g.producer[block] : -1;
        return t < 0 ? -1.0 : est[t] + task_cost(g, t, fp64);
    };
#pragma omp parallel
    {
    std::vector<std::pair<double, int32_t>> key;
    std::vector<int32_t> pa, pb;
#pragma omp for schedule(dynamic, 4096)
    for (int32_t t = 0; t < g.ntasks; t++) {
        const int32_t p0 = g.pair_ptr[t], p1 = g.pair_ptr[t + 1];
        if ((g.kind[t] != K_GEMM && g.kind[t] != K_GEMM_LU && g.kind[t] != K_GEMM_LLT) || p1 - p0 < 2) continue;
        key.clear();
        for (int32_t p = p0; p < p1; p++) {
            const int32_t b = (g.pair_b[p] < 0 ? -g.pair_b[p] : g.pair_b[p]) & ~PAIR_TRANS;
            key.push_back({std::max(ready(g.pair_a[p]), ready(b)), p});
        }
        // stable insertion sort: a product has few pairs (at most ~50), and
        // this avoids a temporary buffer per task
        for (size_t i = 1; i < key.size(); i++) {
            const std::pair<double, int32_t> v = key[i];
            size_t j = i;
            while (j > 0 && v.first < key[j - 1].first) {
                key[j] = key[j - 1];
                j--;
            }
            key[j] = v;
        }
        pa.assign(g.pair_a.begin() + p0, g.pair_a.begin() + p1);
        pb.assign(g.pair_b.begin() + p0, g.pair_b.begin() + p1);
        for (int32_t i = 0; i < p1 - p0; i++) {
            g.pair_a[p0 + i] = pa[key[i].second - p0];
            g.pair_b[p0 + i] = pb[key[i].second - p0];
        }
    }
    }
}

void add_lookahead_products(OpSeq& ops, int32_t& storage_count, int block_rows, const std::vector<Leaf>& L,
                            const std::vector<Leaf>& U, const std::vector<int32_t>& linv,
                            const std::vector<int32_t>& uinv, int dist, std::vector<int32_t>& lla,
                            std::vector<int32_t>& ula) {
    lla.assign(block_rows, 0);
    ula.assign(block_rows, 0);
    int32_t seq = ops.last_seq();
    const int32_t stage = ops.size() == 0 ? 1 : ops.last_stage() + 1;
    for (const Leaf& lf : L)
        if (lf.bj == lf.bi - dist && linv[lf.bi] > 0) {
            const int32_t id = storage_count++;
            ops.extra.push_back({OP_MUL, linv[lf.bi], lf.id, id, 0, stage, ++seq, 0});
            lla[lf.bi] = id;
        }
    for (const Leaf& lf : U)
        if (lf.bj == lf.bi + dist && uinv[lf.bi] > 0) {
            const int32_t id = storage_count++;
            ops.extra.push_back({OP_MUL, uinv[lf.bi], lf.id, id, 0, stage, ++seq, 0});
            ula[lf.bi] = id;
        }
}

void forward_wait_lists(const TaskGraph& g, int block_rows, const std::vector<int32_t>& lptr,
                        const std::vector<int32_t>& lid, const std::vector<int32_t>& linv,
                        const std::vector<const std::vector<int32_t>*>& la, std::vector<int32_t>& ptr,
                        std::vector<int32_t>& list) {
    ptr.assign(block_rows + 1, 0);
    list.clear();
    std::vector<int32_t> row;
    auto add = [&](int32_t blk) {
        if (blk > 0 && blk < (int32_t)g.producer.size() && g.producer[blk] >= 0) row.push_back(g.producer[blk]);
    };
    for (int i = 0; i < block_rows; i++) {
        row.clear();
        for (int32_t q = lptr[i]; q < lptr[i + 1]; q++) add(lid[q]);
        add(linv[i]);
        for (const std::vector<int32_t>* v : la)
            if (!v->empty()) add((*v)[i]);
        std::sort(row.begin(), row.end());
        row.erase(std::unique(row.begin(), row.end()), row.end());
        list.insert(list.end(), row.begin(), row.end());
        ptr[i + 1] = (int32_t)list.size();
    }
}

}  // namespace sog
