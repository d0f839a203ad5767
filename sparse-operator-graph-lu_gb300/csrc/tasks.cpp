#include "tasks.h"

#include <algorithm>
#include <stdexcept>

namespace sog {

TaskGraph build_tasks(const std::vector<Op>& ops, int32_t storage_count, int32_t n_input, int gemm_parts) {
    if (gemm_parts != 1 && gemm_parts != 4) throw std::runtime_error("gemm_parts must be 1 or 4");
    TaskGraph g;
    g.storage_count = storage_count;
    const int64_t nops = (int64_t)ops.size();
    std::vector<int32_t> producer(storage_count, -1);  // block -> task
    std::vector<int64_t> first_write(storage_count, -1);
    auto check_id = [&](int32_t id) {
        if (id < 0 || id >= storage_count) throw std::runtime_error("block id out of range in DAG");
    };
    // pass 1: one task per produced block (LU: per result pair)
    std::vector<int32_t> op_task(nops);
    for (int64_t i = 0; i < nops; i++) {
        const Op& o = ops[i];
        check_id(o.src); check_id(o.src2); check_id(o.res); check_id(o.res2);
        if (o.res <= 0) throw std::runtime_error("op without result");
        if (o.res <= n_input || (o.res2 > 0 && o.res2 <= n_input))
            throw std::runtime_error("op writes an input block");
        uint8_t k;
        switch (o.op) {
            case OP_MUL: case OP_MULNEG: k = K_GEMM; break;
            case OP_LU: k = K_LU; break;
            case OP_LOWERINV: k = K_LINV; break;
            case OP_UPPERINV: k = K_UINV; break;
            case OP_SUB: k = K_SUB; break;
            default: throw std::runtime_error("unsupported op kind " + std::to_string(o.op));
        }
        int32_t t = producer[o.res];
        if (t >= 0) {
            if (k != K_GEMM || g.kind[t] != K_GEMM) throw std::runtime_error("block written by more than one non-accumulating op");
            op_task[i] = t;
            continue;
        }
        t = g.ntasks++;
        g.kind.push_back(k);
        g.parts.push_back(k == K_GEMM ? (uint8_t)gemm_parts : 1);
        g.out.push_back(o.res);
        g.out2.push_back(k == K_LU ? o.res2 : 0);
        if (k == K_SUB) { g.a.push_back(o.src2); g.b.push_back(o.src); }
        else if (k == K_GEMM) { g.a.push_back(0); g.b.push_back(0); }
        else { g.a.push_back(o.src); g.b.push_back(0); }
        producer[o.res] = t;
        first_write[o.res] = i;
        if (k == K_LU) {
            if (o.res2 <= 0 || producer[o.res2] >= 0) throw std::runtime_error("bad LU result pair");
            producer[o.res2] = t;
            first_write[o.res2] = i;
        }
        op_task[i] = t;
    }
    // pass 2: GEMM operand pairs in op order
    std::vector<int32_t> npairs(g.ntasks, 0);
    for (int64_t i = 0; i < nops; i++)
        if (g.kind[op_task[i]] == K_GEMM) npairs[op_task[i]]++;
    g.pair_ptr.assign(g.ntasks + 1, 0);
    for (int32_t t = 0; t < g.ntasks; t++) g.pair_ptr[t + 1] = g.pair_ptr[t] + npairs[t];
    g.pair_a.resize(g.pair_ptr[g.ntasks]);
    g.pair_b.resize(g.pair_ptr[g.ntasks]);
    std::vector<int32_t> fill(g.pair_ptr.begin(), g.pair_ptr.end() - 1);
    for (int64_t i = 0; i < nops; i++) {
        const Op& o = ops[i];
        int32_t t = op_task[i];
        if (g.kind[t] != K_GEMM) continue;
        if (o.src <= 0 || o.src2 <= 0) throw std::runtime_error("mul with absent operand");
        int32_t p = fill[t]++;
        g.pair_a[p] = o.src;
        g.pair_b[p] = o.op == OP_MULNEG ? -o.src2 : o.src2;
    }
    g.gemm_pairs = g.pair_ptr[g.ntasks];
    // pass 3: dependencies (read-after-write on produced blocks)
    std::vector<std::vector<int32_t>> preds(g.ntasks);
    for (int64_t i = 0; i < nops; i++) {
        const Op& o = ops[i];
        int32_t t = op_task[i];
        for (int32_t s : {o.src, o.src2}) {
            if (s <= 0) continue;
            if (s <= n_input) continue;
            int32_t pt = producer[s];
            if (pt < 0) throw std::runtime_error("read of a block that no op produces");
            if (first_write[s] > i) throw std::runtime_error("block read before it is written");
            if (pt == t) throw std::runtime_error("task reads its own result");
            preds[t].push_back(pt);
        }
    }
    g.ndep.assign(g.ntasks, 0);
    std::vector<int32_t> scount(g.ntasks + 1, 0);
    for (int32_t t = 0; t < g.ntasks; t++) {
        auto& p = preds[t];
        std::sort(p.begin(), p.end());
        p.erase(std::unique(p.begin(), p.end()), p.end());
        g.ndep[t] = (int32_t)p.size();
        for (int32_t q : p) scount[q + 1]++;
    }
    g.succ_ptr.assign(g.ntasks + 1, 0);
    for (int32_t t = 0; t < g.ntasks; t++) g.succ_ptr[t + 1] = g.succ_ptr[t] + scount[t + 1];
    g.succ.resize(g.succ_ptr[g.ntasks]);
    std::vector<int32_t> sf(g.succ_ptr.begin(), g.succ_ptr.end() - 1);
    for (int32_t t = 0; t < g.ntasks; t++)
        for (int32_t q : preds[t]) g.succ[sf[q]++] = t;
    // levels: tasks are created in op order, and producers precede readers
    g.level.assign(g.ntasks, 0);
    for (int32_t t = 0; t < g.ntasks; t++) {
        int32_t lv = 0;
        for (int32_t q : preds[t]) lv = std::max(lv, g.level[q] + 1);
        g.level[t] = lv;
        g.nlevels = std::max(g.nlevels, lv + 1);
    }
    // longest path to a sink, for the initial ready order
    std::vector<int32_t> height(g.ntasks, 0);
    for (int32_t t = g.ntasks - 1; t >= 0; t--)
        for (int32_t k = g.succ_ptr[t]; k < g.succ_ptr[t + 1]; k++)
            height[t] = std::max(height[t], height[g.succ[k]] + 1);
    g.level_ptr.assign(g.nlevels + 1, 0);
    for (int32_t t = 0; t < g.ntasks; t++) g.level_ptr[g.level[t] + 1] += g.parts[t];
    for (int32_t l = 0; l < g.nlevels; l++) g.level_ptr[l + 1] += g.level_ptr[l];
    g.level_items.resize(g.level_ptr[g.nlevels]);
    std::vector<int32_t> lf(g.level_ptr.begin(), g.level_ptr.end() - 1);
    for (int32_t t = 0; t < g.ntasks; t++)
        for (int p = 0; p < g.parts[t]; p++) g.level_items[lf[g.level[t]]++] = (t << 2) | p;
    std::vector<int32_t> roots;
    for (int32_t t = 0; t < g.ntasks; t++)
        if (g.ndep[t] == 0) roots.push_back(t);
    std::stable_sort(roots.begin(), roots.end(), [&](int32_t x, int32_t y) { return height[x] > height[y]; });
    for (int32_t t : roots)
        for (int p = 0; p < g.parts[t]; p++) g.ready_items.push_back((t << 2) | p);
    g.total_items = 0;
    for (int32_t t = 0; t < g.ntasks; t++) { g.total_items += g.parts[t]; g.count[g.kind[t]]++; }
    return g;
}

}  // namespace sog
