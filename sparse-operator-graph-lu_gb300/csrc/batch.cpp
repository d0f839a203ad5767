// Batch plans: the block-diagonal union of independent systems' plans.
//
// The reference factors one system per process (solver.cpp:121); a batch of
// independent systems is, to the executor, one block-diagonal system whose op
// DAG is the disjoint union of the systems' DAGs. Merging at the plan level
// keeps every system's ops, stages and leaves exactly as its own planner made
// them, so each system's arithmetic in a batch is the arithmetic it gets
// alone; only block ids and block rows are shifted.
#include <algorithm>
#include <limits>
#include <numeric>
#include <stdexcept>

#include "plan.h"

namespace sog {

Plan merge_plans(const std::vector<const Plan*>& ps) {
    if (ps.empty()) throw std::runtime_error("merge_plans: no plans");
    int64_t n_in = 0, n_other = 0, R = 0, n = 0, ntrip = 0, npad = 0, nops = 0;
    for (const Plan* p : ps) {
        if (!p) throw std::runtime_error("merge_plans: NULL plan");
        if (!p->segs.empty()) throw std::runtime_error("merge_plans: a batch plan cannot be merged again");
        if ((int64_t)p->ord.new_to_old.size() != p->cfg.n)
            throw std::runtime_error("merge_plans: plan has no ordering");
        n_in += p->n_input;
        n_other += p->storage_count - 1 - p->n_input;
        R += p->cfg.block_rows;
        n += p->cfg.n;
        ntrip += (int64_t)p->scatter_tile.size();
        npad += (int64_t)p->pad_tile.size();
        nops += (int64_t)p->ops.size();
    }
    const int64_t storage = 1 + n_in + n_other;
    if (storage > std::numeric_limits<int32_t>::max() || R * 64 > std::numeric_limits<int32_t>::max() ||
        n > std::numeric_limits<int32_t>::max())
        throw std::runtime_error("merge_plans: batch exceeds 32-bit block ids or rows");

    Plan m;
    m.cfg.n = (int)n;
    m.cfg.block_rows = (int)R;
    m.storage_count = (int32_t)storage;
    m.n_input = (int32_t)n_in;
    m.ops.reserve(nops);
    m.input_bi.reserve(n_in);
    m.input_bj.reserve(n_in);
    m.scatter_tile.reserve(ntrip);
    m.scatter_off.reserve(ntrip);
    m.pad_tile.reserve(npad);
    m.pad_off.reserve(npad);
    m.ord.new_to_old.assign(R * 64, -1);

    bool any_mirror = false;
    for (const Plan* p : ps) any_mirror = any_mirror || !p->mirror_src.empty();
    int32_t in_off = 0, other_off = (int32_t)n_in, row_blocks = 0;
    int64_t noff = 0, toff = 0, voff = 0;
    for (size_t k = 0; k < ps.size(); k++) {
        const Plan& p = *ps[k];
        const int32_t ni = p.n_input;
        // block id remap: inputs first, then the rest
        auto id = [&](int32_t b) -> int32_t {
            if (b <= 0) return b;
            return b <= ni ? in_off + b : other_off + (b - ni);
        };
        for (const Op& o : p.ops) {
            m.ops.push_back({o.op, id(o.src), id(o.src2), id(o.res), id(o.res2), o.stage, o.seq, o.group});
        }
        for (int32_t t = 0; t < ni; t++) {
            m.input_bi.push_back(p.input_bi[t] + row_blocks);
            m.input_bj.push_back(p.input_bj[t] + row_blocks);
        }
        for (const Leaf& lf : p.L) m.L.push_back({lf.bi + row_blocks, lf.bj + row_blocks, id(lf.id)});
        for (const Leaf& lf : p.U) m.U.push_back({lf.bi + row_blocks, lf.bj + row_blocks, id(lf.id)});
        for (size_t q = 0; q < p.scatter_tile.size(); q++) {
            const int32_t t = p.scatter_tile[q];
            m.scatter_tile.push_back(t < 0 ? t : t + in_off);
            m.scatter_off.push_back(p.scatter_off[q]);
        }
        if (any_mirror)
            for (size_t q = 0; q < p.scatter_tile.size(); q++)
                m.mirror_src.push_back((int32_t)(voff + (p.mirror_src.empty() ? (int64_t)q : p.mirror_src[q])));
        for (size_t q = 0; q < p.pad_tile.size(); q++) {
            m.pad_tile.push_back(p.pad_tile[q] + in_off);
            m.pad_off.push_back(p.pad_off[q]);
        }
        const int64_t row0 = (int64_t)row_blocks * 64;
        for (int i = 0; i < p.cfg.n; i++) m.ord.new_to_old[row0 + i] = p.ord.new_to_old[i];
        Segment sg;
        sg.row0 = (int32_t)row0;
        sg.n = p.cfg.n;
        sg.R = p.cfg.block_rows;
        sg.noff = noff;
        sg.trip_off = toff;
        sg.ntrip = (int64_t)p.scatter_tile.size();
        sg.symmetric = p.symmetric;
        m.segs.push_back(sg);
        m.stages = std::max(m.stages, p.stages);
        m.t_order += p.t_order;
        m.t_plan += p.t_plan;
        m.coarse_ops += p.coarse_ops;
        m.coarse_ops_emitted += p.coarse_ops_emitted;
        m.fine_ops_emitted += p.fine_ops_emitted;
        in_off += ni;
        other_off += p.storage_count - 1 - ni;
        row_blocks += p.cfg.block_rows;
        noff += p.cfg.n;
        toff += (int64_t)p.scatter_tile.size();
        voff += p.nval;
    }
    m.nval = voff;
    if (voff > std::numeric_limits<int32_t>::max()) throw std::runtime_error("merge_plans: too many values");
    // the executor contract: ops ascending by stage (stable, so each system's
    // own order is kept and systems follow one another within a stage)
    std::vector<int64_t> order(m.ops.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](int64_t a, int64_t b) { return m.ops[a].stage < m.ops[b].stage; });
    OpVec sorted;
    sorted.reserve(m.ops.size());
    for (int64_t i : order) sorted.push_back(m.ops[i]);
    m.ops.swap(sorted);
    return m;
}

}  // namespace sog
