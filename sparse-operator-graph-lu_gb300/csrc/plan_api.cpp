// C-ABI of the host planner (no CUDA): sog_plan_* and sog_last_error.
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "api_internal.h"

namespace sog_internal {
thread_local std::string g_err;
int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}
}  // namespace sog_internal

using sog_internal::fail;

extern "C" {

const char* sog_last_error(void) { return sog_internal::g_err.c_str(); }
const char* sog_version(void) { return "soglu_gb300 0.1 sm_103a"; }

int sog_plan_build(int32_t n, int64_t nnz, int32_t symmetric, const int32_t* I, const int32_t* J, const double* V,
                   int32_t threads, sog_plan** out) {
    if (!out) return fail(SOG_EINVAL, "out is NULL");
    *out = nullptr;
    if (n <= 0 || nnz < 0 || (nnz > 0 && (!I || !J))) return fail(SOG_EINVAL, "bad dimension or triplet arrays");
    try {
        sog_plan* p = new sog_plan();
        p->p = sog::build_plan(n, nnz, symmetric != 0, I, J, V, threads);
        p->nnz = nnz;
        p->symmetric = symmetric != 0;
        *out = p;
        return SOG_OK;
    } catch (const std::bad_alloc&) {
        return fail(SOG_ENOMEM, "host allocation failed while planning");
    } catch (const std::exception& e) {
        return fail(SOG_EINVAL, e.what());
    }
}

int sog_plan_get_info(const sog_plan* plan, sog_plan_info* info) {
    if (!plan || !info) return fail(SOG_EINVAL, "NULL argument");
    const sog::Plan& p = plan->p;
    std::memset(info, 0, sizeof(*info));
    info->n = p.cfg.n;
    info->n_ext = p.cfg.n_ext();
    info->block_rows = p.cfg.block_rows;
    info->block_rows_l2 = p.cfg.block_rows_l2;
    info->block_size_l2 = p.cfg.block_size_l2;
    info->storage_count = p.storage_count;
    info->n_input = p.n_input;
    info->stages = p.stages;
    info->nops = (int64_t)p.ops.size();
    info->n_lleaf = (int64_t)p.L.size();
    info->n_uleaf = (int64_t)p.U.size();
    info->nnz = (int64_t)p.scatter_tile.size();
    for (const sog::Op& o : p.ops)
        if (o.op >= 0 && o.op < 13) info->op_count[o.op]++;
    info->coarse_ops = p.coarse_ops;
    info->fine_ops_emitted = p.fine_ops_emitted;
    info->t_order = p.t_order;
    info->t_plan = p.t_plan;
    return SOG_OK;
}

int sog_plan_export(const sog_plan* plan, int32_t* new_to_old, sog_op* ops, int32_t* lleaf, int32_t* uleaf) {
    if (!plan) return fail(SOG_EINVAL, "NULL plan");
    const sog::Plan& p = plan->p;
    if (new_to_old && !p.ord.new_to_old.empty())
        std::memcpy(new_to_old, p.ord.new_to_old.data(), sizeof(int32_t) * p.ord.new_to_old.size());
    if (ops)
        for (size_t i = 0; i < p.ops.size(); i++) {
            const sog::Op& o = p.ops[i];
            ops[i] = {o.op, o.src, o.src2, o.res, o.res2, o.stage};
        }
    if (lleaf) std::memcpy(lleaf, p.L.data(), sizeof(sog::Leaf) * p.L.size());
    if (uleaf) std::memcpy(uleaf, p.U.data(), sizeof(sog::Leaf) * p.U.size());
    return SOG_OK;
}

int sog_plan_input_tiles(const sog_plan* plan, const double* V, double* tiles) {
    if (!plan || !tiles) return fail(SOG_EINVAL, "NULL argument");
    if (plan->imported) return fail(SOG_ESTATE, "imported plan carries no triplet scatter");
    if (!V && !plan->p.scatter_tile.empty()) return fail(SOG_EINVAL, "NULL values");
    sog::scatter_tiles(plan->p, V, tiles);
    return SOG_OK;
}

int sog_plan_import(int32_t block_rows, int32_t storage_count, int32_t n_input, const sog_op* ops, int64_t nops,
                    const int32_t* lleaf, int64_t n_lleaf, const int32_t* uleaf, int64_t n_uleaf, sog_plan** out) {
    if (!out) return fail(SOG_EINVAL, "out is NULL");
    *out = nullptr;
    if (block_rows <= 0 || (block_rows & (block_rows - 1)) || storage_count <= 0 || n_input < 0 ||
        n_input >= storage_count || nops < 0 || (nops > 0 && !ops) || n_lleaf <= 0 || n_uleaf <= 0 || !lleaf ||
        !uleaf)
        return fail(SOG_EINVAL, "bad plan arguments");
    try {
        sog_plan* p = new sog_plan();
        sog::Plan& q = p->p;
        q.cfg.n = block_rows * 64;
        q.cfg.block_rows = block_rows;
        q.storage_count = storage_count;
        q.n_input = n_input;
        q.ops.resize(nops);
        int32_t maxst = 0;
        for (int64_t i = 0; i < nops; i++) {
            q.ops[i] = {ops[i].op, ops[i].src, ops[i].src2, ops[i].result, ops[i].result2, ops[i].stage,
                        (int32_t)i, 0};
            if (ops[i].stage > maxst) maxst = ops[i].stage;
        }
        q.stages = maxst;
        for (int64_t k = 0; k < n_lleaf; k++) q.L.push_back({lleaf[3 * k], lleaf[3 * k + 1], lleaf[3 * k + 2]});
        for (int64_t k = 0; k < n_uleaf; k++) q.U.push_back({uleaf[3 * k], uleaf[3 * k + 1], uleaf[3 * k + 2]});
        for (const auto* v : {&q.L, &q.U})
            for (const sog::Leaf& lf : *v)
                if (lf.bi < 0 || lf.bi >= block_rows || lf.bj < 0 || lf.bj >= block_rows || lf.id <= 0 ||
                    lf.id >= storage_count) {
                    delete p;
                    return fail(SOG_EINVAL, "leaf out of range");
                }
        q.ord.new_to_old.resize(q.cfg.n);
        q.ord.old_to_new.resize(q.cfg.n);
        for (int i = 0; i < q.cfg.n; i++) q.ord.new_to_old[i] = q.ord.old_to_new[i] = i;
        p->imported = true;
        *out = p;
        return SOG_OK;
    } catch (const std::exception& e) {
        return fail(SOG_EINVAL, e.what());
    }
}

int sog_plan_merge(const sog_plan* const* plans, int32_t count, sog_plan** out) {
    if (!out) return fail(SOG_EINVAL, "out is NULL");
    *out = nullptr;
    if (count <= 0 || !plans) return fail(SOG_EINVAL, "no plans to merge");
    std::vector<const sog::Plan*> ps;
    int64_t nnz = 0;
    for (int32_t k = 0; k < count; k++) {
        if (!plans[k]) return fail(SOG_EINVAL, "NULL plan in batch");
        if (plans[k]->imported) return fail(SOG_EINVAL, "imported plans carry no triplet scatter: cannot batch");
        ps.push_back(&plans[k]->p);
        nnz += plans[k]->nnz;
    }
    try {
        sog_plan* p = new sog_plan();
        p->p = sog::merge_plans(ps);
        p->nnz = nnz;
        *out = p;
        return SOG_OK;
    } catch (const std::bad_alloc&) {
        return fail(SOG_ENOMEM, "host allocation failed while merging plans");
    } catch (const std::exception& e) {
        return fail(SOG_EINVAL, e.what());
    }
}

int sog_plan_segments(const sog_plan* plan, int32_t* count, int32_t* n) {
    if (!plan || !count) return fail(SOG_EINVAL, "NULL argument");
    const sog::Plan& p = plan->p;
    *count = p.segs.empty() ? 1 : (int32_t)p.segs.size();
    if (n) {
        if (p.segs.empty()) n[0] = p.cfg.n;
        else
            for (size_t k = 0; k < p.segs.size(); k++) n[k] = p.segs[k].n;
    }
    return SOG_OK;
}

void sog_plan_destroy(sog_plan* plan) { delete plan; }

int sog_mtx_read(const char* path, int32_t use_cache, sog_mtx** out) {
    if (!path || !out) return fail(SOG_EINVAL, "NULL argument");
    *out = nullptr;
    try {
        sog_mtx* m = new sog_mtx();
        std::string err;
        bool cached = false;
        const bool ok = use_cache ? sog::read_mtx_cached(path, m->d, err, &cached) : sog::read_mtx(path, m->d, err);
        if (!ok) {
            delete m;
            return fail(SOG_EINVAL, err);
        }
        m->from_cache = cached;
        *out = m;
        return SOG_OK;
    } catch (const std::bad_alloc&) {
        return fail(SOG_ENOMEM, "host allocation failed while reading");
    }
}

int sog_mtx_info(const sog_mtx* m, int32_t* n, int64_t* nnz, int32_t* symmetric) {
    if (!m) return fail(SOG_EINVAL, "NULL matrix");
    if (n) *n = m->d.n;
    if (nnz) *nnz = (int64_t)m->d.I.size();
    if (symmetric) *symmetric = m->d.symmetric ? 1 : 0;
    return SOG_OK;
}

int sog_mtx_copy(const sog_mtx* m, int32_t* I, int32_t* J, double* V) {
    if (!m) return fail(SOG_EINVAL, "NULL matrix");
    const size_t k = m->d.I.size();
    if (I) std::memcpy(I, m->d.I.data(), 4 * k);
    if (J) std::memcpy(J, m->d.J.data(), 4 * k);
    if (V) std::memcpy(V, m->d.V.data(), 8 * k);
    return SOG_OK;
}

void sog_mtx_destroy(sog_mtx* m) { delete m; }

}  // extern "C"
