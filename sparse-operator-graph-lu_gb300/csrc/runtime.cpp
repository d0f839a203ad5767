// Host runtime of the GB300 executor: device context with a block-pool arena
// (the device counterpart of memutil's multi-level buffers, memutil.cpp:50-357),
// systems resident in the pool, and the factor / solve / refinement drivers
// behind the C ABI of include/soglu_gb300.h.
#include <cuda_runtime.h>

#include <parallel/algorithm>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "api_internal.h"
#include "kernels.h"
#include "tasks.h"

using sog_internal::fail;
using namespace sog;

#define CK(x)                                                                                   \
    do {                                                                                        \
        cudaError_t e_ = (x);                                                                   \
        if (e_ != cudaSuccess) return fail(SOG_ECUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)

namespace {

uint64_t round256(uint64_t b) { return (b + 255) & ~255ull; }

// Chunked first-fit arena over cudaMalloc'd chunks; freed ranges coalesce.
struct Pool {
    // systems of one context may run on several host threads (each on its own
    // stream), so the arena is locked
    std::mutex mu;
    struct Chunk {
        char* base;
        uint64_t size;
        std::map<uint64_t, uint64_t> free_;  // offset -> size
    };
    uint64_t cap = 0, reserved = 0, used = 0;
    std::vector<Chunk> chunks;

    void* alloc(uint64_t bytes) {
        std::lock_guard<std::mutex> lk(mu);
        bytes = round256(std::max<uint64_t>(bytes, 256));
        for (auto& c : chunks)
            for (auto it = c.free_.begin(); it != c.free_.end(); ++it)
                if (it->second >= bytes) {
                    uint64_t off = it->first, sz = it->second;
                    c.free_.erase(it);
                    if (sz > bytes) c.free_[off + bytes] = sz - bytes;
                    used += bytes;
                    return c.base + off;
                }
        const uint64_t step = 2ull << 20;
        uint64_t cs = std::max<uint64_t>(bytes, 1ull << 30);
        cs = (cs + step - 1) / step * step;
        if (reserved + cs > cap) cs = (bytes + step - 1) / step * step;
        if (reserved + cs > cap) return nullptr;
        char* p = nullptr;
        if (cudaMalloc(&p, cs) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        chunks.push_back({p, cs, {}});
        reserved += cs;
        if (cs > bytes) chunks.back().free_[bytes] = cs - bytes;
        used += bytes;
        return p;
    }
    void release(void* ptr, uint64_t bytes) {
        if (!ptr) return;
        std::lock_guard<std::mutex> lk(mu);
        bytes = round256(std::max<uint64_t>(bytes, 256));
        char* p = static_cast<char*>(ptr);
        for (auto& c : chunks) {
            if (p < c.base || p >= c.base + c.size) continue;
            uint64_t off = p - c.base;
            auto it = c.free_.emplace(off, bytes).first;
            auto nx = std::next(it);
            if (nx != c.free_.end() && it->first + it->second == nx->first) {
                it->second += nx->second;
                c.free_.erase(nx);
            }
            if (it != c.free_.begin()) {
                auto pv = std::prev(it);
                if (pv->first + pv->second == it->first) {
                    pv->second += it->second;
                    c.free_.erase(it);
                }
            }
            used -= bytes;
            return;
        }
    }
    // give chunks without allocations back to the device
    void trim() {
        std::lock_guard<std::mutex> lk(mu);
        std::vector<Chunk> keep;
        for (auto& c : chunks) {
            if (c.free_.size() == 1 && c.free_.begin()->first == 0 && c.free_.begin()->second == c.size) {
                cudaFree(c.base);
                reserved -= c.size;
            } else {
                keep.push_back(std::move(c));
            }
        }
        chunks.swap(keep);
    }
    void destroy() {
        std::lock_guard<std::mutex> lk(mu);
        for (auto& c : chunks) cudaFree(c.base);
        chunks.clear();
        reserved = used = 0;
    }
};

// offsets of sub-arrays inside one pool allocation
struct Layout {
    uint64_t off = 0;
    template <class T>
    uint64_t add(size_t count) {
        uint64_t o = off;
        off += round256(std::max<size_t>(count, 1) * sizeof(T));
        return o;
    }
};

}  // namespace

struct sog_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    int num_sms = 0;
    Pool pool;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
};

// id arrays of the substitution kept per system (six, then two per
// look-ahead distance)
constexpr int NSOL = 6 + 2 * SOLVE_LOOKAHEAD;

struct sog_system {
    sog_ctx* ctx = nullptr;
    // every kernel and copy of this system: the context's stream unless the
    // caller gave the system one of its own (sog_system_set_stream)
    cudaStream_t stream = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    sog_options opt{};
    bool fp64 = true, imported = false, symmetric = false;
    int n = 0, n_ext = 0, R = 0, n_input = 0;
    int32_t storage = 0;
    int64_t ntrip = 0, npad = 0;
    int64_t nval = 0;  // values the caller passes (its own triplets; mirrored inside when symmetric)
    TaskGraph tg;
    // pool allocations
    void* tiles = nullptr;
    uint64_t tiles_bytes = 0;
    char* aux = nullptr;
    uint64_t aux_bytes = 0;
    char* vecs = nullptr;
    uint64_t vec_bytes = 0;
    int vec_nrhs = 0;
    // device views
    DevTasks dt{};
    int32_t *d_ndep0 = nullptr, *d_parts0 = nullptr, *d_ready0 = nullptr, *d_counters0 = nullptr;
    bool early = false;     // mixed path, static order: products start before their last producer
    bool poisoned = false;  // a dependency count raised by the test hook (early start off)
    int32_t* d_level_items = nullptr;
    int nready = 0;
    DevStatus* d_status0 = nullptr;
    // pivot statistics per system: working copy, pristine copy, max |a_ij|
    DevPivot *d_piv = nullptr, *d_piv0 = nullptr;
    unsigned long long* d_amax = nullptr;
    bool amax_global = false;  // factored from tiles: one max over all input tiles
    struct PivotReport {
        double min_pivot = 0, growth = 0;
        int32_t clamped = 0, inv_fail = 0;
        bool tripped = false;
    };
    std::vector<PivotReport> piv;
    DevSolve ds{};
    DevCSR csr{};
    double* d_csr_val = nullptr;
    int32_t* d_csr_pos = nullptr;
    int32_t *d_sc_tile = nullptr, *d_pad_tile = nullptr;
    int16_t *d_sc_off = nullptr, *d_pad_off = nullptr;
    // systems of the plan (one for a plain plan; a batch plan's merged systems)
    std::vector<Segment> segs;
    int32_t *d_seg_brow = nullptr, *d_seg_n = nullptr, *d_n2o = nullptr;
    double* d_V = nullptr;
    int32_t* d_vidx = nullptr;  // symmetric: value index of each mirrored triplet (NULL = identity)
    // vectors (for up to vec_nrhs right-hand sides)
    double *d_bext = nullptr, *d_xext = nullptr, *d_r = nullptr, *d_red = nullptr;
    float* d_v32 = nullptr;
    unsigned long long* d_cnt = nullptr;  // per system
    int32_t *d_seg_nrhs = nullptr, *d_seg_active = nullptr;
    int64_t* d_seg_voff = nullptr;
    // pinned host mirrors: reductions (nseg x 64 x RED), per-system nrhs /
    // active / offsets / non-finite counts
    double* h_red = nullptr;
    int32_t *h_nrhs = nullptr, *h_active = nullptr;
    int64_t* h_voff = nullptr;
    unsigned long long* h_cnt = nullptr;
    std::vector<sog_solve_stats> seg_stats;
    int epoch = 2;
    // epoch of the forward pass that overlapped the last factorisation (its
    // backward pass takes fw_epoch + 1); reserved before that pass starts
    int fw_epoch = 0;
    bool factored = false;
    float t_factor = 0, t_solve = 0;
    int grid_factor = 0;
    int stages = 2;           // tensor-core operand stages of the mixed path
    bool tune_pending = false;  // time the candidate configurations at the next factorisation
    int64_t launches = 0;  // kernels launched by this system
    unsigned long long* trace = nullptr;  // optional timing trace (tasks, then block rows)
    uint64_t trace_bytes = 0;
    DevStatus last{};
    std::vector<Leaf> L, U;
    // resident compaction (sog_options.resident_compact): after a
    // factorisation only the tiles the substitution reads stay resident, in
    // their own allocation; the next factorisation allocates the full set again
    // host copies of l_id, u_id, l_diag, u_diag, l_dinv, u_dinv, then per
    // look-ahead distance d the pair l_la[d], u_la[d]
    std::vector<int32_t> sol_ids[NSOL];
    bool compacted = false;
    char* cbuf = nullptr;  // compact tiles (slot 0 unused), then the remapped id arrays
    uint64_t cbuf_bytes = 0;
    DevSolve ds_full{};
    std::vector<int32_t> cmap;  // block id -> compact slot while compacted
    // factor + solve with the forward pass overlapping the factorisation
    // (sog_factor_solve): per block row the factor tasks producing the tiles
    // the forward pass reads, and a second stream with its events
    int32_t *d_fwait_ptr = nullptr, *d_fwait = nullptr;
    cudaStream_t stream2 = nullptr;
    cudaEvent_t ev_ready = nullptr, ev_lower = nullptr;
};

namespace {

// Tuning memory: task graphs of about the same size and parallelism (tasks per
// dependency level) behave alike.
struct Tuned {
    int executor, stages;
    bool early;  // static order: products may start before their last producer
    bool sparse = true;  // FP64: skip MMAs of all-zero operand fragments
};
std::mutex g_tune_mu;
std::map<uint64_t, Tuned> g_tuned;
uint64_t tune_key(const TaskGraph& g, bool fp64) {
    const double par = (double)g.ntasks / std::max(1, g.nlevels);
    const uint64_t a = (uint64_t)std::lround(2.0 * std::log2(std::max(1.0, par)));
    const uint64_t b = (uint64_t)std::lround(2.0 * std::log2(std::max(1.0, (double)g.ntasks)));
    return (a << 32) | (b << 1) | (fp64 ? 1 : 0);
}
bool tuned_config(uint64_t key, Tuned& t) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tuned.find(key);
    if (it == g_tuned.end()) return false;
    t = it->second;
    return true;
}
void remember_config(uint64_t key, const Tuned& t) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tuned[key] = t;
}

sog_options default_options() {
    sog_options o;
    std::memset(&o, 0, sizeof(o));
    o.precision = SOG_FP64;
    o.executor = SOG_EXEC_PERSISTENT;
    o.max_refine = 10;
    o.tol = 1e-10;
    o.gemm_split = 0;
    return o;
}

DevStatus fresh_status() {
    DevStatus s;
    std::memset(&s, 0, sizeof(s));
    return s;
}

DevPivot fresh_pivot() {
    DevPivot p;
    std::memset(&p, 0, sizeof(p));
    double inf = INFINITY;
    std::memcpy(&p.min_pivot_bits, &inf, 8);
    return p;
}

// The pivot gate's growth limit: 0 = the default for the precision (FP32
// factors lose about growth x 6e-8 of relative accuracy, FP64 ones growth x
// 1.1e-16), < 0 = no gate (the reference's behaviour: clamp and continue).
double growth_limit(const sog_options& o) {
    if (o.growth_limit != 0) return o.growth_limit;
    return o.precision == SOG_FP64 ? 1e8 : 1e4;
}

double bits_to_double(unsigned long long b) {
    double d;
    std::memcpy(&d, &b, 8);
    return d;
}

uint64_t elem_bytes(const sog_options& o) { return o.precision == SOG_FP64 ? 8 : 4; }

// CSR of the permuted padded matrix from the plan's triplet scatter
struct HostCSR {
    std::vector<int32_t> ptr, col, pos;
    std::vector<double> val;  // padded diagonals preset to 1
};
HostCSR build_csr(const Plan& p) {
    HostCSR h;
    const int n_ext = p.cfg.n_ext();
    const int64_t nt = (int64_t)p.scatter_tile.size(), np_ = (int64_t)p.pad_tile.size();
    // (row * n_ext + col, triplet or -1 for a padded row's unit diagonal),
    // sorted by position: every position occurs once (superseded duplicates
    // have no tile), so the order is unique
    std::vector<std::pair<int64_t, int32_t>> e(nt + np_);
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < nt; k++) {
        const int32_t t = p.scatter_tile[k];
        if (t < 0) {
            e[k] = {INT64_MAX, -2};  // sorts last, dropped below
            continue;
        }
        const int64_t row = (int64_t)p.input_bi[t] * 64 + p.scatter_off[k] / 64;
        const int64_t col = (int64_t)p.input_bj[t] * 64 + p.scatter_off[k] % 64;
        e[k] = {row * n_ext + col, (int32_t)k};
    }
    for (int64_t q = 0; q < np_; q++) {
        const int64_t i = (int64_t)p.input_bi[p.pad_tile[q]] * 64 + p.pad_off[q] / 64;
        e[nt + q] = {i * n_ext + i, -1};
    }
    __gnu_parallel::sort(e.begin(), e.end());
    while (!e.empty() && e.back().second == -2) e.pop_back();
    h.ptr.assign(n_ext + 1, 0);
    h.col.resize(e.size());
    h.val.assign(e.size(), 0.0);
    h.pos.assign(nt, -1);
    for (size_t q = 0; q < e.size(); q++) {
        const int64_t kk = e[q].first;
        h.col[q] = (int32_t)(kk % n_ext);
        h.ptr[kk / n_ext + 1]++;
        if (e[q].second >= 0) h.pos[e[q].second] = (int32_t)q;
        else h.val[q] = 1.0;
    }
    for (int i = 0; i < n_ext; i++) h.ptr[i + 1] += h.ptr[i];
    return h;
}

int ensure_vectors(sog_system* s, int nrhs) {
    if (nrhs <= s->vec_nrhs) return SOG_OK;
    if (s->vecs) s->ctx->pool.release(s->vecs, s->vec_bytes);
    s->vecs = nullptr;
    s->vec_nrhs = 0;
    Layout L;
    const size_t ne = (size_t)s->n_ext * nrhs, ns = s->segs.size();
    uint64_t o_bext = L.add<double>(ne), o_xext = L.add<double>(ne), o_r = L.add<double>(ne),
             o_red = L.add<double>((size_t)RED * nrhs * ns), o_v32 = L.add<float>(ne),
             o_cnt = L.add<unsigned long long>(ns), o_nrhs = L.add<int32_t>(ns), o_act = L.add<int32_t>(ns),
             o_voff = L.add<int64_t>(ns);
    char* base = static_cast<char*>(s->ctx->pool.alloc(L.off));
    if (!base) return fail(SOG_ENOMEM, "block pool exhausted (solve vectors)");
    s->vecs = base;
    s->vec_bytes = L.off;
    s->vec_nrhs = nrhs;
    s->d_bext = (double*)(base + o_bext);
    s->d_xext = (double*)(base + o_xext);
    s->d_r = (double*)(base + o_r);
    s->d_red = (double*)(base + o_red);
    s->d_v32 = (float*)(base + o_v32);
    s->d_cnt = (unsigned long long*)(base + o_cnt);
    s->d_seg_nrhs = (int32_t*)(base + o_nrhs);
    s->d_seg_active = (int32_t*)(base + o_act);
    s->d_seg_voff = (int64_t*)(base + o_voff);
    return SOG_OK;
}

DevSegs seg_view(const sog_system* s) {
    DevSegs g;
    g.nseg = (int32_t)s->segs.size();
    g.of_brow = s->d_seg_brow;
    g.n2o = s->d_n2o;
    g.n = s->d_seg_n;
    g.nrhs = s->d_seg_nrhs;
    g.voff = s->d_seg_voff;
    g.active = s->d_seg_active;
    return g;
}

template <class T>
T* put(char* base, uint64_t off, const std::vector<T>& v, cudaStream_t st) {
    T* d = reinterpret_cast<T*>(base + off);
    if (!v.empty()) cudaMemcpyAsync(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st);
    return d;
}

int check_status(sog_system* s, bool factor) {
    sog_ctx* c = s->ctx;
    DevStatus st;
    CK(cudaMemcpy(&st, s->dt.status, sizeof(st), cudaMemcpyDeviceToHost));
    s->last = st;
    if (factor && (st.flags & ST_TIMEOUT)) return fail(SOG_ETIMEOUT, "factor: device queue wait expired");
    if (factor && (st.flags & ST_BAD_ITEM)) return fail(SOG_EINVAL, "factor: corrupt ready queue");
    if (!factor && (st.flags & ST_SOLVE_TIMEOUT)) return fail(SOG_ETIMEOUT, "solve: row readiness wait expired");
    (void)c;
    return SOG_OK;
}

// persistent factor grid: every co-resident CTA, or at most sog_options.max_ctas
// (a system sharing the GPU with others; the executors need no particular
// residency: the claimant of the smallest unfinished position always runs)
int factor_grid(const sog_system* s, int stages) {
    const int g = factor_persistent_grid(s->fp64, stages, s->ctx->num_sms);
    return s->opt.max_ctas > 0 ? std::min(g, s->opt.max_ctas) : g;
}

// working state of the factor kernels, reset from the pristine copies
int factor_reset(sog_system* s) {
    cudaStream_t st = s->stream;
    const TaskGraph& g = s->tg;
    CK(cudaMemcpyAsync(s->dt.dep, s->d_ndep0, sizeof(int32_t) * g.ntasks, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(s->dt.parts_left, s->d_parts0, sizeof(int32_t) * g.ntasks, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemsetAsync(s->dt.queue, 0xff, sizeof(int32_t) * g.total_items, st));
    if (s->nready)
        CK(cudaMemcpyAsync(s->dt.queue, s->d_ready0, sizeof(int32_t) * s->nready, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(s->dt.head, s->d_counters0, sizeof(int32_t) * 3, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(s->dt.status, s->d_status0, sizeof(DevStatus), cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(s->d_piv, s->d_piv0, sizeof(DevPivot) * s->segs.size(), cudaMemcpyDeviceToDevice, st));
    CK(cudaMemsetAsync(s->dt.task_done, 0, sizeof(int32_t) * g.ntasks, st));
    if (s->trace) CK(cudaMemsetAsync(s->trace, 0, sizeof(unsigned long long) * 4 * g.ntasks, st));
    return SOG_OK;
}

int run_factor_once(sog_system* s) {
    cudaStream_t st = s->stream;
    const TaskGraph& g = s->tg;
    if (int r = factor_reset(s)) return r;
    CK(cudaEventRecord(s->e0, st));
    int rc = 0;
    if (s->opt.executor == SOG_EXEC_LEVELS) {
        for (int l = 0; l < g.nlevels && rc == 0; l++) {
            const int a = g.level_ptr[l], b = g.level_ptr[l + 1];
            rc = s->fp64 ? factor_level_launch(s->dt, (double*)s->tiles, s->d_level_items + a, b - a, s->stages, st)
                         : factor_level_launch(s->dt, (float*)s->tiles, s->d_level_items + a, b - a, s->stages, st);
            s->launches++;
        }
    } else if (s->opt.executor == SOG_EXEC_QUEUE) {
        rc = s->fp64 ? factor_queue_launch(s->dt, (double*)s->tiles, s->grid_factor, s->stages, st)
                     : factor_queue_launch(s->dt, (float*)s->tiles, s->grid_factor, s->stages, st);
        s->launches++;
    } else {
        rc = s->fp64 ? factor_ordered_launch(s->dt, (double*)s->tiles, s->grid_factor, s->stages, st)
                     : factor_ordered_launch(s->dt, (float*)s->tiles, s->grid_factor, s->stages, st);
        s->launches++;
    }
    if (rc) return fail(SOG_ECUDA, std::string("factor launch: ") + cudaGetErrorString(cudaGetLastError()));
    CK(cudaEventRecord(s->e1, st));
    CK(cudaStreamSynchronize(st));
    CK(cudaEventElapsedTime(&s->t_factor, s->e0, s->e1));
    int r = check_status(s, true);
    if (r) return r;
    s->factored = true;
    return SOG_OK;
}

// Autotuning (SOG_EXEC_AUTO): the first factorisation of a system whose kind
// of task graph has not been seen runs every candidate configuration twice
// (the second run is timed) and keeps the fastest; the choice is remembered
// per key. Candidates: the static-order and the ready-queue executors, and for
// SOG_MIXED one operand stage where that lets two CTAs share an SM.
int run_factor(sog_system* s) {
    if (!s->tune_pending) return run_factor_once(s);
    s->tune_pending = false;
    std::vector<Tuned> cands = {{SOG_EXEC_PERSISTENT, 2, true}, {SOG_EXEC_QUEUE, 2, false}};
    const int sms = s->ctx->num_sms;
    if (s->fp64) cands.push_back({SOG_EXEC_PERSISTENT, 2, false, false});
    if (!s->fp64) {
        cands.push_back({SOG_EXEC_PERSISTENT, 2, false});
        if (factor_persistent_grid(false, 1, sms) > factor_persistent_grid(false, 2, sms))
            cands.push_back({SOG_EXEC_PERSISTENT, 1, false});
    }
    float best = 1e30f;
    Tuned pick = cands[0];
    for (const Tuned& c : cands) {
        s->opt.executor = c.executor;
        s->stages = c.stages;
        s->dt.early = !s->fp64 && c.early && !s->poisoned;
        s->dt.skip_zero = c.sparse;
        s->grid_factor = factor_grid(s, c.stages);
        for (int rep = 0; rep < 2; rep++) {
            const int r = run_factor_once(s);
            if (r) return r;
        }
        if (s->t_factor < best) {
            best = s->t_factor;
            pick = c;
        }
    }
    remember_config(tune_key(s->tg, s->fp64), pick);
    s->opt.executor = pick.executor;
    s->stages = pick.stages;
    s->early = pick.early;
    s->dt.early = !s->fp64 && pick.early && !s->poisoned;
    s->dt.skip_zero = pick.sparse;
    s->grid_factor = factor_grid(s, pick.stages);
    return run_factor_once(s);
}

// Pivot statistics of the last factorisation per system, and the gate: a
// system whose pivots were clamped, whose U U^-1 check failed, or whose growth
// (largest magnitude a diagonal-block factorisation saw / max |a_ij|)
// exceeded the limit makes the call return SOG_EPIVOT. The factors stay
// resident and can be used.
int check_pivots(sog_system* s) {
    const size_t ns = s->segs.size();
    std::vector<DevPivot> hp(ns);
    std::vector<unsigned long long> ha(ns);
    CK(cudaMemcpyAsync(hp.data(), s->d_piv, sizeof(DevPivot) * ns, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpyAsync(ha.data(), s->d_amax, sizeof(unsigned long long) * ns, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    const double lim = growth_limit(s->opt);
    s->piv.assign(ns, {});
    int bad = 0;
    for (size_t k = 0; k < ns; k++) {
        auto& pr = s->piv[k];
        pr.min_pivot = bits_to_double(hp[k].min_pivot_bits);
        if (std::isinf(pr.min_pivot)) pr.min_pivot = 0;  // no diagonal block factored
        pr.clamped = hp[k].clamped;
        pr.inv_fail = hp[k].inv_fail;
        const double mag = bits_to_double(hp[k].max_mag_bits);
        const double amax = bits_to_double(ha[s->amax_global ? 0 : k]);
        pr.growth = amax > 0 ? mag / amax : (mag > 0 ? INFINITY : 0.0);
        pr.tripped = lim > 0 && (pr.clamped > 0 || pr.inv_fail > 0 || !(pr.growth <= lim));
        bad += pr.tripped;
    }
    if (bad) {
        const auto& p0 = *std::find_if(s->piv.begin(), s->piv.end(), [](const sog_system::PivotReport& r) { return r.tripped; });
        return fail(SOG_EPIVOT, std::to_string(bad) + " system(s) failed the pivot check (first: " +
                                    std::to_string(p0.clamped) + " clamped pivots, " + std::to_string(p0.inv_fail) +
                                    " U*U^-1 check failures, growth " + std::to_string(p0.growth) + " vs limit " +
                                    std::to_string(lim) + "); the factors are resident");
    }
    return SOG_OK;
}

// Keep only the substitution's tiles (L/U leaves, diagonal inverses,
// look-ahead products): gathered into a compact allocation, the id arrays of
// the solve remapped, the full tile set returned to the pool. Without room
// for the compact copy the system simply stays as it is.
int compact_tiles(sog_system* s) {
    sog_ctx* c = s->ctx;
    const uint64_t tile = 4096 * elem_bytes(s->opt);
    std::vector<int32_t> need;
    for (auto& v : s->sol_ids)
        for (int32_t id : v)
            if (id > 0) need.push_back(id);
    for (const Leaf& lf : s->L) need.push_back(lf.id);
    for (const Leaf& lf : s->U) need.push_back(lf.id);
    std::sort(need.begin(), need.end());
    need.erase(std::unique(need.begin(), need.end()), need.end());
    std::vector<int32_t> cmap(s->storage, 0);
    for (size_t k = 0; k < need.size(); k++) cmap[need[k]] = (int32_t)k + 1;
    std::vector<int32_t> remap[NSOL];
    Layout Lc;
    const uint64_t o_t = Lc.add<char>((need.size() + 1) * tile), o_need = Lc.add<int32_t>(need.size());
    uint64_t o_ids[NSOL];
    for (int a = 0; a < NSOL; a++) {
        remap[a].resize(s->sol_ids[a].size());
        for (size_t k = 0; k < remap[a].size(); k++) remap[a][k] = s->sol_ids[a][k] > 0 ? cmap[s->sol_ids[a][k]] : 0;
        o_ids[a] = Lc.add<int32_t>(remap[a].size());
    }
    char* buf = static_cast<char*>(c->pool.alloc(Lc.off));
    if (!buf) return SOG_OK;
    cudaStream_t st = s->stream;
    int32_t* d_need = put(buf, o_need, need, st);
    s->launches++;
    gather_tiles_launch(s->tiles, buf + o_t, d_need, (int64_t)need.size(), tile, st);
    const int32_t* d_ids[NSOL];
    for (int a = 0; a < NSOL; a++) d_ids[a] = remap[a].empty() ? nullptr : put(buf, o_ids[a], remap[a], st);
    if (cudaStreamSynchronize(st) != cudaSuccess) {
        const std::string m = cudaGetErrorString(cudaGetLastError());
        c->pool.release(buf, Lc.off);
        return fail(SOG_ECUDA, "compaction: " + m);
    }
    c->pool.release(s->tiles, s->tiles_bytes);
    s->ds_full = s->ds;
    s->ds.l_id = d_ids[0];
    s->ds.u_id = d_ids[1];
    s->ds.l_diag = d_ids[2];
    s->ds.u_diag = d_ids[3];
    s->ds.l_dinv = d_ids[4];
    s->ds.u_dinv = d_ids[5];
    for (int d = 0; d < SOLVE_LOOKAHEAD; d++) {
        s->ds.l_la[d] = d_ids[6 + 2 * d];
        s->ds.u_la[d] = d_ids[7 + 2 * d];
    }
    s->tiles = buf + o_t;
    s->cbuf = buf;
    s->cbuf_bytes = Lc.off;
    s->cmap.swap(cmap);
    s->compacted = true;
    return SOG_OK;
}

// before a factorisation of a compacted system: the full tile set again
int uncompact_tiles(sog_system* s) {
    if (!s->compacted) return SOG_OK;
    sog_ctx* c = s->ctx;
    CK(cudaStreamSynchronize(s->stream));
    void* t = c->pool.alloc(s->tiles_bytes);
    if (!t) return fail(SOG_ENOMEM, "block pool exhausted (tiles for the refactorisation)");
    c->pool.release(s->cbuf, s->cbuf_bytes);
    s->cbuf = nullptr;
    s->cbuf_bytes = 0;
    s->tiles = t;
    s->ds = s->ds_full;
    s->cmap.clear();
    s->compacted = false;
    return SOG_OK;
}

int factor_checked(sog_system* s) {
    const int r = run_factor(s);
    if (r) return r;
    const int pr = check_pivots(s);
    if (pr && pr != SOG_EPIVOT) return pr;
    if (s->opt.resident_compact) {
        const int cr = compact_tiles(s);
        if (cr) return cr;
    }
    return pr;
}

void fill_pivot_stats(const sog_system* s, size_t k, sog_solve_stats& st) {
    if (k >= s->piv.size()) return;
    const auto& pr = s->piv[k];
    st.min_pivot = pr.min_pivot;
    st.clamped_pivots = pr.clamped;
    st.inv_check_failures = pr.inv_fail;
    st.max_growth = pr.growth;
}

int trisolve(sog_system* s, void* vec, int nrhs) {
    sog_ctx* c = s->ctx;
    const int nch = std::max(1, std::min(nrhs / 8, TRISOLVE_MAX_CHUNKS));  // positions per row
    int grid = std::min(s->R * nch, trisolve_grid(s->fp64, nrhs, c->num_sms));
    if (s->opt.max_ctas > 0) grid = std::min(grid, s->opt.max_ctas);
    int nl = 0;
    int rc = s->fp64 ? trisolve_launch(s->ds, (const double*)s->tiles, (double*)vec, nrhs, s->epoch, grid, s->stream, nl)
                     : trisolve_launch(s->ds, (const float*)s->tiles, (float*)vec, nrhs, s->epoch, grid, s->stream, nl);
    s->launches += nl;
    if (rc) return fail(SOG_ECUDA, std::string("solve launch: ") + cudaGetErrorString(cudaGetLastError()));
    return SOG_OK;
}

// the upper pass of a mixed solve whose lower pass ran overlapped with the
// factorisation (epoch s->fw_epoch; the upper pass takes s->fw_epoch + 1)
int trisolve_upper_only(sog_system* s, float* vec, int nrhs) {
    sog_ctx* c = s->ctx;
    const int nch = std::max(1, std::min(nrhs / 8, TRISOLVE_MAX_CHUNKS));
    int grid = std::min(s->R * nch, trisolve_grid(false, nrhs, c->num_sms));
    if (s->opt.max_ctas > 0) grid = std::min(grid, s->opt.max_ctas);
    const int rc = trisolve_upper_launch(s->ds, (const float*)s->tiles, vec, nrhs, s->fw_epoch + 1, grid, s->stream);
    s->launches++;
    if (rc) return fail(SOG_ECUDA, std::string("solve launch: ") + cudaGetErrorString(cudaGetLastError()));
    return SOG_OK;
}

// Per-system norms of this chunk's residual (columns [c0, c0+nc)), folded
// into the systems' statistics; rel[k] = worst relative residual of system k
// over the chunk's columns it has (0 if none).
int read_norms(sog_system* s, int c0, int nc, std::vector<double>& rel) {
    const size_t ns = s->segs.size();
    CK(cudaMemcpyAsync(s->h_red, s->d_red, sizeof(double) * RED * nc * ns, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    rel.assign(ns, 0.0);
    for (size_t k = 0; k < ns; k++) {
        sog_solve_stats& ss = s->seg_stats[k];
        ss.rel_resid = ss.backward_error = 0;  // the latest iterate's norms
        const int creal = std::min(nc, s->h_nrhs[k] - c0);
        for (int j = 0; j < creal; j++) {
            const double* r = s->h_red + ((size_t)k * nc + j) * RED;
            const double rl = r[1] > 0 ? std::sqrt(r[0]) / std::sqrt(r[1]) : std::sqrt(r[0]);
            const double den = r[5] * r[3] + r[4];
            const double bw = den > 0 ? r[2] / den : r[2];
            if (!(rl <= rel[k])) rel[k] = rl;  // NaN propagates
            if (!(bw <= ss.backward_error)) ss.backward_error = bw;
        }
        ss.rel_resid = rel[k];
    }
    return SOG_OK;
}

// One chunk of <= 64 right-hand-side columns [c0, c0+nc); b_ext already
// gathered into d_bext. Refinement (mixed) corrects only the systems that
// have not converged yet: the others' corrections are masked to zero, which
// leaves their iterates bit for bit unchanged.
// lower_done: the mixed path's first lower pass (of b cast to FP32 in
// d_v32) already ran, overlapped with the factorisation
int solve_chunk(sog_system* s, int c0, int nc, std::vector<sog_solve_stats>& chunk_stats, bool lower_done = false) {
    cudaStream_t st = s->stream;
    const int64_t ne = (int64_t)s->n_ext * nc;
    const size_t ns = s->segs.size();
    const DevSegs g = seg_view(s);
    int r;
    std::vector<double> rel;
    std::vector<int> iters(ns, 0);
    for (size_t k = 0; k < ns; k++) s->seg_stats[k].rel_resid = s->seg_stats[k].backward_error = 0;
    bool have_norms = false;
    if (s->fp64) {
        CK(cudaMemcpyAsync(s->d_xext, s->d_bext, sizeof(double) * ne, cudaMemcpyDeviceToDevice, st));
        if ((r = trisolve(s, s->d_xext, nc))) return r;
        if (s->csr.ptr) {
            s->launches++;
            residual_seg_launch(s->csr, s->d_bext, s->d_xext, s->d_r, c0, nc, s->d_red, g, st);
            if ((r = read_norms(s, c0, nc, rel))) return r;
            have_norms = true;
        }
    } else {
        if (lower_done) {
            if ((r = trisolve_upper_only(s, s->d_v32, nc))) return r;
        } else {
            s->launches++;
            cast_f64_to_f32_launch(s->d_bext, s->d_v32, ne, st);
            if ((r = trisolve(s, s->d_v32, nc))) return r;
        }
        s->launches++;
        axpy_f32_to_f64_launch(s->d_v32, s->d_xext, ne, 1, st);
        if (s->csr.ptr) {
            for (;;) {
                s->launches++;
                residual_seg_launch(s->csr, s->d_bext, s->d_xext, s->d_r, c0, nc, s->d_red, g, st);
                if ((r = read_norms(s, c0, nc, rel))) return r;
                have_norms = true;
                bool any = false;
                for (size_t k = 0; k < ns; k++) {
                    const bool act = !(rel[k] <= s->opt.tol) && !std::isnan(rel[k]) && iters[k] < s->opt.max_refine;
                    s->h_active[k] = act ? 1 : 0;
                    any = any || act;
                }
                if (!any) break;
                CK(cudaMemcpyAsync(s->d_seg_active, s->h_active, sizeof(int32_t) * ns, cudaMemcpyHostToDevice, st));
                s->launches++;
                cast_seg_launch(s->d_r, s->d_v32, s->n_ext, nc, g, st);
                if ((r = trisolve(s, s->d_v32, nc))) return r;
                s->launches++;
                axpy_f32_to_f64_launch(s->d_v32, s->d_xext, ne, 0, st);
                for (size_t k = 0; k < ns; k++) iters[k] += s->h_active[k];
            }
        }
    }
    if ((r = check_status(s, false))) return r;
    for (size_t k = 0; k < ns; k++) {
        if (c0 >= s->h_nrhs[k]) continue;
        sog_solve_stats& cs = chunk_stats[k];
        const sog_solve_stats& ss = s->seg_stats[k];
        cs.iterations = std::max(cs.iterations, iters[k]);
        if (have_norms) {
            if (!(ss.rel_resid <= cs.rel_resid)) cs.rel_resid = ss.rel_resid;
            if (!(ss.backward_error <= cs.backward_error)) cs.backward_error = ss.backward_error;
            if (!s->fp64 && !(ss.rel_resid <= s->opt.tol)) cs.status = SOG_ENOCONV;
        }
    }
    return SOG_OK;
}

// Solve for nrhs[k] right-hand sides of each system k (caller layout: per
// system nrhs[k] x n_k, rhs-major, concatenated). Per-system statistics go to
// s->seg_stats; agg (if not NULL) gets the worst over systems.
int solve_device_impl(sog_system* s, const int32_t* nrhs, const double* b_dev, double* x_dev,
                      sog_solve_stats* agg, bool lower_done = false) {
    cudaStream_t st = s->stream;
    const size_t ns = s->segs.size();
    int maxr = 0;
    int64_t off = 0;
    for (size_t k = 0; k < ns; k++) {
        if (nrhs[k] < 0) return fail(SOG_EINVAL, "negative right-hand-side count");
        s->h_nrhs[k] = nrhs[k];
        s->h_voff[k] = off;
        off += (int64_t)nrhs[k] * s->segs[k].n;
        maxr = std::max(maxr, nrhs[k]);
    }
    sog_solve_stats base;
    std::memset(&base, 0, sizeof(base));
    std::vector<sog_solve_stats> out(ns, base);
    for (size_t k = 0; k < ns; k++) fill_pivot_stats(s, k, out[k]);
    // the aggregate carries the worst system's pivot figures
    for (size_t k = 0; k < ns; k++) {
        if (k == 0 || out[k].min_pivot < base.min_pivot) base.min_pivot = out[k].min_pivot;
        base.clamped_pivots += out[k].clamped_pivots;
        base.inv_check_failures += out[k].inv_check_failures;
        if (!(out[k].max_growth <= base.max_growth)) base.max_growth = out[k].max_growth;
    }
    s->seg_stats = out;
    if (agg) *agg = base;
    if (maxr == 0) return SOG_OK;
    int r = ensure_vectors(s, std::min(maxr, 64));
    if (r) return r;
    CK(cudaMemcpyAsync(s->d_seg_nrhs, s->h_nrhs, sizeof(int32_t) * ns, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(s->d_seg_voff, s->h_voff, sizeof(int64_t) * ns, cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(s->d_cnt, 0, sizeof(unsigned long long) * ns, st));
    const DevSegs g = seg_view(s);
    // solve time from here (lower_done: from the factorisation's end, set by
    // the caller, so that waiting for the overlapped forward pass counts)
    if (!lower_done) CK(cudaEventRecord(s->e0, st));
    for (int c0 = 0; c0 < maxr; c0 += 64) {
        const int nc = std::min(64, maxr - c0);
        const bool pre = lower_done && c0 == 0;  // gathered, cast and forward-solved already
        if (!pre) {
            s->launches++;
            gather_seg_launch(b_dev, g, s->n_ext, c0, nc, s->d_bext, st);
        }
        r = solve_chunk(s, c0, nc, out, pre);
        if (r) return r;
        s->launches++;
        scatter_seg_launch(s->d_xext, g, s->n_ext, c0, nc, x_dev, s->d_cnt, st);
    }
    CK(cudaEventRecord(s->e1, st));
    CK(cudaMemcpyAsync(s->h_cnt, s->d_cnt, sizeof(unsigned long long) * ns, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    CK(cudaEventElapsedTime(&s->t_solve, s->e0, s->e1));
    int worst = SOG_OK;
    for (size_t k = 0; k < ns; k++) {
        out[k].nan_count = (int64_t)s->h_cnt[k];
        if (out[k].nan_count) out[k].status = SOG_ENAN;
        if (out[k].status == SOG_ENAN) worst = SOG_ENAN;
        else if (out[k].status && !worst) worst = out[k].status;
        if (agg) {
            agg->iterations = std::max(agg->iterations, out[k].iterations);
            if (!(out[k].rel_resid <= agg->rel_resid)) agg->rel_resid = out[k].rel_resid;
            if (!(out[k].backward_error <= agg->backward_error)) agg->backward_error = out[k].backward_error;
            agg->nan_count += out[k].nan_count;
        }
    }
    s->seg_stats = out;
    if (agg) agg->status = worst;
    if (worst == SOG_ENAN) return fail(SOG_ENAN, "non-finite values in the solution");
    if (worst) return fail(worst, "iterative refinement did not reach the tolerance");
    return SOG_OK;
}

int64_t solve_values(const sog_system* s, const int32_t* nrhs) {
    int64_t t = 0;
    for (size_t k = 0; k < s->segs.size(); k++) t += (int64_t)nrhs[k] * s->segs[k].n;
    return t;
}

// host b / x through pool staging buffers
int solve_host(sog_system* s, const int32_t* nrhs, const double* b, double* x, sog_solve_stats* agg) {
    sog_ctx* c = s->ctx;
    const uint64_t bytes = sizeof(double) * (uint64_t)solve_values(s, nrhs);
    if (bytes == 0) return solve_device_impl(s, nrhs, nullptr, nullptr, agg);
    double* db = static_cast<double*>(c->pool.alloc(bytes));
    double* dx = static_cast<double*>(c->pool.alloc(bytes));
    if (!db || !dx) {
        c->pool.release(db, bytes);
        c->pool.release(dx, bytes);
        return fail(SOG_ENOMEM, "block pool exhausted (rhs)");
    }
    int r = SOG_OK;
    if (cudaMemcpyAsync(db, b, bytes, cudaMemcpyHostToDevice, s->stream) != cudaSuccess)
        r = fail(SOG_ECUDA, "rhs upload failed");
    if (!r) {
        r = solve_device_impl(s, nrhs, db, dx, agg);
        if (!r || r == SOG_ENOCONV || r == SOG_ENAN) {
            if (cudaMemcpyAsync(x, dx, bytes, cudaMemcpyDeviceToHost, s->stream) != cudaSuccess ||
                cudaStreamSynchronize(s->stream) != cudaSuccess)
                r = fail(SOG_ECUDA, "download failed");
        }
    }
    c->pool.release(db, bytes);
    c->pool.release(dx, bytes);
    return r;
}

// factor inputs from device values: input tiles, the CSR values of the
// residual, max |a_ij| per system
int factor_inputs(sog_system* s, const double* V_dev) {
    if (int r = uncompact_tiles(s)) return r;
    cudaStream_t st = s->stream;
    const uint64_t eb = elem_bytes(s->opt);
    CK(cudaMemsetAsync((char*)s->tiles + 4096 * eb, 0, (uint64_t)s->n_input * 4096 * eb, st));
    // input tile k (0-based, as the scatter map counts) is block id k+1
    s->launches++;
    scatter_values_launch(V_dev, s->d_vidx, s->d_sc_tile, s->d_sc_off, s->ntrip, s->d_pad_tile, s->d_pad_off, s->npad,
                          s->fp64 ? (double*)s->tiles + 4096 : nullptr, s->fp64 ? nullptr : (float*)s->tiles + 4096,
                          st);
    s->launches++;
    scatter_csr_launch(V_dev, s->d_vidx, s->d_csr_pos, s->ntrip, s->d_csr_val, st);
    CK(cudaMemsetAsync(s->d_amax, 0, sizeof(unsigned long long) * s->segs.size(), st));
    s->launches++;
    csr_absmax_seg_launch(s->csr, seg_view(s), s->d_amax, st);
    s->amax_global = false;
    return SOG_OK;
}

// CTAs of the forward pass that overlaps the factorisation, and the SMs the
// factor leaves it (the factor's persistent CTAs fill an SM each); once the
// factor has finished, a launch on the whole GPU takes over the positions
// that pass has not reached
constexpr int OVERLAP_SOLVE_CTAS = 8;
constexpr int OVERLAP_SOLVE_SMS = 4;

// Factor, then solve nrhs right-hand sides (device b, x): the same results as
// sog_factor_device followed by sog_solve_device. A plain mixed system with
// look-ahead products, factored by the static-order executor (tuned, not
// compacted) and nrhs = 1 or a multiple of 8 up to 64, runs the first
// forward pass on a second stream while the factor kernel runs: each block
// row starts once the factor tasks producing its tiles have finished. The
// factor then leaves OVERLAP_SOLVE_SMS SMs to that pass.
int factor_solve_impl(sog_system* s, const double* V_dev, int32_t nrhs, const double* b_dev, double* x_dev,
                      sog_solve_stats* stats) {
    const bool overlap = !s->fp64 && s->segs.size() == 1 && !s->tune_pending &&
                         s->opt.executor == SOG_EXEC_PERSISTENT && !s->opt.resident_compact && s->d_fwait_ptr &&
                         s->csr.ptr && (nrhs == 1 || (nrhs % 8 == 0 && nrhs <= 8 * TRISOLVE_MAX_CHUNKS)) &&
                         s->grid_factor > 2 * OVERLAP_SOLVE_SMS;
    std::vector<int32_t> k(s->segs.size(), nrhs);
    if (!overlap) {
        int r = factor_inputs(s, V_dev);
        if (!r) r = factor_checked(s);
        if (r && r != SOG_EPIVOT) return r;
        const int r2 = solve_device_impl(s, k.data(), b_dev, x_dev, stats);
        return r ? r : r2;
    }
    cudaStream_t st = s->stream;
    if (!s->stream2) {
        CK(cudaStreamCreateWithFlags(&s->stream2, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&s->ev_ready, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&s->ev_lower, cudaEventDisableTiming));
    }
    int r = factor_inputs(s, V_dev);
    if (r) return r;
    // the forward pass's input: b gathered and cast to FP32 (one chunk)
    s->h_nrhs[0] = nrhs;
    s->h_voff[0] = 0;
    if ((r = ensure_vectors(s, nrhs))) return r;
    CK(cudaMemcpyAsync(s->d_seg_nrhs, s->h_nrhs, sizeof(int32_t), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(s->d_seg_voff, s->h_voff, sizeof(int64_t), cudaMemcpyHostToDevice, st));
    const DevSegs g = seg_view(s);
    s->launches += 2;
    gather_seg_launch(b_dev, g, s->n_ext, 0, nrhs, s->d_bext, st);
    cast_f64_to_f32_launch(s->d_bext, s->d_v32, (int64_t)s->n_ext * nrhs, st);
    if ((r = factor_reset(s))) return r;
    CK(cudaEventRecord(s->ev_ready, st));
    // forward pass on the second stream, after the inputs and the reset
    // completion flags
    CK(cudaStreamWaitEvent(s->stream2, s->ev_ready, 0));
    // this solve's two epochs, reserved now: flags a pass that is cut short
    // leaves behind never match a later pass
    s->fw_epoch = s->epoch;
    s->epoch += 2;
    DevSolve dso = s->ds;
    dso.fwait_ptr = s->d_fwait_ptr;
    dso.fwait = s->d_fwait;
    dso.task_done = s->dt.task_done;
    const int grid2 = std::min(OVERLAP_SOLVE_CTAS, s->R * std::max(1, nrhs / 8));
    if (trisolve_lower_overlap_launch(dso, (const float*)s->tiles, s->d_v32, nrhs, s->fw_epoch, grid2, s->stream2))
        return fail(SOG_ECUDA, std::string("solve launch: ") + cudaGetErrorString(cudaGetLastError()));
    s->launches++;
    // from here on every return waits for the forward pass on the second
    // stream (its waits are bounded; a factorisation that cannot run is
    // marked as given up below, which ends them at once)
    struct Join {
        cudaStream_t s2;
        ~Join() { cudaStreamSynchronize(s2); }
    } join{s->stream2};
    CK(cudaEventRecord(s->ev_lower, s->stream2));
    // the factor on the remaining SMs
    CK(cudaEventRecord(s->e0, st));
    const int fgrid = s->grid_factor - OVERLAP_SOLVE_SMS;
    if (factor_ordered_launch(s->dt, (float*)s->tiles, fgrid, s->stages, st)) {
        const std::string m = cudaGetErrorString(cudaGetLastError());
        static const int32_t gave_up = ST_TIMEOUT;
        cudaMemcpy(&s->dt.status->flags, &gave_up, sizeof(gave_up), cudaMemcpyHostToDevice);
        return fail(SOG_ECUDA, "factor launch: " + m);
    }
    s->launches++;
    CK(cudaEventRecord(s->e1, st));
    CK(cudaStreamSynchronize(st));
    CK(cudaEventElapsedTime(&s->t_factor, s->e0, s->e1));
    r = check_status(s, true);
    if (r) return r;
    s->factored = true;
    // the forward pass's positions not yet claimed, on the whole GPU
    {
        const int nch = std::max(1, std::min(nrhs / 8, TRISOLVE_MAX_CHUNKS));
        int grid = std::min(s->R * nch, trisolve_grid(false, nrhs, s->ctx->num_sms));
        if (s->opt.max_ctas > 0) grid = std::min(grid, s->opt.max_ctas);
        if (trisolve_lower_join_launch(s->ds, (const float*)s->tiles, s->d_v32, nrhs, s->fw_epoch, grid, st))
            return fail(SOG_ECUDA, std::string("solve launch: ") + cudaGetErrorString(cudaGetLastError()));
        s->launches++;
    }
    const int pr = check_pivots(s);
    if (pr && pr != SOG_EPIVOT) return pr;
    // the rest of the solve after the forward pass; the solve time counts
    // from the factor kernel's end (its event becomes the solve's start)
    std::swap(s->e0, s->e1);
    CK(cudaStreamWaitEvent(st, s->ev_lower, 0));
    const int r2 = solve_device_impl(s, k.data(), b_dev, x_dev, stats, true);
    return pr ? pr : r2;
}

}  // namespace

double sog_internal::system_parallelism(const sog_system* s, int* full_grid) {
    if (full_grid) *full_grid = factor_persistent_grid(s->fp64, s->stages, s->ctx->num_sms);
    return (double)s->tg.ntasks / std::max(1, s->tg.nlevels);
}

void sog_internal::system_set_grid_cap(sog_system* s, int cap) {
    s->opt.max_ctas = cap > 0 ? cap : 0;
    s->grid_factor = factor_grid(s, s->stages);
}

extern "C" {

int sog_ctx_create(int32_t device, uint64_t pool_bytes, sog_ctx** out) {
    if (!out) return fail(SOG_EINVAL, "out is NULL");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(SOG_ENODEV, "no CUDA device");
    }
    if (device < 0 || device >= ndev) return fail(SOG_EINVAL, "bad device index");
    CK(cudaSetDevice(device));
    sog_ctx* c = new sog_ctx();
    c->device = device;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&c->e0) != cudaSuccess || cudaEventCreate(&c->e1) != cudaSuccess) {
        delete c;
        return fail(SOG_ECUDA, "context set-up failed");
    }
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    c->pool.cap = pool_bytes ? pool_bytes : (uint64_t)(0.9 * (double)fr);
    *out = c;
    return SOG_OK;
}

void sog_ctx_destroy(sog_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    c->pool.destroy();
    if (c->e0) cudaEventDestroy(c->e0);
    if (c->e1) cudaEventDestroy(c->e1);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

int sog_ctx_stream(const sog_ctx* c, void** stream) {
    if (!c || !stream) return fail(SOG_EINVAL, "NULL argument");
    *stream = (void*)c->stream;
    return SOG_OK;
}

int sog_ctx_trim(sog_ctx* c) {
    if (!c) return fail(SOG_EINVAL, "NULL context");
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    c->pool.trim();
    return SOG_OK;
}

int sog_ctx_pool_usage(const sog_ctx* c, uint64_t* used, uint64_t* total) {
    if (!c) return fail(SOG_EINVAL, "NULL context");
    if (used) *used = c->pool.used;
    if (total) *total = c->pool.cap;
    return SOG_OK;
}

int sog_system_bytes(const sog_plan* plan, const sog_options* opt, uint64_t* bytes) {
    if (!plan || !bytes) return fail(SOG_EINVAL, "NULL argument");
    sog_options o = opt ? *opt : default_options();
    const Plan& p = plan->p;
    // + diagonal inverses and look-ahead products added for the substitution,
    // + the transposed L leaves of an LL^T plan
    bool any_sym = p.symmetric;
    for (const Segment& sg : p.segs) any_sym = any_sym || sg.symmetric;
    uint64_t tiles = ((uint64_t)p.storage_count + (2ull + 2 * SOLVE_LOOKAHEAD) * p.cfg.block_rows + (any_sym ? p.L.size() : 0)) * 4096 *
                     elem_bytes(o);
    uint64_t ops = (uint64_t)p.ops.size();
    uint64_t aux = ops * 40 + (uint64_t)p.scatter_tile.size() * 22 + (uint64_t)p.cfg.n_ext() * 64 + (1 << 20);
    *bytes = tiles + aux;
    return SOG_OK;
}

int sog_system_create(sog_ctx* c, const sog_plan* plan, const sog_options* opt, sog_system** out) {
    if (!c || !plan || !out) return fail(SOG_EINVAL, "NULL argument");
    *out = nullptr;
    sog_options o = opt ? *opt : default_options();
    if (o.precision != SOG_FP64 && o.precision != SOG_MIXED) return fail(SOG_EINVAL, "bad precision");
    if (o.executor != SOG_EXEC_PERSISTENT && o.executor != SOG_EXEC_LEVELS && o.executor != SOG_EXEC_QUEUE &&
        o.executor != SOG_EXEC_AUTO)
        return fail(SOG_EINVAL, "bad executor");
    if (o.tol <= 0) o.tol = 1e-10;
    if (o.max_refine < 0) o.max_refine = 0;
    CK(cudaSetDevice(c->device));
    const Plan& p = plan->p;
    sog_system* s = new sog_system();
    s->ctx = c;
    s->stream = c->stream;
    if (cudaEventCreate(&s->e0) != cudaSuccess || cudaEventCreate(&s->e1) != cudaSuccess) {
        cudaGetLastError();
        sog_system_destroy(s);
        return fail(SOG_ECUDA, "system events");
    }
    s->opt = o;
    s->fp64 = o.precision == SOG_FP64;
    s->imported = plan->imported;
    s->n = p.cfg.n;
    s->n_ext = p.cfg.n_ext();
    s->R = p.cfg.block_rows;
    s->n_input = p.n_input;
    s->storage = p.storage_count;
    s->ntrip = (int64_t)p.scatter_tile.size();
    s->nval = p.mirror_src.empty() ? s->ntrip : p.nval;
    s->npad = (int64_t)p.pad_tile.size();
    s->L = p.L;
    s->U = p.U;
    s->symmetric = p.symmetric;
    int gemm_parts = o.gemm_split == 1 ? 1 : (o.gemm_split == 4 ? 4 : (s->fp64 ? 4 : 1));
    if (!s->fp64) gemm_parts = 1;
    // inverses of the diagonal factor blocks for the substitution (reused
    // where the DAG already computes them), look-ahead products and
    // transposed leaves: appended to a view of the plan's ops, which are not
    // copied
    OpSeq ops2(p.ops.data(), (int64_t)p.ops.size());
    ops2.extra.reserve(6 * (size_t)p.cfg.block_rows + p.L.size());
    int32_t storage2 = p.storage_count;
    // LL^T systems: the upper factor of the substitution is L^T (upperSolverT,
    // BlockPlanner.cpp:752-797), materialised as transposed L leaves (in a
    // batch, of the symmetric systems only)
    {
        std::vector<Leaf> lsym;
        if (p.segs.empty()) {
            if (p.symmetric) lsym = s->L;
        } else {
            std::vector<char> sym_row(s->R, 0);
            for (const Segment& sg : p.segs)
                if (sg.symmetric)
                    for (int r = 0; r < sg.R; r++) sym_row[sg.row0 / 64 + r] = 1;
            for (const Leaf& lf : s->L)
                if (sym_row[lf.bi]) lsym.push_back(lf);
        }
        if (!lsym.empty()) {
            std::vector<Leaf> ut;
            add_transposed_leaves(ops2, storage2, lsym, ut);
            s->U.insert(s->U.end(), ut.begin(), ut.end());
            std::sort(s->U.begin(), s->U.end(),
                      [](const Leaf& a, const Leaf& b) { return a.bi != b.bi ? a.bi < b.bi : a.bj < b.bj; });
        }
    }
    std::vector<int32_t> ldinv, udinv;
    add_diag_inverses(ops2, storage2, s->R, s->L, s->U, ldinv, udinv);
    // look-ahead products by distance: lla[d] / ula[d] at distance d + 1
    std::vector<int32_t> lla[SOLVE_LOOKAHEAD], ula[SOLVE_LOOKAHEAD];
    if (o.solve_lookahead >= 0)
        for (int d = 0; d < SOLVE_LOOKAHEAD; d++)
            add_lookahead_products(ops2, storage2, s->R, s->L, s->U, ldinv, udinv, d + 1, lla[d], ula[d]);
    s->storage = storage2;
    std::vector<int32_t> outputs;
    for (const Leaf& lf : s->L) outputs.push_back(lf.id);
    for (const Leaf& lf : s->U) outputs.push_back(lf.id);
    for (int32_t id : ldinv) if (id > 0) outputs.push_back(id);
    for (int32_t id : udinv) if (id > 0) outputs.push_back(id);
    for (int d = 0; d < SOLVE_LOOKAHEAD; d++)
        for (auto* v : {&lla[d], &ula[d]})
            for (int32_t id : *v) if (id > 0) outputs.push_back(id);
    try {
        s->tg = build_tasks(ops2, storage2, p.n_input, outputs, gemm_parts, true, !s->fp64);
        if (!s->fp64) order_pairs_by_ready(s->tg, false);
    } catch (const std::exception& e) {
        delete s;
        return fail(SOG_EINVAL, std::string("DAG: ") + e.what());
    }
    const TaskGraph& g = s->tg;
    // leaves and substitution tiles through the copy aliases: a copied block's
    // value lives in its source's tile
    for (Leaf& lf : s->L) lf.id = g.alias[lf.id];
    for (Leaf& lf : s->U) lf.id = g.alias[lf.id];
    for (auto* v : {&ldinv, &udinv})
        for (int32_t& id : *v)
            if (id > 0) id = g.alias[id];
    for (int d = 0; d < SOLVE_LOOKAHEAD; d++)
        for (auto* v : {&lla[d], &ula[d]})
            for (int32_t& id : *v)
                if (id > 0) id = g.alias[id];
    // solve structure
    std::vector<int32_t> lptr(s->R + 1, 0), uptr(s->R + 1, 0), ldiag(s->R, 0), udiag(s->R, 0);
    std::vector<Leaf> loff, uoff;
    for (const Leaf& lf : s->L) {
        if (lf.bi == lf.bj) ldiag[lf.bi] = lf.id;
        else if (lf.bj < lf.bi) loff.push_back(lf);
    }
    for (const Leaf& lf : s->U) {
        if (lf.bi == lf.bj) udiag[lf.bi] = lf.id;
        else if (lf.bj > lf.bi) uoff.push_back(lf);
    }
    for (int i = 0; i < s->R; i++)
        if (ldiag[i] <= 0 || udiag[i] <= 0) {
            delete s;
            return fail(SOG_EINVAL, "missing diagonal factor block");
        }
    std::sort(loff.begin(), loff.end(), [](const Leaf& a, const Leaf& b) { return a.bi != b.bi ? a.bi < b.bi : a.bj < b.bj; });
    std::sort(uoff.begin(), uoff.end(), [](const Leaf& a, const Leaf& b) { return a.bi != b.bi ? a.bi < b.bi : a.bj > b.bj; });
    std::vector<int32_t> lcol, lid, ucol, uid;
    for (const Leaf& lf : loff) { lptr[lf.bi + 1]++; lcol.push_back(lf.bj); lid.push_back(lf.id); }
    for (const Leaf& lf : uoff) { uptr[lf.bi + 1]++; ucol.push_back(lf.bj); uid.push_back(lf.id); }
    for (int i = 0; i < s->R; i++) { lptr[i + 1] += lptr[i]; uptr[i + 1] += uptr[i]; }
    s->sol_ids[0] = lid;
    s->sol_ids[1] = uid;
    s->sol_ids[2] = ldiag;
    s->sol_ids[3] = udiag;
    s->sol_ids[4] = ldinv;
    s->sol_ids[5] = udinv;
    for (int d = 0; d < SOLVE_LOOKAHEAD; d++) {
        s->sol_ids[6 + 2 * d] = lla[d];
        s->sol_ids[7 + 2 * d] = ula[d];
    }
    std::vector<int32_t> order = static_order(g, s->fp64);
    // mixed path: the ordered executor starts a product before its last
    // producer finished (item bit 3), waiting per operand pair; every pair
    // lists the tasks producing its two tiles, every product the one
    // producing its initial tile (-1: an input, nothing to wait for)
    std::vector<int32_t> pair_wa, pair_wb, init_w;
    if (!s->fp64) {
        for (int32_t& it : order)  // one pair has nothing to overlap with
            if ((g.kind[it >> 4] == K_GEMM || g.kind[it >> 4] == K_GEMM_LU || g.kind[it >> 4] == K_GEMM_LLT) &&
                g.pair_ptr[(it >> 4) + 1] - g.pair_ptr[it >> 4] > 1)
                it |= ITEM_EARLY;
        pair_wa.resize(g.pair_a.size());
        pair_wb.resize(g.pair_b.size());
        for (size_t q = 0; q < g.pair_a.size(); q++) {
            const int32_t b = (g.pair_b[q] < 0 ? -g.pair_b[q] : g.pair_b[q]) & ~PAIR_TRANS;
            pair_wa[q] = g.pair_a[q] > p.n_input ? g.producer[g.pair_a[q]] : -1;
            pair_wb[q] = b > p.n_input ? g.producer[b] : -1;
        }
        init_w.assign(g.ntasks, -1);
        for (int32_t t = 0; t < g.ntasks; t++)
            if ((g.kind[t] == K_GEMM || g.kind[t] == K_GEMM_LU || g.kind[t] == K_GEMM_LLT) && g.a[t] > p.n_input)
                init_w[t] = g.producer[g.a[t]];
    }
    HostCSR hc;
    if (!plan->imported) hc = build_csr(p);
    // systems: a plain plan is one system over all block rows
    if (p.segs.empty()) {
        Segment sg;
        sg.n = p.cfg.n;
        sg.R = p.cfg.block_rows;
        sg.ntrip = (int64_t)p.scatter_tile.size();
        s->segs.push_back(sg);
    } else {
        s->segs = p.segs;
    }
    const size_t ns = s->segs.size();
    std::vector<int32_t> seg_brow(s->R), seg_n(ns), n2o(s->n_ext, -1);
    for (size_t k = 0; k < ns; k++) {
        const Segment& sg = s->segs[k];
        seg_n[k] = sg.n;
        for (int r = 0; r < sg.R; r++) seg_brow[sg.row0 / 64 + r] = (int32_t)k;
    }
    if (p.segs.empty())
        for (int i = 0; i < p.cfg.n; i++) n2o[i] = p.ord.new_to_old[i];
    else
        n2o = p.ord.new_to_old;
    // substitution dealing order of a batch: by row within its system (from
    // the top for L, from the bottom for U), then by system
    std::vector<int32_t> ord_l, ord_u;
    if (ns > 1) {
        int maxR = 0;
        for (const Segment& sg : s->segs) maxR = std::max(maxR, sg.R);
        ord_l.reserve(s->R);
        ord_u.reserve(s->R);
        for (int r = 0; r < maxR; r++)
            for (const Segment& sg : s->segs)
                if (r < sg.R) {
                    ord_l.push_back(sg.row0 / 64 + r);
                    ord_u.push_back(sg.row0 / 64 + sg.R - 1 - r);
                }
    }
    // task arrays
    std::vector<int32_t> parts32(g.ntasks);
    for (int32_t t = 0; t < g.ntasks; t++) parts32[t] = g.parts[t];
    std::vector<int32_t> counters0 = {0, (int32_t)g.ready_items.size(), 0};
    std::vector<DevStatus> st0 = {fresh_status()};
    std::vector<DevPivot> piv0(ns, fresh_pivot());
    // system of each task (batches): through the blocks each op reads, inputs
    // from their block row; every block of a batch belongs to one system
    std::vector<int32_t> task_seg;
    if (ns > 1) {
        std::vector<int32_t> bseg(storage2, 0);
        for (int32_t t = 0; t < p.n_input; t++) bseg[t + 1] = seg_brow[p.input_bi[t]];
        for (int64_t i = 0; i < ops2.size(); i++) {
            const Op& o = ops2[i];
            const int32_t from = o.src > 0 ? bseg[o.src] : (o.src2 > 0 ? bseg[o.src2] : 0);
            if (o.res > 0) bseg[o.res] = from;
            if (o.res2 > 0) bseg[o.res2] = from;
        }
        task_seg.resize(g.ntasks);
        for (int32_t t = 0; t < g.ntasks; t++) {
            const int32_t b = g.kind[t] == K_GEMM_LU || g.kind[t] == K_GEMM_LLT ? g.out3[t] : g.out[t];
            task_seg[t] = b > 0 && b < storage2 ? bseg[b] : 0;
        }
    }
    // forward pass overlapping the factorisation (a plain mixed system with
    // look-ahead products): per block row the tasks producing its off-diagonal
    // L leaves, its diagonal inverse and its look-ahead products
    std::vector<int32_t> fw_ptr, fw;
    if (!s->fp64 && ns == 1 && !lla[0].empty()) {
        std::vector<const std::vector<int32_t>*> las;
        for (int d = 0; d < SOLVE_LOOKAHEAD; d++) las.push_back(&lla[d]);
        forward_wait_lists(g, s->R, lptr, lid, ldinv, las, fw_ptr, fw);
    }
    Layout L;
    uint64_t o_kind = L.add<uint8_t>(g.ntasks), o_parts = L.add<uint8_t>(g.ntasks), o_out = L.add<int32_t>(g.ntasks),
             o_out2 = L.add<int32_t>(g.ntasks), o_a = L.add<int32_t>(g.ntasks), o_b = L.add<int32_t>(g.ntasks),
             o_c = L.add<int32_t>(g.ntasks), o_out3 = L.add<int32_t>(g.ntasks),
             o_pptr = L.add<int32_t>(g.ntasks + 1), o_pa = L.add<int32_t>(g.pair_a.size()),
             o_pb = L.add<int32_t>(g.pair_b.size()), o_sptr = L.add<int32_t>(g.ntasks + 1),
             o_succ = L.add<int32_t>(g.succ.size()), o_ndep0 = L.add<int32_t>(g.ntasks),
             o_dep = L.add<int32_t>(g.ntasks), o_parts0 = L.add<int32_t>(g.ntasks),
             o_pleft = L.add<int32_t>(g.ntasks), o_queue = L.add<int32_t>(g.total_items),
             o_ready = L.add<int32_t>(g.ready_items.size()), o_cnt0 = L.add<int32_t>(3), o_cnt = L.add<int32_t>(3),
             o_prio = L.add<int32_t>(g.ntasks), o_ldinv = L.add<int32_t>(s->R), o_udinv = L.add<int32_t>(s->R),
             o_levels = L.add<int32_t>(g.level_items.size()), o_st0 = L.add<DevStatus>(1), o_st = L.add<DevStatus>(1),
             o_lptr = L.add<int32_t>(lptr.size()), o_lcol = L.add<int32_t>(lcol.size()),
             o_lid = L.add<int32_t>(lid.size()), o_uptr = L.add<int32_t>(uptr.size()),
             o_ucol = L.add<int32_t>(ucol.size()), o_uid = L.add<int32_t>(uid.size()),
             o_ldiag = L.add<int32_t>(ldiag.size()), o_udiag = L.add<int32_t>(udiag.size()),
             o_flags = L.add<int32_t>((size_t)s->R * TRISOLVE_MAX_CHUNKS), o_cptr = L.add<int32_t>(hc.ptr.size()),
             o_ccol = L.add<int32_t>(hc.col.size()), o_cval = L.add<double>(hc.val.size()),
             o_cpos = L.add<int32_t>(hc.pos.size()), o_sct = L.add<int32_t>(p.scatter_tile.size()),
             o_sco = L.add<int16_t>(p.scatter_off.size()), o_pdt = L.add<int32_t>(p.pad_tile.size()),
             o_pdo = L.add<int16_t>(p.pad_off.size()), o_n2o = L.add<int32_t>(n2o.size()),
             o_sbr = L.add<int32_t>(seg_brow.size()), o_sn = L.add<int32_t>(seg_n.size()),
             o_ordl = L.add<int32_t>(ord_l.size()), o_ordu = L.add<int32_t>(ord_u.size()),
             o_claim = L.add<int32_t>(2), o_fwp = L.add<int32_t>(fw_ptr.size()), o_fw = L.add<int32_t>(fw.size()),
             o_order = L.add<int32_t>(order.size()), o_pwa = L.add<int32_t>(pair_wa.size()),
             o_pwb = L.add<int32_t>(pair_wb.size()), o_initw = L.add<int32_t>(init_w.size()),
             o_done = L.add<int32_t>(g.ntasks), o_piv = L.add<DevPivot>(ns), o_piv0 = L.add<DevPivot>(ns),
             o_amax = L.add<unsigned long long>(ns), o_tseg = L.add<int32_t>(task_seg.size()),
             o_V = L.add<double>(s->nval), o_vidx = L.add<int32_t>(p.mirror_src.size());
    uint64_t o_lla[SOLVE_LOOKAHEAD], o_ula[SOLVE_LOOKAHEAD];
    for (int d = 0; d < SOLVE_LOOKAHEAD; d++) {
        o_lla[d] = L.add<int32_t>(lla[d].size());
        o_ula[d] = L.add<int32_t>(ula[d].size());
    }
    s->tiles_bytes = (uint64_t)s->storage * 4096 * elem_bytes(o);
    s->tiles = c->pool.alloc(s->tiles_bytes);
    if (!s->tiles) {
        delete s;
        return fail(SOG_ENOMEM, "block pool exhausted (tiles)");
    }
    s->aux_bytes = L.off;
    s->aux = static_cast<char*>(c->pool.alloc(L.off));
    if (!s->aux) {
        c->pool.release(s->tiles, s->tiles_bytes);
        delete s;
        return fail(SOG_ENOMEM, "block pool exhausted (task tables)");
    }
    cudaStream_t st = s->stream;
    char* A = s->aux;
    DevTasks& dt = s->dt;
    dt.ntasks = g.ntasks;
    dt.total_items = g.total_items;
    dt.kind = put(A, o_kind, g.kind, st);
    dt.parts = put(A, o_parts, g.parts, st);
    dt.out = put(A, o_out, g.out, st);
    dt.out2 = put(A, o_out2, g.out2, st);
    dt.a = put(A, o_a, g.a, st);
    dt.b = put(A, o_b, g.b, st);
    dt.c = put(A, o_c, g.c, st);
    dt.out3 = put(A, o_out3, g.out3, st);
    dt.prio = put(A, o_prio, g.prio, st);
    dt.pair_ptr = put(A, o_pptr, g.pair_ptr, st);
    dt.pair_a = put(A, o_pa, g.pair_a, st);
    dt.pair_b = put(A, o_pb, g.pair_b, st);
    dt.succ_ptr = put(A, o_sptr, g.succ_ptr, st);
    dt.succ = put(A, o_succ, g.succ, st);
    s->d_ndep0 = put(A, o_ndep0, g.ndep, st);
    dt.dep = reinterpret_cast<int32_t*>(A + o_dep);
    s->d_parts0 = put(A, o_parts0, parts32, st);
    dt.parts_left = reinterpret_cast<int32_t*>(A + o_pleft);
    dt.queue = reinterpret_cast<int32_t*>(A + o_queue);
    s->d_ready0 = put(A, o_ready, g.ready_items, st);
    s->nready = (int)g.ready_items.size();
    s->d_counters0 = put(A, o_cnt0, counters0, st);
    dt.head = reinterpret_cast<int32_t*>(A + o_cnt);
    dt.tail = dt.head + 1;
    dt.done = dt.head + 2;
    s->d_level_items = put(A, o_levels, g.level_items, st);
    dt.order = put(A, o_order, order, st);
    dt.early = !s->fp64;  // the tuner may turn it off
    dt.skip_zero = 1;
    s->early = dt.early;
    dt.pair_wa = pair_wa.empty() ? nullptr : put(A, o_pwa, pair_wa, st);
    dt.pair_wb = pair_wb.empty() ? nullptr : put(A, o_pwb, pair_wb, st);
    dt.init_w = init_w.empty() ? nullptr : put(A, o_initw, init_w, st);
    dt.task_done = reinterpret_cast<int32_t*>(A + o_done);
    s->d_status0 = put(A, o_st0, st0, st);
    dt.status = reinterpret_cast<DevStatus*>(A + o_st);
    s->d_piv0 = put(A, o_piv0, piv0, st);
    s->d_piv = reinterpret_cast<DevPivot*>(A + o_piv);
    dt.piv = s->d_piv;
    s->d_amax = reinterpret_cast<unsigned long long*>(A + o_amax);
    cudaMemsetAsync(s->d_amax, 0, sizeof(unsigned long long) * ns, st);
    dt.task_seg = task_seg.empty() ? nullptr : put(A, o_tseg, task_seg, st);
    dt.wait_limit_ns = 10ull * 1000 * 1000 * 1000;
    DevSolve& ds = s->ds;
    ds.block_rows = s->R;
    ds.l_ptr = put(A, o_lptr, lptr, st);
    ds.l_col = put(A, o_lcol, lcol, st);
    ds.l_id = put(A, o_lid, lid, st);
    ds.u_ptr = put(A, o_uptr, uptr, st);
    ds.u_col = put(A, o_ucol, ucol, st);
    ds.u_id = put(A, o_uid, uid, st);
    ds.l_diag = put(A, o_ldiag, ldiag, st);
    ds.u_diag = put(A, o_udiag, udiag, st);
    ds.l_dinv = put(A, o_ldinv, ldinv, st);
    ds.u_dinv = put(A, o_udinv, udinv, st);
    ds.flags = reinterpret_cast<int32_t*>(A + o_flags);
    cudaMemsetAsync(ds.flags, 0, sizeof(int32_t) * s->R * TRISOLVE_MAX_CHUNKS, st);
    ds.status = dt.status;
    ds.wait_limit_ns = dt.wait_limit_ns;
    if (!plan->imported) {
        s->csr.n = s->n_ext;
        s->csr.ptr = put(A, o_cptr, hc.ptr, st);
        s->csr.col = put(A, o_ccol, hc.col, st);
        s->d_csr_val = put(A, o_cval, hc.val, st);
        s->csr.val = s->d_csr_val;
        s->d_csr_pos = put(A, o_cpos, hc.pos, st);
        s->d_sc_tile = put(A, o_sct, p.scatter_tile, st);
        s->d_sc_off = put(A, o_sco, p.scatter_off, st);
        s->d_pad_tile = put(A, o_pdt, p.pad_tile, st);
        s->d_pad_off = put(A, o_pdo, p.pad_off, st);
    }
    s->d_n2o = put(A, o_n2o, n2o, st);
    s->d_seg_brow = put(A, o_sbr, seg_brow, st);
    s->d_seg_n = put(A, o_sn, seg_n, st);
    ds.order_l = ord_l.empty() ? nullptr : put(A, o_ordl, ord_l, st);
    ds.order_u = ord_u.empty() ? nullptr : put(A, o_ordu, ord_u, st);
    for (int d = 0; d < SOLVE_LOOKAHEAD; d++) {
        ds.l_la[d] = lla[d].empty() ? nullptr : put(A, o_lla[d], lla[d], st);
        ds.u_la[d] = ula[d].empty() ? nullptr : put(A, o_ula[d], ula[d], st);
    }
    ds.claim = reinterpret_cast<int32_t*>(A + o_claim);
    if (!fw_ptr.empty()) {
        s->d_fwait_ptr = put(A, o_fwp, fw_ptr, st);
        s->d_fwait = fw.empty() ? reinterpret_cast<int32_t*>(A + o_fw) : put(A, o_fw, fw, st);
    }
    if (cudaMallocHost(&s->h_red, sizeof(double) * RED * 64 * ns) != cudaSuccess ||
        cudaMallocHost(&s->h_nrhs, sizeof(int32_t) * ns) != cudaSuccess ||
        cudaMallocHost(&s->h_active, sizeof(int32_t) * ns) != cudaSuccess ||
        cudaMallocHost(&s->h_voff, sizeof(int64_t) * ns) != cudaSuccess ||
        cudaMallocHost(&s->h_cnt, sizeof(unsigned long long) * ns) != cudaSuccess) {
        cudaGetLastError();
        sog_system_destroy(s);
        return fail(SOG_ENOMEM, "pinned host buffers");
    }
    s->d_V = reinterpret_cast<double*>(A + o_V);
    if (!p.mirror_src.empty()) s->d_vidx = put(A, o_vidx, p.mirror_src, st);
    s->stages = o.pipeline_stages == 1 ? 1 : 2;
    if (o.executor == SOG_EXEC_AUTO) {
        Tuned known;
        if (tuned_config(tune_key(g, s->fp64), known)) {
            s->opt.executor = known.executor;
            s->stages = known.stages;
            s->early = known.early;
            dt.early = !s->fp64 && known.early;
            dt.skip_zero = known.sparse;
        } else {
            s->opt.executor = SOG_EXEC_PERSISTENT;
            s->tune_pending = true;
        }
    }
    s->grid_factor = factor_grid(s, s->stages);
    if (cudaStreamSynchronize(st) != cudaSuccess) {
        std::string m = cudaGetErrorString(cudaGetLastError());
        sog_system_destroy(s);
        return fail(SOG_ECUDA, "system upload: " + m);
    }
    *out = s;
    return SOG_OK;
}

void sog_system_destroy(sog_system* s) {
    if (!s) return;
    sog_ctx* c = s->ctx;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(s->stream);
    if (s->compacted) c->pool.release(s->cbuf, s->cbuf_bytes);
    else c->pool.release(s->tiles, s->tiles_bytes);
    c->pool.release(s->aux, s->aux_bytes);
    c->pool.release(s->vecs, s->vec_bytes);
    c->pool.release(s->trace, s->trace_bytes);
    if (s->h_red) cudaFreeHost(s->h_red);
    if (s->h_nrhs) cudaFreeHost(s->h_nrhs);
    if (s->h_active) cudaFreeHost(s->h_active);
    if (s->h_voff) cudaFreeHost(s->h_voff);
    if (s->h_cnt) cudaFreeHost(s->h_cnt);
    if (s->e0) cudaEventDestroy(s->e0);
    if (s->e1) cudaEventDestroy(s->e1);
    if (s->stream2) {
        cudaStreamSynchronize(s->stream2);
        cudaStreamDestroy(s->stream2);
    }
    if (s->ev_ready) cudaEventDestroy(s->ev_ready);
    if (s->ev_lower) cudaEventDestroy(s->ev_lower);
    delete s;
}

int sog_system_set_stream(sog_system* s, void* stream) {
    if (!s) return fail(SOG_EINVAL, "NULL system");
    CK(cudaSetDevice(s->ctx->device));
    CK(cudaStreamSynchronize(s->stream));  // the system's work so far, on the stream it was issued to
    s->stream = stream ? (cudaStream_t)stream : s->ctx->stream;
    return SOG_OK;
}

int sog_factor_device(sog_system* s, const double* V_dev) {
    if (!s) return fail(SOG_EINVAL, "NULL system");
    if (s->imported) return fail(SOG_ESTATE, "imported plan: use sog_factor_tiles");
    if (!V_dev && s->ntrip) return fail(SOG_EINVAL, "NULL values");
    CK(cudaSetDevice(s->ctx->device));
    if (int r = factor_inputs(s, V_dev)) return r;
    return factor_checked(s);
}

int sog_factor_solve_device(sog_system* s, const double* V_dev, int32_t nrhs, const double* b_dev, double* x_dev,
                            sog_solve_stats* stats) {
    if (!s || nrhs <= 0 || !b_dev || !x_dev) return fail(SOG_EINVAL, "bad argument");
    if (s->imported) return fail(SOG_ESTATE, "imported plan: use sog_factor_tiles");
    if (!V_dev && s->ntrip) return fail(SOG_EINVAL, "NULL values");
    CK(cudaSetDevice(s->ctx->device));
    return factor_solve_impl(s, V_dev, nrhs, b_dev, x_dev, stats);
}

int sog_factor_solve(sog_system* s, const double* V, int32_t nrhs, const double* b, double* x,
                     sog_solve_stats* stats) {
    if (!s || nrhs <= 0 || !b || !x) return fail(SOG_EINVAL, "bad argument");
    if (s->imported) return fail(SOG_ESTATE, "imported plan: use sog_factor_tiles");
    if (!V && s->nval) return fail(SOG_EINVAL, "NULL values");
    sog_ctx* c = s->ctx;
    CK(cudaSetDevice(c->device));
    if (s->nval) CK(cudaMemcpyAsync(s->d_V, V, sizeof(double) * s->nval, cudaMemcpyHostToDevice, s->stream));
    const uint64_t bytes = sizeof(double) * (uint64_t)nrhs * (uint64_t)s->n;
    double* db = static_cast<double*>(c->pool.alloc(bytes));
    double* dx = static_cast<double*>(c->pool.alloc(bytes));
    if (!db || !dx) {
        c->pool.release(db, bytes);
        c->pool.release(dx, bytes);
        return fail(SOG_ENOMEM, "block pool exhausted (rhs)");
    }
    int r = SOG_OK;
    if (cudaMemcpyAsync(db, b, bytes, cudaMemcpyHostToDevice, s->stream) != cudaSuccess)
        r = fail(SOG_ECUDA, "rhs upload failed");
    if (!r) {
        r = factor_solve_impl(s, s->d_V, nrhs, db, dx, stats);
        if (!r || r == SOG_ENOCONV || r == SOG_ENAN || r == SOG_EPIVOT) {
            if (cudaMemcpyAsync(x, dx, bytes, cudaMemcpyDeviceToHost, s->stream) != cudaSuccess ||
                cudaStreamSynchronize(s->stream) != cudaSuccess)
                r = fail(SOG_ECUDA, "download failed");
        }
    }
    c->pool.release(db, bytes);
    c->pool.release(dx, bytes);
    return r;
}

int sog_factor(sog_system* s, const double* V) {
    if (!s) return fail(SOG_EINVAL, "NULL system");
    if (s->imported) return fail(SOG_ESTATE, "imported plan: use sog_factor_tiles");
    if (!V && s->nval) return fail(SOG_EINVAL, "NULL values");
    CK(cudaSetDevice(s->ctx->device));
    if (s->nval)
        CK(cudaMemcpyAsync(s->d_V, V, sizeof(double) * s->nval, cudaMemcpyHostToDevice, s->stream));
    return sog_factor_device(s, s->d_V);
}

int sog_factor_tiles(sog_system* s, const double* tiles) {
    if (!s || !tiles) return fail(SOG_EINVAL, "NULL argument");
    sog_ctx* c = s->ctx;
    CK(cudaSetDevice(c->device));
    if (int r = uncompact_tiles(s)) return r;
    const uint64_t n = (uint64_t)s->n_input * 4096;
    // max |a| over the given tiles, one figure for every system of the plan
    // (it includes the unit diagonal the planner puts on padding rows)
    CK(cudaMemsetAsync(s->d_amax, 0, sizeof(unsigned long long) * s->segs.size(), s->stream));
    s->amax_global = true;
    if (s->fp64) {
        CK(cudaMemcpyAsync((double*)s->tiles + 4096, tiles, n * 8, cudaMemcpyHostToDevice, s->stream));
        s->launches++;
        absmax_launch((double*)s->tiles + 4096, (int64_t)n, s->d_amax, s->stream);
    } else {
        double* stage = static_cast<double*>(c->pool.alloc(n * 8));
        if (!stage) return fail(SOG_ENOMEM, "block pool exhausted (staging)");
        CK(cudaMemcpyAsync(stage, tiles, n * 8, cudaMemcpyHostToDevice, s->stream));
        s->launches += 2;
        absmax_launch(stage, (int64_t)n, s->d_amax, s->stream);
        convert_tiles_launch(stage, (float*)s->tiles + 4096, (int64_t)n, s->stream);
        CK(cudaStreamSynchronize(s->stream));
        c->pool.release(stage, n * 8);
    }
    return factor_checked(s);
}

int sog_solve_device(sog_system* s, int32_t nrhs, const double* b_dev, double* x_dev, sog_solve_stats* stats) {
    if (!s || nrhs <= 0 || !b_dev || !x_dev) return fail(SOG_EINVAL, "bad argument");
    if (!s->factored) return fail(SOG_ESTATE, "solve before factor");
    CK(cudaSetDevice(s->ctx->device));
    std::vector<int32_t> k(s->segs.size(), nrhs);
    return solve_device_impl(s, k.data(), b_dev, x_dev, stats);
}

int sog_solve(sog_system* s, int32_t nrhs, const double* b, double* x, sog_solve_stats* stats) {
    if (!s || nrhs <= 0 || !b || !x) return fail(SOG_EINVAL, "bad argument");
    if (!s->factored) return fail(SOG_ESTATE, "solve before factor");
    CK(cudaSetDevice(s->ctx->device));
    std::vector<int32_t> k(s->segs.size(), nrhs);
    return solve_host(s, k.data(), b, x, stats);
}

int sog_solve_batch(sog_system* s, const int32_t* nrhs, const double* b, double* x, sog_solve_stats* stats) {
    if (!s || !nrhs) return fail(SOG_EINVAL, "bad argument");
    if (!s->factored) return fail(SOG_ESTATE, "solve before factor");
    if (solve_values(s, nrhs) > 0 && (!b || !x)) return fail(SOG_EINVAL, "NULL b or x");
    CK(cudaSetDevice(s->ctx->device));
    const int r = solve_host(s, nrhs, b, x, nullptr);
    if (stats && s->seg_stats.size() == s->segs.size())
        std::memcpy(stats, s->seg_stats.data(), sizeof(sog_solve_stats) * s->segs.size());
    return r;
}

int sog_solve_batch_device(sog_system* s, const int32_t* nrhs, const double* b_dev, double* x_dev,
                           sog_solve_stats* stats) {
    if (!s || !nrhs) return fail(SOG_EINVAL, "bad argument");
    if (!s->factored) return fail(SOG_ESTATE, "solve before factor");
    if (solve_values(s, nrhs) > 0 && (!b_dev || !x_dev)) return fail(SOG_EINVAL, "NULL b or x");
    CK(cudaSetDevice(s->ctx->device));
    const int r = solve_device_impl(s, nrhs, b_dev, x_dev, nullptr);
    if (stats && s->seg_stats.size() == s->segs.size())
        std::memcpy(stats, s->seg_stats.data(), sizeof(sog_solve_stats) * s->segs.size());
    return r;
}

int sog_solve_permuted(sog_system* s, const double* b_ext, double* x_ext) {
    if (!s || !b_ext || !x_ext) return fail(SOG_EINVAL, "bad argument");
    if (!s->factored) return fail(SOG_ESTATE, "solve before factor");
    sog_ctx* c = s->ctx;
    CK(cudaSetDevice(c->device));
    int r = ensure_vectors(s, 1);
    if (r) return r;
    const uint64_t ne = (uint64_t)s->n_ext;
    CK(cudaMemcpyAsync(s->d_xext, b_ext, ne * 8, cudaMemcpyHostToDevice, s->stream));
    CK(cudaEventRecord(s->e0, s->stream));
    if (s->fp64) {
        if ((r = trisolve(s, s->d_xext, 1))) return r;
    } else {
        s->launches++;
        cast_f64_to_f32_launch(s->d_xext, s->d_v32, ne, s->stream);
        if ((r = trisolve(s, s->d_v32, 1))) return r;
        s->launches++;
        axpy_f32_to_f64_launch(s->d_v32, s->d_xext, ne, 1, s->stream);
    }
    CK(cudaEventRecord(s->e1, s->stream));
    CK(cudaMemcpyAsync(x_ext, s->d_xext, ne * 8, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    CK(cudaEventElapsedTime(&s->t_solve, s->e0, s->e1));
    return check_status(s, false);
}

int sog_system_export_factors(sog_system* s, double* ltiles, double* utiles) {
    if (!s) return fail(SOG_EINVAL, "NULL system");
    if (!s->factored) return fail(SOG_ESTATE, "no factors");
    sog_ctx* c = s->ctx;
    CK(cudaSetDevice(c->device));
    const uint64_t eb = elem_bytes(s->opt);
    std::vector<float> tmp(4096);
    for (int side = 0; side < 2; side++) {
        const std::vector<Leaf>& lv = side == 0 ? s->L : s->U;
        double* dst = side == 0 ? ltiles : utiles;
        if (!dst || (side == 1 && s->symmetric)) continue;  // LL^T: the plan has no U leaves
        for (size_t k = 0; k < lv.size(); k++) {
            const int32_t id = s->compacted ? s->cmap[lv[k].id] : lv[k].id;
            const char* src = (const char*)s->tiles + (uint64_t)id * 4096 * eb;
            if (s->fp64) {
                CK(cudaMemcpy(dst + k * 4096, src, 4096 * 8, cudaMemcpyDeviceToHost));
            } else {
                CK(cudaMemcpy(tmp.data(), src, 4096 * 4, cudaMemcpyDeviceToHost));
                for (int e = 0; e < 4096; e++) dst[k * 4096 + e] = tmp[e];
            }
        }
    }
    return SOG_OK;
}

int sog_system_last_times(const sog_system* s, double* factor_ms, double* solve_ms) {
    if (!s) return fail(SOG_EINVAL, "NULL system");
    if (factor_ms) *factor_ms = s->t_factor;
    if (solve_ms) *solve_ms = s->t_solve;
    return SOG_OK;
}

int sog_system_set_wait_limit(sog_system* s, double ms) {
    if (!s || !(ms > 0)) return fail(SOG_EINVAL, "bad argument");
    s->dt.wait_limit_ns = (unsigned long long)(ms * 1e6);
    s->ds.wait_limit_ns = s->dt.wait_limit_ns;
    return SOG_OK;
}

int sog_debug_poison_task(sog_system* s, int32_t task) {
    if (!s || task < 0 || task >= s->tg.ntasks) return fail(SOG_EINVAL, "bad argument");
    CK(cudaSetDevice(s->ctx->device));
    int32_t v = s->tg.ndep[task] + 1;
    CK(cudaMemcpy(s->d_ndep0 + task, &v, sizeof(v), cudaMemcpyHostToDevice));
    s->poisoned = true;  // every task then waits for its whole dependency count
    s->dt.early = 0;
    return SOG_OK;
}

int sog_debug_unpoison(sog_system* s) {
    if (!s) return fail(SOG_EINVAL, "bad argument");
    CK(cudaSetDevice(s->ctx->device));
    CK(cudaMemcpy(s->d_ndep0, s->tg.ndep.data(), sizeof(int32_t) * s->tg.ntasks, cudaMemcpyHostToDevice));
    s->poisoned = false;
    s->dt.early = !s->fp64 && s->early;
    return SOG_OK;
}

int sog_debug_fp64_fragment_skip(sog_system* s, int32_t on) {
    if (!s) return fail(SOG_EINVAL, "NULL system");
    if (!s->fp64) return fail(SOG_EINVAL, "not an FP64 system");
    if (s->tune_pending) {  // keep the tuner's executor choice out of it
        s->tune_pending = false;
        s->opt.executor = SOG_EXEC_PERSISTENT;
        s->grid_factor = factor_grid(s, s->stages);
    }
    s->dt.skip_zero = on ? 1 : 0;
    return SOG_OK;
}

int sog_system_trace_enable(sog_system* s, int32_t on) {
    if (!s) return fail(SOG_EINVAL, "NULL system");
    sog_ctx* c = s->ctx;
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(s->stream));
    if (!on) {
        c->pool.release(s->trace, s->trace_bytes);
        s->trace = nullptr;
        s->dt.trace = nullptr;
        s->ds.trace = nullptr;
        return SOG_OK;
    }
    if (s->trace) return SOG_OK;
    s->trace_bytes = sizeof(unsigned long long) * 4 * ((uint64_t)s->tg.ntasks + s->R);
    s->trace = static_cast<unsigned long long*>(c->pool.alloc(s->trace_bytes));
    if (!s->trace) return fail(SOG_ENOMEM, "block pool exhausted (trace)");
    CK(cudaMemset(s->trace, 0, s->trace_bytes));
    s->dt.trace = s->trace;
    s->ds.trace = s->trace + 4 * (uint64_t)s->tg.ntasks;
    return SOG_OK;
}

int sog_system_trace_get(sog_system* s, uint64_t* task_trace, uint64_t* row_trace, int32_t* task_kind) {
    if (!s) return fail(SOG_EINVAL, "NULL system");
    if (!s->trace) return fail(SOG_ESTATE, "trace not enabled");
    CK(cudaSetDevice(s->ctx->device));
    CK(cudaStreamSynchronize(s->stream));
    if (task_trace)
        CK(cudaMemcpy(task_trace, s->trace, sizeof(uint64_t) * 4 * s->tg.ntasks, cudaMemcpyDeviceToHost));
    if (row_trace)
        CK(cudaMemcpy(row_trace, s->trace + 4 * (uint64_t)s->tg.ntasks, sizeof(uint64_t) * 4 * s->R,
                      cudaMemcpyDeviceToHost));
    if (task_kind)
        for (int32_t t = 0; t < s->tg.ntasks; t++) task_kind[t] = s->tg.kind[t];
    return SOG_OK;
}

int sog_system_task_graph(const sog_system* s, int32_t* succ_ptr, int32_t* succ, int32_t* npairs) {
    if (!s) return fail(SOG_EINVAL, "NULL system");
    const TaskGraph& g = s->tg;
    if (succ_ptr) std::memcpy(succ_ptr, g.succ_ptr.data(), sizeof(int32_t) * (g.ntasks + 1));
    if (succ) std::memcpy(succ, g.succ.data(), sizeof(int32_t) * g.succ.size());
    if (npairs)
        for (int32_t t = 0; t < g.ntasks; t++) npairs[t] = g.pair_ptr[t + 1] - g.pair_ptr[t];
    return SOG_OK;
}

int sog_plan_task_graph_info(const sog_plan* plan, int32_t gemm_split, int64_t* counts) {
    if (!plan || !counts) return fail(SOG_EINVAL, "NULL argument");
    const Plan& p = plan->p;
    try {
        OpSeq ops2(p.ops.data(), (int64_t)p.ops.size());
        int32_t storage2 = p.storage_count;
        std::vector<int32_t> ldinv, udinv, outputs;
        add_diag_inverses(ops2, storage2, p.cfg.block_rows, p.L, p.U, ldinv, udinv);
        for (const Leaf& lf : p.L) outputs.push_back(lf.id);
        for (const Leaf& lf : p.U) outputs.push_back(lf.id);
        TaskGraph g = build_tasks(ops2, storage2, p.n_input, outputs, gemm_split == 4 ? 4 : 1);
        counts[0] = g.ntasks;
        counts[1] = g.nlevels;
        counts[2] = g.total_items;
        counts[3] = g.gemm_pairs;
        for (int k = 0; k < 5; k++) counts[4 + k] = g.count[k];
        counts[5] += g.count[K_LLT];
        counts[9] = g.fused_subs;
        counts[10] = storage2 - p.storage_count;
        counts[11] = g.ntasks ? *std::max_element(g.prio.begin(), g.prio.end()) + 1 : 0;
        counts[12] = g.fused_inverses;
        counts[13] = g.aliased_copies;
        counts[14] = g.aliased_inverses;
    } catch (const std::exception& e) {
        return fail(SOG_EINVAL, std::string("DAG: ") + e.what());
    }
    return SOG_OK;
}

int sog_system_pivots(const sog_system* s, sog_solve_stats* stats) {
    if (!s || !stats) return fail(SOG_EINVAL, "NULL argument");
    if (!s->factored) return fail(SOG_ESTATE, "no factors");
    for (size_t k = 0; k < s->segs.size(); k++) {
        std::memset(&stats[k], 0, sizeof(sog_solve_stats));
        fill_pivot_stats(s, k, stats[k]);
        stats[k].status = k < s->piv.size() && s->piv[k].tripped ? SOG_EPIVOT : SOG_OK;
    }
    return SOG_OK;
}

int sog_system_executor(const sog_system* s, int32_t* executor, int32_t* stages, int32_t* early) {
    if (!s || !executor || !stages || !early) return fail(SOG_EINVAL, "bad argument");
    *executor = s->opt.executor;
    *stages = s->fp64 ? 0 : s->stages;
    *early = s->dt.early && s->opt.executor == SOG_EXEC_PERSISTENT ? 1 : 0;
    return SOG_OK;
}

int sog_system_task_info(const sog_system* s, int64_t* counts) {
    if (!s || !counts) return fail(SOG_EINVAL, "bad argument");
    const TaskGraph& g = s->tg;
    counts[0] = g.ntasks;
    counts[1] = g.nlevels;
    counts[2] = g.total_items;
    counts[3] = g.gemm_pairs;
    for (int k = 0; k < 5; k++) counts[4 + k] = g.count[k];
    counts[5] += g.count[K_LLT];
    counts[8] += g.count[K_TRANS];
    counts[4] += g.count[K_GEMM_LU] + g.count[K_GEMM_LLT];  // a product with its LU counts as both
    counts[5] += g.count[K_GEMM_LU] + g.count[K_GEMM_LLT];
    counts[9] = s->grid_factor;
    counts[10] = s->launches;
    return SOG_OK;
}

int soglu_solveLU(int32_t dim, int64_t valcount, int32_t symmetric, const int32_t* index_i, const int32_t* index_j,
                  const double* vals, const double* b, double* x_out, int32_t precision) {
    if (!b || !x_out || !vals) return fail(SOG_EINVAL, "NULL argument");
    sog_plan* plan = nullptr;
    int r = sog_plan_build(dim, valcount, symmetric, index_i, index_j, vals, 0, &plan);
    if (r) return r;
    sog_ctx* c = nullptr;
    r = sog_ctx_create(0, 0, &c);
    if (r) { sog_plan_destroy(plan); return r; }
    sog_options o = default_options();
    o.precision = precision;
    o.growth_limit = -1;  // solveLU clamps and continues, as the reference does
    sog_system* s = nullptr;
    r = sog_system_create(c, plan, &o, &s);
    if (!r) {
        r = sog_factor(s, vals);
        if (!r) r = sog_solve(s, 1, b, x_out, nullptr);
        sog_system_destroy(s);
    }
    sog_ctx_destroy(c);
    sog_plan_destroy(plan);
    return r;
}

}  // extern "C"
