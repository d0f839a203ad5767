// Host runtime of the GB300 executor: device context with a block-pool arena
// (the device counterpart of memutil's multi-level buffers, memutil.cpp:50-357),
// systems resident in the pool, and the factor / solve / refinement drivers
// behind the C ABI of include/soglu_gb300.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
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
    struct Chunk {
        char* base;
        uint64_t size;
        std::map<uint64_t, uint64_t> free_;  // offset -> size
    };
    uint64_t cap = 0, reserved = 0, used = 0;
    std::vector<Chunk> chunks;

    void* alloc(uint64_t bytes) {
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
    void destroy() {
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
    double* host_red = nullptr;  // pinned
};

struct sog_system {
    sog_ctx* ctx = nullptr;
    sog_options opt{};
    bool fp64 = true, imported = false;
    int n = 0, n_ext = 0, R = 0, n_input = 0;
    int32_t storage = 0;
    int64_t ntrip = 0, npad = 0;
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
    int32_t* d_level_items = nullptr;
    int nready = 0;
    DevStatus* d_status0 = nullptr;
    DevSolve ds{};
    DevCSR csr{};
    double* d_csr_val = nullptr;
    int32_t* d_csr_pos = nullptr;
    int32_t *d_sc_tile = nullptr, *d_pad_tile = nullptr;
    int16_t *d_sc_off = nullptr, *d_pad_off = nullptr;
    int32_t *d_n2o = nullptr, *d_o2n = nullptr;
    double* d_V = nullptr;
    // vectors (for up to vec_nrhs right-hand sides)
    double *d_borig = nullptr, *d_xorig = nullptr, *d_bext = nullptr, *d_xext = nullptr, *d_r = nullptr,
           *d_red = nullptr;
    float* d_v32 = nullptr;
    unsigned long long* d_cnt = nullptr;
    int epoch = 2;
    bool factored = false;
    float t_factor = 0, t_solve = 0;
    int grid_factor = 0;
    int64_t launches = 0;  // kernels launched by this system
    unsigned long long* trace = nullptr;  // optional timing trace (tasks, then block rows)
    uint64_t trace_bytes = 0;
    DevStatus last{};
    std::vector<Leaf> L, U;
};

namespace {

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
    double inf = INFINITY;
    std::memcpy(&s.min_pivot_bits, &inf, 8);
    return s;
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
    const int n_ext = p.cfg.n_ext(), n = p.cfg.n;
    const size_t nt = p.scatter_tile.size();
    std::vector<int64_t> key;
    std::vector<int32_t> trip;
    key.reserve(nt + (n_ext - n));
    for (size_t k = 0; k < nt; k++) {
        int32_t t = p.scatter_tile[k];
        if (t < 0) continue;
        int64_t row = (int64_t)p.input_bi[t] * 64 + p.scatter_off[k] / 64;
        int64_t col = (int64_t)p.input_bj[t] * 64 + p.scatter_off[k] % 64;
        key.push_back(row * n_ext + col);
        trip.push_back((int32_t)k);
    }
    for (int i = n; i < n_ext; i++) {
        key.push_back((int64_t)i * n_ext + i);
        trip.push_back(-1);
    }
    std::vector<int64_t> order(key.size());
    for (size_t i = 0; i < order.size(); i++) order[i] = (int64_t)i;
    std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return key[a] < key[b]; });
    h.ptr.assign(n_ext + 1, 0);
    h.col.resize(key.size());
    h.val.assign(key.size(), 0.0);
    h.pos.assign(nt, -1);
    for (size_t q = 0; q < order.size(); q++) {
        int64_t kk = key[order[q]];
        int row = (int)(kk / n_ext);
        h.col[q] = (int32_t)(kk % n_ext);
        h.ptr[row + 1]++;
        if (trip[order[q]] >= 0) h.pos[trip[order[q]]] = (int32_t)q;
        else h.val[q] = 1.0;
    }
    for (int i = 0; i < n_ext; i++) h.ptr[i + 1] += h.ptr[i];
    return h;
}

int ensure_vectors(sog_system* s, int nrhs) {
    if (nrhs <= s->vec_nrhs) return SOG_OK;
    if (s->vecs) s->ctx->pool.release(s->vecs, s->vec_bytes);
    s->vecs = nullptr;
    Layout L;
    const size_t ne = (size_t)s->n_ext * nrhs, no = (size_t)s->n * nrhs;
    uint64_t o_borig = L.add<double>(no), o_xorig = L.add<double>(no), o_bext = L.add<double>(ne),
             o_xext = L.add<double>(ne), o_r = L.add<double>(ne), o_red = L.add<double>((size_t)RED * nrhs),
             o_v32 = L.add<float>(ne), o_cnt = L.add<unsigned long long>(1);
    char* base = static_cast<char*>(s->ctx->pool.alloc(L.off));
    if (!base) return fail(SOG_ENOMEM, "block pool exhausted (solve vectors)");
    s->vecs = base;
    s->vec_bytes = L.off;
    s->vec_nrhs = nrhs;
    s->d_borig = (double*)(base + o_borig);
    s->d_xorig = (double*)(base + o_xorig);
    s->d_bext = (double*)(base + o_bext);
    s->d_xext = (double*)(base + o_xext);
    s->d_r = (double*)(base + o_r);
    s->d_red = (double*)(base + o_red);
    s->d_v32 = (float*)(base + o_v32);
    s->d_cnt = (unsigned long long*)(base + o_cnt);
    return SOG_OK;
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

int run_factor(sog_system* s) {
    sog_ctx* c = s->ctx;
    cudaStream_t st = c->stream;
    const TaskGraph& g = s->tg;
    DevStatus fs = fresh_status();
    // reset working state from pristine copies
    CK(cudaMemcpyAsync(s->dt.dep, s->d_ndep0, sizeof(int32_t) * g.ntasks, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(s->dt.parts_left, s->d_parts0, sizeof(int32_t) * g.ntasks, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemsetAsync(s->dt.queue, 0xff, sizeof(int32_t) * g.total_items, st));
    if (s->nready)
        CK(cudaMemcpyAsync(s->dt.queue, s->d_ready0, sizeof(int32_t) * s->nready, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(s->dt.head, s->d_counters0, sizeof(int32_t) * 3, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(s->dt.status, s->d_status0, sizeof(DevStatus), cudaMemcpyDeviceToDevice, st));
    (void)fs;
    if (s->trace) CK(cudaMemsetAsync(s->trace, 0, sizeof(unsigned long long) * 4 * g.ntasks, st));
    CK(cudaEventRecord(c->e0, st));
    int rc = 0;
    if (s->opt.executor == SOG_EXEC_LEVELS) {
        for (int l = 0; l < g.nlevels && rc == 0; l++) {
            const int a = g.level_ptr[l], b = g.level_ptr[l + 1];
            rc = s->fp64 ? factor_level_launch(s->dt, (double*)s->tiles, s->d_level_items + a, b - a, st)
                         : factor_level_launch(s->dt, (float*)s->tiles, s->d_level_items + a, b - a, st);
            s->launches++;
        }
    } else {
        rc = s->fp64 ? factor_persistent_launch(s->dt, (double*)s->tiles, s->grid_factor, st)
                     : factor_persistent_launch(s->dt, (float*)s->tiles, s->grid_factor, st);
        s->launches++;
    }
    if (rc) return fail(SOG_ECUDA, std::string("factor launch: ") + cudaGetErrorString(cudaGetLastError()));
    CK(cudaEventRecord(c->e1, st));
    CK(cudaStreamSynchronize(st));
    CK(cudaEventElapsedTime(&s->t_factor, c->e0, c->e1));
    int r = check_status(s, true);
    if (r) return r;
    s->factored = true;
    return SOG_OK;
}

int trisolve(sog_system* s, void* vec, int nrhs) {
    sog_ctx* c = s->ctx;
    const int grid = std::min(s->R, trisolve_grid(s->fp64, nrhs, c->num_sms));
    int nl = 0;
    int rc = s->fp64 ? trisolve_launch(s->ds, (const double*)s->tiles, (double*)vec, nrhs, s->epoch, grid, c->stream, nl)
                     : trisolve_launch(s->ds, (const float*)s->tiles, (float*)vec, nrhs, s->epoch, grid, c->stream, nl);
    s->launches += nl;
    if (rc) return fail(SOG_ECUDA, std::string("solve launch: ") + cudaGetErrorString(cudaGetLastError()));
    return SOG_OK;
}

struct Norms {
    double rel = 0, bwd = 0;
};
int read_norms(sog_system* s, int nrhs, Norms& out) {
    sog_ctx* c = s->ctx;
    CK(cudaMemcpyAsync(c->host_red, s->d_red, sizeof(double) * RED * nrhs, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    out = Norms();
    for (int k = 0; k < nrhs; k++) {
        const double* r = c->host_red + RED * k;
        double rel = r[1] > 0 ? std::sqrt(r[0]) / std::sqrt(r[1]) : std::sqrt(r[0]);
        double den = r[5] * r[3] + r[4];
        double bwd = den > 0 ? r[2] / den : r[2];
        if (!(rel <= out.rel)) out.rel = rel;  // NaN propagates
        if (!(bwd <= out.bwd)) out.bwd = bwd;
    }
    return SOG_OK;
}

// one chunk of <= 64 right-hand sides; b_ext already gathered into d_bext
int solve_chunk(sog_system* s, int nc, sog_solve_stats* stats) {
    sog_ctx* c = s->ctx;
    cudaStream_t st = c->stream;
    const int64_t ne = (int64_t)s->n_ext * nc;
    int r;
    Norms nm;
    int iters = 0;
    if (s->fp64) {
        CK(cudaMemcpyAsync(s->d_xext, s->d_bext, sizeof(double) * ne, cudaMemcpyDeviceToDevice, st));
        if ((r = trisolve(s, s->d_xext, nc))) return r;
        if (s->csr.ptr) {
            s->launches++;
            residual_launch(s->csr, s->d_bext, s->d_xext, s->d_r, nc, s->d_red, s->n, st);
            if ((r = read_norms(s, nc, nm))) return r;
        }
    } else {
        s->launches++;
        cast_f64_to_f32_launch(s->d_bext, s->d_v32, ne, st);
        if ((r = trisolve(s, s->d_v32, nc))) return r;
        s->launches++;
        axpy_f32_to_f64_launch(s->d_v32, s->d_xext, ne, 1, st);
        if (s->csr.ptr) {
            for (;;) {
                s->launches++;
                residual_launch(s->csr, s->d_bext, s->d_xext, s->d_r, nc, s->d_red, s->n, st);
                if ((r = read_norms(s, nc, nm))) return r;
                if (nm.rel <= s->opt.tol || iters >= s->opt.max_refine || std::isnan(nm.rel)) break;
                s->launches++;
                cast_f64_to_f32_launch(s->d_r, s->d_v32, ne, st);
                if ((r = trisolve(s, s->d_v32, nc))) return r;
                s->launches++;
                axpy_f32_to_f64_launch(s->d_v32, s->d_xext, ne, 0, st);
                iters++;
            }
        }
    }
    if ((r = check_status(s, false))) return r;
    if (stats) {
        stats->iterations = std::max(stats->iterations, iters);
        if (!(nm.rel <= stats->rel_resid)) stats->rel_resid = nm.rel;
        if (!(nm.bwd <= stats->backward_error)) stats->backward_error = nm.bwd;
    }
    if (!s->fp64 && s->csr.ptr && !(nm.rel <= s->opt.tol)) return SOG_ENOCONV;
    return SOG_OK;
}

int solve_device_impl(sog_system* s, int nrhs, const double* b_dev, double* x_dev, sog_solve_stats* stats) {
    sog_ctx* c = s->ctx;
    cudaStream_t st = c->stream;
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->min_pivot = bits_to_double(s->last.min_pivot_bits);
        stats->clamped_pivots = s->last.clamped;
    }
    int r = ensure_vectors(s, std::min(nrhs, 64));
    if (r) return r;
    CK(cudaEventRecord(c->e0, st));
    int worst = SOG_OK;
    for (int c0 = 0; c0 < nrhs; c0 += 64) {
        const int nc = std::min(64, nrhs - c0);
        s->launches++;
        gather_rhs_launch(b_dev + (size_t)c0 * s->n, s->d_n2o, s->n, s->n_ext, nc, s->d_bext, st);
        r = solve_chunk(s, nc, stats);
        if (r && r != SOG_ENOCONV) return r;
        if (r) worst = r;
        s->launches++;
        scatter_solution_launch(s->d_xext, s->d_o2n, s->n, nc, x_dev + (size_t)c0 * s->n, st);
    }
    CK(cudaEventRecord(c->e1, st));
    s->launches++;
    count_nonfinite_launch(x_dev, (int64_t)s->n * nrhs, s->d_cnt, st);
    unsigned long long bad = 0;
    CK(cudaMemcpyAsync(&bad, s->d_cnt, sizeof(bad), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    CK(cudaEventElapsedTime(&s->t_solve, c->e0, c->e1));
    if (stats) {
        stats->nan_count = (int64_t)bad;
        stats->status = worst;
    }
    if (bad) return fail(SOG_ENAN, "non-finite values in the solution");
    if (worst) return fail(worst, "iterative refinement did not reach the tolerance");
    return SOG_OK;
}

}  // namespace

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
        cudaEventCreate(&c->e0) != cudaSuccess || cudaEventCreate(&c->e1) != cudaSuccess ||
        cudaMallocHost(&c->host_red, sizeof(double) * RED * 64) != cudaSuccess) {
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
    if (c->host_red) cudaFreeHost(c->host_red);
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
    uint64_t tiles = (uint64_t)p.storage_count * 4096 * elem_bytes(o);
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
    if (o.executor != SOG_EXEC_PERSISTENT && o.executor != SOG_EXEC_LEVELS) return fail(SOG_EINVAL, "bad executor");
    if (o.tol <= 0) o.tol = 1e-10;
    if (o.max_refine < 0) o.max_refine = 0;
    CK(cudaSetDevice(c->device));
    const Plan& p = plan->p;
    sog_system* s = new sog_system();
    s->ctx = c;
    s->opt = o;
    s->fp64 = o.precision == SOG_FP64;
    s->imported = plan->imported;
    s->n = p.cfg.n;
    s->n_ext = p.cfg.n_ext();
    s->R = p.cfg.block_rows;
    s->n_input = p.n_input;
    s->storage = p.storage_count;
    s->ntrip = (int64_t)p.scatter_tile.size();
    s->npad = (int64_t)p.pad_tile.size();
    s->L = p.L;
    s->U = p.U;
    int gemm_parts = o.gemm_split == 1 ? 1 : (o.gemm_split == 4 ? 4 : (s->fp64 ? 4 : 1));
    if (!s->fp64) gemm_parts = 1;
    // inverses of the diagonal factor blocks for the substitution (reused
    // where the DAG already computes them)
    std::vector<Op> ops2 = p.ops;
    int32_t storage2 = p.storage_count;
    std::vector<int32_t> ldinv, udinv;
    add_diag_inverses(ops2, storage2, s->R, p.L, p.U, ldinv, udinv);
    s->storage = storage2;
    std::vector<int32_t> outputs;
    for (const Leaf& lf : p.L) outputs.push_back(lf.id);
    for (const Leaf& lf : p.U) outputs.push_back(lf.id);
    for (int32_t id : ldinv) if (id > 0) outputs.push_back(id);
    for (int32_t id : udinv) if (id > 0) outputs.push_back(id);
    try {
        s->tg = build_tasks(ops2, storage2, p.n_input, outputs, gemm_parts);
    } catch (const std::exception& e) {
        delete s;
        return fail(SOG_EINVAL, std::string("DAG: ") + e.what());
    }
    const TaskGraph& g = s->tg;
    // solve structure
    std::vector<int32_t> lptr(s->R + 1, 0), uptr(s->R + 1, 0), ldiag(s->R, 0), udiag(s->R, 0);
    std::vector<Leaf> loff, uoff;
    for (const Leaf& lf : p.L) {
        if (lf.bi == lf.bj) ldiag[lf.bi] = lf.id;
        else if (lf.bj < lf.bi) loff.push_back(lf);
    }
    for (const Leaf& lf : p.U) {
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
    HostCSR hc;
    if (!plan->imported) hc = build_csr(p);
    // task arrays
    std::vector<int32_t> parts32(g.ntasks);
    for (int32_t t = 0; t < g.ntasks; t++) parts32[t] = g.parts[t];
    std::vector<int32_t> counters0 = {0, (int32_t)g.ready_items.size(), 0};
    std::vector<DevStatus> st0 = {fresh_status()};
    Layout L;
    uint64_t o_kind = L.add<uint8_t>(g.ntasks), o_parts = L.add<uint8_t>(g.ntasks), o_out = L.add<int32_t>(g.ntasks),
             o_out2 = L.add<int32_t>(g.ntasks), o_a = L.add<int32_t>(g.ntasks), o_b = L.add<int32_t>(g.ntasks),
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
             o_flags = L.add<int32_t>(s->R), o_cptr = L.add<int32_t>(hc.ptr.size()),
             o_ccol = L.add<int32_t>(hc.col.size()), o_cval = L.add<double>(hc.val.size()),
             o_cpos = L.add<int32_t>(hc.pos.size()), o_sct = L.add<int32_t>(p.scatter_tile.size()),
             o_sco = L.add<int16_t>(p.scatter_off.size()), o_pdt = L.add<int32_t>(p.pad_tile.size()),
             o_pdo = L.add<int16_t>(p.pad_off.size()), o_n2o = L.add<int32_t>(p.ord.new_to_old.size()),
             o_o2n = L.add<int32_t>(p.ord.old_to_new.size()), o_V = L.add<double>(s->ntrip);
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
    cudaStream_t st = c->stream;
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
    s->d_status0 = put(A, o_st0, st0, st);
    dt.status = reinterpret_cast<DevStatus*>(A + o_st);
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
    cudaMemsetAsync(ds.flags, 0, sizeof(int32_t) * s->R, st);
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
    s->d_n2o = put(A, o_n2o, p.ord.new_to_old, st);
    s->d_o2n = put(A, o_o2n, p.ord.old_to_new, st);
    s->d_V = reinterpret_cast<double*>(A + o_V);
    s->grid_factor = factor_persistent_grid(s->fp64, c->num_sms);
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
    cudaStreamSynchronize(c->stream);
    c->pool.release(s->tiles, s->tiles_bytes);
    c->pool.release(s->aux, s->aux_bytes);
    c->pool.release(s->vecs, s->vec_bytes);
    c->pool.release(s->trace, s->trace_bytes);
    delete s;
}

int sog_factor_device(sog_system* s, const double* V_dev) {
    if (!s) return fail(SOG_EINVAL, "NULL system");
    if (s->imported) return fail(SOG_ESTATE, "imported plan: use sog_factor_tiles");
    if (!V_dev && s->ntrip) return fail(SOG_EINVAL, "NULL values");
    sog_ctx* c = s->ctx;
    CK(cudaSetDevice(c->device));
    cudaStream_t st = c->stream;
    const uint64_t eb = elem_bytes(s->opt);
    CK(cudaMemsetAsync((char*)s->tiles + 4096 * eb, 0, (uint64_t)s->n_input * 4096 * eb, st));
    // input tile k (0-based, as the scatter map counts) is block id k+1
    s->launches++;
    scatter_values_launch(V_dev, s->d_sc_tile, s->d_sc_off, s->ntrip, s->d_pad_tile, s->d_pad_off, s->npad,
                          s->fp64 ? (double*)s->tiles + 4096 : nullptr, s->fp64 ? nullptr : (float*)s->tiles + 4096,
                          st);
    s->launches++;
    scatter_csr_launch(V_dev, s->d_csr_pos, s->ntrip, s->d_csr_val, st);
    return run_factor(s);
}

int sog_factor(sog_system* s, const double* V) {
    if (!s) return fail(SOG_EINVAL, "NULL system");
    if (s->imported) return fail(SOG_ESTATE, "imported plan: use sog_factor_tiles");
    if (!V && s->ntrip) return fail(SOG_EINVAL, "NULL values");
    CK(cudaSetDevice(s->ctx->device));
    if (s->ntrip)
        CK(cudaMemcpyAsync(s->d_V, V, sizeof(double) * s->ntrip, cudaMemcpyHostToDevice, s->ctx->stream));
    return sog_factor_device(s, s->d_V);
}

int sog_factor_tiles(sog_system* s, const double* tiles) {
    if (!s || !tiles) return fail(SOG_EINVAL, "NULL argument");
    sog_ctx* c = s->ctx;
    CK(cudaSetDevice(c->device));
    const uint64_t n = (uint64_t)s->n_input * 4096;
    if (s->fp64) {
        CK(cudaMemcpyAsync((double*)s->tiles + 4096, tiles, n * 8, cudaMemcpyHostToDevice, c->stream));
    } else {
        double* stage = static_cast<double*>(c->pool.alloc(n * 8));
        if (!stage) return fail(SOG_ENOMEM, "block pool exhausted (staging)");
        CK(cudaMemcpyAsync(stage, tiles, n * 8, cudaMemcpyHostToDevice, c->stream));
        s->launches++;
        convert_tiles_launch(stage, (float*)s->tiles + 4096, (int64_t)n, c->stream);
        CK(cudaStreamSynchronize(c->stream));
        c->pool.release(stage, n * 8);
    }
    return run_factor(s);
}

int sog_solve_device(sog_system* s, int32_t nrhs, const double* b_dev, double* x_dev, sog_solve_stats* stats) {
    if (!s || nrhs <= 0 || !b_dev || !x_dev) return fail(SOG_EINVAL, "bad argument");
    if (!s->factored) return fail(SOG_ESTATE, "solve before factor");
    CK(cudaSetDevice(s->ctx->device));
    return solve_device_impl(s, nrhs, b_dev, x_dev, stats);
}

int sog_solve(sog_system* s, int32_t nrhs, const double* b, double* x, sog_solve_stats* stats) {
    if (!s || nrhs <= 0 || !b || !x) return fail(SOG_EINVAL, "bad argument");
    if (!s->factored) return fail(SOG_ESTATE, "solve before factor");
    sog_ctx* c = s->ctx;
    CK(cudaSetDevice(c->device));
    const uint64_t bytes = sizeof(double) * (uint64_t)s->n * nrhs;
    double* db = static_cast<double*>(c->pool.alloc(bytes));
    double* dx = static_cast<double*>(c->pool.alloc(bytes));
    if (!db || !dx) {
        c->pool.release(db, bytes);
        c->pool.release(dx, bytes);
        return fail(SOG_ENOMEM, "block pool exhausted (rhs)");
    }
    int r = SOG_OK;
    if (cudaMemcpyAsync(db, b, bytes, cudaMemcpyHostToDevice, c->stream) != cudaSuccess)
        r = fail(SOG_ECUDA, "rhs upload failed");
    if (!r || r == SOG_ENOCONV) {
        r = solve_device_impl(s, nrhs, db, dx, stats);
        if (!r || r == SOG_ENOCONV || r == SOG_ENAN) {
            if (cudaMemcpyAsync(x, dx, bytes, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
                cudaStreamSynchronize(c->stream) != cudaSuccess)
                r = fail(SOG_ECUDA, "download failed");
        }
    }
    c->pool.release(db, bytes);
    c->pool.release(dx, bytes);
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
    CK(cudaMemcpyAsync(s->d_xext, b_ext, ne * 8, cudaMemcpyHostToDevice, c->stream));
    CK(cudaEventRecord(c->e0, c->stream));
    if (s->fp64) {
        if ((r = trisolve(s, s->d_xext, 1))) return r;
    } else {
        s->launches++;
        cast_f64_to_f32_launch(s->d_xext, s->d_v32, ne, c->stream);
        if ((r = trisolve(s, s->d_v32, 1))) return r;
        s->launches++;
        axpy_f32_to_f64_launch(s->d_v32, s->d_xext, ne, 1, c->stream);
    }
    CK(cudaEventRecord(c->e1, c->stream));
    CK(cudaMemcpyAsync(x_ext, s->d_xext, ne * 8, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaEventElapsedTime(&s->t_solve, c->e0, c->e1));
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
        if (!dst) continue;
        for (size_t k = 0; k < lv.size(); k++) {
            const char* src = (const char*)s->tiles + (uint64_t)lv[k].id * 4096 * eb;
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
    return SOG_OK;
}

int sog_debug_unpoison(sog_system* s) {
    if (!s) return fail(SOG_EINVAL, "bad argument");
    CK(cudaSetDevice(s->ctx->device));
    CK(cudaMemcpy(s->d_ndep0, s->tg.ndep.data(), sizeof(int32_t) * s->tg.ntasks, cudaMemcpyHostToDevice));
    return SOG_OK;
}

int sog_system_trace_enable(sog_system* s, int32_t on) {
    if (!s) return fail(SOG_EINVAL, "NULL system");
    sog_ctx* c = s->ctx;
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
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
    if (!s || !s->trace) return fail(SOG_ESTATE, "trace not enabled");
    CK(cudaSetDevice(s->ctx->device));
    CK(cudaStreamSynchronize(s->ctx->stream));
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
        std::vector<Op> ops2 = p.ops;
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
        counts[9] = g.fused_subs;
        counts[10] = storage2 - p.storage_count;
        counts[11] = g.ntasks ? *std::max_element(g.prio.begin(), g.prio.end()) + 1 : 0;
        counts[12] = g.fused_inverses;
    } catch (const std::exception& e) {
        return fail(SOG_EINVAL, std::string("DAG: ") + e.what());
    }
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
    sog_system* s = nullptr;
    r = sog_system_create(c, plan, &o, &s);
    if (!r) {
        std::vector<int32_t> Io, Jo;
        std::vector<double> Vo;
        mirror_triplets(dim, valcount, symmetric != 0, index_i, index_j, vals, Io, Jo, Vo);
        r = sog_factor(s, Vo.data());
        if (!r) r = sog_solve(s, 1, b, x_out, nullptr);
        sog_system_destroy(s);
    }
    sog_ctx_destroy(c);
    sog_plan_destroy(plan);
    return r;
}

}  // extern "C"
