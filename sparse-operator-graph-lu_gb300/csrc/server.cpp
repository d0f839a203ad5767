// Serving engine: a request loop over the executor with continuous batching.
//
// No counterpart in the reference, which solves one system per process
// (main.cpp, solver.cpp:121). Requests (a sparse system and its right-hand
// sides) are planned on host worker threads as they arrive. A scheduler
// thread admits planned requests (first come, first served, as far as the
// block pool can hold them) to the first free lane, merging those that are
// waiting into one batch plan. Each lane is a host thread with its own CUDA
// stream: it factors its batch in one executor launch and solves all the
// batch's right-hand sides in shared substitution launches. Lanes run at the
// same time, so a request that arrives while another batch is on the GPU
// starts on a free lane at once and its kernels run beside the other
// batch's; each batch's persistent grid is sized to its task graph's
// parallelism and, while other lanes exist, leaves a quarter of the GPU to
// them. Factors stay resident after the answer, for further right-hand sides,
// until the request is released; a batch's pool memory returns when all its
// requests are.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "api_internal.h"

using sog_internal::fail;

namespace {

using Clock = std::chrono::steady_clock;
double ms_since(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

enum ReqState { R_QUEUED, R_PLANNING, R_PLANNED, R_RUNNING, R_DONE, R_FAILED };

struct Batch;

struct Request {
    int64_t id = 0;
    int32_t n = 0, nrhs = 0;
    bool symmetric = false;
    std::vector<int32_t> I, J;
    std::vector<double> V, b, x;
    sog_plan* plan = nullptr;
    uint64_t bytes = 0;
    ReqState state = R_QUEUED;
    int status = SOG_OK;
    std::string err;
    sog_solve_stats stats{};
    std::shared_ptr<Batch> batch;
    int seg = 0;
    bool released = false;
    int jobs = 0;  // further solves queued or running
    Clock::time_point t_submit, t_planned, t_start, t_done;
    double plan_ms = 0, setup_ms = 0, gpu_ms = 0;
};

struct Batch {
    int64_t id = 0;
    sog_plan* plan = nullptr;
    sog_system* sys = nullptr;
    std::vector<Request*> members;
    int live = 0;
    ~Batch() {
        if (sys) sog_system_destroy(sys);
        if (plan) sog_plan_destroy(plan);
    }
};

// a further solve on resident factors, executed by the scheduler thread
struct SolveJob {
    Request* r = nullptr;
    int32_t nrhs = 0;
    const double* b = nullptr;
    double* x = nullptr;
    sog_solve_stats stats{};
    int status = SOG_OK;
    std::string err;
    bool done = false;
};

}  // namespace

struct sog_server {
    // a host thread and stream that run one batch at a time
    struct Lane {
        std::thread th;
        cudaStream_t stream = nullptr;
        std::vector<Request*> group;  // assigned by the scheduler, taken by the lane
        bool busy = false;
        uint64_t reserved = 0;  // pool bytes promised to its group until its system exists
    };
    sog_ctx* ctx = nullptr;
    sog_options opt{};
    sog_server_options sopt{};
    std::mutex mu;
    std::condition_variable cv_work;   // planners and scheduler wait here
    std::condition_variable cv_done;   // callers of wait / solve wait here
    bool stop = false;
    int64_t next_id = 1, next_batch = 1;
    std::map<int64_t, std::unique_ptr<Request>> reqs;
    std::deque<Request*> to_plan, planned;
    std::deque<SolveJob*> jobs;
    std::vector<std::shared_ptr<Batch>> dead;  // batches whose requests are all released
    int freeing = 0;  // batches taken from dead that the scheduler is destroying right now
    uint64_t mem_gen = 0;  // counts the returns of pool memory (released batches destroyed)
    std::vector<std::thread> planners;
    std::thread sched;
    std::vector<Lane> lanes;
    std::condition_variable cv_lane;  // lanes wait here for a group
    uint64_t reserved_total = 0;      // sum of the lanes' reservations
    bool mem_blocked = false;         // a lone request waits for pool memory held by resident requests
    // counters
    int64_t batches = 0, admitted = 0, completed = 0, rejected = 0;
    int64_t max_batch_seen = 0;
    int planning = 0;  // requests being planned right now

    void planner_loop();
    void scheduler_loop();
    void lane_loop(int k);
    // 0 = ran (or failed for good); 1 = too little pool memory: retry with the
    // group shrunk to its first half; 2 = single request blocked on memory
    // held by resident requests: wait for a release
    int run_batch(std::vector<Request*>& group, int lane);
    bool any_resident() const {
        for (auto& kv : reqs)
            if (kv.second->batch) return true;
        return false;
    }
};

void sog_server::planner_loop() {
    for (;;) {
        Request* r = nullptr;
        {
            std::unique_lock<std::mutex> lk(mu);
            cv_work.wait(lk, [&] { return stop || !to_plan.empty(); });
            if (stop) return;
            r = to_plan.front();
            to_plan.pop_front();
            r->state = R_PLANNING;
            planning++;
        }
        const Clock::time_point t0 = Clock::now();
        sog_plan* p = nullptr;
        int rc = sog_plan_build(r->n, (int64_t)r->I.size(), r->symmetric ? 1 : 0, r->I.data(), r->J.data(), r->V.data(),
                                sopt.planner_omp_threads, &p);
        std::string err = rc ? sog_last_error() : "";
        uint64_t bytes = 0;
        if (!rc) rc = sog_system_bytes(p, &opt, &bytes);
        std::lock_guard<std::mutex> lk(mu);
        planning--;
        r->plan_ms = ms_since(t0, Clock::now());
        r->t_planned = Clock::now();
        if (rc) {
            if (p) sog_plan_destroy(p);
            r->state = R_FAILED;
            r->status = rc;
            r->err = err.empty() ? "planning failed" : err;
            r->t_done = r->t_planned;
            rejected++;
            cv_done.notify_all();
            continue;
        }
        r->plan = p;
        // pool need with a margin for the batch's solve vectors and alignment
        r->bytes = bytes + bytes / 16 + (8ull << 20);
        r->state = R_PLANNED;
        planned.push_back(r);
        cv_work.notify_all();
    }
}

int sog_server::run_batch(std::vector<Request*>& group, int lane) {
    auto bt = std::make_shared<Batch>();
    // a lone request runs on its own plan (a merge would copy it); the plan
    // goes back to the request if the batch is requeued
    const bool single = group.size() == 1;
    int rc = SOG_OK;
    if (single) {
        bt->plan = group[0]->plan;
        group[0]->plan = nullptr;
    } else {
        std::vector<const sog_plan*> plans;
        for (Request* r : group) plans.push_back(r->plan);
        rc = sog_plan_merge(plans.data(), (int32_t)plans.size(), &bt->plan);
    }
    uint64_t gen0;
    {
        std::lock_guard<std::mutex> lk(mu);
        gen0 = mem_gen;
    }
    if (!rc) rc = sog_system_create(ctx, bt->plan, &opt, &bt->sys);
    if (rc == SOG_ENOMEM) {  // chunks left empty by released batches go back to the device first
        sog_ctx_trim(ctx);
        rc = sog_system_create(ctx, bt->plan, &opt, &bt->sys);
    }
    {
        std::lock_guard<std::mutex> lk(mu);  // the system exists (or failed): its pool use is counted now
        reserved_total -= lanes[lane].reserved;
        lanes[lane].reserved = 0;
    }
    if (!rc) {
        // this lane's stream; a grid for the batch's parallelism, leaving a
        // quarter of the GPU to the other lanes
        rc = sog_system_set_stream(bt->sys, lanes[lane].stream);
        int full = 0;
        const double par = sog_internal::system_parallelism(bt->sys, &full);
        int cap = std::max(16, (int)(3.0 * par));
        if (lanes.size() > 1) cap = std::min(cap, std::max(1, 3 * full / 4));
        sog_internal::system_set_grid_cap(bt->sys, cap < full ? cap : 0);
    }
    if (rc == SOG_ENOMEM) {
        std::lock_guard<std::mutex> lk(mu);
        if (group.size() > 1) {
            // the admission estimate was optimistic (fragmentation): requeue
            // the second half in order, retry with the first
            const size_t keep = group.size() / 2;
            for (size_t k = group.size(); k-- > keep;) {
                group[k]->state = R_PLANNED;
                planned.push_front(group[k]);
            }
            group.resize(keep);
            return 1;
        }
        // memory still held by resident requests, by released batches the
        // scheduler has not freed yet, or by other lanes' batches: wait for it
        // instead of failing; memory returned since the attempt: retry at once
        bool others = false;
        for (size_t k = 0; k < lanes.size(); k++) others = others || ((int)k != lane && lanes[k].busy);
        const bool returned = mem_gen != gen0;
        if (returned || any_resident() || !dead.empty() || freeing > 0 || others) {
            if (single) {
                group[0]->plan = bt->plan;
                bt->plan = nullptr;
            }
            group[0]->state = R_PLANNED;
            planned.push_front(group[0]);
            group.clear();
            mem_blocked = !returned;
            return 2;
        }
    }
    std::vector<double> V, B;
    std::vector<int32_t> cnt;
    for (Request* r : group) {
        V.insert(V.end(), r->V.begin(), r->V.end());
        B.insert(B.end(), r->b.begin(), r->b.end());
        cnt.push_back(r->nrhs);
    }
    std::vector<double> X(B.size());
    std::vector<sog_solve_stats> st(group.size());
    std::string err;
    const Clock::time_point t0 = Clock::now();
    for (Request* r : group) r->setup_ms = ms_since(r->t_start, t0);
    if (!rc) rc = sog_factor(bt->sys, V.data());
    // a system that failed the pivot gate is answered with SOG_EPIVOT (and its
    // solution); the batch's other systems are not affected
    std::vector<sog_solve_stats> piv;
    if (rc == SOG_EPIVOT) {
        piv.resize(group.size());
        rc = sog_system_pivots(bt->sys, piv.data());
    }
    if (!rc || rc == SOG_ENOCONV) {
        const int r2 = sog_solve_batch(bt->sys, cnt.data(), B.data(), X.data(), st.data());
        if (!rc) rc = r2;
    }
    // further solves on these factors (sog_server_solve, scheduler thread) run
    // on the context's stream, beside the lanes
    if (bt->sys) {
        sog_internal::system_set_grid_cap(bt->sys, 0);
        sog_system_set_stream(bt->sys, nullptr);
    }
    if (rc) err = sog_last_error();
    const Clock::time_point t1 = Clock::now();
    std::lock_guard<std::mutex> lk(mu);
    batches++;
    max_batch_seen = std::max<int64_t>(max_batch_seen, (int64_t)group.size());
    bt->id = next_batch++;
    size_t o = 0;
    for (size_t k = 0; k < group.size(); k++) {
        Request* r = group[k];
        const size_t m = (size_t)r->nrhs * r->n;
        r->x.assign(X.begin() + o, X.begin() + o + m);
        o += m;
        r->stats = st[k];
        r->gpu_ms = ms_since(t0, t1);
        r->t_done = t1;
        // a request's own status: its refinement result, or the batch's failure
        r->status = (rc == SOG_OK || rc == SOG_ENOCONV || rc == SOG_ENAN) ? st[k].status : rc;
        if (rc && rc != SOG_ENOCONV && rc != SOG_ENAN) r->err = err;
        else if (r->status) r->err = "refinement did not reach the tolerance or the solution is not finite";
        else if (!piv.empty() && piv[k].status == SOG_EPIVOT) {
            r->status = SOG_EPIVOT;
            r->err = "pivot check failed (clamped pivot, U*U^-1 check or growth above the limit); solution returned";
        }
        r->state = r->status == SOG_OK || r->status == SOG_ENOCONV || r->status == SOG_ENAN ||
                           r->status == SOG_EPIVOT
                       ? R_DONE
                       : R_FAILED;
        r->seg = (int)k;
        sog_plan_destroy(r->plan);
        r->plan = nullptr;
        r->V.clear();
        r->V.shrink_to_fit();
        completed++;
        if (r->state == R_DONE && bt->sys) {
            r->batch = bt;
            bt->members.push_back(r);
            bt->live++;
            if (r->released) bt->live--;  // released while running
        }
    }
    if (bt->live == 0) dead.push_back(bt);
    cv_done.notify_all();
    return 0;
}

void sog_server::lane_loop(int k) {
    for (;;) {
        std::vector<Request*> group;
        {
            std::unique_lock<std::mutex> lk(mu);
            cv_lane.wait(lk, [&] { return stop || !lanes[k].group.empty(); });
            if (stop) return;
            group.swap(lanes[k].group);
        }
        int rb;
        while ((rb = run_batch(group, k)) == 1) {
        }
        {
            std::lock_guard<std::mutex> lk(mu);
            reserved_total -= lanes[k].reserved;
            lanes[k].reserved = 0;
            lanes[k].busy = false;
            if (rb != 2) mem_blocked = false;  // this lane's memory use is settled: a blocked request may fit
        }
        cv_work.notify_all();
    }
}

void sog_server::scheduler_loop() {
    for (;;) {
        std::vector<std::shared_ptr<Batch>> to_free;
        SolveJob* job = nullptr;
        int lane = -1;
        {
            std::unique_lock<std::mutex> lk(mu);
            auto free_lane = [&] {
                for (size_t k = 0; k < lanes.size(); k++)
                    if (!lanes[k].busy) return (int)k;
                return -1;
            };
            cv_work.wait(lk, [&] {
                return stop || !jobs.empty() || !dead.empty() ||
                       (!planned.empty() && !mem_blocked && free_lane() >= 0);
            });
            if (stop) return;
            to_free.swap(dead);
            freeing = (int)to_free.size();  // their memory is on its way back
            if (!jobs.empty()) {
                job = jobs.front();
                jobs.pop_front();
            } else if (!planned.empty() && !mem_blocked) {
                lane = free_lane();
            }
        }
        if (!to_free.empty()) {
            to_free.clear();  // destroys systems (on the context's stream)
            std::lock_guard<std::mutex> lk(mu);
            freeing = 0;
            mem_gen++;
            mem_blocked = false;  // memory returned: a blocked request may fit now
        }
        if (job) {
            Request* r = job->r;
            int32_t ns = 0;
            sog_plan_segments(r->batch->plan, &ns, nullptr);
            std::vector<int32_t> cnt(ns, 0);
            cnt[r->seg] = job->nrhs;
            // other systems' blocks get no right-hand sides: b / x cover this request only
            std::vector<sog_solve_stats> st(ns);
            const int rc = sog_solve_batch(r->batch->sys, cnt.data(), job->b, job->x, st.data());
            std::lock_guard<std::mutex> lk(mu);
            job->status = rc;
            if (rc) job->err = sog_last_error();
            job->stats = st[r->seg];
            job->done = true;
            r->jobs--;
            cv_done.notify_all();
            continue;
        }
        if (lane < 0) continue;
        std::unique_lock<std::mutex> lk(mu);
        if (planned.empty() || lanes[lane].busy) continue;
        // batching window: give requests still being planned a chance to
        // join this launch
        if (sopt.batch_window_ms > 0) {
            const Clock::time_point until =
                planned.front()->t_planned +
                std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double, std::milli>(
                    sopt.batch_window_ms));
            cv_work.wait_until(lk, until, [&] { return stop || (to_plan.empty() && planning == 0); });
            if (stop) return;
            if (planned.empty()) continue;
        }
        uint64_t used = 0, total = 0;
        sog_ctx_pool_usage(ctx, &used, &total);
        const uint64_t taken = used + reserved_total;
        uint64_t avail = total > taken ? total - taken : 0, need = 0;
        const int cap = sopt.max_batch > 0 ? sopt.max_batch : 256;
        std::vector<Request*> group;
        while (!planned.empty() && (int)group.size() < cap) {
            Request* r = planned.front();
            if (need + r->bytes > avail) break;
            need += r->bytes;
            group.push_back(r);
            planned.pop_front();
        }
        if (group.empty()) {
            Request* r = planned.front();
            bool others = false;
            for (auto& ln : lanes) others = others || ln.busy;
            if (!any_resident() && dead.empty() && freeing == 0 && !others) {
                // larger than the whole pool: refuse it rather than wait forever
                planned.pop_front();
                r->state = R_FAILED;
                r->status = SOG_ENOMEM;
                r->err = "request does not fit in the block pool";
                r->t_done = Clock::now();
                sog_plan_destroy(r->plan);
                r->plan = nullptr;
                rejected++;
                cv_done.notify_all();
            } else {
                mem_blocked = true;  // until a batch is freed or a lane finishes
            }
            continue;
        }
        for (Request* r : group) {
            r->state = R_RUNNING;
            r->t_start = Clock::now();
        }
        admitted += (int64_t)group.size();
        lanes[lane].busy = true;
        lanes[lane].reserved = need;
        reserved_total += need;
        lanes[lane].group.swap(group);
        cv_lane.notify_all();
    }
}

extern "C" {

int sog_server_create(sog_ctx* ctx, const sog_options* opt, const sog_server_options* sopt, sog_server** out) {
    if (!ctx || !out) return fail(SOG_EINVAL, "NULL argument");
    *out = nullptr;
    sog_server* s = new sog_server();
    s->ctx = ctx;
    if (opt) s->opt = *opt;
    else {
        std::memset(&s->opt, 0, sizeof(s->opt));
        s->opt.precision = SOG_MIXED;
        s->opt.max_refine = 10;
        s->opt.tol = 1e-10;
    }
    // resident requests keep only what their further solves read
    s->opt.resident_compact = 1;
    if (sopt) s->sopt = *sopt;
    const int np = s->sopt.planner_threads > 0 ? s->sopt.planner_threads : 2;
    const int nl = s->sopt.lanes > 0 ? s->sopt.lanes : 2;
    s->lanes.resize(nl);
    for (auto& ln : s->lanes)
        if (cudaStreamCreateWithFlags(&ln.stream, cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            for (auto& l2 : s->lanes)
                if (l2.stream) cudaStreamDestroy(l2.stream);
            delete s;
            return fail(SOG_ECUDA, "server lane streams");
        }
    try {
        for (int k = 0; k < np; k++) s->planners.emplace_back([s] { s->planner_loop(); });
        for (int k = 0; k < nl; k++) s->lanes[k].th = std::thread([s, k] { s->lane_loop(k); });
        s->sched = std::thread([s] { s->scheduler_loop(); });
    } catch (const std::exception& e) {
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stop = true;
        }
        s->cv_work.notify_all();
        s->cv_lane.notify_all();
        for (auto& t : s->planners) t.join();
        for (auto& ln : s->lanes)
            if (ln.th.joinable()) ln.th.join();
        for (auto& ln : s->lanes) cudaStreamDestroy(ln.stream);
        delete s;
        return fail(SOG_EINVAL, std::string("server threads: ") + e.what());
    }
    *out = s;
    return SOG_OK;
}

int sog_server_submit(sog_server* s, int32_t n, int64_t nnz, const int32_t* I, const int32_t* J, const double* V,
                      int32_t symmetric, int32_t nrhs, const double* b, int64_t* id) {
    if (!s || !id || n <= 0 || nnz < 0 || nrhs <= 0 || !b || (nnz > 0 && (!I || !J || !V)))
        return fail(SOG_EINVAL, "bad request");
    auto r = std::make_unique<Request>();
    r->n = n;
    r->nrhs = nrhs;
    r->symmetric = symmetric != 0;
    r->I.assign(I, I + nnz);
    r->J.assign(J, J + nnz);
    r->V.assign(V, V + nnz);
    r->b.assign(b, b + (size_t)nrhs * n);
    r->t_submit = Clock::now();
    std::lock_guard<std::mutex> lk(s->mu);
    r->id = s->next_id++;
    *id = r->id;
    s->to_plan.push_back(r.get());
    s->reqs[r->id] = std::move(r);
    s->cv_work.notify_all();
    return SOG_OK;
}

int sog_server_wait(sog_server* s, int64_t id, double timeout_ms, double* x, sog_request_info* info) {
    if (!s) return fail(SOG_EINVAL, "NULL server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return fail(SOG_EINVAL, "unknown request");
    Request* r = it->second.get();
    auto ready = [&] { return r->state == R_DONE || r->state == R_FAILED; };
    if (timeout_ms < 0) s->cv_done.wait(lk, ready);
    else if (!s->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), ready))
        return fail(SOG_ETIMEOUT, "request still running");
    if (x && r->state == R_DONE) std::memcpy(x, r->x.data(), sizeof(double) * r->x.size());
    if (info) {
        std::memset(info, 0, sizeof(*info));
        info->status = r->status;
        info->stats = r->stats;
        info->batch_id = r->batch ? r->batch->id : 0;
        info->batch_size = r->batch ? (int32_t)r->batch->members.size() : 0;
        info->plan_ms = r->plan_ms;
        info->queue_ms = r->state == R_DONE ? ms_since(r->t_planned, r->t_start) : 0;
        info->setup_ms = r->setup_ms;
        info->gpu_ms = r->gpu_ms;
        info->total_ms = ms_since(r->t_submit, r->t_done);
    }
    if (r->status && r->status != SOG_ENOCONV) return fail(r->status, r->err);
    return r->status;
}

int sog_server_solve(sog_server* s, int64_t id, int32_t nrhs, const double* b, double* x, sog_solve_stats* stats) {
    if (!s || nrhs <= 0 || !b || !x) return fail(SOG_EINVAL, "bad argument");
    SolveJob job;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        auto it = s->reqs.find(id);
        if (it == s->reqs.end()) return fail(SOG_EINVAL, "unknown request");
        Request* r = it->second.get();
        if (r->state != R_DONE || !r->batch || r->released) return fail(SOG_ESTATE, "no resident factors");
        job.r = r;
        r->jobs++;
        job.nrhs = nrhs;
        job.b = b;
        job.x = x;
        s->jobs.push_back(&job);
        s->cv_work.notify_all();
        s->cv_done.wait(lk, [&] { return job.done; });
    }
    if (stats) *stats = job.stats;
    if (job.status && job.status != SOG_ENOCONV) return fail(job.status, job.err);
    return job.status;
}

int sog_server_release(sog_server* s, int64_t id) {
    if (!s) return fail(SOG_EINVAL, "NULL server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return fail(SOG_EINVAL, "unknown request");
    Request* r = it->second.get();
    if ((r->state != R_DONE && r->state != R_FAILED) || r->jobs)
        return fail(SOG_ESTATE, "request still running");
    if (!r->released && r->batch) {
        r->released = true;
        if (--r->batch->live == 0) s->dead.push_back(r->batch);
        s->cv_work.notify_all();
    }
    r->batch.reset();
    s->reqs.erase(it);
    return SOG_OK;
}

int sog_server_counters(sog_server* s, int64_t* counts) {
    if (!s || !counts) return fail(SOG_EINVAL, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    int64_t resident = 0;
    for (auto& kv : s->reqs)
        if (kv.second->batch) resident++;
    counts[0] = s->batches;
    counts[1] = s->admitted;
    counts[2] = s->completed;
    counts[3] = s->rejected;
    counts[4] = s->max_batch_seen;
    counts[5] = resident;
    counts[6] = (int64_t)s->planned.size();
    counts[7] = (int64_t)s->to_plan.size();
    return SOG_OK;
}

void sog_server_destroy(sog_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    s->cv_lane.notify_all();
    for (auto& t : s->planners) t.join();
    if (s->sched.joinable()) s->sched.join();
    // a lane finishes the batch it is running (its requests are answered)
    for (auto& ln : s->lanes)
        if (ln.th.joinable()) ln.th.join();
    for (auto& ln : s->lanes) {
        cudaStreamSynchronize(ln.stream);
        cudaStreamDestroy(ln.stream);
    }
    // in-flight work ends with the scheduler; drop the resident batches
    s->dead.clear();
    for (auto& kv : s->reqs) {
        if (kv.second->plan) sog_plan_destroy(kv.second->plan);
        kv.second->batch.reset();
    }
    s->reqs.clear();
    delete s;
}

}  // extern "C"
