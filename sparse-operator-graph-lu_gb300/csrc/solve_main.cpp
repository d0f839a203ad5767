// ./solve file.mtx [options] — the reference's command line front end
// (main.cpp:34-66) on the GB300 executor.
//
// Reads file.mtx and file_b.mtx (missing entries = 1, mtx.cpp:145-181),
// plans on the host, factors and solves on the GPU, prints the reference's
// phase lines and the max |b - A x| check (mtx.cpp:183-215), and writes the
// solution to file_x.mtx. (The reference writes its permuted, eliminated
// right-hand side there, main.cpp:61; this writes x.)
//
// options: --mixed (FP32 factors + FP64 refinement) | --fp64 (default)
//          --levels (stage-synchronous executor) --queue (ready-queue executor)
//          --cache (binary cache of the parsed matrix beside the .mtx file)
//          --device N --threads N
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "plan.h"
#include "soglu_gb300.h"

static double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int main(int argc, char** argv) {
    if (argc <= 1 || std::string(argv[1]).find(".mtx") == std::string::npos) {
        std::printf("usage: ./solve filename.mtx [--fp64|--mixed] [--levels|--queue] [--cache] [--device N] [--threads N]\n");
        return 0;
    }
    std::string fname = argv[1];
    int precision = SOG_FP64, executor = SOG_EXEC_PERSISTENT, device = 0, threads = 0;
    bool cache = false;
    for (int i = 2; i < argc; i++) {
        std::string a = argv[i];
        if (a == "--mixed") precision = SOG_MIXED;
        else if (a == "--fp64") precision = SOG_FP64;
        else if (a == "--levels") executor = SOG_EXEC_LEVELS;
        else if (a == "--queue") executor = SOG_EXEC_QUEUE;
        else if (a == "--device" && i + 1 < argc) device = std::atoi(argv[++i]);
        else if (a == "--threads" && i + 1 < argc) threads = std::atoi(argv[++i]);
        else if (a == "--cache") cache = true;
    }
    std::string base = fname.substr(0, fname.find(".mtx"));
    sog::MtxData m;
    std::string err;
    const double tr = now_s();
    if (!(cache ? sog::read_mtx_cached(fname, m, err) : sog::read_mtx(fname, m, err)) || m.I.empty()) {
        std::printf("%s\n", err.empty() ? "empty matrix" : err.c_str());
        return 1;
    }
    std::vector<double> b = sog::read_rhs(base + "_b.mtx", m.n);
    std::printf("read time: %g\n", now_s() - tr);
    double t0 = now_s();
    sog_plan* plan = nullptr;
    int r = sog_plan_build(m.n, (int64_t)m.I.size(), m.symmetric, m.I.data(), m.J.data(), m.V.data(), threads, &plan);
    if (r) { std::printf("plan failed (%d): %s\n", r, sog_last_error()); return 2; }
    sog_plan_info info;
    sog_plan_get_info(plan, &info);
    std::printf("re Order time: %g\n", info.t_order);
    std::printf("blocks: %d blockSize: 64 inputSize: %d extend: %d op count: %lld storage: %d\n", info.block_rows,
                info.n, info.n_ext, (long long)info.nops, info.storage_count);
    std::printf("plan time: %g\n", info.t_plan);
    sog_ctx* ctx = nullptr;
    if ((r = sog_ctx_create(device, 0, &ctx))) { std::printf("device: %s\n", sog_last_error()); return 3; }
    sog_options opt;
    std::memset(&opt, 0, sizeof(opt));
    opt.precision = precision;
    opt.executor = executor;
    opt.max_refine = 10;
    opt.tol = 1e-10;
    sog_system* sys = nullptr;
    if ((r = sog_system_create(ctx, plan, &opt, &sys))) { std::printf("system: %s\n", sog_last_error()); return 4; }
    if ((r = sog_factor(sys, m.V.data()))) { std::printf("factor: %s\n", sog_last_error()); return 5; }
    std::vector<double> x(m.n);
    sog_solve_stats st;
    r = sog_solve(sys, 1, b.data(), x.data(), &st);
    double fms = 0, sms = 0;
    sog_system_last_times(sys, &fms, &sms);
    std::printf("kernel time: %g\n", fms * 1e-3);
    std::printf("solve triangled :%g\n", sms * 1e-3);
    std::printf("totaltime: %g\n", now_s() - t0);
    if (r && r != SOG_ENOCONV) std::printf("solve: %s\n", sog_last_error());
    if (st.nan_count > 0) std::printf("found NaN:  %lld\n", (long long)st.nan_count);
    // residual in the original ordering (mtx.cpp:183-215)
    std::vector<double> bb(m.n, 0.0);
    for (size_t k = 0; k < m.I.size(); k++) {
        bb[m.I[k]] += m.V[k] * x[m.J[k]];
        if (m.symmetric && m.I[k] != m.J[k]) bb[m.J[k]] += m.V[k] * x[m.I[k]];
    }
    double mx = 0;
    for (int i = 0; i < m.n; i++) {
        double t = std::fabs(b[i] - bb[i]);
        if (t > mx || std::isnan(t) || std::isinf(t)) mx = t;
    }
    std::printf("max rhs error:%g\n", mx);
    std::printf("rel residual: %g backward error: %g refinement steps: %d\n", st.rel_resid, st.backward_error,
                st.iterations);
    std::ofstream out(base + "_x.mtx");
    out << "%%MatrixMarket matrix array real general\n" << m.n << " 1\n";
    out.precision(17);
    for (int i = 0; i < m.n; i++) out << x[i] << "\n";
    if (m.n > 3)
        std::printf("%g %g %g ... %g %g %g\n", x[0], x[1], x[2], x[m.n - 3], x[m.n - 2], x[m.n - 1]);
    sog_system_destroy(sys);
    sog_ctx_destroy(ctx);
    sog_plan_destroy(plan);
    return r == SOG_OK ? 0 : 6;
}
