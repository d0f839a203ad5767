#!/usr/bin/env python3
"""Benchmark of the factor-and-solve path on GB300.

Default workload (--workload lap64): 3D 7-point Laplacian on a 64^3 grid
(n = 262,144, 1,810,432 nnz, diagonal 6.01, off-diagonals -1) with 64
right-hand sides b = A x_true, x_true ~ U[-1,1] seed 0, seeded synthetic
data. A step = numeric factorisation of the planned op DAG (7.1M unit ops)
plus the solve of all 64 right-hand sides to ||b - A x||_2 / ||b||_2 <= 1e-10.
Host ordering and planning (the symbolic analysis) happen once before timing,
in both arms.

Other workloads: var48 = 3D 7-point variable-coefficient diffusion on a 48^3
grid (n = 110,592, k = exp(N(0,1)) seed 1, harmonic-mean faces, diagonal
shift 1e-3, 1 right-hand side, 1.08M unit ops); batch1024 = 1,024
independent 2D convection-diffusion systems (side ~ U{16..96}, cell Peclet ~
U[0,10], angle ~ U[0,2pi), 5-point upwind, 4 N(0,1) right-hand sides each),
merged into one batch plan and factored in one executor launch per step;
var24 = the var-coef system on 24^3, a small case of the same kernels for
profiler captures. A "solve" is one system factored and solved for all its
right-hand sides.

  value   mixed precision (FP32 factors, 3xTF32 tile products, FP64
          refinement), inputs resident in HBM, solves/s over all ranks
  e2e     the same through the C ABI with host buffers: values and b copied
          in from pinned memory and x copied out inside every step
  fp64    the plain FP64 GPU path (DMMA tile products), same step

--impl reference times the reference's CPU executor path (BlockPlanner::
calculate + BlockPlanner::solve restated in oracle/soglu_oracle.c, with the
reference's block lifetime: blocks freed after the last stage that reads
them; the reference's own AVX-512 build does not compile on the Arm host) on
all host cores, each step one full factor + solve of the same system (its
right-hand sides solved in parallel). A 64^3 step takes tens of seconds on
the host, so that arm times at most 3 steps after no warm-up, whatever
--steps / --warmup ask, and reports the counts it ran.
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG_DIR = os.path.join(ROOT, "sparse-operator-graph-lu_gb300")
METRIC = "solves/s mixed+IR vs plain FP64 GPU LU at resid<=1e-10; p50/p99 latency"
WORKLOADS = {
    "var48": "3D 7-point var-coef diffusion 48^3 (n=110592, nnz=760320), 1 RHS, factor+solve to rel resid<=1e-10",
    "lap64": "3D 7-point Laplacian 64^3 (n=262144, nnz=1810432), 64 RHS, factor+solve to rel resid<=1e-10",
    "lap64spd": "3D 7-point Laplacian 64^3 given as its lower triangle (symmetric: LL^T path), 64 RHS, "
                "factor+solve to rel resid<=1e-10",
    "var24": "3D 7-point var-coef diffusion 24^3 (n=13824, nnz=93312), 1 RHS, factor+solve to rel resid<=1e-10",
    "serving": "serving stream: Poisson arrivals, random band systems n log-uniform [2000, 200000], 3-27 nnz/row "
               "within half-band 0.02n, diag 1.1 x row abs sum, 1-16 RHS; continuous batching, pool admission",
    "batch1024": "1,024 nonsymmetric 2D conv-diff systems (side U{16..96}, n 256-9216, Pe U[0,10]), 4 RHS each, "
                 "one batch plan, one factor launch per step, factor+solve to rel resid<=1e-10 per system",
}


class Work:
    """A benchmark workload: its systems, the plan the executor runs (a batch
    plan for several systems) and the flat value / right-hand-side arrays in
    the C-ABI layout (per system, rhs-major, concatenated)."""

    def __init__(self, name: str, sg):
        self.name = name
        self.desc = WORKLOADS[name]
        self.systems = make_workload(name)
        t0 = time.perf_counter()
        self.plans = [sg.Plan(s.n, s.rows, s.cols, s.vals, symmetric=s.symmetric) for s in self.systems]
        self.plan = self.plans[0] if len(self.plans) == 1 else sg.merge_plans(self.plans)
        self.t_plan = time.perf_counter() - t0
        s0 = self.systems[0]
        self.nrhs = 1 if s0.b.ndim == 1 else s0.b.shape[0]
        self.vals = np.concatenate([s.vals for s in self.systems])
        self.b = np.concatenate([s.b.ravel() for s in self.systems])
        self.count = len(self.systems)
        self.nnz = int(self.vals.size)
        self.n = int(sum(s.n for s in self.systems))
        self.flops = sum(algorithmic_flops(p.info.op_count) for p in self.plans)

    def split(self, x):
        out, o = [], 0
        for s in self.systems:
            m = s.n * self.nrhs
            out.append(x[o:o + m].reshape(s.b.shape))
            o += m
        return out



def load_package():
    if "soglu_gb300" in sys.modules:
        return sys.modules["soglu_gb300"]
    spec = importlib.util.spec_from_file_location("soglu_gb300", os.path.join(PKG_DIR, "__init__.py"),
                                                  submodule_search_locations=[PKG_DIR])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["soglu_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def build_native():
    spec = importlib.util.spec_from_file_location("soglu_build", os.path.join(PKG_DIR, "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    b.build()


def make_workload(name: str):
    load_package()
    import soglu_gb300.workloads as wl
    if name == "lap64":
        return [wl.lap3d(64, nrhs=64)]
    if name == "lap64spd":
        return [wl.spd_lower(wl.lap3d(64, nrhs=64))]
    if name == "batch1024":
        return wl.convdiff_batch(1024)
    return [wl.varcoef3d(24 if name == "var24" else 48)]


def _measured_peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


MEASURED = _measured_peaks()

# DRAM bytes (read + write) of one mixed factor launch, NOT measured in the
# run that prints them: taken from the committed ncu summaries under
# profiles/ (dram__bytes_read.sum + dram__bytes_write.sum of one launch);
# None where no capture covers the workload. The 64^3 figure is the 48^3
# capture scaled by the FP32 tile count (25.06 GB / 5.83 GB of tiles): the
# factor writes each tile once and reads its operands mostly from L2.
_T48 = 253.46e6 + 3505.47e6
TRAFFIC: dict = {
    "var48": (_T48, "profiles/dram_factor_var48.md (one-pass ncu, full-size launch)"),
    "lap64": (_T48 * 25.06 / 5.83, "profiles/dram_factor_var48.md, scaled by the tile count (25.06 / 5.83 GB)"),
}


def algorithmic_flops(op_count) -> float:
    """Dense-tile flops of the DAG: mul/mulneg/mult 2*64^3, lu 2/3*64^3,
    llt and lowerInv/upperInv 1/3*64^3, sub 64^2 (per unit op)."""
    t = 64.0 ** 3
    return (op_count[8] + op_count[9] + op_count[11]) * 2 * t + op_count[1] * 2 / 3 * t \
        + (op_count[2] + op_count[3] + op_count[10]) * t / 3 + op_count[4] * 64.0 ** 2


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.lines: list[str] = []
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200", "-i", str(device)], stdout=subprocess.PIPE,
                                      stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.p = None

    def _read(self):
        for line in self.p.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.t.join(timeout=2)
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1])); smax.append(float(f[2])); power.append(float(f[3]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "power_w_max": max(power) if power else None}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(v: float, world: int, device=None) -> float:
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def measure_peaks(torch, device) -> dict:
    """cuBLAS TF32 and FP64 GEMM throughput on this GPU (denominators for the
    3xTF32 and DMMA tile products; MEASURED_PEAKS.json holds bf16 and HBM figures only)."""
    out = {}
    torch.backends.cuda.matmul.allow_tf32 = True
    for name, dt, n, reps in (("tf32_tflops", torch.float32, 8192, 5), ("fp64_tflops", torch.float64, 4096, 3)):
        a = torch.randn(n, n, dtype=dt, device=device)
        b = torch.randn(n, n, dtype=dt, device=device)
        torch.matmul(a, b)
        torch.cuda.synchronize()
        best = 1e30
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(); torch.matmul(a, b); e1.record(); e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        out[name] = 2 * n ** 3 / (best * 1e-3) / 1e12
        del a, b
    torch.backends.cuda.matmul.allow_tf32 = False
    return out


def cpu_sample(work, sg, threads: int, budget_s: float = 15.0):
    """The oracle (C restatement of the reference's calculate + solve) on the
    host cores: whole systems in order, each factored once and solved for its
    right-hand sides, until about budget_s seconds of work. Returns (systems
    done, seconds, worst relative residual)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    done, t_tot, worst = 0, 0.0, 0.0
    for s, p in zip(work.systems, work.plans):
        perm, ops, L, U = p.export()
        tiles_in = p.input_tiles(s.vals)
        t0 = time.perf_counter()
        X = oracle.solve_system_multi(perm, s.n, p.info.block_rows, ops, p.info.storage_count, tiles_in, L, U,
                                      s.b, threads=threads)
        t_tot += time.perf_counter() - t0
        done += 1
        B = np.atleast_2d(s.b)
        worst = max(worst, float(np.linalg.norm(B - np.atleast_2d(s.matvec(X))) / np.linalg.norm(B)))
        if t_tot >= budget_s:
            break
    return done, t_tot, worst


def run_serving(args):
    """Serving stream (sog_server_*): requests arrive as a Poisson process at
    each rate of the sweep; each is planned on host threads, admitted by free
    pool memory, merged with whatever else is ready into shared launches,
    answered and released. Latency = submit -> answer (host clock);
    throughput = requests answered / (last answer - first arrival)."""
    import threading
    import torch
    torch.cuda.set_device(0)
    build_native()
    sg = load_package()
    import soglu_gb300.workloads as wl
    rng = np.random.default_rng(17)
    spec = wl.serving_requests(args.requests, seed=3)
    t0 = time.perf_counter()
    systems = [wl.random_band(n, seed=sd, nrhs=k) for n, sd, k in spec]
    t_gen = time.perf_counter() - t0
    ctx = sg.Context(0)
    rates = [float(r) for r in args.rates.split(",")]
    sweep = []
    for prec_name, prec in (("mixed", sg.MIXED), ("fp64", sg.FP64)):
        if prec_name == "fp64" and not args.serving_fp64:
            continue
        for lam in (rates if prec_name == "mixed" else rates[-1:]):
            srv = sg.Server(ctx, precision=prec, planners=args.planners, omp_threads=max(1, (os.cpu_count() or 2)
                                                                                        // args.planners))
            gaps = rng.exponential(1.0 / lam, len(systems))
            arrivals = np.cumsum(gaps) - gaps[0]
            ids = [None] * len(systems)
            t_start = time.perf_counter()

            def submitter():
                for k, s in enumerate(systems):
                    d = t_start + arrivals[k] - time.perf_counter()
                    if d > 0:
                        time.sleep(d)
                    ids[k] = srv.submit(s.n, s.rows, s.cols, s.vals, s.b)

            th = threading.Thread(target=submitter)
            th.start()
            lat, worst, stat_bad, t_last, infos = [], 0.0, 0, t_start, []
            for k, s in enumerate(systems):
                while ids[k] is None:
                    time.sleep(0.001)
                x, info = srv.wait(ids[k], allow_noconv=True)
                t_last = max(t_last, time.perf_counter())
                srv.release(ids[k])
                lat.append(info["total_ms"])
                infos.append(info)
                if info["status"] != sg.SOG_OK:
                    stat_bad += 1
                worst = max(worst, info["rel_resid"])
            th.join()
            wall = t_last - t_start
            c = srv.counters()
            srv.close()
            sweep.append({"precision": prec_name, "rate_per_s": lam, "requests": len(systems),
                          "throughput_per_s": len(systems) / wall, "wall_s": wall,
                          "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                          "mean_plan_ms": float(np.mean([i["plan_ms"] for i in infos])),
                          "mean_queue_ms": float(np.mean([i["queue_ms"] for i in infos])),
                          "mean_setup_ms": float(np.mean([i["setup_ms"] for i in infos])),
                          "mean_gpu_ms": float(np.mean([i["gpu_ms"] for i in infos])),
                          "batches": c["batches"], "largest_batch": c["max_batch"],
                          "worst_rel_resid": worst, "not_ok": stat_bad,
                          "slowest": (lambda k: {"n": int(systems[k].n), "total_ms": lat[k],
                                                 "plan_ms": infos[k]["plan_ms"], "queue_ms": infos[k]["queue_ms"],
                                                 "setup_ms": infos[k]["setup_ms"],
                                                 "gpu_ms": infos[k]["gpu_ms"]})(int(np.argmax(lat)))})
    ctx.close()
    top = [r for r in sweep if r["precision"] == "mixed"][-1]
    line = {"metric": METRIC, "value": top["throughput_per_s"], "unit": "requests/s", "n_gpus": 1,
            "steps": len(systems), "warmup": 0, "ms_per_step": 1e3 * top["wall_s"] / len(systems),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic", "config": {"workload": WORKLOADS["serving"], "requests": len(systems),
                                            "rates_per_s": rates, "planner_threads": args.planners,
                                            "n": [int(s.n) for s in systems]},
            "p50_ms": top["p50_ms"], "p99_ms": top["p99_ms"], "sweep": sweep, "generate_s": t_gen}
    print(json.dumps(line), flush=True)
    return 0


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    build_native()
    sg = load_package()
    if args.workload == "serving":
        print(json.dumps({"impl": "reference", "unavailable": "the reference solves one system per process and has "
                          "no request loop; its per-system CPU rate is the default workload's reference line"}))
        return 0
    work = Work(args.workload, sg)
    cores = os.cpu_count() or 1
    # each step a bounded sample: the whole system (single-system workloads)
    # or as many of the batch's systems as fit in the budget; a 64^3 step is
    # tens of seconds of host work, so at most 3 of them and no warm-up
    budget = 1e9 if work.count == 1 else 6.0
    heavy = args.workload in ("lap64", "lap64spd")
    warmup = 0 if heavy else args.warmup
    steps = min(args.steps, 3) if heavy else args.steps
    for _ in range(warmup):
        cpu_sample(work, sg, cores, budget)
    times, worst, done = [], 0.0, 0
    for _ in range(steps):
        d, dt, w = cpu_sample(work, sg, cores, budget)
        times.append(dt / d * work.count)  # seconds for the whole workload at the sampled rate
        worst = max(worst, w)
        done = d
    tot = sum(times)
    v = steps * work.count / tot
    sample = (f"{steps} full factor+solve steps of the {args.workload} system ({work.nrhs} right-hand sides "
              f"solved in parallel)" if work.count == 1 else
              f"per step the first {done} of the {work.count} systems, factor + {work.nrhs} solves each, "
              f"rate scaled to the whole batch")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "solves/s", "n_gpus": args.gpus,
            "steps": steps, "warmup": warmup, "steps_requested": args.steps, "warmup_requested": args.warmup,
            "ms_per_step": 1e3 * tot / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": work.desc, "precision": "fp64 CPU", "parallelism": "host cores",
                       "timed": "numeric factor + solve; ordering and planning (symbolic analysis) before timing, "
                                "as in the GPU arm"},
            "rel_resid": worst,
            "p50_ms": 1e3 * statistics.median(times), "p99_ms": 1e3 * max(times),
            "cpu_baseline": {"value": v, "unit": "solves/s", "cores": cores, "kind": "port",
                             "sample": sample + " (the reference's AVX-512 kernels do not compile on the aarch64 "
                                       "host; the C restatement of its executor path, pinned to the reference's "
                                       "outputs, is timed)"},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import ctypes
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = local
    torch.cuda.set_device(dev)
    build_native()
    sg = load_package()
    work = Work(args.workload, sg)
    plan = work.plan
    info = plan.info
    flops = work.flops
    nrhs = work.nrhs
    ctx = sg.Context(dev)
    stream = torch.cuda.ExternalStream(ctx.stream())
    V = torch.from_numpy(work.vals).to(dev)
    b = torch.from_numpy(work.b).to(dev)
    x = torch.empty_like(b)
    torch.cuda.synchronize()
    L = sg.lib()
    # host buffers for the end-to-end leg: pinned, C-ABI calls with host pointers
    hv = torch.from_numpy(work.vals).pin_memory()
    hb = torch.from_numpy(work.b).pin_memory()
    hx = torch.empty_like(hb).pin_memory()

    # one call per step: factor, then solve (a plain mixed system runs its
    # first forward substitution while the factorisation runs)
    def step(sysm, host):
        if not host:
            return sysm.factor_solve_device(V.data_ptr(), nrhs, b.data_ptr(), x.data_ptr())
        st = sg.SolveStats()
        sg._check(L.sog_factor_solve(sysm._h, ctypes.c_void_p(hv.data_ptr()), nrhs, ctypes.c_void_p(hb.data_ptr()),
                                     ctypes.c_void_p(hx.data_ptr()), ctypes.byref(st)))
        return st.as_dict()

    def timed(sysm, steps, warmup, host=False):
        lat, fms, sms, iters, st = [], [], [], [], None
        for _ in range(warmup):
            step(sysm, host)
        barrier(world)
        torch.cuda.synchronize()
        l0 = sysm.task_info()["launches"]
        clk = ClockSampler(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            h0 = time.perf_counter()
            st = step(sysm, host)
            lat.append(1e3 * (time.perf_counter() - h0))
            f, so = sysm.last_times()
            fms.append(f); sms.append(so); iters.append(st["iterations"])
        e1.record(stream)
        e1.synchronize()
        clocks = clk.stop()
        torch.cuda.synchronize()
        barrier(world)
        ms = e0.elapsed_time(e1)
        return {"ms": max_over_ranks(ms, world, dev), "lat": lat, "factor_ms": fms, "solve_ms": sms,
                "iters": iters, "stats": st, "clocks": clocks, "launches": sysm.task_info()["launches"] - l0}

    t_sys = time.perf_counter()
    mixed = sg.System(ctx, plan, precision=sg.MIXED, max_refine=20, tol=1e-10, executor=args.executor,
                      pipeline_stages=args.stages)
    t_sys = time.perf_counter() - t_sys
    rm = timed(mixed, args.steps, args.warmup)
    # device time of a whole solve (every pass on the system's stream), from
    # separate factor and solve calls after the timed region: in the timed
    # steps the first forward pass overlaps the factorisation
    mixed.factor_device(V.data_ptr())
    mixed.solve_device(nrhs, b.data_ptr(), x.data_ptr())
    solve_ms_whole = mixed.last_times()[1]
    grid_mixed = mixed.task_info()["grid"]
    ex = mixed.executor_config()
    chosen = (["persistent, static order", "per level", "persistent, ready queue"][ex["executor"]]
              + (", early products" if ex["early_products"] else "") + f", {ex['stages']} operand stages")
    x_mixed = x.cpu().numpy()
    re2e = timed(mixed, args.steps, args.warmup, host=True)
    x_e2e = hx.numpy().copy()
    mixed.close()
    fp64 = sg.System(ctx, plan, precision=sg.FP64, executor=args.executor)
    k64 = max(3, args.steps // 3)
    r64 = timed(fp64, k64, args.warmup)
    x_fp64 = x.cpu().numpy()
    ti = fp64.task_info()
    fp64.close()

    total = args.steps * work.count * world
    value = total / (rm["ms"] * 1e-3)
    e2e_value = total / (re2e["ms"] * 1e-3)
    v64 = k64 * work.count * world / (r64["ms"] * 1e-3)
    if rank == 0:
        peaks = measure_peaks(torch, dev)
        fm = statistics.mean(rm["factor_ms"])
        sm_ = statistics.mean(rm["solve_ms"])
        f64m = statistics.mean(r64["factor_ms"])
        dominant = "factor" if fm >= sm_ else "solve"
        # 3xTF32: three TF32 products per FP32 product -> effective peak = TF32 peak / 3
        eff_peak = peaks["tf32_tflops"] / 3
        ach = flops / (fm * 1e-3) / 1e12
        tr = TRAFFIC.get(args.workload)
        roof = {"bound": "tensor", "kernel": "factor_ordered_kernel<float> (3xTF32 tile products on tcgen05 + LU/"
                                                "inverse tasks, one launch per factorisation)",
                "achieved": ach, "peak": eff_peak, "unit": "TFLOP/s", "frac": ach / eff_peak,
                "traffic": tr[0] if tr else None, "traffic_source": tr[1] if tr else None,
                "peak_source": f"cuBLAS TF32 GEMM measured in this run ({peaks['tf32_tflops']:.1f} TFLOP/s) / 3",
                "algorithmic_flop_per_launch": flops, "avg_launch_ms": fm}
        # substitution: HBM-bound by its algorithmic bytes per pass (every factor
        # tile it reads once, FP32: off-diagonal L/U leaves, diagonal inverses,
        # look-ahead products; the vectors), passes = 1 + refinement steps
        R = info.block_rows
        tiles_read = (info.n_lleaf + info.n_uleaf - 2 * R) + 2 * R + 2 * R
        pass_bytes = tiles_read * 4096 * 4 + 3 * info.n_ext * 4 * nrhs
        passes = 1 + statistics.mean(rm["iters"])
        s_ach = pass_bytes / (solve_ms_whole * 1e-3 / passes) / 1e9
        hbm_peak, hbm_src = (MEASURED.get("hbm_gbs"), "MEASURED_PEAKS.json hbm_gbs (measured copy)") \
            if MEASURED.get("hbm_gbs") else (6800.0, "fallback 6.8 TB/s")
        solve_roof = {"bound": "hbm", "kernel": "trisolve_kernel<float> (L and U passes)", "achieved": s_ach,
                      "peak": hbm_peak, "unit": "GB/s", "frac": s_ach / hbm_peak, "peak_source": hbm_src,
                      "algorithmic_bytes_per_pass": pass_bytes, "passes_per_solve": passes,
                      "solve_ms": solve_ms_whole, "solve_ms_source": "separate factor and solve calls after "
                                                                     "the timed steps"}
        fp64_roof = {"achieved": flops / (f64m * 1e-3) / 1e12, "peak": peaks["fp64_tflops"], "unit": "TFLOP/s",
                     "frac": flops / (f64m * 1e-3) / 1e12 / peaks["fp64_tflops"],
                     "peak_source": "cuBLAS DGEMM measured in this run", "avg_factor_ms": f64m}
        cpu = None
        if world == 1 and not args.no_cpu_baseline:
            cores = os.cpu_count() or 1
            d, dt, _ = cpu_sample(work, sg, cores, 15.0)
            cpu = {"value": d / dt, "unit": "solves/s", "cores": cores, "kind": "port",
                   "sample": (f"one full factor+solve of the {args.workload} system" if work.count == 1 else
                              f"the first {d} of the {work.count} systems, factor + {nrhs} solves each") +
                             " through the C restatement of the reference's executor path (the reference's "
                             "AVX-512 build does not compile on aarch64)",
                   "seconds": dt}
        fwd = {}
        xt = [s.x_true for s in work.systems]
        if all(t is not None for t in xt):
            def ferr(xx):
                parts = work.split(xx)
                return max(float(np.linalg.norm(p - t) / np.linalg.norm(t)) for p, t in zip(parts, xt))
            fwd = {"fwd_err_vs_x_true": ferr(x_mixed)}
        e2e_match = bool(np.array_equal(x_e2e, x_mixed))
        line = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": rm["ms"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": work.desc, "systems_per_step": work.count, "rhs": nrhs,
                       "precision": "mixed: FP32 factors, 3xTF32 tile products, FP64 IR",
                       "parallelism": f"replicas x{world}",
                       "l2": f"inputs larger than L2 (FP32 tiles {info.storage_count * 16384 / 1e9:.2f} GB)",
                       "executor": ["persistent, static order", "per level", "persistent, ready queue",
                                    "autotuned"][args.executor] + f" ({chosen})",
                       "factor_ctas": grid_mixed, "pipeline_stages": args.stages or "tuned",
                       "timed": "numeric factor + solve; ordering and planning (symbolic analysis) before timing, "
                                "as in the reference arm",
                       "step_call": "sog_factor_solve_device (a single system: the first forward substitution "
                                    "overlaps the factorisation; solve_ms is the device time after the factor)"},
            "p50_ms": statistics.median(rm["lat"]), "p99_ms": float(np.percentile(rm["lat"], 99)),
            "factor_ms": fm, "solve_ms": sm_, "refine_steps": max(rm["iters"]),
            "factor_ms_steps": [round(v, 3) for v in rm["factor_ms"]],
            "rel_resid": rm["stats"]["rel_resid"], "backward_error": rm["stats"]["backward_error"], **fwd,
            "fp64_plain": {"value": v64, "unit": "solves/s", "steps": k64, "ms_per_step": r64["ms"] / k64,
                           "factor_ms": f64m, "solve_ms": statistics.mean(r64["solve_ms"]),
                           "rel_resid": r64["stats"]["rel_resid"],
                           **({"fwd_err_vs_x_true": max(float(np.linalg.norm(p - t) / np.linalg.norm(t))
                                                        for p, t in zip(work.split(x_fp64), xt))} if fwd else {}),
                           "roofline": fp64_roof},
            "mixed_over_fp64": value / v64,
            "dominant": dominant,
            "roofline": roof,
            "solve_roofline": solve_roof,
            "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": int(work.nnz * 8 + work.b.size * 8),
                    "d2h_bytes_per_step": int(work.b.size * 8), "ms_per_step": re2e["ms"] / args.steps,
                    "path": "sog_factor_solve with pinned host buffers", "x_equals_device_path": e2e_match},
            "cpu_baseline": cpu,
            "clocks": rm["clocks"],
            "gpu_launches": int(rm["launches"]),
            "plan": {"host_plan_s": work.t_plan, "host_system_s": t_sys, "ops": int(info.nops),
                     "stages": int(info.stages),
                     "tasks": ti["tasks"], "levels": ti["levels"], "algorithmic_gflop": flops / 1e9},
        }
        print(json.dumps(line), flush=True)
    barrier(world)
    ctx.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="lap64")
    ap.add_argument("--executor", type=int, default=3,
                    help="0 persistent (static order), 1 per level, 2 ready queue, 3 autotuned (default: the "
                         "first, untimed factorisation times the persistent executors and keeps the faster)")
    ap.add_argument("--stages", type=int, default=0, help="mixed path operand stages: 1, 2, or 0 = tuned")
    ap.add_argument("--requests", type=int, default=32, help="serving: requests per rate")
    ap.add_argument("--rates", default="0.5,2,8", help="serving: Poisson arrival rates (requests/s)")
    ap.add_argument("--planners", type=int, default=4, help="serving: host planning threads")
    ap.add_argument("--serving-fp64", action="store_true", help="serving: also run the plain FP64 path")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "serving":
        return run_serving(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
