"""soglu_gb300: GB300 (sm_103a) executor for sparse-operator-graph-LU's
factor-and-solve path, driven through the C ABI of include/soglu_gb300.h.

The reference's public entry point is SOGLU::solveLU (solver.cpp:121); its
executor boundary is BlockPlanner::calculate / BlockPlanner::solve
(BlockPlanner.cpp:376, :834). This module mirrors them:

    solveLU(dim, rows, cols, vals, b)        -> x          (solver.cpp:121)
    Plan(n, rows, cols, vals)                 host planner (GPSOrder + BlockPlanner)
    System(Context(), plan).factor(vals)      BlockPlanner::calculate on the GPU
    System.solve(b)                           BlockPlanner::solve + reOrderResult

There is no CPU fallback: without the built library or a CUDA device every
call raises SOGError.
"""
from __future__ import annotations

import ctypes as C
import os
import weakref

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "lib", "libsoglu_gb300.so")

SOG_OK, SOG_EINVAL, SOG_ENOMEM, SOG_EPIVOT, SOG_ENAN, SOG_ETIMEOUT, SOG_ECUDA, SOG_ENOCONV, SOG_ESTATE, SOG_ENODEV = range(10)
FP64, MIXED = 0, 1
EXEC_PERSISTENT, EXEC_LEVELS, EXEC_QUEUE, EXEC_AUTO = 0, 1, 2, 3
OP_NAMES = ["inv", "lu", "lowerInv", "upperInv", "sub", "add", "neg", "copy", "mul", "mulneg", "llt", "mult", "noop"]
_CODES = {0: "OK", 1: "EINVAL", 2: "ENOMEM", 3: "EPIVOT", 4: "ENAN", 5: "ETIMEOUT", 6: "ECUDA", 7: "ENOCONV",
          8: "ESTATE", 9: "ENODEV"}


class SOGError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_CODES.get(code, code)}: {msg}")
        self.code = code


class PlanInfo(C.Structure):
    _fields_ = [("n", C.c_int32), ("n_ext", C.c_int32), ("block_rows", C.c_int32), ("block_rows_l2", C.c_int32),
                ("block_size_l2", C.c_int32), ("storage_count", C.c_int32), ("n_input", C.c_int32),
                ("stages", C.c_int32), ("nops", C.c_int64), ("n_lleaf", C.c_int64), ("n_uleaf", C.c_int64),
                ("nnz", C.c_int64), ("op_count", C.c_int64 * 13), ("coarse_ops", C.c_int64),
                ("fine_ops_emitted", C.c_int64), ("t_order", C.c_double), ("t_plan", C.c_double)]


class Options(C.Structure):
    _fields_ = [("precision", C.c_int32), ("executor", C.c_int32), ("max_refine", C.c_int32), ("tol", C.c_double),
                ("gemm_split", C.c_int32), ("solve_lookahead", C.c_int32), ("pipeline_stages", C.c_int32),
                ("max_ctas", C.c_int32), ("growth_limit", C.c_double), ("resident_compact", C.c_int32),
                ("reserved", C.c_int32)]


class SolveStats(C.Structure):
    _fields_ = [("status", C.c_int32), ("iterations", C.c_int32), ("rel_resid", C.c_double),
                ("backward_error", C.c_double), ("nan_count", C.c_int64), ("min_pivot", C.c_double),
                ("clamped_pivots", C.c_int32), ("inv_check_failures", C.c_int32), ("max_growth", C.c_double),
                ("reserved", C.c_int32 * 2)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class ServerOptions(C.Structure):
    _fields_ = [("planner_threads", C.c_int32), ("planner_omp_threads", C.c_int32), ("max_batch", C.c_int32),
                ("lanes", C.c_int32), ("batch_window_ms", C.c_double), ("reserved", C.c_int32 * 2)]


class RequestInfo(C.Structure):
    _fields_ = [("status", C.c_int32), ("batch_size", C.c_int32), ("batch_id", C.c_int64), ("plan_ms", C.c_double),
                ("queue_ms", C.c_double), ("setup_ms", C.c_double), ("gpu_ms", C.c_double), ("total_ms", C.c_double),
                ("stats", SolveStats)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "stats"}
        d.update(self.stats.as_dict())
        d["status"] = self.status
        return d


# every symbol declared in include/soglu_gb300.h
EXPORTS = [
    "sog_last_error", "sog_version", "sog_plan_build", "sog_plan_get_info", "sog_plan_export", "sog_plan_input_tiles",
    "sog_plan_import", "sog_plan_destroy", "sog_ctx_create", "sog_ctx_destroy", "sog_ctx_pool_usage", "sog_ctx_stream",
    "sog_system_create", "sog_system_bytes", "sog_factor", "sog_factor_device", "sog_factor_tiles", "sog_solve",
    "sog_solve_device", "sog_solve_permuted", "sog_system_export_factors", "sog_system_last_times",
    "sog_system_destroy", "sog_system_task_info", "sog_system_executor", "sog_system_set_wait_limit", "sog_debug_poison_task",
    "sog_debug_unpoison", "sog_debug_fp64_fragment_skip", "soglu_solveLU", "sog_system_trace_enable", "sog_system_trace_get",
    "sog_system_task_graph", "sog_plan_task_graph_info", "sog_residual_noalloc", "sog_plan_merge",
    "sog_plan_segments", "sog_solve_batch", "sog_solve_batch_device", "sog_ctx_trim", "sog_server_create",
    "sog_server_submit", "sog_server_wait", "sog_server_solve", "sog_server_release", "sog_server_counters",
    "sog_server_destroy", "sog_mtx_read", "sog_mtx_info", "sog_mtx_copy", "sog_mtx_destroy", "sog_system_pivots",
    "sog_system_set_stream", "sog_factor_solve", "sog_factor_solve_device",
]

_lib = None


def lib() -> C.CDLL:
    """Load the in-tree native library (built by build.py / __graft_entry__.build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise SOGError(SOG_ENODEV, f"native library not built: {LIB_PATH} (run build.py)")
    L = C.CDLL(LIB_PATH)
    P, I32, I64, D = C.c_void_p, C.c_int32, C.c_int64, C.c_double
    sig = {
        "sog_last_error": ([], C.c_char_p), "sog_version": ([], C.c_char_p),
        "sog_plan_build": ([I32, I64, I32, P, P, P, I32, P], I32),
        "sog_plan_get_info": ([P, P], I32), "sog_plan_export": ([P, P, P, P, P], I32),
        "sog_plan_input_tiles": ([P, P, P], I32),
        "sog_plan_import": ([I32, I32, I32, P, I64, P, I64, P, I64, P], I32),
        "sog_plan_destroy": ([P], None), "sog_ctx_create": ([I32, C.c_uint64, P], I32),
        "sog_ctx_destroy": ([P], None), "sog_ctx_pool_usage": ([P, P, P], I32), "sog_ctx_stream": ([P, P], I32),
        "sog_system_create": ([P, P, P, P], I32), "sog_system_bytes": ([P, P, P], I32),
        "sog_factor": ([P, P], I32), "sog_factor_device": ([P, P], I32), "sog_factor_tiles": ([P, P], I32),
        "sog_solve": ([P, I32, P, P, P], I32), "sog_solve_device": ([P, I32, P, P, P], I32),
        "sog_factor_solve": ([P, P, I32, P, P, P], I32), "sog_factor_solve_device": ([P, P, I32, P, P, P], I32),
        "sog_solve_permuted": ([P, P, P], I32), "sog_system_export_factors": ([P, P, P], I32),
        "sog_system_last_times": ([P, P, P], I32), "sog_system_destroy": ([P], None),
        "sog_system_task_info": ([P, P], I32), "sog_system_executor": ([P, P, P, P], I32),
        "sog_system_pivots": ([P, P], I32), "sog_system_set_stream": ([P, P], I32), "sog_system_set_wait_limit": ([P, D], I32),
        "sog_debug_poison_task": ([P, I32], I32), "sog_debug_unpoison": ([P], I32),
        "sog_debug_fp64_fragment_skip": ([P, I32], I32),
        "soglu_solveLU": ([I32, I64, I32, P, P, P, P, P, I32], I32),
        "sog_system_trace_enable": ([P, I32], I32), "sog_system_trace_get": ([P, P, P, P], I32),
        "sog_system_task_graph": ([P, P, P, P], I32), "sog_plan_task_graph_info": ([P, I32, P], I32),
        "sog_residual_noalloc": ([I32, P, P, P, I32, P, P, P, P, P, P], I32),
        "sog_plan_merge": ([P, I32, P], I32), "sog_plan_segments": ([P, P, P], I32),
        "sog_solve_batch": ([P, P, P, P, P], I32), "sog_solve_batch_device": ([P, P, P, P, P], I32),
        "sog_ctx_trim": ([P], I32), "sog_server_create": ([P, P, P, P], I32),
        "sog_server_submit": ([P, I32, I64, P, P, P, I32, I32, P, P], I32),
        "sog_server_wait": ([P, I64, D, P, P], I32), "sog_server_solve": ([P, I64, I32, P, P, P], I32),
        "sog_server_release": ([P, I64], I32), "sog_server_counters": ([P, P], I32),
        "sog_server_destroy": ([P], None),
        "sog_mtx_read": ([C.c_char_p, I32, P], I32), "sog_mtx_info": ([P, P, P, P], I32),
        "sog_mtx_copy": ([P, P, P, P], I32), "sog_mtx_destroy": ([P], None),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def _check(code: int) -> None:
    if code != SOG_OK:
        raise SOGError(code, lib().sog_last_error().decode())


def _p(a: np.ndarray) -> int:
    return a.ctypes.data


class Plan:
    """Host planner output for one sparsity pattern (GOrder + BlockPlanner)."""

    def __init__(self, n: int, rows, cols, vals=None, symmetric: bool = False, threads: int = 0, _handle=None):
        self._h = C.c_void_p()
        if _handle is not None:
            self._h = _handle
            self.nnz = 0
        else:
            self.rows = np.ascontiguousarray(rows, dtype=np.int32)
            self.cols = np.ascontiguousarray(cols, dtype=np.int32)
            v = None if vals is None else np.ascontiguousarray(vals, dtype=np.float64)
            self.nnz = int(self.rows.size)
            _check(lib().sog_plan_build(int(n), self.nnz, int(symmetric), _p(self.rows), _p(self.cols),
                                        None if v is None else _p(v), int(threads), C.byref(self._h)))
        self.info = PlanInfo()
        _check(lib().sog_plan_get_info(self._h, C.byref(self.info)))

    @classmethod
    def imported(cls, block_rows: int, storage_count: int, n_input: int, ops: np.ndarray, lleaf: np.ndarray,
                 uleaf: np.ndarray) -> "Plan":
        """Wrap a DAG produced elsewhere (e.g. the reference planner's)."""
        ops = np.ascontiguousarray(ops, dtype=np.int32).reshape(-1, 6)
        lleaf = np.ascontiguousarray(lleaf, dtype=np.int32).reshape(-1, 3)
        uleaf = np.ascontiguousarray(uleaf, dtype=np.int32).reshape(-1, 3)
        h = C.c_void_p()
        _check(lib().sog_plan_import(block_rows, storage_count, n_input, _p(ops), ops.shape[0], _p(lleaf),
                                     lleaf.shape[0], _p(uleaf), uleaf.shape[0], C.byref(h)))
        return cls(0, None, None, _handle=h)

    def segments(self) -> list[int]:
        """Dimensions of the systems in this plan (one entry for a plain plan)."""
        cnt = C.c_int32()
        _check(lib().sog_plan_segments(self._h, C.byref(cnt), None))
        n = np.zeros(cnt.value, np.int32)
        _check(lib().sog_plan_segments(self._h, C.byref(cnt), _p(n)))
        return [int(v) for v in n]

    def info_dict(self) -> dict:
        d = {k: getattr(self.info, k) for k, _ in PlanInfo._fields_ if k != "op_count"}
        d["ops"] = {OP_NAMES[i]: int(self.info.op_count[i]) for i in range(13) if self.info.op_count[i]}
        return d

    def export(self):
        """(new_to_old[n], ops[nops, 6] = op,src,src2,result,result2,stage, L[k,3], U[k,3]).
        For a batch plan new_to_old has n_ext entries (row within its system, -1 = padding)."""
        i = self.info
        nperm = i.n_ext if getattr(self, "batch", False) else i.n
        perm = np.empty(max(nperm, 1), np.int32)
        ops = np.empty((max(i.nops, 1), 6), np.int32)
        L = np.empty((max(i.n_lleaf, 1), 3), np.int32)
        U = np.empty((max(i.n_uleaf, 1), 3), np.int32)
        _check(lib().sog_plan_export(self._h, _p(perm), _p(ops), _p(L), _p(U)))
        return perm[:nperm], ops[:i.nops], L[:i.n_lleaf], U[:i.n_uleaf]

    def input_tiles(self, vals) -> np.ndarray:
        v = np.ascontiguousarray(vals, dtype=np.float64)
        t = np.empty((self.info.n_input, 64, 64), np.float64)
        _check(lib().sog_plan_input_tiles(self._h, _p(v), _p(t)))
        return t

    def task_graph_info(self, gemm_split: int = 1) -> dict:
        """Device task graph built on the host (no GPU needed)."""
        c = np.zeros(15, np.int64)
        _check(lib().sog_plan_task_graph_info(self._h, gemm_split, _p(c)))
        keys = ["tasks", "levels", "items", "pairs", "gemm", "lu", "linv", "uinv", "sub", "fused_subs",
                "added_inverses", "critical_path", "fused_inverses", "aliased_copies", "aliased_inverses"]
        return dict(zip(keys, (int(v) for v in c)))

    def bytes_needed(self, precision: int = FP64) -> int:
        o = Options(precision=precision)
        out = C.c_uint64()
        _check(lib().sog_system_bytes(self._h, C.byref(o), C.byref(out)))
        return int(out.value)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.sog_plan_destroy(self._h)
            self._h = None


def merge_plans(plans) -> Plan:
    """Batch plan: the block-diagonal union of independent systems' plans
    (sog_plan_merge). A System on it factors every system in one executor
    launch; values are the systems' triplet values concatenated, and solves go
    through System.solve_batch."""
    plans = list(plans)
    arr = (C.c_void_p * len(plans))(*[p._h.value for p in plans])
    h = C.c_void_p()
    _check(lib().sog_plan_merge(arr, len(plans), C.byref(h)))
    m = Plan(0, None, None, _handle=h)
    m.nnz = sum(p.nnz for p in plans)
    m.batch = True
    return m


class Context:
    """One GPU, one stream, the device block-pool arena."""

    def __init__(self, device: int = 0, pool_bytes: int = 0):
        self._h = C.c_void_p()
        # systems and servers on this context: closed before the context, in
        # whatever order the interpreter finalises objects
        self._children = weakref.WeakSet()
        _check(lib().sog_ctx_create(device, pool_bytes, C.byref(self._h)))

    def stream(self) -> int:
        """The context's cudaStream_t as an integer (every kernel runs on it)."""
        s = C.c_void_p()
        _check(lib().sog_ctx_stream(self._h, C.byref(s)))
        return int(s.value or 0)

    def pool_usage(self):
        u, t = C.c_uint64(), C.c_uint64()
        _check(lib().sog_ctx_pool_usage(self._h, C.byref(u), C.byref(t)))
        return int(u.value), int(t.value)

    def close(self):
        if getattr(self, "_h", None):
            for child in list(getattr(self, "_children", ())):
                child.close()
            lib().sog_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        if _lib is not None:
            self.close()


class System:
    """One system resident in the device pool: factor once, solve many."""

    def __init__(self, ctx: Context, plan: Plan, precision: int = FP64, executor: int = EXEC_PERSISTENT,
                 max_refine: int = 10, tol: float = 1e-10, gemm_split: int = 0, solve_lookahead: int = 0,
                 pipeline_stages: int = 0, growth_limit: float = 0.0, max_ctas: int = 0, resident_compact: bool = False):
        """growth_limit: the pivot gate (0 = default for the precision, < 0 =
        off, as the reference); a factorisation that fails it raises
        SOGError(EPIVOT) unless factor(..., allow_epivot=True)."""
        self.ctx, self.plan = ctx, plan
        self.n = plan.info.n
        self._h = C.c_void_p()
        self.opt = Options(precision=precision, executor=executor, max_refine=max_refine, tol=tol,
                           gemm_split=gemm_split, solve_lookahead=solve_lookahead,
                           pipeline_stages=pipeline_stages, growth_limit=growth_limit, max_ctas=max_ctas,
                           resident_compact=int(resident_compact))
        _check(lib().sog_system_create(ctx._h, plan._h, C.byref(self.opt), C.byref(self._h)))
        ctx._children.add(self)

    @staticmethod
    def _factor_rc(rc: int, allow_epivot: bool) -> int:
        if not (rc == SOG_OK or (allow_epivot and rc == SOG_EPIVOT)):
            _check(rc)
        return rc

    def factor(self, vals, allow_epivot: bool = False) -> int:
        """Factor on host values; returns SOG_OK, or SOG_EPIVOT when allowed
        (the factors are resident either way)."""
        v = np.ascontiguousarray(vals, dtype=np.float64)
        if v.shape != (self.plan.nnz,):
            raise ValueError(f"values must have shape ({self.plan.nnz},)")
        return self._factor_rc(lib().sog_factor(self._h, _p(v)), allow_epivot)

    def factor_device(self, vals_ptr: int, allow_epivot: bool = False) -> int:
        return self._factor_rc(lib().sog_factor_device(self._h, C.c_void_p(vals_ptr)), allow_epivot)

    def factor_tiles(self, tiles, allow_epivot: bool = False) -> int:
        t = np.ascontiguousarray(tiles, dtype=np.float64)
        if t.shape != (self.plan.info.n_input, 64, 64):
            raise ValueError(f"tiles must have shape ({self.plan.info.n_input}, 64, 64)")
        return self._factor_rc(lib().sog_factor_tiles(self._h, _p(t)), allow_epivot)

    def set_stream(self, stream: int) -> None:
        """Run this system on the given cudaStream_t (0 = the context's)."""
        _check(lib().sog_system_set_stream(self._h, C.c_void_p(stream or None)))

    def pivots(self) -> list[dict]:
        """Per system of the plan: min_pivot, clamped_pivots,
        inv_check_failures, max_growth and status (SOG_EPIVOT if it failed
        the pivot gate) of the last factorisation."""
        ns = len(self.plan.segments())
        st = (SolveStats * ns)()
        _check(lib().sog_system_pivots(self._h, st))
        keys = ("status", "min_pivot", "clamped_pivots", "inv_check_failures", "max_growth")
        return [{k: getattr(st[i], k) for k in keys} for i in range(ns)]

    def solve(self, b, allow_noconv: bool = False):
        """x (same shape as b: (n,) or (k, n)) and the solve statistics."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        if b.ndim not in (1, 2) or b.shape[-1] != self.n:
            raise ValueError(f"right-hand side must have shape (n,) or (k, n) with n = {self.n}")
        if b.ndim == 2 and len(self.plan.segments()) > 1:
            raise ValueError("several right-hand sides of a batch: use solve_batch")
        k = 1 if b.ndim == 1 else b.shape[0]
        x = np.empty_like(b)
        st = SolveStats()
        rc = lib().sog_solve(self._h, k, _p(b), _p(x), C.byref(st))
        if not (rc == SOG_OK or (allow_noconv and rc == SOG_ENOCONV)):
            _check(rc)
        return x, st.as_dict()

    def factor_solve(self, vals, b, allow_epivot: bool = False, allow_noconv: bool = False):
        """factor(vals) then solve(b) in one call (a plain mixed system
        overlaps the first forward substitution with the factorisation):
        x, the solve statistics and the factor's return code."""
        v = np.ascontiguousarray(vals, dtype=np.float64)
        if v.shape != (self.plan.nnz,):
            raise ValueError(f"values must have shape ({self.plan.nnz},)")
        b = np.ascontiguousarray(b, dtype=np.float64)
        if b.ndim not in (1, 2) or b.shape[-1] != self.n:
            raise ValueError(f"right-hand side must have shape (n,) or (k, n) with n = {self.n}")
        if b.ndim == 2 and len(self.plan.segments()) > 1:
            raise ValueError("several right-hand sides of a batch: use solve_batch")
        k = 1 if b.ndim == 1 else b.shape[0]
        x = np.empty_like(b)
        st = SolveStats()
        rc = lib().sog_factor_solve(self._h, _p(v), k, _p(b), _p(x), C.byref(st))
        if not (rc == SOG_OK or (allow_epivot and rc == SOG_EPIVOT) or (allow_noconv and rc == SOG_ENOCONV)):
            _check(rc)
        return x, st.as_dict(), rc

    def factor_solve_device(self, vals_ptr: int, nrhs: int, b_ptr: int, x_ptr: int) -> dict:
        st = SolveStats()
        _check(lib().sog_factor_solve_device(self._h, C.c_void_p(vals_ptr), nrhs, C.c_void_p(b_ptr),
                                             C.c_void_p(x_ptr), C.byref(st)))
        return st.as_dict()

    def solve_batch(self, bs, allow_noconv: bool = False):
        """Per-system right-hand sides of a batch system: bs[k] of shape (n_k,)
        or (r_k, n_k) (r_k may differ between systems, and may be 0). Returns
        the per-system solutions (shaped as given) and statistics."""
        ns = self.plan.segments()
        if len(bs) != len(ns):
            raise ValueError(f"expected {len(ns)} right-hand-side blocks, got {len(bs)}")
        arrs, cnt = [], np.zeros(len(ns), np.int32)
        for k, (bk, n) in enumerate(zip(bs, ns)):
            a = np.ascontiguousarray(bk, dtype=np.float64)
            if a.shape[-1] != n or a.ndim not in (1, 2):
                raise ValueError(f"system {k}: right-hand side must have shape ({n},) or (r, {n})")
            cnt[k] = 1 if a.ndim == 1 else a.shape[0]
            arrs.append(a)
        b = np.concatenate([a.ravel() for a in arrs]) if arrs else np.zeros(0)
        x = np.empty_like(b)
        st = (SolveStats * len(ns))()
        rc = lib().sog_solve_batch(self._h, _p(cnt), _p(b) if b.size else None, _p(x) if x.size else None, st)
        if not (rc == SOG_OK or (allow_noconv and rc == SOG_ENOCONV)):
            _check(rc)
        xs, o = [], 0
        for a in arrs:
            xs.append(x[o:o + a.size].reshape(a.shape))
            o += a.size
        return xs, [st[k].as_dict() for k in range(len(ns))]

    def solve_batch_device(self, nrhs, b_ptr: int, x_ptr: int) -> list[dict]:
        cnt = np.ascontiguousarray(nrhs, dtype=np.int32)
        st = (SolveStats * cnt.size)()
        _check(lib().sog_solve_batch_device(self._h, _p(cnt), C.c_void_p(b_ptr), C.c_void_p(x_ptr), st))
        return [st[k].as_dict() for k in range(cnt.size)]

    def solve_device(self, nrhs: int, b_ptr: int, x_ptr: int) -> dict:
        st = SolveStats()
        _check(lib().sog_solve_device(self._h, nrhs, C.c_void_p(b_ptr), C.c_void_p(x_ptr), C.byref(st)))
        return st.as_dict()

    def solve_permuted(self, b_ext) -> np.ndarray:
        b = np.ascontiguousarray(b_ext, dtype=np.float64)
        if b.shape != (self.plan.info.block_rows * 64,):
            raise ValueError("b_ext must have the padded length block_rows * 64")
        x = np.empty_like(b)
        _check(lib().sog_solve_permuted(self._h, _p(b), _p(x)))
        return x

    def export_factors(self):
        i = self.plan.info
        L = np.empty((i.n_lleaf, 64, 64), np.float64)
        U = np.empty((i.n_uleaf, 64, 64), np.float64)
        _check(lib().sog_system_export_factors(self._h, _p(L), _p(U)))
        return L, U

    def last_times(self):
        f, s = C.c_double(), C.c_double()
        _check(lib().sog_system_last_times(self._h, C.byref(f), C.byref(s)))
        return f.value, s.value

    def task_info(self) -> dict:
        c = np.zeros(11, np.int64)
        _check(lib().sog_system_task_info(self._h, _p(c)))
        keys = ["tasks", "levels", "items", "pairs", "gemm", "lu", "linv", "uinv", "sub", "grid", "launches"]
        return dict(zip(keys, (int(v) for v in c)))

    def executor_config(self) -> dict:
        """Executor in use (the autotuner's pick once the first factor ran)."""
        e, st, ea = C.c_int32(), C.c_int32(), C.c_int32()
        _check(lib().sog_system_executor(self._h, C.byref(e), C.byref(st), C.byref(ea)))
        return {"executor": e.value, "stages": st.value, "early_products": bool(ea.value)}

    def trace_enable(self, on: bool = True) -> None:
        _check(lib().sog_system_trace_enable(self._h, int(on)))

    def trace_get(self):
        """(tasks[t] = (ready_ns, start_ns, end_ns, sm), kinds[t], rows[i] = (l0, l1, u0, u1))."""
        ti = self.task_info()
        tt = np.zeros((ti["tasks"], 4), np.uint64)
        rt = np.zeros((self.plan.info.block_rows, 4), np.uint64)
        kind = np.zeros(ti["tasks"], np.int32)
        _check(lib().sog_system_trace_get(self._h, _p(tt), _p(rt), _p(kind)))
        tt[:, 1] = ~tt[:, 1]
        return tt, kind, rt

    def task_graph(self):
        """(succ_ptr, succ, npairs) of the device task graph."""
        ti = self.task_info()
        sp = np.zeros(ti["tasks"] + 1, np.int32)
        _check(lib().sog_system_task_graph(self._h, _p(sp), None, None))
        sc = np.zeros(max(int(sp[-1]), 1), np.int32)
        npairs = np.zeros(ti["tasks"], np.int32)
        _check(lib().sog_system_task_graph(self._h, _p(sp), _p(sc), _p(npairs)))
        return sp, sc[:sp[-1]], npairs

    def set_wait_limit(self, ms: float) -> None:
        _check(lib().sog_system_set_wait_limit(self._h, ms))

    def close(self):
        if getattr(self, "_h", None):
            lib().sog_system_destroy(self._h)
            self._h = None

    def __del__(self):
        if _lib is not None:
            self.close()


class Server:
    """Request loop with continuous batching on one context (sog_server_*):
    submit returns at once; requests are planned on host threads and merged
    into shared launches as the GPU and the block pool allow; factors stay
    resident until release."""

    def __init__(self, ctx: Context, precision: int = MIXED, max_refine: int = 10, tol: float = 1e-10,
                 planners: int = 2, omp_threads: int = 0, max_batch: int = 0, batch_window_ms: float = 0.0,
                 lanes: int = 0):
        self.ctx = ctx
        self._h = C.c_void_p()
        self.opt = Options(precision=precision, executor=EXEC_PERSISTENT, max_refine=max_refine, tol=tol)
        self.sopt = ServerOptions(planner_threads=planners, planner_omp_threads=omp_threads, max_batch=max_batch,
                                  batch_window_ms=batch_window_ms, lanes=lanes)
        self._n = {}
        _check(lib().sog_server_create(ctx._h, C.byref(self.opt), C.byref(self.sopt), C.byref(self._h)))
        ctx._children.add(self)

    def submit(self, n: int, rows, cols, vals, b, symmetric: bool = False) -> int:
        r = np.ascontiguousarray(rows, dtype=np.int32)
        c = np.ascontiguousarray(cols, dtype=np.int32)
        v = np.ascontiguousarray(vals, dtype=np.float64)
        bb = np.ascontiguousarray(b, dtype=np.float64)
        k = 1 if bb.ndim == 1 else bb.shape[0]
        if bb.size != k * n:
            raise ValueError(f"right-hand sides must have shape ({n},) or (k, {n})")
        rid = C.c_int64()
        _check(lib().sog_server_submit(self._h, int(n), r.size, _p(r), _p(c), _p(v), int(symmetric), k, _p(bb),
                                       C.byref(rid)))
        self._n[rid.value] = (n, bb.shape)
        return rid.value

    def wait(self, rid: int, timeout_ms: float = -1.0, allow_noconv: bool = False, allow_epivot: bool = False):
        """(x shaped like the submitted b, info dict). allow_epivot: return the
        solution of a system that failed the pivot gate instead of raising."""
        if rid not in self._n:
            raise SOGError(SOG_EINVAL, f"unknown or released request {rid}")
        n, shape = self._n[rid]
        x = np.empty(shape, np.float64)
        info = RequestInfo()
        rc = lib().sog_server_wait(self._h, rid, timeout_ms, _p(x), C.byref(info))
        if not (rc == SOG_OK or (allow_noconv and rc == SOG_ENOCONV) or (allow_epivot and rc == SOG_EPIVOT)):
            _check(rc)
        return x, info.as_dict()

    def solve(self, rid: int, b):
        if rid not in self._n:
            raise SOGError(SOG_EINVAL, f"unknown or released request {rid}")
        n, _ = self._n[rid]
        bb = np.ascontiguousarray(b, dtype=np.float64)
        k = 1 if bb.ndim == 1 else bb.shape[0]
        x = np.empty_like(bb)
        st = SolveStats()
        _check(lib().sog_server_solve(self._h, rid, k, _p(bb), _p(x), C.byref(st)))
        return x, st.as_dict()

    def release(self, rid: int) -> None:
        _check(lib().sog_server_release(self._h, rid))
        self._n.pop(rid, None)

    def counters(self) -> dict:
        c = np.zeros(8, np.int64)
        _check(lib().sog_server_counters(self._h, _p(c)))
        keys = ["batches", "admitted", "completed", "rejected", "max_batch", "resident", "planned_waiting",
                "to_plan"]
        return dict(zip(keys, (int(v) for v in c)))

    def close(self):
        if getattr(self, "_h", None):
            lib().sog_server_destroy(self._h)
            self._h = None

    def __del__(self):
        if _lib is not None:
            self.close()


def read_mtx(path: str, cache: bool = False):
    """MatrixMarket coordinate file with the reference reader's rules
    (sog_mtx_read): (n, rows, cols, vals, symmetric), 0-based."""
    h = C.c_void_p()
    _check(lib().sog_mtx_read(os.fsencode(path), int(cache), C.byref(h)))
    try:
        n, nnz, sym = C.c_int32(), C.c_int64(), C.c_int32()
        _check(lib().sog_mtx_info(h, C.byref(n), C.byref(nnz), C.byref(sym)))
        r = np.empty(nnz.value, np.int32)
        c = np.empty(nnz.value, np.int32)
        v = np.empty(nnz.value, np.float64)
        _check(lib().sog_mtx_copy(h, _p(r), _p(c), _p(v)))
        return n.value, r, c, v, bool(sym.value)
    finally:
        lib().sog_mtx_destroy(h)


def solveLU(dim: int, rows, cols, vals, b, symmetric: bool = False, precision: int = FP64) -> np.ndarray:
    """Drop-in for SOGLU::solveLU (solver.cpp:121-184): x in the original ordering."""
    r = np.ascontiguousarray(rows, dtype=np.int32)
    c = np.ascontiguousarray(cols, dtype=np.int32)
    v = np.ascontiguousarray(vals, dtype=np.float64)
    bb = np.ascontiguousarray(b, dtype=np.float64)
    x = np.empty(dim, np.float64)
    _check(lib().soglu_solveLU(dim, r.size, int(symmetric), _p(r), _p(c), _p(v), _p(bb), _p(x), precision))
    return x
