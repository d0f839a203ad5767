"""Analysis of the executor's device timestamps (System.trace_get).

Splits the factorisation time into task execution and scheduling latency,
per task kind and along the critical path (the chain of tasks that finished
last, each joined to the predecessor that finished last before it).
"""
from __future__ import annotations

import numpy as np

KIND_NAMES = ["gemm", "lu", "linv", "uinv", "sub", "llt", "trans", "gemm+lu", "gemm+llt"]


def analyze(tt: np.ndarray, kind: np.ndarray, succ_ptr: np.ndarray, succ: np.ndarray,
            npairs: np.ndarray | None = None) -> dict:
    tt = tt.astype(np.int64)
    ready, start, end = tt[:, 0], tt[:, 1], tt[:, 2]
    t0 = int(start.min())
    ready = np.where(ready == 0, t0, ready)
    dur = (end - start) / 1e3  # us
    wait = (start - ready) / 1e3
    out = {"span_us": (int(end.max()) - t0) / 1e3, "tasks": int(tt.shape[0]), "kinds": {}}
    for k, name in enumerate(KIND_NAMES):
        m = kind == k
        if not m.any():
            continue
        d = {"count": int(m.sum()), "dur_mean_us": float(dur[m].mean()), "dur_p50_us": float(np.median(dur[m])),
             "dur_p99_us": float(np.percentile(dur[m], 99)), "wait_mean_us": float(wait[m].mean()),
             "busy_us": float(dur[m].sum())}
        if name == "gemm" and npairs is not None:
            d["us_per_pair"] = float(dur[m].sum() / max(1, npairs[m].sum()))
        out["kinds"][name] = d
    # predecessors
    n = tt.shape[0]
    pred_of = [[] for _ in range(n)]
    for t in range(n):
        for s in succ[succ_ptr[t]:succ_ptr[t + 1]]:
            pred_of[s].append(t)
    cur = int(np.argmax(end))
    path = []
    while cur >= 0:
        path.append(cur)
        ps = pred_of[cur]
        cur = max(ps, key=lambda p: end[p]) if ps else -1
    path.reverse()
    seg = {"exec_us": {}, "latency_us": 0.0, "length": len(path)}
    prev_end = t0
    for t in path:
        nm = KIND_NAMES[kind[t]]
        seg["exec_us"][nm] = seg["exec_us"].get(nm, 0.0) + float(dur[t])
        seg["latency_us"] += (int(start[t]) - prev_end) / 1e3
        prev_end = int(end[t])
    seg["count_by_kind"] = {KIND_NAMES[k]: int(sum(1 for t in path if kind[t] == k)) for k in range(len(KIND_NAMES))}
    out["critical_path"] = seg
    return out


def analyze_rows(rt: np.ndarray) -> dict:
    rt = rt.astype(np.int64)
    lo = {"span_us": (rt[:, 1].max() - rt[:, 0].min()) / 1e3, "row_us_mean": float(((rt[:, 1] - rt[:, 0]) / 1e3).mean())}
    up = {"span_us": (rt[:, 3].max() - rt[:, 2].min()) / 1e3, "row_us_mean": float(((rt[:, 3] - rt[:, 2]) / 1e3).mean())}
    # publish-to-publish gap along consecutive rows
    lo["step_us_mean"] = float(np.diff(np.sort(rt[:, 1])).mean() / 1e3)
    up["step_us_mean"] = float(np.diff(np.sort(rt[:, 3])).mean() / 1e3)
    return {"lower": lo, "upper": up}
