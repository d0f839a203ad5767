"""The C-ABI library loads and exports every entry point include/soglu_gb300.h
declares; host-only entry points work without a GPU; device entry points fail
loudly (no CPU fallback)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, gpu_available


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "soglu_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b((?:sog|soglu)_[A-Za-z_0-9]+)\s*\(", txt)))


def test_exports_every_declared_symbol(sg):
    L = ctypes.CDLL(sg.LIB_PATH)
    syms = header_symbols()
    assert len(syms) >= 25
    for s in syms:
        assert hasattr(L, s), f"{s} declared but not exported"
    assert sorted(sg.EXPORTS) == syms


def test_version_and_error_string(sg):
    assert b"sm_103a" in sg.lib().sog_version()
    with pytest.raises(sg.SOGError):
        sg.Plan(-1, np.zeros(0), np.zeros(0), np.zeros(0))
    assert len(sg.lib().sog_last_error()) > 0


@pytest.mark.skipif(gpu_available(), reason="checks the no-device path")
def test_no_device_is_an_error_not_a_fallback(sg, wl):
    with pytest.raises(sg.SOGError) as e:
        sg.Context()
    assert e.value.code in (sg.SOG_ENODEV, sg.SOG_ECUDA)
    s = wl.lap2d(16)
    with pytest.raises(sg.SOGError):
        sg.solveLU(s.n, s.rows, s.cols, s.vals, s.b)


def test_cli_plans_like_the_reference(sg, wl, tmp_path):
    s = wl.lap2d(32)
    wl.write_mtx(str(tmp_path / "a.mtx"), s)
    wl.write_rhs(str(tmp_path / "a_b.mtx"), s.b)
    exe = os.path.join(ROOT, "sparse-operator-graph-lu_gb300", "bin", "solve")
    r = subprocess.run([exe], capture_output=True, text=True)
    assert "usage" in r.stdout
    r = subprocess.run([exe, str(tmp_path / "a.mtx")], capture_output=True, text=True, timeout=120)
    assert "op count: 173 storage: 386" in r.stdout
    if not gpu_available():
        assert r.returncode != 0  # no device: loud failure


def test_mtx_reader_acceptance_rules(sg, tmp_path):
    """Reader rules of mtx.cpp:44-117: '%' lines and lines of <= 3 chars are
    skipped, zero values dropped, out-of-range rows dropped."""
    p = tmp_path / "r.mtx"
    p.write_text("%%MatrixMarket matrix coordinate real general\n% comment\n\n"
                 "64 64 70\n" + "".join(f"{i} {i} 4\n" for i in range(1, 65)) +
                 "1 2 0\n65 1 7\n1 2 -1\n2 1 -1\n")
    exe = os.path.join(ROOT, "sparse-operator-graph-lu_gb300", "bin", "solve")
    r = subprocess.run([exe, str(p)], capture_output=True, text=True, timeout=60)
    # 66 accepted entries, n = 64 -> 2 block rows, one lu per block row
    assert "inputSize: 64" in r.stdout and "op count: 2" in r.stdout


def test_mtx_reader_triplets_parallel_and_cache(sg, wl, tmp_path):
    """sog_mtx_read returns the accepted triplets in file order, also when the
    entry lines are parsed in parallel chunks (a file of several MB), and the
    binary cache returns the same triplets until the text file changes."""
    import numpy as np
    s = wl.lap3d(40)  # 438k entries: several parallel chunks
    p = tmp_path / "lap.mtx"
    with open(p, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real general\n%\n")
        f.write(f"{s.n} {s.n} {s.nnz + 3}\n")
        f.write("1 1 0\n")  # zero value: dropped
        for k in range(s.nnz):
            f.write(f"{s.rows[k] + 1} {s.cols[k] + 1} {float(s.vals[k])!r}\n")
            if k == s.nnz // 2:
                f.write("% a comment in the middle\n12\n")  # skipped lines
        f.write(f"{s.n + 5} 1 3.0\n")  # beyond the size: dropped
    n, r, c, v, sym = sg.read_mtx(str(p))
    assert n == s.n and not sym
    np.testing.assert_array_equal(r, s.rows)
    np.testing.assert_array_equal(c, s.cols)
    np.testing.assert_array_equal(v, s.vals)
    cache = tmp_path / "lap.mtx.sogbin"
    assert not cache.exists()
    first = sg.read_mtx(str(p), cache=True)
    assert cache.exists()
    second = sg.read_mtx(str(p), cache=True)
    for a, b in zip(first[1:4], second[1:4]):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(second[3], s.vals)
    # the text file changes: the stale cache is not used
    with open(p, "a") as f:
        f.write("1 2 -0.5\n")
    third = sg.read_mtx(str(p), cache=True)
    assert third[1].size == s.nnz + 1 and third[3][-1] == -0.5
    with pytest.raises(sg.SOGError):
        sg.read_mtx(str(tmp_path / "missing.mtx"))


# entry points whose first argument is an opaque handle (plan, context,
# system, server) or an array of them
HANDLE_ENTRIES = [
    "sog_plan_get_info", "sog_plan_export", "sog_plan_input_tiles", "sog_plan_segments", "sog_plan_task_graph_info",
    "sog_ctx_pool_usage", "sog_ctx_stream", "sog_ctx_trim", "sog_system_create", "sog_system_bytes",
    "sog_factor", "sog_factor_device", "sog_factor_tiles", "sog_solve", "sog_solve_device", "sog_factor_solve",
    "sog_factor_solve_device", "sog_solve_permuted", "sog_solve_batch", "sog_solve_batch_device",
    "sog_system_export_factors", "sog_system_last_times", "sog_system_task_info", "sog_system_executor",
    "sog_system_pivots", "sog_system_set_stream", "sog_system_set_wait_limit", "sog_debug_poison_task",
    "sog_debug_unpoison", "sog_debug_fp64_fragment_skip", "sog_system_trace_enable", "sog_system_trace_get",
    "sog_system_task_graph", "sog_plan_merge", "sog_server_create", "sog_server_submit", "sog_server_wait",
    "sog_server_solve", "sog_server_release", "sog_server_counters", "sog_mtx_info", "sog_mtx_copy",
]


def test_null_handles_are_rejected(sg):
    """Every entry point that takes a handle answers a NULL handle (and NULL
    outputs) with SOG_EINVAL, without touching the device; the destructors
    accept NULL."""
    L = sg.lib()
    for name in HANDLE_ENTRIES:
        f = getattr(L, name)
        args = []
        for t in f.argtypes:
            if t is ctypes.c_void_p or t is ctypes.c_char_p:
                args.append(None)
            elif t is ctypes.c_double:
                args.append(1.0)
            else:
                args.append(1)
        assert f(*args) == sg.SOG_EINVAL, name
    for name in ("sog_plan_destroy", "sog_ctx_destroy", "sog_system_destroy", "sog_server_destroy",
                 "sog_mtx_destroy"):
        getattr(L, name)(None)
