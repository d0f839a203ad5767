"""ORACLE — test infrastructure, not the product.

ctypes wrapper around oracle/soglu_oracle.c, the plain-C restatement of the
reference's executor path (BlockPlanner::calculate, BlockPlanner.cpp:376-651,
and BlockPlanner::solve, BlockPlanner.cpp:652-862). Only tests/, the smoke
check and bench.py's CPU-baseline leg use it, as the checker or as the timed
CPU baseline. Pinned against the compiled reference through tests/golden/.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "soglu_oracle.c")
SO = os.path.join(HERE, "liboracle.so")

_lib = None


def build() -> str:
    """Compile liboracle.so (portable flags; OpenMP)."""
    if not os.path.exists(SO) or os.path.getmtime(SO) < os.path.getmtime(SRC):
        subprocess.run(["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp", SRC, "-o", SO, "-lm"], check=True)
    return SO


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(SO)
        P = C.c_void_p
        L.oracle_calculate.argtypes = [C.c_int64, P, C.c_int32, P, C.c_int]
        L.oracle_calculate.restype = C.c_int
        L.oracle_solve.argtypes = [C.c_int32, C.c_int64, P, C.c_int64, P, P, P, P]
        L.oracle_solve.restype = C.c_int64
        L.oracle_solve_lean.argtypes = [C.c_int64, P, C.c_int32, C.c_int32, P, C.c_int32, C.c_int64, P, C.c_int64,
                                        P, C.c_int32, P, P, C.c_int, P]
        L.oracle_solve_lean.restype = C.c_int64
        _lib = L
    return _lib


def calculate(ops: np.ndarray, storage_count: int, input_tiles: np.ndarray, threads: int = 0) -> np.ndarray:
    """Run the op DAG; returns all tiles (storage_count x 64 x 64), block id = index."""
    ops = np.ascontiguousarray(ops, dtype=np.int32).reshape(-1, 6)
    tiles = np.zeros((storage_count, 64, 64), np.float64)
    n_in = input_tiles.shape[0]
    tiles[1:1 + n_in] = input_tiles
    rc = lib().oracle_calculate(ops.shape[0], ops.ctypes.data, storage_count, tiles.ctypes.data, threads)
    if rc != 0:
        raise RuntimeError(f"oracle_calculate failed ({rc})")
    return tiles


def solve(block_rows: int, L: np.ndarray, U: np.ndarray, tiles: np.ndarray, b_ext: np.ndarray):
    """Block forward/back substitution; returns (x_ext, nan_count)."""
    L = np.ascontiguousarray(L, dtype=np.int32)
    U = np.ascontiguousarray(U, dtype=np.int32)
    b = np.array(b_ext, dtype=np.float64, copy=True)
    x = np.zeros(block_rows * 64, np.float64)
    nan = lib().oracle_solve(block_rows, L.shape[0], L.ctypes.data, U.shape[0], U.ctypes.data, tiles.ctypes.data,
                             b.ctypes.data, x.ctypes.data)
    return x, int(nan)


def transposed_upper(L: np.ndarray, tiles: np.ndarray):
    """For an LL^T plan (no U leaves): U = L^T as leaves over transposed copies
    of the L tiles appended to `tiles` (upperSolverT, BlockPlanner.cpp:752-797,
    solves with the transposed L blocks). Returns (tiles, U leaves)."""
    L = np.asarray(L, dtype=np.int32).reshape(-1, 3)
    extra = np.ascontiguousarray(np.transpose(tiles[L[:, 2]], (0, 2, 1)))
    ids = np.arange(tiles.shape[0], tiles.shape[0] + L.shape[0], dtype=np.int32)
    U = np.stack([L[:, 1], L[:, 0], ids], axis=1).astype(np.int32)
    return np.concatenate([tiles, extra]), U


def solve_system(perm_new_to_old: np.ndarray, n: int, block_rows: int, ops, storage_count, input_tiles, L, U,
                 b: np.ndarray, threads: int = 0):
    """Full executor path in the original ordering: permute b (padded rows = 1,
    solver.cpp:159-161), calculate, substitute, un-permute (GPSOrder.cpp:41-53).
    An empty U means an LL^T plan: the back substitution uses L^T."""
    tiles = calculate(ops, storage_count, input_tiles, threads)
    if len(U) == 0:
        tiles, U = transposed_upper(L, tiles)
    b_ext = np.ones(block_rows * 64)
    b_ext[:n] = np.asarray(b)[perm_new_to_old]
    x_ext, nan = solve(block_rows, L, U, tiles, b_ext)
    x = np.empty(n)
    x[perm_new_to_old] = x_ext[:n]
    return x, tiles, nan


def solve_system_multi(perm_new_to_old: np.ndarray, n: int, block_rows: int, ops, storage_count, input_tiles, L, U,
                       B: np.ndarray, threads: int = 0, stats: dict | None = None) -> np.ndarray:
    """One calculate, then one substitution per right-hand side (rows of B,
    original ordering, solved in parallel): the reference's factor-once,
    solve-each path, with its block lifetime (allocate on first write, free
    after the last stage that reads a block), so the host memory it needs is
    the reference's. stats (optional) receives the peak live block count."""
    ops = np.ascontiguousarray(ops, dtype=np.int32).reshape(-1, 6)
    L = np.ascontiguousarray(L, dtype=np.int32).reshape(-1, 3)
    U = np.ascontiguousarray(U, dtype=np.int32).reshape(-1, 3)
    tin = np.ascontiguousarray(input_tiles, dtype=np.float64)
    B = np.atleast_2d(np.asarray(B, dtype=np.float64))
    nrhs, n_ext = B.shape[0], block_rows * 64
    b_ext = np.ones((nrhs, n_ext))
    b_ext[:, :n] = B[:, perm_new_to_old]
    x_ext = np.zeros((nrhs, n_ext))
    peak = C.c_int64(0)
    rc = lib().oracle_solve_lean(ops.shape[0], ops.ctypes.data, storage_count, tin.shape[0], tin.ctypes.data,
                                 block_rows, L.shape[0], L.ctypes.data, U.shape[0], U.ctypes.data, nrhs,
                                 b_ext.ctypes.data, x_ext.ctypes.data, threads, C.byref(peak))
    if rc < 0:
        raise RuntimeError(f"oracle_solve_lean failed ({rc})")
    if stats is not None:
        stats["peak_blocks"] = int(peak.value)
        stats["nan"] = int(rc)
    X = np.empty_like(B)
    X[:, perm_new_to_old] = x_ext[:, :n]
    return X
