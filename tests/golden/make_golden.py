"""Generate the golden fixtures in this directory from the REFERENCE solver.

Runs oracle/_ref/ref_solve (the reference's own sources compiled by
oracle/build_ref.sh; x86-64 with AVX-512 only) on seeded synthetic systems
and stores, per case, in <case>.npz:
  perm   final permutation (GOrder::newOrder after sortInBlock)
  dag    fine op DAG after the last blockPlan, rows {op,src,src2,result,result2,stage}
  lleaf, uleaf   L/U quadtree leaves {bi, bj, block id}
  x      the reference's solution in the original ordering (solveLU's return value)
  tiles  (small cases) dense L/U tiles in lleaf/uleaf order
  stats  the reference's key=value summary (op counts, stages, phase times)
  ahash  sha256 of the generated triplets, to detect generator drift
For the large cases (48^3 var-coef, 64^3 Laplacian) only hashes, counts and x
are stored.

usage: python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import hashlib
import importlib.util
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def load_workloads():
    path = os.path.join(ROOT, "sparse-operator-graph-lu_gb300", "workloads.py")
    spec = importlib.util.spec_from_file_location("soglu_workloads", path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules["soglu_workloads"] = mod
    spec.loader.exec_module(mod)
    return mod


def triplet_hash(s) -> str:
    h = hashlib.sha256()
    h.update(np.int64(s.n).tobytes())
    h.update(s.rows.tobytes()); h.update(s.cols.tobytes()); h.update(s.vals.tobytes())
    return h.hexdigest()


def zero_diag_case(wl):
    """Random band system whose diagonal is exactly zero on a few rows of the
    leading half of some 64-row blocks, so the in-block diagonal sort
    (GPSOrder.cpp:55-150) reorders rows."""
    s = wl.random_band(600, seed=11, band_frac=0.05)
    d = (s.rows == s.cols)
    idx = np.nonzero(d)[0]
    kill = idx[(s.rows[idx] % 97) == 3]
    keep = np.ones(s.nnz, bool)
    keep[kill] = False
    s.rows, s.cols, s.vals = s.rows[keep], s.cols[keep], s.vals[keep]
    s.b = s.b[0]
    s.name = "zdiag_600"
    return s


LARGE = ("var3d_48", "lap3d_64")


def cases(wl):
    c = {
        "lap2d_32": (lambda: wl.lap2d(32), True),
        "lap2d_128": (lambda: wl.lap2d(128), False),
        "var3d_16": (lambda: wl.varcoef3d(16), False),
        "cd_40": (lambda: wl.convdiff2d(40, 5.0, 1.0, nrhs=1), False),
        "cd_17": (lambda: wl.convdiff2d(17, 9.0, 4.0, nrhs=1), True),
        "band_3000": (lambda: wl.random_band(3000, seed=5), False),
        "band_130": (lambda: wl.random_band(130, seed=7), True),
        "lap2d_8": (lambda: wl.lap2d(8), True),
        "zdiag_600": (lambda: zero_diag_case(wl), False),
        "var3d_48": (lambda: wl.varcoef3d(48), False),
        # 3D 7-point Laplacian 64^3 (7.1M ops): x for the first right-hand side
        # of the 64-RHS bench system (same x_true stream, seed 0)
        "lap3d_64": (lambda: wl.lap3d(64), False),
        # symmetric input: lower triangle given, the reference factors L L^T
        "spd_lap2d_32": (lambda: wl.spd_lower(wl.lap2d(32)), True),
        "spd_var3d_16": (lambda: wl.spd_lower(wl.varcoef3d(16)), False),
        "spd_lap2d_8": (lambda: wl.spd_lower(wl.lap2d(8)), True),
    }
    return c


def run_case(wl, name, make, with_tiles, ref_bin, tmp):
    s = make()
    b = s.b if s.b.ndim == 1 else s.b[0]
    mtx = os.path.join(tmp, f"{name}.mtx")
    wl.write_mtx(mtx, s)
    wl.write_rhs(os.path.join(tmp, f"{name}_b.mtx"), b)
    out = os.path.join(tmp, name)
    os.makedirs(out, exist_ok=True)
    cmd = [ref_bin, mtx, os.path.join(tmp, f"{name}_b.mtx"), out] + (["--tiles"] if with_tiles else [])
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL)
    rd = lambda f, dt: np.fromfile(os.path.join(out, f), dtype=dt)
    dag = rd("dag.i32", np.int32).reshape(-1, 6)
    stats = open(os.path.join(out, "stats.txt")).read()
    arrs = dict(perm=rd("perm.i32", np.int32), lleaf=rd("lblk.i32", np.int32).reshape(-1, 3),
                uleaf=rd("ublk.i32", np.int32).reshape(-1, 3), x=rd("x.f64", np.float64),
                stats=np.array(stats), ahash=np.array(triplet_hash(s)),
                daghash=np.array(hashlib.sha256(dag.tobytes()).hexdigest()))
    if name in LARGE:  # keep x, hash the structure
        for k in ("perm", "lleaf", "uleaf"):
            a = arrs.pop(k)
            if k != "perm":  # leaves hashed in (block row, block col) order
                a = np.ascontiguousarray(a[np.lexsort((a[:, 1], a[:, 0]))])
            arrs[k + "hash"] = np.array(hashlib.sha256(a.tobytes()).hexdigest())
    else:
        arrs["dag"] = dag
    if with_tiles:
        arrs["tiles"] = rd("tiles.f64", np.float64).reshape(-1, 64, 64)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrs)
    print(name, s.n, s.nnz, dag.shape[0], "ops")


def main(argv):
    wl = load_workloads()
    ref_bin = os.path.join(ROOT, "oracle", "_ref", "ref_solve")
    subprocess.run(["sh", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    if not os.path.exists(ref_bin):
        sys.exit("reference build unavailable on this host")
    want = argv or list(cases(wl).keys())
    with tempfile.TemporaryDirectory() as tmp:
        for name, (make, tiles) in cases(wl).items():
            if name in want:
                run_case(wl, name, make, tiles, ref_bin, tmp)


if __name__ == "__main__":
    main(sys.argv[1:])
