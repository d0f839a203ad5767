"""Host planner vs the reference planner (golden fixtures from the compiled
reference): permutation, op DAG and L/U leaves must be identical, op for op."""
import hashlib

import numpy as np
import pytest

from conftest import golden, golden_cases, load_package


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def triplet_hash(s):
    h = hashlib.sha256()
    h.update(np.int64(s.n).tobytes())
    h.update(s.rows.tobytes()); h.update(s.cols.tobytes()); h.update(s.vals.tobytes())
    return h.hexdigest()


@pytest.mark.parametrize("name", ["lap2d_8", "lap2d_32", "lap2d_128", "var3d_16", "cd_40", "cd_17", "band_3000",
                                  "band_130", "zdiag_600", "spd_lap2d_8", "spd_lap2d_32", "spd_var3d_16"])
def test_plan_matches_reference(sg, wl, name):
    """symmetric (spd_*) inputs give the reference's LL^T DAG (llt / mult ops, L leaves only)."""
    s = golden_cases(wl)[name]()
    g = golden(name)
    assert triplet_hash(s) == str(g["ahash"]), "generator drifted from the fixture"
    p = sg.Plan(s.n, s.rows, s.cols, s.vals, symmetric=s.symmetric)
    perm, ops, L, U = p.export()
    np.testing.assert_array_equal(perm, g["perm"])
    assert ops.shape == g["dag"].shape
    np.testing.assert_array_equal(ops, g["dag"])
    key = lambda a: a[np.lexsort((a[:, 1], a[:, 0]))]
    np.testing.assert_array_equal(key(L), key(g["lleaf"]))
    np.testing.assert_array_equal(key(U), key(g["uleaf"]))
    stats = dict(l.split("=") for l in str(g["stats"]).split())
    assert p.info.storage_count == int(stats["storage_count"])
    assert p.info.stages == int(stats["stages"])
    assert p.info.coarse_ops == int(stats["coarse_ops"])
    assert p.info.fine_ops_emitted == int(stats["fine_ops_emitted"])


def test_plan_48cube_matches_reference_hashes(sg, wl):
    """The bench configuration (3D var-coef 48^3, 1.08M ops): full-size DAG identity."""
    s = wl.varcoef3d(48)
    g = golden("var3d_48")
    assert triplet_hash(s) == str(g["ahash"])
    p = sg.Plan(s.n, s.rows, s.cols, s.vals)
    perm, ops, L, U = p.export()
    assert _sha(perm) == str(g["permhash"])
    assert _sha(ops) == str(g["daghash"])
    assert _sha(L) == str(g["lleafhash"]) and _sha(U) == str(g["uleafhash"])
    info = p.info_dict()
    assert info["nops"] == 1082718 and info["stages"] == 11904
    assert info["ops"] == {"lu": 2048, "lowerInv": 3679, "upperInv": 3679, "sub": 72926, "mul": 839513,
                           "mulneg": 160873}


def test_plan_64cube_matches_reference_hashes(sg, wl):
    """The headline configuration (3D 7-point Laplacian 64^3, 7.1M ops):
    full-size DAG identity with the reference's."""
    s = wl.lap3d(64)
    g = golden("lap3d_64")
    assert triplet_hash(s) == str(g["ahash"])
    p = sg.Plan(s.n, s.rows, s.cols, s.vals)
    perm, ops, L, U = p.export()
    assert _sha(perm) == str(g["permhash"])
    assert _sha(ops) == str(g["daghash"])
    assert _sha(L) == str(g["lleafhash"]) and _sha(U) == str(g["uleafhash"])
    info = p.info_dict()
    stats = dict(l.split("=") for l in str(g["stats"]).split())
    assert info["nops"] == 7106089 and info["stages"] == int(stats["stages"])
    assert info["block_rows"] == int(stats["block_rows"]) and info["storage_count"] == int(stats["storage_count"])


def test_config_rounding(sg, wl):
    # block rows = next power of two strictly above n/64 (config.cpp:30-49)
    for side, br in ((8, 2), (16, 8), (32, 32), (128, 512)):
        s = wl.lap2d(side)
        assert sg.Plan(s.n, s.rows, s.cols, s.vals).info.block_rows == br


def test_input_tiles_scatter(sg, wl):
    s = wl.lap2d(32)
    p = sg.Plan(s.n, s.rows, s.cols, s.vals)
    perm, ops, L, U = p.export()
    t = p.input_tiles(s.vals)
    # reassemble the permuted matrix from tiles and compare with P A P^T
    A = np.zeros((s.n, s.n))
    A[s.rows, s.cols] = s.vals
    Ap = A[np.ix_(perm, perm)]
    R = p.info.block_rows
    full = np.zeros((R * 64, R * 64))
    # input tile k carries block id k+1, allocated in (block row, block col)
    # order of the permuted triplets (BlockPlanner.cpp:1491-1520)
    o2n = np.argsort(perm)
    keys = sorted({(i // 64, j // 64) for i, j in zip(o2n[s.rows], o2n[s.cols])})
    for k, (bi, bj) in enumerate(keys):
        full[bi * 64:(bi + 1) * 64, bj * 64:(bj + 1) * 64] = t[k]
    np.testing.assert_array_equal(full[:s.n, :s.n], Ap)


@pytest.mark.parametrize("bad", ["index", "zero_block"])
def test_plan_rejects_bad_input(sg, wl, bad):
    s = wl.lap2d(16)
    rows, cols, vals = s.rows.copy(), s.cols.copy(), s.vals.copy()
    sym = False
    if bad == "index":
        rows[3] = s.n + 5
    else:  # drop every entry of block row 0 -> structurally zero diagonal block
        keep = (rows >= 64) & (cols >= 64)
        rows, cols, vals = rows[keep], cols[keep], vals[keep]
    with pytest.raises(sg.SOGError) as e:
        sg.Plan(s.n, rows, cols, vals, symmetric=sym)
    assert e.value.code == sg.SOG_EINVAL


def test_disconnected_and_isolated_nodes(sg):
    # two decoupled chains plus isolated diagonal-only rows: ordering covers all nodes
    n = 300
    r, c, v = [], [], []
    for i in range(n):
        r.append(i); c.append(i); v.append(4.0)
        if i % 3 != 2 and i + 3 < n:
            r += [i, i + 3]; c += [i + 3, i]; v += [-1.0, -1.0]
    p = sg.Plan(n, np.array(r), np.array(c), np.array(v))
    perm = p.export()[0]
    assert sorted(perm.tolist()) == list(range(n))


@pytest.mark.parametrize("name", ["lap2d_32", "var3d_16", "band_3000", "cd_17"])
def test_task_graph(sg, wl, name):
    """Device task graph (host-built): every op becomes part of exactly one
    task, each Schur sub is fused into its product, levels <= the reference's
    stages, acyclic (the builder checks)."""
    s = golden_cases(wl)[name]()
    p = sg.Plan(s.n, s.rows, s.cols, s.vals)
    info = p.info_dict()
    tg = p.task_graph_info(gemm_split=1)
    ops = info["ops"]
    assert tg["lu"] == ops.get("lu", 0)
    assert tg["pairs"] == ops.get("mul", 0) + ops.get("mulneg", 0)
    assert tg["sub"] + tg["fused_subs"] + tg["aliased_copies"] == ops.get("sub", 0)
    assert tg["linv"] + tg["uinv"] + tg["fused_inverses"] + tg["aliased_inverses"] == \
        ops.get("lowerInv", 0) + ops.get("upperInv", 0) + tg["added_inverses"]
    assert 0 < tg["fused_inverses"] <= 2 * tg["lu"]  # lowerInv and upperInv of each LU
    assert tg["levels"] <= info["stages"]
    assert tg["critical_path"] == tg["levels"]
    tg4 = p.task_graph_info(gemm_split=4)
    assert tg4["items"] == tg["items"] + 3 * tg["gemm"]


def test_task_graph_48cube(sg, wl):
    s = wl.varcoef3d(48)
    tg = sg.Plan(s.n, s.rows, s.cols, s.vals).task_graph_info()
    assert tg["fused_subs"] > 40000 and tg["levels"] < 11904
