"""Batch plans: the block-diagonal union of independent systems (sog_plan_merge).

CPU tests check the merged DAG against its parts (every op, leaf and value
scatter of each system, shifted); GPU tests check that a system factored and
solved inside a batch gives the result it gets alone, and the oracle's.
"""
import numpy as np
import pytest


def _systems(wl, sides=(16, 23, 9, 30), nrhs=2):
    out = []
    for k, side in enumerate(sides):
        out.append(wl.convdiff2d(side, 2.0 + k, 0.7 * k, nrhs=nrhs, seed=100 + k))
    return out


def _remap(plans):
    """Per system the block-id map of the merge: inputs first, then the rest."""
    n_in = sum(p.info.n_input for p in plans)
    maps, in_off, other_off = [], 0, n_in
    for p in plans:
        ni, st = p.info.n_input, p.info.storage_count
        m = np.zeros(st, np.int64)
        ids = np.arange(st)
        m[1:ni + 1] = in_off + ids[1:ni + 1]
        m[ni + 1:] = other_off + (ids[ni + 1:] - ni)
        maps.append(m)
        in_off += ni
        other_off += st - 1 - ni
    return maps


def test_merge_plans_structure(sg, wl):
    systems = _systems(wl)
    plans = [sg.Plan(s.n, s.rows, s.cols, s.vals) for s in systems]
    m = sg.merge_plans(plans)
    i = m.info
    assert m.segments() == [s.n for s in systems]
    assert i.n == sum(s.n for s in systems)
    assert i.block_rows == sum(p.info.block_rows for p in plans)
    assert i.n_ext == 64 * i.block_rows
    assert i.n_input == sum(p.info.n_input for p in plans)
    assert i.storage_count == 1 + sum(p.info.storage_count - 1 for p in plans)
    assert i.nops == sum(p.info.nops for p in plans)
    assert i.stages == max(p.info.stages for p in plans)
    assert list(i.op_count) == list(np.sum([list(p.info.op_count) for p in plans], axis=0))
    assert m.nnz == sum(s.nnz for s in systems)
    # ops: every system's ops, remapped, in its own order; whole list by stage
    _, mops, mL, mU = m.export()
    assert np.all(np.diff(mops[:, 5]) >= 0)
    maps = _remap(plans)
    owner = np.full(i.storage_count, -1)
    for k, mp in enumerate(maps):
        owner[mp[1:]] = k
    assert np.all(owner[1:] >= 0)  # the remap is a bijection onto 1..storage-1
    res_owner = owner[mops[:, 3]]
    rows0 = np.cumsum([0] + [p.info.block_rows for p in plans])
    for k, p in enumerate(plans):
        _, ops, L, U = p.export()
        mine = mops[res_owner == k]
        exp = ops.copy()
        for c in (1, 2, 3, 4):
            exp[:, c] = np.where(ops[:, c] > 0, maps[k][np.maximum(ops[:, c], 0)], ops[:, c])
        # stable sort by stage keeps the system's own order
        np.testing.assert_array_equal(mine, exp[np.argsort(exp[:, 5], kind="stable")])
        for mine_l, leaves in ((mL, L), (mU, U)):
            sel = owner[mine_l[:, 2]] == k
            exp_l = leaves.copy()
            exp_l[:, :2] += rows0[k]
            exp_l[:, 2] = maps[k][leaves[:, 2]]
            np.testing.assert_array_equal(mine_l[sel], exp_l)


def test_merge_plans_input_tiles(sg, wl):
    """The merged value scatter places each system's values in its own tiles."""
    systems = _systems(wl, sides=(12, 17))
    plans = [sg.Plan(s.n, s.rows, s.cols, s.vals) for s in systems]
    m = sg.merge_plans(plans)
    t = m.input_tiles(np.concatenate([s.vals for s in systems]))
    o = 0
    for p, s in zip(plans, systems):
        tk = p.input_tiles(s.vals)
        np.testing.assert_array_equal(t[o:o + tk.shape[0]], tk)
        o += tk.shape[0]
    assert o == t.shape[0]


def test_merge_plans_task_graph(sg, wl):
    systems = _systems(wl)
    plans = [sg.Plan(s.n, s.rows, s.cols, s.vals) for s in systems]
    m = sg.merge_plans(plans)
    g = m.task_graph_info()
    parts = [p.task_graph_info() for p in plans]
    for key in ("tasks", "pairs", "gemm", "lu", "linv", "uinv", "sub", "fused_subs", "aliased_copies"):
        assert g[key] == sum(q[key] for q in parts), key
    assert g["critical_path"] == max(q["critical_path"] for q in parts)


def test_merge_plans_rejects(sg, wl):
    s = wl.convdiff2d(10, 1.0, 0.0)
    p = sg.Plan(s.n, s.rows, s.cols, s.vals)
    m = sg.merge_plans([p, p])
    assert m.segments() == [s.n, s.n]
    with pytest.raises(sg.SOGError, match="EINVAL"):
        sg.merge_plans([m, p])
    _, ops, L, U = p.export()
    imp = sg.Plan.imported(p.info.block_rows, p.info.storage_count, p.info.n_input, ops, L, U)
    with pytest.raises(sg.SOGError, match="EINVAL"):
        sg.merge_plans([p, imp])
    with pytest.raises(sg.SOGError, match="EINVAL"):
        sg.merge_plans([])


def _alone(sg, ctx, s, precision, nrhs):
    p = sg.Plan(s.n, s.rows, s.cols, s.vals)
    sysm = sg.System(ctx, p, precision=precision)
    sysm.factor(s.vals)
    xs = []
    for r in range(nrhs):
        x, st = sysm.solve(s.b[r])
        xs.append(x)
    sysm.close()
    return np.array(xs).reshape(nrhs, s.n)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_matches_alone(sg, wl, oracle, precision):
    prec = sg.FP64 if precision == "fp64" else sg.MIXED
    systems = _systems(wl, sides=(16, 23, 9, 30, 41, 12), nrhs=3)
    counts = [3, 1, 0, 2, 3, 1]  # right-hand sides per system, one system without any
    plans = [sg.Plan(s.n, s.rows, s.cols, s.vals) for s in systems]
    ctx = sg.Context()
    m = sg.merge_plans(plans)
    bs = sg.System(ctx, m, precision=prec)
    bs.factor(np.concatenate([s.vals for s in systems]))
    assert bs.task_info()["launches"] >= 1
    xs, stats = bs.solve_batch([s.b[:c] for s, c in zip(systems, counts)])
    for k, (s, c) in enumerate(zip(systems, counts)):
        assert xs[k].shape == (c, s.n)
        if c == 0:
            continue
        assert stats[k]["status"] == sg.SOG_OK
        assert stats[k]["rel_resid"] <= 1e-10
        alone = _alone(sg, ctx, s, prec, c)
        if precision == "fp64":
            # same ops, same order, same kernels: bit-identical to the system alone
            np.testing.assert_array_equal(xs[k], alone)
            perm, ops, L, U = plans[k].export()
            for r in range(c):
                xo, _, _ = oracle.solve_system(perm, s.n, plans[k].info.block_rows, ops, plans[k].info.storage_count,
                                               plans[k].input_tiles(s.vals), L, U, s.b[r])
                assert np.linalg.norm(xs[k][r] - xo) <= 1e-10 * np.linalg.norm(xo)
        else:
            # refinement stops per system, so the iterates match the system alone
            # (up to the order of the residual norm's parallel sums deciding a step)
            assert np.linalg.norm(xs[k] - alone) <= 1e-10 * np.linalg.norm(alone)
            res = s.b[:c] - s.matvec(xs[k])
            assert np.linalg.norm(res) <= 1e-10 * np.linalg.norm(s.b[:c]) * np.sqrt(c)
    bs.close()
    ctx.close()


@pytest.mark.gpu
def test_batch_uniform_rhs_and_device_entry(sg, wl):
    """sog_solve on a batch (uniform count, one rhs) equals sog_solve_batch."""
    torch = pytest.importorskip("torch")
    systems = _systems(wl, sides=(14, 19, 25), nrhs=1)
    plans = [sg.Plan(s.n, s.rows, s.cols, s.vals) for s in systems]
    ctx = sg.Context()
    bs = sg.System(ctx, sg.merge_plans(plans), precision=sg.MIXED)
    bs.factor(np.concatenate([s.vals for s in systems]))
    b = np.concatenate([s.b[0] for s in systems])
    x1, st = bs.solve(b)
    xs, _ = bs.solve_batch([s.b[0] for s in systems])
    np.testing.assert_array_equal(x1, np.concatenate(xs))
    db = torch.tensor(b, device="cuda:0")
    dx = torch.empty_like(db)
    stats = bs.solve_batch_device([1, 1, 1], db.data_ptr(), dx.data_ptr())
    np.testing.assert_array_equal(dx.cpu().numpy(), x1)
    assert all(q["rel_resid"] <= 1e-10 for q in stats)
    bs.close()
    ctx.close()


@pytest.mark.gpu
def test_clustered_substitution_matches_batch_path(sg, wl):
    """A plain system's full 8-column chunks run the substitution in thread-
    block clusters (rows handed over through distributed shared memory); the
    same system inside a batch runs the unclustered kernel. FP64 results are
    bit-identical (same products in the same order), with 16 right-hand sides
    (two chunks of one launch) and a 40x40 grid (32 block rows)."""
    big = wl.convdiff2d(40, 3.0, 0.5, nrhs=16, seed=7)
    small = wl.convdiff2d(9, 2.0, 0.0, nrhs=1, seed=8)
    ctx = sg.Context()
    p = sg.Plan(big.n, big.rows, big.cols, big.vals)
    alone = sg.System(ctx, p, precision=sg.FP64)
    alone.factor(big.vals)
    xa, sa = alone.solve(big.b)
    alone.close()
    plans = [p, sg.Plan(small.n, small.rows, small.cols, small.vals)]
    bs = sg.System(ctx, sg.merge_plans(plans), precision=sg.FP64)
    bs.factor(np.concatenate([big.vals, small.vals]))
    xs, stats = bs.solve_batch([big.b, small.b[:1]])
    bs.close()
    assert sa["rel_resid"] <= 1e-12 and stats[0]["rel_resid"] <= 1e-12
    np.testing.assert_array_equal(xs[0], xa)
    ctx.close()
