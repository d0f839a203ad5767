"""Serving engine (sog_server_*): continuous batching over the executor.

Each result must be the same alone and in the mix: a request answered while
others share its launches gets the solution it gets as the only request
(bit-identical for FP64, where the batch runs the same ops in the same order;
within the refinement tolerance for the mixed path). Admission by pool
memory: requests wait for releases when the pool is full, and a request
larger than the whole pool is refused.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests(wl, ns=(2100, 4500, 3000, 7000, 2600, 5200), seed=11):
    out = []
    for k, n in enumerate(ns):
        out.append(wl.random_band(n, seed=seed + k, nrhs=1 + (k % 4)))
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_alone_equals_mix(sg, wl, precision):
    prec = sg.FP64 if precision == "fp64" else sg.MIXED
    reqs = _requests(wl)
    ctx = sg.Context()
    # alone: one request in flight at a time, so every batch holds one system
    srv = sg.Server(ctx, precision=prec, planners=2)
    alone = []
    for s in reqs:
        rid = srv.submit(s.n, s.rows, s.cols, s.vals, s.b)
        x, info = srv.wait(rid)
        assert info["batch_size"] == 1 and info["status"] == sg.SOG_OK
        alone.append(x)
        srv.release(rid)
    assert srv.counters()["batches"] == len(reqs)
    srv.close()
    # mix: everything submitted at once; the batching window lets requests
    # still being planned join the first launch
    srv = sg.Server(ctx, precision=prec, planners=3, batch_window_ms=5000)
    ids = [srv.submit(s.n, s.rows, s.cols, s.vals, s.b) for s in reqs]
    mixed, infos = [], []
    for rid in ids:
        x, info = srv.wait(rid)
        mixed.append(x)
        infos.append(info)
    c = srv.counters()
    assert c["completed"] == len(reqs) and c["max_batch"] > 1 and c["batches"] < len(reqs)
    for s, xa, xm, info in zip(reqs, alone, mixed, infos):
        assert info["status"] == sg.SOG_OK and info["rel_resid"] <= 1e-10
        if precision == "fp64":
            np.testing.assert_array_equal(xm, xa)
        else:
            assert np.linalg.norm(xm - xa) <= 1e-10 * np.linalg.norm(xa)
        r = np.atleast_2d(s.b) - np.atleast_2d(s.matvec(xm))
        assert np.linalg.norm(r) <= 1e-10 * np.linalg.norm(s.b) * 2
    for rid in ids:
        srv.release(rid)
    assert srv.counters()["resident"] == 0
    srv.close()
    ctx.close()


def test_admission_by_pool_memory(sg, wl):
    reqs = _requests(wl, ns=(6000, 6100, 6200, 6300), seed=31)
    plans = [sg.Plan(s.n, s.rows, s.cols, s.vals) for s in reqs]
    need = max(p.bytes_needed(sg.MIXED) for p in plans)
    # room for about two requests at a time
    ctx = sg.Context(pool_bytes=int(2.6 * need))
    srv = sg.Server(ctx, precision=sg.MIXED, planners=2)
    ids = [srv.submit(s.n, s.rows, s.cols, s.vals, s.b) for s in reqs]
    done = []
    for rid, s in zip(ids, reqs):
        x, info = srv.wait(rid, timeout_ms=120000)
        assert info["status"] == sg.SOG_OK
        r = np.atleast_2d(s.b) - np.atleast_2d(s.matvec(x))
        assert np.linalg.norm(r) <= 1e-10 * np.linalg.norm(s.b) * 2
        done.append(rid)
        srv.release(rid)  # frees pool memory for the requests still waiting
    c = srv.counters()
    assert c["completed"] == len(reqs) and c["rejected"] == 0
    # larger than the whole pool: refused, not queued forever
    big = wl.random_band(40000, seed=5)
    assert sg.Plan(big.n, big.rows, big.cols, big.vals).bytes_needed(sg.MIXED) > ctx.pool_usage()[1]
    rid = srv.submit(big.n, big.rows, big.cols, big.vals, big.b)
    with pytest.raises(sg.SOGError, match="ENOMEM"):
        srv.wait(rid, timeout_ms=120000)
    assert srv.counters()["rejected"] == 1
    srv.close()
    ctx.close()


def test_further_rhs_on_resident_factors(sg, wl):
    s = wl.random_band(3500, seed=41, nrhs=2)
    ctx = sg.Context()
    srv = sg.Server(ctx, precision=sg.MIXED)
    rid = srv.submit(s.n, s.rows, s.cols, s.vals, s.b)
    x, info = srv.wait(rid)
    b2 = np.random.default_rng(3).standard_normal((3, s.n))
    x2, st = srv.solve(rid, b2)
    assert st["rel_resid"] <= 1e-10
    r = b2 - s.matvec(x2)
    assert np.linalg.norm(r) <= 1e-10 * np.linalg.norm(b2) * 2
    # the same right-hand sides again give the first answer
    x3, _ = srv.solve(rid, s.b)
    np.testing.assert_array_equal(x3, x)
    srv.release(rid)
    with pytest.raises(sg.SOGError):
        srv.solve(rid, b2)
    srv.close()
    ctx.close()


def test_symmetric_request_in_a_mixed_batch(sg, wl):
    """A symmetric request (lower triangle, LL^T) and general requests share
    one launch; each gets its own solution."""
    spd = wl.spd_lower(wl.lap2d(40))
    gen = wl.random_band(2500, seed=77, nrhs=2)
    ctx = sg.Context()
    srv = sg.Server(ctx, precision=sg.MIXED, planners=2, batch_window_ms=5000)
    a = srv.submit(spd.n, spd.rows, spd.cols, spd.vals, spd.b, symmetric=True)
    g = srv.submit(gen.n, gen.rows, gen.cols, gen.vals, gen.b)
    xa, ia = srv.wait(a)
    xg, ig = srv.wait(g)
    assert ia["batch_id"] == ig["batch_id"] and ia["batch_size"] == 2
    assert np.linalg.norm(xa - spd.x_true) <= 1e-8 * np.linalg.norm(spd.x_true)
    r = gen.b - gen.matvec(xg)
    assert np.linalg.norm(r) <= 1e-10 * np.linalg.norm(gen.b) * 2
    srv.release(a)
    srv.release(g)
    srv.close()
    ctx.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_arrival_overlaps_running_batch(sg, wl, precision):
    """A small request that arrives while a large batch is already on the GPU
    starts on a free lane and is answered before the large one, with the
    same result it gets alone (FP64 bit for bit, mixed within the refinement
    tolerance)."""
    import time
    prec = sg.FP64 if precision == "fp64" else sg.MIXED
    big = wl.varcoef3d(40)
    small = wl.random_band(2400, seed=5, nrhs=2)
    ctx = sg.Context()
    alone = {}
    for name, s in (("big", big), ("small", small)):
        p = sg.Plan(s.n, s.rows, s.cols, s.vals)
        sysm = sg.System(ctx, p, precision=prec, max_refine=10)
        sysm.factor(s.vals)
        alone[name], _ = sysm.solve(s.b)
        sysm.close()
    srv = sg.Server(ctx, precision=prec, planners=2, lanes=2)
    rb = srv.submit(big.n, big.rows, big.cols, big.vals, big.b)
    t0 = time.time()
    while srv.counters()["admitted"] < 1:  # the big request has been handed to a lane
        assert time.time() - t0 < 60
        time.sleep(0.001)
    rs = srv.submit(small.n, small.rows, small.cols, small.vals, small.b)
    xs, info_s = srv.wait(rs)
    # the small one is answered while the big one is still running
    with pytest.raises(sg.SOGError, match="ETIMEOUT"):
        srv.wait(rb, timeout_ms=0)
    xb, info_b = srv.wait(rb)
    assert info_s["batch_id"] != info_b["batch_id"] and info_s["batch_size"] == 1
    for x, key in ((xs, "small"), (xb, "big")):
        if precision == "fp64":
            np.testing.assert_array_equal(x, alone[key])
        else:
            assert np.linalg.norm(x - alone[key]) <= 1e-9 * np.linalg.norm(alone[key])
    srv.release(rs)
    srv.release(rb)
    srv.close()
    ctx.close()
