"""Failure handling without a GPU fault: a dependency count poisoned on the
host makes one task never ready; the persistent kernel's bounded queue wait
runs out, the call returns SOG_ETIMEOUT, and the same context then factors
and solves correctly."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("executor", [0, 2], ids=["persistent", "queue"])
def test_poisoned_dependency_times_out_then_recovers(sg, wl, executor):
    ctx = sg.Context()
    s = wl.lap2d(32)
    p = sg.Plan(s.n, s.rows, s.cols, s.vals)
    sys_ = sg.System(ctx, p, precision=sg.FP64, executor=executor)
    sys_.set_wait_limit(200.0)
    ntasks = sys_.task_info()["tasks"]
    assert sg.lib().sog_debug_poison_task(sys_._h, ntasks // 2) == 0
    with pytest.raises(sg.SOGError) as e:
        sys_.factor(s.vals)
    assert e.value.code == sg.SOG_ETIMEOUT
    assert sg.lib().sog_debug_unpoison(sys_._h) == 0
    sys_.factor(s.vals)
    x, st = sys_.solve(s.b)
    assert np.linalg.norm(x - s.x_true) / np.linalg.norm(s.x_true) < 1e-12
    with pytest.raises(ValueError):
        sys_.solve(np.zeros(3))  # wrong length is refused before any device call
    sys_.close()
    ctx.close()


def test_poisoned_factor_solve_times_out_then_recovers(sg, wl):
    """The combined call with a factor task that never becomes ready: the
    factor kernel's bounded wait runs out and the forward pass overlapping it
    stops on the factorisation's status; the call returns SOG_ETIMEOUT. The
    next combined call on the same system (with the flags the cut-short pass
    left behind) gives the results of factor then solve bit for bit."""
    import time
    ctx = sg.Context()
    s = wl.lap2d(128)
    p = sg.Plan(s.n, s.rows, s.cols, s.vals)
    ref = sg.System(ctx, p, precision=sg.MIXED, max_refine=20, tol=1e-10)
    ref.factor(s.vals)
    xr, _ = ref.solve(s.b)
    sys_ = sg.System(ctx, p, precision=sg.MIXED, max_refine=20, tol=1e-10)
    x0, _, _ = sys_.factor_solve(s.vals, s.b)
    np.testing.assert_array_equal(x0, xr)
    sys_.set_wait_limit(200.0)
    ntasks = sys_.task_info()["tasks"]
    assert sg.lib().sog_debug_poison_task(sys_._h, ntasks // 2) == 0
    t0 = time.perf_counter()
    with pytest.raises(sg.SOGError) as e:
        sys_.factor_solve(s.vals, s.b)
    assert e.value.code == sg.SOG_ETIMEOUT
    assert time.perf_counter() - t0 < 10.0
    assert sg.lib().sog_debug_unpoison(sys_._h) == 0
    x, st, rc = sys_.factor_solve(s.vals, s.b)
    assert rc == sg.SOG_OK
    np.testing.assert_array_equal(x, xr)
    sys_.close()
    ref.close()
    ctx.close()


def test_solve_before_factor_is_state_error(sg, wl):
    ctx = sg.Context()
    s = wl.lap2d(16)
    p = sg.Plan(s.n, s.rows, s.cols, s.vals)
    sys_ = sg.System(ctx, p)
    with pytest.raises(sg.SOGError) as e:
        sys_.solve(s.b)
    assert e.value.code == sg.SOG_ESTATE
    sys_.close()
    ctx.close()


def test_pool_admission_refuses_without_side_effects(sg, wl):
    s = wl.lap2d(64)
    p = sg.Plan(s.n, s.rows, s.cols, s.vals)
    need = p.bytes_needed(sg.FP64)
    ctx = sg.Context(pool_bytes=need // 4)
    with pytest.raises(sg.SOGError) as e:
        sg.System(ctx, p)
    assert e.value.code == sg.SOG_ENOMEM
    used, total = ctx.pool_usage()
    assert used == 0
    ctx.close()
