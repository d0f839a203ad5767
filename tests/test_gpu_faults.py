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
