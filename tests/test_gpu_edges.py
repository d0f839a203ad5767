"""Edge cases of the executor path on the GPU: tiny systems (one real row,
fewer rows than a tile), duplicate triplets (the last one wins, as the
reference's block fill), a zero pivot (clamped to 1e-9 like ludcmpSimple and
counted), more than 64 right-hand sides (chunked), a right-hand side of
zeros, and non-finite input reported as NaNs rather than hidden."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _solve(sg, n, r, c, v, b, precision, symmetric=False, growth_limit=0.0):
    ctx = sg.Context()
    p = sg.Plan(n, r, c, v, symmetric=symmetric)
    s = sg.System(ctx, p, precision=precision, max_refine=20, tol=1e-10, growth_limit=growth_limit)
    s.factor(v)
    x, st = s.solve(b, allow_noconv=True)
    s.close()
    ctx.close()
    return x, st


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("n", [1, 5, 63, 64, 65])
def test_tiny_and_ragged_sizes(sg, precision, n):
    rng = np.random.default_rng(n)
    a = np.diag(4.0 + rng.random(n))
    for i in range(n - 1):
        a[i, i + 1] = -1.0
        a[i + 1, i] = -1.5
    r, c = np.nonzero(a)
    v = a[r, c]
    b = rng.standard_normal(n)
    prec = sg.FP64 if precision == "fp64" else sg.MIXED
    x, st = _solve(sg, n, r, c, v, b, prec)
    xr = np.linalg.solve(a, b)
    assert np.linalg.norm(x - xr) <= 1e-10 * max(1.0, np.linalg.norm(xr))
    assert st["rel_resid"] <= 1e-10


def test_duplicate_triplets_last_wins(sg):
    n = 70
    a = np.diag(np.full(n, 5.0))
    r, c = np.nonzero(a)
    v = a[r, c].copy()
    # a duplicate of (3, 3) with another value after the original: the later value is used
    r = np.append(r, [3, 10]); c = np.append(c, [3, 11]); v = np.append(v, [2.0, -1.0])
    a[3, 3] = 2.0
    a[10, 11] = -1.0
    b = np.arange(1.0, n + 1)
    x, st = _solve(sg, n, r, c, v, b, sg.FP64)
    np.testing.assert_allclose(x, np.linalg.solve(a, b), rtol=1e-12)


def test_zero_pivot_is_clamped_and_counted(sg):
    """[[1, 1], [1, 1]] without pivoting: u_11 = 1 - 1 = 0 exactly, raised to
    1e-9 as ludcmpSimple does; the clamp is reported and b = (2, 2) gives the
    clamped system's solution: 2 for the row ordered first, 0 for the other
    (the ordering may swap them). (A zero leading diagonal would instead be
    moved by the in-block diagonal sort of the ordering.) With the pivot gate
    off (growth_limit < 0) the factorisation is the reference's
    clamp-and-continue."""
    r = np.array([0, 0, 1, 1]); c = np.array([0, 1, 0, 1]); v = np.ones(4)
    x, st = _solve(sg, 2, r, c, v, np.array([2.0, 2.0]), sg.FP64, growth_limit=-1.0)
    assert st["clamped_pivots"] >= 1 and st["min_pivot"] == 0.0
    assert sorted(x.tolist()) == [0.0, 2.0]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_many_rhs_chunks(sg, wl, precision):
    s = wl.convdiff2d(20, 3.0, 0.5, nrhs=130)
    prec = sg.FP64 if precision == "fp64" else sg.MIXED
    x, st = _solve(sg, s.n, s.rows, s.cols, s.vals, s.b, prec)
    assert x.shape == (130, s.n)
    res = s.b - s.matvec(x)
    assert np.linalg.norm(res) <= 1e-10 * np.linalg.norm(s.b) * 12
    assert st["rel_resid"] <= 1e-10


def test_zero_rhs_gives_zero(sg, wl):
    s = wl.lap2d(20)
    x, st = _solve(sg, s.n, s.rows, s.cols, s.vals, np.zeros(s.n), sg.MIXED)
    assert np.all(x == 0) and st["nan_count"] == 0


def test_nonfinite_input_is_reported(sg, wl):
    s = wl.lap2d(16)
    v = s.vals.copy()
    v[5] = np.nan
    ctx = sg.Context()
    p = sg.Plan(s.n, s.rows, s.cols, v)
    sys_ = sg.System(ctx, p, precision=sg.FP64)
    # the pivot gate sees the non-finite factor (U U^-1 check) ...
    with pytest.raises(sg.SOGError, match="EPIVOT"):
        sys_.factor(v)
    assert sys_.pivots()[0]["inv_check_failures"] >= 1
    # ... and a caller that goes on anyway gets the NaNs reported by the solve
    assert sys_.factor(v, allow_epivot=True) == sg.SOG_EPIVOT
    with pytest.raises(sg.SOGError, match="ENAN"):
        sys_.solve(s.b)
    sys_.close()
    ctx.close()
