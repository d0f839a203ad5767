"""The pivot gate on the GPU. The method factors without pivoting, so the
executor checks every diagonal-block factorisation: the pivots (clamped to
+-1e-9 as ludcmpSimple does, MatrixStdDouble.cpp:2751-2761), the reference's
U U^-1 check after upperInv (inv_check_diag, MatrixStdDouble.cpp:2871-2937),
and the element growth against sog_options.growth_limit. All inputs are
crafted on the host; nothing here faults the device."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(sg):
    c = sg.Context()
    yield c
    c.close()


def growth_system(n=200, eps=1e-7, seed=0):
    """Identity except a coupled pair [[eps, 1], [1, eps]]: whichever of the
    two rows the ordering puts first, its pivot is eps and the other's is
    eps - 1/eps, so the element growth is about 1/eps (max |a_ij| = 1) in
    every ordering."""
    a_r, a_c, a_v = list(range(n)), list(range(n)), [1.0] * n
    i, j = 37, 38
    a_v[i] = a_v[j] = eps
    a_r += [i, j]; a_c += [j, i]; a_v += [1.0, 1.0]
    r, c, v = np.array(a_r, np.int32), np.array(a_c, np.int32), np.array(a_v)
    b = np.random.default_rng(seed).standard_normal(n)
    return n, r, c, v, b


def singular_system(n=130):
    """Identity except an exactly singular coupled pair [[1, 1], [1, 1]]: the
    second pivot is 1 - 1 = 0 and gets clamped."""
    a_r, a_c, a_v = list(range(n)), list(range(n)), [1.0] * n
    i, j = 5, 90
    a_r += [i, j]; a_c += [j, i]; a_v += [1.0, 1.0]
    return n, np.array(a_r, np.int32), np.array(a_c, np.int32), np.array(a_v)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_growth_reported_and_gated(sg, ctx, precision):
    prec = sg.FP64 if precision == "fp64" else sg.MIXED
    n, r, c, v, b = growth_system()
    p = sg.Plan(n, r, c, v)
    s = sg.System(ctx, p, precision=prec, max_refine=30)
    # default limits: 1e8 (FP64), 1e4 (mixed); the growth here is ~1e7
    if prec == sg.FP64:
        assert s.factor(v) == sg.SOG_OK
    else:
        with pytest.raises(sg.SOGError, match="EPIVOT"):
            s.factor(v)
    pv = s.pivots()[0]
    assert pv["max_growth"] == pytest.approx(1e7, rel=1e-3)
    assert pv["min_pivot"] == pytest.approx(1e-7, rel=1e-6)
    assert pv["clamped_pivots"] == 0 and pv["inv_check_failures"] == 0
    assert pv["status"] == (sg.SOG_OK if prec == sg.FP64 else sg.SOG_EPIVOT)
    # the figures also travel with every solve's statistics
    if prec == sg.FP64:
        x, st = s.solve(b)
        assert st["max_growth"] == pytest.approx(pv["max_growth"])
        assert st["min_pivot"] == pv["min_pivot"]
    s.close()
    # an explicit limit below the growth gates FP64 too; the factors stay usable
    s = sg.System(ctx, p, precision=sg.FP64, growth_limit=1e6)
    assert s.factor(v, allow_epivot=True) == sg.SOG_EPIVOT
    x, st = s.solve(b)
    A = np.zeros((n, n)); A[r, c] = v
    assert np.linalg.norm(A @ x - b) <= 1e-6 * np.linalg.norm(b)
    s.close()
    # the gate off: the reference's behaviour
    s = sg.System(ctx, p, precision=prec, growth_limit=-1.0)
    assert s.factor(v) == sg.SOG_OK
    assert s.pivots()[0]["status"] == sg.SOG_OK
    s.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_singular_block_is_clamped_and_gated(sg, ctx, precision):
    prec = sg.FP64 if precision == "fp64" else sg.MIXED
    n, r, c, v = singular_system()
    p = sg.Plan(n, r, c, v)
    s = sg.System(ctx, p, precision=prec)
    with pytest.raises(sg.SOGError, match="EPIVOT"):
        s.factor(v)
    pv = s.pivots()[0]
    assert pv["clamped_pivots"] == 1 and pv["min_pivot"] == 0.0 and pv["status"] == sg.SOG_EPIVOT
    # the clamped pivot is the pair's last one: nothing is eliminated with it, U stays O(1)
    assert pv["max_growth"] == pytest.approx(1.0)
    s.close()


@pytest.mark.parametrize("name", ["lap2d_32", "cd_17", "band_3000", "var3d_16"])
def test_well_conditioned_inputs_pass(sg, wl, ctx, name):
    """Diagonally dominant (band, upwind convection-diffusion) and SPD inputs:
    growth at most 2 (dominant) or 1 (SPD), no clamp, no failed check."""
    from conftest import golden_cases
    s = golden_cases(wl)[name]()
    p = sg.Plan(s.n, s.rows, s.cols, s.vals)
    for prec in (sg.FP64, sg.MIXED):
        sysm = sg.System(ctx, p, precision=prec)
        assert sysm.factor(s.vals) == sg.SOG_OK
        pv = sysm.pivots()[0]
        assert pv["status"] == sg.SOG_OK and pv["clamped_pivots"] == 0 and pv["inv_check_failures"] == 0
        assert 0 < pv["max_growth"] <= 2.0 + 1e-6
        sysm.close()


def test_spd_llt_growth_at_most_one(sg, wl, ctx):
    s = wl.spd_lower(wl.varcoef3d(12))
    p = sg.Plan(s.n, s.rows, s.cols, s.vals, symmetric=True)
    sysm = sg.System(ctx, p, precision=sg.FP64)
    assert sysm.factor(s.vals) == sg.SOG_OK
    pv = sysm.pivots()[0]
    assert pv["status"] == sg.SOG_OK and 0 < pv["max_growth"] <= 1.0 + 1e-9
    sysm.close()


def test_batch_gate_is_per_system(sg, wl, ctx):
    """In a batch only the system that failed the gate is flagged, and every
    system's pivot figures are the ones it gets alone."""
    good = wl.lap2d(20)
    n, r, c, v, b = growth_system()
    plans = [sg.Plan(good.n, good.rows, good.cols, good.vals), sg.Plan(n, r, c, v),
             sg.Plan(good.n, good.rows, good.cols, good.vals)]
    alone = []
    for pl, vals in zip(plans, [good.vals, v, good.vals]):
        sysm = sg.System(ctx, pl, precision=sg.MIXED)
        sysm.factor(vals, allow_epivot=True)
        alone.append(sysm.pivots()[0])
        sysm.close()
    m = sg.merge_plans(plans)
    bs = sg.System(ctx, m, precision=sg.MIXED)
    assert bs.factor(np.concatenate([good.vals, v, good.vals]), allow_epivot=True) == sg.SOG_EPIVOT
    got = bs.pivots()
    assert [g["status"] for g in got] == [sg.SOG_OK, sg.SOG_EPIVOT, sg.SOG_OK]
    for g, a in zip(got, alone):
        assert g["max_growth"] == a["max_growth"] and g["min_pivot"] == a["min_pivot"]
        assert g["clamped_pivots"] == a["clamped_pivots"]
    bs.close()


def test_solveLU_keeps_reference_behaviour(sg):
    """The outer drop-in (SOGLU::solveLU) clamps and continues like the
    reference: no gate."""
    n, r, c, v = singular_system()
    x = sg.solveLU(n, r, c, v, np.ones(n))
    assert np.isfinite(x).all()
