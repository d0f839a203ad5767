"""Pin the oracle (oracle/soglu_oracle.c, a C restatement of the reference's
executor path) against the compiled reference's own outputs stored in
tests/golden/: solution vectors and L/U tiles."""
import numpy as np
import pytest

from conftest import golden, golden_cases, rhs_of


@pytest.mark.parametrize("name", ["lap2d_8", "lap2d_32", "lap2d_128", "var3d_16", "cd_40", "cd_17", "band_3000",
                                  "band_130", "spd_lap2d_8", "spd_lap2d_32", "spd_var3d_16"])
def test_oracle_solution_matches_reference(sg, wl, oracle, name):
    """spd_* cases take the reference's LL^T path (llt / mult ops; the back
    substitution with L^T)."""
    s = golden_cases(wl)[name]()
    g = golden(name)
    # run the oracle on the REFERENCE's own DAG and ordering
    plan = sg.Plan(s.n, s.rows, s.cols, s.vals, symmetric=s.symmetric)
    n_input = plan.info.n_input
    tiles_in = plan.input_tiles(s.vals)
    stats = dict(l.split("=") for l in str(g["stats"]).split())
    R = int(stats["block_rows"])
    x, tiles, nan = oracle.solve_system(g["perm"], s.n, R, g["dag"], int(stats["storage_count"]), tiles_in,
                                        g["lleaf"], g["uleaf"], rhs_of(s))
    assert nan == 0
    rel = np.linalg.norm(x - g["x"]) / np.linalg.norm(g["x"])
    assert rel <= 1e-12, rel
    if "tiles" in g:
        nl = len(g["lleaf"])
        for k, (_, _, bid) in enumerate(g["lleaf"]):
            np.testing.assert_allclose(tiles[bid], g["tiles"][k], rtol=0, atol=1e-12)
        for k, (_, _, bid) in enumerate(g["uleaf"]):
            np.testing.assert_allclose(tiles[bid], g["tiles"][nl + k], rtol=0, atol=1e-12)
    assert n_input > 0


def test_oracle_reference_accuracy(sg, wl, oracle):
    """Known-answer check: b = A x_true."""
    s = wl.varcoef3d(12)
    p = sg.Plan(s.n, s.rows, s.cols, s.vals)
    perm, ops, L, U = p.export()
    x, _, _ = oracle.solve_system(perm, s.n, p.info.block_rows, ops, p.info.storage_count, p.input_tiles(s.vals),
                                  L, U, s.b)
    assert np.linalg.norm(x - s.x_true) / np.linalg.norm(s.x_true) < 1e-10


def test_oracle_detects_planted_error(sg, wl, oracle):
    """A mistake planted in the oracle's inputs (one DAG op dropped) is caught
    by the same comparison the tests rely on."""
    s = wl.lap2d(32)
    g = golden("lap2d_32")
    p = sg.Plan(s.n, s.rows, s.cols, s.vals)
    stats = dict(l.split("=") for l in str(g["stats"]).split())
    dag = g["dag"].copy()
    k = int(np.nonzero(dag[:, 0] == 8)[0][0])  # first mul
    dag = np.delete(dag, k, axis=0)
    x, _, _ = oracle.solve_system(g["perm"], s.n, int(stats["block_rows"]), dag, int(stats["storage_count"]),
                                  p.input_tiles(s.vals), g["lleaf"], g["uleaf"], s.b)
    assert np.linalg.norm(x - g["x"]) / np.linalg.norm(g["x"]) > 1e-6


@pytest.mark.parametrize("name", ["lap2d_32", "var3d_16", "cd_17", "band_3000", "zdiag_600", "spd_lap2d_32",
                                  "spd_var3d_16"])
def test_oracle_lean_path_matches_flat_and_reference(sg, wl, oracle, name):
    """The reference's block lifetime in the oracle (lazy allocation, free
    after the last reading stage; solve_system_multi) gives bit for bit the
    flat-array result on the reference's own DAG, and holds fewer blocks than
    the DAG names."""
    s = golden_cases(wl)[name]()
    g = golden(name)
    plan = sg.Plan(s.n, s.rows, s.cols, s.vals, symmetric=s.symmetric)
    tiles_in = plan.input_tiles(s.vals)
    stats = dict(l.split("=") for l in str(g["stats"]).split())
    R, sc = int(stats["block_rows"]), int(stats["storage_count"])
    b = rhs_of(s)
    x_flat, _, _ = oracle.solve_system(g["perm"], s.n, R, g["dag"], sc, tiles_in, g["lleaf"], g["uleaf"], b)
    st = {}
    B = np.stack([b, 2.0 * b, -b])
    X = oracle.solve_system_multi(g["perm"], s.n, R, g["dag"], sc, tiles_in, g["lleaf"], g["uleaf"], B, stats=st)
    assert st["nan"] == 0
    np.testing.assert_array_equal(X[0], x_flat)
    assert np.linalg.norm(X[0] - g["x"]) / np.linalg.norm(g["x"]) <= 1e-12
    # columns are independent solves: a scaled right-hand side scales x (up to rounding)
    np.testing.assert_allclose(X[1], 2.0 * X[0], rtol=0, atol=1e-12 * np.abs(X[0]).max())
    np.testing.assert_allclose(X[2], -X[0], rtol=0, atol=1e-12 * np.abs(X[0]).max())
    assert 0 < st["peak_blocks"] < sc
