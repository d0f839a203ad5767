"""Seeded synthetic sparse systems for the factor-and-solve path.

The reference ships no matrices and no benchmark suite; these generators stand
in for its inputs with the shapes, sizes and value distributions of the five
benchmark configurations. Every generator returns 0-based COO triplets
(rows, cols, vals) in int32/int32/float64, the dimension, and where it
applies x_true and b = A @ x_true. MatrixMarket I/O follows the acceptance
rules of the reference reader (mtx.cpp:44-117, 145-181).
"""
from __future__ import annotations

import dataclasses
import numpy as np


@dataclasses.dataclass
class System:
    n: int
    rows: np.ndarray  # int32, 0-based
    cols: np.ndarray  # int32, 0-based
    vals: np.ndarray  # float64
    b: np.ndarray  # float64, (n,) or (n, nrhs) column-major stacked as (nrhs, n)
    x_true: np.ndarray | None = None
    name: str = ""
    symmetric: bool = False  # triplets hold the lower triangle of a symmetric A

    @property
    def nnz(self) -> int:
        return int(self.vals.shape[0])

    def matvec(self, x: np.ndarray) -> np.ndarray:
        """y = A @ x in float64 (x: (n,) or (k, n))."""
        x = np.asarray(x, dtype=np.float64)
        if x.ndim == 1:
            y = np.zeros(self.n)
            np.add.at(y, self.rows, self.vals * x[self.cols])
            if self.symmetric:
                off = self.rows != self.cols
                np.add.at(y, self.cols[off], self.vals[off] * x[self.rows[off]])
            return y
        if self.symmetric:
            return np.stack([self.matvec(xi) for xi in x])
        import scipy.sparse as sp
        a = sp.csr_matrix((self.vals, (self.rows, self.cols)), shape=(self.n, self.n))
        return np.ascontiguousarray((a @ x.T).T)

    def to_scipy(self):
        import scipy.sparse as sp
        a = sp.csr_matrix((self.vals, (self.rows, self.cols)), shape=(self.n, self.n))
        if self.symmetric:
            a = a + sp.tril(a, -1).T.tocsr()
        return a


def spd_lower(s: "System") -> "System":
    """The same symmetric system given as its lower triangle (MatrixMarket
    `symmetric` storage: the reader mirrors it, solveLU factors it as L L^T)."""
    keep = s.rows >= s.cols
    out = System(n=s.n, rows=np.ascontiguousarray(s.rows[keep]), cols=np.ascontiguousarray(s.cols[keep]),
                 vals=np.ascontiguousarray(s.vals[keep]), b=s.b, x_true=s.x_true, name="spd_" + s.name,
                 symmetric=True)
    return out


def _finish(n, r, c, v, x_true, name, nrhs_b=None):
    r = np.ascontiguousarray(r, dtype=np.int32)
    c = np.ascontiguousarray(c, dtype=np.int32)
    v = np.ascontiguousarray(v, dtype=np.float64)
    s = System(n=n, rows=r, cols=c, vals=v, b=None, x_true=x_true, name=name)
    if x_true is not None:
        s.b = s.matvec(x_true)
    return s


def lap2d(side: int = 128, diag: float = 4.01, seed: int = 0) -> System:
    """2D 5-point Laplacian on side x side (n = side^2); diagonal `diag`,
    off-diagonals -1; x_true ~ U[-1, 1] from default_rng(seed); b = A x_true."""
    n = side * side
    idx = np.arange(n).reshape(side, side)
    r = [idx.ravel()]
    c = [idx.ravel()]
    v = [np.full(n, diag)]
    for a, b_ in ((idx[1:, :], idx[:-1, :]), (idx[:-1, :], idx[1:, :]),
                  (idx[:, 1:], idx[:, :-1]), (idx[:, :-1], idx[:, 1:])):
        r.append(a.ravel()); c.append(b_.ravel()); v.append(np.full(a.size, -1.0))
    x_true = np.random.default_rng(seed).uniform(-1.0, 1.0, n)
    return _finish(n, np.concatenate(r), np.concatenate(c), np.concatenate(v), x_true, f"lap2d_{side}")


def lap3d(side: int = 64, diag: float = 6.01, seed: int = 0, nrhs: int = 1) -> System:
    """3D 7-point Laplacian on side^3; diagonal `diag`, off-diagonals -1;
    x_true ~ U[-1, 1] from default_rng(seed): shape (n,) for one right-hand
    side, (nrhs, n) otherwise; b = A x_true column by column."""
    n = side ** 3
    idx = np.arange(n).reshape(side, side, side)
    r = [idx.ravel()]
    c = [idx.ravel()]
    v = [np.full(n, diag)]
    for ax in range(3):
        lo = [slice(None)] * 3
        hi = [slice(None)] * 3
        lo[ax] = slice(0, side - 1)
        hi[ax] = slice(1, side)
        a, b_ = idx[tuple(lo)].ravel(), idx[tuple(hi)].ravel()
        r += [a, b_]; c += [b_, a]; v += [np.full(a.size, -1.0)] * 2
    shape = n if nrhs == 1 else (nrhs, n)
    x_true = np.random.default_rng(seed).uniform(-1.0, 1.0, shape)
    return _finish(n, np.concatenate(r), np.concatenate(c), np.concatenate(v), x_true, f"lap3d_{side}")


def varcoef3d(side: int = 48, shift: float = 1e-3, kseed: int = 1, xseed: int = 0) -> System:
    """3D 7-point variable-coefficient diffusion on side^3.

    Per-cell k = exp(N(0,1)) from default_rng(kseed). Interior face coefficient
    = harmonic mean 2 k_i k_j / (k_i + k_j). Dirichlet boundary: a face on the
    domain boundary contributes the cell's own k to the diagonal (our fixed
    choice; the configuration leaves it open). diag = sum of face coefficients
    + shift. x_true ~ U[-1, 1] from default_rng(xseed)."""
    n = side ** 3
    k = np.exp(np.random.default_rng(kseed).standard_normal(n)).reshape(side, side, side)
    idx = np.arange(n).reshape(side, side, side)
    d = np.full((side, side, side), shift)
    r, c, v = [], [], []
    for ax in range(3):
        lo = [slice(None)] * 3
        hi = [slice(None)] * 3
        lo[ax] = slice(0, side - 1)
        hi[ax] = slice(1, side)
        kl, kh = k[tuple(lo)], k[tuple(hi)]
        f = 2.0 * kl * kh / (kl + kh)
        d[tuple(lo)] += f
        d[tuple(hi)] += f
        a, b_ = idx[tuple(lo)].ravel(), idx[tuple(hi)].ravel()
        r += [a, b_]; c += [b_, a]; v += [-f.ravel(), -f.ravel()]
        first = [slice(None)] * 3
        last = [slice(None)] * 3
        first[ax] = 0
        last[ax] = side - 1
        d[tuple(first)] += k[tuple(first)]
        d[tuple(last)] += k[tuple(last)]
    r = [idx.ravel()] + r
    c = [idx.ravel()] + c
    v = [d.ravel()] + v
    x_true = np.random.default_rng(xseed).uniform(-1.0, 1.0, n)
    return _finish(n, np.concatenate(r), np.concatenate(c), np.concatenate(v), x_true, f"varcoef3d_{side}")


def convdiff2d(side: int, peclet: float, theta: float, nrhs: int = 4, seed: int = 0) -> System:
    """Nonsymmetric 2D convection-diffusion, 5-point first-order upwind on
    side x side with Dirichlet boundary. Velocity (cos theta, sin theta), cell
    Peclet number `peclet`: each face carries diffusion 1 plus the upwind
    convective flux peclet*max(+-v, 0). b holds `nrhs` right-hand sides
    ~ N(0,1) from default_rng(seed), shape (nrhs, n)."""
    n = side * side
    vx, vy = np.cos(theta), np.sin(theta)
    idx = np.arange(n).reshape(side, side)  # [iy, ix]
    # coefficients for the west/east/south/north neighbours
    cw = -(1.0 + peclet * max(vx, 0.0))
    ce = -(1.0 + peclet * max(-vx, 0.0))
    cs = -(1.0 + peclet * max(vy, 0.0))
    cn = -(1.0 + peclet * max(-vy, 0.0))
    dg = 4.0 + peclet * (abs(vx) + abs(vy))
    r, c, v = [idx.ravel()], [idx.ravel()], [np.full(n, dg)]
    for (a, b_, coef) in ((idx[:, 1:], idx[:, :-1], cw), (idx[:, :-1], idx[:, 1:], ce),
                          (idx[1:, :], idx[:-1, :], cs), (idx[:-1, :], idx[1:, :], cn)):
        r.append(a.ravel()); c.append(b_.ravel()); v.append(np.full(a.size, coef))
    s = _finish(n, np.concatenate(r), np.concatenate(c), np.concatenate(v), None,
                f"convdiff_{side}_{peclet:.2f}_{theta:.2f}")
    s.b = np.random.default_rng(seed).standard_normal((nrhs, n))
    return s


def convdiff_batch(count: int = 1024, seed: int = 2, nrhs: int = 4) -> list[System]:
    """The batch configuration: `count` independent conv-diff systems with
    side ~ U{16..96}, Peclet ~ U[0,10], angle ~ U[0, 2 pi) from
    default_rng(seed); each with `nrhs` N(0,1) right-hand sides."""
    g = np.random.default_rng(seed)
    sides = g.integers(16, 97, count)
    pes = g.uniform(0.0, 10.0, count)
    ths = g.uniform(0.0, 2 * np.pi, count)
    return [convdiff2d(int(sides[i]), float(pes[i]), float(ths[i]), nrhs=nrhs, seed=seed * 100003 + i)
            for i in range(count)]


def random_band(n: int, seed: int, band_frac: float = 0.02, nnz_lo: int = 3, nnz_hi: int = 27,
                nrhs: int = 1) -> System:
    """Serving request: n x n with 3..27 off-diagonal entries per row placed
    uniformly within half-band band_frac*n, off-diagonals ~ N(0,1), diagonal
    = 1.1 x row abs sum (diagonally dominant). b: (nrhs, n) ~ N(0,1)."""
    g = np.random.default_rng(seed)
    hb = max(1, int(band_frac * n))
    per = g.integers(nnz_lo, nnz_hi + 1, n)
    rr = np.repeat(np.arange(n), per)
    off = g.integers(-hb, hb + 1, rr.size)
    off[off == 0] = 1
    cc = np.clip(rr + off, 0, n - 1)
    keep = cc != rr
    rr, cc = rr[keep], cc[keep]
    key = np.unique(rr.astype(np.int64) * n + cc)
    rr, cc = (key // n).astype(np.int64), (key % n).astype(np.int64)
    vv = g.standard_normal(rr.size)
    dg = 1.1 * np.bincount(rr, weights=np.abs(vv), minlength=n)
    dg[dg == 0] = 1.0
    s = _finish(n, np.concatenate([np.arange(n), rr]), np.concatenate([np.arange(n), cc]),
                np.concatenate([dg, vv]), None, f"band_{n}_{seed}")
    s.b = g.standard_normal((nrhs, n))
    return s


def serving_requests(count: int, seed: int = 3, n_lo: int = 2000, n_hi: int = 200000):
    """Request stream for the serving configuration: n log-uniform in
    [n_lo, n_hi], 1..16 right-hand sides per request."""
    g = np.random.default_rng(seed)
    ns = np.exp(g.uniform(np.log(n_lo), np.log(n_hi), count)).astype(int)
    ks = g.integers(1, 17, count)
    return [(int(ns[i]), int(seed * 7919 + i), int(ks[i])) for i in range(count)]


# ---------------------------------------------------------------- MatrixMarket
def write_mtx(path: str, s: System) -> None:
    """Write A as `%%MatrixMarket matrix coordinate real general` (or
    `symmetric`, lower triangle, for a symmetric system), 1-based."""
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real " + ("symmetric" if s.symmetric else "general") + "\n")
        f.write(f"{s.n} {s.n} {s.nnz}\n")
        lines = [f"{r + 1} {c + 1} {v:.17g}\n" for r, c, v in zip(s.rows.tolist(), s.cols.tolist(), s.vals.tolist())]
        f.writelines(lines)


def write_rhs(path: str, b: np.ndarray) -> None:
    """Write one right-hand side as `%%MatrixMarket matrix array real general`."""
    b = np.asarray(b, dtype=np.float64).ravel()
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix array real general\n")
        f.write(f"{b.size} 1\n")
        f.writelines(f"{v:.17g}\n" for v in b.tolist())


CONFIGS = {
    # name: (factory, description)
    "lap2d_128": (lambda: lap2d(128), "2D 5-point Laplacian 128x128, diag 4.01"),
    "varcoef3d_48": (lambda: varcoef3d(48), "3D 7-point var-coef diffusion 48^3"),
    "lap3d_64": (lambda: lap3d(64), "3D 7-point Laplacian 64^3, diag 6.01"),
}
