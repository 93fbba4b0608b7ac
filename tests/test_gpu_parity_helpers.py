"""Leaf IB fractions of the fixture problems (ProbeSolver::injectIBFrac of
oracle/ref_dump.cpp), shared by the CPU and GPU parity tests."""
import numpy as np

from cases import CASES


def _frac(c, pts, h):
    nd = len(pts)
    d2 = np.zeros_like(pts[0])
    for d in range(nd):
        d2 = d2 + (pts[d] - c["ibc"][d]) * (pts[d] - c["ibc"][d])
    s = (np.sqrt(d2) - c["ibr"]) / h + 0.5
    s = np.clip(s, 0.0, 1.0)
    return np.floor(s * 64.0) / 64.0


def fractional_ib(name, tb):
    """leaf IB fractions exactly as ProbeSolver::injectIBFrac computes them"""
    c = CASES[name]
    nd, nb, n = tb["ndim"], tb["nb"], tb["num_blocks"]
    lo = tb["block_lo"].reshape(n, 3)
    dx = tb["block_len"].reshape(n, 3).copy()
    dx[:, :nd] = dx[:, :nd] / nb
    vol = np.zeros((n,) + (nb,) * nd)
    areas = []
    # cell centres, [k][j][i] order
    grids = np.meshgrid(*[np.arange(nb)] * nd, indexing="ij")[::-1]  # i, j, (k)
    for b in range(n):
        pts = [lo[b, d] + (grids[d] + 0.5) * dx[b, d] for d in range(nd)]
        vol[b] = _frac(c, pts, dx[b, 0])
    for fd in range(nd):
        ext = [nb + (d == fd) for d in range(nd)]
        g = np.meshgrid(*[np.arange(e) for e in ext[::-1]], indexing="ij")[::-1]
        a = np.zeros((n,) + tuple(ext[::-1]))
        for b in range(n):
            pts = []
            for d in range(nd):
                x = lo[b, d] + (g[d] + 0.5) * dx[b, d]
                if d == fd:
                    x = x - 0.5 * dx[b, d]
                pts.append(x)
            a[b] = _frac(c, pts, dx[b, 0])
        areas.append(a.reshape(-1))
    return vol.reshape(-1), areas


