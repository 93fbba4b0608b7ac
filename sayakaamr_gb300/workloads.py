"""Seeded synthetic MAC-Poisson problems with the shapes of the benchmark
configurations (there is no public data set; the reference's own drivers use
analytic geometry the same way, src/Test6.h:1045-1101).

Every problem is built through this package's tree mirror and returned as
compact all-block arrays:
    tables (dict)      tree tables (AmrTree.tables())
    bc     [n*6]       math BC per block face
    vol    [n*ncell]   IB volume fraction (leaf values)
    area   [ndim][n*nfb] IB area fractions (leaf values)
    bface  [ndim][n*nfb] face coefficient B = 1/rho (leaf values)
    rhs    [n*ncell]   right-hand side (leaf cells; the reference solves
                       -div(B grad p) = rhs, so rhs = -f)
"""
import math

import numpy as np

from . import AmrTree, DIRICHLET, NEUMANN


class Problem:
    def __init__(self, name, tree, tables, bc, vol, area, bface, rhs, params):
        self.name, self.tree, self.tables = name, tree, tables
        self.bc, self.vol, self.area, self.bface, self.rhs = bc, vol, area, bface, rhs
        self.params = params
        nd, nb = tables["ndim"], tables["nb"]
        self.ndim, self.nb, self.num_blocks = nd, nb, tables["num_blocks"]
        self.ncell = nb ** nd
        self.nfb = (nb + 1) * nb ** (nd - 1)
        self.leaf = np.nonzero(tables["node_type"] == 1)[0]
        self.leaf_cells = len(self.leaf) * self.ncell

    def describe(self):
        lv = self.tables["level"]
        return dict(blocks=int(self.num_blocks), leaf_blocks=int(len(self.leaf)), leaf_cells=int(self.leaf_cells),
                    levels=int(lv.max()), nb=int(self.nb), ndim=int(self.ndim))


def _block_geom(tb):
    n, nd, nb = tb["num_blocks"], tb["ndim"], tb["nb"]
    lo = tb["block_lo"].reshape(n, 3)[:, :nd]
    dx = tb["block_len"].reshape(n, 3)[:, :nd] / nb
    return lo, dx


def cell_centres(tb):
    """[n, nb^nd, nd] cell-centre coordinates ([k][j][i] cell order)."""
    n, nd, nb = tb["num_blocks"], tb["ndim"], tb["nb"]
    lo, dx = _block_geom(tb)
    g = np.meshgrid(*[np.arange(nb)] * nd, indexing="ij")[::-1]  # i, j, (k)
    idx = np.stack([a.reshape(-1) for a in g], axis=1)  # [ncell, nd]
    return lo[:, None, :] + (idx[None, :, :] + 0.5) * dx[:, None, :]


def face_centres(tb, fd):
    n, nd, nb = tb["num_blocks"], tb["ndim"], tb["nb"]
    lo, dx = _block_geom(tb)
    ext = [nb + (d == fd) for d in range(nd)]
    g = np.meshgrid(*[np.arange(e) for e in ext[::-1]], indexing="ij")[::-1]
    idx = np.stack([a.reshape(-1) for a in g], axis=1).astype(np.float64) + 0.5
    idx[:, fd] -= 0.5
    return lo[:, None, :] + idx[None, :, :] * dx[:, None, :]


# the class that builds the trees: this package's AmrTree, or any class with
# its interface (init_uniform_root, init_refine_to_min_level,
# set_refine_flags, regrid, tables) and the same tables
_tree_class = AmrTree


def use_tree_builder(cls=None):
    """build the workloads' trees with `cls` (None: this package's AmrTree)"""
    global _tree_class
    _tree_class = cls or AmrTree


def refine_tree(ndim, nb, nroot, lo, hi, min_level, max_level, need_refine, bc_code=(-20,) * 6, capacity=200000):
    """Root grid + static refinement to min_level + level-by-level refinement
    of the leaf blocks for which need_refine(block_lo, block_hi, level) is true."""
    t = _tree_class(ndim, nb, min_level, max_level, capacity)
    t.init_uniform_root(nroot, lo, hi, bc_code, (0,) * 6)
    t.init_refine_to_min_level()
    for level in range(1, max_level):
        tb = t.tables()
        n = tb["num_blocks"]
        blo = tb["block_lo"].reshape(n, 3)[:, :ndim]
        bhi = tb["block_hi"].reshape(n, 3)[:, :ndim]
        sel = (tb["level"] == level) & (tb["node_type"] == 1)
        flags = np.zeros(n, dtype=np.int32)
        idx = np.nonzero(sel)[0]
        if len(idx):
            flags[idx] = need_refine(blo[idx], bhi[idx], level).astype(np.int32)
        if not flags.any():
            continue
        t.set_refine_flags(flags)
        t.regrid()
    return t


def _straddle(sdf, blo, bhi, pad):
    """sdf changes sign (with a margin of `pad` block widths) over the block"""
    nd = blo.shape[1]
    corners = []
    for c in range(1 << nd):
        pts = np.where([(c >> d) & 1 for d in range(nd)], bhi, blo)
        corners.append(sdf(pts))
    corners = np.stack(corners, axis=1)
    h = np.max(bhi - blo, axis=1) * pad
    centre = sdf(0.5 * (blo + bhi))
    return (corners.min(axis=1) < h) & (corners.max(axis=1) > -h) | (np.abs(centre) < h)


def _smooth_heaviside(phi, w):
    return np.clip(0.5 - phi / w, 0.0, 1.0)


def gaussian_rhs(rng, pts, ndim, n_g=8, sigma=0.05):
    amp = rng.standard_normal(n_g)
    cen = rng.uniform(0.1, 0.9, size=(n_g, ndim))
    f = np.zeros(pts.shape[:-1])
    for g in range(n_g):
        r2 = np.sum((pts - cen[g]) ** 2, axis=-1)
        f += amp[g] * np.exp(-r2 / (2 * sigma * sigma))
    return f


def _close_isolated(vol, area, n, nb, nd):
    """a cell with fluid volume but every face closed has no equation (zero
    operator row, a zero divisor in the smoother): make it solid"""
    shp = (n,) + (nb,) * nd
    v = vol.reshape(shp).copy()
    closed = np.ones(shp, dtype=bool)
    for d in range(nd):
        fs = [nb] * nd
        fs[nd - 1 - d] += 1  # face arrays are [block][k][j][i], dimension d has nb+1 entries
        a = area[d].reshape((n,) + tuple(fs))
        lo = [slice(None)] * (nd + 1)
        hi = [slice(None)] * (nd + 1)
        lo[nd - d] = slice(0, nb)
        hi[nd - d] = slice(1, nb + 1)
        closed &= (a[tuple(lo)] == 0) & (a[tuple(hi)] == 0)
    v[closed] = 0.0
    return v.reshape(-1)


def _close_solid_faces(tb, vol, area):
    """close every face of a leaf block that borders a solid cell (vf = 0)
    on either side, across block and coarse/fine boundaries too: the
    reference's IB rule a_f = [both sides fluid] (src/SayakaMacIB.cpp:38-154)
    on top of the fractional area.  An open face into a solid cell would tie
    the fluid cell to the solid cell's value (held at 0) -- a Dirichlet sink
    that the coarse levels' averaged fractions cannot represent."""
    n, nd, nb = tb["num_blocks"], tb["ndim"], tb["nb"]
    leaf = tb["node_type"] == 1
    nbr = tb["neighbor"].reshape(n, 6)
    par = tb["parent"]
    lo, dx = _block_geom(tb)
    v = vol.reshape((n,) + (nb,) * nd)
    out = []
    for d in range(nd):
        ax = nd - d
        fs = [nb] * nd
        fs[nd - 1 - d] += 1
        a = area[d].reshape((n,) + tuple(fs)).copy()

        def sl(arr, i, axis=ax):
            idx = [slice(None)] * arr.ndim
            idx[axis] = i
            return tuple(idx)
        shut = np.zeros(a.shape, dtype=bool)
        shut[sl(shut, slice(1, nb))] = (v[sl(v, slice(0, nb - 1))] == 0) | (v[sl(v, slice(1, nb))] == 0)
        for side in (0, 1):
            own = v[sl(v, 0 if side == 0 else nb - 1)]  # [n, transverse]
            across = np.ones_like(own)
            fc = 2 * d + side
            B = nbr[:, fc]
            same = (B >= 0) & leaf
            same &= np.where(B >= 0, leaf[np.maximum(B, 0)], False)
            if same.any():
                across[same] = v[B[same]][sl(v[B[same]], nb - 1 if side == 0 else 0)]
            cf = leaf & (B < 0) & (B > -20) & (par >= 0)
            for b in np.nonzero(cf)[0]:
                P = nbr[par[b], fc]
                if P < 0 or not leaf[P]:
                    continue
                # the coarse cell across each fine face: the point half a fine
                # cell beyond the face, located in the coarse block
                tr = [q for q in range(nd) if q != d]
                grids = np.meshgrid(*[np.arange(nb)] * (nd - 1), indexing="ij")[::-1]
                pts = np.zeros(grids[0].shape + (nd,)) if nd > 1 else np.zeros((1, nd))
                for gi, q in enumerate(tr):
                    pts[..., q] = lo[b, q] + (grids[gi] + 0.5) * dx[b, q]
                pts[..., d] = lo[b, d] + (0 if side == 0 else nb) * dx[b, d] + (-0.5 if side == 0 else 0.5) * dx[b, d]
                ci = np.clip(np.floor((pts - lo[P]) / dx[P]).astype(int), 0, nb - 1)
                flat = ci[..., 0] + nb * ci[..., 1] + (nb * nb * ci[..., 2] if nd == 3 else 0)
                across[b] = vol.reshape(n, -1)[P][flat]
            shut[sl(shut, 0 if side == 0 else nb)] |= (own == 0) | (across == 0)
        a[shut & leaf.reshape((n,) + (1,) * nd)] = 0.0
        out.append(a.reshape(-1))
    return out


# cut cells and faces below this fraction are solid: a sliver with volume
# fraction 1e-5 scales its operator row by 1e5 and makes the residual there
# ill-conditioned (rounding differences amplified by 1/(dv vf))
MIN_FRACTION = 1e-3


def _finish(name, t, tb, vol, area, bface, f, neumann, params, dirichlet_faces=()):
    n, nd = tb["num_blocks"], tb["ndim"]
    ncell = tb["nb"] ** nd
    vol = np.asarray(vol, dtype=np.float64).reshape(-1)
    vol = np.where(vol < MIN_FRACTION, 0.0, vol)
    area = [np.where(np.asarray(a) < MIN_FRACTION, 0.0, np.asarray(a, dtype=np.float64)) for a in area]
    for _ in range(4):
        area = _close_solid_faces(tb, vol, [a.reshape(-1) for a in area])
        v2 = _close_isolated(vol, area, n, tb["nb"], nd)
        if np.array_equal(v2, vol):
            break
        vol = v2
    leaf = tb["node_type"] == 1
    lens = tb["block_len"].reshape(n, 3)[:, :nd] / tb["nb"]
    dv = np.prod(lens, axis=1)
    vol2 = vol.reshape(n, ncell)
    f = f.reshape(n, ncell) * leaf[:, None]
    if neumann:
        w = (dv[:, None] * vol2) * leaf[:, None]
        m = np.sum(f * w) / np.sum(w)
        f = np.where(leaf[:, None], f - m, 0.0)
    bc = np.full((n, 6), -1, dtype=np.int32)
    nbr = tb["neighbor"].reshape(n, 6)
    for fc in range(2 * nd):
        bc[nbr[:, fc] <= -20, fc] = DIRICHLET if fc in dirichlet_faces else NEUMANN
    return Problem(name, t, tb, bc.reshape(-1), vol.reshape(-1), [a.reshape(-1) for a in area],
                   [b.reshape(-1) for b in bface], (-f).reshape(-1), params)


def config1(seed=20251):
    """2D unit square, 4x4 roots of 8x8, levels 1..4 refined around the circle
    r=0.25 at the centre; beta=1, Neumann walls, 8 Gaussians, tol 1e-10."""
    def sdf(p):
        return np.sqrt(np.sum((p - 0.5) ** 2, axis=-1)) - 0.25

    t = refine_tree(2, 8, (4, 4, 1), (0, 0, 0), (1, 1, 0), 1, 4,
                    lambda lo, hi, l: _corner_straddle(sdf, lo, hi))
    tb = t.tables()
    n, ncell, nfb = tb["num_blocks"], 64, 72
    rng = np.random.default_rng(seed)
    f = gaussian_rhs(rng, cell_centres(tb), 2)
    ones_c = np.ones(n * ncell)
    ones_f = [np.ones(n * nfb) for _ in range(2)]
    return _finish("config1", t, tb, ones_c, ones_f, [np.ones(n * nfb) for _ in range(2)], f, True,
                   dict(tol_rel=1e-10))


def _corner_straddle(sdf, blo, bhi):
    nd = blo.shape[1]
    nin = np.zeros(len(blo), dtype=int)
    for c in range(1 << nd):
        pts = np.where([(c >> d) & 1 for d in range(nd)], bhi, blo)
        nin += sdf(pts) < 0
    return (nin > 0) & (nin < (1 << nd))


def config2(seed=2, nb=16, max_level=6, roots=2):
    """2D, 16x16 blocks, 6 levels (~1.3k leaf blocks); two-phase B = 1/rho with
    rho 1 | 1000 across a seeded ellipse smoothed over 2 cells; solid disk IB
    with fractional volume/area fractions from its signed distance; Neumann
    side and bottom walls, p = 0 (Dirichlet) outflow on the top wall; seeded
    zero-mean 8-Gaussian right-hand side."""
    rng = np.random.default_rng(seed)
    ec = rng.uniform(0.35, 0.65, 2)
    ea, eb = rng.uniform(0.24, 0.30), rng.uniform(0.14, 0.18)
    th = rng.uniform(0, math.pi)
    dc = rng.uniform(0.25, 0.75, 2)
    dr = rng.uniform(0.06, 0.09)
    ct, st = math.cos(th), math.sin(th)

    def ellipse(p):
        x = p[..., 0] - ec[0]
        y = p[..., 1] - ec[1]
        u = (x * ct + y * st) / ea
        v = (-x * st + y * ct) / eb
        # approximate signed distance (scaled by the minor axis)
        return (np.sqrt(u * u + v * v) - 1.0) * min(ea, eb)

    def disk(p):
        return np.sqrt(np.sum((p - dc) ** 2, axis=-1)) - dr

    def need(lo, hi, level):
        return _straddle(ellipse, lo, hi, 1.5) | _straddle(disk, lo, hi, 1.5)

    t = refine_tree(2, nb, (roots, roots, 1), (0, 0, 0), (1, 1, 0), 2, max_level, need)
    tb = t.tables()
    n = tb["num_blocks"]
    lo, dx = _block_geom(tb)
    pc = cell_centres(tb)
    h = dx[:, 0][:, None]
    vol = np.clip(disk(pc) / h + 0.5, 0.0, 1.0)
    area, bface = [], []
    for fd in range(2):
        pf = face_centres(tb, fd)
        area.append(np.clip(disk(pf) / h + 0.5, 0.0, 1.0))
        rho = 1.0 + 999.0 * _smooth_heaviside(ellipse(pf), 2.0 * h)
        bface.append(1.0 / rho)
    f = gaussian_rhs(rng, pc, 2)
    return _finish("config2", t, tb, vol, area, bface, f, True, dict(tol_rel=1e-8), dirichlet_faces=(3,))


def config3(seed=3, nb=16, max_level=5, band=3.0):
    """3D, 16^3 blocks, 5 levels refined on the sphere r=0.2 (a band of 3
    block widths: 3872 leaf blocks, 15.9M cells), IB solid sphere r=0.08
    (binary mask), B ratio 100 across a seeded blob, p=0 on the top wall.
    A narrower band (in block widths) gives a smaller tree of the same shape."""
    rng = np.random.default_rng(seed)
    bc_ = rng.uniform(0.35, 0.65, 3)
    br = rng.uniform(0.12, 0.18)
    sc = np.array([0.5, 0.5, 0.5])

    def sphere(p):
        return np.sqrt(np.sum((p - sc) ** 2, axis=-1)) - 0.2

    def blob(p):
        r = np.sqrt(np.sum((p - bc_) ** 2, axis=-1))
        return r - br

    def need(lo, hi, level):
        return _straddle(sphere, lo, hi, band)

    t = refine_tree(3, nb, (1, 1, 1), (0, 0, 0), (1, 1, 1), 2, max_level, need)
    tb = t.tables()
    lo, dx = _block_geom(tb)
    pc = cell_centres(tb)
    h = dx[:, 0][:, None]
    solid = lambda p: np.sqrt(np.sum((p - sc) ** 2, axis=-1)) - 0.08  # noqa: E731
    vol = (solid(pc) > 0).astype(np.float64)
    area, bface = [], []
    for fd in range(3):
        pf = face_centres(tb, fd)
        area.append((solid(pf) > 0).astype(np.float64))
        rho = 1.0 + 99.0 * _smooth_heaviside(blob(pf), 2.0 * h)
        bface.append(1.0 / rho)
    f = gaussian_rhs(rng, pc, 3, sigma=0.08)
    return _finish("config3", t, tb, vol, area, bface, f, True, dict(tol_rel=1e-8), dirichlet_faces=(5,))


def _ellipse_sdf(c, a, b, th):
    ct, st = math.cos(th), math.sin(th)

    def sdf(p):
        x = p[..., 0] - c[0]
        y = p[..., 1] - c[1]
        u = (x * ct + y * st) / a
        v = (-x * st + y * ct) / b
        return (np.sqrt(u * u + v * v) - 1.0) * min(a, b)
    return sdf


def batch_problem(rng, name, nb=16, max_leaves=1024):
    """One problem of the batch workload: unit square, 8x8 blocks at level 4,
    refined (up to 7 levels) around 1-4 seeded ellipse IB solids (fractional
    fractions) and a seeded density ellipse (rho ratio 10-1000, smoothed over
    2 cells); Neumann walls with p = 0 on the top wall; 8-Gaussian zero-mean
    right-hand side scaled to |rhs|_inf = 1 over the fluid cells."""
    solids = []
    for _ in range(int(rng.integers(1, 5))):
        a = rng.uniform(0.04, 0.10)
        solids.append(_ellipse_sdf(rng.uniform(0.2, 0.8, 2), a, a * rng.uniform(0.4, 1.0), rng.uniform(0, math.pi)))
    da = rng.uniform(0.12, 0.22)
    dens = _ellipse_sdf(rng.uniform(0.3, 0.7, 2), da, da * rng.uniform(0.5, 1.0), rng.uniform(0, math.pi))
    ratio = 10.0 ** rng.uniform(1.0, 3.0)
    max_level = int(rng.integers(5, 8))

    def need(lo, hi, level):
        m = _straddle(dens, lo, hi, 1.0)
        for sd in solids:
            m = m | _straddle(sd, lo, hi, 1.0)
        return m

    while True:
        t = refine_tree(2, nb, (1, 1, 1), (0, 0, 0), (1, 1, 0), 4, max_level, need, capacity=8000)
        tb = t.tables()
        if (tb["node_type"] == 1).sum() <= max_leaves or max_level <= 5:
            break
        max_level -= 1
    lo, dx = _block_geom(tb)
    pc = cell_centres(tb)
    h = dx[:, 0][:, None]

    def frac(p):
        v = np.ones(p.shape[:-1])
        for sd in solids:
            v = np.minimum(v, np.clip(sd(p) / h + 0.5, 0.0, 1.0))
        return v
    vol = frac(pc)
    area, bface = [], []
    for fd in range(2):
        pf = face_centres(tb, fd)
        area.append(frac(pf))
        bface.append(1.0 / (1.0 + (ratio - 1.0) * _smooth_heaviside(dens(pf), 2.0 * h)))
    f = gaussian_rhs(rng, pc, 2)
    prob = _finish(name, t, tb, vol, area, bface, f, True, dict(tol_rel=1e-8), dirichlet_faces=(3,))
    fluid = prob.vol > 0
    m = np.abs(prob.rhs[fluid]).max()
    prob.rhs = prob.rhs / (m if m > 0 else 1.0)
    return prob


def forest(problems, name):
    """Independent problems as one forest: their block tables concatenated
    with block-id offsets (neighbour, child and parent links stay inside each
    problem; physical-boundary codes are kept), fields concatenated.  One
    solve of the forest is one block-diagonal system: with every right-hand
    side scaled to |r0|_inf = 1, the joint criterion |r|_inf < 1e-8 holds for
    every problem."""
    tbs = [p.tables for p in problems]
    off = np.cumsum([0] + [t["num_blocks"] for t in tbs[:-1]])
    cat = {}
    for key in ("level", "which_child", "node_type", "block_len", "block_lo", "block_hi", "block_center"):
        cat[key] = np.concatenate([t[key] for t in tbs])
    for key in ("neighbor", "child", "parent"):
        cat[key] = np.concatenate([np.where(t[key] >= 0, t[key] + o, t[key]) for t, o in zip(tbs, off)]).astype(
            np.int32)
    cat["node_type2"] = np.concatenate([t["node_type2"] for t in tbs])
    t0 = tbs[0]
    cat.update(ndim=t0["ndim"], nb=t0["nb"], num_blocks=int(sum(t["num_blocks"] for t in tbs)),
               min_level=int(min(t["min_level"] for t in tbs)), max_level=int(max(t["max_level"] for t in tbs)))
    nd = t0["ndim"]
    prob = Problem(name, None, cat, np.concatenate([p.bc for p in problems]),
                   np.concatenate([p.vol for p in problems]),
                   [np.concatenate([p.area[d] for p in problems]) for d in range(nd)],
                   [np.concatenate([p.bface[d] for p in problems]) for d in range(nd)],
                   np.concatenate([p.rhs for p in problems]), dict(tol_rel=1e-8))
    prob.block_offsets = off
    prob.parts = problems
    return prob


def config4(seed=4, n_problems=256, nb=16):
    """Batch of independent 2D problems of uneven size (64-1024 leaf blocks
    of 16x16 cells), each with 1-4 seeded ellipse IB solids and rho ratio
    10-1000, solved together as one forest."""
    rng = np.random.default_rng(seed)
    return forest([batch_problem(rng, "config4_%d" % k, nb) for k in range(n_problems)], "config4")


# ---- elbow pipe with a moving sphere (3D, 8^3 blocks, regrid every few solves)
ELBOW_C = np.array([0.15, 0.15, 0.5])
ELBOW_R, ELBOW_TUBE, SPHERE_R = 0.3, 0.1, 0.04


def _seg_dist(p, a, b):
    ab = b - a
    t = np.clip(np.sum((p - a) * ab, axis=-1) / np.dot(ab, ab), 0.0, 1.0)
    return np.linalg.norm(p - (a + t[..., None] * ab), axis=-1)


def elbow_dist(p):
    """distance to the centreline of a 90-degree elbow in the plane z = 0.5:
    inlet leg along y from y = 0, quarter arc of radius 0.3 about (0.15,
    0.15), outlet leg along x to x = 0"""
    c, R = ELBOW_C, ELBOW_R
    x, y, z = p[..., 0] - c[0], p[..., 1] - c[1], p[..., 2] - c[2]
    ang = np.arctan2(y, x)
    d = np.where((ang >= 0) & (ang <= 0.5 * math.pi), np.sqrt((np.hypot(x, y) - R) ** 2 + z * z), np.inf)
    d = np.minimum(d, _seg_dist(p, np.array([c[0] + R, 0.0, c[2]]), np.array([c[0] + R, c[1], c[2]])))
    return np.minimum(d, _seg_dist(p, np.array([c[0], c[1] + R, c[2]]), np.array([0.0, c[1] + R, c[2]])))


def elbow_point(s):
    """centreline point at arc length fraction s in [0, 1] from the inlet"""
    c, R = ELBOW_C, ELBOW_R
    l1, la, l2 = c[1], 0.5 * math.pi * R, c[0]
    t = s * (l1 + la + l2)
    if t <= l1:
        return np.array([c[0] + R, t, c[2]])
    if t <= l1 + la:
        a = (t - l1) / R
        return np.array([c[0] + R * math.cos(a), c[1] + R * math.sin(a), c[2]])
    return np.array([c[0] - (t - l1 - la), c[1] + R, c[2]])


def elbow_target_level(blo, bhi, sc, max_level=7):
    """refinement target per block: max_level within 0.04 of the tube wall's
    outside (the tube and a band around it) and around the moving sphere,
    one level less up to 0.2 outside the tube, the far solid at level 2
    (about 30k blocks of 8^3 cells at 7 levels)"""
    centre = 0.5 * (blo + bhi)
    half = 0.5 * np.max(bhi - blo, axis=1) * math.sqrt(3.0)
    d = elbow_dist(centre) - half  # lower bound of the centreline distance over the block
    tgt = np.full(blo.shape[0], 2)
    tgt = np.where(d < ELBOW_TUBE + 0.2, max_level - 1, tgt)
    tgt = np.where(d < ELBOW_TUBE + 0.04, max_level, tgt)
    sph = lambda p: np.linalg.norm(p - sc, axis=-1) - SPHERE_R  # noqa: E731
    return np.where(_straddle(sph, blo, bhi, 1.0), max_level, tgt)


def elbow_tree(sc, nb=8, max_level=7):
    def need(lo, hi, level):
        return elbow_target_level(lo, hi, sc, max_level) > level
    return refine_tree(3, nb, (1, 1, 1), (0, 0, 0), (1, 1, 1), 2, max_level, need, capacity=400000)


def elbow_regrid(t, sc, max_level=7):
    """refine / coarsen the leaves toward the new targets (max_level passes,
    as the reference's regrid driver does)"""
    for _ in range(max_level):
        tb = t.tables()
        n = tb["num_blocks"]
        blo = tb["block_lo"].reshape(n, 3)
        bhi = tb["block_hi"].reshape(n, 3)
        leaf = tb["node_type"] == 1
        tgt = elbow_target_level(blo, bhi, sc, max_level)
        ref = (leaf & (tb["level"] < tgt)).astype(np.int32)
        crs = (leaf & (tb["level"] > tgt)).astype(np.int32)
        if not ref.any() and not crs.any():
            break
        t.set_refine_flags(ref)
        t.set_coarsen_flags(crs)
        t.regrid()
    return t


def elbow_problem(t, sc, seed, name="config5"):
    """fractions, B and right-hand side of the elbow on tree t with the sphere
    at sc: fluid inside the tube and outside the sphere (fractional
    fractions), B = 1, p = 0 on the outlet face x = 0, Neumann elsewhere"""
    tb = t.tables()
    rng = np.random.default_rng(seed)
    lo, dx = _block_geom(tb)
    h = dx[:, 0][:, None]
    phi = lambda p: np.minimum(ELBOW_TUBE - elbow_dist(p), np.linalg.norm(p - sc, axis=-1) - SPHERE_R)  # noqa
    vol = np.clip(phi(cell_centres(tb)) / h + 0.5, 0.0, 1.0)
    area, bface = [], []
    for fd in range(3):
        pf = face_centres(tb, fd)
        area.append(np.clip(phi(pf) / h + 0.5, 0.0, 1.0))
        bface.append(np.ones(pf.shape[:2]))
    f = gaussian_rhs(rng, cell_centres(tb), 3, sigma=0.08)
    return _finish(name, t, tb, vol, area, bface, f, False, dict(tol_rel=1e-8), dirichlet_faces=(0,))


def config5_sequence(steps=100, regrid_every=5, max_level=7, seed=5):
    """the elbow sequence: the sphere moves along the centreline over `steps`
    pressure solves; the tree is regridded every `regrid_every` steps.
    Yields (step, regridded, problem)."""
    sc = elbow_point(0.1)
    t = elbow_tree(sc, max_level=max_level)
    for k in range(steps):
        sc = elbow_point(0.1 + 0.8 * k / max(1, steps - 1))
        regridded = k > 0 and k % regrid_every == 0
        if regridded:
            elbow_regrid(t, sc, max_level)
        yield k, regridded or k == 0, elbow_problem(t, sc, seed * 1000 + k)


def config5(max_level=7):
    """one pressure solve of the elbow sequence (the first step)"""
    return next(config5_sequence(steps=1, max_level=max_level))[2]


CONFIGS = {"config1": config1, "config2": config2, "config3": config3, "config4": config4, "config5": config5}


def make_solver(prob, **params):
    """A MacSolver set up with the problem's BCs, fractions, B and RHS."""
    from . import MacSolver
    S = MacSolver(prob.tables)
    S.set_bc(prob.bc)
    S.set_ib_frac_compact(prob.vol, prob.area)
    for d in range(prob.ndim):
        S.set_coef_b(d, prob.bface[d])
    S.set_rhs_compact(prob.rhs)
    S.set_zero_sol()
    if params:
        S.set_params(**params)
    return S
