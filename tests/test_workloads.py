"""The synthetic workloads' geometry (CPU): immersed-boundary fractions in
[0, 1], no face open between a fluid cell and a solid one -- inside a block,
across same-level block faces and across coarse/fine faces -- (the
reference's IB rule a_f = [both sides fluid], src/SayakaMacIB.cpp:38-154),
zero-mean right-hand sides on all-Neumann problems, and seeded
reproducibility.  An open face into a solid cell, whose value the solver
holds at zero, acts as a hidden Dirichlet sink that the coarse levels do not
see: the reference's V-cycle diverged on such a workload."""
import numpy as np
import pytest

from sayakaamr_gb300 import workloads as W


def open_faces_into_solid(prob):
    """count open faces with a solid cell on one side, over leaf blocks:
    inside blocks and across same-level neighbours"""
    tb = prob.tables
    n, nd, nb = prob.num_blocks, prob.ndim, prob.nb
    leaf = tb["node_type"] == 1
    nbr = tb["neighbor"].reshape(n, 6)
    v = prob.vol.reshape((n,) + (nb,) * nd)
    bad = 0
    for d in range(nd):
        ax = nd - d
        fs = [nb] * nd
        fs[nd - 1 - d] += 1
        a = prob.area[d].reshape((n,) + tuple(fs))

        def sl(arr, i):
            idx = [slice(None)] * arr.ndim
            idx[ax] = i
            return tuple(idx)
        inner = a[sl(a, slice(1, nb))]
        solid = (v[sl(v, slice(0, nb - 1))] == 0) | (v[sl(v, slice(1, nb))] == 0)
        bad += int(((inner > 0) & solid)[leaf].sum())
        for side in (0, 1):
            faces = a[sl(a, 0 if side == 0 else nb)]  # [n, transverse...]
            own = v[sl(v, 0 if side == 0 else nb - 1)]
            other = np.ones_like(own)
            B = nbr[:, 2 * d + side]
            same = leaf & (B >= 0)
            same &= np.where(B >= 0, leaf[np.maximum(B, 0)], False)
            other[same] = v[B[same]][sl(v[B[same]], nb - 1 if side == 0 else 0)]
            bad += int(((faces > 0) & ((own == 0) | (other == 0)))[leaf].sum())
    return bad


@pytest.mark.parametrize("name", ["config1", "config2"])
def test_ib_faces_consistent_with_cells(name):
    p = W.CONFIGS[name]()
    assert np.all((p.vol >= 0) & (p.vol <= 1))
    for a in p.area:
        assert np.all((a >= 0) & (a <= 1))
    assert open_faces_into_solid(p) == 0


def test_ib_faces_consistent_3d():
    p = W.config3(max_level=4)
    assert open_faces_into_solid(p) == 0


def test_coarse_fine_faces_consistent():
    """a fine face on a coarse/fine interface is closed when the coarse cell
    across it is solid"""
    p = W.config2()
    tb = p.tables
    n, nb = p.num_blocks, p.nb
    leaf = tb["node_type"] == 1
    nbr = tb["neighbor"].reshape(n, 6)
    par = tb["parent"]
    lo = tb["block_lo"].reshape(n, 3)[:, :2]
    dx = tb["block_len"].reshape(n, 3)[:, :2] / nb
    v = p.vol.reshape(n, -1)
    checked = 0
    for d in range(2):
        a = p.area[d].reshape((n,) + ((nb, nb + 1) if d == 0 else (nb + 1, nb)))
        for side in (0, 1):
            for b in np.nonzero(leaf & (nbr[:, 2 * d + side] < 0) & (nbr[:, 2 * d + side] > -20))[0]:
                P = nbr[par[b], 2 * d + side]
                if P < 0 or not leaf[P]:
                    continue
                q = 1 - d
                for m in range(nb):
                    pt = np.zeros(2)
                    pt[q] = lo[b, q] + (m + 0.5) * dx[b, q]
                    pt[d] = lo[b, d] + (0 if side == 0 else nb) * dx[b, d] + (-0.5 if side == 0 else 0.5) * dx[b, d]
                    ci = np.clip(np.floor((pt - lo[P]) / dx[P]).astype(int), 0, nb - 1)
                    coarse = v[P][ci[0] + nb * ci[1]]
                    face = a[b][m, 0 if side == 0 else nb] if d == 0 else a[b][0 if side == 0 else nb, m]
                    checked += 1
                    assert not (coarse == 0 and face > 0), (b, d, side, m)
    assert checked > 0


def test_neumann_rhs_has_zero_mean_and_seeds_repeat():
    p1, p2 = W.config1(), W.config1()
    assert np.array_equal(p1.rhs, p2.rhs)
    n, nc = p1.num_blocks, p1.ncell
    leaf = p1.tables["node_type"] == 1
    dv = np.prod(p1.tables["block_len"].reshape(n, 3)[:, :2] / p1.nb, axis=1)
    w = (dv[:, None] * p1.vol.reshape(n, nc)) * leaf[:, None]
    assert abs(np.sum(p1.rhs.reshape(n, nc) * w)) < 1e-12 * np.sum(np.abs(p1.rhs.reshape(n, nc)) * w)


def test_checker_finds_faces_left_open(monkeypatch):
    """without the face closing (the first version of the workloads) the
    checker finds open faces into solid cells on config2"""
    monkeypatch.setattr(W, "_close_solid_faces", lambda tb, vol, area: [a.reshape(-1) for a in area])
    p = W.config2()
    assert open_faces_into_solid(p) > 100


def test_forest_keeps_every_link_inside_its_problem():
    """the batch forest: block ids offset per problem, every neighbour / child
    / parent link stays inside its problem, physical-boundary codes (<= -20)
    and -1 kept, fields concatenated in problem order, each right-hand side
    scaled to |rhs|_inf = 1 over its fluid cells"""
    rng = np.random.default_rng(11)
    parts = [W.batch_problem(rng, "p%d" % k) for k in range(4)]
    f = W.forest(parts, "forest")
    tb = f.tables
    n = tb["num_blocks"]
    assert n == sum(p.num_blocks for p in parts)
    off = list(f.block_offsets) + [n]
    owner = np.zeros(n, dtype=int)
    for k in range(len(parts)):
        owner[off[k]:off[k + 1]] = k
    for key, width in (("neighbor", 6), ("child", 8), ("parent", 1)):
        links = tb[key].reshape(n, width)
        for k, p in enumerate(parts):
            mine = links[off[k]:off[k + 1]]
            orig = p.tables[key].reshape(-1, width)
            assert np.array_equal(mine[orig < 0], orig[orig < 0])  # -1 and boundary codes kept
            inside = mine[orig >= 0]
            assert np.all(owner[inside] == k)
            assert np.array_equal(inside - off[k], orig[orig >= 0])
    nc = f.ncell
    for k, p in enumerate(parts):
        assert np.array_equal(f.rhs[off[k] * nc:off[k + 1] * nc], p.rhs)
        assert np.array_equal(f.vol[off[k] * nc:off[k + 1] * nc], p.vol)
        fluid = p.vol > 0
        assert abs(np.abs(p.rhs[fluid]).max() - 1.0) < 1e-12
