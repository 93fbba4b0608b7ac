"""The solution carried across a regrid (sayaka_mac_init_from), on the GPU
through the C ABI, against a numpy restatement bit for bit: blocks matched by
root and child path are copied, refined blocks take injection from their
nearest old leaf ancestor (the reference's prolongBlock of a new child,
level by level: src/SayakaRegrid.cpp:987-1105), blocks that became leaves by
coarsening take the average of their old children, blocks over a deeper old
subtree start from zero.  The elbow sequence then warm-starts every solve
after a regrid from the previous tree's solution."""
import numpy as np
import pytest

import sayakaamr_gb300 as sg
from sayakaamr_gb300 import workloads

pytestmark = pytest.mark.gpu


def path_key(tb, b):
    path = []
    while tb["parent"][b] >= 0:
        path.append(int(tb["which_child"][b]))
        b = int(tb["parent"][b])
    return (b, tuple(reversed(path)))


def cell_ijk(nb, nd):
    c = np.arange(nb ** nd)
    return [c % nb, (c // nb) % nb if nd >= 2 else 0 * c, c // (nb * nb) if nd == 3 else 0 * c]


def encode(ijk, nb, nd):
    out = ijk[0] + nb * ijk[1]
    return out + nb * nb * ijk[2] if nd == 3 else out


def expected_transfer(tb_old, x_old, tb_new):
    nd, nb = int(tb_new["ndim"]), int(tb_new["nb"])
    ncell, half = nb ** nd, nb // 2
    x_old = x_old.reshape(-1, ncell)
    where = {path_key(tb_old, b): b for b in range(tb_old["num_blocks"])}
    old_leaf = tb_old["node_type"] == 1
    out = np.zeros((tb_new["num_blocks"], ncell))
    ijk = cell_ijk(nb, nd)
    kinds = [0, 0, 0, 0]
    for b in np.nonzero(tb_new["node_type"] == 1)[0]:
        root, path = path_key(tb_new, b)
        ob = where.get((root, path))
        if ob is not None and old_leaf[ob]:
            out[b] = x_old[ob]
            kinds[0] += 1
            continue
        if ob is None:
            # nearest old ancestor, then injection one level at a time
            for up in range(1, len(path) + 1):
                oa = where.get((root, path[:len(path) - up]))
                if oa is not None:
                    break
            if oa is not None and old_leaf[oa]:
                pc = [a.copy() for a in ijk]
                for digit in reversed(path[len(path) - up:]):
                    for q in range(nd):
                        pc[q] = ((digit >> q) & 1) * half + (pc[q] >> 1)
                out[b] = x_old[oa][encode(pc, nb, nd)]
                kinds[1] += 1
                continue
        if ob is not None:
            kids = tb_old["child"].reshape(-1, 8)[ob][:1 << nd]
            if np.all(kids >= 0) and np.all(old_leaf[kids]):
                sq = [(a >= half).astype(int) for a in ijk]
                cidx = sum(sq[q] << q for q in range(nd))
                fb = [2 * (ijk[q] - sq[q] * half) for q in range(nd)] + [0] * (3 - nd)
                acc = np.zeros(ncell)
                for kk in range(2 if nd == 3 else 1):
                    for jj in range(2):
                        for ii in range(2):
                            fi = [fb[0] + ii, fb[1] + jj, fb[2] + kk]
                            acc = acc + x_old[kids[cidx], encode(fi, nb, nd)]
                out[b] = acc / float(1 << nd)
                kinds[2] += 1
                continue
        kinds[3] += 1
    return out.reshape(-1), kinds


def test_transfer_across_multilevel_refine_and_coarsen():
    nb, nd = 8, 2
    t = sg.AmrTree(nd, nb, 2, 5, 4000)
    t.init_uniform_root((1, 1, 1), (0, 0, 0), (1, 1, 0), (-20,) * 6, (0,) * 6)
    t.init_refine_to_min_level()
    # level 3 under the first two level-2 blocks
    tb = t.tables()
    lv2 = np.nonzero((tb["level"] == 2) & (tb["node_type"] == 1))[0]
    f = np.zeros(tb["num_blocks"], np.int32)
    f[lv2[:2]] = 1
    t.set_refine_flags(f)
    t.regrid()
    tb_old = t.tables()
    rng = np.random.default_rng(21)
    S_old = sg.MacSolver(tb_old)
    x_old = rng.standard_normal(tb_old["num_blocks"] * nb ** nd)
    S_old.set_init_sol(x_old, ncomp=1, ngrow=0, comp=0)
    # coarsen the children of the first refined block, refine another level-2
    # leaf twice (two regrid passes)
    kids1 = tb_old["child"].reshape(-1, 8)[lv2[0]][:4]
    c = np.zeros(tb_old["num_blocks"], np.int32)
    c[kids1] = 1
    f = np.zeros(tb_old["num_blocks"], np.int32)
    f[lv2[3]] = 1
    t.set_refine_flags(f)
    t.set_coarsen_flags(c)
    t.regrid()
    tb1 = t.tables()
    f = np.zeros(tb1["num_blocks"], np.int32)
    f[np.nonzero((tb1["level"] == 3) & (tb1["node_type"] == 1))[0][-1]] = 1
    t.set_refine_flags(f)
    t.regrid()
    tb_new = t.tables()
    want, kinds = expected_transfer(tb_old, x_old, tb_new)
    assert kinds[0] > 0 and kinds[1] > 0 and kinds[2] > 0, kinds
    S_new = sg.MacSolver(tb_new)
    S_new.init_from(S_old)
    got = S_new.get_sol_compact()
    assert np.array_equal(got, want)


def test_elbow_warm_start_after_regrid():
    """the sequence's solve after each regrid starts from the previous tree's
    solution carried over; the carried field matches the restatement and the
    warm-started solve reaches the criterion"""
    S = tb_prev = None
    its = []
    for k, regridded, prob in workloads.config5_sequence(steps=5, regrid_every=2, max_level=5):
        if regridded:
            S_new = workloads.make_solver(prob)
            S_new.set_params(tol_rel=1e-8, tol_abs=0.0, use_mg_precond=1, max_iter=500, precision=1, bottom=1)
            if S is not None:
                x_prev = S.get_sol_compact()
                S_new.init_from(S)
                want, kinds = expected_transfer(tb_prev, x_prev, prob.tables)
                assert np.array_equal(S_new.get_sol_compact(), want), kinds
                assert kinds[0] > 0, kinds
            S, tb_prev = S_new, prob.tables
        else:
            S.set_ib_frac_compact(prob.vol, prob.area)
            S.set_rhs_compact(prob.rhs)
        info = S.cg_solve()
        assert info["status"] == 0, (k, info)
        assert info["rnorm"] < 1e-8 * info["rnorm0"]
        its.append((k, regridded, info["iterations"]))
    print("step, regridded, iterations:", its)
