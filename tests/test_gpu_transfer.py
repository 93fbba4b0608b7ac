"""The solution carried across a regrid, on the GPU through the C ABI.
sayaka_mac_init_new_block_data (the reference's initNewBlockDataAfterRegrid
with centered-linear prolongation, src/SayakaRegrid.cpp:987-1105) against the
reference's own outputs (tests/golden/tf2, tf3) and the pinned numpy
restatement (oracle/transfer_oracle.py) bit for bit; sayaka_mac_init_from
(injection) against its restatement: blocks matched by root and child path
are copied, refined blocks take injection from their nearest old leaf
ancestor, blocks that became leaves by coarsening take the average of their
old children, blocks over a deeper old subtree start from zero.  The elbow
sequence then warm-starts every solve after a regrid from the previous
tree's solution."""
import numpy as np
import pytest

import sayakaamr_gb300 as sg
from golden_io import load, seeded
from oracle import transfer_oracle as to
from sayakaamr_gb300 import workloads
from test_transfer_oracle import TF, bc_types, build_trees

pytestmark = pytest.mark.gpu


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
    want, kinds = to.transfer_injection(tb_old, x_old, tb_new)
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
                want, kinds = to.transfer_injection(tb_prev, x_prev, prob.tables)
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


@pytest.mark.parametrize("name", ["tf2", "tf3"])
def test_centered_linear_transfer_matches_reference(name):
    """the reference's regrid transfer (average-down, kept blocks, centered-
    linear new blocks with same-level and Dirichlet / Neumann / SimpleFill
    ghosts) through the C ABI, against the reference's dump"""
    g = load(name)
    tb_old, tb_new = build_trees(name)
    nc = tb_old["nb"] ** tb_old["ndim"]
    S_old = sg.MacSolver(tb_old)
    S_old.set_init_sol(seeded(TF[name]["seed"], 1, tb_old["num_blocks"] * nc), ncomp=1, ngrow=0, comp=0)
    S_new = sg.MacSolver(tb_new)
    S_new.set_bc(bc_types(tb_new, g["bc_math"]))
    S_new.init_from(S_old, prolong="centered_linear", bc_val=g["bc_val"])
    assert np.array_equal(S_new.get_sol_compact(), g["new_x"])


def test_centered_linear_transfer_across_several_regrids():
    """old and new trees several regrids apart (new blocks whose parents are
    new too): the CUDA transfer against the restatement"""
    nb, nd = 8, 2
    t = sg.AmrTree(nd, nb, 2, 5, 4000)
    t.init_uniform_root((1, 1, 1), (0, 0, 0), (1, 1, 0), (-20,) * 6, (0,) * 6)
    t.init_refine_to_min_level()
    tb = t.tables()
    lv2 = np.nonzero((tb["level"] == 2) & (tb["node_type"] == 1))[0]
    f = np.zeros(tb["num_blocks"], np.int32)
    f[lv2[:2]] = 1
    t.set_refine_flags(f)
    t.regrid()
    tb_old = t.tables()
    rng = np.random.default_rng(23)
    x_old = rng.standard_normal(tb_old["num_blocks"] * nb ** nd)
    S_old = sg.MacSolver(tb_old)
    S_old.set_init_sol(x_old, ncomp=1, ngrow=0, comp=0)
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
    bct = np.where(np.asarray(tb_new["neighbor"]).reshape(-1, 6) <= to.PHYS_BNDRY,
                   np.array([1, 2, 0, 1, 0, 0]), -1).astype(np.int32).reshape(-1)
    bc_val = np.array([0.5, -1.25, 0.0, 2.0, 0.0, 0.0])
    want, new = to.transfer_reference(tb_old, x_old, tb_new, bct, bc_val)
    assert new.sum() > 0
    # a new block whose parent is new as well
    par = np.asarray(tb_new["parent"])
    assert any(new[par[b]] for b in np.nonzero(new)[0])
    S_new = sg.MacSolver(tb_new)
    S_new.set_bc(bct)
    S_new.init_from(S_old, prolong="centered_linear", bc_val=bc_val)
    assert np.array_equal(S_new.get_sol_compact(), want)
