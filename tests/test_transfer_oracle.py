"""The CPU restatement of the regrid transfer (oracle/transfer_oracle.py)
against fixtures written by the reference itself (tests/golden/tf2, tf3:
FillPatch::restrictAll, one regrid, AmrTree::initNewBlockDataAfterRegrid
with centered-linear prolongation and a BC register using every math BC
kind), bit for bit; and the repository's tree mirror rebuilding the same
two trees, so that the GPU test can run the same transfer through the C ABI."""
import math

import numpy as np
import pytest

import sayakaamr_gb300 as sg
from golden_io import load, seeded
from oracle import transfer_oracle as to

# parameters of run_transfer_case() in oracle/ref_dump.cpp
TF = {
    "tf2": dict(ndim=2, nb=8, minlevel=2, maxlevel=5, seed=8802),
    "tf3": dict(ndim=3, nb=4, minlevel=2, maxlevel=4, seed=8803),
}
# the circle (sphere) of the initial refinement, then the one the regrid follows
OLD_RC, OLD_RR = (0.41, 0.33, 0.45), 0.26
NEW_RC, NEW_RR = (0.47, 0.71, 0.5), 0.56


def tables(g, prefix):
    n = int(g[prefix + "num_blocks"][0])
    tb = dict(ndim=int(g["ndim"][0]), nb=int(g["nb"][0]), num_blocks=n)
    for k in ("level", "neighbor", "child", "parent", "which_child", "node_type"):
        tb[k] = g[prefix + k]
    return tb


def bc_types(tb, bc_math):
    """math BC per block face: the register's kind on physical faces, -1 inside"""
    nbr = np.asarray(tb["neighbor"]).reshape(-1, 6)
    out = np.full(nbr.shape, -1, dtype=np.int32)
    for f in range(2 * tb["ndim"]):
        out[:, f] = np.where(nbr[:, f] <= to.PHYS_BNDRY, bc_math[f], -1)
    return out.reshape(-1)


def _straddles(rc, rr, lo, hi, nd):
    nin = nout = 0
    for corner in range(1 << nd):
        d2 = 0.0
        for d in range(nd):
            x = hi[d] if (corner >> d) & 1 else lo[d]
            d2 += (x - rc[d]) * (x - rc[d])
        if math.sqrt(d2) - rr < 0:
            nin += 1
        else:
            nout += 1
    return nin > 0 and nout > 0


def build_trees(name):
    """the old tree, then the tree after the moved circle's regrid, through
    the repository's tree mirror (same sequence as run_transfer_case)"""
    c = TF[name]
    nd = c["ndim"]
    t = sg.AmrTree(nd, c["nb"], c["minlevel"], c["maxlevel"], 20000)
    hi = (1, 1, 1) if nd == 3 else (1, 1, 0)
    t.init_uniform_root((1, 1, 1), (0, 0, 0), hi, (-20,) * 6, (0,) * 6)
    t.init_refine_to_min_level()
    for level in range(1, c["maxlevel"]):
        tb = t.tables()
        f = np.zeros(tb["num_blocks"], np.int32)
        for b in range(tb["num_blocks"]):
            if tb["level"][b] == level and tb["node_type"][b] == 1:
                if _straddles(OLD_RC, OLD_RR, tb["block_lo"][3 * b:3 * b + 3], tb["block_hi"][3 * b:3 * b + 3], nd):
                    f[b] = 1
        t.set_refine_flags(f)
        t.regrid()
    tb_old = t.tables()
    n = tb_old["num_blocks"]
    rf, cf = np.zeros(n, np.int32), np.zeros(n, np.int32)
    for b in range(n):
        if tb_old["node_type"][b] != 1:
            continue
        near = _straddles(NEW_RC, NEW_RR, tb_old["block_lo"][3 * b:3 * b + 3], tb_old["block_hi"][3 * b:3 * b + 3], nd)
        if near and tb_old["level"][b] < c["maxlevel"]:
            rf[b] = 1
        if not near and tb_old["level"][b] > c["minlevel"]:
            cf[b] = 1
    t.set_refine_flags(rf)
    t.set_coarsen_flags(cf)
    t.regrid()
    return tb_old, t.tables()


@pytest.mark.parametrize("name", ["tf2", "tf3"])
def test_transfer_restatement_matches_reference(name):
    g = load(name)
    tb_old, tb_new = tables(g, "old_"), tables(g, "new_")
    nc = tb_old["nb"] ** tb_old["ndim"]
    x_in = seeded(TF[name]["seed"], 1, tb_old["num_blocks"] * nc)
    # the averaged-down old field
    assert np.array_equal(to.average_down(tb_old, x_in).reshape(-1), g["old_x"])
    x_new, new = to.transfer_reference(tb_old, x_in, tb_new, bc_types(tb_new, g["bc_math"]), g["bc_val"])
    assert np.array_equal(new, g["new_child_flag"])
    assert new.sum() > 0
    assert np.array_equal(x_new, g["new_x"])
    # every math BC kind is on a face some new block's parent reads
    kinds = set()
    nbr = np.asarray(tb_new["neighbor"]).reshape(-1, 6)
    for b in np.nonzero(new)[0]:
        P = tb_new["parent"][b]
        kinds |= {int(g["bc_math"][f]) for f in range(2 * tb_new["ndim"]) if nbr[P, f] <= to.PHYS_BNDRY}
    assert kinds == {to.NEUMANN, to.DIRICHLET, to.SIMPLE_FILL}, kinds


def test_planted_mistake_is_caught():
    """a transfer that drops the Dirichlet lift (ghost = interior) differs"""
    g = load("tf2")
    tb_old, tb_new = tables(g, "old_"), tables(g, "new_")
    x_in = seeded(TF["tf2"]["seed"], 1, tb_old["num_blocks"] * 64)
    bct = bc_types(tb_new, g["bc_math"])
    bct[bct == to.DIRICHLET] = to.NEUMANN
    x_new, _ = to.transfer_reference(tb_old, x_in, tb_new, bct, g["bc_val"])
    assert not np.array_equal(x_new, g["new_x"])


@pytest.mark.parametrize("name", ["tf2", "tf3"])
def test_tree_mirror_rebuilds_the_transfer_trees(name):
    g = load(name)
    tb_old, tb_new = build_trees(name)
    for mine, prefix in ((tb_old, "old_"), (tb_new, "new_")):
        assert mine["num_blocks"] == int(g[prefix + "num_blocks"][0])
        for k in ("level", "neighbor", "child", "parent", "which_child", "node_type"):
            assert np.array_equal(np.asarray(mine[k]).reshape(-1), g[prefix + k]), (prefix, k)
