"""Bit-exact tree / tower tables of the host tree mirror against the
reference's own AmrTree, regrid and MGLevelTower (golden fixtures written by
oracle/ref_dump.cpp from the reference library)."""
import numpy as np
import pytest

import golden_io
from cases import CASES, build_tree

FIXTURES = sorted(CASES)


@pytest.fixture(scope="module", params=FIXTURES)
def pair(request):
    name = request.param
    return name, golden_io.load(name), build_tree(name)


def test_block_tables(pair):
    name, g, t = pair
    tb = t.tables()
    assert tb["num_blocks"] == g["num_blocks"][0]
    n = tb["num_blocks"]
    for key in ("level", "neighbor", "child", "parent", "which_child", "node_type", "node_type2"):
        np.testing.assert_array_equal(tb[key], g[key], err_msg="%s %s" % (name, key))
    # geometry is compared bit for bit (same floating-point operations)
    for key in ("block_lo", "block_hi", "block_center"):
        assert np.array_equal(tb[key].view(np.int64), g[key].view(np.int64)), (name, key)
    assert np.array_equal(tb["block_len"].view(np.int64), g["block_len"].view(np.int64)), name
    assert n == len(g["level"])


def test_surrounding_blocks(pair):
    name, g, t = pair
    blocks, types, bcrefs = t.surrounding()
    np.testing.assert_array_equal(blocks, g["surr_blocks"], err_msg=name)
    np.testing.assert_array_equal(types, g["surr_types"], err_msg=name)
    np.testing.assert_array_equal(bcrefs, g["surr_bcrefs"], err_msg=name)


def test_level_lists(pair):
    name, g, t = pair
    tb = t.tables()
    for L in range(1, tb["max_level"] + 1):
        mine = np.nonzero(tb["level"] == L)[0].astype(np.int32)
        np.testing.assert_array_equal(mine, g["tree_level_%d" % L], err_msg="%s level %d" % (name, L))


def test_towers_and_face_registers(pair):
    name, g, t = pair
    tb = t.tables()
    for L in range(1, tb["max_level"] + 1):
        blocks, be = t.tower(L)
        np.testing.assert_array_equal(blocks, g["tower_%d_blocks" % L], err_msg="%s tower %d" % (name, L))
        gbe = g["tower_%d_begin_end" % L]
        if len(gbe):
            np.testing.assert_array_equal(be, gbe, err_msg="%s tower %d begin/end" % (name, L))
        else:
            assert len(blocks) == 0
        np.testing.assert_array_equal(t.face_regs(L), g["tower_%d_face_regs" % L],
                                      err_msg="%s tower %d face regs" % (name, L))


def test_regrid_with_coarsening_is_consistent():
    """Coarsen-and-refine cycles keep a 2:1 balanced, packed tree."""
    import sayakaamr_gb300 as sg
    t = build_tree("t2s")
    tb = t.tables()
    n = tb["num_blocks"]
    # coarsen every leaf at the finest level, then regrid
    finest = tb["level"].max()
    flags = ((tb["level"] == finest) & (tb["node_type"] == 1)).astype(np.int32)
    t.set_coarsen_flags(flags)
    t.regrid()
    tb2 = t.tables()
    assert tb2["num_blocks"] < n
    nb6 = tb2["neighbor"].reshape(-1, 6)
    lev = tb2["level"]
    par = tb2["parent"]
    ch = tb2["child"].reshape(-1, 8)
    for b in range(tb2["num_blocks"]):
        if par[b] >= 0:
            assert b in ch[par[b]]
        for f in range(4):
            nbr = nb6[b, f]
            if nbr >= 0:
                assert lev[nbr] == lev[b]
                assert nb6[nbr, f ^ 1] == b
            elif nbr == -1:
                # coarse neighbour: the parent's neighbour exists and is a leaf
                pn = nb6[par[b], f]
                assert pn >= 0 and tb2["node_type"][pn] == sg.NEUMANN + 1
