"""Refine + coarsen cycles of a moving circle/sphere through the host tree
mirror, compared after every step with the reference's own AmrTree::regrid
(fixtures rg2 / rg3 from oracle/ref_dump.cpp::run_regrid_case).  Coarsening
repacks block ids, so this pins coarsenBlocks (src/SayakaRegrid.cpp:515-632)."""
import math

import numpy as np
import pytest

import golden_io
import sayakaamr_gb300 as sg


def straddles(rc, rr, lo, hi, nd):
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


@pytest.mark.parametrize("name,nd", [("rg2", 2), ("rg3", 3)])
def test_regrid_sequence(name, nd):
    g = golden_io.load(name)
    minl, maxl = 2, (4 if nd == 3 else 6)
    rr = 0.22
    rc = [0.35, 0.45, 0.5]
    t = sg.AmrTree(nd, 4, minl, maxl, 20000)
    hi = (1.5, 1.0, 1.0 if nd == 3 else 0.0)
    t.init_uniform_root((3, 2, 1), (0, 0, 0), hi, (-20,) * 6, (0,) * 6)
    t.init_refine_to_min_level()

    def flags(kind):
        tb = t.tables()
        n = tb["num_blocks"]
        ref = np.zeros(n, np.int32)
        crs = np.zeros(n, np.int32)
        for b in range(n):
            if tb["node_type"][b] != 1:
                continue
            near = straddles(rc, rr, tb["block_lo"][3 * b:3 * b + 3], tb["block_hi"][3 * b:3 * b + 3], nd)
            lv = tb["level"][b]
            if kind == "build":
                ref[b] = near
            else:
                ref[b] = near and lv < maxl
                crs[b] = (not near) and lv > minl
        return ref, crs

    for level in range(1, maxl):  # build_tree(): refine level by level
        tb = t.tables()
        ref, _ = flags("build")
        ref = ref * (tb["level"] == level)
        t.set_refine_flags(ref)
        t.regrid()
    for step in range(int(g["steps"][0])):
        rc[0] += 0.11
        rc[1] += 0.03 * (-1 if step % 2 else 1)
        for _ in range(maxl):
            ref, crs = flags("move")
            t.set_refine_flags(ref)
            t.set_coarsen_flags(crs)
            t.regrid()
        tb = t.tables()
        p = "step_%d_" % step
        for key in ("level", "neighbor", "child", "parent"):
            np.testing.assert_array_equal(tb[key], g[p + key], err_msg="%s %s" % (p, key))
        np.testing.assert_array_equal(t.surrounding()[0], g[p + "surr_blocks"], err_msg=p)
