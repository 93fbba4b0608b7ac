"""The fixture problems of oracle/ref_dump.cpp (make_case), rebuilt through this
repository's own tree mirror so that tables, fields and results can be compared
with the reference's dumps."""
import math

import numpy as np

import sayakaamr_gb300 as sg

# parameters must match make_case() in oracle/ref_dump.cpp
CASES = {
    "c1": dict(ndim=2, nroot=(4, 4, 1), nb=8, minlevel=1, maxlevel=4, lo=(0, 0, 0), hi=(1, 1, 0),
               rc=(0.5, 0.5, 0), rr=0.25, bc_code=(-20,) * 6, bc_m20=sg.NEUMANN, bc_m21=sg.NEUMANN,
               ibc=(0, 0, 0), ibr=0.0, ib_binary=0, bamp=0.0, do_ops=0, tol_rel=1e-10),
    "t2s": dict(ndim=2, nroot=(2, 2, 1), nb=4, minlevel=2, maxlevel=5, lo=(0, 0, 0), hi=(1, 1, 0),
                rc=(0.43, 0.56, 0), rr=0.3, bc_code=(-20, -20, -21, -21, -20, -20), bc_m20=sg.NEUMANN,
                bc_m21=sg.DIRICHLET, ibc=(0.62, 0.40, 0), ibr=0.12, ib_binary=0, bamp=0.5, do_ops=1,
                tol_rel=1e-12),
    "t2b": dict(ndim=2, nroot=(2, 1, 1), nb=8, minlevel=2, maxlevel=4, lo=(0, 0, 0), hi=(2, 1, 0),
                rc=(1.1, 0.45, 0), rr=0.33, bc_code=(-20,) * 6, bc_m20=sg.NEUMANN, bc_m21=sg.NEUMANN,
                ibc=(0.7, 0.55, 0), ibr=0.15, ib_binary=1, bamp=0.25, do_ops=1, tol_rel=1e-11),
    "t3s": dict(ndim=3, nroot=(1, 1, 1), nb=4, minlevel=2, maxlevel=4, lo=(0, 0, 0), hi=(1, 1, 1),
                rc=(0.47, 0.52, 0.55), rr=0.21, bc_code=(-20, -20, -20, -20, -21, -21), bc_m20=sg.NEUMANN,
                bc_m21=sg.DIRICHLET, ibc=(0.6, 0.45, 0.5), ibr=0.14, ib_binary=0, bamp=0.5, do_ops=1,
                tol_rel=1e-11),
    "t3n": dict(ndim=3, nroot=(1, 1, 1), nb=4, minlevel=2, maxlevel=4, lo=(0, 0, 0), hi=(1, 1, 1),
                rc=(0.5, 0.5, 0.5), rr=0.2, bc_code=(-20,) * 6, bc_m20=sg.NEUMANN, bc_m21=sg.NEUMANN,
                ibc=(0.35, 0.6, 0.45), ibr=0.12, ib_binary=1, bamp=0.0, do_ops=1, tol_rel=1e-10),
    # the benchmark block size (16^d cells); fixtures hold digests of the
    # reference's results, and its solve ran with a converged bottom solve
    "n2": dict(ndim=2, nroot=(2, 2, 1), nb=16, minlevel=2, maxlevel=5, lo=(0, 0, 0), hi=(1, 1, 0),
               rc=(0.45, 0.52, 0), rr=0.3, bc_code=(-20, -20, -21, -21, -20, -20), bc_m20=sg.NEUMANN,
               bc_m21=sg.DIRICHLET, ibc=(0.58, 0.41, 0), ibr=0.11, ib_binary=0, bamp=0.5, do_ops=1,
               tol_rel=1e-10, bot_tol=(1e-10, 0.0)),
    "n3": dict(ndim=3, nroot=(1, 1, 1), nb=16, minlevel=2, maxlevel=4, lo=(0, 0, 0), hi=(1, 1, 1),
               rc=(0.47, 0.52, 0.55), rr=0.16, bc_code=(-20, -20, -20, -20, -20, -21), bc_m20=sg.NEUMANN,
               bc_m21=sg.DIRICHLET, ibc=(0.45, 0.5, 0.52), ibr=0.06, ib_binary=0, bamp=0.5, do_ops=1,
               tol_rel=1e-10, bot_tol=(1e-10, 0.0)),
}


def _straddles(c, lo, hi, ndim):
    nin = nout = 0
    for corner in range(1 << ndim):
        d2 = 0.0
        for d in range(ndim):
            x = hi[d] if (corner >> d) & 1 else lo[d]
            d2 += (x - c["rc"][d]) * (x - c["rc"][d])
        if math.sqrt(d2) - c["rr"] < 0:
            nin += 1
        else:
            nout += 1
    return nin > 0 and nout > 0


def build_tree(name, capacity=20000):
    """Same construction sequence as build_tree() in oracle/ref_dump.cpp."""
    c = CASES[name]
    nd = c["ndim"]
    t = sg.AmrTree(nd, c["nb"], c["minlevel"], c["maxlevel"], capacity)
    t.init_uniform_root(c["nroot"], c["lo"], c["hi"], c["bc_code"], (0,) * 6)
    t.init_refine_to_min_level()
    for level in range(1, c["maxlevel"]):
        tb = t.tables()
        n = tb["num_blocks"]
        flags = np.zeros(n, dtype=np.int32)
        for b in range(n):
            if tb["level"][b] == level and tb["node_type"][b] == 1:
                lo = tb["block_lo"][3 * b:3 * b + 3]
                hi = tb["block_hi"][3 * b:3 * b + 3]
                if _straddles(c, lo, hi, nd):
                    flags[b] = 1
        t.set_refine_flags(flags)
        t.regrid()
    return t


def bc_table(name, tables):
    """BlockBCRecord types per block face, as setBC resolves the case's register."""
    c = CASES[name]
    nb6 = tables["neighbor"].reshape(-1, 6)
    out = np.full(nb6.shape, -1, dtype=np.int32)
    for f in range(2 * c["ndim"]):
        out[nb6[:, f] == -20, f] = c["bc_m20"]
        out[nb6[:, f] == -21, f] = c["bc_m21"]
    return out.reshape(-1)


def all_neumann(name):
    c = CASES[name]
    return c["bc_m20"] == sg.NEUMANN and c["bc_m21"] == sg.NEUMANN
