"""The oracle's restatement of the reference's tree (oracle/tree_oracle.py),
which builds the reference arm's workloads without the product library:
its tables against the reference's own dumps (every fixture case), and the
workloads it builds against those of the product's tree mirror."""
import os
import subprocess
import sys

import numpy as np
import pytest

import cases
from golden_io import load
from oracle.tree_oracle import TreeOracle

KEYS = ("level", "neighbor", "child", "parent", "which_child", "node_type", "node_type2", "block_lo", "block_hi",
        "block_len", "block_center")


def oracle_tree(name):
    """build_tree() of oracle/ref_dump.cpp on the oracle's tree"""
    c = cases.CASES[name]
    nd = c["ndim"]
    t = TreeOracle(nd, c["nb"], c["minlevel"], c["maxlevel"], 20000)
    t.init_uniform_root(c["nroot"], c["lo"], c["hi"], c["bc_code"], (0,) * 6)
    t.init_refine_to_min_level()
    for level in range(1, c["maxlevel"]):
        tb = t.tables()
        f = np.zeros(tb["num_blocks"], np.int32)
        for b in range(tb["num_blocks"]):
            if tb["level"][b] == level and tb["node_type"][b] == 1:
                if cases._straddles(c, tb["block_lo"][3 * b:3 * b + 3], tb["block_hi"][3 * b:3 * b + 3], nd):
                    f[b] = 1
        t.set_refine_flags(f)
        t.regrid()
    return t.tables()


@pytest.mark.parametrize("name", ["c1", "t2s", "t2b", "t3s", "t3n", "n2", "n3"])
def test_oracle_tree_matches_reference(name):
    g = load(name)
    tb = oracle_tree(name)
    assert tb["num_blocks"] == int(g["num_blocks"][0])
    for k in KEYS:
        assert np.array_equal(np.asarray(tb[k]).reshape(-1), g[k]), k


def test_workload_built_with_oracle_tree_is_identical():
    from sayakaamr_gb300 import workloads
    a = workloads.config2()
    workloads.use_tree_builder(TreeOracle)
    try:
        b = workloads.config2()
    finally:
        workloads.use_tree_builder(None)
    for k in KEYS:
        assert np.array_equal(np.asarray(a.tables[k]), np.asarray(b.tables[k])), k
    assert np.array_equal(a.rhs, b.rhs) and np.array_equal(a.vol, b.vol)
    for d in range(2):
        assert np.array_equal(a.area[d], b.area[d]) and np.array_equal(a.bface[d], b.bface[d])


def test_oracle_workload_loads_no_product_library():
    """a process that builds a workload with the oracle's tree never loads
    the product library"""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = ("import sys; sys.path.insert(0, %r)\n"
            "import sayakaamr_gb300 as sg\n"
            "from sayakaamr_gb300 import workloads\n"
            "from oracle.tree_oracle import TreeOracle\n"
            "workloads.use_tree_builder(TreeOracle)\n"
            "p = workloads.config1()\n"
            "maps = open('/proc/self/maps').read()\n"
            "assert sg._lib is None and 'libsayaka_gb300' not in maps\n"
            "print(p.leaf_cells)\n" % root)
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
