"""The C-ABI library loads without a GPU and exports every function that
include/*.h declares; host-only entry points (the tree mirror, parameter
defaults, input validation) work without a GPU."""
import ctypes
import glob
import os
import re

import sayakaamr_gb300 as sg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(sayaka_[a-z0-9_]+)\s*\(", src):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(sg.LIB_PATH)
    names = declared_functions()
    assert len(names) > 40
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_abi():
    assert declared_functions() == set(sg.SIGNATURES), sorted(declared_functions() ^ set(sg.SIGNATURES))


def test_params_defaults_match_the_reference():
    lib = sg.load_library()
    p = sg.Params()
    lib.sayaka_params_default(ctypes.byref(p))
    # MacSolver constructor defaults (src/SayakaMacSolver.h:68-83)
    assert p.max_iter == 2000 and p.tol_rel == 1e-6 and p.tol_abs == 0.0
    assert p.n_post_smooth == 2 and p.use_mg_precond == 0
    assert p.bot_tol_rel == 1e-6 and p.bot_tol_abs == 1e-6 and p.bot_max_iter == 2000


def test_bad_inputs_are_rejected_without_a_gpu():
    lib = sg.load_library()
    h = ctypes.c_void_p()
    assert lib.sayaka_tree_create(4, 8, 1, 2, 10, ctypes.byref(h)) == sg.BAD_INPUT      # ndim 4
    assert lib.sayaka_tree_create(2, 7, 1, 2, 10, ctypes.byref(h)) == sg.BAD_INPUT      # odd nb
    assert lib.sayaka_tree_create(2, 8, 3, 2, 10, ctypes.byref(h)) == sg.BAD_INPUT      # min > max
    assert lib.sayaka_mac_create(None, ctypes.byref(h)) == sg.BAD_INPUT
    t = sg.TreeTables()
    t.ndim, t.nb, t.num_blocks, t.min_level, t.max_level = 2, 8, 0, 1, 1
    assert lib.sayaka_mac_create(ctypes.byref(t), ctypes.byref(h)) == sg.BAD_INPUT  # no blocks


def test_tree_capacity_overflow_is_an_error_not_an_exit():
    t = sg.AmrTree(2, 4, 1, 6, capacity=20)
    t.init_uniform_root((2, 2, 1), (0, 0, 0), (1, 1, 0), (-20,) * 6)
    t.init_refine_to_min_level()
    t.set_refine_flags([1] * t.num_blocks)
    t.regrid()          # 4 + 16 blocks: fits exactly
    t.set_refine_flags([1] * t.num_blocks)
    try:
        t.regrid()
    except sg.SayakaError:
        return
    raise AssertionError("capacity overflow not reported")
