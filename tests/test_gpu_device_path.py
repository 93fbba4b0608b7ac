"""Device-resident solve path (device scalars, CUDA-graph WHILE loop, dense
FP64 bottom solve, FP64 or FP32 V-cycle) against the reference solutions and
the C oracle."""
import numpy as np
import pytest

import golden_io
from cases import CASES, build_tree
from test_gpu_parity import block_slice, reference_solution, setup_solver, solution_error

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", sorted(CASES))
def test_device_solve_matches_reference(name, precision):
    g, t, tb, S = setup_solver(name)
    S.set_rhs_compact(g["sv_rhs"])
    S.set_zero_sol()
    S.set_params(tol_rel=1e-11, tol_abs=0.0, use_mg_precond=1, max_iter=500, precision=precision, bottom=1)
    info = S.cg_solve()
    assert info["status"] == 0, info
    blocks, _ = t.tower(tb["level"].max())
    sol = block_slice(S.get_sol_compact(), blocks, S.ncell)
    err = solution_error(name, tb, S, blocks, sol, reference_solution(name, g, t, tb, S))
    assert err < 1e-8, (name, precision, err, info)


def test_async_solve_and_info():
    g, t, tb, S = setup_solver("t2s")
    S.set_params(tol_rel=1e-10, tol_abs=0.0, use_mg_precond=1, max_iter=500, precision=1, bottom=1)
    S.prepare()
    S.set_rhs_compact(g["sv_rhs"])
    for _ in range(2):
        S.set_zero_sol()
        S.cg_solve_async()
        info = S.solve_info()
        assert info["status"] == 0 and info["iterations"] > 0, info
        assert info["rnorm"] < 1e-10 * info["rnorm0"]


def test_device_path_matches_oracle_on_workload():
    """config-1 workload: device-resident FP32/FP64 solves against the C
    oracle's converged solve of the same problem"""
    from oracle import pyoracle
    from sayakaamr_gb300 import workloads
    p = workloads.config1()
    S = workloads.make_solver(p)
    vf, af, bc = pyoracle.setup_coefficients(p.tables, p.bc, p.vol, p.area, p.bface)
    O = pyoracle.Oracle(p.tables, p.bc, vf, af, bc)
    ref, oinfo = O.cg_solve(p.rhs, pyoracle.params(tol_rel=1e-11, tol_abs=0.0, bot_tol_rel=1e-10, bot_tol_abs=0.0))
    assert oinfo["status"] == 0, oinfo
    leaf = p.leaf
    nc = p.ncell
    w = np.repeat(np.prod(p.tables["block_len"].reshape(-1, 3)[leaf, :2] / p.nb, axis=1), nc)
    for precision in (0, 1):
        S.set_zero_sol()
        S.set_params(tol_rel=1e-11, tol_abs=0.0, use_mg_precond=1, max_iter=500, precision=precision, bottom=1)
        info = S.cg_solve()
        assert info["status"] == 0, info
        a = S.get_sol_compact().reshape(-1, nc)[leaf].reshape(-1)
        r = ref.reshape(-1, nc)[leaf].reshape(-1)
        a = a - np.sum(a * w) / np.sum(w)
        r = r - np.sum(r * w) / np.sum(w)
        assert np.linalg.norm(a - r) / np.linalg.norm(r) < 1e-8, (precision, info)


@pytest.mark.parametrize("order", [0, 1])
@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", ["t2s", "t3s", "c1"])
def test_fused_vcycles_match_per_phase_launches(name, precision, order):
    """the one-launch cooperative V-cycle and the thread-block-cluster V-cycle
    run the same cell functions in the same phase order (either sublevel
    order): identical iterations and bit-identical solutions"""
    g, t, tb, S = setup_solver(name)
    S.set_rhs_compact(g["sv_rhs"])
    out = []
    # (vcycle_kernel, cluster_cells): per-phase, cooperative, cluster with a
    # mix of cluster runs and full launches, whole V-cycle in the cluster
    for vk, cc in ((0, 16384), (1, 16384), (2, 600), (2, 1 << 30)):
        S.set_zero_sol()
        S.set_params(tol_rel=1e-10, tol_abs=0.0, use_mg_precond=1, max_iter=500, precision=precision, bottom=1,
                     vcycle_kernel=vk, cluster_cells=cc, sublevel_order=order)
        info = S.cg_solve()
        assert info["status"] == 0, info
        out.append((info["iterations"], S.get_sol_compact()))
    for k in (1, 2, 3):
        assert out[0][0] == out[k][0], k
        assert np.array_equal(out[0][1], out[k][1]), k


@pytest.mark.parametrize("name", ["t2s", "t3n", "c1"])
def test_programmatic_dependent_launch_is_transparent(name):
    """PDL changes launch timing only: identical iterations and solution"""
    g, t, tb, S = setup_solver(name)
    S.set_rhs_compact(g["sv_rhs"])
    out = []
    for pdl in (0, 1):
        S.set_zero_sol()
        S.set_params(tol_rel=1e-10, tol_abs=0.0, use_mg_precond=1, max_iter=500, precision=1, bottom=1, pdl=pdl)
        info = S.cg_solve()
        assert info["status"] == 0, info
        out.append((info["iterations"], S.get_sol_compact()))
    assert out[0][0] == out[1][0]
    assert np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", ["t2s", "t3s", "c1"])
def test_smoother_variants_are_bit_identical(name, precision):
    """the autotuner's launch-bounds variants differ in register caps only:
    identical iterations and solutions, and the tuner reports its timings"""
    g, t, tb, S = setup_solver(name)
    S.set_rhs_compact(g["sv_rhs"])
    out = []
    for var in (-1, 0, 4, 5, 7, 8, 9, 10, 11, 12):
        S.set_zero_sol()
        S.set_params(tol_rel=1e-10, tol_abs=0.0, use_mg_precond=1, max_iter=500, precision=precision, bottom=1,
                     smooth_variant=var)
        info = S.cg_solve()
        assert info["status"] == 0, info
        out.append((info["iterations"], S.get_sol_compact()))
        if var == -1:
            v, us = S.tuned_smoother(precision)
            assert 0 <= v < 14 and all(u > 0 for u in us), (v, us)
    for k in range(1, len(out)):
        assert out[0][0] == out[k][0], k
        assert np.array_equal(out[0][1], out[k][1]), k


def test_nan_in_the_rhs_ends_as_breakdown_not_convergence():
    """a NaN anywhere (here planted in the right-hand side) reaches the max
    norms of the device solve and ends it as a breakdown"""
    g, t, tb, S = setup_solver("t2s")
    rhs = np.array(g["sv_rhs"], dtype=np.float64)
    leaf = np.nonzero(tb["node_type"] == 1)[0]
    rhs.reshape(tb["num_blocks"], -1)[leaf[0], 3] = np.nan
    S.set_rhs_compact(rhs)
    S.set_zero_sol()
    S.set_params(tol_rel=1e-10, tol_abs=0.0, use_mg_precond=1, max_iter=50, precision=1, bottom=1)
    info = S.cg_solve()
    assert info["status"] == 1, info


@pytest.mark.parametrize("name", ["config1", "config2"])
def test_sublevel_orders_both_converge(name):
    """the parity-grouped smoothing order (default) and the reference's
    per-sublevel order are both fixed linear preconditioners: both reach the
    criterion, within a few iterations of each other"""
    from sayakaamr_gb300 import workloads
    p = workloads.CONFIGS[name]()
    S = workloads.make_solver(p)
    its = []
    for order in (0, 1):
        S.set_zero_sol()
        S.set_params(tol_rel=1e-8, tol_abs=0.0, use_mg_precond=1, max_iter=500, precision=1, bottom=1,
                     sublevel_order=order)
        info = S.cg_solve()
        assert info["status"] == 0, (order, info)
        assert info["rnorm"] < 1e-8 * info["rnorm0"]
        its.append(info["iterations"])
    print(name, "iterations per-sublevel order %d, parity order %d" % tuple(its))
    assert abs(its[0] - its[1]) <= max(3, its[0] // 4), its


@pytest.mark.parametrize("name", ["config2", "config5"])
def test_bottom_level_above_one(name):
    """the dense bottom solve on a finer uniform level (level 2 on both
    workloads: asked for on config2, chosen automatically on the 3D elbow)
    replaces the V-cycle's coarsest levels; the solve reaches the
    criterion, in no more iterations than with the level-1 bottom"""
    from sayakaamr_gb300 import workloads
    p = workloads.CONFIGS[name]() if name != "config5" else workloads.config5(max_level=5)
    S = workloads.make_solver(p)
    its = {}
    for lvl in (1, 2 if name == "config2" else 0):
        S.set_zero_sol()
        S.set_params(tol_rel=1e-8, tol_abs=0.0, use_mg_precond=1, max_iter=500, precision=1, bottom=1,
                     bottom_level=lvl)
        info = S.cg_solve()
        assert info["status"] == 0, (lvl, info)
        assert info["rnorm"] < 1e-8 * info["rnorm0"]
        its[lvl] = (info["iterations"], S.bottom_level())
    k = 2 if name == "config2" else 0
    print(name, "bottom level 1: %d iterations; level %d: %d" % (its[1][0], its[k][1], its[k][0]))
    assert its[1][1] == 1 and its[k][1] == 2
    assert its[k][0] <= its[1][0]
    # the FP16 copy of the level-2 inverse (row scales): same criterion, at
    # most one iteration more
    S.set_zero_sol()
    S.set_params(bottom_level=2, bottom_half=1)
    info = S.cg_solve()
    assert info["status"] == 0 and info["rnorm"] < 1e-8 * info["rnorm0"], info
    assert info["iterations"] <= its[k][0] + 1, (info["iterations"], its)
    S.set_params(bottom_level=0, bottom_half=0)
    S.prepare()
    assert S.bottom_level() == (1 if name == "config2" else 2)
    # a solve after the rebuild uses only the new bottom's arrays, and the
    # handle's teardown frees each array once: no CUDA error is left pending
    S.set_zero_sol()
    info = S.cg_solve()
    assert info["status"] == 0 and info["rnorm"] < 1e-8 * info["rnorm0"], info
    import gc
    import sayakaamr_gb300 as sg
    del S
    gc.collect()
    assert sg.cuda_peek_error() == 0
