"""Constant-coefficient block records (params.uniform): blocks whose face
coefficients are constant per direction and whose cells are all fluid read
those coefficients (and the interior cells' operator and smoother factors)
from a per-block record instead of the face arrays.  The arithmetic is the
same operation for operation, so every device kernel and every device solve
must give bit-identical results with the records on and off."""
import numpy as np
import pytest

from test_gpu_parity import setup_solver

pytestmark = pytest.mark.gpu


def _workload(name):
    from sayakaamr_gb300 import workloads
    p = workloads.CONFIGS[name]()
    return p, workloads.make_solver(p)


@pytest.mark.parametrize("name", ["c1", "t3n", "t2s"])
def test_records_found_where_coefficients_are_constant(name):
    """c1 (B = 1, no IB) is constant everywhere; t3n has a binary IB and
    B = 1, so every block away from the solid qualifies; t2s has a smooth B
    field, so few blocks or none do"""
    g, t, tb, S = setup_solver(name)
    S.set_params(use_mg_precond=1, bottom=1)
    n = S.uniform_blocks()
    nb = tb["num_blocks"]
    vf = S.get_coef(2).reshape(nb, -1)
    # a block with a non-fluid cell is never a constant-coefficient block
    cut = int((vf != 1.0).any(1).sum())
    assert 0 <= n <= nb - cut
    if name == "c1":
        assert n == nb
    if name == "t3n":
        assert n > 0


@pytest.mark.parametrize("name", ["c1", "t3n", "t2s"])
def test_device_kernels_bit_identical_with_records(name):
    """the fast operator, every smoother launch variant and the block-hybrid
    pass: records on and off give the same bits"""
    g, t, tb, S = setup_solver(name)
    n = S.num_blocks * S.ncell
    rng = np.random.default_rng(11)
    phi = rng.standard_normal(n)
    rhs = rng.standard_normal(n)
    L = int(tb["level"].max())
    out = {}
    for uni in (0, 1):
        S.set_params(use_mg_precond=1, bottom=1, precision=0, uniform=uni)
        r = [S.device_apply(phi)]
        for var in (0, 4, 5, 7):
            r.append(S.device_smooth(L, phi, rhs, var))
        r.append(S.device_hybrid_pass(L, phi, rhs, 3))
        out[uni] = r
    for k, (a, b) in enumerate(zip(out[0], out[1])):
        assert np.array_equal(a, b), (name, k)


@pytest.mark.parametrize("smoother", [0, 1])
@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", ["c1", "t3n", "t2s", "config2"])
def test_device_solve_bit_identical_with_records(name, precision, smoother):
    """whole device solves (graph, FP32 or FP64 V-cycle, either smoother):
    identical iteration counts and bit-identical solutions"""
    if name.startswith("config"):
        p, S = _workload(name)
    else:
        g, t, tb, S = setup_solver(name)
        S.set_rhs_compact(g["sv_rhs"])
    res = []
    for uni in (0, 1):
        S.set_zero_sol()
        S.set_params(tol_rel=1e-10, tol_abs=0.0, use_mg_precond=1, max_iter=500, precision=precision, bottom=1,
                     smoother=smoother, uniform=uni)
        info = S.cg_solve()
        assert info["status"] == 0, info
        res.append((info["iterations"], S.get_sol_compact()))
    assert res[0][0] == res[1][0]
    assert np.array_equal(res[0][1], res[1][1])
    if name == "config2":
        assert S.uniform_blocks() > 0


@pytest.mark.parametrize("name", ["config2", "config4"])
def test_warp_per_block_sweep_is_bit_identical(name):
    """the FP32 sweep of 16x16 blocks with one warp per block (registers,
    shuffles, 16-byte loads; autotuner variants 11, 12, and 13 with every
    load issued before the first branch) against the one-thread-per-cell
    sweep (variant 3): identical iterations and solutions, on a
    workload with constant-coefficient blocks (its fast path) and cut or
    coarse/fine blocks (its cell-by-cell path), and on a small forest solved
    with one state per problem"""
    from sayakaamr_gb300 import workloads
    p = workloads.config4(n_problems=6) if name == "config4" else workloads.config2()
    S = workloads.make_solver(p)
    res = []
    for var in (3, 11, 12, 13):
        S.set_zero_sol()
        S.set_params(tol_rel=1e-10, tol_abs=0.0, use_mg_precond=1, max_iter=500, precision=1, bottom=1,
                     smooth_variant=var)
        info = S.cg_solve()
        assert info["status"] == 0, info
        res.append((info["iterations"], S.get_sol_compact()))
    for k in (1, 2, 3):
        assert res[0][0] == res[k][0], k
        assert np.array_equal(res[0][1], res[k][1]), k
    assert S.uniform_blocks() > 0


@pytest.mark.parametrize("name", ["config2", "config4", "c1"])
def test_warp_prolongation_is_bit_identical(name):
    """the prolongation fused with the first red sweep, one warp per block
    (prolong_form 1, 2D FP32 16x16 blocks) against one CTA per block with a
    shared-memory tile (prolong_form 0): identical iterations and solutions
    (c1 has 8x8 blocks, where form 1 falls back to form 0)"""
    from sayakaamr_gb300 import workloads
    if name == "c1":
        g, t, tb, S = setup_solver(name)
        S.set_rhs_compact(g["sv_rhs"])
    else:
        p = workloads.config4(n_problems=6) if name == "config4" else workloads.config2()
        S = workloads.make_solver(p)
    res = []
    for form in (0, 1):
        S.set_zero_sol()
        S.set_params(tol_rel=1e-10, tol_abs=0.0, use_mg_precond=1, max_iter=500, precision=1, bottom=1,
                     prolong_form=form, smooth_variant=12)
        info = S.cg_solve()
        assert info["status"] == 0, info
        res.append((info["iterations"], S.get_sol_compact()))
    assert res[0][0] == res[1][0]
    assert np.array_equal(res[0][1], res[1][1])
