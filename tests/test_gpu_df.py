"""The double-float operator of the BiCGSTAB iteration (params.vcycle_out 1:
the FP32 V-cycle's output read in place, products and sums on the FP32 pipe
as hi + lo float pairs, rounded to FP64 once) against the FP64 operator of
the same FP32 input, and its effect on whole solves."""
import numpy as np
import pytest

from test_gpu_parity import setup_solver

pytestmark = pytest.mark.gpu

# about 48 significand bits: a few units of 2^-44 of the largest term
DF_RTOL = 1e-12


def _solver(name):
    if name.startswith("config"):
        from sayakaamr_gb300 import workloads
        p = workloads.CONFIGS[name]()
        return workloads.make_solver(p)
    g, t, tb, S = setup_solver(name)
    S.set_rhs_compact(g["sv_rhs"])
    return S


@pytest.mark.parametrize("name", ["c1", "t2s", "t3n", "t3s", "config2"])
def test_double_float_operator_matches_fp64(name):
    S = _solver(name)
    S.set_params(use_mg_precond=1, bottom=1, precision=1)
    rng = np.random.default_rng(3)
    # FP32-representable input, so both operators see the same values
    x = rng.standard_normal(S.num_blocks * S.ncell).astype(np.float32).astype(np.float64)
    y64 = S.device_apply(x)
    ydf = S.device_apply_f32(x)
    scale = np.abs(y64).max()
    assert scale > 0
    err = np.abs(ydf - y64).max()
    assert err <= DF_RTOL * scale, (err, scale)
    # the block records give the same bits in double-float too
    S.set_params(uniform=0)
    assert np.array_equal(S.device_apply_f32(x), ydf)


@pytest.mark.parametrize("name", ["t2s", "t3s", "config2", "config3"])
def test_solve_with_double_float_operator(name):
    """the FP32 V-cycle solve with the double-float operator (vcycle_out 1)
    and with the FP64 operator of the widened output (vcycle_out 2): both
    reach the criterion, within one iteration of each other, and their
    solutions agree to the tolerance"""
    S = _solver(name)
    res = []
    for vo in (1, 2):
        S.set_zero_sol()
        S.set_params(tol_rel=1e-10, tol_abs=0.0, use_mg_precond=1, max_iter=500, precision=1, bottom=1,
                     vcycle_out=vo)
        info = S.cg_solve()
        assert info["status"] == 0, (vo, info)
        assert info["rnorm"] < 1e-10 * info["rnorm0"]
        res.append((info["iterations"], S.get_sol_compact()))
    assert abs(res[0][0] - res[1][0]) <= 1, (res[0][0], res[1][0])
    a, b = res[0][1], res[1][1]
    assert np.linalg.norm(a - b) <= 1e-7 * max(np.linalg.norm(b), 1e-300)
