"""Over-relaxed red-black smoothing in the device V-cycle (params.relax_omega):
every fluid cell's update becomes u_old + omega (u_gs - u_old).  The device
solve's FP64 sweeps against the oracle's relaxed sweep (orc_smooth_relaxed,
the reference's Gauss-Seidel with the same relaxation), and whole solves
with the relaxed V-cycle in both precisions against the plain ones: another
fixed linear preconditioner, the same solution."""
import numpy as np
import pytest

import golden_io
from test_gpu_parity import block_slice, case_oracle, setup_solver

pytestmark = pytest.mark.gpu

FAST_RTOL = 1e-13  # FMA and precomputed factors against the reference's operation order, relaxed


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("variant", [-1, 0, 9])
@pytest.mark.parametrize("name", ["n2", "n3", "t2s", "t3s"])
def test_relaxed_sweeps_match_oracle(name, variant):
    g, t, tb, S = setup_solver(name)
    om = 1.25
    S.set_params(use_mg_precond=1, bottom=1, precision=0, relax_omega=om)
    n, nc = tb["num_blocks"], S.ncell
    corr = golden_io.seeded_input(name, "sm_corr0", n * nc)
    res = golden_io.seeded_input(name, "sm_resid", n * nc)
    O = case_oracle(name, tb, S)
    finest = int(tb["level"].max())
    for L in (finest, finest - 1):
        blocks, _ = t.tower(L)
        ref = block_slice(O.smooth(L, corr, res, omega=om), blocks, nc)
        plain = block_slice(O.smooth(L, corr, res), blocks, nc)
        assert rel(plain, ref) > 1e-3  # the relaxation changes the sweep
        fast = block_slice(S.device_smooth(L, corr, res, variant), blocks, nc)
        assert rel(fast, ref) < FAST_RTOL, (name, L, variant, rel(fast, ref))


def _solver(name):
    if name.startswith("config"):
        from sayakaamr_gb300 import workloads
        p = workloads.CONFIGS[name]()
        return workloads.make_solver(p)
    g, t, tb, S = setup_solver(name)
    S.set_rhs_compact(g["sv_rhs"])
    return S


@pytest.mark.parametrize("name", ["t2s", "t3s", "config2"])
def test_relaxed_solves_reach_the_same_solution(name):
    S = _solver(name)
    its = {}
    for precision in (0, 1):
        sols = []
        for om in (1.0, 1.15):
            S.set_zero_sol()
            S.set_params(tol_rel=1e-10, tol_abs=0.0, use_mg_precond=1, max_iter=500, precision=precision, bottom=1,
                         relax_omega=om)
            info = S.cg_solve()
            assert info["status"] == 0, (precision, om, info)
            assert info["rnorm"] < 1e-10 * info["rnorm0"]
            its[(precision, om)] = info["iterations"]
            sols.append(S.get_sol_compact())
        a, b = sols
        assert np.linalg.norm(a - b) <= 1e-7 * max(np.linalg.norm(b), 1e-300), precision
    print(name, "iterations (precision, omega):", its)
    S.set_params(relax_omega=1.0)


def test_relax_weight_outside_zero_two_is_refused():
    g, t, tb, S = setup_solver("t2s")
    for bad in (0.0, 2.0, -1.0, float("nan")):
        with pytest.raises(Exception):
            S.set_params(relax_omega=bad)
    S.set_params(relax_omega=1.0)
