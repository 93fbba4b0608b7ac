"""The batch workload (independent 2D problems solved as one forest) on the
GPU: the forest's block-diagonal bottom solve has one component per problem,
every problem's own residual under the reference-exact FP64 operator is
below 1e-8 (each right-hand side has |r0|_inf = 1), and the per-problem
solutions agree with solving each problem on its own."""
import numpy as np
import pytest

from sayakaamr_gb300 import workloads

pytestmark = pytest.mark.gpu

SOL_RTOL = 1e-6  # two solves to a 1e-8 residual, compared over fluid leaf cells


def solve(prob, precision):
    S = workloads.make_solver(prob)
    S.set_params(tol_rel=1e-8, tol_abs=0.0, use_mg_precond=1, max_iter=500, precision=precision, bottom=1)
    info = S.cg_solve()
    assert info["status"] == 0, info
    return S, info, S.get_sol_compact()


@pytest.mark.parametrize("precision", [0, 1])
def test_forest_matches_individual_problems(precision):
    rng = np.random.default_rng(44)
    parts = [workloads.batch_problem(rng, "b%d" % k) for k in range(5)]
    F = workloads.forest(parts, "batch")
    S, info, x = solve(F, precision)
    nc = F.ncell
    finest = int(F.tables["level"].max())
    r = S.residual(finest, x, F.rhs).reshape(-1, nc)
    xs = x.reshape(-1, nc)
    for k, (p, o) in enumerate(zip(parts, F.block_offsets)):
        blocks = slice(o, o + p.num_blocks)
        leaf = p.leaf
        fluid = (p.vol.reshape(-1, nc)[leaf] > 0)
        # this problem's residual on its own leaf cells
        assert np.abs(r[blocks][leaf][fluid]).max() < 1e-8, k
        _, _, xk = solve(p, precision)
        a = xs[blocks][leaf][fluid]
        b = xk.reshape(-1, nc)[leaf][fluid]
        assert np.linalg.norm(a - b) <= SOL_RTOL * np.linalg.norm(b), (k, np.linalg.norm(a - b) / np.linalg.norm(b))
