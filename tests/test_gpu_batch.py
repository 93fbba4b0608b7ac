"""The batch workload (independent 2D problems solved as one forest) on the
GPU: the forest's block-diagonal bottom solve has one component per problem,
every problem's own residual under the reference-exact FP64 operator is
below 1e-8 (each right-hand side has |r0|_inf = 1), and the per-problem
solutions agree with solving each problem on its own.  With one BiCGSTAB
state per problem (the default) every problem stops at its own iteration
count, as the reference's one solve per tree does
(src/SayakaMacSolver.cpp:683-920)."""
import numpy as np
import pytest

from sayakaamr_gb300 import workloads

pytestmark = pytest.mark.gpu

SOL_RTOL = 1e-6  # two solves to a 1e-8 residual, compared over fluid leaf cells


def solve(prob, precision, per_problem=1):
    S = workloads.make_solver(prob)
    S.set_params(tol_rel=1e-8, tol_abs=0.0, use_mg_precond=1, max_iter=500, precision=precision, bottom=1,
                 per_problem=per_problem)
    info = S.cg_solve()
    assert info["status"] == 0, info
    return S, info, S.get_sol_compact()


@pytest.mark.parametrize("per_problem", [1, 0])
@pytest.mark.parametrize("precision", [0, 1])
def test_forest_matches_individual_problems(precision, per_problem):
    rng = np.random.default_rng(44)
    parts = [workloads.batch_problem(rng, "b%d" % k) for k in range(5)]
    F = workloads.forest(parts, "batch")
    S, info, x = solve(F, precision, per_problem)
    states = S.problem_states()
    assert (states is None) == (per_problem == 0)
    if per_problem:
        its, rel = states
        assert len(its) == len(parts)
        assert np.all(rel < 1e-8), rel
        assert info["iterations"] == its.max()
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
        _, ik, xk = solve(p, precision)
        if per_problem and int(p.tables["level"].max()) == finest:
            # its own stopping point: the same iterations as alone, up to the
            # rounding of differently ordered dot products.  (A problem
            # shallower than the forest is smoothed once more per extra tower
            # of the forest's V-cycle, so it may take fewer.)
            assert abs(int(its[k]) - ik["iterations"]) <= 1, (k, its[k], ik["iterations"])
        a = xs[blocks][leaf][fluid]
        b = xk.reshape(-1, nc)[leaf][fluid]
        assert np.linalg.norm(a - b) <= SOL_RTOL * np.linalg.norm(b), (k, np.linalg.norm(a - b) / np.linalg.norm(b))


def test_per_problem_states_take_fewer_iteration_blocks():
    """the same forest: with one state per problem no problem runs longer than
    with the shared state, and the total work (iterations times cells) falls"""
    rng = np.random.default_rng(45)
    parts = [workloads.batch_problem(rng, "c%d" % k) for k in range(8)]
    F = workloads.forest(parts, "batch")
    S, shared, _ = solve(F, 1, per_problem=0)
    S, own, _ = solve(F, 1, per_problem=1)
    its, rel = S.problem_states()
    cells = np.array([p.leaf_cells for p in parts])
    assert own["iterations"] <= shared["iterations"] + 1
    assert np.sum(its * cells) < shared["iterations"] * np.sum(cells), (its, shared["iterations"])
