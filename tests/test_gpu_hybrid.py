"""The block-hybrid smoother of the device V-cycle (params.smoother = 1):
Gauss-Seidel inside a block from shared memory, Jacobi between blocks.  It
is a different preconditioner from the reference's red-black sweeps, so its
solves are checked against the reference's solutions (not iterates), and the
pass itself against the property that defines it."""
import numpy as np
import pytest

from test_gpu_parity import block_slice, reference_solution, setup_solver, solution_error

pytestmark = pytest.mark.gpu

BLOCK_RTOL = 1e-8   # converged block solves: 64 sweeps on 4^d-cell blocks reduce the residual by 1e-10 or more


@pytest.mark.parametrize("name", ["t2s", "t3s"])
def test_hybrid_pass_solves_each_block_with_frozen_neighbours(name):
    """with enough sweeps per block, one pass solves every block's equations
    exactly with the values outside the block taken from the input: the
    reference-arithmetic residual of (input outside, pass output inside)
    vanishes on the block"""
    g, t, tb, S = setup_solver(name)
    S.set_params(use_mg_precond=1, bottom=1, precision=0)
    n, nc = tb["num_blocks"], S.ncell
    rng = np.random.default_rng(5)
    phi = rng.standard_normal(n * nc)
    rhs = rng.standard_normal(n * nc)
    L = int(tb["level"].max())
    out = S.device_hybrid_pass(L, phi, rhs, 64)
    blocks, _ = t.tower(L)
    r_in = S.residual(L, phi, rhs)
    for b in blocks[:: max(1, len(blocks) // 24)]:
        sl = slice(int(b) * nc, (int(b) + 1) * nc)
        w = phi.copy()
        w[sl] = out[sl]
        r = S.residual(L, w, rhs)[sl]
        # (<=: an all-solid block has no equations, its residual is 0 before and after)
        assert np.abs(r).max() <= BLOCK_RTOL * np.abs(r_in[sl]).max(), (b, np.abs(r).max(), np.abs(r_in[sl]).max())
    # cells outside the tower keep their input values
    mask = np.ones(n, dtype=bool)
    mask[blocks] = False
    assert np.array_equal(out.reshape(n, nc)[mask], phi.reshape(n, nc)[mask])


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", ["n2", "n3", "t2s", "t3s", "c1"])
def test_hybrid_solve_matches_reference(name, precision):
    g, t, tb, S = setup_solver(name)
    S.set_rhs_compact(g["sv_rhs"])
    out = []
    for _ in range(2):
        S.set_zero_sol()
        S.set_params(tol_rel=1e-11, tol_abs=0.0, use_mg_precond=1, max_iter=500, precision=precision, bottom=1,
                     smoother=1, inner_sweeps=2, n_post_smooth=2)
        info = S.cg_solve()
        assert info["status"] == 0, info
        out.append((info["iterations"], S.get_sol_compact()))
    # a fixed linear map: the same iterations and bit-identical solutions
    assert out[0][0] == out[1][0]
    assert np.array_equal(out[0][1], out[1][1])
    blocks, _ = t.tower(tb["level"].max())
    sol = block_slice(out[0][1], blocks, S.ncell)
    err = solution_error(name, tb, S, blocks, sol, reference_solution(name, g, t, tb, S))
    assert err < 1e-8, (name, precision, err)
