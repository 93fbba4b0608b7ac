"""MacSolver::mg_solve and relax_solve on the GPU through the C ABI, against
the reference's own results (golden fixtures, a fixed number of iterations
each).  relax_solve is pure reference-arithmetic smoothing: bit for bit.
mg_solve's bottom BiCGSTAB sums its dot products in another order than the
reference: with the fixtures' bottom tolerances it agrees to MG_RTOL, and
against the bit-pinned oracle with a converged bottom (1e-13) to
MG_ORACLE_RTOL."""
import numpy as np
import pytest

import golden_io
from test_gpu_parity import block_slice, case_oracle, setup_solver

pytestmark = pytest.mark.gpu

MG_RTOL = 1e-3          # bottom stopped at the fixture's tolerance after differently rounded iterates
MG_ORACLE_RTOL = 1e-9   # converged bottoms: rounding only (the stand-alone iteration amplifies it per V-cycle)


@pytest.mark.parametrize("name", ["t2s", "t3s", "n2", "n3"])
def test_relax_solve_bit_exact(name):
    g, t, tb, S = setup_solver(name)
    S.set_rhs_compact(g["sv_rhs"])
    S.set_zero_sol()
    S.set_params(tol_rel=1e-30, tol_abs=0.0, max_iter=golden_io.RELAX_ITERS, precision=0, bottom=0)
    info = S.relax_solve()
    assert info["iterations"] == golden_io.RELAX_ITERS and info["status"] == 2, info
    blocks, _ = t.tower(tb["level"].max())
    assert golden_io.matches(block_slice(S.get_sol_compact(), blocks, S.ncell), g["rx_sol"]), name


@pytest.mark.parametrize("name", ["t2s", "t3s", "n2", "n3"])
def test_mg_solve_matches_reference(name):
    from oracle import pyoracle
    g, t, tb, S = setup_solver(name)
    blocks, _ = t.tower(tb["level"].max())
    bot = (float(g["sv_bot_tol_rel"][0]), float(g["sv_bot_tol_abs"][0]))
    O = case_oracle(name, tb, S)
    # the reference's parameters: its result, to the bottom tolerance's effect
    S.set_rhs_compact(g["sv_rhs"])
    S.set_zero_sol()
    S.set_params(tol_rel=1e-30, tol_abs=0.0, max_iter=golden_io.MG_ITERS, precision=0, bottom=0,
                 bot_tol_rel=bot[0], bot_tol_abs=bot[1])
    info = S.mg_solve()
    assert info["iterations"] == golden_io.MG_ITERS and info["status"] == 2, info
    ref = g["mg_sol"]
    if isinstance(ref, golden_io.Digest):
        ref, _ = O.mg_solve(g["sv_rhs"], pyoracle.params(max_iter=golden_io.MG_ITERS, tol_rel=1e-30, tol_abs=0.0,
                                                          bot_tol_rel=bot[0], bot_tol_abs=bot[1]))
        ref = block_slice(ref, blocks, S.ncell)
        assert g["mg_sol"].matches(ref), name
    mine = block_slice(S.get_sol_compact(), blocks, S.ncell)
    assert np.linalg.norm(mine - ref) <= MG_RTOL * np.linalg.norm(ref), (name, np.linalg.norm(mine - ref) /
                                                                            np.linalg.norm(ref))
    # converged bottoms on both sides
    S.set_zero_sol()
    S.set_params(bot_tol_rel=1e-13, bot_tol_abs=0.0)
    S.mg_solve()
    mine = block_slice(S.get_sol_compact(), blocks, S.ncell)
    orc, _ = O.mg_solve(g["sv_rhs"], pyoracle.params(max_iter=golden_io.MG_ITERS, tol_rel=1e-30, tol_abs=0.0,
                                                      bot_tol_rel=1e-13, bot_tol_abs=0.0))
    orc = block_slice(orc, blocks, S.ncell)
    assert np.linalg.norm(mine - orc) <= MG_ORACLE_RTOL * np.linalg.norm(orc), (name, np.linalg.norm(mine - orc) /
                                                                                  np.linalg.norm(orc))
