"""Pins the C oracle (oracle/mac_oracle.c) against the reference library's own
outputs (golden fixtures from oracle/ref_dump.cpp).  The oracle keeps the
reference's serial operation order, so every comparison here is bit-exact,
including the V-cycle (bottom BiCGSTAB) and whole solves."""
import numpy as np
import pytest

import golden_io
from cases import CASES, all_neumann, bc_table, build_tree
from oracle import pyoracle

OPS = [n for n in sorted(CASES) if CASES[n]["do_ops"]]


def oracle_for(name):
    g = golden_io.load(name)
    t = build_tree(name)
    tb = t.tables()
    nd, nb, n = tb["ndim"], tb["nb"], tb["num_blocks"]
    nc, nfb = nb ** nd, (nb + 1) * nb ** (nd - 1)
    if isinstance(g.get("vf"), golden_io.Digest):
        # digest fixture: the oracle's own coefficient setup, pinned against
        # the reference's synced fields by test_coefficient_setup
        from test_gpu_parity_helpers import fractional_ib
        vol, areas = fractional_ib(name, tb)
        vf, af, bc = pyoracle.setup_coefficients(tb, bc_table(name, tb), vol, areas,
                                                 [g["in_b%d" % d] for d in range(nd)])
    else:
        vf = g["vf"] if "vf" in g else np.ones(n * nc)
        af = [g["af%d" % d] if "af%d" % d in g else np.ones(n * nfb) for d in range(nd)]
        bc = [g["bcoef%d" % d] if "bcoef%d" % d in g else np.ones(n * nfb) for d in range(nd)]
    return g, t, tb, pyoracle.Oracle(tb, bc_table(name, tb), vf, af, bc)


@pytest.fixture(scope="module", params=OPS)
def prob(request):
    return (request.param,) + oracle_for(request.param)


def rows(a, blocks, per):
    return a.reshape(-1, per)[np.asarray(blocks)].reshape(-1)


def exact(a, b):
    """bit-for-bit (fixture arrays or their digests)"""
    return golden_io.matches(a, b)


def test_towers(prob):
    name, g, t, tb, O = prob
    for L in range(1, tb["max_level"] + 1):
        blocks, be, ft = O.tower(L)
        np.testing.assert_array_equal(blocks, g["tower_%d_blocks" % L])
        regs = g["tower_%d_face_regs" % L].reshape(-1, 2 * tb["ndim"], 9)
        np.testing.assert_array_equal(ft.reshape(-1, 6)[:, :2 * tb["ndim"]], regs[:, :, 0])


def test_apply_residual(prob):
    name, g, t, tb, O = prob
    n, nc = tb["num_blocks"], O.ncell
    x = golden_io.seeded_input(name, "op_x", n * nc)
    for L in range(1, tb["level"].max() + 1):
        if "op_apply_%d" % L in g:
            assert exact(rows(O.apply(L, x), t.tower(L)[0], nc), g["op_apply_%d" % L]), (name, L)
    finest = tb["level"].max()
    r = O.residual(finest, x, golden_io.seeded_input(name, "op_rhs", n * nc))
    assert exact(rows(r, t.tower(finest)[0], nc), g["op_resid"])


def test_smooth(prob):
    name, g, t, tb, O = prob
    n, nc = tb["num_blocks"], O.ncell
    corr = golden_io.seeded_input(name, "sm_corr0", n * nc)
    res = golden_io.seeded_input(name, "sm_resid", n * nc)
    for L in range(1, tb["level"].max() + 1):
        if "sm_out_%d" % L in g:
            assert exact(rows(O.smooth(L, corr, res), t.tower(L)[0], nc), g["sm_out_%d" % L]), (name, L)


def test_transfers_flux_bc(prob):
    name, g, t, tb, O = prob
    n, nc, nd, nb = tb["num_blocks"], O.ncell, tb["ndim"], tb["nb"]
    assert exact(O.restrict_sweep(golden_io.seeded_input(name, "rs_in", n * nc)), g["rs_out"])
    assert exact(O.prolong_sweep(golden_io.seeded_input(name, "pr_in", n * nc)), g["pr_out"])
    phi = golden_io.seeded_input(name, "fx_phi", n * nc)
    leaf = t.tower(tb["level"].max())[0]
    for d in range(nd):
        assert exact(rows(O.flux(d, phi), leaf, O.nfb), g["fx_out%d" % d]), (name, d)
    phig = golden_io.seeded_input(name, "bc_phi", n * (nb + 2) ** nd)
    r0 = golden_io.seeded_input(name, "bc_rhs0", n * nc)
    assert exact(O.fix_bc(phig, r0), g["bc_rhs"])


def vc_input(name, g, t, tb, vf):
    n, nc, nd, nb = tb["num_blocks"], tb["nb"] ** tb["ndim"], tb["ndim"], tb["nb"]
    p = golden_io.seeded_input(name, "vc_p", n * nc)
    if all_neumann(name):
        lens = tb["block_len"].reshape(n, 3)
        s = v = 0.0
        leaf = t.tower(tb["level"].max())[0]
        for b in leaf:
            dv = 1.0
            for d in range(nd):
                dv *= lens[b, d] / nb
            for q in range(nc):
                w = vf[b * nc + q]
                if w > 0:
                    s += p[b * nc + q] * dv * w
                    v += dv * w
        for b in leaf:
            p[b * nc:(b + 1) * nc] -= s / v
    return p


def test_vcycle_bit_exact(prob):
    name, g, t, tb, O = prob
    n, nc = tb["num_blocks"], O.ncell
    vf = g["vf"] if "vf" in g and not isinstance(g["vf"], golden_io.Digest) else oracle_vf(O, n * nc)
    p = vc_input(name, g, t, tb, vf)
    phat = O.vcycle(p, pyoracle.params())
    assert exact(rows(phat, t.tower(tb["level"].max())[0], nc), g["vc_phat"]), name


def oracle_vf(O, n):
    """the volume fraction the oracle was given"""
    return np.ctypeslib.as_array(O.P.vf, shape=(n,)).copy()


def solve_params(name, g):
    """the reference solve's parameters as the fixture records them"""
    c = CASES[name]
    kw = dict(tol_rel=c["tol_rel"], tol_abs=0.0)
    if "sv_bot_tol_rel" in g:
        kw.update(bot_tol_rel=float(g["sv_bot_tol_rel"][0]), bot_tol_abs=float(g["sv_bot_tol_abs"][0]))
    return pyoracle.params(**kw)


@pytest.mark.parametrize("name", ["t2b", "t3n", "t3s", "n2", "n3"])
def test_solve_bit_exact(name):
    g, t, tb, O = oracle_for(name)
    sol, info = O.cg_solve(g["sv_rhs"], solve_params(name, g))
    assert info["status"] == 0
    leaf = t.tower(tb["level"].max())[0]
    assert exact(rows(sol, leaf, O.ncell), g["sv_sol"]), name


@pytest.mark.parametrize("name", ["t2s", "t3s", "n2", "n3"])
def test_coefficient_setup(name):
    """setCoefB / IB-fraction sync + restriction against the reference"""
    from test_gpu_parity_helpers import fractional_ib
    g = golden_io.load(name)
    t = build_tree(name)
    tb = t.tables()
    vol, areas = fractional_ib(name, tb)
    nd = tb["ndim"]
    vf, af, bc = pyoracle.setup_coefficients(tb, bc_table(name, tb), vol, areas, [g["in_b%d" % d] for d in range(nd)])
    assert exact(vf, g["vf"])
    for d in range(nd):
        assert exact(af[d], g["af%d" % d]), d
        assert exact(bc[d], g["bcoef%d" % d]), d


@pytest.mark.parametrize("name", ["t2s", "t3s", "n2", "n3"])
def test_mg_and_relax_solves_bit_exact(name):
    """mg_solve (stand-alone V-cycles, bottom BiCGSTAB with the solve's bottom
    tolerances) and relax_solve (Gauss-Seidel sweeps), a fixed number of
    iterations each, against the reference's"""
    g, t, tb, O = oracle_for(name)
    leaf = t.tower(tb["level"].max())[0]
    kw = dict(tol_rel=1e-30, tol_abs=0.0, bot_tol_rel=float(g["sv_bot_tol_rel"][0]),
              bot_tol_abs=float(g["sv_bot_tol_abs"][0]))
    sol, info = O.mg_solve(g["sv_rhs"], pyoracle.params(max_iter=golden_io.MG_ITERS, **kw))
    assert info["iterations"] == golden_io.MG_ITERS and info["status"] == 2, info
    assert exact(rows(sol, leaf, O.ncell), g["mg_sol"]), name
    sol, info = O.relax_solve(g["sv_rhs"], pyoracle.params(max_iter=golden_io.RELAX_ITERS, **kw))
    assert info["iterations"] == golden_io.RELAX_ITERS, info
    assert exact(rows(sol, leaf, O.ncell), g["rx_sol"]), name


@pytest.mark.parametrize("name", ["t2s", "t3s"])
def test_relaxed_smoother(name):
    """the over-relaxed smoother (orc_params.omega, the product's
    params.relax_omega): omega 1 is the reference's sweep bit for bit, a
    sweep's red cells (updated from old black values only) are
    u_old + omega (u_gs - u_old) of the plain sweep's red cells, and the
    relaxed V-cycle is another preconditioner with the same solution"""
    g, t, tb, O = oracle_for(name)
    n, nc, nb, nd = tb["num_blocks"], O.ncell, tb["nb"], tb["ndim"]
    L = int(tb["level"].max())
    rng = np.random.default_rng(5)
    phi, rhs = rng.standard_normal(n * nc), rng.standard_normal(n * nc)
    plain = O.smooth(L, phi, rhs)
    w1 = np.empty_like(plain)
    O.lib.orc_smooth_relaxed(pyoracle.C.byref(O.P), L, O._in(phi), O._in(rhs), pyoracle.C.c_double(1.0),
                             w1.ctypes.data_as(pyoracle._f64p))
    assert exact(w1, plain)
    # red cells (i+j+k even) of the finest level's blocks, swept first: both
    # sweeps read the same old values when they update them
    om = 1.3
    relaxed = O.smooth(L, phi, rhs, omega=om)
    idx = np.indices((nb,) * nd).reshape(nd, -1)[::-1]  # cell index ci = i + nb j (+ nb^2 k)
    red = (idx.sum(axis=0) % 2) == 0
    vf = oracle_vf(O, n * nc).reshape(n, nc)
    blocks = [b for b in t.tower(L)[0] if tb["level"][b] == L]
    checked = 0
    for b in blocks:
        m = red & (vf[b] > 0)
        if not m.any():
            continue
        checked += 1
        a = relaxed.reshape(n, nc)[b][m]
        want = om * plain.reshape(n, nc)[b][m] + (1 - om) * phi.reshape(n, nc)[b][m]
        assert np.allclose(a, want, rtol=1e-13, atol=1e-13 * np.abs(want).max()), b
    assert checked > 0
    sols = []
    for omega in (1.0, 1.1):
        sol, info = O.cg_solve(g["sv_rhs"], pyoracle.params(tol_rel=1e-11, tol_abs=0.0, bot_tol_rel=1e-10,
                                                            bot_tol_abs=0.0, omega=omega))
        assert info["status"] == 0, (omega, info)
        sols.append(rows(sol, t.tower(L)[0], nc))
    d = sols[1] - sols[0]
    if tb["neighbor"].min() > -30:  # all-Neumann trees: compare up to a constant
        d = d - d.mean()
    assert np.linalg.norm(d) <= 1e-8 * np.linalg.norm(sols[0])
