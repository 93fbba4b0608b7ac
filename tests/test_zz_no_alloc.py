"""sayaka_mac_residual_norm_noalloc, the residual entry point that allocates no
device memory, called through the C ABI and checked against the existing
entry points: the residual of sayaka_mac_residual_compact (same operator
arithmetic, so bit-identical), its max norm (order-independent, so exact) and
the initial residual norm that the device solve's fused residual kernel
reports.  r.r is a sum in a different order: relative tolerance 1e-12."""
import numpy as np
import pytest

import sayakaamr_gb300 as sg
from test_gpu_parity import setup_solver

pytestmark = pytest.mark.gpu

MAX_CELLS = 8192 * 256  # the entry point's stated limit
SUM_RTOL = 1e-12


def _entry(lib):
    # (h, L, x, rhs, r, norms, stream): device pointers and a cudaStream_t
    return lib.sayaka_mac_residual_norm_noalloc


def _noalloc_twice(S, L, inputs):
    """consecutive calls on one stream with no synchronisation between them"""
    import torch
    fn = _entry(S.lib)
    stream = torch.cuda.Stream()
    outs = []
    with torch.cuda.stream(stream):
        for x, rhs in inputs:
            dx = torch.from_numpy(x).cuda()
            drhs = torch.from_numpy(rhs).cuda()
            dr = torch.zeros_like(dx)
            dn = torch.zeros(2, dtype=torch.float64, device="cuda")
            rc = fn(S.h, L, dx.data_ptr(), drhs.data_ptr(), dr.data_ptr(), dn.data_ptr(), stream.cuda_stream)
            assert rc == sg.OK, S.lib.sayaka_mac_last_error(S.h)
            outs.append((dx, drhs, dr, dn))
    torch.cuda.synchronize()
    return [(dr.cpu().numpy(), dn.cpu().numpy()) for (_, _, dr, dn) in outs]


def _check_against_existing(S, L, x, rhs, r, norms):
    r_ref = S.residual(L, x, rhs)
    assert np.array_equal(r, r_ref)
    assert norms[0] == np.max(np.abs(r_ref))
    rr = float(np.dot(r_ref, r_ref))
    assert abs(norms[1] - rr) <= SUM_RTOL * rr


@pytest.mark.parametrize("name", ["t2s", "t3n", "c1"])
def test_noalloc_residual_matches_existing_entry_points(name):
    g, t, tb, S = setup_solver(name)
    L = int(tb["level"].max())
    n = S.num_blocks * S.ncell
    rng = np.random.default_rng(1234)
    inputs = [(rng.standard_normal(n), rng.standard_normal(n)) for _ in range(2)]
    res = _noalloc_twice(S, L, inputs)
    for (x, rhs), (r, norms) in zip(inputs, res):
        _check_against_existing(S, L, x, rhs, r, norms)
    # the device solve's own fused residual kernel reports the same max norm
    x, rhs = inputs[1]
    S.set_init_sol(x, ncomp=1, ngrow=0, comp=0)
    S.set_rhs_compact(rhs)
    S.set_params(use_mg_precond=1, bottom=1, max_iter=2)
    info = S.cg_solve()
    assert info["rnorm0"] == res[1][1][0]


def _uniform_3d(nroot, level):
    t = sg.AmrTree(3, 16, level, level, 4096)
    t.init_uniform_root(nroot, (0, 0, 0), tuple(float(v) for v in nroot), (-20,) * 6, (0,) * 6)
    t.init_refine_to_min_level()
    return sg.MacSolver(t.tables())


def test_noalloc_residual_at_the_size_limit_and_beyond():
    import torch
    # 512 level-4 blocks of 16^3 cells: exactly the limit, accepted
    S = _uniform_3d((1, 1, 1), 4)
    assert S.tower_size(4) * S.ncell == MAX_CELLS
    n = S.num_blocks * S.ncell
    rng = np.random.default_rng(99)
    inputs = [(rng.standard_normal(n), rng.standard_normal(n)) for _ in range(2)]
    for (x, rhs), (r, norms) in zip(inputs, _noalloc_twice(S, 4, inputs)):
        _check_against_existing(S, 4, x, rhs, r, norms)
    del S
    # 1024 blocks: twice the limit, rejected before any launch (buffers are
    # full size all the same)
    S = _uniform_3d((2, 1, 1), 4)
    n = S.num_blocks * S.ncell
    assert S.tower_size(4) * S.ncell == 2 * MAX_CELLS
    buf = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    dn = torch.zeros(2, dtype=torch.float64, device="cuda")
    rc = _entry(S.lib)(S.h, 4, buf[0].data_ptr(), buf[1].data_ptr(), buf[2].data_ptr(), dn.data_ptr(), None)
    assert rc == sg.BAD_INPUT
    msg = S.lib.sayaka_mac_last_error(S.h).decode()
    assert "4194304 cells" in msg and "2097152" in msg, msg
    torch.cuda.synchronize()
    assert float(dn.abs().sum()) == 0.0


def test_noalloc_residual_keeps_nan():
    """a NaN in the residual reaches |r|_inf (a dropped NaN would let a
    diverged iterate pass a convergence test)"""
    g, t, tb, S = setup_solver("t2s")
    L = int(tb["level"].max())
    n = S.num_blocks * S.ncell
    rng = np.random.default_rng(7)
    x, rhs = rng.standard_normal(n), rng.standard_normal(n)
    blocks, _ = t.tower(L)
    vf = S.get_coef(2)
    cell = next(int(b) * S.ncell + q for b in blocks for q in range(S.ncell) if vf[int(b) * S.ncell + q] > 0)
    rhs[cell] = np.nan
    (r, norms), = _noalloc_twice(S, L, [(x, rhs)])
    assert np.isnan(r[cell])
    assert np.isnan(norms[0]) and np.isnan(norms[1]), norms


def test_noalloc_residual_allocates_nothing():
    """free device memory is the same before and after warmed-up calls (the
    inputs and outputs are made beforehand)"""
    import torch
    g, t, tb, S = setup_solver("t3n")
    L = int(tb["level"].max())
    n = S.num_blocks * S.ncell
    rng = np.random.default_rng(11)
    dx = torch.from_numpy(rng.standard_normal(n)).cuda()
    drhs = torch.from_numpy(rng.standard_normal(n)).cuda()
    dr = torch.zeros_like(dx)
    dn = torch.zeros(2, dtype=torch.float64, device="cuda")
    fn = _entry(S.lib)
    stream = torch.cuda.current_stream()

    def call():
        rc = fn(S.h, L, dx.data_ptr(), drhs.data_ptr(), dr.data_ptr(), dn.data_ptr(), stream.cuda_stream)
        assert rc == sg.OK, S.lib.sayaka_mac_last_error(S.h)

    call()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        call()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    r = S.residual(L, dx.cpu().numpy(), drhs.cpu().numpy())
    assert np.array_equal(dr.cpu().numpy(), r)


def test_noalloc_residual_runs_on_the_handle_device():
    """with another device current, the call still runs on the device the
    handle's buffers live on (needs two GPUs)"""
    import torch
    if torch.cuda.device_count() < 2:
        pytest.skip("needs two visible GPUs")
    torch.cuda.set_device(0)
    g, t, tb, S = setup_solver("t2s")
    L = int(tb["level"].max())
    n = S.num_blocks * S.ncell
    rng = np.random.default_rng(3)
    x, rhs = rng.standard_normal(n), rng.standard_normal(n)
    dx = torch.from_numpy(x).to("cuda:0")
    drhs = torch.from_numpy(rhs).to("cuda:0")
    dr = torch.zeros_like(dx)
    dn = torch.zeros(2, dtype=torch.float64, device="cuda:0")
    try:
        torch.cuda.set_device(1)
        rc = _entry(S.lib)(S.h, L, dx.data_ptr(), drhs.data_ptr(), dr.data_ptr(), dn.data_ptr(), None)
        assert rc == sg.OK, S.lib.sayaka_mac_last_error(S.h)
        assert torch.cuda.current_device() == 1
    finally:
        torch.cuda.set_device(0)
    torch.cuda.synchronize(0)
    _check_against_existing(S, L, x, rhs, dr.cpu().numpy(), dn.cpu().numpy())
