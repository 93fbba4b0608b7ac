"""TreeData-layout host buffers through the C ABI on a field large enough to
be split over the host worker pool (config2: 1768 blocks, 3.6 MB per
component): set_rhs / set_init_sol read exactly the valid cells of the
chosen component, get_sol writes exactly those and leaves ghosts and the
other components untouched (TreeData::Copy, src/SayakaTreeData.cpp:230-249)."""
import numpy as np
import pytest

from sayakaamr_gb300 import workloads

pytestmark = pytest.mark.gpu


def treedata(compact, n, nb, nd, ncomp, comp, ngrow, fill):
    G = nb + 2 * ngrow
    out = np.full((n, ncomp) + (G,) * nd, fill)
    sl = (slice(None), comp) + (slice(ngrow, ngrow + nb),) * nd
    out[sl] = compact.reshape((n,) + (nb,) * nd)
    return out


@pytest.mark.parametrize("ncomp,comp,ngrow", [(1, 0, 1), (3, 2, 2)])
def test_treedata_round_trip_on_config2(ncomp, comp, ngrow):
    p = workloads.config2()
    S = workloads.make_solver(p)
    n, nb, nd = S.num_blocks, S.nb, S.ndim
    rng = np.random.default_rng(ncomp * 10 + ngrow)
    x = rng.standard_normal(n * S.ncell)
    buf = treedata(x, n, nb, nd, ncomp, comp, ngrow, np.nan)
    S.set_rhs(buf.reshape(-1), ncomp=ncomp, ngrow=ngrow, comp=comp)
    assert np.array_equal(S.get_rhs_compact(), x)
    S.set_init_sol(buf.reshape(-1), ncomp=ncomp, ngrow=ngrow, comp=comp)
    assert np.array_equal(S.get_sol_compact(), x)
    out = np.full(buf.size, -7.0)
    S.get_sol(out, ncomp=ncomp, ngrow=ngrow, comp=comp)
    want = treedata(x, n, nb, nd, ncomp, comp, ngrow, -7.0).reshape(-1)
    assert np.array_equal(out, want)


@pytest.mark.parametrize("name,ncomp,comp,ngrow", [("config2", 1, 0, 1), ("config2", 3, 2, 2), ("config3", 2, 1, 1)])
def test_pinned_treedata_is_gathered_by_the_gpu(name, ncomp, comp, ngrow):
    """a pinned (page-locked) TreeData buffer is read and written by the GPU
    directly (no staging copy): the same valid cells as the pageable path,
    ghosts and the other components untouched"""
    torch = pytest.importorskip("torch")
    p = workloads.config3(max_level=3) if name == "config3" else workloads.config2()
    S = workloads.make_solver(p)
    n, nb, nd = S.num_blocks, S.nb, S.ndim
    rng = np.random.default_rng(ncomp * 10 + ngrow + 3)
    x = rng.standard_normal(n * S.ncell)
    buf = treedata(x, n, nb, nd, ncomp, comp, ngrow, np.nan).reshape(-1)
    pin = torch.from_numpy(buf).pin_memory()
    pin_np = pin.numpy()
    S.set_rhs(pin_np, ncomp=ncomp, ngrow=ngrow, comp=comp)
    assert np.array_equal(S.get_rhs_compact(), x)
    S.set_init_sol(pin_np, ncomp=ncomp, ngrow=ngrow, comp=comp)
    assert np.array_equal(S.get_sol_compact(), x)
    out = torch.full((buf.size,), -7.0, dtype=torch.float64).pin_memory()
    S.get_sol(out.numpy(), ncomp=ncomp, ngrow=ngrow, comp=comp)
    want = treedata(x, n, nb, nd, ncomp, comp, ngrow, -7.0).reshape(-1)
    assert np.array_equal(out.numpy(), want)
