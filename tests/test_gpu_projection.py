"""The projection step around the solve, on the GPU through the C ABI, against
a numpy restatement in the reference's operation order (bit for bit):
  * rhs = sum_d (scale/dh_d) * (u_d(i+1) - u_d(i)) on every block
    (src/Test7.h:587-609 with scale = -1/dt; src/Test6.h:798-830 with
    scale = 1 and the 1/rho face weight);
  * u_dir += dt * mg_flux_level(finest, dir, solution) on the finest tower
    (src/Test7.h:634-645), the flux checked against sayaka_mac_flux, which
    the parity tests pin to the reference."""
import numpy as np
import pytest

from test_gpu_parity import setup_solver

pytestmark = pytest.mark.gpu


def face_index(d, ijk, s, nb):
    f = [ijk[0], ijk[1], ijk[2]]
    f[d] = f[d] + s
    e0 = nb + (d == 0)
    e1 = nb + (d == 1)
    return f[0] + e0 * (f[1] + e1 * f[2])


def cell_ijk(nb, nd):
    c = np.arange(nb ** nd)
    return [c % nb, (c // nb) % nb if nd >= 2 else 0 * c, c // (nb * nb) if nd == 3 else 0 * c]


def face_treedata(comps, nb, nd, d, ngrow):
    """compact face arrays (one per component, [block][face]) -> the
    reference's TreeData face layout with ngrow ghost layers"""
    n = comps[0].shape[0]
    dims = [nb + 2 * ngrow] * nd
    dims[d] += 1
    shape = tuple(reversed(dims))  # [k][j][i]
    out = np.full((n, len(comps)) + shape, np.nan)
    valid = [nb] * nd
    valid[d] += 1
    sl = tuple(slice(ngrow, ngrow + v) for v in reversed(valid))
    for c, a in enumerate(comps):
        out[(slice(None), c) + sl] = a.reshape((n,) + tuple(reversed(valid)))
    return out.reshape(-1)


def treedata_to_face(buf, n, ncomp, comp, nb, nd, d, ngrow):
    dims = [nb + 2 * ngrow] * nd
    dims[d] += 1
    a = buf.reshape((n, ncomp) + tuple(reversed(dims)))[:, comp]
    valid = [nb] * nd
    valid[d] += 1
    sl = tuple(slice(ngrow, ngrow + v) for v in reversed(valid))
    return a[(slice(None),) + sl].reshape(n, -1)


@pytest.mark.parametrize("weighted", [False, True])
@pytest.mark.parametrize("name", ["t2s", "t3n"])
def test_rhs_from_face_velocity(name, weighted):
    g, t, tb, S = setup_solver(name)
    nb, nd, n = S.nb, S.ndim, S.num_blocks
    rng = np.random.default_rng(7)
    u = [rng.standard_normal((n, S.nfb)) for _ in range(nd)]
    w = [rng.uniform(0.001, 1.0, (n, S.nfb)) for _ in range(nd)]
    bufs = [face_treedata([u[d], w[d]], nb, nd, d, 1) for d in range(nd)]
    scale = -1.0 / 0.0125 if not weighted else 1.0
    S.set_rhs_div(bufs, scale, ncomp=2, ngrow=1, ucomp=0, wcomp=1 if weighted else -1)
    got = S.get_rhs_compact().reshape(n, -1)
    dh = tb["block_len"].reshape(n, 3)[:, :nd] / nb
    ijk = cell_ijk(nb, nd)
    acc = np.zeros((n, nb ** nd))
    for d in range(nd):
        fl = face_index(d, ijk, 0, nb)
        fr = face_index(d, ijk, 1, nb)
        ul, ur = u[d][:, fl], u[d][:, fr]
        if weighted:
            ul = ul * w[d][:, fl]
            ur = ur * w[d][:, fr]
        acc = acc + (scale / dh[:, d])[:, None] * (ur - ul)
    assert np.array_equal(got, acc)


@pytest.mark.parametrize("name", ["t2s", "t3n"])
def test_velocity_correction_uses_the_device_solution(name):
    g, t, tb, S = setup_solver(name)
    nb, nd, n = S.nb, S.ndim, S.num_blocks
    rng = np.random.default_rng(11)
    p = rng.standard_normal(n * S.ncell)
    S.set_init_sol(p, ncomp=1, ngrow=0, comp=0)
    tower = np.zeros(n, bool)
    blocks, _ = t.tower(int(tb["level"].max()))
    tower[np.asarray(blocks)] = True
    dt = 0.0125
    for d in range(nd):
        u = rng.standard_normal((n, S.nfb))
        buf = face_treedata([u], nb, nd, d, 1)
        flux = S.flux_compact(d, p).reshape(n, -1)
        S.correct_vel(d, dt, buf, ncomp=1, ngrow=1, comp=0)
        got = treedata_to_face(buf, n, 1, 0, nb, nd, d, 1)
        want = u.copy()
        want[tower] = u[tower] + dt * flux[tower]
        assert np.array_equal(got, want)
