"""ctypes binding of the C oracle (oracle/mac_oracle.c).

ORACLE -- test infrastructure: imported only by tests/, __graft_entry__.smoke()
and bench.py's CPU-baseline leg, as the checker / CPU reference timing.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "libsayaka_oracle.so")

_i32p = C.POINTER(C.c_int32)
_f64p = C.POINTER(C.c_double)


class _Problem(C.Structure):
    _fields_ = [("ndim", C.c_int), ("nb", C.c_int), ("nblocks", C.c_int), ("max_level", C.c_int),
                ("level", _i32p), ("neighbor", _i32p), ("child", _i32p), ("parent", _i32p),
                ("which_child", _i32p), ("node_type", _i32p), ("block_len", _f64p), ("bc_type", _i32p),
                ("vf", _f64p), ("af", _f64p * 3), ("bcoef", _f64p * 3), ("alpha", C.c_double),
                ("beta", C.c_double)]


class _Params(C.Structure):
    _fields_ = [("max_iter", C.c_int), ("tol_rel", C.c_double), ("tol_abs", C.c_double), ("n_post", C.c_int),
                ("use_precond", C.c_int), ("bot_tol_rel", C.c_double), ("bot_tol_abs", C.c_double),
                ("bot_max_iter", C.c_int), ("omega", C.c_double)]


class _Info(C.Structure):
    _fields_ = [("status", C.c_int), ("iterations", C.c_int), ("rnorm0", C.c_double), ("rnorm", C.c_double)]


_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from sayakaamr_gb300 import build
            build.build_oracle()
        _lib = C.CDLL(LIB_PATH)
    return _lib


def params(max_iter=2000, tol_rel=1e-6, tol_abs=0.0, n_post=2, use_precond=1, bot_tol_rel=1e-6, bot_tol_abs=1e-6,
           bot_max_iter=2000, omega=1.0):
    return _Params(max_iter, tol_rel, tol_abs, n_post, use_precond, bot_tol_rel, bot_tol_abs, bot_max_iter, omega)


def setup_coefficients(tables, bc, vf=None, af=None, bcoef=None):
    """Coefficient sync + restriction of the reference on leaf-valued arrays
    (returns new arrays; None entries are skipped)."""
    lib = load()
    nd = int(tables["ndim"])
    keep = []
    vf2 = None if vf is None else np.array(vf, dtype=np.float64)
    af2 = [None] * 3 if af is None else [np.array(a, dtype=np.float64) for a in af] + [None] * (3 - len(af))
    b2 = [None] * 3 if bcoef is None else [np.array(a, dtype=np.float64) for a in bcoef] + [None] * (3 - len(bcoef))
    n = int(tables["num_blocks"])
    nb = int(tables["nb"])
    ones_c = np.ones(n * nb ** nd)
    ones_f = [np.ones(n * (nb + 1) * nb ** (nd - 1)) for _ in range(nd)]
    O = Oracle(tables, bc, vf2 if vf2 is not None else ones_c, [a if a is not None else ones_f[d] for d, a in
                                                                 enumerate(af2[:nd])],
               [a if a is not None else ones_f[d] for d, a in enumerate(b2[:nd])])

    def ptr(a):
        return C.cast(0, _f64p) if a is None else a.ctypes.data_as(_f64p)

    lib.orc_setup_coefficients(C.byref(O.P), ptr(vf2), ptr(af2[0]), ptr(af2[1]), ptr(af2[2]), ptr(b2[0]), ptr(b2[1]),
                               ptr(b2[2]))
    return vf2, af2[:nd], b2[:nd]


class Oracle:
    """CPU restatement of the reference MAC solver over one tree.

    tables: dict of tree tables (sayakaamr_gb300.AmrTree.tables()); bc: math BC
    per block face; vf / af / bcoef: the synced/restricted coefficient fields
    over all blocks (compact layouts)."""

    def __init__(self, tables, bc, vf, af, bcoef, alpha=0.0, beta=1.0):
        self.lib = load()
        t = tables
        self.nd, self.nb, self.n = int(t["ndim"]), int(t["nb"]), int(t["num_blocks"])
        self.ncell = self.nb ** self.nd
        self.nfb = (self.nb + 1) * self.nb ** (self.nd - 1)
        self._keep = []

        def i32(a):
            a = np.ascontiguousarray(a, dtype=np.int32)
            self._keep.append(a)
            return a.ctypes.data_as(_i32p)

        def f64(a):
            a = np.ascontiguousarray(a, dtype=np.float64)
            self._keep.append(a)
            return a.ctypes.data_as(_f64p)

        P = _Problem()
        P.ndim, P.nb, P.nblocks, P.max_level = self.nd, self.nb, self.n, int(t["max_level"])
        P.level, P.neighbor, P.child = i32(t["level"]), i32(t["neighbor"]), i32(t["child"])
        P.parent, P.which_child, P.node_type = i32(t["parent"]), i32(t["which_child"]), i32(t["node_type"])
        P.block_len = f64(t["block_len"])
        P.bc_type = i32(bc)
        P.vf = f64(vf)
        for d in range(3):
            P.af[d] = f64(af[d]) if d < self.nd else C.cast(0, _f64p)
            P.bcoef[d] = f64(bcoef[d]) if d < self.nd else C.cast(0, _f64p)
        P.alpha, P.beta = alpha, beta
        self.P = P

    def _cells(self):
        return np.zeros(self.n * self.ncell)

    def _in(self, x):
        a = np.ascontiguousarray(x, dtype=np.float64)
        self._keep.append(a)
        return a.ctypes.data_as(_f64p)

    def apply(self, L, x):
        y = self._cells()
        self.lib.orc_apply(C.byref(self.P), int(L), self._in(x), y.ctypes.data_as(_f64p))
        return y

    def residual(self, L, x, rhs):
        r = self._cells()
        self.lib.orc_residual(C.byref(self.P), int(L), self._in(x), self._in(rhs), r.ctypes.data_as(_f64p))
        return r

    def smooth(self, L, phi, rhs, omega=1.0):
        out = self._cells()
        if omega == 1.0:
            self.lib.orc_smooth(C.byref(self.P), int(L), self._in(phi), self._in(rhs), out.ctypes.data_as(_f64p))
        else:
            self.lib.orc_smooth_relaxed(C.byref(self.P), int(L), self._in(phi), self._in(rhs), C.c_double(omega),
                                        out.ctypes.data_as(_f64p))
        return out

    def restrict_sweep(self, x):
        out = self._cells()
        self.lib.orc_restrict_sweep(C.byref(self.P), self._in(x), out.ctypes.data_as(_f64p))
        return out

    def prolong_sweep(self, x):
        out = self._cells()
        self.lib.orc_prolong_sweep(C.byref(self.P), self._in(x), out.ctypes.data_as(_f64p))
        return out

    def flux(self, d, phi):
        out = np.zeros(self.n * self.nfb)
        self.lib.orc_flux(C.byref(self.P), int(d), self._in(phi), out.ctypes.data_as(_f64p))
        return out

    def fix_bc(self, phi_grown, rhs):
        r = np.ascontiguousarray(rhs, dtype=np.float64).copy()
        self.lib.orc_fix_bc(C.byref(self.P), self._in(phi_grown), r.ctypes.data_as(_f64p))
        return r

    def vcycle(self, p, prm=None):
        out = self._cells()
        prm = prm or params()
        self.lib.orc_vcycle(C.byref(self.P), C.byref(prm), self._in(p), out.ctypes.data_as(_f64p))
        return out

    def cg_solve(self, rhs, prm=None, sol0=None):
        prm = prm or params()
        sol = np.zeros(self.n * self.ncell) if sol0 is None else np.array(sol0, dtype=np.float64)
        info = _Info()
        self.lib.orc_cg_solve(C.byref(self.P), C.byref(prm), self._in(rhs), sol.ctypes.data_as(_f64p),
                              C.byref(info))
        return sol, dict(status=info.status, iterations=info.iterations, rnorm0=info.rnorm0, rnorm=info.rnorm)

    def mg_solve(self, rhs, prm=None, sol0=None):
        """mg_solve: stand-alone V-cycle iterations (src/SayakaMacSolver.cpp:43-162)"""
        return self._solve(self.lib.orc_mg_solve, rhs, prm, sol0)

    def relax_solve(self, rhs, prm=None, sol0=None):
        """relax_solve: Gauss-Seidel sweeps of the finest tower (src/SayakaMacSolver.cpp:377-452)"""
        return self._solve(self.lib.orc_relax_solve, rhs, prm, sol0)

    def _solve(self, fn, rhs, prm, sol0):
        prm = prm or params()
        sol = np.zeros(self.n * self.ncell) if sol0 is None else np.array(sol0, dtype=np.float64)
        info = _Info()
        fn(C.byref(self.P), C.byref(prm), self._in(rhs), sol.ctypes.data_as(_f64p), C.byref(info))
        return sol, dict(status=info.status, iterations=info.iterations, rnorm0=info.rnorm0, rnorm=info.rnorm)

    def tower(self, L):
        blocks = np.zeros(self.n, dtype=np.int32)
        n = C.c_int32()
        be = np.zeros(2 * L, dtype=np.int32)
        ft = np.zeros(self.n * 6, dtype=np.int32)
        self.lib.orc_tower(C.byref(self.P), int(L), blocks.ctypes.data_as(_i32p), C.byref(n), be.ctypes.data_as(_i32p),
                           ft.ctypes.data_as(_i32p))
        return blocks[:n.value], be, ft[:n.value * 6]
