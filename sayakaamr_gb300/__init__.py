"""sayakaamr_gb300 -- GB300-native MAC pressure-Poisson solver for block-structured
AMR trees, a drop-in for the MacSolver path of the SayakaAmr library.

Python binding of the C ABI in include/sayaka_gb300.h.  The classes mirror the
reference's interface: AmrTree (src/SayakaTree.h) and MacSolver
(src/SayakaMacSolver.h).  All computation happens in the native library
(_lib/libsayaka_gb300.so); importing this module does not touch the GPU, and
every solver call fails loudly when the library or a GPU is missing.
"""
import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_lib", "libsayaka_gb300.so")

OK, BREAKDOWN, NOT_CONVERGED, STALL_FALLBACK, BAD_INPUT, CUDA_ERROR = range(6)
STATUS_NAMES = {0: "OK", 1: "BREAKDOWN", 2: "NOT_CONVERGED", 3: "STALL_FALLBACK", 4: "BAD_INPUT",
                5: "CUDA_ERROR"}
# math boundary conditions (BCType, src/SayakaBoundaryPatch.h:53-58)
NEUMANN, DIRICHLET, SIMPLE_FILL = 0, 1, 2
PHYS_BNDRY = -20

_i32p = C.POINTER(C.c_int32)
_f64p = C.POINTER(C.c_double)
_f32p = C.POINTER(C.c_float)


class TreeTables(C.Structure):
    _fields_ = [("ndim", C.c_int32), ("nb", C.c_int32), ("num_blocks", C.c_int32), ("min_level", C.c_int32),
                ("max_level", C.c_int32), ("level", _i32p), ("neighbor", _i32p), ("child", _i32p),
                ("parent", _i32p), ("which_child", _i32p), ("node_type", _i32p), ("block_len", _f64p)]


class Params(C.Structure):
    _fields_ = [("max_iter", C.c_int32), ("tol_rel", C.c_double), ("tol_abs", C.c_double),
                ("n_post_smooth", C.c_int32), ("use_mg_precond", C.c_int32), ("bot_tol_rel", C.c_double),
                ("bot_tol_abs", C.c_double), ("bot_max_iter", C.c_int32), ("precision", C.c_int32),
                ("bottom", C.c_int32), ("verbose", C.c_int32), ("graph", C.c_int32),
                ("vcycle_kernel", C.c_int32), ("pdl", C.c_int32),
                ("cluster_cells", C.c_int32), ("smooth_variant", C.c_int32), ("learned", C.c_int32),
                ("bottom_level", C.c_int32), ("bottom_half", C.c_int32), ("sublevel_order", C.c_int32),
                ("smoother", C.c_int32), ("inner_sweeps", C.c_int32), ("per_problem", C.c_int32),
                ("uniform", C.c_int32), ("bottom_refresh", C.c_int32),
                ("learned_tc05", C.c_int32), ("vcycle_out", C.c_int32), ("prolong_form", C.c_int32),
                ("learned_loss", C.c_int32), ("relax_omega", C.c_double)]


class SolveInfo(C.Structure):
    _fields_ = [("status", C.c_int32), ("iterations", C.c_int32), ("rnorm0", C.c_double), ("rnorm", C.c_double),
                ("seconds", C.c_double)]


# exported symbols and their signatures (restype, argtypes)
_V = C.c_void_p
_PV = C.POINTER(C.c_void_p)
SIGNATURES = {
    "sayaka_tree_create": (C.c_int, [C.c_int32] * 5 + [_PV]),
    "sayaka_tree_destroy": (None, [_V]),
    "sayaka_tree_init_uniform_root": (C.c_int, [_V, _i32p, _f64p, _f64p, _i32p, _i32p]),
    "sayaka_tree_init_refine_to_min_level": (C.c_int, [_V]),
    "sayaka_tree_set_refine_flags": (C.c_int, [_V, _i32p, C.c_int32]),
    "sayaka_tree_set_coarsen_flags": (C.c_int, [_V, _i32p, C.c_int32]),
    "sayaka_tree_regrid": (C.c_int, [_V]),
    "sayaka_tree_num_blocks": (C.c_int32, [_V]),
    "sayaka_tree_get_tables": (C.c_int, [_V, C.POINTER(TreeTables)]),
    "sayaka_tree_get_geometry": (C.c_int, [_V, _f64p, _f64p, _f64p]),
    "sayaka_tree_get_node_type2": (C.c_int, [_V, _i32p]),
    "sayaka_tree_get_surrounding": (C.c_int, [_V, _i32p, _i32p, _i32p]),
    "sayaka_tree_get_tower": (C.c_int, [_V, C.c_int32, _i32p, _i32p, _i32p]),
    "sayaka_tree_get_face_regs": (C.c_int, [_V, C.c_int32, _i32p]),
    "sayaka_params_default": (None, [C.POINTER(Params)]),
    "sayaka_mac_create": (C.c_int, [C.POINTER(TreeTables), _PV]),
    "sayaka_mac_destroy": (None, [_V]),
    "sayaka_mac_last_error": (C.c_char_p, [_V]),
    "sayaka_mac_set_scalars": (C.c_int, [_V, C.c_double, C.c_double]),
    "sayaka_mac_set_coef_b": (C.c_int, [_V, C.c_int32, _f64p, C.c_int32, C.c_int32, C.c_int32]),
    "sayaka_mac_set_ib_frac_by_ls": (C.c_int, [_V, _f64p, C.c_int32, C.c_int32, C.c_int32]),
    "sayaka_mac_set_ib_frac_compact": (C.c_int, [_V, _f64p, _f64p, _f64p, _f64p]),
    "sayaka_mac_set_ib_frac_by_ls_compact": (C.c_int, [_V, _V, C.c_int32, C.c_int32]),
    "sayaka_mac_set_bc": (C.c_int, [_V, _i32p]),
    "sayaka_mac_fix_bc": (C.c_int, [_V, _f64p, C.c_int32, C.c_int32, C.c_int32, _f64p, C.c_int32, C.c_int32,
                                    C.c_int32]),
    "sayaka_mac_set_rhs": (C.c_int, [_V, _f64p, C.c_int32, C.c_int32, C.c_int32]),
    "sayaka_mac_set_init_sol": (C.c_int, [_V, _f64p, C.c_int32, C.c_int32, C.c_int32]),
    "sayaka_mac_set_zero_sol": (C.c_int, [_V]),
    "sayaka_mac_get_sol": (C.c_int, [_V, _f64p, C.c_int32, C.c_int32, C.c_int32]),
    "sayaka_mac_set_rhs_compact": (C.c_int, [_V, _V, C.c_int32]),
    "sayaka_mac_get_sol_compact": (C.c_int, [_V, _V, C.c_int32]),
    "sayaka_mac_set_params": (C.c_int, [_V, C.POINTER(Params)]),
    "sayaka_mac_cg_solve": (C.c_int, [_V, C.POINTER(SolveInfo)]),
    "sayaka_mac_mg_solve": (C.c_int, [_V, C.POINTER(SolveInfo)]),
    "sayaka_mac_relax_solve": (C.c_int, [_V, C.POINTER(SolveInfo)]),
    "sayaka_mac_prepare": (C.c_int, [_V]),
    "sayaka_mac_cg_solve_async": (C.c_int, [_V]),
    "sayaka_mac_solve_info": (C.c_int, [_V, C.POINTER(SolveInfo)]),
    "sayaka_mac_stream": (C.c_void_p, [_V]),
    "sayaka_mac_enqueue_kernel": (C.c_int, [_V, C.c_int32, C.c_int32]),
    "sayaka_mac_tower_size": (C.c_int32, [_V, C.c_int32, C.c_int32]),
    "sayaka_mac_tuned_smoother": (C.c_int32, [_V, C.c_int32, C.POINTER(C.c_float), C.c_int32]),
    "sayaka_smoother_variants": (C.c_int32, []),
    "sayaka_mac_launch_counts": (C.c_int, [_V, _i32p, _i32p, _i32p]),
    "sayaka_mac_flux": (C.c_int, [_V, C.c_int32, _f64p, C.c_int32, C.c_int32, C.c_int32, _f64p, C.c_int32,
                                  C.c_int32, C.c_int32]),
    "sayaka_mac_apply_compact": (C.c_int, [_V, C.c_int32, _f64p, _f64p]),
    "sayaka_mac_residual_compact": (C.c_int, [_V, C.c_int32, _f64p, _f64p, _f64p]),
    "sayaka_mac_residual_norm_noalloc": (C.c_int, [_V, C.c_int32, _V, _V, _V, _V, _V]),
    "sayaka_mac_set_rhs_div": (C.c_int, [_V, C.POINTER(_f64p), C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                         C.c_double]),
    "sayaka_mac_correct_vel": (C.c_int, [_V, C.c_int32, C.c_double, _f64p, C.c_int32, C.c_int32, C.c_int32]),
    "sayaka_mac_get_rhs_compact": (C.c_int, [_V, _f64p]),
    "sayaka_mac_init_from": (C.c_int, [_V, _V]),
    "sayaka_mac_init_new_block_data": (C.c_int, [_V, _V, _f64p]),
    "sayaka_mac_bottom_level": (C.c_int32, [_V]),
    "sayaka_mac_problem_count": (C.c_int32, [_V]),
    "sayaka_mac_uniform_blocks": (C.c_int32, [_V]),
    "sayaka_mac_problem_states": (C.c_int32, [_V, _i32p, _f64p, C.c_int32]),
    "sayaka_cuda_peek_error": (C.c_int32, []),
    "sayaka_fp_selftest": (C.c_int, [_f64p, _f32p, C.c_int, _f32p, _f32p, _f64p, _f64p, _f64p, _f64p]),
    "sayaka_mac_learned_nparam": (C.c_int32, []),
    "sayaka_mac_learned_collect": (C.c_int, [_V, C.c_int32, _i32p]),
    "sayaka_mac_learned_collect_sampled": (C.c_int, [_V, C.c_int32, C.c_int32, _i32p]),
    "sayaka_mac_learned_train": (C.c_int, [_V, C.c_int32, C.c_float, C.c_int32, C.c_uint32, _f32p]),
    "sayaka_mac_learned_eval": (C.c_int, [_V, _f32p]),
    "sayaka_mac_learned_get_weights": (C.c_int, [_V, _f32p, C.c_int32]),
    "sayaka_mac_learned_set_weights": (C.c_int, [_V, _f32p, C.c_int32]),
    "sayaka_mac_learned_loss_grad": (C.c_int, [_V, _f32p, _f32p, C.c_int32, _f32p, _f32p]),
    "sayaka_mac_learned_forward": (C.c_int, [_V, _f32p, C.c_int32, _f32p]),
    "sayaka_mac_smooth_compact": (C.c_int, [_V, C.c_int32, _f64p, _f64p, _f64p]),
    "sayaka_mac_device_kernel_compact": (C.c_int, [_V, C.c_int32, C.c_int32, C.c_int32, _f64p, _f64p, _f64p]),
    "sayaka_mac_restrict_compact": (C.c_int, [_V, _f64p, _f64p]),
    "sayaka_mac_prolong_compact": (C.c_int, [_V, _f64p, _f64p]),
    "sayaka_mac_vcycle_compact": (C.c_int, [_V, _f64p, _f64p]),
    "sayaka_mac_flux_compact": (C.c_int, [_V, C.c_int32, _f64p, _f64p]),
    "sayaka_mac_fix_bc_compact": (C.c_int, [_V, _f64p, C.c_int32, _f64p]),
    "sayaka_mac_get_coef_compact": (C.c_int, [_V, C.c_int32, C.c_int32, _f64p]),
}

_lib = None


def load_library(path=None):
    """Load the native library (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError("native library missing: %s (run python -m sayakaamr_gb300.build)" % p)
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def _i32(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(_i32p)


def _f64(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(_f64p)


class SayakaError(RuntimeError):
    pass


def cuda_peek_error():
    """the library's pending CUDA runtime error code on this thread (0: none)"""
    return int(load_library().sayaka_cuda_peek_error())


def fp_selftest(d, f):
    """the device solve's integer-pipe conversions next to the hardware ones:
    (narrow, narrow_hw, widen, widen_hw, widen0, widen0_hw) for doubles d
    and floats f of the same length"""
    lib = load_library()
    d = np.ascontiguousarray(d, dtype=np.float64)
    f = np.ascontiguousarray(f, dtype=np.float32)
    n = len(d)
    assert len(f) == n
    outs = [np.zeros(n, np.float32), np.zeros(n, np.float32)] + [np.zeros(n, np.float64) for _ in range(4)]
    ptr = [o.ctypes.data_as(_f32p if o.dtype == np.float32 else _f64p) for o in outs]
    _check(lib.sayaka_fp_selftest(d.ctypes.data_as(_f64p), f.ctypes.data_as(_f32p), n, *ptr), "fp_selftest")
    return tuple(outs)


def _check(rc, what, handle=None):
    if rc != OK:
        msg = ""
        if handle is not None:
            m = load_library().sayaka_mac_last_error(handle)
            msg = m.decode() if m else ""
        raise SayakaError("%s failed: %s %s" % (what, STATUS_NAMES.get(rc, rc), msg))


class AmrTree:
    """Host block tree (AmrTree + regrid of src/SayakaTree.h, src/SayakaRegrid.cpp)."""

    def __init__(self, ndim, nb, min_level, max_level, capacity=40000):
        self.lib = load_library()
        h = C.c_void_p()
        _check(self.lib.sayaka_tree_create(ndim, nb, min_level, max_level, capacity, C.byref(h)), "tree_create")
        self.h = h
        self.ndim, self.nb, self.min_level, self.max_level, self.capacity = ndim, nb, min_level, max_level, capacity

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.sayaka_tree_destroy(self.h)
            self.h = None

    def init_uniform_root(self, ndiv, lo, hi, bc_type, periodic=(0,) * 6):
        nd, pnd = _i32(ndiv)
        l, pl = _f64(lo)
        u, pu = _f64(hi)
        b, pb = _i32(bc_type)
        pe, ppe = _i32([int(x) for x in periodic])
        _check(self.lib.sayaka_tree_init_uniform_root(self.h, pnd, pl, pu, pb, ppe), "init_uniform_root")

    def init_refine_to_min_level(self):
        _check(self.lib.sayaka_tree_init_refine_to_min_level(self.h), "init_refine_to_min_level")

    def set_refine_flags(self, flags):
        f, pf = _i32(flags)
        _check(self.lib.sayaka_tree_set_refine_flags(self.h, pf, len(f)), "set_refine_flags")

    def set_coarsen_flags(self, flags):
        f, pf = _i32(flags)
        _check(self.lib.sayaka_tree_set_coarsen_flags(self.h, pf, len(f)), "set_coarsen_flags")

    def regrid(self):
        _check(self.lib.sayaka_tree_regrid(self.h), "regrid")

    @property
    def num_blocks(self):
        return self.lib.sayaka_tree_num_blocks(self.h)

    def tables(self):
        t = TreeTables()
        _check(self.lib.sayaka_tree_get_tables(self.h, C.byref(t)), "get_tables")
        n = t.num_blocks

        def arr(p, k, dt):
            return np.ctypeslib.as_array(p, shape=(n * k,)).astype(dt).copy()

        d = dict(ndim=t.ndim, nb=t.nb, num_blocks=n, min_level=t.min_level, max_level=t.max_level,
                 level=arr(t.level, 1, np.int32), neighbor=arr(t.neighbor, 6, np.int32),
                 child=arr(t.child, 8, np.int32), parent=arr(t.parent, 1, np.int32),
                 which_child=arr(t.which_child, 1, np.int32), node_type=arr(t.node_type, 1, np.int32),
                 block_len=arr(t.block_len, 3, np.float64))
        lo = np.zeros(n * 3)
        hi = np.zeros(n * 3)
        ce = np.zeros(n * 3)
        self.lib.sayaka_tree_get_geometry(self.h, lo.ctypes.data_as(_f64p), hi.ctypes.data_as(_f64p),
                                          ce.ctypes.data_as(_f64p))
        d.update(block_lo=lo, block_hi=hi, block_center=ce)
        nt2 = np.zeros(n * 6, dtype=np.int32)
        self.lib.sayaka_tree_get_node_type2(self.h, nt2.ctypes.data_as(_i32p))
        d["node_type2"] = nt2
        return d

    def surrounding(self):
        n = self.num_blocks
        out = [np.zeros(n * 27, dtype=np.int32) for _ in range(3)]
        self.lib.sayaka_tree_get_surrounding(self.h, *[o.ctypes.data_as(_i32p) for o in out])
        return out

    def tower(self, L):
        n = self.num_blocks
        blocks = np.zeros(max(n, 1), dtype=np.int32)
        cnt = C.c_int32()
        be = np.zeros(2 * L, dtype=np.int32)
        _check(self.lib.sayaka_tree_get_tower(self.h, L, blocks.ctypes.data_as(_i32p), C.byref(cnt),
                                              be.ctypes.data_as(_i32p)), "get_tower")
        return blocks[:cnt.value].copy(), be

    def face_regs(self, L):
        blocks, _ = self.tower(L)
        regs = np.zeros(max(len(blocks), 1) * 2 * self.ndim * 9, dtype=np.int32)
        _check(self.lib.sayaka_tree_get_face_regs(self.h, L, regs.ctypes.data_as(_i32p)), "get_face_regs")
        return regs[:len(blocks) * 2 * self.ndim * 9].copy()


def tables_struct(tb):
    """TreeTables ctypes struct over a dict of numpy tables (keeps references)."""
    keep = {}
    t = TreeTables()
    t.ndim, t.nb, t.num_blocks = int(tb["ndim"]), int(tb["nb"]), int(tb["num_blocks"])
    t.min_level, t.max_level = int(tb["min_level"]), int(tb["max_level"])
    for k in ("level", "neighbor", "child", "parent", "which_child", "node_type"):
        a, p = _i32(tb[k])
        keep[k] = a
        setattr(t, k, p)
    a, p = _f64(tb["block_len"])
    keep["block_len"] = a
    t.block_len = p
    return t, keep


class MacSolver:
    """GPU MAC solver (sayaka::MacSolver of src/SayakaMacSolver.h)."""

    def __init__(self, tables):
        self.lib = load_library()
        if isinstance(tables, AmrTree):
            tables = tables.tables()
        self.tb = tables
        self.ndim, self.nb, self.num_blocks = int(tables["ndim"]), int(tables["nb"]), int(tables["num_blocks"])
        self.ncell = self.nb ** self.ndim
        self.nfb = (self.nb + 1) * self.nb ** (self.ndim - 1)
        t, self._keep = tables_struct(tables)
        h = C.c_void_p()
        rc = self.lib.sayaka_mac_create(C.byref(t), C.byref(h))
        _check(rc, "mac_create")
        self.h = h
        self.params = self.default_params()

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.sayaka_mac_destroy(self.h)
            self.h = None

    # --- configuration ---
    def default_params(self):
        p = Params()
        self.lib.sayaka_params_default(C.byref(p))
        return p

    def set_params(self, **kw):
        for k, v in kw.items():
            setattr(self.params, k, v)
        _check(self.lib.sayaka_mac_set_params(self.h, C.byref(self.params)), "set_params", self.h)

    def set_scalars(self, alpha, beta):
        _check(self.lib.sayaka_mac_set_scalars(self.h, alpha, beta), "set_scalars", self.h)

    def set_coef_b(self, d, face, ncomp=1, ngrow=0, comp=0):
        a, p = _f64(face)
        _check(self.lib.sayaka_mac_set_coef_b(self.h, d, p, ncomp, ngrow, comp), "set_coef_b", self.h)

    def set_ib_frac_by_ls(self, ls, ncomp=1, ngrow=1, comp=0):
        a, p = _f64(ls)
        _check(self.lib.sayaka_mac_set_ib_frac_by_ls(self.h, p, ncomp, ngrow, comp), "set_ib_frac_by_ls", self.h)

    def set_ib_frac_by_ls_device(self, ptr, ngrow=1):
        """binary fractions from a level set already on the device: ptr is the
        device address of every block's grown box (one component)"""
        _check(self.lib.sayaka_mac_set_ib_frac_by_ls_compact(self.h, C.c_void_p(int(ptr)), int(ngrow), 1),
               "set_ib_frac_by_ls", self.h)

    def set_rhs_device(self, ptr):
        """the right-hand side from device memory (compact, all blocks)"""
        _check(self.lib.sayaka_mac_set_rhs_compact(self.h, C.c_void_p(int(ptr)), 1), "set_rhs", self.h)

    def set_ib_frac_compact(self, vol, areas):
        v, pv = _f64(vol)
        arrs = [_f64(a) for a in areas] + [(None, None)] * (3 - len(areas))
        _check(self.lib.sayaka_mac_set_ib_frac_compact(self.h, pv, arrs[0][1], arrs[1][1], arrs[2][1]),
               "set_ib_frac", self.h)

    def set_bc(self, bc_type):
        a, p = _i32(bc_type)
        _check(self.lib.sayaka_mac_set_bc(self.h, p), "set_bc", self.h)

    def fix_bc(self, phi, rhs, phi_ncomp=1, phi_ngrow=1, phi_comp=0, rhs_ncomp=1, rhs_ngrow=0, rhs_comp=0):
        a, pa = _f64(phi)
        rhs_arr = np.ascontiguousarray(rhs, dtype=np.float64)
        _check(self.lib.sayaka_mac_fix_bc(self.h, pa, phi_ncomp, phi_ngrow, phi_comp,
                                          rhs_arr.ctypes.data_as(_f64p), rhs_ncomp, rhs_ngrow, rhs_comp),
               "fix_bc", self.h)
        return rhs_arr

    # --- vectors ---
    def set_rhs(self, data, ncomp=1, ngrow=0, comp=0):
        a, p = _f64(data)
        _check(self.lib.sayaka_mac_set_rhs(self.h, p, ncomp, ngrow, comp), "set_rhs", self.h)

    def set_init_sol(self, data, ncomp=1, ngrow=0, comp=0):
        a, p = _f64(data)
        _check(self.lib.sayaka_mac_set_init_sol(self.h, p, ncomp, ngrow, comp), "set_init_sol", self.h)

    def set_zero_sol(self):
        _check(self.lib.sayaka_mac_set_zero_sol(self.h), "set_zero_sol", self.h)

    def get_sol(self, out=None, ncomp=1, ngrow=0, comp=0):
        if out is None:
            G = self.nb + 2 * ngrow
            out = np.zeros(self.num_blocks * ncomp * G ** self.ndim)
        _check(self.lib.sayaka_mac_get_sol(self.h, out.ctypes.data_as(_f64p), ncomp, ngrow, comp), "get_sol",
               self.h)
        return out

    def set_rhs_compact(self, cells):
        a, p = _f64(cells)
        _check(self.lib.sayaka_mac_set_rhs_compact(self.h, C.c_void_p(a.ctypes.data), 0), "set_rhs", self.h)

    def get_sol_compact(self):
        out = np.zeros(self.num_blocks * self.ncell)
        _check(self.lib.sayaka_mac_get_sol_compact(self.h, C.c_void_p(out.ctypes.data), 0), "get_sol", self.h)
        return out

    def mg_solve(self):
        """stand-alone V-cycles (MacSolver::mg_solve)"""
        return self._solve(self.lib.sayaka_mac_mg_solve, "mg_solve")

    def relax_solve(self):
        """Gauss-Seidel sweeps of the finest tower (MacSolver::relax_solve)"""
        return self._solve(self.lib.sayaka_mac_relax_solve, "relax_solve")

    def _solve(self, fn, what):
        info = SolveInfo()
        rc = fn(self.h, C.byref(info))
        if rc not in (OK, BREAKDOWN, NOT_CONVERGED):
            _check(rc, what, self.h)
        return dict(status=info.status, iterations=info.iterations, rnorm0=info.rnorm0, rnorm=info.rnorm,
                    seconds=info.seconds, rc=rc)

    def cg_solve(self):
        info = SolveInfo()
        rc = self.lib.sayaka_mac_cg_solve(self.h, C.byref(info))
        if rc not in (OK, BREAKDOWN, NOT_CONVERGED):
            _check(rc, "cg_solve", self.h)
        return dict(status=info.status, iterations=info.iterations, rnorm0=info.rnorm0, rnorm=info.rnorm,
                    seconds=info.seconds, rc=rc)

    # --- device-resident path ---
    def prepare(self):
        _check(self.lib.sayaka_mac_prepare(self.h), "prepare", self.h)

    def cg_solve_async(self):
        _check(self.lib.sayaka_mac_cg_solve_async(self.h), "cg_solve_async", self.h)

    def solve_info(self):
        info = SolveInfo()
        _check(self.lib.sayaka_mac_solve_info(self.h, C.byref(info)), "solve_info", self.h)
        return dict(status=info.status, iterations=info.iterations, rnorm0=info.rnorm0, rnorm=info.rnorm)

    def stream(self):
        return self.lib.sayaka_mac_stream(self.h)

    def enqueue_kernel(self, which, L):
        _check(self.lib.sayaka_mac_enqueue_kernel(self.h, int(which), int(L)), "enqueue_kernel", self.h)

    def launch_counts(self):
        a, b, c = C.c_int32(), C.c_int32(), C.c_int32()
        _check(self.lib.sayaka_mac_launch_counts(self.h, C.byref(a), C.byref(b), C.byref(c)), "launch_counts",
               self.h)
        return a.value, b.value, c.value

    # --- learned block correction ---
    def learned_collect(self, max_iter=200, max_samples=0):
        n = C.c_int32()
        _check(self.lib.sayaka_mac_learned_collect_sampled(self.h, int(max_iter), int(max_samples), C.byref(n)),
               "learned_collect", self.h)
        return n.value

    def learned_train_on_workload(self, max_samples=40000, epochs=10, lr=1e-3, batch=256, seed=1):
        """training pairs from this solver's own plain solve of its current
        right-hand side (at most max_samples blocks), then Adam on the GPU;
        the right-hand side and a zero solution are left in place"""
        its = self.learned_collect(200, max_samples)
        first = self.learned_train(epochs=1, lr=lr, batch=batch, seed=seed)
        last = self.learned_train(epochs=max(0, epochs - 1), lr=lr, batch=batch, seed=seed + 1)
        return dict(iterates=its, loss_first_epoch=first, loss_last_epoch=last, epochs=epochs,
                    max_samples=max_samples)

    def learned_train(self, epochs=20, lr=1e-3, batch=256, seed=1):
        loss = C.c_float()
        _check(self.lib.sayaka_mac_learned_train(self.h, int(epochs), float(lr), int(batch), int(seed),
                                                 C.byref(loss)), "learned_train", self.h)
        return loss.value

    def learned_eval(self):
        """mean loss of the collected pairs under the current weights (no training)"""
        loss = C.c_float()
        _check(self.lib.sayaka_mac_learned_eval(self.h, C.byref(loss)), "learned_eval", self.h)
        return loss.value

    def learned_weights(self):
        n = self.lib.sayaka_mac_learned_nparam()
        w = np.zeros(n, dtype=np.float32)
        _check(self.lib.sayaka_mac_learned_get_weights(self.h, w.ctypes.data_as(_f32p), n), "learned_weights",
               self.h)
        return w

    def set_learned_weights(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        _check(self.lib.sayaka_mac_learned_set_weights(self.h, w.ctypes.data_as(_f32p), w.size),
               "set_learned_weights", self.h)

    def learned_loss_grad(self, feat, aux):
        feat, aux = (np.ascontiguousarray(a, dtype=np.float32) for a in (feat, aux))
        n = feat.shape[0]
        g = np.zeros(self.lib.sayaka_mac_learned_nparam(), dtype=np.float32)
        loss = C.c_float()
        _check(self.lib.sayaka_mac_learned_loss_grad(self.h, feat.ctypes.data_as(_f32p), aux.ctypes.data_as(_f32p),
                                                     n, g.ctypes.data_as(_f32p), C.byref(loss)),
               "learned_loss_grad", self.h)
        return loss.value, g

    def learned_forward(self, feat):
        feat = np.ascontiguousarray(feat, dtype=np.float32)
        n = feat.shape[0]
        y = np.zeros((n, feat.shape[-1]), dtype=np.float32)
        _check(self.lib.sayaka_mac_learned_forward(self.h, feat.ctypes.data_as(_f32p), n, y.ctypes.data_as(_f32p)),
               "learned_forward", self.h)
        return y

    # --- projection step around the solve ---
    def set_rhs_div(self, u, scale, ncomp=1, ngrow=0, ucomp=0, wcomp=-1):
        """rhs = sum_d (scale/dh_d) (u_d(i+1) - u_d(i)) from face TreeData
        buffers u[d] (optionally weighted by component wcomp)"""
        keep = [np.ascontiguousarray(a, dtype=np.float64) for a in u]
        arr = (_f64p * 3)(*[k.ctypes.data_as(_f64p) for k in keep] + [None] * (3 - len(keep)))
        _check(self.lib.sayaka_mac_set_rhs_div(self.h, arr, ncomp, ngrow, ucomp, wcomp, float(scale)),
               "set_rhs_div", self.h)

    def correct_vel(self, d, dt, u, ncomp=1, ngrow=0, comp=0):
        """u_d += dt * flux of the solution on the finest tower, in place"""
        assert u.dtype == np.float64 and u.flags.c_contiguous
        _check(self.lib.sayaka_mac_correct_vel(self.h, int(d), float(dt), u.ctypes.data_as(_f64p), ncomp, ngrow,
                                               comp), "correct_vel", self.h)

    def init_from(self, old, prolong="injection", bc_val=None):
        """the solution of `old` (the solver of the tree before a regrid) as
        this solver's initial solution: prolong "injection" (copy, injection
        from the nearest old leaf ancestor, average of old children) or
        "centered_linear" (the reference's initNewBlockDataAfterRegrid after an
        average-down, with the BC values bc_val[face position], default 0)"""
        if prolong == "injection":
            _check(self.lib.sayaka_mac_init_from(self.h, old.h), "init_from", self.h)
        elif prolong == "centered_linear":
            v = None
            if bc_val is not None:
                v = np.zeros(6)
                b = np.asarray(bc_val, dtype=np.float64).reshape(-1)
                v[:b.size] = b  # one value per face position (2 * ndim), the rest unused
            _check(self.lib.sayaka_mac_init_new_block_data(self.h, old.h, None if v is None else v.ctypes.data_as(_f64p)),
                   "init_new_block_data", self.h)
        else:
            raise ValueError("prolong must be 'injection' or 'centered_linear'")

    def get_rhs_compact(self):
        r = self._cells()
        _check(self.lib.sayaka_mac_get_rhs_compact(self.h, r.ctypes.data_as(_f64p)), "get_rhs", self.h)
        return r

    def tuned_smoother(self, precision):
        """(chosen variant, microseconds per variant) of the smoother autotuner"""
        us = (C.c_float * 16)()
        v = self.lib.sayaka_mac_tuned_smoother(self.h, int(precision), us, 16)
        n = int(self.lib.sayaka_smoother_variants())
        return int(v), [float(x) for x in us][:n]

    def problem_count(self):
        """independent problems (connected components) of the tree"""
        return self.lib.sayaka_mac_problem_count(self.h)

    def problem_states(self):
        """per-problem (iterations, relative residual) of the last device solve
        with one state per problem, or None"""
        n = self.problem_count()
        it = np.zeros(max(n, 1), dtype=np.int32)
        rr = np.zeros(max(n, 1))
        r = self.lib.sayaka_mac_problem_states(self.h, it.ctypes.data_as(_i32p), rr.ctypes.data_as(_f64p), n)
        return None if r < 0 else (it[:r], rr[:r])

    def uniform_blocks(self):
        """constant-coefficient blocks of the tree (prepares the device solve)"""
        n = self.lib.sayaka_mac_uniform_blocks(self.h)
        if n < 0:
            _check(CUDA_ERROR, "uniform_blocks", self.h)
        return n

    def bottom_level(self):
        """level of the device solve's dense bottom solve (-1 before prepare)"""
        return int(self.lib.sayaka_mac_bottom_level(self.h))

    def tower_size(self, L, sublevel=0):
        return self.lib.sayaka_mac_tower_size(self.h, int(L), int(sublevel))

    # --- parity hooks (compact arrays over all blocks) ---
    def _cells(self):
        return np.zeros(self.num_blocks * self.ncell)

    def apply(self, L, x):
        y = self._cells()
        a, p = _f64(x)
        _check(self.lib.sayaka_mac_apply_compact(self.h, int(L), p, y.ctypes.data_as(_f64p)), "apply", self.h)
        return y

    def residual(self, L, x, rhs):
        r = self._cells()
        a, pa = _f64(x)
        b, pb = _f64(rhs)
        _check(self.lib.sayaka_mac_residual_compact(self.h, L, pa, pb, r.ctypes.data_as(_f64p)), "residual",
               self.h)
        return r

    def smooth(self, L, phi, rhs):
        out = self._cells()
        a, pa = _f64(phi)
        b, pb = _f64(rhs)
        _check(self.lib.sayaka_mac_smooth_compact(self.h, L, pa, pb, out.ctypes.data_as(_f64p)), "smooth", self.h)
        return out

    def device_apply(self, x):
        """the device solve's FP64 operator on the finest tower"""
        y = self._cells()
        a, pa = _f64(x)
        _check(self.lib.sayaka_mac_device_kernel_compact(self.h, 0, 0, -1, pa, None, y.ctypes.data_as(_f64p)),
               "device_apply", self.h)
        return y

    def device_apply_f32(self, x):
        """the BiCGSTAB iteration's operator on x rounded to FP32 (the
        double-float path that reads the FP32 V-cycle's output)"""
        y = self._cells()
        a, pa = _f64(x)
        _check(self.lib.sayaka_mac_device_kernel_compact(self.h, 3, 0, -1, pa, None, y.ctypes.data_as(_f64p)),
               "device_apply_f32", self.h)
        return y

    def device_smooth(self, L, phi, rhs, variant=-1):
        """one smoothing pass of tower L by the device solve's FP64 sweep"""
        out = self._cells()
        a, pa = _f64(phi)
        b, pb = _f64(rhs)
        _check(self.lib.sayaka_mac_device_kernel_compact(self.h, 1, int(L), int(variant), pa, pb,
                                                         out.ctypes.data_as(_f64p)), "device_smooth", self.h)
        return out

    def device_hybrid_pass(self, L, phi, rhs, sweeps):
        """one block-hybrid smoothing pass of tower L (FP64), `sweeps`
        red-black sweeps per block, values outside each block frozen"""
        out = self._cells()
        a, pa = _f64(phi)
        b, pb = _f64(rhs)
        _check(self.lib.sayaka_mac_device_kernel_compact(self.h, 2, int(L), int(sweeps), pa, pb,
                                                         out.ctypes.data_as(_f64p)), "device_hybrid_pass", self.h)
        return out

    def restrict_sweep(self, x):
        out = self._cells()
        a, pa = _f64(x)
        _check(self.lib.sayaka_mac_restrict_compact(self.h, pa, out.ctypes.data_as(_f64p)), "restrict", self.h)
        return out

    def prolong_sweep(self, x):
        out = self._cells()
        a, pa = _f64(x)
        _check(self.lib.sayaka_mac_prolong_compact(self.h, pa, out.ctypes.data_as(_f64p)), "prolong", self.h)
        return out

    def vcycle(self, p):
        out = self._cells()
        a, pa = _f64(p)
        _check(self.lib.sayaka_mac_vcycle_compact(self.h, pa, out.ctypes.data_as(_f64p)), "vcycle", self.h)
        return out

    def flux_compact(self, d, phi):
        out = np.zeros(self.num_blocks * self.nfb)
        a, pa = _f64(phi)
        _check(self.lib.sayaka_mac_flux_compact(self.h, d, pa, out.ctypes.data_as(_f64p)), "flux", self.h)
        return out

    def fix_bc_compact(self, phi_grown, ngrow, rhs):
        a, pa = _f64(phi_grown)
        r = np.ascontiguousarray(rhs, dtype=np.float64).copy()
        _check(self.lib.sayaka_mac_fix_bc_compact(self.h, pa, ngrow, r.ctypes.data_as(_f64p)), "fix_bc", self.h)
        return r

    def get_coef(self, which, d=0):
        n = self.num_blocks * (self.ncell if which == 2 else self.nfb)
        out = np.zeros(n)
        _check(self.lib.sayaka_mac_get_coef_compact(self.h, which, d, out.ctypes.data_as(_f64p)), "get_coef",
               self.h)
        return out
