"""Python mirror of the SSIDS user interface for the GB300 numeric path.

Mirrors ``spral_ssids`` (src/ssids/ssids.f90:51-84; C API
include/spral_ssids.h:69-127): ``analyse`` -> akeep, ``factor`` -> fkeep +
inform, ``solve`` with the same ``job`` codes, ``enquire_indef`` and
``alter``.  Inputs are 0-based lower-triangle CSC arrays (the reference's
``array_base = 0`` convention of the C API).

The numeric phase runs entirely on the GPU through the C-ABI declared in
``include/spral_ssids_gpu.h`` (the drop-in for the GPU subtree of
src/ssids/gpu/subtree.f90).  There is no CPU fallback: without a CUDA device
or without the native library, ``factor`` raises.
"""
import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _native
from ._native import CpuFactorOptions, GpuOptions, ThreadStats

# SSIDS flags (src/ssids/datatypes.f90:25-59)
SSIDS_SUCCESS = 0
SSIDS_ERROR_SINGULAR = -5
SSIDS_ERROR_NOT_POS_DEF = -6
SSIDS_ERROR_JOB_OOR = -14
SSIDS_ERROR_ALLOCATION = -50
SSIDS_ERROR_CUDA_UNKNOWN = -51
SSIDS_WARNING_FACT_SINGULAR = 7

PRECISION_FP64 = 0
PRECISION_MIXED = 1


def _P(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


@dataclass
class Options:
    """Subset of ``ssids_options`` (src/ssids/datatypes.f90:188-284) used by
    the numeric phase, plus the GPU path's out-of-band knobs."""
    print_level: int = 0
    action: bool = True
    small: float = 1e-20
    u: float = 0.01
    nemin: int = 32
    pivot_method: int = 2          # 2 = app_block, 3 = tpp
    failed_pivot_method: int = 1   # 1 = tpp, 2 = pass
    # GPU path only
    precision: int = PRECISION_FP64
    max_refine: int = 10
    refine_tol: float = 1e-15
    small_front_cols: int = 0      # 0 = library default
    fp64_fallback: bool = True     # FP32 factors that cannot reach refine_tol: refactor in FP64

    def cpu_options(self):
        return CpuFactorOptions(print_level=self.print_level, action=self.action, small=self.small,
                                u=self.u, multiplier=1.1, small_subtree_threshold=4 * 10 ** 6,
                                cpu_block_size=256, pivot_method=self.pivot_method,
                                failed_pivot_method=self.failed_pivot_method)

    def gpu_options(self):
        g = GpuOptions()
        g.precision = self.precision
        g.max_refine = self.max_refine
        g.refine_tol = self.refine_tol
        g.small_front_cols = self.small_front_cols
        g.use_graph = 0
        g.no_fp64_fallback = 0 if self.fp64_fallback else 1
        return g


@dataclass
class Inform:
    """Subset of ``ssids_inform`` (src/ssids/inform.f90:17-50)."""
    flag: int = 0
    matrix_rank: int = 0
    maxfront: int = 0
    maxsupernode: int = 0
    num_delay: int = 0
    num_factor: int = 0
    num_flops: int = 0
    num_neg: int = 0
    num_sup: int = 0
    num_two: int = 0
    not_first_pass: int = 0
    not_second_pass: int = 0
    cuda_error: int = 0
    extra: dict = field(default_factory=dict)


class Akeep:
    """Result of analyse: the 1-based arrays the numeric subtree consumes
    (sptr, sparent, rptr, rlist, nptr, nlist) and the pivot order."""

    def __init__(self, n, ptr, row, order, nemin):
        L = _native.lib()
        ptr = np.ascontiguousarray(ptr, dtype=np.int64)
        row = np.ascontiguousarray(row, dtype=np.int32)
        order = None if order is None else np.ascontiguousarray(order, dtype=np.int32)
        info = ctypes.c_int(0)
        h = L.spral_gb300_analyse(n, _P(ptr), _P(row), _P(order), nemin, ctypes.byref(info))
        if not h:
            raise RuntimeError(f"analyse failed, flag {info.value}")
        sizes = np.zeros(8, dtype=np.int64)
        L.spral_gb300_akeep_sizes(h, _P(sizes))
        self.n, self.nnodes = int(sizes[0]), int(sizes[1])
        self.nfact, self.nflops = int(sizes[4]), int(sizes[5])
        self.maxfront, self.maxsupernode = int(sizes[6]), int(sizes[7])
        self.sptr = np.zeros(self.nnodes + 1, dtype=np.int32)
        self.sparent = np.zeros(self.nnodes, dtype=np.int32)
        self.rptr = np.zeros(self.nnodes + 1, dtype=np.int64)
        self.rlist = np.zeros(int(sizes[2]), dtype=np.int32)
        self.nptr = np.zeros(self.nnodes + 1, dtype=np.int64)
        self.nlist = np.zeros(2 * int(sizes[3]), dtype=np.int64)
        self.invp = np.zeros(self.n, dtype=np.int32)
        L.spral_gb300_akeep_arrays(h, _P(self.sptr), _P(self.sparent), _P(self.rptr),
                                   _P(self.rlist), _P(self.nptr), _P(self.nlist), _P(self.invp))
        L.spral_gb300_akeep_free(h)
        self.nnz = int(ptr[-1])
        self.ptr = ptr
        self.row = row

    def front_sizes(self):
        """(nrow, ncol) per node, before delays."""
        return np.diff(self.rptr).astype(np.int64), np.diff(self.sptr).astype(np.int64)


def order_mindeg(ptr, row):
    """Minimum-degree ordering (order[i] = pivot position of variable i)."""
    L = _native.lib()
    n = len(ptr) - 1
    ptr = np.ascontiguousarray(ptr, dtype=np.int64)
    row = np.ascontiguousarray(row, dtype=np.int32)
    order = np.zeros(n, dtype=np.int32)
    st = L.spral_gb300_order_mindeg(n, _P(ptr), _P(row), _P(order))
    if st != 0:
        raise MemoryError("order_mindeg")
    return order


def order_amd(ptr, row):
    """Approximate minimum-degree ordering (order[i] = pivot position of
    variable i) for general sparse matrices, e.g. KKT systems."""
    L = _native.lib()
    n = len(ptr) - 1
    ptr = np.ascontiguousarray(ptr, dtype=np.int64)
    row = np.ascontiguousarray(row, dtype=np.int32)
    order = np.zeros(n, dtype=np.int32)
    st = L.spral_gb300_order_amd(n, _P(ptr), _P(row), _P(order))
    if st != 0:
        raise RuntimeError(f"order_amd failed ({st})")
    return order


def analyse(ptr, row, order=None, options=None):
    """Symbolic analyse (ssids_analyse, src/ssids/ssids.f90:148), host-side."""
    options = options or Options()
    n = len(ptr) - 1
    return Akeep(n, ptr, row, order, options.nemin)


def device_count():
    return _native.lib().spral_ssids_gpu_device_count()


class Fkeep:
    """Numeric factors on the GPU (the drop-in for ssids_factor with
    options%use_gpu; src/ssids/ssids.f90:767).  Solves take right-hand sides
    in the user's variable order."""

    def __init__(self, akeep, val, options=None, posdef=False, scaling=None):
        """scaling: optional symmetric scaling s (user variable order); the
        factors are those of S A S with S = diag(s), and solves scale the
        right-hand side and the solution as inner_solve_cpu does
        (src/ssids/fkeep.F90:249-315)."""
        L = _native.lib()
        if L.spral_ssids_gpu_device_count() < 1:
            raise RuntimeError("spral_gb300: no CUDA device; the numeric path has no CPU fallback")
        self.akeep = akeep
        self.options = options or Options()
        self.posdef = bool(posdef)
        a = akeep
        self._copts = self.options.cpu_options()
        self.sym = L.spral_ssids_gpu_create_symbolic_subtree(
            0, a.n, 1, a.nnodes + 1, _P(a.sptr), _P(a.sparent), _P(a.rptr), _P(a.rlist),
            _P(a.nptr), _P(a.nlist), ctypes.byref(self._copts))
        if not self.sym:
            raise RuntimeError("spral_gb300: symbolic setup failed")
        g = self.options.gpu_options()
        L.spral_ssids_gpu_set_options(self.sym, ctypes.byref(g))
        self.val = np.ascontiguousarray(val, dtype=np.float64)
        # the subtree takes the scaling in pivot order, as fkeep%scaling
        self.scaling = (None if scaling is None else
                        np.ascontiguousarray(np.asarray(scaling, dtype=np.float64)[a.invp]))
        st = ThreadStats()
        self.num = L.spral_ssids_gpu_create_num_subtree_dbl(
            self.posdef, self.sym, _P(self.val),
            None if self.scaling is None else _P(self.scaling), None,
            ctypes.byref(self._copts), ctypes.byref(st))
        self.stats = {k: getattr(st, k) for k, _ in ThreadStats._fields_}
        self.inform = self._inform(st)
        if not self.num:
            raise RuntimeError(f"spral_gb300: numeric setup failed, flag {st.flag}")

    def _inform(self, st):
        inf = Inform(flag=st.flag, maxfront=st.maxfront, maxsupernode=st.maxsupernode,
                     num_delay=st.num_delay, num_factor=st.num_factor, num_flops=st.num_flops,
                     num_neg=st.num_neg, num_sup=self.akeep.nnodes, num_two=st.num_two,
                     not_first_pass=st.not_first_pass, not_second_pass=st.not_second_pass)
        inf.matrix_rank = self.akeep.n - st.num_zero
        return inf

    def refactor(self, val, scaling=None):
        """Same-pattern refactorisation from host values (scaling in user
        variable order; default: the scaling given at construction)."""
        st = ThreadStats()
        self.val = np.ascontiguousarray(val, dtype=np.float64)
        if scaling is not None:
            self.scaling = np.ascontiguousarray(
                np.asarray(scaling, dtype=np.float64)[self.akeep.invp])
        sc = self.scaling
        fl = _native.lib().spral_ssids_gpu_refactor(self.num, _P(self.val),
                                                    None if sc is None else _P(sc),
                                                    ctypes.byref(st))
        self.stats = {k: getattr(st, k) for k, _ in ThreadStats._fields_}
        self.inform = self._inform(st)
        return fl

    def node_inertia(self):
        """(nnodes, 3) array: negative eigenvalues, 2x2 pivots and zero
        pivots of each node's D from the last factorisation."""
        out = np.zeros(3 * self.akeep.nnodes, dtype=np.int32)
        fl = _native.lib().spral_ssids_gpu_node_inertia(self.num, _P(out))
        if fl != 0:
            raise RuntimeError(f"spral_gb300 node_inertia failed, flag {fl}")
        return out.reshape(-1, 3)

    def refactor_dev(self, val_dev_ptr, stream=0):
        """Same-pattern refactorisation from a device pointer of values."""
        st = ThreadStats()
        fl = _native.lib().spral_ssids_gpu_refactor_dev(self.num, ctypes.c_void_p(val_dev_ptr),
                                                         ctypes.byref(st), ctypes.c_void_p(stream))
        self.stats = {k: getattr(st, k) for k, _ in ThreadStats._fields_}
        self.inform = self._inform(st)
        return fl

    def solve_dev(self, x_dev_ptr, nrhs, ldx, job=0, stream=0):
        """Solve with x (pivot order, FP64) already in device memory."""
        return _native.lib().spral_ssids_gpu_solve_dev(self.num, job, nrhs,
                                                        ctypes.c_void_p(x_dev_ptr), ldx,
                                                        ctypes.c_void_p(stream))

    def solve(self, b, job=0):
        """ssids_solve (src/ssids/ssids.f90:1140) job codes: 0 full, 1 fwd,
        2 diag, 3 bwd, 4 diag_bwd."""
        if job not in (0, 1, 2, 3, 4) or (self.posdef and job in (2, 4)):
            # posdef has no diagonal solve (src/ssids/ssids.f90:1234-1238)
            raise ValueError(f"job out of range (SSIDS_ERROR_JOB_OOR={SSIDS_ERROR_JOB_OOR})")
        L = _native.lib()
        b = np.asarray(b, dtype=np.float64)
        one = b.ndim == 1
        B = b[:, None] if one else b
        invp = self.akeep.invp
        xp = np.asfortranarray(B[invp, :])
        sc = self.scaling
        if sc is not None and job in (0, 1):  # x2 = S b (fkeep.F90:253-260)
            xp *= sc[:, None]
        nrhs, ldx = xp.shape[1], xp.shape[0]
        fns = {1: ["fwd"], 2: ["diag"], 3: ["bwd"], 4: ["diag_bwd"], 0: ["fwd", "diag_bwd"]}
        for nm in fns[job]:
            fl = getattr(L, f"spral_ssids_gpu_subtree_solve_{nm}_dbl")(self.posdef, self.num, nrhs,
                                                                       _P(xp), ldx)
            if fl != 0:
                raise RuntimeError(f"spral_gb300 solve failed, flag {fl}")
        if sc is not None and job in (0, 3, 4):  # x = S x2 (fkeep.F90:300-308)
            xp *= sc[:, None]
        x = np.empty_like(B)
        x[invp, :] = xp
        return x[:, 0] if one else x

    def solve_refined(self, b):
        """Full solve followed by FP64 iterative refinement on the device
        (against the unscaled matrix: not available with a scaling)."""
        if self.scaling is not None:
            raise ValueError("solve_refined refines against the unscaled matrix; "
                             "use solve() with a scaled factorisation")
        L = _native.lib()
        b = np.asarray(b, dtype=np.float64)
        one = b.ndim == 1
        B = b[:, None] if one else b
        invp = self.akeep.invp
        xp = np.asfortranarray(B[invp, :])
        it = ctypes.c_int(0)
        nfb = self.fallbacks
        fl = L.spral_ssids_gpu_solve_refined(self.num, xp.shape[1], _P(xp), xp.shape[0],
                                             ctypes.byref(it))
        if fl != 0:
            raise RuntimeError(f"spral_gb300 refined solve failed, flag {fl}")
        self.last_refine_iters = it.value
        if self.fallbacks != nfb:
            # FP32 factors could not reach the target: the solve was finished
            # with an FP64 factorisation, whose statistics now apply
            st = ThreadStats()
            L.spral_ssids_gpu_fp64_fallbacks(self.num, ctypes.byref(st))
            self.stats = {k: getattr(st, k) for k, _ in ThreadStats._fields_}
            self.inform = self._inform(st)
        x = np.empty_like(B)
        x[invp, :] = xp
        return x[:, 0] if one else x

    @property
    def fallbacks(self):
        """FP64 refactorisations the refined solves of an FP32-factor handle
        have taken (always 0 for FP64 factors)."""
        return _native.lib().spral_ssids_gpu_fp64_fallbacks(self.num, None)

    def enquire_posdef(self):
        """Diagonal entries of the Cholesky factor of a posdef factorisation,
        node by node in pivot order (ssids_enquire_posdef)."""
        if not self.posdef:
            raise ValueError("enquire_posdef needs a posdef factorisation")
        d = np.zeros(self.akeep.n, dtype=np.float64)
        _native.lib().spral_ssids_gpu_subtree_enquire_dbl(True, self.num, None, _P(d))
        return d

    def enquire_indef(self):
        """piv_order (indexed by pivot position, negative for 2x2) and d (n x 2),
        as the subtree's enquire (src/ssids/cpu/NumericSubtree.hxx:402-445)."""
        piv = np.zeros(self.akeep.n, dtype=np.int32)
        d = np.zeros(2 * self.akeep.n, dtype=np.float64)
        _native.lib().spral_ssids_gpu_subtree_enquire_dbl(self.posdef, self.num, _P(piv), _P(d))
        return piv, d.reshape(-1, 2)

    def alter(self, d):
        d = np.ascontiguousarray(d, dtype=np.float64).reshape(-1)
        _native.lib().spral_ssids_gpu_subtree_alter_dbl(self.posdef, self.num, _P(d))

    def front(self, node):
        """Diagnostics: one front of the factors (m, n, nelim, L, D, perm)."""
        info = np.zeros(5, dtype=np.int32)
        _native.lib().spral_ssids_gpu_debug_front(self.num, node, _P(info), None, None, None)
        m, n = int(info[0]), int(info[1])
        L = np.zeros((n, m))
        D = np.zeros(2 * n)
        perm = np.zeros(n, dtype=np.int32)
        _native.lib().spral_ssids_gpu_debug_front(self.num, node, _P(info), _P(L), _P(D), _P(perm))
        return dict(m=m, n=n, nelim=int(info[2]), ndin=int(info[3]), L=L.T.copy(), D=D, perm=perm)

    def timing(self):
        out = np.zeros(5, dtype=np.float64)
        _native.lib().spral_ssids_gpu_last_timing(self.num, _P(out))
        return out

    def free(self):
        L = _native._lib
        if L is None:
            return
        if getattr(self, "num", None):
            L.spral_ssids_gpu_destroy_num_subtree_dbl(self.posdef, self.num)
            self.num = None
        if getattr(self, "sym", None):
            L.spral_ssids_gpu_destroy_symbolic_subtree(self.sym)
            self.sym = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def factor(akeep, val, options=None, posdef=False):
    """ssids_factor on the GPU; returns (fkeep, inform)."""
    fk = Fkeep(akeep, val, options, posdef)
    return fk, fk.inform
