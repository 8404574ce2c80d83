"""ORACLE -- test infrastructure only (see ssids_oracle.c header).

Python access to
  * ``liboracle.so``: the C restatement of SSIDS's CPU numeric factor/solve;
  * ``_ref/libspral_cpu_ref.so``: the reference's own C++ CPU numeric core,
    compiled from its sources by ``make -C oracle ref`` where the reference
    source tree exists (never on the GPU host).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline arm use it.
"""
import ctypes
import glob
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libspral_cpu_ref.so")
REF_SRC = os.environ.get("SPRAL_REF_SRC", "/root/reference")


def build(with_ref=None):
    """Compile the restatement, and the reference's CPU core if its sources exist."""
    if with_ref is None:
        with_ref = os.path.isdir(os.path.join(REF_SRC, "src", "ssids", "cpu"))
    target = "ref" if with_ref else "all"
    subprocess.check_call(["make", "-s", "-C", HERE, target, f"REF={REF_SRC}",
                           f"-j{os.cpu_count() or 4}"])


def find_openblas():
    """(path, symbol prefix) of an OpenBLAS shipped with scipy or numpy, or (None, None)."""
    try:
        import scipy
        d = os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs")
        for p in sorted(glob.glob(os.path.join(d, "libscipy_openblas*.so"))):
            if "64_" not in os.path.basename(p):
                return os.path.abspath(p), "scipy_"
    except ImportError:
        pass
    return None, None


from spral_gb300._native import CpuFactorOptions, ThreadStats  # noqa: E402  (same layouts)

_olib = None
_rlib = None


def _P(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def oracle_lib():
    global _olib
    if _olib is None:
        if not os.path.exists(ORACLE_LIB):
            build(with_ref=False)
        _olib = ctypes.CDLL(ORACLE_LIB)
        L = _olib
        L.oracle_factor.restype = ctypes.c_void_p
        L.oracle_factor.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 7 + [
            ctypes.POINTER(CpuFactorOptions), ctypes.POINTER(ThreadStats)]
        L.oracle_solve.restype = ctypes.c_int
        L.oracle_solve.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                   ctypes.c_int]
        L.oracle_free.argtypes = [ctypes.c_void_p]
        L.oracle_node_info.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.oracle_enquire.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.oracle_node_data.argtypes = [ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 3
        L.oracle_set_blas.restype = ctypes.c_int
        L.oracle_set_blas.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
    return _olib


def ref_available():
    return os.path.exists(REF_LIB)


def ref_lib():
    global _rlib
    if _rlib is None:
        path, prefix = find_openblas()
        if path:
            os.environ.setdefault("SPRAL_REF_BLAS", path)
            os.environ.setdefault("SPRAL_REF_BLAS_PREFIX", prefix)
        _rlib = ctypes.CDLL(REF_LIB)
        L = _rlib
        vp = ctypes.c_void_p
        L.spral_ssids_cpu_create_symbolic_subtree.restype = vp
        L.spral_ssids_cpu_create_symbolic_subtree.argtypes = [
            ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, vp, vp, vp, vp, vp, ctypes.c_int, vp,
            ctypes.POINTER(CpuFactorOptions)]
        L.spral_ssids_cpu_destroy_symbolic_subtree.argtypes = [vp]
        L.spral_ssids_cpu_create_num_subtree_dbl.restype = vp
        L.spral_ssids_cpu_create_num_subtree_dbl.argtypes = [
            ctypes.c_bool, vp, vp, vp, vp, ctypes.POINTER(CpuFactorOptions),
            ctypes.POINTER(ThreadStats)]
        L.spral_ssids_cpu_destroy_num_subtree_dbl.argtypes = [ctypes.c_bool, vp]
        for nm in ("fwd", "diag", "diag_bwd", "bwd"):
            fn = getattr(L, f"spral_ssids_cpu_subtree_solve_{nm}_dbl")
            fn.restype = ctypes.c_int
            fn.argtypes = [ctypes.c_bool, vp, ctypes.c_int, vp, ctypes.c_int]
        L.spral_ssids_cpu_subtree_enquire_dbl.argtypes = [ctypes.c_bool, vp, vp, vp]
    return _rlib


def default_options(**kw):
    """SSIDS defaults (src/ssids/datatypes.f90:188-284)."""
    o = CpuFactorOptions(print_level=0, action=True, small=1e-20, u=0.01, multiplier=1.1,
                         small_subtree_threshold=4 * 10 ** 6, cpu_block_size=256,
                         pivot_method=2, failed_pivot_method=1)
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def _stats_dict(st):
    return {k: getattr(st, k) for k, _ in ThreadStats._fields_}


class _Base:
    def solve(self, b, job=0):
        """Solve with b in the user's variable order (n or n x nrhs)."""
        b = np.asarray(b, dtype=np.float64)
        one = b.ndim == 1
        B = b[:, None] if one else b
        invp = self.akeep.invp
        xp = np.asfortranarray(B[invp, :])
        self._solve_pivot_order(xp, job)
        x = np.empty_like(B)
        x[invp, :] = xp
        return x[:, 0] if one else x


class OracleFactor(_Base):
    """C restatement (liboracle.so)."""

    def __init__(self, akeep, val, options=None, blas=False):
        L = oracle_lib()
        if blas:
            path, prefix = find_openblas()
            if path:
                L.oracle_set_blas(path.encode(), (prefix + "dgemm_").encode())
        else:
            L.oracle_set_blas(None, None)
        self.akeep = akeep
        self.opts = options or default_options()
        self.val = np.ascontiguousarray(val, dtype=np.float64)
        st = ThreadStats()
        a = akeep
        self.h = L.oracle_factor(a.n, a.nnodes, _P(a.sptr), _P(a.sparent), _P(a.rptr), _P(a.rlist),
                                 _P(a.nptr), _P(a.nlist), _P(self.val), ctypes.byref(self.opts),
                                 ctypes.byref(st))
        self.stats = _stats_dict(st)

    def _solve_pivot_order(self, xp, job):
        oracle_lib().oracle_solve(self.h, job, xp.shape[1], _P(xp), xp.shape[0])

    def node_info(self):
        out = np.zeros((self.akeep.nnodes, 4), dtype=np.int32)
        tmp = np.zeros(4, dtype=np.int32)
        for i in range(self.akeep.nnodes):
            oracle_lib().oracle_node_info(self.h, i, _P(tmp))
            out[i] = tmp
        return out

    def front(self, node):
        m, n, nelim, ndin = self.node_info()[node]
        L = np.zeros((n, m))
        D = np.zeros(2 * n)
        perm = np.zeros(n, dtype=np.int32)
        oracle_lib().oracle_node_data(self.h, node, _P(L), _P(D), _P(perm))
        return dict(m=m, n=n, nelim=nelim, ndin=ndin, L=L.T.copy(), D=D, perm=perm)

    def enquire_indef(self):
        piv = np.zeros(self.akeep.n, dtype=np.int32)
        d = np.zeros(2 * self.akeep.n, dtype=np.float64)
        oracle_lib().oracle_enquire(self.h, _P(piv), _P(d))
        return piv, d.reshape(-1, 2)

    def __del__(self):
        if getattr(self, "h", None):
            oracle_lib().oracle_free(self.h)
            self.h = None


class RefFactor(_Base):
    """The reference's own CPU numeric subtree (compiled from its sources)."""

    def __init__(self, akeep, val, options=None):
        L = ref_lib()
        self.akeep = akeep
        self.opts = options or default_options()
        self.val = np.ascontiguousarray(val, dtype=np.float64)
        a = akeep
        self.sym = L.spral_ssids_cpu_create_symbolic_subtree(
            a.n, 1, a.nnodes + 1, _P(a.sptr), _P(a.sparent), _P(a.rptr), _P(a.rlist), _P(a.nptr),
            _P(a.nlist), 0, None, ctypes.byref(self.opts))
        st = ThreadStats()
        self.h = L.spral_ssids_cpu_create_num_subtree_dbl(False, self.sym, _P(self.val), None, None,
                                                          ctypes.byref(self.opts), ctypes.byref(st))
        self.stats = _stats_dict(st)

    def _solve_pivot_order(self, xp, job):
        L = ref_lib()
        nrhs, ldx = xp.shape[1], xp.shape[0]
        if job in (0, 1):
            L.spral_ssids_cpu_subtree_solve_fwd_dbl(False, self.h, nrhs, _P(xp), ldx)
        if job == 0 or job == 4:
            L.spral_ssids_cpu_subtree_solve_diag_bwd_dbl(False, self.h, nrhs, _P(xp), ldx)
        elif job == 2:
            L.spral_ssids_cpu_subtree_solve_diag_dbl(False, self.h, nrhs, _P(xp), ldx)
        elif job == 3:
            L.spral_ssids_cpu_subtree_solve_bwd_dbl(False, self.h, nrhs, _P(xp), ldx)

    def enquire_indef(self):
        piv = np.zeros(self.akeep.n, dtype=np.int32)
        d = np.zeros(2 * self.akeep.n, dtype=np.float64)
        ref_lib().spral_ssids_cpu_subtree_enquire_dbl(False, self.h, _P(piv), _P(d))
        return piv, d.reshape(-1, 2)

    def __del__(self):
        L = _rlib
        if L is None:
            return
        if getattr(self, "h", None):
            L.spral_ssids_cpu_destroy_num_subtree_dbl(False, self.h)
            self.h = None
        if getattr(self, "sym", None):
            L.spral_ssids_cpu_destroy_symbolic_subtree(self.sym)
            self.sym = None
