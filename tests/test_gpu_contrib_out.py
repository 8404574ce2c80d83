"""get_contrib of a subtree whose root has a parent outside it (the
generalised element the reference's GPU subtree hands to a CPU parent,
src/ssids/gpu/factor.f90:155-221): factor the subtree under each node of a
tree on its own and check what get_contrib returns against dense linear
algebra on the host.  With I' the subtree's eliminated variables, D the
root's delayed ones and B the root's rows beyond its columns (all in pivot
order):
  contribution block  C = -A[B,I'] A[I',I']^-1 A[I',B]
  delayed columns     S[X,d] = A[X,d] - A[X,I'] A[I',I']^-1 A[I',d], X = D + B
"""
import ctypes

import numpy as np
import pytest

from spral_gb300 import _native, matrices as M, ssids

pytestmark = pytest.mark.gpu

P = ctypes.c_void_p


def _dense_pivot_order(p, r, v, invp):
    n = len(p) - 1
    A = np.zeros((n, n))
    for j in range(n):
        for k in range(p[j], p[j + 1]):
            A[r[k], j] = v[k]
            A[j, r[k]] = v[k]
    return A[np.ix_(invp, invp)]


def _subtree_ranges(ak):
    """(sa, en) 1-based for the subtree under every node that has a parent
    and contribution rows (post-order: a subtree is a contiguous range)."""
    nn = ak.nnodes
    parent = ak.sparent[:nn] - 1
    first = np.arange(nn)
    for i in range(nn):  # children come before parents
        if parent[i] < nn:
            first[parent[i]] = min(first[parent[i]], first[i])
    nrow, ncol = ak.front_sizes()
    return [(int(first[i]) + 1, i + 2) for i in range(nn)
            if parent[i] < nn and nrow[i] > ncol[i]]


def _get_contrib(L, num):
    n, ld, nd, ldd = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    val, rl, dp, dv = P(), P(), P(), P()
    rc = L.spral_ssids_gpu_subtree_get_contrib_dbl(False, num, ctypes.byref(n), ctypes.byref(val),
                                                   ctypes.byref(ld), ctypes.byref(rl),
                                                   ctypes.byref(nd), ctypes.byref(dp),
                                                   ctypes.byref(dv), ctypes.byref(ldd))
    assert rc == 0
    n, nd, ldd = n.value, nd.value, ldd.value
    assert ld.value == n
    C = np.ctypeslib.as_array(ctypes.cast(val, ctypes.POINTER(ctypes.c_double)),
                              (n * n,)).reshape(n, n, order="F").copy() if n else None
    rows = np.ctypeslib.as_array(ctypes.cast(rl, ctypes.POINTER(ctypes.c_int)),
                                 (n,)).copy() if n else np.zeros(0, int)
    perm = dval = None
    if nd:
        assert ldd == n + nd
        perm = np.ctypeslib.as_array(ctypes.cast(dp, ctypes.POINTER(ctypes.c_int)), (nd,)).copy()
        dval = np.ctypeslib.as_array(ctypes.cast(dv, ctypes.POINTER(ctypes.c_double)),
                                     (ldd * nd,)).reshape(ldd, nd, order="F").copy()
    return C, rows, perm, dval


def _check_case(p, r, v, ak, precision, tol):
    L = _native.lib()
    A = _dense_pivot_order(p, r, v, ak.invp)
    opts = ssids.Options(precision=precision)
    copts = opts.cpu_options()
    g = opts.gpu_options()
    delays_seen = 0
    for sa, en in _subtree_ranges(ak):
        sym = L.spral_ssids_gpu_create_symbolic_subtree(
            0, ak.n, sa, en, ak.sptr.ctypes.data_as(P), ak.sparent.ctypes.data_as(P),
            ak.rptr.ctypes.data_as(P), ak.rlist.ctypes.data_as(P), ak.nptr.ctypes.data_as(P),
            ak.nlist.ctypes.data_as(P), ctypes.byref(copts))
        assert sym
        L.spral_ssids_gpu_set_options(sym, ctypes.byref(g))
        st = _native.ThreadStats()
        num = L.spral_ssids_gpu_create_num_subtree_dbl(False, sym, v.ctypes.data_as(P), None,
                                                       None, ctypes.byref(copts),
                                                       ctypes.byref(st))
        assert num and st.flag >= 0
        C, rows, perm, dval = _get_contrib(L, num)
        root = en - 2
        nr, nc = ak.front_sizes()
        Bv = ak.rlist[ak.rptr[root] - 1 + nc[root]:ak.rptr[root + 1] - 1] - 1
        assert np.array_equal(rows - 1, Bv)
        sub = np.concatenate([np.arange(ak.sptr[i] - 1, ak.sptr[i + 1] - 1)
                              for i in range(sa - 1, en - 1)])
        D = (perm - 1) if perm is not None else np.zeros(0, int)
        Ie = np.setdiff1d(sub, D)
        W = np.linalg.solve(A[np.ix_(Ie, Ie)], A[Ie, :])  # A[I',I']^-1 A[I',:]
        S = A - A[:, Ie] @ W                              # Schur complement of I'
        Cexp = -(A[np.ix_(Bv, Ie)] @ W[:, Bv])
        scale = 1.0 + np.abs(Cexp).max()
        assert np.abs(C - Cexp).max() <= tol * scale
        assert np.array_equal(C, C.T)
        if perm is not None:
            delays_seen += 1
            nd = len(D)
            X = np.concatenate([D, Bv])
            for i in range(nd):
                got = dval[i:, i]                     # from the diagonal down
                exp = S[X[i:], D[i]]
                assert np.abs(got - exp).max() <= tol * (1.0 + np.abs(exp).max())
        L.spral_ssids_gpu_subtree_free_contrib_dbl(False, num)
        L.spral_ssids_gpu_destroy_num_subtree_dbl(False, num)
        L.spral_ssids_gpu_destroy_symbolic_subtree(sym)
    return delays_seen


@pytest.mark.parametrize("precision,tol", [(ssids.PRECISION_FP64, 1e-10),
                                           (ssids.PRECISION_MIXED, 1e-4)])
def test_get_contrib_laplacian_subtrees(precision, tol):
    p, r, v = M.laplacian_2d(18, 18, -0.3)
    ak = ssids.analyse(p, r, M.nd_order_grid(18, 18))
    _check_case(p, r, v, ak, precision, tol)


def test_get_contrib_with_delayed_columns():
    p, r, v = M.random_indef(400, density=0.02, seed=11, diag_scale=0.01)
    ak = ssids.analyse(p, r, ssids.order_mindeg(p, r))
    # every node that delays has a parent, so some subtree root here delays
    assert _check_case(p, r, v, ak, ssids.PRECISION_FP64, 1e-8) > 0
