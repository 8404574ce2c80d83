"""Level schedule of the numeric factorisation (host logic, no GPU):
leaf-aligned levels (height above the leaves), root-aligned levels (depth
below the root, src/ssids/gpu/factor.f90:824-879, assign_nodes_to_levels,
with the small leaf subtrees kept leaf-aligned) and the choice between them
by APP block steps (root-aligned for at least 10% fewer)."""
import ctypes

import numpy as np
import pytest

from spral_gb300 import _native, matrices as M, ssids

P = ctypes.c_void_p


def _schedule(parent, ncol, small=None, align=0):
    L = _native.lib()
    nn = len(parent)
    parent = np.ascontiguousarray(parent, dtype=np.int32)
    ncol = np.ascontiguousarray(ncol, dtype=np.int32)
    sm = None if small is None else np.ascontiguousarray(small, dtype=np.int8)
    lev = np.zeros(max(nn, 1), dtype=np.int32)
    nlev = ctypes.c_int(0)
    steps = ctypes.c_int64(0)
    rc = L.spral_ssids_gpu_level_schedule(nn, parent.ctypes.data_as(P), ncol.ctypes.data_as(P),
                                          None if sm is None else sm.ctypes.data_as(P), align,
                                          lev.ctypes.data_as(P), ctypes.byref(nlev),
                                          ctypes.byref(steps))
    return rc, lev[:nn], nlev.value, steps.value


def _random_tree(rng, nn):
    """A random postordered forest: parent[i] > i or -1."""
    parent = np.full(nn, -1, dtype=np.int32)
    for i in range(nn - 1):
        if rng.random() < 0.95:
            parent[i] = rng.integers(i + 1, min(nn, i + 8))
    return parent


def _heights(parent):
    h = np.zeros(len(parent), dtype=int)
    for i in range(len(parent)):
        if parent[i] >= 0:
            h[parent[i]] = max(h[parent[i]], h[i] + 1)
    return h


def _small_subtrees(parent, nrow, ncol, thr):
    """The small-leaf-subtree rule of the symbolic build: flops below each
    node, then from every leaf up while below the threshold."""
    nn = len(parent)
    fl = np.zeros(nn + 1, dtype=np.int64)
    kids = [[] for _ in range(nn)]
    for i in range(nn):
        for k in range(ncol[i]):
            fl[i] += (nrow[i] - k) ** 2
        fl[parent[i] if parent[i] >= 0 else nn] += fl[i]
        if parent[i] >= 0:
            kids[parent[i]].append(i)
    small = np.zeros(nn, dtype=np.int8)
    i = 0
    while i < nn:
        if kids[i]:
            i += 1
            continue
        last, cur = i, i
        while cur >= 0 and fl[cur] < thr:
            last, cur = cur, parent[cur]
        if last == i:
            i += 1
            continue
        small[i:last + 1] = 1
        i = last + 1
    return small


@pytest.mark.parametrize("seed", range(6))
def test_schedules_are_valid(seed):
    rng = np.random.default_rng(seed)
    nn = int(rng.integers(1, 400))
    parent = _random_tree(rng, nn)
    ncol = rng.integers(1, 300, nn)
    small = (rng.random(nn) < 0.3).astype(np.int8)
    # small marks must be whole subtrees: close the marks downwards
    for i in range(nn - 1, -1, -1):
        if parent[i] >= 0 and small[parent[i]]:
            small[i] = 1
    h = _heights(parent)
    for align in (0, 1, 2):
        for sm in (None, small):
            rc, lev, nlev, steps = _schedule(parent, ncol, sm, align)
            assert rc in (0, 1)
            assert nlev == h.max() + 1
            assert lev.min() >= 0 and lev.max() < nlev
            for i in range(nn):
                if parent[i] >= 0:
                    assert lev[i] < lev[parent[i]], (align, i)
            if rc == 0:
                assert np.array_equal(lev, h)
            else:
                for i in range(nn):
                    if sm is not None and sm[i]:
                        assert lev[i] == h[i]
                    elif parent[i] < 0:
                        assert lev[i] == nlev - 1
                    else:
                        assert lev[i] == lev[parent[i]] - 1
    # root-aligned when it takes at least 10% fewer block steps
    _, _, _, s_leaf = _schedule(parent, ncol, small, 1)
    _, _, _, s_root = _schedule(parent, ncol, small, 2)
    rc, _, _, s = _schedule(parent, ncol, small, 0)
    assert rc == (1 if 10 * s_root <= 9 * s_leaf else 0)
    assert s == (s_root if rc else s_leaf)


def test_root_alignment_shares_levels_between_sibling_separators():
    # root 3 (64 columns) with two branches of different height: a leaf
    # separator 0 (96 columns) and a chain 1 -> 2 (96 and 32 columns)
    parent = [3, 2, 3, -1]
    ncol = [96, 96, 32, 64]
    rc_leaf, lev_leaf, _, s_leaf = _schedule(parent, ncol, None, 1)
    rc_root, lev_root, _, s_root = _schedule(parent, ncol, None, 2)
    assert list(lev_leaf) == [0, 0, 1, 2] and s_leaf == 3 + 1 + 2
    assert list(lev_root) == [1, 0, 1, 2] and s_root == 3 + 3 + 2
    rc, lev, _, s = _schedule(parent, ncol, None, 0)
    assert rc == 0 and s == s_leaf
    # a chain of one wide and one narrow separator on the other side
    parent = [2, 3, 3, -1]
    ncol = [32, 96, 96, 64]
    _, _, _, s_leaf = _schedule(parent, ncol, None, 1)
    rc, lev, _, s = _schedule(parent, ncol, None, 0)
    assert s_leaf == 3 + 3 + 2 and rc == 1 and s == 1 + 3 + 2 and list(lev) == [0, 1, 1, 2]


def test_lap3d48_tree_takes_root_alignment():
    k = 48
    p, r, _ = M.laplacian_3d(k, shift=-0.3)
    ak = ssids.analyse(p, r, M.nd_order_grid(k, k, k))
    nn = ak.nnodes
    ncol = np.diff(ak.sptr[:nn + 1]).astype(np.int64)
    nrow = np.diff(ak.rptr[:nn + 1]).astype(np.int64)
    par = ak.sparent[:nn].astype(np.int64) - 1
    par = np.where((par >= 0) & (par < nn), par, -1).astype(np.int32)
    small = _small_subtrees(par, nrow, ncol, 4000000)
    _, _, nl_leaf, s_leaf = _schedule(par, ncol, small, 1)
    rc, lev, nlev, s = _schedule(par, ncol, small, 0)
    assert nlev == nl_leaf == 20
    assert rc == 1 and s_leaf == 274 and s == 185


def test_bad_arguments():
    L = _native.lib()
    nlev = ctypes.c_int(0)
    lev = np.zeros(2, dtype=np.int32)
    ncol = np.ones(2, dtype=np.int32)
    bad = np.array([0, -1], dtype=np.int32)  # a node its own parent
    assert L.spral_ssids_gpu_level_schedule(2, bad.ctypes.data_as(P), ncol.ctypes.data_as(P),
                                            None, 0, lev.ctypes.data_as(P), ctypes.byref(nlev),
                                            None) == -1
    good = np.array([1, -1], dtype=np.int32)
    assert L.spral_ssids_gpu_level_schedule(2, good.ctypes.data_as(P), ncol.ctypes.data_as(P),
                                            None, 3, lev.ctypes.data_as(P), ctypes.byref(nlev),
                                            None) == -1
    assert L.spral_ssids_gpu_level_schedule(0, None, None, None, 0, None, ctypes.byref(nlev),
                                            None) == 0
    assert nlev.value == 0
