"""CPU tests of the host analyse restatement and the C-ABI library."""
import ctypes
import os
import re

import numpy as np

from spral_gb300 import _native, matrices as M, ssids

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_analyse_structure():
    p, r, v = M.laplacian_2d(24, 24, -0.5)
    ak = ssids.analyse(p, r, M.nd_order_grid(24, 24))
    n = ak.n
    assert sorted(ak.invp.tolist()) == list(range(n))
    # supernodes partition the pivots; rows start with the node's own pivots
    assert ak.sptr[0] == 1 and ak.sptr[-1] == n + 1
    for s in range(ak.nnodes):
        rows = ak.rlist[ak.rptr[s] - 1:ak.rptr[s + 1] - 1]
        assert np.all(np.diff(rows) > 0)
        own = np.arange(ak.sptr[s], ak.sptr[s + 1])
        assert np.array_equal(rows[:len(own)], own)
        par = ak.sparent[s]
        assert par > s + 1  # postordered tree (1-based)
        if par <= ak.nnodes:
            prow = set(ak.rlist[ak.rptr[par - 1] - 1:ak.rptr[par] - 1].tolist())
            assert set(rows[len(own):].tolist()) <= prow
    # every A entry mapped exactly once
    src = ak.nlist[0::2]
    assert np.array_equal(np.sort(src), np.arange(1, ak.nnz + 1))


def test_analyse_nemin_merges():
    p, r, v = M.laplacian_2d(32, 32)
    o = M.nd_order_grid(32, 32)
    a1 = ssids.analyse(p, r, o, ssids.Options(nemin=1))
    a32 = ssids.analyse(p, r, o)
    assert a32.nnodes < a1.nnodes
    assert a32.nflops >= a1.nflops


def test_mindeg_is_permutation():
    p, r, v = M.kkt(100, 40, seed=1)
    o = ssids.order_mindeg(p, r)
    assert sorted(o.tolist()) == list(range(len(p) - 1))


def test_library_exports_header_symbols():
    hdr = open(os.path.join(ROOT, "include", "spral_ssids_gpu.h")).read()
    names = re.findall(r"\b(spral_ssids_gpu_\w+)\s*\(", hdr)
    assert len(names) >= 14
    lib = ctypes.CDLL(_native.LIB_PATH)
    for nm in set(names):
        assert hasattr(lib, nm), nm


def test_no_cuda_device_raises_cleanly():
    if ssids.device_count() > 0:
        return
    p, r, v = M.laplacian_2d(4, 4)
    ak = ssids.analyse(p, r)
    try:
        ssids.factor(ak, v)
    except RuntimeError as e:
        assert "no CUDA device" in str(e)
    else:
        raise AssertionError("factor must fail loudly without a GPU")
