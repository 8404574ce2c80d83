"""The SIMT contribution update of one front, C -= L21 (L21 D)^T on the lower
triangle (spral_ssids_gpu_contrib_update, the kernel the numeric
factorisation runs for fronts below the tensor-core crossover), against an
FP64 product on the host: partial tiles, depths that span several 32-column
batches or end inside one, diagonal tiles, repeated application."""
import ctypes

import numpy as np
import pytest

from spral_gb300 import _native


def _front(cm, k, dbl, seed):
    rng = np.random.default_rng(seed)
    dt = np.float64 if dbl else np.float32
    ld = cm + k + 3  # a leading dimension above the minimum
    L = rng.standard_normal((ld, k)).astype(dt)
    LD = rng.standard_normal((cm, k)).astype(dt)
    C = rng.standard_normal((cm, cm)).astype(dt)
    return ld, L, LD, C


def _call(torch, dbl, ld, L, LD, C, cm, k, reps):
    dL = torch.tensor(L.ravel(order="F"), device="cuda")
    dLD = torch.tensor(LD.ravel(order="F"), device="cuda")
    dC = torch.tensor(C.ravel(order="F"), device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = _native.lib().spral_ssids_gpu_contrib_update(dbl, dL.data_ptr(), ld, dLD.data_ptr(),
                                                      dC.data_ptr(), cm, k, reps, stream)
    assert rc == 0
    return dC.cpu().numpy().reshape(cm, cm, order="F")


@pytest.mark.gpu
@pytest.mark.parametrize("dbl", [0, 1])
@pytest.mark.parametrize("cm,k", [(1, 1), (63, 31), (64, 32), (65, 33), (200, 64),
                                  (130, 100), (1000, 32), (517, 7)])
def test_contrib_update_matches_fp64(dbl, cm, k):
    torch = pytest.importorskip("torch")
    ld, L, LD, C = _front(cm, k, dbl, 100 * cm + k + dbl)
    got = _call(torch, dbl, ld, L, LD, C, cm, k, 1)
    ref = C.astype(np.float64) - L[k:k + cm, :].astype(np.float64) @ LD.astype(np.float64).T
    low = np.tril(np.ones((cm, cm), dtype=bool))
    assert np.array_equal(got[~low], C[~low])  # strict upper part never written
    # N(0,1) data: each entry is a sum of k products of size ~sqrt(k)
    tol = (1e-13 if dbl else 4e-6) * k
    assert np.abs(got[low] - ref[low]).max() <= tol


@pytest.mark.gpu
@pytest.mark.parametrize("dbl", [0, 1])
def test_contrib_update_repeats_and_is_deterministic(dbl):
    torch = pytest.importorskip("torch")
    cm, k = 700, 45
    ld, L, LD, C = _front(cm, k, dbl, 7 + dbl)
    a = _call(torch, dbl, ld, L, LD, C, cm, k, 3)
    b = _call(torch, dbl, ld, L, LD, C, cm, k, 3)
    assert np.array_equal(a, b)
    ref = C.astype(np.float64) - 3 * (L[k:k + cm, :].astype(np.float64)
                                      @ LD.astype(np.float64).T)
    low = np.tril(np.ones((cm, cm), dtype=bool))
    assert np.abs(a[low] - ref[low]).max() <= (1e-12 if dbl else 5e-5) * k


def test_contrib_update_rejects_bad_arguments():
    """Argument checks return before any CUDA call (no GPU needed)."""
    lib = _native.lib()
    f = lib.spral_ssids_gpu_contrib_update
    buf = (ctypes.c_double * 4)()
    p = ctypes.cast(buf, ctypes.c_void_p).value
    assert f(1, p, 4, p, p, 2, 2, 0, None) == -1   # reps < 1
    assert f(1, p, 3, p, p, 2, 2, 1, None) == -1   # ld < cm + k
    assert f(1, None, 4, p, p, 2, 2, 1, None) == -1
    assert f(1, p, 4, p, p, -1, 2, 1, None) == -1
    assert f(0, p, 4, p, p, 0, 2, 1, None) == 0    # empty update: nothing to do
