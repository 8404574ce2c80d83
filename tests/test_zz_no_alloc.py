"""The allocation-free dense front factorization against the allocating one.

spral_ssids_gpu_ldlt_app_factor_noalloc serves callers that cannot allocate
device memory while they factor (their memory belongs to another allocator,
their budget is fixed at load time, or cudaMalloc would stall a
latency-critical path); it works in a fixed scratch array inside the library.
Here it must reproduce spral_ssids_gpu_ldlt_app_factor on two calls in a row
(the second call sees whatever the first left in the shared array), and it
must refuse a front larger than the array serves.  This file is collected
last so that a run stopping at its first failure has run every other test.
"""
import ctypes

import numpy as np
import pytest

from dense_cases import cause_delays, gen_sym_indef

pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative, as the other dense factor comparisons


def _run(fn, a, m, n, torch, opts):
    lda = m
    a_d = torch.tensor(np.asfortranarray(a).ravel(order="F"), dtype=torch.float64, device="cuda")
    d_d = torch.zeros(2 * n + 2, dtype=torch.float64, device="cuda")
    p_d = torch.arange(n, dtype=torch.int32, device="cuda")
    upd = a_d.data_ptr() + 8 * (n * lda + n) if m > n else None
    ne = fn(m, n, ctypes.c_void_p(p_d.data_ptr()), ctypes.c_void_p(a_d.data_ptr()), lda,
            ctypes.c_void_p(d_d.data_ptr()), 1.0, ctypes.c_void_p(upd) if upd else None, lda,
            ctypes.byref(opts), None)
    torch.cuda.synchronize()
    return ne, a_d.cpu().numpy().reshape(m, m, order="F"), d_d.cpu().numpy(), p_d.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    from spral_gb300 import _native
    import oracle
    lib = _native.lib()
    opts = oracle.default_options()
    for seed, (m, n) in ((21, (700, 300)), (22, (250, 250))):
        rng = np.random.default_rng(seed)
        a = gen_sym_indef(m, rng)
        cause_delays(a, rng)
        ne1, l1, d1, p1 = _run(lib.spral_ssids_gpu_ldlt_app_factor, a, m, n, torch, opts)
        ne2, l2, d2, p2 = _run(lib.spral_ssids_gpu_ldlt_app_factor_noalloc, a, m, n, torch, opts)
        assert ne1 >= 0 and ne2 == ne1
        assert np.array_equal(p1, p2)
        fin = np.isfinite(d1)
        assert np.array_equal(fin, np.isfinite(d2))
        assert np.abs(d2[fin] - d1[fin]).max() <= TOL * max(np.abs(d1[fin]).max(), 1.0)
        low = np.tril(np.ones((m, m), dtype=bool))
        assert np.abs(l2[low] - l1[low]).max() <= TOL * max(np.abs(l1[low]).max(), 1.0)


def test_noalloc_leaves_device_memory_untouched():
    """After one warm-up call, a further call changes neither the device's
    free memory nor torch's allocations: nothing is allocated or freed."""
    torch = pytest.importorskip("torch")
    from spral_gb300 import _native
    import oracle
    lib = _native.lib()
    opts = oracle.default_options()
    m, n = 600, 200
    a = gen_sym_indef(m, np.random.default_rng(31))
    a_d = torch.tensor(np.asfortranarray(a).ravel(order="F"), dtype=torch.float64, device="cuda")
    a0 = a_d.clone()
    d_d = torch.zeros(2 * n + 2, dtype=torch.float64, device="cuda")
    p_d = torch.arange(n, dtype=torch.int32, device="cuda")
    p0 = p_d.clone()

    def call():
        a_d.copy_(a0)
        p_d.copy_(p0)
        torch.cuda.synchronize()
        return lib.spral_ssids_gpu_ldlt_app_factor_noalloc(
            m, n, ctypes.c_void_p(p_d.data_ptr()), ctypes.c_void_p(a_d.data_ptr()), m,
            ctypes.c_void_p(d_d.data_ptr()), 1.0, ctypes.c_void_p(a_d.data_ptr() + 8 * (n * m + n)),
            m, ctypes.byref(opts), None)

    assert call() >= 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    alloc0 = torch.cuda.memory_allocated()
    assert call() >= 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert torch.cuda.memory_allocated() == alloc0


def test_noalloc_rejects_front_beyond_fixed_scratch():
    torch = pytest.importorskip("torch")
    from spral_gb300 import _native
    import oracle
    lib = _native.lib()
    m = n = 1100
    a_d = torch.zeros(m * m, dtype=torch.float64, device="cuda")
    d_d = torch.zeros(2 * n, dtype=torch.float64, device="cuda")
    p_d = torch.arange(n, dtype=torch.int32, device="cuda")
    rc = lib.spral_ssids_gpu_ldlt_app_factor_noalloc(
        m, n, ctypes.c_void_p(p_d.data_ptr()), ctypes.c_void_p(a_d.data_ptr()), m,
        ctypes.c_void_p(d_d.data_ptr()), 1.0, None, 0, ctypes.byref(oracle.default_options()), None)
    assert rc == -60
    # the leading dimension alone is limited too (a small front stored in a
    # taller array), while an empty front succeeds whatever its lda
    m, n, lda = 64, 32, 1100
    a2 = torch.zeros(lda * n, dtype=torch.float64, device="cuda")
    rc = lib.spral_ssids_gpu_ldlt_app_factor_noalloc(
        m, n, ctypes.c_void_p(p_d.data_ptr()), ctypes.c_void_p(a2.data_ptr()), lda,
        ctypes.c_void_p(d_d.data_ptr()), 1.0, None, 0, ctypes.byref(oracle.default_options()), None)
    assert rc == -60
    rc = lib.spral_ssids_gpu_ldlt_app_factor_noalloc(
        m, 0, ctypes.c_void_p(p_d.data_ptr()), ctypes.c_void_p(a2.data_ptr()), lda,
        ctypes.c_void_p(d_d.data_ptr()), 1.0, None, 0, ctypes.byref(oracle.default_options()), None)
    assert rc == 0
