"""GPU tests of the dense per-front entry point spral_ssids_gpu_ldlt_app_factor,
following the reference's kernel tests (tests/ssids/kernels/ldlt_app.cxx:
277-400): factor the first n columns of an m x m matrix, update the trailing
block, factor the remainder, and require a scaled backward error <= 1e-13."""
import ctypes

import numpy as np
import pytest

from dense_cases import backward_error, cause_delays, full_solve, gen_sym_indef, make_singular

pytestmark = pytest.mark.gpu


def _factor(lib, opts, m, n, a_d, lda, off, d_d, perm_d, torch):
    """Call the entry point on the trailing (m-off) x (m-off) part at (off, off)."""
    base = a_d.data_ptr() + 8 * (off * lda + off)
    upd = base + 8 * (n * lda + n) if m > n else None
    return lib.spral_ssids_gpu_ldlt_app_factor(
        m, n, ctypes.c_void_p(perm_d.data_ptr() + 4 * off), ctypes.c_void_p(base), lda,
        ctypes.c_void_p(d_d.data_ptr() + 8 * 2 * off), 1.0,
        ctypes.c_void_p(upd) if upd else None, lda, ctypes.byref(opts), None)


@pytest.mark.parametrize("m,n,delays,singular,seed", [
    (2, 1, False, False, 1), (5, 3, False, False, 2), (64, 24, False, False, 3),
    (64, 64, False, False, 4), (100, 37, True, False, 5), (256, 96, True, False, 6),
    (300, 300, True, False, 7), (500, 130, True, True, 8), (700, 260, True, False, 9),
])
def test_gpu_dense_ldlt_app_bwd_error(m, n, delays, singular, seed):
    torch = pytest.importorskip("torch")
    from spral_gb300 import _native
    import oracle
    lib = _native.lib()
    rng = np.random.default_rng(seed)
    a = gen_sym_indef(m, rng)
    if delays:
        cause_delays(a, rng)
    if singular and n > 1:
        c1, c2 = rng.choice(n, 2, replace=False)
        make_singular(a, int(c1), int(c2))
    lda = m
    a_d = torch.tensor(np.asfortranarray(a).ravel(order="F"), dtype=torch.float64, device="cuda")
    d_d = torch.zeros(2 * m + 2, dtype=torch.float64, device="cuda")
    perm_d = torch.arange(m, dtype=torch.int32, device="cuda")
    opts = oracle.default_options()
    q1 = _factor(lib, opts, m, n, a_d, lda, 0, d_d, perm_d, torch)
    assert 0 <= q1 <= n
    perm1 = perm_d.cpu().numpy().copy()
    if m > n or q1 < n:
        # the remaining (m - q1) x (m - q1) matrix is factored as a square front
        rest = m - q1
        q2 = _factor(lib, opts, rest, rest, a_d, lda, q1, d_d, perm_d, torch)
        assert q2 == rest
    perm = perm_d.cpu().numpy()
    l = a_d.cpu().numpy().reshape(m, m, order="F").copy()
    if m > n or q1 < n:
        # rows of the first call's columns follow the second call's pivoting
        # (permute_rows in the reference test, ldlt_app.cxx:360)
        where = {int(v): k for k, v in enumerate(perm1[q1:])}
        rows = np.array([q1 + where[int(v)] for v in perm[q1:]], dtype=np.int64)
        l[q1:, :q1] = l[rows, :q1]
    d = d_d.cpu().numpy()
    b = a @ np.ones(m)  # consistent right-hand side (solution of ones), as gen_rhs
    x = full_solve(m, q1, l, d, perm, b)
    assert backward_error(a, x, b) <= 1e-13


@pytest.mark.parametrize("case", ["lap3d", "kkt"])
@pytest.mark.parametrize("warps", ["4", "8", "17"])
def test_gpu_fp32_diag_block_warp_counts_agree(warps, case, monkeypatch):
    """The FP32 diagonal-block kernel with 4, 8 or 17 warps (pairs per
    thread 5, 3, 1) takes the same pivots and gives the same bits (fronts
    above the small leaf subtrees, so the APP block steps run)."""
    import numpy as np
    from spral_gb300 import matrices as M, ssids
    if case == "lap3d":
        p, r, v = M.laplacian_3d(20, shift=-0.3)
        ak = ssids.analyse(p, r, M.nd_order_grid(20, 20, 20))
    else:
        p, r, v = M.kkt(4000, 2000, seed=5)
        ak = ssids.analyse(p, r, ssids.order_amd(p, r))
    b = np.random.default_rng(3).standard_normal((len(p) - 1, 2))
    opts = ssids.Options(precision=ssids.PRECISION_MIXED)
    monkeypatch.setenv("SPRAL_GB300_DIAG_WARPS", "17")
    f0, i0 = ssids.factor(ak, v, opts)
    x0 = f0.solve(b)
    monkeypatch.setenv("SPRAL_GB300_DIAG_WARPS", warps)
    f1, i1 = ssids.factor(ak, v, opts)
    x1 = f1.solve(b)
    assert (i1.num_neg, i1.num_two, i1.num_delay) == (i0.num_neg, i0.num_two, i0.num_delay)
    assert np.array_equal(x0, x1)
    f0.free()
    f1.free()
