"""The one-warp FP32 diagonal-block kernel against the 17-warp one
(SPRAL_GB300_DIAG_WARP=0): same inertia, 2x2 pivots and delays exercised,
refined solutions at the FP64 oracle's, on a Laplacian and on matrices
with many delayed columns."""
import numpy as np
import pytest

from spral_gb300 import matrices as M, ssids
import oracle

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("case", ["lap3d", "kkt", "rand"])
def test_gpu_one_warp_diag_matches_block_kernel(case, monkeypatch):
    if case == "lap3d":
        k = 20
        p, r, v = M.laplacian_3d(k, shift=-0.3)
        ak = ssids.analyse(p, r, M.nd_order_grid(k, k, k))
    elif case == "kkt":
        p, r, v = M.kkt(2000, 900, seed=8)
        ak = ssids.analyse(p, r, ssids.order_amd(p, r))
    else:
        p, r, v = M.random_indef(1500, density=0.004, seed=31, diag_scale=0.1)
        ak = ssids.analyse(p, r, ssids.order_mindeg(p, r))
    n = len(p) - 1
    opts = ssids.Options(precision=ssids.PRECISION_MIXED, max_refine=30, refine_tol=1e-15)
    b = np.random.default_rng(4).standard_normal((n, 2))
    fw, infw = ssids.factor(ak, v, opts)
    monkeypatch.setenv("SPRAL_GB300_DIAG_WARP", "0")
    fb, infb = ssids.factor(ak, v, opts)
    assert infw.flag >= 0 and infw.num_neg == infb.num_neg
    if case != "lap3d":
        assert infw.num_two > 0 and infw.num_delay > 0
    xw, xb = fw.solve_refined(b), fb.solve_refined(b)
    assert M.scaled_bwd_error(p, r, v, xw, b).max() <= 1e-14
    xo = oracle.OracleFactor(ak, v, blas=True).solve(b)
    assert _rel(xw, xo) < 1e-9 and _rel(xb, xo) < 1e-9
    fw.free()
    fb.free()
