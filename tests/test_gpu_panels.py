"""APP panels of the FP32-factor path: fronts wider than the panel width
(256 columns) are factored panel by panel, each panel's trailing update on
the tensor cores.  Checked against the same factorisation without panels
(SPRAL_GB300_PANEL=0) and against the FP64 oracle: exact inertia, refined
backward error, solutions; and a captured refactorisation with panels equal
bit for bit to the eager one."""
import numpy as np
import pytest

from spral_gb300 import matrices as M, ssids
import oracle

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _mixed():
    return ssids.Options(precision=ssids.PRECISION_MIXED, max_refine=30, refine_tol=1e-15)


@pytest.mark.parametrize("kind", ["lap3d", "kkt"])
def test_gpu_panels_match_unpaneled_and_oracle(kind, monkeypatch):
    monkeypatch.setenv("SPRAL_GB300_PANEL_MIN_N", "257")
    if kind == "lap3d":
        k = 24
        p, r, v = M.laplacian_3d(k, shift=-0.3)
        ak = ssids.analyse(p, r, M.nd_order_grid(k, k, k))
        neg, _, _ = M.laplacian_eig_count_3d(k, k, k, -0.3)
    else:
        p, r, v = M.kkt(3000, 1500, seed=7)
        ak = ssids.analyse(p, r, ssids.order_amd(p, r))
        neg = 1500  # Sylvester: H SPD, A full row rank
    assert ak.maxsupernode > 256  # the case must have fronts with panels
    n = len(p) - 1
    b = np.random.default_rng(5).standard_normal((n, 3))
    fk, inf = ssids.factor(ak, v, _mixed())
    assert inf.flag >= 0 and inf.num_neg == neg
    x = fk.solve_refined(b)
    assert M.scaled_bwd_error(p, r, v, x, b).max() <= 1e-14
    monkeypatch.setenv("SPRAL_GB300_PANEL", "0")
    f0, inf0 = ssids.factor(ak, v, _mixed())
    assert inf0.num_neg == neg
    x0 = f0.solve_refined(b)
    xo = oracle.OracleFactor(ak, v, blas=True).solve(b)
    assert _rel(x, xo) < 1e-10 and _rel(x0, xo) < 1e-10
    if kind == "kkt":
        assert inf.num_two > 0 and inf.num_delay > 0
    fk.free()
    f0.free()


def test_gpu_panels_captured_refactorisation_matches_eager(monkeypatch):
    monkeypatch.setenv("SPRAL_GB300_PANEL_MIN_N", "257")
    k = 24
    p, r, v = M.laplacian_3d(k, shift=-0.3)
    ak = ssids.analyse(p, r, M.nd_order_grid(k, k, k))
    fk, inf = ssids.factor(ak, v, _mixed())
    assert inf.num_delay == 0
    b = np.random.default_rng(6).standard_normal(k ** 3)
    x_eager = fk.solve(b)
    for _ in range(2):  # the second refactorisation replays the captured graph
        assert fk.refactor(v) == 0
        assert np.array_equal(fk.solve(b), x_eager)
    fk.free()
