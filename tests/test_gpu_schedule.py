"""The two level schedules of the numeric factorisation (leaf-aligned and
root-aligned levels) give the same factorisation: each front's arithmetic
does not depend on which fronts share its launches.  A nested-dissection
Laplacian, a KKT system with delayed pivots and a forest of small
matrices, FP64 and FP32 factors."""
import numpy as np
import pytest

from spral_gb300 import batch, matrices as M, ssids

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _problem(case):
    if case == "lap3d":
        k = 22
        p, r, v = M.laplacian_3d(k, shift=-0.3)
        return p, r, v, ssids.analyse(p, r, M.nd_order_grid(k, k, k))
    if case == "kkt":
        p, r, v = M.kkt(1500, 700, seed=5)
        return p, r, v, ssids.analyse(p, r, ssids.order_amd(p, r))
    rng = np.random.default_rng(8)
    sides = rng.integers(6, 40, 24)
    mats = [M.laplacian_2d(int(k), int(k), float(-rng.uniform())) for k in sides]
    bak = batch.BatchAkeep([(p, r) for p, r, _ in mats],
                           [M.nd_order_grid(int(k), int(k)) for k in sides])
    v = bak.stack_values([v for _, _, v in mats])
    return bak.ptr, bak.row, v, bak.akeep


@pytest.mark.parametrize("precision,tol", [(ssids.PRECISION_FP64, 1e-12),
                                           (ssids.PRECISION_MIXED, 1e-4)], ids=["fp64", "mixed"])
@pytest.mark.parametrize("case", ["lap3d", "kkt", "forest"])
def test_gpu_level_alignments_agree(case, precision, tol, monkeypatch):
    p, r, v, ak = _problem(case)
    n = len(p) - 1
    b = np.random.default_rng(3).standard_normal((n, 2))
    out = {}
    for align in ("leaf", "root"):
        monkeypatch.setenv("SPRAL_GB300_LEVEL_ALIGN", align)
        fk, inf = ssids.factor(ak, v, ssids.Options(precision=precision))
        assert inf.flag >= 0
        out[align] = (fk.solve(b), inf.num_neg, inf.num_delay, inf.num_two)
        fk.free()
    (xl, negl, dell, twol), (xr, negr, delr, twor) = out["leaf"], out["root"]
    assert (negl, dell, twol) == (negr, delr, twor)
    if case == "kkt":
        assert dell > 0
    assert _rel(xr, xl) < tol
