"""The wavefront solves (one persistent launch per pass over the whole tree,
items waiting on the flags and counters of the items they need; the default
for FP32 factors) against the chain of block step launches (the default for
FP64 factors): every job, several right-hand side counts, FP64 and FP32
factors, a tree with delayed columns, a forest of many small matrices."""
import numpy as np
import pytest

from spral_gb300 import matrices as M, ssids

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


# FP32 factors: the two summation orders differ by FP32 rounding, amplified
# by the matrices' condition numbers (~1e3)
@pytest.mark.parametrize("precision,tol", [(ssids.PRECISION_FP64, 1e-12),
                                           (ssids.PRECISION_MIXED, 1e-3)], ids=["fp64", "mixed"])
@pytest.mark.parametrize("case", ["lap3d", "kkt"])
def test_gpu_wave_solves_match_block_steps(case, precision, tol, monkeypatch):
    if case == "lap3d":
        k = 20
        p, r, v = M.laplacian_3d(k, shift=-0.3)
        ak = ssids.analyse(p, r, M.nd_order_grid(k, k, k))
    else:
        p, r, v = M.kkt(1500, 700, seed=3)
        ak = ssids.analyse(p, r, ssids.order_amd(p, r))
    n = len(p) - 1
    opts = ssids.Options(precision=precision)
    monkeypatch.setenv("SPRAL_GB300_SOLVE_WAVE", "1")
    fw, infw = ssids.factor(ak, v, opts)
    monkeypatch.setenv("SPRAL_GB300_SOLVE_WAVE", "0")
    fs, infs = ssids.factor(ak, v, opts)
    if case == "kkt":
        assert infw.num_delay > 0
    rng = np.random.default_rng(11)
    for nrhs in (1, 5, 16):
        b = rng.standard_normal((n, nrhs))
        for job in (0, 1, 2, 3, 4):
            xw, xs = fw.solve(b, job=job), fs.solve(b, job=job)
            assert _rel(xw, xs) < tol, (nrhs, job)
    b = rng.standard_normal((n, 3))
    x = fw.solve(b)
    bound = 5e-14 if precision == ssids.PRECISION_FP64 else 1e-5
    assert M.scaled_bwd_error(p, r, v, x, b).max() <= bound
    fw.free()
    fs.free()


def test_gpu_wave_posdef_solves(monkeypatch):
    monkeypatch.setenv("SPRAL_GB300_SOLVE_WAVE", "1")
    k = 16
    p, r, v = M.laplacian_3d(k, shift=0.5)  # positive definite
    ak = ssids.analyse(p, r, M.nd_order_grid(k, k, k))
    fk, inf = ssids.factor(ak, v, posdef=True)
    assert inf.flag == 0
    b = np.random.default_rng(2).standard_normal((k ** 3, 4))
    x = fk.solve(b)
    assert M.scaled_bwd_error(p, r, v, x, b).max() <= 5e-14
    y = fk.solve(b, job=1)
    assert _rel(fk.solve(y, job=3), x) < 1e-12
    fk.free()


@pytest.mark.parametrize("precision,tol", [(ssids.PRECISION_FP64, 1e-12),
                                           (ssids.PRECISION_MIXED, 1e-3)], ids=["fp64", "mixed"])
def test_gpu_wave_solves_on_a_forest(precision, tol, monkeypatch):
    """A batch of 40 small indefinite 2D Laplacians (one forest whose levels
    hold many small fronts, taken whole by one item each): the wavefront
    passes against the block steps, matrix by matrix."""
    from spral_gb300 import batch
    rng = np.random.default_rng(40)
    sides = rng.integers(4, 40, 40)
    mats = [M.laplacian_2d(int(k), int(k), float(s))
            for k, s in zip(sides, rng.uniform(-1, 0, 40))]
    bak = batch.BatchAkeep([(p, r) for p, r, _ in mats],
                           [M.nd_order_grid(int(k), int(k)) for k in sides])
    vals = [v for _, _, v in mats]
    opts = ssids.Options(precision=precision)
    monkeypatch.setenv("SPRAL_GB300_SOLVE_WAVE", "1")
    bw = batch.BatchFkeep(bak, vals, opts)
    monkeypatch.setenv("SPRAL_GB300_SOLVE_WAVE", "0")
    bs_ = batch.BatchFkeep(bak, vals, opts)
    b = [rng.standard_normal((len(p) - 1, 3)) for p, _, _ in mats]
    for xw, xs in zip(bw.solve(b), bs_.solve(b)):
        assert _rel(xw, xs) < tol
    bw.free()
    bs_.free()
