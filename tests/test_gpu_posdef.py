"""Positive-definite (Cholesky) factorisation: no pivoting, L_chol = L D^(1/2)
semantics for the partial solves and enquire_posdef, -6 for matrices that
are not positive definite (src/ssids/cpu/kernels/cholesky.cxx,
NumericSubtree.hxx:318-431)."""
import numpy as np
import pytest

from spral_gb300 import matrices as M, ssids

pytestmark = pytest.mark.gpu


def _dense(p, r, v, n):
    A = np.zeros((n, n))
    for j in range(n):
        for k in range(p[j], p[j + 1]):
            A[r[k], j] = v[k]
            A[j, r[k]] = v[k]
    return A


@pytest.mark.parametrize("precision", [ssids.PRECISION_FP64, ssids.PRECISION_MIXED])
def test_gpu_posdef_matches_dense_cholesky(precision):
    k = 9
    p, r, v = M.laplacian_3d(k, shift=0.5)  # SPD
    n = k ** 3
    ak = ssids.analyse(p, r, M.nd_order_grid(k, k, k))
    fk = ssids.Fkeep(ak, v, ssids.Options(precision=precision), posdef=True)
    assert fk.inform.flag == 0
    assert fk.inform.num_neg == 0 and fk.inform.num_delay == 0
    A = _dense(p, r, v, n)
    Ap = A[np.ix_(ak.invp, ak.invp)]  # pivot order
    Lc = np.linalg.cholesky(Ap)
    rtol = 1e-12 if precision == ssids.PRECISION_FP64 else 1e-5
    d = fk.enquire_posdef()
    assert np.allclose(d, np.diag(Lc), rtol=rtol, atol=0)
    b = np.random.default_rng(1).standard_normal((n, 2))
    # forward solve with the Cholesky factor, in the user's variable order
    y = fk.solve(b, job=1)
    yref = np.empty_like(b)
    yref[ak.invp] = np.linalg.solve(Lc, b[ak.invp])
    assert np.abs(y - yref).max() <= rtol * 10 * np.abs(yref).max()
    # backward solve of that: the full solution
    x = fk.solve(y, job=3)
    assert M.scaled_bwd_error(p, r, v, x, b).max() <= (1e-14 if rtol < 1e-6 else 1e-5)
    xf = fk.solve(b)
    assert np.allclose(xf, x, rtol=1e-12 if rtol < 1e-6 else 1e-4, atol=0)
    with pytest.raises(ValueError):
        fk.solve(b, job=2)  # no diagonal solve for posdef
    if precision == ssids.PRECISION_MIXED:
        xr = fk.solve_refined(b)
        assert M.scaled_bwd_error(p, r, v, xr, b).max() <= 1e-14
    fk.free()


def test_gpu_posdef_rejects_indefinite():
    p, r, v = M.laplacian_3d(8, shift=-0.5)
    ak = ssids.analyse(p, r, M.nd_order_grid(8, 8, 8))
    fk = ssids.Fkeep(ak, v, posdef=True)
    assert fk.inform.flag == -6
    fk.free()


def test_gpu_posdef_refactor_graph_and_kkt_block():
    """Same-pattern posdef refactorisation (captured graph) and an SPD block
    with random sparsity (the H block of the KKT workload)."""
    p, r, v = M.kkt(800, 1, seed=3)  # H (800 x 800 SPD) plus one constraint row
    # take the H block alone: columns < 800, rows < 800
    keep = r < 800
    cols = np.repeat(np.arange(len(p) - 1), np.diff(p))
    sel = keep & (cols < 800)
    ph = np.concatenate([[0], np.cumsum(np.bincount(cols[sel], minlength=800))])
    rh, vh = r[sel], v[sel]
    ak = ssids.analyse(ph, rh, ssids.order_mindeg(ph, rh))
    fk = ssids.Fkeep(ak, vh, posdef=True)
    assert fk.inform.flag == 0
    b = np.random.default_rng(4).standard_normal(800)
    for scale in (1.0, 2.0, 0.5):
        assert fk.refactor(vh * scale) == 0
        x = fk.solve(b)
        assert M.scaled_bwd_error(ph, rh, vh * scale, x, b).max() <= 1e-14
    fk.free()
