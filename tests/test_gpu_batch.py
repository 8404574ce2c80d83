"""Batched factor + solve of many independent indefinite 2D Laplacians (the
batching workload at a reduced count): per-matrix inertia against the
analytic eigenvalue count, and every matrix's solution identical to
factoring it alone."""
import numpy as np
import pytest

from spral_gb300 import batch, matrices as M, ssids

pytestmark = pytest.mark.gpu


def _batch(count, lo, hi, seed):
    rng = np.random.default_rng(seed)
    sides = np.exp(rng.uniform(np.log(lo), np.log(hi), count)).astype(int)
    shifts = rng.uniform(-1.0, 0.0, count)
    mats = [M.laplacian_2d(int(s), int(s), float(sh)) for s, sh in zip(sides, shifts)]
    orders = [M.nd_order_grid(int(s), int(s)) for s in sides]
    return sides, shifts, mats, orders


@pytest.mark.parametrize("precision", [ssids.PRECISION_FP64, ssids.PRECISION_MIXED])
def test_gpu_batch_matches_individual_factorisations(precision):
    sides, shifts, mats, orders = _batch(24, 8, 40, 4)
    bak = batch.BatchAkeep([(p, r) for p, r, _ in mats], orders)
    opts = ssids.Options(precision=precision)
    bf = batch.BatchFkeep(bak, [v for _, _, v in mats], opts)
    assert bf.inform.flag >= 0
    inert = bf.inertia()
    for i, (s, sh) in enumerate(zip(sides, shifts)):
        neg, zero, _ = M.laplacian_eig_count_2d(int(s), int(s), float(sh))
        assert inert[i, 0] == neg and inert[i, 2] == zero
    rng = np.random.default_rng(9)
    bs = [rng.uniform(-1, 1, len(p) - 1) for p, _, _ in mats]
    xs = bf.solve(bs)
    # direct solves without refinement: the FP64 bound is 5e-14, as for the
    # reference fixtures (the reference's TPP in small leaf subtrees takes
    # 2x2 pivots whose growth bound is 1/u); FP32 factors the same bound in
    # units of their precision, 5e-14 * eps32/eps64 = 5e-14 * 2^29 = 2.7e-5
    # (measured up to 1.3e-5 on these matrices)
    tol = 5e-14 if precision == ssids.PRECISION_FP64 else 5e-14 * 2.0 ** 29
    for i, (p, r, v) in enumerate(mats):
        assert M.scaled_bwd_error(p, r, v, xs[i], bs[i]).max() <= tol
    # alone: the same kernels on the same data give the same bits
    for i in (0, 7, 23):
        p, r, v = mats[i]
        ak = ssids.analyse(p, r, orders[i])
        fk = ssids.Fkeep(ak, v, opts)
        assert fk.inform.num_neg == inert[i, 0]
        assert np.array_equal(fk.solve(bs[i]), xs[i])
        fk.free()
    bf.free()


def test_gpu_batch_refactor_replays_graph():
    sides, shifts, mats, orders = _batch(16, 8, 32, 5)
    bak = batch.BatchAkeep([(p, r) for p, r, _ in mats], orders)
    bf = batch.BatchFkeep(bak, [v for _, _, v in mats])
    rng = np.random.default_rng(2)
    for rep in range(3):
        # rescale the diagonal (same pattern): the shift changes each time
        new_shift = rng.uniform(-1.0, 0.0, len(mats))
        vals = []
        for (p, r, v), s, sh, nsh in zip(mats, sides, shifts, new_shift):
            dpos = np.array([p[j] + np.nonzero(r[p[j]:p[j + 1]] == j)[0][0] for j in range(len(p) - 1)])
            w = v.copy()
            w[dpos] = 4.0 + nsh
            vals.append(w)
        assert bf.refactor(vals) >= 0
        inert = bf.inertia()
        for i, (s, nsh) in enumerate(zip(sides, new_shift)):
            assert inert[i, 0] == M.laplacian_eig_count_2d(int(s), int(s), float(nsh))[0]
        bs = [np.ones(len(p) - 1) for p, _, _ in mats]
        xs = bf.solve(bs)
        for i, (p, r, _) in enumerate(mats):
            assert M.scaled_bwd_error(p, r, vals[i], xs[i], bs[i]).max() <= 1e-14
    bf.free()


@pytest.mark.parametrize("precision", [ssids.PRECISION_FP64, ssids.PRECISION_MIXED])
def test_gpu_batch_refined_meets_target_per_matrix(precision):
    """Refinement of a batch stops only when every matrix's own scaled
    backward error (its own norms) meets the target, not the stacked
    system's."""
    sides, shifts, mats, orders = _batch(32, 8, 64, 6)
    bak = batch.BatchAkeep([(p, r) for p, r, _ in mats], orders)
    opts = ssids.Options(precision=precision, max_refine=20, refine_tol=1e-14)
    bf = batch.BatchFkeep(bak, [v for _, _, v in mats], opts)
    rng = np.random.default_rng(11)
    # right-hand sides of very different sizes per matrix, so that the
    # stacked system's norms say little about the small ones
    bs = [rng.uniform(-1, 1, len(p) - 1) * 10.0 ** rng.integers(-6, 3) for p, _, _ in mats]
    xs = bf.solve_refined(bs)
    worst = max(float(M.scaled_bwd_error(p, r, v, xs[i], bs[i]).max())
                for i, (p, r, v) in enumerate(mats))
    assert worst <= 1e-14
    bf.free()


def test_gpu_mixed_batch_falls_back_per_matrix():
    """A batch of FP32 factors in which one matrix is too ill-conditioned for
    FP32 (a shifted 2D Laplacian with an eigenvalue 3e-9 from zero): only
    that matrix is refactored in FP64 (a sub-batch of its own), every
    matrix's refined solve meets 1e-14, the inertia is exact for all, and a
    refactorisation with the same values repeats the same fallback."""
    nx, ny = 30, 34
    lam = (2 - 2 * np.cos(np.pi * 3 / (nx + 1))) + (2 - 2 * np.cos(np.pi * 5 / (ny + 1)))
    bad_shift = 3e-9 - lam
    specs = [(12, 12, -0.4), (nx, ny, bad_shift), (20, 17, -0.7), (9, 25, -0.2)]
    mats = [M.laplacian_2d(a, b, s) for a, b, s in specs]
    bak = batch.BatchAkeep([(p, r) for p, r, _ in mats],
                           [M.nd_order_grid(a, b) for a, b, _ in specs])
    opts = ssids.Options(precision=ssids.PRECISION_MIXED, max_refine=20, refine_tol=1e-14)
    bf = batch.BatchFkeep(bak, [v for _, _, v in mats], opts)
    rng = np.random.default_rng(8)
    bs = [rng.uniform(-1, 1, (a * b, 2)) for a, b, _ in specs]
    xs = bf.solve_refined(bs)
    assert list(bf.failed) == [1]
    assert bf.fk.fallbacks == 0  # the batch handle itself never refactors in FP64
    for (p, r, v), x, b in zip(mats, xs, bs):
        assert M.scaled_bwd_error(p, r, v, x, b).max() <= 1e-14
    inert = bf.inertia()
    for i, (a, b, s) in enumerate(specs):
        assert inert[i, 0] == M.laplacian_eig_count_2d(a, b, s)[0]
    bf.refactor([v for _, _, v in mats])
    xs2 = bf.solve_refined(bs)
    assert list(bf.failed) == [1] and bf.fallback_matrices == 2
    for x, x2 in zip(xs, xs2):
        assert np.array_equal(x, x2)
    bf.free()
