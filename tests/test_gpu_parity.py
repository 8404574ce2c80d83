"""GPU parity tests: the CUDA factor/solve through the C-ABI against the
analytic inertia, the committed reference fixtures and the oracle."""
import glob
import os

import numpy as np
import pytest

from spral_gb300 import matrices as M, ssids
import oracle

pytestmark = pytest.mark.gpu
GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))

# tolerances: inertia exact; scaled backward error of an FP64 direct solve;
# solution against the FP64 reference within 1e-10 relative
BWD_TOL = 1e-14
SOL_TOL = 1e-10


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_gpu_lap2d_64_analytic():
    p, r, v = M.laplacian_2d(64, 64, -0.5)
    ak = ssids.analyse(p, r, M.nd_order_grid(64, 64))
    fk, inf = ssids.factor(ak, v)
    assert inf.flag == 0
    assert inf.num_neg == 158
    assert inf.matrix_rank == 4096
    b = np.random.default_rng(0).uniform(-1, 1, 4096)
    x = fk.solve(b)
    assert M.scaled_bwd_error(p, r, v, x, b).max() <= BWD_TOL
    xo = oracle.OracleFactor(ak, v).solve(b)
    assert _rel(x, xo) < SOL_TOL


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_gpu_matches_reference_fixture(path):
    g = np.load(path)
    p, r, v, b = g["ptr"], g["row"], g["val"], g["b"]
    ak = ssids.analyse(p, r, g["order"])
    fk, inf = ssids.factor(ak, v)
    assert inf.flag == int(g["stat_flag"])
    assert inf.num_neg == int(g["stat_num_neg"])
    assert inf.matrix_rank == len(p) - 1 - int(g["stat_num_zero"])
    x = fk.solve(b)
    assert M.scaled_bwd_error(p, r, v, x, b).max() <= 5e-14
    assert _rel(x, g["x"]) < SOL_TOL


@pytest.mark.parametrize("seed", [11, 12])
def test_gpu_vs_oracle_with_delays(seed):
    p, r, v = M.random_indef(400, density=0.02, seed=seed, diag_scale=0.01)
    ak = ssids.analyse(p, r, ssids.order_mindeg(p, r))
    fk, inf = ssids.factor(ak, v)
    F = oracle.OracleFactor(ak, v)
    assert inf.num_neg == F.stats["num_neg"]
    assert inf.num_delay > 0  # the case must exercise delayed pivots
    b = np.random.default_rng(seed).uniform(-1, 1, (400, 3))
    x = fk.solve(b)
    assert M.scaled_bwd_error(p, r, v, x, b).max() <= 1e-13
    assert _rel(x, F.solve(b)) < 1e-8


def test_gpu_kkt_2x2_and_delays():
    p, r, v = M.kkt(600, 250, seed=2)
    ak = ssids.analyse(p, r, ssids.order_mindeg(p, r))
    fk, inf = ssids.factor(ak, v)
    assert inf.num_neg == 250  # Sylvester: A has full row rank
    assert inf.num_two > 0
    b = np.random.default_rng(2).standard_normal((850, 2))
    x = fk.solve(b)
    assert M.scaled_bwd_error(p, r, v, x, b).max() <= 1e-14


def test_gpu_partial_solves_compose():
    p, r, v = M.random_indef(300, density=0.03, seed=5, diag_scale=0.01)
    ak = ssids.analyse(p, r, ssids.order_mindeg(p, r))
    fk, _ = ssids.factor(ak, v)
    b = np.random.default_rng(5).uniform(-1, 1, (300, 2))
    x_full = fk.solve(b)
    y = fk.solve(b, job=1)
    x2 = fk.solve(y, job=4)
    assert _rel(x2, x_full) < 1e-12
    z = fk.solve(fk.solve(y, job=2), job=3)
    assert _rel(z, x_full) < 1e-12


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_gpu_pivots_and_partial_solves_match_reference_fixture(path):
    """The reference's own pivot order, D^{-1} and partial solves (fixture
    fields piv_order, d, x_fwd, x_diag): small leaf subtrees are factored by
    TPP and children are visited last first as in the reference, so the GPU
    takes the same pivots; jobs 3 and 4 against the oracle, which takes the
    same pivots too."""
    g = np.load(path)
    p, r, v, b = g["ptr"], g["row"], g["val"], g["b"]
    ak = ssids.analyse(p, r, g["order"])
    fk, inf = ssids.factor(ak, v)
    assert inf.num_two == int(g["stat_num_two"])
    assert inf.num_delay == int(g["stat_num_delay"])
    piv, d = fk.enquire_indef()
    assert np.array_equal(piv, g["piv_order"])
    assert np.abs(d - g["d"]).max() <= 1e-12 * np.abs(g["d"]).max()
    assert _rel(fk.solve(b, job=1), g["x_fwd"]) < SOL_TOL
    assert _rel(fk.solve(b, job=2), g["x_diag"]) < SOL_TOL
    F = oracle.OracleFactor(ak, v)
    for job in (3, 4):
        assert _rel(fk.solve(b, job=job), F.solve(b, job=job)) < SOL_TOL
    # alter with the reference's d (equal to ours to ~1e-14) leaves the
    # solution unchanged to the solution tolerance
    x0 = fk.solve(b)
    fk.alter(g["d"])
    assert _rel(fk.solve(b), x0) < SOL_TOL


@pytest.mark.parametrize("seed", [21, 22, 23])
def test_gpu_partial_solves_and_enquire_match_oracle(seed):
    """A random indefinite matrix with APP fronts and delayed columns (random
    values: no ties in the pivot searches): the GPU and the oracle take the
    same pivots, so every partial solve and enquire_indef agree."""
    p, r, v = M.random_indef(1500, density=0.004, seed=seed, diag_scale=0.1)
    ak = ssids.analyse(p, r, ssids.order_mindeg(p, r))
    fk, inf = ssids.factor(ak, v)
    F = oracle.OracleFactor(ak, v)
    assert inf.num_delay == F.stats["num_delay"] and inf.num_delay > 0
    assert inf.num_two == F.stats["num_two"]
    pg, dg = fk.enquire_indef()
    po, do = F.enquire_indef()
    assert np.array_equal(pg, po)
    assert np.abs(dg - do).max() <= 1e-10 * np.abs(do).max()
    b = np.random.default_rng(seed).uniform(-1, 1, (1500, 2))
    for job in (0, 1, 2, 3, 4):
        assert _rel(fk.solve(b, job=job), F.solve(b, job=job)) < 1e-9, job


def test_gpu_many_rhs_chunks():
    p, r, v = M.laplacian_3d(10, shift=-0.5)
    ak = ssids.analyse(p, r, M.nd_order_grid(10, 10, 10))
    fk, _ = ssids.factor(ak, v)
    b = np.random.default_rng(3).standard_normal((1000, 37))
    x = fk.solve(b)
    assert M.scaled_bwd_error(p, r, v, x, b).max() <= BWD_TOL
    x1 = fk.solve(b[:, 5])
    assert _rel(x1, x[:, 5]) < 1e-14


def test_gpu_3d_analytic_inertia():
    k = 20
    p, r, v = M.laplacian_3d(k, shift=-0.3)
    ak = ssids.analyse(p, r, M.nd_order_grid(k, k, k))
    fk, inf = ssids.factor(ak, v)
    neg, zero, _ = M.laplacian_eig_count_3d(k, k, k, -0.3)
    assert inf.num_neg == neg
    b = np.random.default_rng(4).standard_normal((k ** 3, 8))
    x = fk.solve(b)
    assert M.scaled_bwd_error(p, r, v, x, b).max() <= BWD_TOL


@pytest.mark.parametrize("precision", [ssids.PRECISION_FP64, ssids.PRECISION_MIXED],
                         ids=["fp64", "mixed"])
def test_gpu_lap3d_32_vs_oracle(precision):
    """3D 7-point Laplacian on a 32^3 grid (n = 32,768), shift -0.3: inertia
    equal to the analytic count, scaled backward error <= 1e-14 and the
    solution within 1e-10 of the FP64 oracle, for FP64 factors and for FP32
    factors with FP64 refinement."""
    k = 32
    p, r, v = M.laplacian_3d(k, shift=-0.3)
    ak = ssids.analyse(p, r, M.nd_order_grid(k, k, k))
    opts = ssids.Options(precision=precision, max_refine=20, refine_tol=1e-15)
    fk, inf = ssids.factor(ak, v, opts)
    neg, zero, _ = M.laplacian_eig_count_3d(k, k, k, -0.3)
    assert inf.num_neg == neg and inf.matrix_rank == k ** 3 - zero
    b = np.random.default_rng(32).standard_normal((k ** 3, 4))
    # both paths refine in FP64 to the 1e-14 target, as the benchmark does
    # (an unrefined FP64 solve with the reference's TPP pivots in the small
    # leaf subtrees lands at about 1e-14 on this matrix)
    x = fk.solve_refined(b)
    assert M.scaled_bwd_error(p, r, v, x, b).max() <= BWD_TOL
    xo = oracle.OracleFactor(ak, v, blas=True).solve(b)
    assert _rel(x, xo) < SOL_TOL


def test_gpu_singular_flags():
    p, r, v = M.laplacian_2d(6, 6, -0.5)
    v = v.copy()
    cols = np.repeat(np.arange(36), np.diff(p))
    v[(r == 7) | (cols == 7)] = 0.0
    ak = ssids.analyse(p, r, M.nd_order_grid(6, 6))
    fk, inf = ssids.factor(ak, v)
    assert inf.flag == ssids.SSIDS_WARNING_FACT_SINGULAR
    assert inf.matrix_rank == 35
    fk2, inf2 = ssids.factor(ak, v, ssids.Options(action=False))
    assert inf2.flag == ssids.SSIDS_ERROR_SINGULAR


def test_gpu_tpp_only():
    p, r, v = M.random_indef(150, density=0.04, seed=9, diag_scale=0.01)
    ak = ssids.analyse(p, r, ssids.order_mindeg(p, r))
    fk, inf = ssids.factor(ak, v, ssids.Options(pivot_method=3))
    F = oracle.OracleFactor(ak, v, options=oracle.default_options(pivot_method=3))
    assert inf.num_neg == F.stats["num_neg"]
    b = np.random.default_rng(9).uniform(-1, 1, 150)
    assert M.scaled_bwd_error(p, r, v, fk.solve(b), b).max() <= 1e-13


def test_gpu_enquire_alter_roundtrip():
    p, r, v = M.kkt(120, 40, seed=4)
    ak = ssids.analyse(p, r, ssids.order_mindeg(p, r))
    fk, _ = ssids.factor(ak, v)
    piv, d = fk.enquire_indef()
    b = np.random.default_rng(4).standard_normal(160)
    x0 = fk.solve(b)
    fk.alter(d)
    assert _rel(fk.solve(b), x0) < 1e-15
    # negative piv_order marks 2x2 pivots; every variable appears once
    assert sorted(np.abs(piv).tolist())[-1] == 159


def test_gpu_refactor_same_pattern_device_values():
    torch = pytest.importorskip("torch")
    p, r, v = M.laplacian_3d(12, shift=-0.4)
    ak = ssids.analyse(p, r, M.nd_order_grid(12, 12, 12))
    fk, inf0 = ssids.factor(ak, v)
    v2 = v.copy()
    cols = np.repeat(np.arange(len(p) - 1), np.diff(p))
    v2[r == cols] *= 1.7
    dv = torch.tensor(v2, dtype=torch.float64, device="cuda")
    assert fk.refactor_dev(dv.data_ptr()) == 0
    fresh, inf1 = ssids.factor(ak, v2)
    assert fk.inform.num_neg == inf1.num_neg
    b = np.random.default_rng(0).standard_normal(len(p) - 1)
    assert _rel(fk.solve(b), fresh.solve(b)) < 1e-12


@pytest.mark.parametrize("k", [16, 24])
def test_gpu_mixed_precision_refined(k):
    p, r, v = M.laplacian_3d(k, shift=-0.3)
    ak = ssids.analyse(p, r, M.nd_order_grid(k, k, k))
    fk, inf = ssids.factor(ak, v, ssids.Options(precision=ssids.PRECISION_MIXED, max_refine=20,
                                                refine_tol=1e-15))
    neg, _, _ = M.laplacian_eig_count_3d(k, k, k, -0.3)
    assert inf.num_neg == neg  # exact inertia from the FP32 factor's FP64 pivots
    b = np.random.default_rng(k).standard_normal((k ** 3, 4))
    x = fk.solve_refined(b)
    assert M.scaled_bwd_error(p, r, v, x, b).max() <= BWD_TOL
    xd, _ = ssids.factor(ak, v)
    assert _rel(x, xd.solve(b)) < SOL_TOL


def test_gpu_mixed_falls_back_to_fp64_when_refinement_cannot_converge():
    """A shifted 2D Laplacian with one eigenvalue 3e-9 away from zero
    (condition number ~3e9): FP32 factors cannot drive the refinement to the
    target (kappa * eps32 >> 1), so the refined solve refactors in FP64 on the
    GPU once and finishes there; the result meets the FP64 bar and the
    statistics (inertia) are the FP64 factorisation's."""
    nx, ny = 30, 34
    lam = (2 - 2 * np.cos(np.pi * 3 / (nx + 1))) + (2 - 2 * np.cos(np.pi * 5 / (ny + 1)))
    shift = 3e-9 - lam
    p, r, v = M.laplacian_2d(nx, ny, shift)
    ak = ssids.analyse(p, r, M.nd_order_grid(nx, ny))
    opts = ssids.Options(precision=ssids.PRECISION_MIXED, max_refine=20, refine_tol=1e-14)
    fk, _ = ssids.factor(ak, v, opts)
    assert fk.fallbacks == 0
    b = np.random.default_rng(3).uniform(-1, 1, (nx * ny, 2))
    x = fk.solve_refined(b)
    assert fk.fallbacks == 1
    assert M.scaled_bwd_error(p, r, v, x, b).max() <= 1e-14
    neg, _, _ = M.laplacian_eig_count_2d(nx, ny, shift)
    assert fk.inform.num_neg == neg
    xd, _ = ssids.factor(ak, v, ssids.Options(max_refine=10, refine_tol=1e-14))
    assert _rel(x, xd.solve_refined(b)) < 1e-5  # kappa ~3e9: agreement limited by conditioning
    # a second solve reuses the FP64 factors; a refactorisation makes them stale
    x2 = fk.solve_refined(b)
    assert fk.fallbacks == 1 and np.array_equal(x, x2)
    fk.refactor(v)
    fk.solve_refined(b)
    assert fk.fallbacks == 2
    # a well-conditioned matrix never falls back
    p2, r2, v2 = M.laplacian_2d(nx, ny, -0.5)
    fk2, _ = ssids.factor(ssids.analyse(p2, r2, M.nd_order_grid(nx, ny)), v2, opts)
    fk2.solve_refined(b)
    assert fk2.fallbacks == 0


def _stack_lower_csc(mats, orders):
    """Block-diagonal stacking of lower-CSC matrices (and their orders)."""
    ptr, row, val, order = [np.zeros(1, dtype=np.int64)], [], [], []
    off = 0
    for (p, r, v), o in zip(mats, orders):
        ptr.append(p[1:] + ptr[-1][-1])
        row.append(r + off)
        val.append(v)
        order.append(o + off)
        off += len(p) - 1
    return (np.concatenate(ptr), np.concatenate(row).astype(np.int32), np.concatenate(val),
            np.concatenate(order).astype(np.int32))


def test_gpu_mixed_fallback_on_a_front_local_failure():
    """Two independent blocks in one tree (a forest): a well-conditioned 3D
    Laplacian and a 2D Laplacian with an eigenvalue 3e-9 from zero.  Only the
    fronts of the second block carry the ill-conditioning; the FP32 refinement
    stalls and the refined solve refactors the whole matrix in FP64 (the
    fallback is per matrix, not per front), after which both blocks meet the
    FP64 bar and the inertia is exact."""
    nx, ny = 30, 34
    lam = (2 - 2 * np.cos(np.pi * 3 / (nx + 1))) + (2 - 2 * np.cos(np.pi * 5 / (ny + 1)))
    shift = 3e-9 - lam
    k = 16
    good = M.laplacian_3d(k, shift=-0.3)
    bad = M.laplacian_2d(nx, ny, shift)
    p, r, v, order = _stack_lower_csc([good, bad], [M.nd_order_grid(k, k, k),
                                                     M.nd_order_grid(nx, ny)])
    ak = ssids.analyse(p, r, order)
    opts = ssids.Options(precision=ssids.PRECISION_MIXED, max_refine=20, refine_tol=1e-14)
    fk, _ = ssids.factor(ak, v, opts)
    b = np.random.default_rng(7).uniform(-1, 1, (len(p) - 1, 2))
    x = fk.solve_refined(b)
    assert fk.fallbacks == 1
    assert M.scaled_bwd_error(p, r, v, x, b).max() <= 1e-14
    neg3, _, _ = M.laplacian_eig_count_3d(k, k, k, -0.3)
    neg2, _, _ = M.laplacian_eig_count_2d(nx, ny, shift)
    assert fk.inform.num_neg == neg3 + neg2
    fk.free()


def test_gpu_recip_within_one_ulp():
    """The Newton reciprocal on the pivot-decision path agrees with IEEE
    division to one unit in the last place (and exactly at special values)."""
    torch = pytest.importorskip("torch")
    from spral_gb300 import _native
    rng = np.random.default_rng(7)
    x = np.concatenate([rng.uniform(-1, 1, 4000) * 10.0 ** rng.integers(-40, 40, 4000),
                        np.array([1.0, -1.0, 3.0, 1e-20, 1e20, 2.0 ** -100, 2.0 ** 100,
                                  1e-300, 1e300, 0.0, np.inf, -np.inf])])
    xd = torch.tensor(x, dtype=torch.float64, device="cuda")
    yd = torch.empty_like(xd)
    assert _native.lib().spral_ssids_gpu_recip_probe(xd.data_ptr(), yd.data_ptr(), len(x)) == 0
    y = yd.cpu().numpy()
    with np.errstate(divide="ignore"):
        ref = 1.0 / x
    fin = np.isfinite(ref) & (ref != 0)
    ulp = np.spacing(np.abs(ref[fin]))
    assert np.all(np.abs(y[fin] - ref[fin]) <= ulp)
    assert np.array_equal(y[~fin], ref[~fin])


@pytest.mark.parametrize("precision", [ssids.PRECISION_FP64, ssids.PRECISION_MIXED])
def test_gpu_graph_replay_matches_direct_launches(precision, monkeypatch):
    """Solves replayed from a captured CUDA graph give bitwise the same result
    as the directly launched sequence, across repeated solves and a
    same-pattern refactorisation with new values."""
    torch = pytest.importorskip("torch")
    k = 12
    p, r, v = M.laplacian_3d(k, shift=-0.3)
    ak = ssids.analyse(p, r, M.nd_order_grid(k, k, k))
    b = np.random.default_rng(5).standard_normal((ak.n, 3))
    v2 = v.copy()
    v2[p[:-1]] *= 1.25  # diagonal entries (first in each CSC column) rescaled
    res = {}
    for graphs in ("1", "0"):
        monkeypatch.setenv("SPRAL_GB300_GRAPHS", graphs)
        fk = ssids.Fkeep(ak, v, ssids.Options(precision=precision))
        x1 = fk.solve(b)
        x2 = fk.solve(b)          # replay
        v2d = torch.tensor(v2, dtype=torch.float64, device="cuda")
        assert fk.refactor_dev(v2d.data_ptr()) == 0
        x3 = fk.solve(b)
        res[graphs] = (x1, x2, x3)
        fk.free()
    for a, c in zip(res["1"], res["0"]):
        assert np.array_equal(a, c)
    assert np.array_equal(res["1"][0], res["1"][1])
    tol = BWD_TOL if precision == ssids.PRECISION_FP64 else 1e-5
    assert M.scaled_bwd_error(p, r, v2, res["1"][2], b).max() <= tol


def _diag_positions(p, r):
    """Index of each column's diagonal entry in lower-CSC value order."""
    return np.array([p[j] + np.nonzero(r[p[j]:p[j + 1]] == j)[0][0] for j in range(len(p) - 1)])


@pytest.mark.parametrize("precision", [ssids.PRECISION_FP64, ssids.PRECISION_MIXED])
def test_gpu_captured_refactorisation_matches_eager(precision, monkeypatch):
    """Same-pattern refactorisations replayed from the captured graph give
    bitwise the results of the eager launch sequence; a refactorisation whose
    values cause delayed pivots falls back to the eager path and is still
    correct; the graph is used again afterwards."""
    torch = pytest.importorskip("torch")
    p, r, v = M.random_indef(400, density=0.02, seed=11, diag_scale=0.01)
    ak = ssids.analyse(p, r, ssids.order_mindeg(p, r))
    dpos = _diag_positions(p, r)
    v_dd = v.copy()
    v_dd[dpos] = 50.0  # strongly diagonal: no delays
    v_dd2 = v_dd.copy()
    v_dd2[dpos] = 40.0
    b = np.random.default_rng(3).standard_normal((400, 2))
    seq = [v_dd, v_dd2, v, v_dd2]  # the third set delays pivots
    res = {}
    for graphs in ("1", "0"):
        monkeypatch.setenv("SPRAL_GB300_GRAPHS", graphs)
        fk = ssids.Fkeep(ak, seq[0], ssids.Options(precision=precision))
        assert fk.inform.num_delay == 0
        out = []
        for vals in seq[1:]:
            vd = torch.tensor(vals, dtype=torch.float64, device="cuda")
            assert fk.refactor_dev(vd.data_ptr()) >= 0
            out.append((fk.solve(b), fk.inform.num_neg, fk.inform.num_delay))
        res[graphs] = out
        fk.free()
    for (xa, na, da), (xb, nb, db) in zip(res["1"], res["0"]):
        assert na == nb and da == db
        assert np.array_equal(xa, xb)
    assert res["1"][1][2] > 0  # the third value set exercised delays
    tol = 1e-13 if precision == ssids.PRECISION_FP64 else 1e-4
    for (x, _, _), vals in zip(res["1"], seq[1:]):
        assert M.scaled_bwd_error(p, r, vals, x, b).max() <= tol


@pytest.mark.parametrize("seed,diag_scale", [(1, 0.01), (2, 0.001), (3, 0.1), (5, 1e-5)])
def test_gpu_mixed_indefinite_pivots(seed, diag_scale):
    """FP32 factors of nonsingular matrices with many 2x2 pivots and delays
    (FP32 pivot decisions, FP64 D^{-1}): the inertia equals the FP64
    factorisation's and FP64 refinement reaches the backward-error target.
    (For a singular matrix the rank found depends on the factor precision:
    FP32 rounding noise stays far above the zero-pivot threshold.)"""
    p, r, v = M.random_indef(600, density=0.02, seed=seed, diag_scale=diag_scale)
    ak = ssids.analyse(p, r, ssids.order_mindeg(p, r))
    fd, infd = ssids.factor(ak, v)
    fm, infm = ssids.factor(ak, v, ssids.Options(precision=ssids.PRECISION_MIXED,
                                                 max_refine=30, refine_tol=1e-15))
    assert infm.flag >= 0
    assert infm.num_two > 0
    assert (infm.num_neg, infm.matrix_rank) == (infd.num_neg, infd.matrix_rank)
    b = np.random.default_rng(seed).standard_normal((600, 3))
    x = fm.solve_refined(b)
    assert M.scaled_bwd_error(p, r, v, x, b).max() <= BWD_TOL
    fd.free()
    fm.free()
