"""CPU tests of the oracle: analytic inertia, the reference's own CPU core
(when its sources are present), and the committed golden fixtures."""
import glob
import os

import numpy as np
import pytest

from spral_gb300 import matrices as M, ssids
import oracle

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


@pytest.mark.parametrize("nx,shift", [(16, -0.5), (64, -0.5), (20, -1.3)])
def test_oracle_2d_analytic_inertia(nx, shift):
    p, r, v = M.laplacian_2d(nx, nx, shift)
    ak = ssids.analyse(p, r, M.nd_order_grid(nx, nx))
    F = oracle.OracleFactor(ak, v)
    neg, zero, gap = M.laplacian_eig_count_2d(nx, nx, shift)
    assert F.stats["num_neg"] == neg
    assert F.stats["num_zero"] == zero
    b = np.random.default_rng(0).uniform(-1, 1, len(p) - 1)
    x = F.solve(b)
    assert M.scaled_bwd_error(p, r, v, x, b).max() < 5e-14


def test_oracle_3d_analytic_inertia():
    k = 12
    p, r, v = M.laplacian_3d(k, shift=-0.9)
    ak = ssids.analyse(p, r, M.nd_order_grid(k, k, k))
    F = oracle.OracleFactor(ak, v)
    neg, zero, gap = M.laplacian_eig_count_3d(k, k, k, -0.9)
    assert F.stats["num_neg"] == neg


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_oracle_matches_golden(path):
    g = np.load(path)
    p, r, v = g["ptr"], g["row"], g["val"]
    ak = ssids.analyse(p, r, g["order"])
    F = oracle.OracleFactor(ak, v)
    # inertia is a property of the matrix: must match the reference exactly
    assert F.stats["num_neg"] == int(g["stat_num_neg"])
    assert F.stats["num_zero"] == int(g["stat_num_zero"])
    assert F.stats["flag"] == int(g["stat_flag"])
    x = F.solve(g["b"])
    bwd = M.scaled_bwd_error(p, r, v, x, g["b"]).max()
    assert bwd < 5e-11  # tests/ssids/ssids.f90:28 err_tol
    rel = np.abs(x - g["x"]).max() / np.abs(g["x"]).max()
    assert rel < 1e-10


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_oracle_pivots_match_reference_fixture(path):
    """The oracle takes the reference's pivots: small leaf subtrees by TPP,
    children visited last first, so the pivot order, D^{-1} and the partial
    solves equal the reference's own outputs stored in the fixture."""
    g = np.load(path)
    ak = ssids.analyse(g["ptr"], g["row"], g["order"])
    F = oracle.OracleFactor(ak, g["val"])
    for k in ("num_neg", "num_two", "num_delay", "num_zero", "not_first_pass",
              "not_second_pass"):
        assert F.stats[k] == int(g["stat_" + k]), k
    piv, d = F.enquire_indef()
    assert np.array_equal(piv, g["piv_order"])
    assert np.abs(d - g["d"]).max() <= 1e-12 * np.abs(g["d"]).max()
    for job, key in ((1, "x_fwd"), (2, "x_diag"), (0, "x")):
        x = F.solve(g["b"], job=job)
        assert np.abs(x - g[key]).max() <= 1e-10 * np.abs(g[key]).max(), key


@pytest.mark.skipif(not oracle.ref_available(), reason="reference CPU core not built here")
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_oracle_vs_reference_random(seed):
    p, r, v = M.random_indef(250, density=0.03, seed=seed, diag_scale=0.01)
    ak = ssids.analyse(p, r, ssids.order_mindeg(p, r))
    F = oracle.OracleFactor(ak, v)
    R = oracle.RefFactor(ak, v)
    assert F.stats["num_neg"] == R.stats["num_neg"]
    b = np.random.default_rng(seed).uniform(-1, 1, (250, 3))
    xf, xr = F.solve(b), R.solve(b)
    assert M.scaled_bwd_error(p, r, v, xf, b).max() < 1e-12
    assert np.abs(xf - xr).max() / np.abs(xr).max() < 1e-8


def test_oracle_tpp_only_matches_app():
    p, r, v = M.random_indef(200, density=0.03, seed=7, diag_scale=0.01)
    ak = ssids.analyse(p, r, ssids.order_mindeg(p, r))
    A = oracle.OracleFactor(ak, v)
    T = oracle.OracleFactor(ak, v, options=oracle.default_options(pivot_method=3))
    assert A.stats["num_neg"] == T.stats["num_neg"]


def test_oracle_singular_action():
    # a zero row/column makes the matrix singular
    p, r, v = M.laplacian_2d(6, 6, -0.5)
    v = v.copy()
    cols = np.repeat(np.arange(36), np.diff(p))
    kill = (r == 7) | (cols == 7)
    v[kill] = 0.0
    ak = ssids.analyse(p, r, M.nd_order_grid(6, 6))
    F = oracle.OracleFactor(ak, v)
    assert F.stats["flag"] == ssids.SSIDS_WARNING_FACT_SINGULAR
    assert F.stats["num_zero"] == 1
    G = oracle.OracleFactor(ak, v, options=oracle.default_options(action=False))
    assert G.stats["flag"] == ssids.SSIDS_ERROR_SINGULAR


def test_every_called_c_entry_point_has_a_prototype():
    """ctypes passes arguments of an unprototyped function as C ints, which
    truncates 64-bit handles (a crash once the handle lies above 4 GiB, as
    it does for handles made in worker threads)."""
    import glob
    import re
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    files = (glob.glob(os.path.join(root, "spral_gb300", "*.py")) +
             glob.glob(os.path.join(root, "tests", "*.py")) +
             [os.path.join(root, "bench.py"), os.path.join(root, "__graft_entry__.py")])
    called = set()
    for f in files:
        called |= set(re.findall(r"\.(spral_ssids_gpu_\w+|spral_gb300_\w+)\(", open(f).read()))
    declared = set(re.findall(r'f\("(\w+)"',
                              open(os.path.join(root, "spral_gb300", "_native.py")).read()))
    assert called <= declared, sorted(called - declared)
