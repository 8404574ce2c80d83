"""Scaled factorisation (the subtree's `scaling` argument; cu_load_nodes_sc):
factors of S A S, solves scaled as inner_solve_cpu, inertia unchanged
(Sylvester), the solution that of the unscaled system."""
import numpy as np
import pytest

from spral_gb300 import matrices as M, ssids

pytestmark = pytest.mark.gpu


def test_gpu_scaled_factor_solves_unscaled_system():
    p, r, v = M.kkt(500, 200, seed=7)
    n = len(p) - 1
    s = M.equilibrate(p, r, v) * np.random.default_rng(1).uniform(0.5, 2.0, n)
    ak = ssids.analyse(p, r, ssids.order_mindeg(p, r))
    fk = ssids.Fkeep(ak, v, scaling=s)
    assert fk.inform.flag >= 0
    assert fk.inform.num_neg == 200  # inertia of A = inertia of S A S
    b = np.random.default_rng(2).standard_normal((n, 2))
    x = fk.solve(b)
    assert M.scaled_bwd_error(p, r, v, x, b).max() <= 1e-13
    # the factors are those of S A S: factoring the explicitly scaled matrix
    cols = np.repeat(np.arange(n), np.diff(p))
    vs = v * s[r] * s[cols]
    fs = ssids.Fkeep(ak, vs)
    y = fs.solve(b * s[:, None])
    assert np.allclose(x, y * s[:, None], rtol=1e-9, atol=1e-12)
    fs.free()
    fk.free()
