"""Failure detection without a GPU fault: bounded waits that give up and
report an error status (the context stays usable), and a host-injected
allocation failure mapped to SSIDS_ERROR_ALLOCATION."""
import numpy as np
import pytest

from spral_gb300 import _native, matrices as M, ssids

pytestmark = pytest.mark.gpu


def _small_factor_ok():
    p, r, v = M.laplacian_2d(12, 12, -0.5)
    ak = ssids.analyse(p, r, M.nd_order_grid(12, 12))
    fk, inf = ssids.factor(ak, v)
    b = np.random.default_rng(0).uniform(-1, 1, 144)
    ok = inf.flag == 0 and M.scaled_bwd_error(p, r, v, fk.solve(b), b).max() <= 5e-14
    fk.free()
    return ok


@pytest.mark.parametrize("probe", ["spral_ssids_gpu_mbar_timeout_probe",
                                   "spral_ssids_gpu_wave_timeout_probe"])
def test_gpu_bounded_wait_gives_up_with_error_status(probe):
    lib = _native.lib()
    # a barrier / flag that nothing completes: the wait must give up
    assert getattr(lib, probe)(1 << 12) == ssids.SSIDS_ERROR_CUDA_UNKNOWN
    # and the context is still usable
    assert _small_factor_ok()


def test_gpu_injected_allocation_failure_reports_minus_50():
    lib = _native.lib()
    p, r, v = M.laplacian_3d(10, shift=-0.3)
    ak = ssids.analyse(p, r, M.nd_order_grid(10, 10, 10))
    # the first allocation fails: no handle at all (create_num_subtree
    # returns NULL with stats.flag = -50)
    lib.spral_ssids_gpu_inject_alloc_failure(0)
    try:
        with pytest.raises(RuntimeError, match="flag -50"):
            ssids.factor(ak, v)
        # a later one fails inside the factorisation: the handle reports -50
        lib.spral_ssids_gpu_inject_alloc_failure(2)
        fk, inf = ssids.factor(ak, v)
        assert inf.flag == ssids.SSIDS_ERROR_ALLOCATION
        fk.free()
    finally:
        lib.spral_ssids_gpu_inject_alloc_failure(-1)
    fk, inf = ssids.factor(ak, v)
    assert inf.flag == 0
    fk.free()
    assert _small_factor_ok()
