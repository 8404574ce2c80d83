"""The tcgen05 tensor-core Schur update (3xTF32 split products, chunked
FP32 accumulation) against an FP64 reference of the same update."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(M, N, K, lower, chunk, seed, bn=None):
    torch = pytest.importorskip("torch")
    from spral_gb300 import _native
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((N, K)).astype(np.float32)
    C = rng.standard_normal((M, N)).astype(np.float32)
    dA = torch.tensor(A.ravel(order="F"), device="cuda")
    dB = torch.tensor(B.ravel(order="F"), device="cuda")
    dC = torch.tensor(C.ravel(order="F"), device="cuda")
    if bn is None:
        rc = _native.lib().spral_ssids_gpu_tc_gemm_f32(M, N, K, dA.data_ptr(), M, dB.data_ptr(),
                                                        N, dC.data_ptr(), M, lower, chunk, 0, None)
    else:
        rc = _native.lib().spral_ssids_gpu_tc_gemm_f32_bn(M, N, K, dA.data_ptr(), M,
                                                           dB.data_ptr(), N, dC.data_ptr(), M,
                                                           lower, chunk, 0, None, bn)
    assert rc == 0
    got = dC.cpu().numpy().reshape(M, N, order="F")
    ref = C.astype(np.float64) - A.astype(np.float64) @ B.astype(np.float64).T
    return C, got, ref


@pytest.mark.parametrize("M,N,K,lower", [(128, 128, 32, 0), (300, 200, 100, 0),
                                         (260, 260, 517, 1), (1000, 700, 64, 0),
                                         (513, 513, 300, 1), (129, 1000, 33, 0)])
@pytest.mark.parametrize("chunk", [-1, 0, 1])
def test_tc_gemm_matches_fp64(M, N, K, lower, chunk):
    C, got, ref = _run(M, N, K, lower, chunk, M + N + K)
    if lower:
        mask = np.tril(np.ones((M, N), dtype=bool))
        assert np.array_equal(got[~mask], C[~mask])   # strict upper part untouched
        got, ref = got[mask], ref[mask]
    # FP32-class accuracy: error relative to the size of the sums (N(0,1) data)
    scale = np.sqrt(K)
    assert np.abs(got - ref).max() <= 2e-5 * scale


def test_tc_gemm_chunked_accuracy_matches_fp32():
    """A deep update (3K = 3456 split products): with chunked accumulation the
    rms error stays at the level of an FP32 GEMM (rms/sqrt(K) ~ 6e-7 for an
    FP32 dot product of this depth)."""
    _, got, ref = _run(384, 384, 1152, 0, -1, 7)
    rms = np.sqrt(np.mean((got - ref) ** 2)) / np.sqrt(1152)
    assert rms <= 1.5e-6


def test_tc_crossover_is_measured_once_per_device():
    from spral_gb300 import _native
    L = _native.lib()
    a = L.spral_ssids_gpu_tc_crossover()
    b = L.spral_ssids_gpu_tc_crossover()
    assert a == b  # cached per device
    assert 64 <= a <= 513  # a size of the grid, or "never" (one past the largest)


@pytest.mark.parametrize("bn", [64, 128, 256])
@pytest.mark.parametrize("M,N,K,lower", [(300, 200, 100, 0), (513, 513, 300, 1),
                                         (129, 1000, 33, 0), (700, 700, 64, 1)])
def test_tc_gemm_tile_widths_match_fp64(bn, M, N, K, lower):
    """Every tile width the autotuner may pick gives the same FP32-class result."""
    C, got, ref = _run(M, N, K, lower, -1, M + 3 * N + K + bn, bn=bn)
    if lower:
        mask = np.tril(np.ones((M, N), dtype=bool))
        assert np.array_equal(got[~mask], C[~mask])
        got, ref = got[mask], ref[mask]
    assert np.abs(got - ref).max() <= 2e-5 * np.sqrt(K)


def test_tc_gemm_rejects_unknown_tile_width():
    from spral_gb300 import _native
    assert _native.lib().spral_ssids_gpu_tc_gemm_f32_bn(128, 128, 32, None, 128, None, 128, None,
                                                        128, 0, -1, 0, None, 96) == -4
