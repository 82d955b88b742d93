"""Tensor-core conventions (tcgen05 kind::tf32, TMEM accumulators) on one 128 x N x K tile.

Split TF32 (3 products) must match the float64 product to 2e-6 relative (Frobenius);
plain TF32 to 2e-3.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N,K", [(16, 8), (64, 56), (256, 56), (96, 24)])
def test_tc_gemm_tile(built_lib, N, K):
    from seissol_gb300.lib import tc_gemm_check
    rng = np.random.default_rng(N * 100 + K)
    A = rng.standard_normal((128, K)).astype(np.float32)
    B = rng.standard_normal((N, K)).astype(np.float32)
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    d3 = tc_gemm_check(A, B, terms=3)
    err3 = np.linalg.norm(d3 - ref) / np.linalg.norm(ref)
    assert err3 < 2e-6, err3
    d1 = tc_gemm_check(A, B, terms=1)
    err1 = np.linalg.norm(d1 - ref) / np.linalg.norm(ref)
    assert err1 < 2e-3, err1
    assert err1 > err3


def _int_tile(M, N, K, seed):
    rng = np.random.default_rng(seed)
    A = rng.integers(-3, 4, (M, K)).astype(np.float32)
    B = rng.integers(-3, 4, (N, K)).astype(np.float32)
    return A, B, A.astype(np.float64) @ B.astype(np.float64).T


def _m64_lane(k):
    return 32 * (k // 16) + k % 16


@pytest.mark.parametrize("M,N,K,b_mn,a_mn", [(128, 80, 64, 0, 0), (64, 72, 64, 0, 0), (64, 72, 48, 0, 0),
                                             (64, 128, 32, 0, 0), (128, 64, 32, 1, 0), (64, 72, 64, 1, 0),
                                             (64, 64, 96, 0, 1), (128, 64, 32, 0, 1), (64, 72, 96, 1, 1)])
def test_tc_f16_operand_layouts(built_lib, M, N, K, b_mn, a_mn):
    """kind::f16 tiles with exact small-integer operands: the result is exact, M = 128 rows sit on
    lanes 0..127, M = 64 rows on lanes 32 (k / 16) + k % 16 (16 per lane quarter; the kernels'
    epilogues read them there), and an MN-major A or B operand reads with the descriptor's leading
    offset holding the stride between K groups."""
    from seissol_gb300.lib import tc_layout_check
    A, B, ref = _int_tile(M, N, K, M * 1000 + N + K)
    D = tc_layout_check(A, B, b_mn=b_mn, lbo_is_k=1, a_mn=a_mn)[:, :N]
    lanes = [k if M == 128 else _m64_lane(k) for k in range(M)]
    assert np.array_equal(D[lanes], ref)
