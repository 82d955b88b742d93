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
