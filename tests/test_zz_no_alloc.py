"""sei_mlp_gradient_noalloc (static device scratch, no allocation) against sei_mlp_gradient, through
the C ABI, on two calls in a row (the second smaller, so that a stale accumulator or sample of the
first call would show).  Tolerances are those of the gradient tests: 1e-4 relative L2 on the
gradient and 1e-5 relative on the loss (both FP32 with atomically accumulated sums, whose order
differs between calls).  A request above the fixed capacity returns SEI_ERR_CAPACITY.

This file is named to be collected last and also runs alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import mlp as M
from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu

SEI_ERR_CAPACITY = -8
MAX_SAMPLES = 16384


def _samples(n, seed):
    rng = np.random.default_rng(seed)
    return np.ascontiguousarray(np.stack([rng.uniform(-120e6, -40e6, n), rng.uniform(20e6, 75e6, n),
                                          rng.uniform(0.3, 0.9, n), rng.uniform(0.008, 0.02, n), np.full(n, 0.014),
                                          rng.uniform(-40, 1, n)], axis=1), np.float32)


def _call(fn, p, norm, S):
    g = np.zeros(p.shape[0], np.float32)
    loss = C.c_float()
    rc = fn(p.ctypes.data, norm.ctypes.data, S.ctypes.data, S.shape[0], g.ctypes.data, C.byref(loss))
    return rc, g, loss.value


def test_noalloc_gradient_matches_allocating_entry_point(built_lib):
    from seissol_gb300 import load_library
    lib = load_library()
    norm = np.ascontiguousarray(M.normalisation(_samples(500, 1), 1e-6), np.float32)
    for call, (n, seed) in enumerate(((MAX_SAMPLES, 2), (700, 3))):
        p = np.ascontiguousarray(M.glorot(10 + call), np.float32)
        S = _samples(n, seed)
        rc_ref, g_ref, l_ref = _call(lib.sei_mlp_gradient, p, norm, S)
        rc, g, l = _call(lib.sei_mlp_gradient_noalloc, p, norm, S)
        assert rc_ref == 0 and rc == 0, (rc_ref, rc)
        assert abs(l - l_ref) <= 1e-5 * abs(l_ref), (call, l, l_ref)
        assert rel_l2(g, g_ref) < 1e-4, (call, rel_l2(g, g_ref))


def test_noalloc_rejects_more_samples_than_its_scratch_holds(built_lib):
    from seissol_gb300 import load_library
    lib = load_library()
    p = np.ascontiguousarray(M.glorot(1), np.float32)
    norm = np.ascontiguousarray(M.normalisation(_samples(100, 1), 1e-6), np.float32)
    rc, _, _ = _call(lib.sei_mlp_gradient_noalloc, p, norm, _samples(MAX_SAMPLES + 1, 4))
    assert rc == SEI_ERR_CAPACITY
