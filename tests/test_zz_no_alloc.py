"""sei_mlp_gradient_noalloc (static device scratch, no allocation) against sei_mlp_gradient, through
the C ABI, on two calls in a row (the second smaller, so that a stale accumulator or sample of the
first call would show).  Tolerances are those of the gradient tests: 1e-4 relative L2 on the
gradient and 1e-5 relative on the loss (both FP32 with atomically accumulated sums, whose order
differs between calls).  A request above the fixed capacity returns SEI_ERR_CAPACITY.

Two more properties of the entry point itself: once its module is loaded (first call), further
calls leave the device's free memory unchanged, so nothing is allocated; and a call returns while
a long kernel is still running on a caller's stream created with the default (blocking) flags, so
the call does not wait for the caller's other streams.

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


def _torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device visible to torch")
    return torch


def test_noalloc_calls_leave_device_free_memory_unchanged(built_lib):
    from seissol_gb300 import load_library
    torch = _torch_cuda()
    lib = load_library()
    p = np.ascontiguousarray(M.glorot(5), np.float32)
    norm = np.ascontiguousarray(M.normalisation(_samples(300, 1), 1e-6), np.float32)
    S = _samples(4096, 6)
    assert _call(lib.sei_mlp_gradient_noalloc, p, norm, S)[0] == 0  # first call: module load and set-up
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert _call(lib.sei_mlp_gradient_noalloc, p, norm, S)[0] == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_noalloc_does_not_wait_for_a_blocking_caller_stream(built_lib):
    from seissol_gb300 import load_library
    torch = _torch_cuda()
    lib = load_library()
    p = np.ascontiguousarray(M.glorot(6), np.float32)
    norm = np.ascontiguousarray(M.normalisation(_samples(300, 1), 1e-6), np.float32)
    S = _samples(2048, 7)
    assert _call(lib.sei_mlp_gradient_noalloc, p, norm, S)[0] == 0
    torch.cuda.synchronize()
    caller = torch.cuda.Stream()  # default flags: a blocking stream
    done = torch.cuda.Event()
    with torch.cuda.stream(caller):
        torch.cuda._sleep(1_500_000_000)  # a bounded spin of about a second on one SM
        done.record(caller)
    rc, g, _ = _call(lib.sei_mlp_gradient_noalloc, p, norm, S)
    still_running = not done.query()
    caller.synchronize()
    assert rc == 0 and np.all(np.isfinite(g))
    assert still_running, "the call waited for the caller's blocking stream"
