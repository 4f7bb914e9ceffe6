"""Failure detection on the GPU without a fault: every pipelined kernel of the
library waits on mbarriers through one bounded-wait helper; when a wait runs
out, the kernel records an error code, returns, and the host reports
MNPBEM_ERR_TIMEOUT with the context still usable.

The self-test entry point makes such a wait run out (a barrier that nothing
completes, 2 ms limit) and the test checks the status, the message, and that
a tensor-core product right after still gives correct results."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MNPBEM_ERR_TIMEOUT = 6


def test_bounded_wait_expiry_reports_timeout(gpu_lib):
    st = gpu_lib.mnpbem_selftest_bounded_wait(0, 2000)
    assert st == MNPBEM_ERR_TIMEOUT
    assert b"expired" in gpu_lib.mnpbem_last_error()
    # twice in a row: nothing is left behind by the first expiry
    assert gpu_lib.mnpbem_selftest_bounded_wait(0, 500) == MNPBEM_ERR_TIMEOUT


def test_context_usable_after_expiry(gpu_lib):
    from mnpbem_gb300 import _lib
    assert gpu_lib.mnpbem_selftest_bounded_wait(0, 1000) == MNPBEM_ERR_TIMEOUT
    rng = np.random.default_rng(11)
    M, N, K = 512, 256, 128
    A = (rng.standard_normal((M, K)) + 1j * rng.standard_normal((M, K))).astype(np.complex64)
    B = (rng.standard_normal((K, N)) + 1j * rng.standard_normal((K, N))).astype(np.complex64)
    C = np.zeros((M, N), dtype=np.complex64)
    al = np.array([1.0, 0.0], dtype=np.float32)
    be = np.array([0.0, 0.0], dtype=np.float32)
    _lib.check(gpu_lib.mnpbem_gemm_c64(0, 1, M, N, K, al.ctypes.data, A.ctypes.data, K, B.ctypes.data, N,
                                       be.ctypes.data, C.ctypes.data, N))
    ref = A.astype(np.complex128) @ B.astype(np.complex128)
    assert np.max(np.abs(C - ref)) / np.max(np.abs(ref)) < 5e-3
