"""GPU tests of the complex64 GEMM paths through the C ABI (mnpbem_gemm_c64).

The tcgen05 tensor-core kernel (TF32 inputs, FP32 accumulation) and the
CUDA-core kernel are compared with a complex128 NumPy product on seeded
random matrices, including ragged shapes (M, N, K not multiples of the
tile, and more output tiles than SMs so that the persistent tensor-core kernel
runs several tiles per CTA), alpha = -1 / complex alpha, and beta = 1
accumulation.
Tolerances (max |diff| / max |ref|): CUDA core 1e-5, tensor core 5e-3.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(256, 128, 64), (300, 200, 70), (1000, 64, 1000), (129, 258, 34), (640, 640, 512),
          (4000, 4, 4000), (700, 16, 900),
          # more tiles than SMs: each persistent CTA runs several tiles
          (3000, 2000, 256), (1100, 1300, 514)]


def run(lib, path, M, N, K, alpha, beta, seed):
    from mnpbem_gb300 import _lib
    rng = np.random.default_rng(seed)
    A = (rng.standard_normal((M, K)) + 1j * rng.standard_normal((M, K))).astype(np.complex64)
    B = (rng.standard_normal((K, N)) + 1j * rng.standard_normal((K, N))).astype(np.complex64)
    C0 = (rng.standard_normal((M, N)) + 1j * rng.standard_normal((M, N))).astype(np.complex64)
    C = C0.copy()
    al = np.array([alpha.real, alpha.imag], dtype=np.float32)
    be = np.array([beta, 0.0], dtype=np.float32)
    st = lib.mnpbem_gemm_c64(0, path, M, N, K, al.ctypes.data, A.ctypes.data, K, B.ctypes.data, N,
                             be.ctypes.data, C.ctypes.data, N)
    _lib.check(st)
    ref = alpha * (A.astype(np.complex128) @ B.astype(np.complex128)) + beta * C0.astype(np.complex128)
    return float(np.max(np.abs(C - ref)) / np.max(np.abs(ref)))


@pytest.mark.parametrize("shape", SHAPES)
def test_cuda_core_gemm(gpu_lib, shape):
    assert run(gpu_lib, 0, *shape, 1.0 + 0j, 0.0, 1) < 1e-5
    assert run(gpu_lib, 0, *shape, -1.0 + 0j, 1.0, 2) < 1e-5


@pytest.mark.parametrize("shape", [s for s in SHAPES if s[1] >= 64])
def test_tensor_core_gemm(gpu_lib, shape):
    e1 = run(gpu_lib, 1, *shape, 1.0 + 0j, 0.0, 3)
    e2 = run(gpu_lib, 1, *shape, -1.0 + 0j, 1.0, 4)
    e3 = run(gpu_lib, 1, *shape, 0.5 - 0.25j, 1.0, 5)
    assert e1 < 5e-3 and e2 < 5e-3 and e3 < 5e-3, (e1, e2, e3)
    # TF32 rounding must be visible (the kernel really runs at reduced precision)
    assert max(e1, e2, e3) > 1e-6


def test_tensor_core_gemm_rejects_odd_leading_dimension(gpu_lib):
    # a complex64 row of odd length is not a multiple of 16 bytes: TMA cannot stage it
    from mnpbem_gb300 import _lib
    with pytest.raises(_lib.MnpbemError) as e:
        run(gpu_lib, 1, 256, 128, 33, 1.0 + 0j, 0.0, 6)
    assert e.value.status == 7
