"""GPU tests of the complex64 GEMM paths through the C ABI (mnpbem_gemm_c64).

The tcgen05 tensor-core kernels (TF32 inputs, FP32 accumulation; one CTA per
128 x 256 tile, or CTA pairs per 256 x 256 tile; FP16 inputs scaled per row /
column, kind::f16, path 4) and the CUDA-core kernel are compared with a
complex128 NumPy product on seeded
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


def run(lib, path, M, N, K, alpha, beta, seed, ldc=None):
    """max relative error of one product; ``ldc`` > N pads the rows of C (the
    padding must come back untouched)."""
    from mnpbem_gb300 import _lib
    ldc = N if ldc is None else ldc
    rng = np.random.default_rng(seed)
    A = (rng.standard_normal((M, K)) + 1j * rng.standard_normal((M, K))).astype(np.complex64)
    B = (rng.standard_normal((K, N)) + 1j * rng.standard_normal((K, N))).astype(np.complex64)
    C0 = (rng.standard_normal((M, ldc)) + 1j * rng.standard_normal((M, ldc))).astype(np.complex64)
    C = C0.copy()
    al = np.array([alpha.real, alpha.imag], dtype=np.float32)
    be = np.array([beta, 0.0], dtype=np.float32)
    st = lib.mnpbem_gemm_c64(0, path, M, N, K, al.ctypes.data, A.ctypes.data, K, B.ctypes.data, N,
                             be.ctypes.data, C.ctypes.data, ldc)
    _lib.check(st)
    assert np.array_equal(C[:, N:], C0[:, N:])
    ref = alpha * (A.astype(np.complex128) @ B.astype(np.complex128)) + beta * C0[:, :N].astype(np.complex128)
    return float(np.max(np.abs(C[:, :N] - ref)) / np.max(np.abs(ref)))


@pytest.mark.parametrize("shape", SHAPES)
def test_cuda_core_gemm(gpu_lib, shape):
    assert run(gpu_lib, 0, *shape, 1.0 + 0j, 0.0, 1) < 1e-5
    assert run(gpu_lib, 0, *shape, -1.0 + 0j, 1.0, 2) < 1e-5


@pytest.mark.parametrize("path", [1, 2, 3, 4])
@pytest.mark.parametrize("shape", [s for s in SHAPES if s[1] >= 64])
def test_tensor_core_gemm(gpu_lib, shape, path):
    # paths 2, 3: CTA pairs (cta_group::2, 256 x 256 tiles) for M >= 256, TMA or
    # load-store-path epilogue
    e1 = run(gpu_lib, path, *shape, 1.0 + 0j, 0.0, 3)
    e2 = run(gpu_lib, path, *shape, -1.0 + 0j, 1.0, 4)
    e3 = run(gpu_lib, path, *shape, 0.5 - 0.25j, 1.0, 5)
    assert e1 < 5e-3 and e2 < 5e-3 and e3 < 5e-3, (e1, e2, e3)
    # TF32 rounding must be visible (the kernel really runs at reduced precision)
    assert max(e1, e2, e3) > 1e-6


@pytest.mark.parametrize("path", [1, 2, 3, 4])
def test_tensor_core_gemm_odd_columns_padded_rows(gpu_lib, path):
    # N odd with an even leading dimension: the last complex column of a row is
    # a lone pair of floats at the edge of the tile, and the padding of C stays
    for beta, seed in ((0.0, 7), (1.0, 8)):
        e = run(gpu_lib, path, 520, 203, 96, 1.0 - 0.5j, beta, seed, ldc=206)
        assert e < 5e-3, (beta, e)


def test_tensor_core_gemm_rejects_odd_leading_dimension(gpu_lib):
    # a complex64 row of odd length is not a multiple of 16 bytes: TMA cannot stage it
    from mnpbem_gb300 import _lib
    with pytest.raises(_lib.MnpbemError) as e:
        run(gpu_lib, 1, 256, 128, 33, 1.0 + 0j, 0.0, 6)
    assert e.value.status == 7


def test_fp16_path_scales_rows_and_columns(gpu_lib):
    """Rows and columns spanning 1e-6 .. 1e6 (far outside FP16's range without
    scaling): the per-row / per-column powers of two keep the product at the
    accuracy of the 10-bit significand, row by row."""
    from mnpbem_gb300 import _lib
    rng = np.random.default_rng(21)
    M, N, K = 384, 320, 200
    ra = 10.0 ** rng.uniform(-6, 6, M)
    cb = 10.0 ** rng.uniform(-6, 6, N)
    A = ((rng.standard_normal((M, K)) + 1j * rng.standard_normal((M, K))) * ra[:, None]).astype(np.complex64)
    B = ((rng.standard_normal((K, N)) + 1j * rng.standard_normal((K, N))) * cb[None, :]).astype(np.complex64)
    C = np.zeros((M, N), dtype=np.complex64)
    al = np.array([1.0, 0.0], dtype=np.float32)
    be = np.array([0.0, 0.0], dtype=np.float32)
    _lib.check(gpu_lib.mnpbem_gemm_c64(0, 4, M, N, K, al.ctypes.data, A.ctypes.data, K, B.ctypes.data, N,
                                       be.ctypes.data, C.ctypes.data, N))
    ref = A.astype(np.complex128) @ B.astype(np.complex128)
    err = np.abs(C - ref) / (ra[:, None] * cb[None, :] * np.sqrt(K))
    assert np.max(err) < 5e-3
