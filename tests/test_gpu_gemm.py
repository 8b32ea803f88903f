"""The LU's complex64 trailing-update kernels (SIMT, tcgen05 3xFP16 and
3xTF32) on their own, through the diagnostic C-ABI entry point, against a
complex128 product. The split products keep FP32-level accuracy (FP16 and TF32
both carry 10 explicit mantissa bits): the tolerance is 2e-6 relative."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run(lib, ctx, A, B, Cm, engine):
    m, k = A.shape
    n = B.shape[1]
    a = np.asfortranarray(A, np.complex64)
    b = np.asfortranarray(B, np.complex64)
    c = np.array(Cm, dtype=np.complex64, order="F", copy=True)
    p = lambda x: x.ctypes.data_as(C.c_void_p)  # noqa: E731
    rc = lib.frico_gpu_debug_cgemm(ctx, m, n, k, p(a), p(b), p(c), engine)
    assert rc == 0, lib.frico_gpu_last_error(ctx).decode()
    return c


@pytest.fixture(scope="module")
def ctx(gpu_lib):
    h = C.c_void_p()
    assert gpu_lib.frico_gpu_ctx_create(C.byref(h), 0, None) == 0
    yield h
    gpu_lib.frico_gpu_ctx_destroy(h)


@pytest.mark.parametrize("m,n,k", [(128, 128, 64), (300, 200, 64), (1000, 700, 64), (257, 129, 50), (64, 300, 17),
                                   (1000, 700, 128), (777, 513, 128),
                                   (2048, 1536, 64)])
@pytest.mark.parametrize("engine", ["simt", "tc", "tc_f16"])
def test_cgemm(gpu_lib, ctx, m, n, k, engine):
    from frico_gb300 import _abi
    rng = np.random.default_rng(m * 7 + n * 3 + k)
    A = (rng.standard_normal((m, k)) + 1j * rng.standard_normal((m, k))).astype(np.complex64)
    B = (rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n))).astype(np.complex64)
    C0 = (rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))).astype(np.complex64)
    ref = C0.astype(np.complex128) - A.astype(np.complex128) @ B.astype(np.complex128)
    eng = {"simt": _abi.GEMM_SIMT, "tc": _abi.GEMM_TC, "tc_f16": _abi.GEMM_TC_F16}[engine]
    out = run(gpu_lib, ctx, A, B, C0, eng)
    err = np.abs(out - ref).max() / np.abs(ref).max()
    # FP32 accumulation (both engines): rounding grows with the K terms summed
    assert err < 2e-6 * max(1.0, k / 64) ** 0.75, err
