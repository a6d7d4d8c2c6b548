"""The 5th-generation tensor-core path (tcgen05 MMA, tensor memory,
K-major shared-memory descriptors) used by the learned closure, checked
against a CPU product of the same BF16-rounded operands."""
import ctypes as C

import numpy as np
import pytest

from nimblesm_gb300 import engine as E

pytestmark = pytest.mark.gpu


def bf16(x):
    """Round float32 to the nearest BF16 (ties to even), returned as float32."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


@pytest.mark.parametrize("N,K", [(16, 16), (64, 32), (48, 64), (128, 64), (256, 128), (112, 128)])
def test_tcgen05_gemm(N, K):
    from nimblesm_gb300 import build as B
    B.build()
    rng = np.random.default_rng(N * 1000 + K)
    A = rng.normal(size=(128, K)).astype(np.float32)
    Bm = rng.normal(size=(N, K)).astype(np.float32)
    D = np.zeros((128, N), dtype=np.float32)
    fp = C.POINTER(C.c_float)
    rc = E.library().nsm_tc_selftest(N, K, A.ctypes.data_as(fp), Bm.ctypes.data_as(fp), D.ctypes.data_as(fp))
    assert rc == 0
    ref = bf16(A).astype(np.float64) @ bf16(Bm).astype(np.float64).T
    err = np.abs(D - ref).max() / np.abs(ref).max()
    assert err < 1e-5, err


def test_bounded_wait_times_out_and_context_stays_usable():
    """Every tensor-core wait is bounded: a wait that nothing completes runs
    out, the kernel frees its tensor memory and reports, and the next
    tensor-core kernel in the same context runs normally."""
    from nimblesm_gb300 import build as B
    B.build()
    flag = C.c_int(0)
    assert E.library().nsm_tc_wait_timeout_selftest(1000, C.byref(flag)) == 0
    assert flag.value == 1
    test_tcgen05_gemm(64, 32)
