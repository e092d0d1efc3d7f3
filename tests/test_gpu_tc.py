"""tcgen05 building blocks (matx_gb300/csrc/tc.cuh): a test-only self-test GEMM
(tests/tc_selftest/) against an FP64 torch reference.

bf16 (one term) must match the FP64 product of the bf16-rounded operands closely
and the FP32 product to bf16 accuracy; bf16x3 (three terms, six products) must
recover FP32 accuracy (rel-L2 <= 1e-6 against FP64)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tc_selftest.build import build
    so = ctypes.CDLL(build())
    so.tc_gemm_selftest.restype = ctypes.c_int
    so.tc_gemm_selftest.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int32] * 4 + [ctypes.c_void_p] * 2
    return so


def run(lib, A, B, terms):
    import torch
    M, K = A.shape
    N = B.shape[0]
    C = torch.zeros(M, N, dtype=torch.float32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.tc_gemm_selftest(ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(B.data_ptr()),
                              ctypes.c_void_p(C.data_ptr()), M, N, K, terms, ctypes.c_void_p(st.data_ptr()), s)
    assert rc == 0, rc
    torch.cuda.synchronize()
    assert int(st.item()) == 0, "bounded wait gave up"
    return C


def rel(a, b):
    return float((a - b).norm() / b.norm())


@pytest.mark.parametrize("MNK", [(128, 16, 16), (128, 64, 32), (256, 128, 64), (128, 256, 64), (384, 48, 48)])
def test_tc_gemm_bf16_and_bf16x3(lib, MNK):
    import torch
    M, N, K = MNK
    g = torch.Generator(device="cuda").manual_seed(M + N + K)
    A = torch.randn(M, K, device="cuda", generator=g)
    B = torch.randn(N, K, device="cuda", generator=g)
    ref = A.double() @ B.double().T
    ref_b = A.bfloat16().double() @ B.bfloat16().double().T
    c1 = run(lib, A, B, 1)
    assert rel(c1.double(), ref_b) < 1e-6  # exact bf16 products, FP32 accumulation
    assert rel(c1.double(), ref) < 2e-2
    c3 = run(lib, A, B, 3)
    assert rel(c3.double(), ref) < 1e-6
