"""Tensor-core tile self-test (tcgen05.mma, TMEM, 128B-swizzled operands)
against a torch fp32 matmul of the same bf16 inputs."""
import ctypes as C

import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N,K", [(256, 128), (64, 192), (16, 64), (128, 256)])
def test_umma_tile_matches_torch(N, K):
    from analyticmesh_gb300 import _lib
    L = _lib.lib()
    L.am_selftest_umma.argtypes = [C.c_void_p] * 3 + [C.c_int, C.c_int]
    g = torch.Generator(device="cuda").manual_seed(N * 1000 + K)
    A = torch.randn(128, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    D = torch.empty(128, N, device="cuda", dtype=torch.float32)
    rc = L.am_selftest_umma(A.data_ptr(), B.data_ptr(), D.data_ptr(), N, K)
    assert rc == 0
    ref = A.float() @ B.float().t()
    torch.testing.assert_close(D, ref, rtol=1e-5, atol=1e-4)


def test_umma_accumulation_bits():
    """Effective accumulation precision of tcgen05 kind::f16 (bf16 in, fp32
    accumulate): D = 1*1 + 2^-k * 1 over one K=16 MMA.  Records the largest
    k for which the small term survives (fp32 round-to-nearest keeps k <= 23)."""
    from analyticmesh_gb300 import _lib
    L = _lib.lib()
    L.am_selftest_umma.argtypes = [C.c_void_p] * 3 + [C.c_int, C.c_int]
    K, N = 64, 16
    survived = []
    for k in range(8, 26):
        A = torch.zeros(128, K, device="cuda")
        A[:, 0] = 1.0
        A[:, 1] = 2.0 ** -k
        B = torch.zeros(N, K, device="cuda")
        B[:, 0] = 1.0
        B[:, 1] = 1.0
        D = torch.empty(128, N, device="cuda")
        assert L.am_selftest_umma(A.bfloat16().data_ptr(), B.bfloat16().data_ptr(), D.data_ptr(), N, K) == 0
        if float(D[0, 0]) - 1.0 == 2.0 ** -k:
            survived.append(k)
    bits = max(survived) if survived else 0
    print("tcgen05 bf16 accumulation keeps 1 + 2^-k up to k =", bits)
    assert bits >= 8


@pytest.mark.parametrize("N,K", [(256, 128), (64, 192), (16, 64), (128, 256), (48, 64), (160, 128)])
def test_umma_tile_mn_major_b_matches_torch(N, K):
    """B staged MN-major (the composition's operand layout), including MN
    extents that fill only part of the last 64-wide atom."""
    from analyticmesh_gb300 import _lib
    L = _lib.lib()
    L.am_selftest_umma_bmn.argtypes = [C.c_void_p] * 3 + [C.c_int, C.c_int]
    g = torch.Generator(device="cuda").manual_seed(N * 1000 + K + 7)
    A = torch.randn(128, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    D = torch.empty(128, N, device="cuda", dtype=torch.float32)
    assert L.am_selftest_umma_bmn(A.data_ptr(), B.data_ptr(), D.data_ptr(), N, K) == 0
    torch.testing.assert_close(D, A.float() @ B.float().t(), rtol=1e-5, atol=1e-4)
