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
