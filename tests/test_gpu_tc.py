"""The tcgen05 tensor-core tile used by the learned preconditioner: one 128 x N tile of
A (bf16) * B^T (bf16) with FP32 accumulation in TMEM, against a host FP32 GEMM."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N,K", [(16, 16), (32, 48), (64, 64), (128, 32)])
def test_tcgen05_tile_matches_host_gemm(pic, N, K):
    torch = pytest.importorskip("torch")
    L = pic.library()
    f = L.pic_tc_gemm_check
    f.argtypes = [C.c_void_p] * 3 + [C.c_int, C.c_int, C.c_void_p]
    f.restype = C.c_int
    g = torch.Generator().manual_seed(N * 1000 + K)
    A = torch.randn(128, K, generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, generator=g).to(torch.bfloat16)
    ref = A.float() @ B.float().T
    dA, dB = A.cuda(), B.cuda()
    dD = torch.zeros(128, N, dtype=torch.float32, device="cuda")
    rc = f(dA.data_ptr(), dB.data_ptr(), dD.data_ptr(), N, K, None)
    assert rc == 0
    D = dD.cpu()
    assert torch.allclose(D, ref, rtol=1e-4, atol=1e-3), (D - ref).abs().max()
