"""BF16 tensor-core kernels of the learned warm start (tcgen05 + TMA).

The GEMM is checked against an FP32 matrix product of the same BF16
operands: products of BF16 values are exact in FP32, so only the
accumulation order differs (tolerance 1e-5 relative to the row scale)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _gemm(native_lib, A, B, splits=1):
    import torch
    M, K = A.shape
    N = B.shape[0]
    nsp = native_lib.hamstr_mlp_gemm_splits(K, splits) if hasattr(native_lib, "hamstr_mlp_gemm_splits") else splits
    C = torch.zeros((max(nsp, 1), M, N), dtype=torch.float32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    fn = native_lib.hamstr_mlp_gemm
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p] * 2 + [ctypes.c_int] * 4 + [ctypes.c_void_p] * 3
    st = fn(A.data_ptr(), B.data_ptr(), M, N, K, splits, C.data_ptr(), err.data_ptr(), None)
    torch.cuda.synchronize()
    assert st == 0
    assert int(err.item()) == 0, "a wait timed out"
    return C


@pytest.mark.parametrize("M,N,K,splits", [(128, 16, 64, 1), (128, 64, 64, 1), (256, 128, 256, 1),
                                          (256, 256, 256, 1), (1024, 256, 256, 1), (256, 256, 4096, 8),
                                          (512, 64, 1024, 4), (384, 512, 192, 1)])
def test_gemm_matches_fp32_product(native_lib, M, N, K, splits):
    import torch
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N * 3 + K)
    A = torch.randn((M, K), generator=g, device="cuda").to(torch.bfloat16)
    B = torch.randn((N, K), generator=g, device="cuda").to(torch.bfloat16)
    C = _gemm(native_lib, A, B, splits).sum(dim=0)
    ref = A.float() @ B.float().T
    scale = ref.abs().max().item()
    err = (C - ref).abs().max().item()
    assert err <= 1e-5 * scale * max(1.0, K / 256), (err, scale)
