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


def _data(n, seed):
    import torch
    rng = np.random.default_rng(seed)
    f = rng.uniform(-1.0, 1.0, (n, 5)).astype(np.float32)
    # a smooth target of the inputs
    t = np.stack([np.sin(f[:, 0] + f[:, 2]), f[:, 1] * f[:, 3], np.cos(f[:, 4]) - 0.5, f[:, 0] * 0.3 + f[:, 2] ** 2],
                 axis=1).astype(np.float32)
    return f, t, torch.from_numpy(f).cuda(), torch.from_numpy(t).cuda()


def test_forward_and_gradient_match_the_oracle(native_lib, oracle_lib):
    from hamstr_oop_gb300 import native
    net = native.Mlp(batch_capacity=512, seed=7)
    p = net.get_params().astype(np.float64)
    f, t, fd, td = _data(384, 3)
    y_gpu = net.forward(fd).cpu().numpy()
    loss_o, g_o, y_o = oracle_lib.mlp_loss_grad(p, f, t, bf16=True)
    assert np.max(np.abs(y_gpu - y_o)) <= 1e-2 * np.max(np.abs(y_o)) + 1e-3
    loss_g = net.grad(fd, td)
    assert abs(loss_g - loss_o) <= 2e-3 * loss_o, (loss_g, loss_o)
    g_g = net.get_grads().astype(np.float64)
    bounds = np.cumsum([0, 1280, 256, 65536, 256, 65536, 256, 1024, 4])
    names = ["W1", "b1", "W2", "b2", "W3", "b3", "W4", "b4"]
    for name, a, b in zip(names, bounds[:-1], bounds[1:]):
        rel = np.linalg.norm(g_g[a:b] - g_o[a:b]) / max(np.linalg.norm(g_o[a:b]), 1e-30)
        assert rel <= 2e-2, (name, rel)


def test_training_reduces_the_loss(native_lib):
    from hamstr_oop_gb300 import native
    net = native.Mlp(batch_capacity=4096, seed=11)
    f, t, fd, td = _data(20000, 5)
    first = None
    for step in range(300):
        loss = net.train_step(fd, td, batch=2048, seed=99, step=step, lr=2e-3)
        if first is None:
            first = loss
    assert loss < 0.1 * first, (first, loss)
