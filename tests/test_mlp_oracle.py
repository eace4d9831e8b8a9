"""The warm-start network's CPU restatement (oracle/mlp_oracle.c) against
finite differences: the oracle that checks the tensor-core gradients must
itself be right."""
import numpy as np


def test_oracle_gradient_matches_finite_differences(oracle_lib):
    rng = np.random.default_rng(0)
    P = oracle_lib.mlp_nparams()
    assert P == 256 * 5 + 256 + 2 * (256 * 256 + 256) + 4 * 256 + 4
    p = 0.1 * rng.standard_normal(P)
    f = rng.standard_normal((6, 5))
    t = rng.standard_normal((6, 4))
    _, g, _ = oracle_lib.mlp_loss_grad(p, f, t, bf16=False)
    h = 1e-6
    # parameters from every tensor: W1, b1, W2, b2, W3, b3, W4, b4
    bounds = np.cumsum([0, 1280, 256, 65536, 256, 65536, 256, 1024, 4])
    for a, b in zip(bounds[:-1], bounds[1:]):
        for i in rng.choice(np.arange(a, b), 3, replace=False):
            pp, pm = p.copy(), p.copy()
            pp[i] += h
            pm[i] -= h
            fd = (oracle_lib.mlp_loss_grad(pp, f, t, False, False)[0] -
                  oracle_lib.mlp_loss_grad(pm, f, t, False, False)[0]) / (2 * h)
            assert abs(g[i] - fd) <= 1e-5 * max(abs(fd), 1e-4), (i, g[i], fd)


def test_bf16_emulation_is_close_to_fp64(oracle_lib):
    rng = np.random.default_rng(1)
    P = oracle_lib.mlp_nparams()
    p = 0.1 * rng.standard_normal(P)
    f = rng.standard_normal((32, 5))
    t = rng.standard_normal((32, 4))
    l0, g0, _ = oracle_lib.mlp_loss_grad(p, f, t, bf16=False)
    l1, g1, _ = oracle_lib.mlp_loss_grad(p, f, t, bf16=True)
    assert abs(l1 - l0) <= 1e-2 * l0
    assert np.linalg.norm(g1 - g0) <= 3e-2 * np.linalg.norm(g0)
