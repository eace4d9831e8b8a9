"""Batched 4x4 block-tridiagonal solves on the GPU vs the CPU oracle (bit-exact).

hamstr_gpu_block_tridag4 stands in for the reference's
TRISOLVER::blockTridag4 / blockTridagPeriodic4 (triSolvers.cpp:769-1046).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _systems(rng, nlines, n, dominance=6.0):
    a = rng.standard_normal((nlines, n, 4, 4))
    b = rng.standard_normal((nlines, n, 4, 4)) + dominance * np.eye(4)
    c = rng.standard_normal((nlines, n, 4, 4))
    f = rng.standard_normal((nlines, n, 4))
    return a, b, c, f


@pytest.mark.parametrize("periodic", [False, True])
@pytest.mark.parametrize("n", [2, 3, 7, 64, 257])
def test_block_tridag_bitexact(oracle_lib, native_lib, periodic, n):
    import torch
    from hamstr_oop_gb300 import native
    rng = np.random.default_rng(100 + n + (1000 if periodic else 0))
    a, b, c, f = _systems(rng, 9, n)
    ta, tb, tc = (torch.from_numpy(x).cuda() for x in (a, b, c))
    tf = torch.from_numpy(f).cuda()
    native.block_tridag4(ta, tb, tc, tf, periodic)
    got = tf.cpu().numpy()
    for line in range(a.shape[0]):
        want = oracle_lib.block_tridag4(a[line], b[line], c[line], f[line], periodic)
        assert np.array_equal(got[line], want), "line %d differs" % line
    # inputs untouched
    assert np.array_equal(tb.cpu().numpy(), b) and np.array_equal(tc.cpu().numpy(), c)


def test_block_tridag_rejects_bad_sizes(native_lib):
    import torch
    from hamstr_oop_gb300 import native
    z = torch.zeros((1, 1, 4, 4), dtype=torch.float64, device="cuda")
    f = torch.zeros((1, 1, 4), dtype=torch.float64, device="cuda")
    with pytest.raises(native.HamstrError):
        native.block_tridag4(z, z, z, f, True)     # periodic line of one row


@pytest.mark.parametrize("fn", ["block_tridag4", "block_tridag4_noalloc"])
def test_block_tridag_rejects_mismatched_operands(native_lib, fn):
    """Operands smaller than F's (nlines, N) would be read past their end by
    the kernel; the binding refuses them before anything is launched."""
    import torch
    from hamstr_oop_gb300 import native
    solve = getattr(native, fn)
    full = torch.zeros((3, 8, 4, 4), dtype=torch.float64, device="cuda")
    short = torch.zeros((3, 7, 4, 4), dtype=torch.float64, device="cuda")
    f = torch.zeros((3, 8, 4), dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError):
        solve(short, full, full, f, False)
    with pytest.raises(ValueError):
        solve(full, full, short, f, True)
    with pytest.raises(ValueError):
        solve(full, full, full, f.reshape(3, 32), False)
    with pytest.raises(ValueError):
        solve(full.float(), full, full, f, False)
