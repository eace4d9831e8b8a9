"""The 5-variable (3D strand) numerics at function level against the oracle.

hamstr_gpu_flux_roe3d / _jacobian_roe3d / _block_tridag5 stand in for
SOLVER::fluxRoe3D (interfaceFlux.cpp:176-319), jacobianRoe3D
(jacobianRoe.cpp:92-620) and TRISOLVER::blockTridag / blockTridagPeriodic
(triSolvers.cpp:443-766).  The oracle's restatements are pinned to the
reference in tests/test_oracle_vs_reference.py.  Bit for bit.
"""
import numpy as np
import pytest

from pointwise_inputs import GAMMA, blocks5, faces3d

pytestmark = pytest.mark.gpu


def _cuda(*arrays):
    import torch
    return [torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda() for a in arrays]


def test_flux_roe3d_bitexact(oracle_lib, native_lib):
    from hamstr_oop_gb300 import native
    nxyz, ql, qr = faces3d(1500, 51)
    flux, spec = native.flux_roe3d(*_cuda(nxyz, ql, qr), gamma=GAMMA)
    wf, ws = oracle_lib.flux_roe3d(nxyz, ql, qr, GAMMA)
    assert np.array_equal(flux.cpu().numpy(), wf) and np.array_equal(spec.cpu().numpy(), ws)


def test_jacobian_roe3d_bitexact(oracle_lib, native_lib):
    from hamstr_oop_gb300 import native
    nxyz, ql, qr = faces3d(1500, 52)
    lm, rm = native.jacobian_roe3d(*_cuda(nxyz, ql, qr), gamma=GAMMA)
    wl, wr = oracle_lib.jacobian_roe3d(nxyz, ql, qr, GAMMA)
    assert np.array_equal(lm.cpu().numpy(), wl) and np.array_equal(rm.cpu().numpy(), wr)


@pytest.mark.parametrize("periodic", [False, True])
@pytest.mark.parametrize("n", [2, 3, 8, 65])
def test_block_tridag5_bitexact(oracle_lib, native_lib, periodic, n):
    """Every line's solution and the scratch left in a, b, c equal one
    oracle call's."""
    from hamstr_oop_gb300 import native
    a, b, c, f = blocks5(37, n, 60 + n + 100 * int(periodic))
    ta, tb, tc, tf = _cuda(a, b, c, f)
    native.block_tridag5(ta, tb, tc, tf, periodic)
    got = [t.cpu().numpy() for t in (ta, tb, tc, tf)]
    for k in range(a.shape[0]):
        want = oracle_lib.block_tridag5(a[k], b[k], c[k], f[k], periodic)
        for g, w, what in zip(got, want, "abcf"):
            assert np.array_equal(g[k], w), (k, what)


def test_block_tridag5_rejects_bad_sizes(native_lib):
    import torch
    from hamstr_oop_gb300 import native
    z = torch.zeros((2, 1, 5, 5), dtype=torch.float64, device="cuda")
    f = torch.zeros((2, 1, 5), dtype=torch.float64, device="cuda")
    with pytest.raises(native.HamstrError):
        native.block_tridag5(z, z.clone(), z.clone(), f, True)     # periodic line of one row
    with pytest.raises(ValueError):
        native.block_tridag5(z, z.clone(), z[:, :, :4, :4].contiguous(), f, False)
