"""Function-level entry points against the oracle, bit for bit.

hamstr_gpu_flux_roe2d / _jacobian_roe2d stand in for SOLVER::fluxRoe2D /
jacobianRoe2D (interfaceFlux.cpp:24-169, jacobianRoe.cpp:9-70) and
hamstr_gpu_muscl / _muscl_deriv / _weno / _weno_deriv for
RECONSTRUCTION::MUSCL / MUSCL_DERIV / WENO / WENO_DERIV
(reconstruction.cpp:16-386).  The oracle's per-face and per-line
restatements are pinned to the reference in tests/test_oracle_vs_reference.py.
"""
import numpy as np
import pytest

from pointwise_inputs import GAMMA, faces, lines

pytestmark = pytest.mark.gpu


def _cuda(*arrays):
    import torch
    return [torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda() for a in arrays]


def test_flux_roe2d_bitexact(oracle_lib, native_lib):
    from hamstr_oop_gb300 import native
    nxy, ql, qr = faces(2000, 3)
    flux, spec = native.flux_roe2d(*_cuda(nxy, ql, qr), gamma=GAMMA)
    wf, ws = oracle_lib.flux_roe2d(nxy, ql, qr, GAMMA)
    assert np.array_equal(flux.cpu().numpy(), wf)
    assert np.array_equal(spec.cpu().numpy(), ws)


def test_jacobian_roe2d_bitexact(oracle_lib, native_lib):
    from hamstr_oop_gb300 import native
    nxy, ql, qr = faces(2000, 4)
    lm, rm = native.jacobian_roe2d(*_cuda(nxy, ql, qr), gamma=GAMMA)
    wl, wr = oracle_lib.jacobian_roe2d(nxy, ql, qr, GAMMA)
    # entries the 5-variable embedding forms as exact zeros may differ in sign only
    assert np.array_equal(lm.cpu().numpy(), wl) and np.array_equal(rm.cpu().numpy(), wr)


def test_flux_roe2d_nan_is_passed_on(native_lib):
    """A negative pressure makes the sound speed NaN: the reference exits
    (interfaceFlux.cpp:117-124); the entry point leaves the NaN in spec."""
    from hamstr_oop_gb300 import native
    nxy, ql, qr = faces(8, 5)
    ql[3, 3] = -5.0
    _, spec = native.flux_roe2d(*_cuda(nxy, ql, qr))
    s = spec.cpu().numpy()
    assert np.isnan(s[3]) and np.all(np.isfinite(np.delete(s, 3)))


CASES = [("muscl", 1, 2, 0.25), ("muscl", 3, 5, 0.25), ("muscl", 0, 1, 0.0), ("muscl_deriv", 1, 2, 0.25),
         ("muscl_deriv", 2, 1, 0.0), ("weno", 2, 1, 0.25), ("weno", 4, 1, 0.25), ("weno_deriv", 2, 1, 0.25)]


@pytest.mark.parametrize("name,is_,ie_off,qt", CASES)
@pytest.mark.parametrize("imax", [7, 33, 130])
def test_reconstruction_lines_bitexact(oracle_lib, native_lib, name, is_, ie_off, qt, imax):
    """Every line of a batch equals one oracle call on it: ql, qr and the
    f2 work array, with entries outside the written range left as they were."""
    from hamstr_oop_gb300 import native
    f, dq, prior = lines(12, imax, 4, 7 + imax)
    ie = imax - ie_off
    eps = 1e-10 if name != "weno" else 0.0
    tf, tdq, tql, tqr, tf2 = _cuda(f, dq, prior[0], prior[1], prior[2])
    native.reconstruct(name, tf, tql, tqr, is_, ie, dq=tdq, f2=tf2, qt=qt, eps=eps)
    got = [t.cpu().numpy() for t in (tql, tqr, tf2)]
    for k in range(f.shape[0]):
        want = oracle_lib.recon_line(name, f[k], is_, ie, dq=dq[k], qt=qt, eps=eps, ql=prior[0, k],
                                     qr=prior[1, k], f2=prior[2, k])
        for g, w, what in zip(got, want, ("ql", "qr", "f2")):
            assert np.array_equal(g[k], w), (name, k, what)


def test_reconstruction_rejects_out_of_range_indices(native_lib):
    """Index ranges where the reference reads outside the line (or reads
    left-over work-array entries) are refused before any launch."""
    from hamstr_oop_gb300 import native
    f, dq, prior = lines(2, 9, 4, 1)
    tf, tdq, tql, tqr, tf2 = _cuda(f, dq, prior[0], prior[1], prior[2])
    bad = [("muscl", 0, 7, 0.25), ("muscl", 1, 8, 0.25), ("muscl_deriv", 1, 8, 0.25), ("weno", 1, 8, 0.25),
           ("weno_deriv", 2, 9, 0.25), ("muscl", 2, 9, 0.0)]
    for name, is_, ie, qt in bad:
        with pytest.raises(native.HamstrError) as ei:
            native.reconstruct(name, tf, tql, tqr, is_, ie, dq=tdq, f2=tf2, qt=qt)
        assert ei.value.status == -1, (name, is_, ie)
