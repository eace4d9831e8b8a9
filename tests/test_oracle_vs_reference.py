"""The C restatement (oracle/hamstr_oracle.c) against the reference compiled
from its own sources: bit-identical arrays.  Runs where the reference sources
are present; elsewhere the committed golden fixtures pin the restatement."""
import numpy as np
import pytest

from conftest import has_reference_sources

pytestmark = pytest.mark.skipif(not has_reference_sources(), reason="reference sources not present")


@pytest.mark.parametrize("order,loop_start", [(1, None), (3, None), (3, 0), (5, None)])
def test_march_bitexact(make_case, oracle_lib, order, loop_start):
    case = make_case(20, 6, order=order, CFL=10.0, msweep=2, loop_start=loop_start)
    ref = oracle_lib.OracleCase(case, "reference")
    port = oracle_lib.OracleCase(case, "port")
    assert ref.sizes == port.sizes and ref.params == port.params
    for name in ("faces", "chainConn", "faceStartPerChain", "c2chain", "bFaces"):
        assert np.array_equal(ref.get_int(name), port.get_int(name)), name
    for name in ("x", "vol", "normVec", "refMtx", "q"):
        assert np.array_equal(ref.get(name), port.get(name)), name
    for _ in range(6):
        assert np.array_equal(ref.step(), port.step())
    for name in ("q", "r", "r0", "dq", "sigma", "ff"):
        assert np.array_equal(ref.get(name), port.get(name)), name


@pytest.mark.parametrize("periodic", [False, True])
def test_block_tridag_bitexact(oracle_lib, periodic):
    rng = np.random.default_rng(5)
    for n in (2, 3, 4, 17):
        a = rng.standard_normal((n, 4, 4))
        b = rng.standard_normal((n, 4, 4)) + 5 * np.eye(4)
        c = rng.standard_normal((n, 4, 4))
        f = rng.standard_normal((n, 4))
        x1 = oracle_lib.block_tridag4(a, b, c, f, periodic, "port")
        x2 = oracle_lib.block_tridag4(a, b, c, f, periodic, "reference")
        assert np.array_equal(x1, x2)


@pytest.mark.parametrize("order", [1, 3, 5])
def test_explicit_schemes_bitexact(make_case, oracle_lib, order):
    case = make_case(20, 6, order=order, CFL=0.8)
    ref = oracle_lib.OracleCase(case, "reference")
    port = oracle_lib.OracleCase(case, "port")
    for scheme in ("euler", "rk3", "rk3", "euler"):
        assert np.array_equal(ref.step_explicit(scheme), port.step_explicit(scheme))
    for name in ("q", "qt", "r", "sigma"):
        assert np.array_equal(ref.get(name), port.get(name)), name


def test_flux_and_jacobian_per_face_bitexact(make_case, oracle_lib):
    """ho_flux_roe2d / ho_jacobian_roe2d against SOLVER::fluxRoe2D /
    jacobianRoe2D of the reference, face by face."""
    from pointwise_inputs import faces
    ref = oracle_lib.OracleCase(make_case(16, 4), "reference")
    nxy, ql, qr = faces(300, 21)
    f1, s1 = oracle_lib.flux_roe2d(nxy, ql, qr, kind="port")
    f2, s2 = oracle_lib.flux_roe2d(nxy, ql, qr, kind="reference", case=ref)
    assert np.array_equal(f1, f2) and np.array_equal(s1, s2)
    l1, r1 = oracle_lib.jacobian_roe2d(nxy, ql, qr, kind="port")
    l2, r2 = oracle_lib.jacobian_roe2d(nxy, ql, qr, kind="reference", case=ref)
    assert np.array_equal(l1, l2) and np.array_equal(r1, r2)


@pytest.mark.parametrize("name,is_,ie_off,qt", [("muscl", 1, 2, 0.25), ("muscl", 1, 1, 0.25), ("muscl", 0, 1, 0.0),
                                                ("muscl_deriv", 2, 2, 0.25), ("muscl_deriv", 1, 1, 0.0),
                                                ("weno", 2, 1, 0.25), ("weno_deriv", 2, 1, 0.25),
                                                ("weno_deriv", 3, 1, 0.25)])
def test_reconstructions_per_line_bitexact(oracle_lib, name, is_, ie_off, qt):
    """ho_*_line against RECONSTRUCTION::* of the reference on one line,
    outputs and the f2 work array (ie = imax - ie_off)."""
    from pointwise_inputs import lines
    f, dq, prior = lines(3, 23, 4, 9)
    for k in range(f.shape[0]):
        kw = dict(dq=dq[k], qt=qt, th=1.0 / 3.0, eps=1e-10, ql=prior[0, k], qr=prior[1, k], f2=prior[2, k])
        ie = f.shape[1] - ie_off
        a = oracle_lib.recon_line(name, f[k], is_, ie, kind="port", **kw)
        b = oracle_lib.recon_line(name, f[k], is_, ie, kind="reference", **kw)
        for x, y, what in zip(a, b, ("ql", "qr", "f2")):
            assert np.array_equal(x, y), (name, k, what)


def test_flux_and_jacobian_3d_per_face_bitexact(make_case, oracle_lib):
    """ho_flux_roe3d / ho_jacobian_roe3d against SOLVER::fluxRoe3D /
    jacobianRoe3D of the reference (5 variables, any normal)."""
    from pointwise_inputs import faces3d
    ref = oracle_lib.OracleCase(make_case(16, 4), "reference")
    nxyz, ql, qr = faces3d(300, 41)
    f1, s1 = oracle_lib.flux_roe3d(nxyz, ql, qr, kind="port")
    f2, s2 = oracle_lib.flux_roe3d(nxyz, ql, qr, kind="reference", case=ref)
    assert np.array_equal(f1, f2) and np.array_equal(s1, s2)
    l1, r1 = oracle_lib.jacobian_roe3d(nxyz, ql, qr, kind="port")
    l2, r2 = oracle_lib.jacobian_roe3d(nxyz, ql, qr, kind="reference", case=ref)
    assert np.array_equal(l1, l2) and np.array_equal(r1, r2)


@pytest.mark.parametrize("periodic", [False, True])
def test_block_tridag5_bitexact(oracle_lib, periodic):
    """ho_block_tridag5 against TRISOLVER::blockTridag / blockTridagPeriodic:
    the solution and the scratch the reference leaves in a, b and c."""
    from pointwise_inputs import blocks5
    a, b, c, f = blocks5(1, 19, 7 + int(periodic))
    for n in (2, 3, 5, 19):
        x1 = oracle_lib.block_tridag5(a[0, :n], b[0, :n], c[0, :n], f[0, :n], periodic, "port")
        x2 = oracle_lib.block_tridag5(a[0, :n], b[0, :n], c[0, :n], f[0, :n], periodic, "reference")
        for u, v, what in zip(x1, x2, "abcf"):
            assert np.array_equal(u, v), (n, what)
