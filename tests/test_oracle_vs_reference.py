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
