"""Wall pressure forces (a project addition; the reference computes none).

ho_forces / hamstr_gpu_forces integrate p * (dy, -dx) over the wall faces
(bFaces, preprocess.cpp:180-184) in ascending face order; the GPU sums in the
same order, so the two agree bit for bit."""
import numpy as np
import pytest


def _oracle(oracle_lib, case, rule=0):
    o = oracle_lib.OracleCase(case, "port")
    o.set_option("chain_end_rule", rule)
    return o


def test_freestream_has_no_force(make_case, oracle_lib):
    f = _oracle(oracle_lib, make_case(32, 8)).forces()
    # a closed wall: the normals sum to zero, so a uniform pressure gives none
    for k in ("CL", "CD", "CM"):
        assert abs(f[k]) < 1e-13, (k, f[k])


def test_converged_lift_is_plausible(make_case, oracle_lib):
    # NACA 0012, M 0.5, alpha 1.25 deg: thin-aerofoil lift with the
    # Prandtl-Glauert factor is about 0.158; first order on a coarse grid
    # loses some of it and adds numerical drag
    o = _oracle(oracle_lib, make_case(64, 16, order=1, CFL=10.0, msweep=2))
    h = o.march(1500)
    assert h[-1, 0] < 1e-10
    f = o.forces()
    assert 0.10 < f["CL"] < 0.19, f
    assert 0.0 < f["CD"] < 0.12, f


@pytest.mark.gpu
@pytest.mark.parametrize("split,order,rule", [(0.0, 5, 0), (0.5, 3, 1)])
def test_gpu_forces_bitexact(make_case, oracle_lib, native_lib, split, order, rule):
    from hamstr_oop_gb300 import native
    case = make_case(32, 8, split=split, seed=1, order=order, CFL=5.0, msweep=2)
    o = _oracle(oracle_lib, case, rule)
    c = native.Case(case)
    c.set_option("chain_end_rule", rule)
    g = native.GpuSolver(c)
    assert g.forces() == o.forces()
    o.march(15)
    g.march(15, 0.0)
    fo, fg = o.forces(), g.forces()
    assert fg == fo, (fg, fo)
    assert abs(fg["CL"]) > 1e-6
