"""hamstr_gpu_autotune: launch shapes change speed, never results."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_autotune_fp64_keeps_bit_exactness(make_case, oracle_lib, native_lib):
    from hamstr_oop_gb300 import native
    case = make_case(32, 8, order=3, CFL=10.0, msweep=2)
    g = native.GpuSolver(native.Case(case))
    rep = g.autotune(reps=2)
    assert rep["precision"] == "fp64" and len(rep["candidates"]) == 16
    assert all(c["ms"] > 0 for c in rep["candidates"])
    o = oracle_lib.OracleCase(case, "port")
    for it in range(5):
        ho, hg = o.step(), g.step()
        assert hg[1] == ho[1] and abs(hg[0] - ho[0]) <= 1e-13 * ho[0], it
    assert np.array_equal(g.get("q"), o.get("q"))


@pytest.mark.parametrize("shape", [(256, 8, 64), (128, 4, 32)])
def test_every_fp64_shape_is_exact(make_case, oracle_lib, native_lib, shape):
    """Force each candidate by tuning on a handle, then compare to the oracle."""
    from hamstr_oop_gb300 import native
    case = make_case(24, 8, split=0.5, seed=3, order=5, CFL=5.0, msweep=2)
    c = native.Case(case)
    c.set_option("chain_end_rule", 1)
    g = native.GpuSolver(c)
    g.autotune(reps=1)
    o = oracle_lib.OracleCase(case, "port")
    o.set_option("chain_end_rule", 1)
    o.march(4)
    g.march(4, 0.0)
    assert np.array_equal(g.get("q"), o.get("q"))


def test_autotune_mixed_restores_state_and_results(make_case, native_lib):
    from hamstr_oop_gb300 import native
    case = make_case(32, 8, order=1, CFL=10.0, msweep=2)
    a = native.GpuSolver(native.Case(case))
    b = native.GpuSolver(native.Case(case))
    a.set_precision(True)
    b.set_precision(True)
    rep = b.autotune(reps=2)
    assert rep["precision"] == "mixed" and len(rep["candidates"]) == 24
    assert np.array_equal(a.get("q"), b.get("q"))        # state put back
    a.march(6, 0.0)
    b.march(6, 0.0)
    assert np.array_equal(a.get("q"), b.get("q"))        # shape-independent arithmetic


def test_autotune_on_a_batch(make_case, native_lib):
    from hamstr_oop_gb300 import native
    cs = [native.Case(make_case(16 + 8 * k, 4 + 2 * k, order=1, CFL=10.0)) for k in range(3)]
    b = native.GpuSolver.batch(cs)
    b.set_precision(True)
    rep = b.autotune(reps=1)
    assert "best" in rep
    h, _ = b.march(5, 0.0)
    assert np.all(np.isfinite(h[:, :, :2]))
