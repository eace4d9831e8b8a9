"""hamstr_gpu_autotune: launch shapes change speed, never results."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_autotune_fp64_keeps_bit_exactness(make_case, oracle_lib, native_lib):
    from hamstr_oop_gb300 import native
    case = make_case(32, 8, order=3, CFL=10.0, msweep=2)
    g = native.GpuSolver(native.Case(case))
    rep = g.autotune(reps=2)
    assert rep["precision"] == "fp64" and len(rep["candidates"]) == 256
    assert all(c["ms"] > 0 for c in rep["candidates"])
    o = oracle_lib.OracleCase(case, "port")
    for it in range(5):
        ho, hg = o.step(), g.step()
        assert hg[1] == ho[1] and abs(hg[0] - ho[0]) <= 1e-13 * ho[0], it
    assert np.array_equal(g.get("q"), o.get("q"))


FP64_SHAPES = [dict(face_block=fb, adi_warps_per_sm=w, face_softdiv=fs, pivot_softdiv=ps, adi_open_lanes=ln,
                    adi_bundle_rows=bu)
               for fb in (128, 256) for w in (4, 8) for fs in (0, 1) for ps in (0, 1) for ln in (32, 16, 4)
               for bu in (0, 4, 64)]
# with the first wave's first-sweep solve in its own launch (the default
# runs it inside the factorisation kernel)
FP64_SHAPES += [dict(sh, adi_fuse=0) for sh in FP64_SHAPES[::4]]
# the factorisation kernel with a warp count of its own
FP64_SHAPES += [dict(sh, adi_factor_warps_per_sm=8 if sh["adi_warps_per_sm"] == 4 else 4) for sh in FP64_SHAPES[1::4]]


@pytest.mark.parametrize("order,split", [(3, 0.5), (5, 0.5), (5, 0.0)])
def test_every_fp64_shape_is_exact(make_case, oracle_lib, native_lib, order, split):
    """Each FP64 launch shape, set explicitly, against the oracle: on a split
    mesh (open chains of many lengths) and on the plain O-grid (periodic
    loops beside open lines)."""
    from hamstr_oop_gb300 import native
    case = make_case(24, 8, split=split, seed=3, order=order, CFL=5.0, msweep=2)
    c = native.Case(case)
    c.set_option("chain_end_rule", 1)
    o = oracle_lib.OracleCase(case, "port")
    o.set_option("chain_end_rule", 1)
    o.march(4)
    want = o.get("q")
    g = native.GpuSolver(c)
    q0 = g.get("q")
    shapes = FP64_SHAPES + ([dict(s, weno_keep=0) for s in FP64_SHAPES[::3]] if order == 5 else [])
    for shp in shapes:
        g.set("q", q0)
        g.set_shape(**shp)
        assert {k: g.shape()[k] for k in shp} == shp
        g.march(4, 0.0)
        assert np.array_equal(g.get("q"), want), shp


def test_set_shape_rejects_bad_values(make_case, native_lib):
    from hamstr_oop_gb300 import native
    g = native.GpuSolver(native.Case(make_case(16, 4, order=1, CFL=5.0)))
    before = g.shape()
    for bad in (dict(face_block=192), dict(adi_warps_per_sm=6), dict(mx_block=96), dict(adi_open_lanes=8), dict(adi_bundle_rows=65),
                dict(mx_spike=3), dict(adi_fuse=2), dict(adi_factor_warps_per_sm=6)):
        with pytest.raises(native.HamstrError):
            g.set_shape(**bad)
    assert g.shape() == before


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
    q0 = a.get("q")
    for fused in (0, 1):
        for mb in (32, 64, 128):
            b.set("q", q0)
            b.set_shape(mx_fused=fused, mx_block=mb, face_block=128 if mb == 64 else 256)
            a.set("q", q0)
            a.march(3, 0.0)
            b.march(3, 0.0)
            assert np.array_equal(a.get("q"), b.get("q")), (fused, mb)


def test_autotune_on_a_batch(make_case, native_lib):
    from hamstr_oop_gb300 import native
    cs = [native.Case(make_case(16 + 8 * k, 4 + 2 * k, order=1, CFL=10.0)) for k in range(3)]
    b = native.GpuSolver.batch(cs)
    b.set_precision(True)
    rep = b.autotune(reps=1)
    assert "best" in rep
    h, _ = b.march(5, 0.0)
    assert np.all(np.isfinite(h[:, :, :2]))
