"""The batched form: several cases in one handle (hamstr_gpu_create_batch).

Every instance of a batch must compute exactly what a plain handle computes
on its case: fields bit for bit, per-instance norms equal (each instance's
norm blocks are laid out as in a plain handle), forces equal."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [dict(ni=24, nj=8, Mach=0.5, alpha=1.25), dict(ni=32, nj=8, Mach=0.7, alpha=-1.0),
         dict(ni=40, nj=12, Mach=0.4, alpha=3.0)]


def _cases(make_case, specs, split=0.0, rule=0, **inputs):
    from hamstr_oop_gb300 import native
    out = []
    for k, c in enumerate(specs):
        d = make_case(c["ni"], c["nj"], Mach=c["Mach"], alpha=c["alpha"], split=split, seed=k, **inputs)
        h = native.Case(d)
        h.set_option("chain_end_rule", rule)
        out.append((d, h))
    return out


@pytest.mark.parametrize("order,split", [(1, 0.0), (3, 0.0), (5, 0.0), (3, 0.5)])
def test_batch_equals_single_handles(make_case, native_lib, order, split):
    from hamstr_oop_gb300 import native
    rule = 1 if split else 0
    cs = _cases(make_case, CASES, split=split, rule=rule, order=order, CFL=5.0, msweep=2)
    b = native.GpuSolver.batch([h for _, h in cs])
    assert b.n_instances == 3
    singles = [native.GpuSolver(h) for _, h in cs]
    hb, _ = b.march(8, 0.0)
    assert hb.shape == (8, 3, 4)
    cell0 = b.instance_cells()
    qb = b.get("q").reshape(-1, 4)
    for k, s in enumerate(singles):
        hs, _ = s.march(8, 0.0)
        np.testing.assert_array_equal(hb[:, k, :], hs)
        assert np.array_equal(qb[cell0[k]:cell0[k + 1]], s.get("q").reshape(-1, 4)), k
    fb = b.batch_forces()
    for k, s in enumerate(singles):
        f = s.forces()
        assert np.array_equal(fb[k], [f[n] for n in ("Fx", "Fy", "M", "CL", "CD", "CM")]), k
    nb = b.instance_norms()
    assert np.array_equal(nb[0], hb[-1, 0])


def test_batch_matches_the_oracle(make_case, oracle_lib, native_lib):
    from hamstr_oop_gb300 import native
    cs = _cases(make_case, CASES, order=3, CFL=5.0, msweep=2)
    b = native.GpuSolver.batch([h for _, h in cs])
    b.march(6, 0.0)
    cell0 = b.instance_cells()
    qb = b.get("q").reshape(-1, 4)
    for k, (d, _) in enumerate(cs):
        o = oracle_lib.OracleCase(d, "port")
        o.march(6)
        assert np.array_equal(qb[cell0[k]:cell0[k + 1]], o.get("q").reshape(-1, 4)), k


@pytest.mark.parametrize("mixed", [False, True])
def test_batch_march_freezes_each_instance_where_a_plain_march_stops(make_case, native_lib, mixed):
    """Each instance stops at its own tolerance step: its final state equals
    a plain handle's march on its case bit for bit; the march ends when the
    last instance converges, and a frozen instance's history rows stay NaN."""
    from hamstr_oop_gb300 import native
    cs = _cases(make_case, CASES, order=1, CFL=10.0, msweep=2)
    b = native.GpuSolver.batch([h for _, h in cs])
    b.set_precision(mixed)
    hist, conv = b.march(6000, 1e-10)
    assert conv
    first = [int(np.argmax(hist[:, k, 0] <= 1e-10)) for k in range(3)]
    assert hist.shape[0] == max(first) + 1
    cell0 = b.instance_cells()
    qb = b.get("q").reshape(-1, 4)
    for k, (_, h) in enumerate(cs):
        assert np.all(np.isnan(hist[first[k] + 1:, k, 0]))
        s = native.GpuSolver(h)
        s.set_precision(mixed)
        hs, cs_ = s.march(6000, 1e-10)
        assert cs_ and hs.shape[0] == first[k] + 1, (k, hs.shape, first[k])
        np.testing.assert_array_equal(hist[:first[k] + 1, k, :2], hs[:, :2])
        assert np.array_equal(qb[cell0[k]:cell0[k + 1]], s.get("q").reshape(-1, 4)), k


def test_batch_mixed_precision_converges(make_case, native_lib):
    from hamstr_oop_gb300 import native
    cs = _cases(make_case, CASES, order=1, CFL=10.0, msweep=2)
    b = native.GpuSolver.batch([h for _, h in cs])
    b.set_precision(True)
    hist, conv = b.march(6000, 1e-10)
    assert conv
    for k in range(3):
        # rows up to the instance's stop are finite; frozen rows stay NaN
        kk = int(np.argmax(hist[:, k, 0] <= 1e-10))
        assert np.all(np.isfinite(hist[:kk + 1, k, :2])) and np.all(np.isfinite(hist[:kk, k]))


def test_batch_rejects_mismatched_runs(make_case, native_lib):
    from hamstr_oop_gb300 import native
    a = native.Case(make_case(16, 4, order=3, CFL=5.0))
    c = native.Case(make_case(16, 4, order=1, CFL=5.0))
    with pytest.raises(native.HamstrError) as ei:
        native.GpuSolver.batch([a, c])
    assert ei.value.status == -1
