"""Mixed-precision defect correction against the FP64 path and the oracle.

The FP64 residual of the mixed form is the reference's, bit for bit; its
implicit operator (Jacobians, ADI, linear residual) is FP32.  The form must
converge to the FP64 steady state: converged fields within 1e-8 relative of
the CPU oracle's converged fields, in about as many steps."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELD_RTOL = 1e-8


def _solver(make_case, ni, nj, mixed, **inputs):
    from hamstr_oop_gb300 import native
    case = make_case(ni, nj, **inputs)
    g = native.GpuSolver(native.Case(case))
    g.set_precision(mixed)
    return case, g


@pytest.mark.parametrize("order", [1, 3, 5])
def test_first_residual_is_the_fp64_residual(make_case, native_lib, order):
    from hamstr_oop_gb300 import native
    case, gm = _solver(make_case, 24, 6, True, order=order)
    gp = native.GpuSolver(native.Case(case))
    hm, hp = gm.step(), gp.step()
    assert hm[0] == hp[0] and hm[1] == hp[1]
    # one mixed step moves q close to the FP64 step (FP32 operator)
    qm, qp = gm.get("q"), gp.get("q")
    assert np.max(np.abs(qm - qp)) < 1e-4 * np.max(np.abs(qp))


@pytest.mark.parametrize("order,cfl", [(1, 10.0), (3, 10.0)])
def test_mixed_converges_to_oracle_solution(make_case, oracle_lib, native_lib, order, cfl):
    case, gm = _solver(make_case, 32, 8, True, order=order, CFL=cfl, msweep=2)
    hist, conv = gm.march(4000, 1e-10)
    assert conv, "mixed form did not reach 1e-10 (last %r)" % hist[-1, 0]
    orc = oracle_lib.OracleCase(case, "port")
    ho = orc.march(4000)
    k = int(np.argmax(ho[:, 0] <= 1e-10))
    assert ho[k, 0] <= 1e-10
    assert hist.shape[0] <= 1.2 * (k + 1) + 10, (hist.shape[0], k + 1)
    orc2 = oracle_lib.OracleCase(case, "port")
    orc2.march(k)
    qo, qm = orc2.get("q"), gm.get("q")
    err = np.max(np.abs(qm - qo)) / np.max(np.abs(qo))
    assert err <= FIELD_RTOL, err


def test_mixed_batched_line_solve_runs_all_orders(make_case, native_lib):
    for order in (1, 3, 5):
        case, g = _solver(make_case, 16, 5, True, order=order, msweep=3)
        h, _ = g.march(5, 0.0)
        assert np.all(np.isfinite(h[:, :2]))


@pytest.mark.parametrize("split,order", [(0.0, 1), (0.5, 5)])
def test_chunked_fp32_solve_matches_row_by_row(make_case, native_lib, split, order):
    """The FP32 line solve that loads rows four at a time (shape key mx_chunk)
    does the row-by-row solve's operations in its order: identical states, on
    periodic loops and open lines, with either block assembly."""
    from hamstr_oop_gb300 import native
    case = make_case(40, 12, split=split, seed=1, order=order, CFL=10.0, msweep=2)
    solvers = []
    for _ in range(2):
        host = native.Case(case)
        if split:
            host.set_option("chain_end_rule", 1)     # the split mesh's open chains end at interior faces
        solvers.append(native.GpuSolver(host))
    a, b = solvers
    for g in (a, b):
        g.set_precision(True)
    assert a.shape()["mx_chunk"] == 1
    b.set_shape(mx_chunk=0)
    q0 = a.get("q")
    for fused in (0, 1):
        for g in (a, b):
            g.set("q", q0)
            g.set_shape(mx_fused=fused)
        ha, _ = a.march(4, 0.0)
        hb, _ = b.march(4, 0.0)
        assert np.array_equal(ha, hb) and np.array_equal(a.get("q"), b.get("q")), fused


def _spike_pair(make_case, ni, nj, rule=0, **inputs):
    """Two FP32-operator handles on one case: long chains by segments
    (shape key mx_spike 2: periodic and open ones) and by one thread each."""
    from hamstr_oop_gb300 import native
    case = make_case(ni, nj, **inputs)
    hosts = [native.Case(case), native.Case(case)]
    for h in hosts:
        h.set_option("chain_end_rule", rule)
    a, b = native.GpuSolver(hosts[0]), native.GpuSolver(hosts[1])
    for g in (a, b):
        g.set_precision(True)
    assert a.shape()["mx_spike"] == 1
    a.set_shape(mx_spike=2)
    b.set_shape(mx_spike=0)
    return case, a, b


@pytest.mark.parametrize("ni,nj,split,order", [(64, 8, 0.0, 1), (128, 8, 0.0, 3), (384, 8, 0.0, 1),
                                              (64, 40, 0.0, 1), (96, 64, 0.5, 5)])
def test_segmented_periodic_solve_is_the_same_linear_solve(make_case, native_lib, ni, nj, split, order):
    """One step of the FP32 operator with the long chains solved by
    segments against the sequential solve: periodic loops of 64, 128 and
    384 rows (4, 8 and 24 segments), open lines of 40 rows (2 segments), and
    the open chains of 32 rows or more on a half-split mesh.  The same
    linear system, so the increments agree to FP32 rounding."""
    case, a, b = _spike_pair(make_case, ni, nj, rule=1 if split else 0, split=split, seed=2, order=order,
                             CFL=10.0, msweep=2)
    rng = np.random.default_rng(ni)
    q0 = a.get("q").reshape(-1, 4)
    q0 = (q0 * (1.0 + 0.01 * rng.standard_normal(q0.shape))).ravel()
    for g in (a, b):
        g.set("q", q0)
        g.step()
    da, db = a.get("q") - q0, b.get("q") - q0
    assert np.all(np.isfinite(da))
    err = np.max(np.abs(da - db)) / np.max(np.abs(db))
    assert err < 1e-4, err


def test_segmented_periodic_solve_converges_to_the_oracle(make_case, oracle_lib, native_lib):
    """With 64-row loops in segments the FP32 form reaches L2 <= 1e-10 in
    as many steps as the sequential form, at the same state, and that state
    is the FP64 oracle's to 1e-8."""
    case, a, b = _spike_pair(make_case, 64, 16, order=1, CFL=10.0, msweep=2)
    ha, ca = a.march(4000, 1e-10)
    hb, cb = b.march(4000, 1e-10)
    assert ca and cb
    assert abs(ha.shape[0] - hb.shape[0]) <= 2, (ha.shape[0], hb.shape[0])
    qa, qb = a.get("q"), b.get("q")
    assert np.max(np.abs(qa - qb)) <= 1e-8 * np.max(np.abs(qb))
    orc = oracle_lib.OracleCase(case, "port")
    ho = orc.march(4000)
    k = int(np.argmax(ho[:, 0] <= 1e-10))
    orc2 = oracle_lib.OracleCase(case, "port")
    orc2.march(k)
    qo = orc2.get("q")
    assert np.max(np.abs(qa - qo)) / np.max(np.abs(qo)) <= FIELD_RTOL


def test_segmented_branch_runs_beside_the_others(make_case, native_lib):
    """In the captured FP32 step the segmented chains' kernels run on a
    parallel branch beside the other chains' kernels; the per-kernel
    profile launches everything in one line.  Both orders give the same
    state bit for bit (the two touch disjoint chains and cells)."""
    from hamstr_oop_gb300 import native
    case = make_case(128, 8, order=3, CFL=10.0, msweep=2)
    a, b = native.GpuSolver(native.Case(case)), native.GpuSolver(native.Case(case))
    for g in (a, b):
        g.set_precision(True)
        assert g.shape()["mx_spike"] == 1
    a.march(4, 0.0)
    b.profile_step(4)
    assert np.array_equal(a.get("q"), b.get("q"))
