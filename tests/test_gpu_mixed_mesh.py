"""CUDA path vs the oracle on mixed tri/quad meshes (bit-exact fields).

Half-split O-grids use the extended chain end rule (open chains ending at
interior faces); the lightly split mesh also runs under the reference's own
rule, which the oracle restates exactly (tests/test_mixed_mesh.py pins it to
the reference).  Comparisons are ==, except the tree-reduced L2 norm
(1e-13 relative).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

L2_RTOL = 1e-13
HALF = dict(ni=32, nj=8, split=0.5, seed=1)
LIGHT = dict(ni=32, nj=12, split=0.04, seed=29)


def _pair(make_case, oracle_lib, mesh, rule, **inputs):
    from hamstr_oop_gb300 import native
    case = make_case(mesh["ni"], mesh["nj"], split=mesh["split"], seed=mesh["seed"], **inputs)
    orc = oracle_lib.OracleCase(case, "port")
    orc.set_option("chain_end_rule", rule)
    host = native.Case(case)
    host.set_option("chain_end_rule", rule)
    return orc, native.GpuSolver(host)


def _eq(a, b, name):
    a, b = np.asarray(a), np.asarray(b)
    bad = np.flatnonzero(~(a == b))
    assert bad.size == 0, "%s differs at %d entries; first %d: %r vs %r" % (
        name, bad.size, bad[0], a[bad[0]], b[bad[0]])


def _close(x, y, name):
    assert abs(x - y) <= L2_RTOL * max(abs(x), abs(y), 1e-300), "%s: %r vs %r" % (name, x, y)


def _perturb(orc, gpu, seed, amp):
    q = orc.get("q").reshape(-1, 4)
    q = q * (1.0 + amp * np.random.default_rng(seed).standard_normal(q.shape))
    orc.set("q", q)
    gpu.set("q", q)


@pytest.mark.parametrize("order", [1, 3, 5])
def test_compute_rhs_extended(make_case, oracle_lib, native_lib, order):
    orc, gpu = _pair(make_case, oracle_lib, HALF, 1, order=order)
    _perturb(orc, gpu, 7, 0.05)
    lo, go = orc.compute_rhs(True), gpu.compute_rhs(True)
    for name in ("r", "sigma", "ff"):
        _eq(gpu.get(name), orc.get(name), name)
    _close(go[0], lo[0], "L2")
    assert go[1] == lo[1]


@pytest.mark.parametrize("order", [1, 3, 5])
@pytest.mark.parametrize("msweep", [1, 2, 3])
def test_adi_extended(make_case, oracle_lib, native_lib, order, msweep):
    orc, gpu = _pair(make_case, oracle_lib, HALF, 1, order=order, msweep=msweep, CFL=5.0)
    _perturb(orc, gpu, 11, 0.03)
    orc.compute_rhs(True)
    gpu.compute_rhs(True)
    lo, go = orc.adi(), gpu.adi()
    for name in ("dq", "r0", "q", "r"):
        _eq(gpu.get(name), orc.get(name), name)
    _close(go[0], lo[0], "linear L2")


@pytest.mark.parametrize("order", [1, 3, 5])
def test_step_history_extended(make_case, oracle_lib, native_lib, order):
    orc, gpu = _pair(make_case, oracle_lib, HALF, 1, order=order, CFL=5.0, msweep=2)
    for it in range(10):
        ho, hg = orc.step(), gpu.step()
        _close(hg[0], ho[0], "rhs L2 step %d" % it)
        assert hg[1] == ho[1] and hg[3] == ho[3]
    for name in ("q", "dq", "r", "sigma"):
        _eq(gpu.get(name), orc.get(name), name)


@pytest.mark.parametrize("order", [1, 3, 5])
def test_step_history_reference_rule_light_split(make_case, oracle_lib, native_lib, order):
    # the reference's rule puts freestream ghosts inside this mesh, which
    # diverges above CFL 3; a few steps at CFL 2 exercise it
    orc, gpu = _pair(make_case, oracle_lib, LIGHT, 0, order=order, CFL=2.0, msweep=2)
    for it in range(5):
        ho, hg = orc.step(), gpu.step()
        _close(hg[0], ho[0], "rhs L2 step %d" % it)
        assert hg[1] == ho[1]
    _eq(gpu.get("q"), orc.get("q"), "q")


def test_march_to_tolerance_extended(make_case, oracle_lib, native_lib):
    orc, gpu = _pair(make_case, oracle_lib, HALF, 1, order=1, CFL=10.0, msweep=2)
    hist_g, conv = gpu.march(3000, 1e-10)
    assert conv
    # the march stops before the ADI of the step whose residual met the tolerance
    n = hist_g.shape[0]
    hist_o = orc.march(n - 1)
    np.testing.assert_allclose(hist_g[:n - 1, 0], hist_o[:, 0], rtol=L2_RTOL, atol=0)
    _eq(gpu.get("q"), orc.get("q"), "converged q")


@pytest.mark.parametrize("scheme", ["euler", "rk3"])
def test_explicit_extended(make_case, oracle_lib, native_lib, scheme):
    orc, gpu = _pair(make_case, oracle_lib, HALF, 1, order=3, CFL=0.5)
    for it in range(3):
        no, ng = orc.step_explicit(scheme), gpu.step_explicit(scheme)
        _close(ng[0], no[0], "L2 step %d" % it)
    _eq(gpu.get("q"), orc.get("q"), "q")


def test_mixed_precision_on_split_mesh(make_case, oracle_lib, native_lib):
    """FP32 operator on a half-split mesh reaches the FP64 oracle's steady state.

    On this coarse mesh the state at L2 = 1e-10 is still ~6e-4 from the
    steady state (slow modes; 1e-14 still ~1e-8), so both run 8000 steps,
    to below 1e-15, before comparing."""
    orc, gpu = _pair(make_case, oracle_lib, HALF, 1, order=1, CFL=10.0, msweep=2)
    gpu.set_precision(True)
    hist, _ = gpu.march(8000, 0.0)
    assert hist[-1, 0] <= 1e-15, hist[-1, 0]
    ho = orc.march(8000)
    assert ho[-1, 0] <= 1e-15
    qo, qg = orc.get("q"), gpu.get("q")
    assert np.max(np.abs(qg - qo)) / np.max(np.abs(qo)) < 1e-8


def test_cfl_ramp_matches_oracle(make_case, oracle_lib, native_lib):
    """hamstr_gpu_set_cfl between steps equals the oracle run at each CFL."""
    orc, gpu = _pair(make_case, oracle_lib, HALF, 1, order=5, CFL=2.0, msweep=2)
    for cfl, n in ((2.0, 3), (5.0, 3), (20.0, 3)):
        orc.set_run(5, 2, cfl)
        gpu.set_cfl(cfl)
        for it in range(n):
            ho, hg = orc.step(), gpu.step()
            _close(hg[0], ho[0], "L2 at CFL %g step %d" % (cfl, it))
    _eq(gpu.get("q"), orc.get("q"), "q after the ramp")


@pytest.mark.parametrize("order,mixed_precision", [(3, False), (5, False), (5, True)])
def test_first_order_sweeps(make_case, oracle_lib, native_lib, order, mixed_precision):
    """hamstr_gpu_set_sweep_order(1): the sweeps' linearised residual at
    first order.  FP64: equal to the oracle's option bit for bit.  The
    first residual of every form is the plain one (the residual itself is
    unchanged)."""
    orc, gpu = _pair(make_case, oracle_lib, HALF, 1, order=order, CFL=5.0, msweep=2)
    orc.set_option("sweep_order", 1)
    gpu.set_sweep_order(1)
    gpu.set_precision(mixed_precision)
    _perturb(orc, gpu, 13, 0.02)
    for it in range(5):
        ho, hg = orc.step(), gpu.step()
        if it == 0 or not mixed_precision:
            _close(hg[0], ho[0], "rhs L2 step %d" % it)
    if not mixed_precision:
        for name in ("q", "dq", "r", "sigma"):
            _eq(gpu.get(name), orc.get(name), name)
    else:
        q, qo = gpu.get("q"), orc.get("q")
        assert np.max(np.abs(q - qo)) < 1e-5 * np.max(np.abs(qo))
    gpu.set_sweep_order(0)
    with pytest.raises(Exception):
        gpu.set_sweep_order(2)


def test_mixed_precision_order5_split_mesh_plateau(make_case, oracle_lib, native_lib):
    """FP32 operator, WENO, half-split mesh, against the FP64 oracle.

    On split meshes the WENO residual has no smooth zero: both forms stop at
    the same L2 plateau (~4e-8 here) and circle there, so the check is that
    the FP32-operator march reaches the oracle's plateau and that its state
    lies within 1e-6 of the oracle's (first-order sweeps, whose plateau is
    the residual's own; measured gaps 3e-9 .. 4e-8)."""
    from hamstr_oop_gb300 import native
    case = make_case(64, 16, split=0.5, seed=0, order=5, CFL=5.0, msweep=2, Mach=0.5, alpha=1.25)
    orc = oracle_lib.OracleCase(case, "port")
    orc.set_option("chain_end_rule", 1)
    orc.set_option("sweep_order", 1)
    host = native.Case(case)
    host.set_option("chain_end_rule", 1)
    gpu = native.GpuSolver(host)
    gpu.set_sweep_order(1)
    gpu.set_precision(True)
    n = 3000
    hg, _ = gpu.march(n, 0.0)
    ho = orc.march(n)
    lo, lg = ho[-1000:, 0].min(), hg[-1000:, 0].min()
    assert lo < 1e-7 and abs(lg / lo - 1.0) < 0.2, (lo, lg)
    qo, qg = orc.get("q"), gpu.get("q")
    assert np.max(np.abs(qg - qo)) / np.max(np.abs(qo)) < 1e-6
