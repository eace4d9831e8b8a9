"""The learned warm start end to end on a small case: converged training
states from the batched solver, a few epochs on the tensor cores, and the
held-out conditions solved from the network's guess and from freestream.
The network must cut the iterations to the tolerance; the converged states
must not depend on the start."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_warm_start_cuts_iterations(make_case, native_lib):
    from hamstr_oop_gb300 import native, warmstart
    case = native.Case(make_case(64, 16, order=1, CFL=10.0, msweep=2))
    train = warmstart.conditions(48, seed=0)
    data = warmstart.solve_batch(case, train, 1e-10, 6000)
    assert data["all_converged"]
    model, rep = warmstart.train(case, data["q"], train, epochs=200, batch=4096, lr=2e-3)
    assert rep["loss_last"] < 0.05 * rep["loss_first"], rep
    test = warmstart.conditions(12, seed=1)
    ev = warmstart.evaluate(case, model, test, 1e-10, 6000)
    assert ev["all_converged"]
    assert ev["guess_max_rel_error_median"] < 0.05, ev
    assert ev["steps_warm_mean"] < ev["steps_freestream_mean"], ev
    # the probe guard keeps the network's start where it helps
    assert ev["steps_guard_probe_mean"] < ev["steps_freestream_mean"], ev
    # both starts reach the same steady state (to the tolerance's reach)
    assert ev["converged_state_difference_max"] < 1e-3, ev
    # and so does the plain FP64 drop-in from freestream (the oracle's own steps)
    plain = warmstart.plain_fp64_solves(case, test[:3], 1e-10, 6000)
    assert plain["all_converged"]
    for qw, qp in zip(ev["_q_warm"][:3], plain["q"]):
        assert np.max(np.abs(qw - qp)) / np.max(np.abs(qp)) < 1e-3
    # at L2 <= 1e-10 each start stops short of the fixed point in its own
    # direction; to a tight tolerance the warm-started batched FP32-operator
    # form and the plain FP64 drop-in reach the same steady state
    tight = test[:2]
    plain_t = warmstart.plain_fp64_solves(case, tight, 1e-15, 20000)
    warm_t = warmstart.solve_batch(case, tight, 1e-15, 20000, q0=model.predict(tight))
    assert plain_t["all_converged"] and warm_t["all_converged"]
    for qw, qp in zip(warm_t["q"], plain_t["q"]):
        assert np.max(np.abs(qw - qp)) / np.max(np.abs(qp)) < 1e-8


def test_features_and_geometry(make_case, native_lib):
    from hamstr_oop_gb300 import native, warmstart
    case = native.Case(make_case(32, 8))
    xc, yc, d = warmstart.cell_geometry(case)
    assert xc.shape == (256,) and np.all(d > 0)
    # the first ring of cells sits next to the wall, the last near the far field
    assert d[:32].max() < 0.05 and d[-32:].min() > 5.0
    f = warmstart.features(0.5, 1.25, (xc, yc, d))
    assert f.shape == (256, 5) and np.all(np.isfinite(f))
