"""Golden fixtures written by the reference itself (tests/golden/make_golden.py).

The C restatement must reproduce them bit for bit on any host (CPU test); the
CUDA path must reproduce every field bit for bit and the L2 norms to 1e-13
relative (GPU test).  The freestream is set from the fixture so hosts whose
libm cos/sin round differently still start from the reference's state."""
import glob
import os

import numpy as np
import pytest

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(HERE, "*.npz")))
FIELDS = ("q", "dq", "r", "r0", "sigma", "ff")


def _load(name):
    return dict(np.load(os.path.join(HERE, name + ".npz")))


def test_fixtures_present():
    assert len(CASES) >= 6


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_golden(oracle_lib, name):
    g = _load(name)
    orc = oracle_lib.OracleCase(os.path.join(HERE, name), "port")
    orc.set_option("chain_end_rule", int(g.get("end_rule", 0)))
    orc.set_freestream(*g["freestream"])
    orc.set("q", g["q0"])
    hist = orc.march(g["hist"].shape[0])
    assert np.array_equal(hist, g["hist"])
    for f in FIELDS:
        assert np.array_equal(orc.get(f), g[f]), f


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_reproduces_golden(native_lib, name):
    from hamstr_oop_gb300 import native
    g = _load(name)
    case = native.Case(os.path.join(HERE, name))
    case.set_freestream(*g["freestream"])
    case.set_option("chain_end_rule", int(g.get("end_rule", 0)))
    gpu = native.GpuSolver(case)
    gpu.set("q", g["q0"])
    for i, want in enumerate(g["hist"]):
        got = gpu.step()
        for k in (0, 2):
            assert abs(got[k] - want[k]) <= 1e-13 * abs(want[k]), (i, k, got[k], want[k])
        assert got[1] == want[1] and got[3] == want[3]
    for f in FIELDS:
        a, b = gpu.get(f), g[f]
        assert np.array_equal(a, b), "%s: %d entries differ" % (f, int(np.sum(a != b)))
