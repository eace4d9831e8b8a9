"""The drop-in C++ layer against the oracle and the reference's output.

* SOLVER::fluxRoe2D / jacobianRoe2D, RECONSTRUCTION::MUSCL / MUSCL_DERIV /
  WENO / WENO_DERIV and TRISOLVER::blockTridag4 / blockTridagPeriodic4 with
  the reference's pointer-array signatures (hamstr_oop_gb300/csrc/host/),
  called from a C++ program built against the library (tests/dropin_check.cpp),
  equal the oracle's per-face and per-line functions bit for bit.
* bin/hamstr_gb300 on the golden cases prints the reference's table
  (march.cpp:39-54) with the norms the reference wrote to the fixtures.
"""
import os
import re
import subprocess

import numpy as np
import pytest

from pointwise_inputs import GAMMA, faces, lines

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module")
def dropin_check(tmp_path_factory, native_lib):
    from hamstr_oop_gb300 import native
    exe = str(tmp_path_factory.mktemp("dropin") / "dropin_check")
    lib = os.path.dirname(native.LIB_PATH)
    subprocess.run(["g++", "-O1", "-std=c++17", "-I" + os.path.join(ROOT, "hamstr_oop_gb300", "csrc", "host"),
                    "-I" + os.path.join(ROOT, "include"), "-I/usr/local/cuda/include",
                    os.path.join(ROOT, "tests", "dropin_check.cpp"), "-o", exe, "-L" + lib, "-lhamstr_gb300",
                    "-Wl,-rpath," + lib], check=True)
    return exe


def test_cpp_dropin_functions_bitexact(dropin_check, tmp_path, oracle_lib):
    nf, nl, imax, nq, N = 64, 3, 19, 4, 23
    nxy, ql, qr = faces(nf, 31)
    f, dq, prior = lines(nl, imax, nq, 32)
    rng = np.random.default_rng(33)
    a, c = rng.standard_normal((N, 4, 4)), rng.standard_normal((N, 4, 4))
    b = rng.standard_normal((N, 4, 4)) + 6.0 * np.eye(4)
    rhs = rng.standard_normal((N, 4))
    blob = np.concatenate([[nf, nl, imax, nq, N], nxy.ravel(), ql.ravel(), qr.ravel(), f.ravel(), dq.ravel(),
                           prior[0].ravel(), prior[1].ravel(), prior[2].ravel(), a.ravel(), b.ravel(), c.ravel(),
                           rhs.ravel()]).astype(np.float64)
    fin, fout = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    blob.tofile(fin)
    subprocess.run([dropin_check, fin, fout], check=True)
    out = np.fromfile(fout, dtype=np.float64)
    pos = [0]

    def take(n):
        v = out[pos[0]:pos[0] + n]
        pos[0] += n
        return v
    wf, ws = oracle_lib.flux_roe2d(nxy, ql, qr, GAMMA)
    assert np.array_equal(take(4 * nf), wf.ravel()) and np.array_equal(take(nf), ws)
    wl, wr = oracle_lib.jacobian_roe2d(nxy, ql, qr, GAMMA)
    assert np.array_equal(take(16 * nf), wl.ravel()) and np.array_equal(take(16 * nf), wr.ravel())
    # the five reconstruction calls of dropin_check.cpp; the second asks for
    # ie = imax-1, which leaves entry imax-1 of ql and qr as it was
    calls = [("muscl", 1, imax - 2, {}), ("muscl", 2, imax - 2, {}), ("muscl_deriv", 1, imax - 2, {}),
             ("weno", 2, imax - 1, {}), ("weno_deriv", 2, imax - 1, {})]
    for name, is_, ie, _ in calls:
        for k in range(nl):
            want = oracle_lib.recon_line(name, f[k], is_, ie, dq=dq[k], qt=0.25, eps=1e-10, ql=prior[0, k],
                                         qr=prior[1, k], f2=prior[2, k])
            for w, what in zip(want, ("ql", "qr", "f2")):
                got = take(imax * nq).reshape(imax, nq)
                assert np.array_equal(got, w), (name, k, what)
    for periodic in (False, True):
        want = oracle_lib.block_tridag4(a, b, c, rhs, periodic)
        assert np.array_equal(take(4 * N).reshape(N, 4), want), periodic
    assert take(1)[0] == 1.0, "a NaN spectral radius did not raise HAMSTR_GPU_ERR_NAN"
    assert pos[0] == out.size


ROW = re.compile(r"^ \|  ( *\d+)  \|  (\S+) \|   (\S+)  \|  (\S+)  \|$")
RULE = " --------------------------------------------------------------"
HEAD = " |   Iter  | L_2 (density) | L_inf (density) | CPU Time (sec) |"


@pytest.mark.parametrize("case", ["ogrid16x4_o1", "ogrid16x4_o3", "ogrid16x5_o5", "ogrid16x4_o3_loop0",
                                  "split32x12_light_o3"])
def test_executable_prints_the_reference_table(native_lib, tmp_path, case):
    """bin/hamstr_gb300 <case> runs the reference's main sequence and prints
    its per-step table: the header and rule lines of march.cpp:39-54 and
    one row per step with the final linear L2 and Linf of that step (the
    norms the reference leaves in sb->L2Norm after ADI), which the fixture
    holds as written by the reference."""
    from hamstr_oop_gb300 import build
    g = np.load(os.path.join(GOLDEN, case + ".npz"))
    r = subprocess.run([build.EXE, os.path.join(GOLDEN, case)], cwd=str(tmp_path), stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines_ = r.stdout.splitlines()
    i0 = lines_.index(HEAD)
    assert lines_[i0 - 1] == RULE and lines_[i0 + 1] == RULE
    hist = g["hist"]
    rows = lines_[i0 + 2:i0 + 2 + hist.shape[0]]
    for n, ln in enumerate(rows):
        m = ROW.match(ln)
        assert m, ln
        assert len(m.group(1)) == 5 and int(m.group(1)) == n
        l2, linf = float(m.group(2)), float(m.group(3))
        # printed with %e: 7 significant digits
        assert abs(l2 - hist[n, 2]) <= 5e-7 * abs(hist[n, 2]), (n, l2, hist[n, 2])
        assert abs(linf - hist[n, 3]) <= 5e-7 * abs(hist[n, 3]), (n, linf, hist[n, 3])
    tail = lines_[i0 + 2 + hist.shape[0]:i0 + 5 + hist.shape[0]]
    assert tail == [RULE, HEAD, RULE]
