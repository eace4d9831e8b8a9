"""CUDA path vs the oracle on the benchmark configurations at full size.

The other parity tests use meshes of a few hundred cells.  Several code paths
depend on size and only meet the oracle here:
  - the FP64 line kernels' job queues: half-warp pairs, quads and the
    one-chain-per-lane bundles of short open chains on the 98k-cell and
    341k-cell split meshes, under every launch shape that changes them;
  - the 512-row periodic loops of the unsplit 512 x 128 O-grid (one warp
    each, a long dependent row recurrence);
  - the batched union of many conditions on the four O-grids of the batched
    configuration, where the FP32 line kernels run their chains in several
    rounds and the chunked row loads are switched off by occupancy.

FP64 fields are compared with == (reference operation order, see
tests/test_gpu_parity.py); the tree-reduced L2 norm to 1e-13 relative.
Each configuration starts from a developed flow: 100 steps of the GPU from
freestream at CFL 2 and 5 (the ramp WENO at CFL 20 needs on the split mesh),
perturbed by a seeded 0.1% so every limiter, WENO and Roe branch is taken;
from there the oracle and the GPU run two steps at the configuration's CFL.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

L2_RTOL = 1e-13

# The benchmark configurations (NACA 0012 O-grids; split = probability that a
# quad is split into two triangles, seeded; rule 1 = extended chain end rule
# for the split meshes; limiter 1 = minmod, 2 = van Albada).
CONFIGS = {
    "c1_128x32_muscl_minmod": dict(ni=128, nj=32, split=0.0, seed=0, rule=0, order=3, limiter=1, CFL=10.0,
                                   Mach=0.5, alpha=1.25),
    "c2_512x128_split50_weno": dict(ni=512, nj=128, split=0.5, seed=0, rule=1, order=5, limiter=0, CFL=20.0,
                                    Mach=0.5, alpha=1.25),
    "c2quad_512x128_weno": dict(ni=512, nj=128, split=0.0, seed=0, rule=0, order=5, limiter=0, CFL=20.0,
                                Mach=0.5, alpha=1.25),
    "c3_1024x256_split30_vanalbada": dict(ni=1024, nj=256, split=0.3, seed=0, rule=1, order=3, limiter=2,
                                          CFL=10.0, Mach=0.8, alpha=1.25),
}
BATCH_MESHES = ((128, 32), (256, 64), (384, 96), (512, 128))

# FP64 launch shapes that change the line kernels' job queues or the face
# kernels' code paths, each set on top of the default shape
SHAPES = ([dict(adi_bundle_rows=b) for b in (0, 4, 8, 16, 64)] +
          [dict(adi_open_lanes=n) for n in (32, 16, 4)] +
          [dict(adi_warps_per_sm=8), dict(face_block=256), dict(face_softdiv=0), dict(pivot_softdiv=1),
           dict(adi_fuse=0), dict(adi_factor_warps_per_sm=8)])


@pytest.fixture(scope="module")
def case_dirs(tmp_path_factory):
    """Case directory of each configuration, generated once."""
    from hamstr_oop_gb300 import meshgen
    base = tmp_path_factory.mktemp("configs")
    cache = {}

    def get(name):
        if name not in cache:
            c = CONFIGS[name]
            cache[name] = meshgen.make_case(str(base / name), c["ni"], c["nj"], order=c["order"], CFL=c["CFL"],
                                            msweep=2, Mach=c["Mach"], alpha=c["alpha"], split=c["split"],
                                            seed=c["seed"])
        return cache[name]
    return get


def _eq(a, b, name):
    a, b = np.asarray(a), np.asarray(b)
    bad = np.flatnonzero(~(a == b))
    assert bad.size == 0, "%s differs at %d of %d entries; first %d: %r vs %r" % (
        name, bad.size, a.size, bad[0], a[bad[0]], b[bad[0]])


def _close(x, y, name):
    assert abs(x - y) <= L2_RTOL * max(abs(x), abs(y), 1e-300), "%s: %r vs %r" % (name, x, y)


def _pair(oracle_lib, case_dir, cfg):
    from hamstr_oop_gb300 import native
    orc = oracle_lib.OracleCase(case_dir, "port")
    host = native.Case(case_dir)
    for h in (orc, host):
        h.set_option("chain_end_rule", cfg["rule"])
        h.set_option("limiter", cfg["limiter"])
    return orc, native.GpuSolver(host)


def _perturbed(q, seed=2024, amp=1e-3):
    q = q.reshape(-1, 4)
    return (q * (1.0 + amp * np.random.default_rng(seed).standard_normal(q.shape))).ravel()


@pytest.mark.parametrize("name", sorted(CONFIGS))
def test_config_two_steps_bitexact(case_dirs, oracle_lib, native_lib, name):
    """computeRHS, ADI and a second step at full size, field by field, with
    the autotuner's shape and then with each shape of SHAPES."""
    cfg = CONFIGS[name]
    orc, gpu = _pair(oracle_lib, case_dirs(name), cfg)
    for cfl in (2.0, 5.0):
        gpu.set_cfl(cfl)
        gpu.march(50, 0.0)
    q0 = _perturbed(gpu.get("q"))
    rep = gpu.autotune(reps=1)                  # at CFL 5; the state is put back
    gpu.set_cfl(cfg["CFL"])
    orc.set("q", q0)
    gpu.set("q", q0)
    lo, go = orc.compute_rhs(True), gpu.compute_rhs(True)
    for f in ("r", "sigma", "ff"):
        _eq(gpu.get(f), orc.get(f), "%s: %s after computeRHS (shape %r)" % (name, f, rep["best"]))
    _close(go[0], lo[0], name + ": computeRHS L2")
    assert go[1] == lo[1]
    lo, go = orc.adi(), gpu.adi()
    for f in ("dq", "r0", "q", "r"):
        _eq(gpu.get(f), orc.get(f), "%s: %s after ADI" % (name, f))
    _close(go[0], lo[0], name + ": linear L2")
    ho, hg = orc.step(), gpu.step()
    _close(hg[0], ho[0], name + ": step 2 L2")
    assert hg[1] == ho[1] and hg[3] == ho[3]
    want = orc.get("q")
    for f in ("q", "dq", "r", "sigma"):
        _eq(gpu.get(f), orc.get(f), "%s: %s after step 2" % (name, f))
    shapes = SHAPES + ([dict(weno_keep=0)] if cfg["order"] == 5 else [])
    for shp in shapes:
        gpu.set("q", q0)
        gpu.set_shape(**dict(rep["best"], **shp))
        gpu.march(2, 0.0)
        _eq(gpu.get("q"), want, "%s: q after 2 steps with shape %r" % (name, shp))


def _batch(native_lib, tmp_path_factory, n, order=1):
    """n seeded conditions on the four O-grids, round-robin: host cases and
    their mesh directories."""
    from hamstr_oop_gb300 import meshgen, native
    base = tmp_path_factory.mktemp("batch")
    dirs = [meshgen.make_case(str(base / ("%dx%d" % m)), m[0], m[1], order=order, CFL=10.0, msweep=2, nsteps=1)
            for m in BATCH_MESHES]
    rng = np.random.default_rng(0)
    mach, alpha = rng.uniform(0.3, 0.85, n), rng.uniform(-2.0, 4.0, n)
    meshes = [native.Case(d) for d in dirs]
    cases, where = [], []
    for k in range(n):
        c = meshes[k % 4].clone()
        c.set_flow(float(mach[k]), float(alpha[k]))
        cases.append(c)
        where.append(dirs[k % 4])
    return cases, where


def test_batch_of_sixteen_conditions_on_four_meshes_bitexact(tmp_path_factory, oracle_lib, native_lib):
    """A batched FP64 handle of 16 conditions on the four O-grids (128x32 ..
    512x128) against the oracle, one condition at a time."""
    from hamstr_oop_gb300 import native
    cases, where = _batch(native_lib, tmp_path_factory, 16)
    b = native.GpuSolver.batch(cases)
    q0 = np.concatenate([_perturbed_case(c, k) for k, c in enumerate(cases)])
    b.set("q", q0)
    hb, _ = b.march(2, 0.0)
    cell0 = b.instance_cells()
    qb = b.get("q").reshape(-1, 4)
    for k, (c, d) in enumerate(zip(cases, where)):
        o = oracle_lib.OracleCase(d, "port")
        p = c.params
        o.set_freestream(p["uinf"], p["vinf"], p["einf"])
        o.set("q", q0.reshape(-1, 4)[cell0[k]:cell0[k + 1]])
        ho = o.march(2)
        _close(hb[1, k, 0], ho[1, 0], "instance %d L2" % k)
        _eq(qb[cell0[k]:cell0[k + 1]], o.get("q").reshape(-1, 4), "instance %d q" % k)
        o.close()


def _perturbed_case(case, k, amp=0.02):
    q = case.get("q").reshape(-1, 4)
    return (q * (1.0 + amp * np.random.default_rng(100 + k).standard_normal(q.shape))).ravel()


def test_full_batch_fp32_rounds_are_shape_independent(tmp_path_factory, native_lib):
    """The 256-condition batch (7.9 M cells, ~100k chains) with the FP32
    operator: its chains do not all fit on the GPU at once, so the line
    kernels run them in several rounds and the chunked row loads are off by
    occupancy.  Every FP32 line-kernel shape must give the same states, and
    each instance must equal a plain handle on its condition."""
    from hamstr_oop_gb300 import native
    cases, _ = _batch(native_lib, tmp_path_factory, 256)
    b = native.GpuSolver.batch(cases)
    b.set_precision(True)
    q0 = b.get("q")
    b.march(2, 0.0)
    want = b.get("q")
    assert np.all(np.isfinite(want))
    for shp in (dict(mx_chunk=0), dict(mx_fused=1), dict(mx_block=128), dict(mx_block=32, mx_fused=1)):
        b.set("q", q0)
        b.set_shape(**shp)
        b.march(2, 0.0)
        _eq(b.get("q"), want, "batch q with FP32 shape %r" % shp)
    cell0 = b.instance_cells()
    qb = want.reshape(-1, 4)
    b.close()
    for k in (0, 3, 131, 255):                   # the 512x128 mesh is every fourth, from 3
        s = native.GpuSolver(cases[k])
        s.set_precision(True)
        s.march(2, 0.0)
        _eq(s.get("q").reshape(-1, 4), qb[cell0[k]:cell0[k + 1]], "FP32 instance %d vs its own handle" % k)
        s.close()
