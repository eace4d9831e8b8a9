"""Mixed tri/quad meshes: the chain extractor and the extended chain end rule (CPU).

The reference reads line chains from files but ships no extractor, and its
ghost rule assumes every open chain ends at a wall or the far field
(computeRHS.cpp:86-149, 154-260; ADI.cpp:126-190).  meshgen.extract_chains
builds chains for split O-grids; the extended end rule (oracle option
``chain_end_rule`` = 1) handles chains that end at interior faces.
"""
import numpy as np
import pytest

from hamstr_oop_gb300 import meshgen

# a lightly split mesh whose open chains all have >= 3 cells, so the
# reference's own ghost rule is well defined on it (20 interior chain ends)
LIGHT = dict(ni=32, nj=12, split=0.04, seed=29)


@pytest.mark.parametrize("ni,nj,p,seed", [(24, 8, 0.5, 1), (32, 8, 0.3, 3), (64, 16, 0.5, 2),
                                          (64, 16, 0.9, 5), (63, 16, 1.0, 5), (16, 4, 0.7, 4)])
def test_extracted_chains_are_valid(ni, nj, p, seed):
    m = meshgen.naca0012_ogrid(ni, nj, split=p, seed=seed)
    st = meshgen.validate(m)
    tri = m.conn[:, 2] == m.conn[:, 3]
    # every triangle lies on one chain, every quad on two
    assert st["tris_on_one"] == int(tri.sum())
    assert st["quads_on_two"] == int((~tri).sum())
    assert st["cells"] == ni * nj + int(tri.sum()) // 2
    assert st["faces"] == ni * (2 * nj + 1) + int(tri.sum()) // 2
    assert len(m.colors) == 2 and sum(m.colors) == len(m.chains)


def test_split_is_seeded_and_deterministic():
    a = meshgen.naca0012_ogrid(32, 8, split=0.5, seed=4)
    b = meshgen.naca0012_ogrid(32, 8, split=0.5, seed=4)
    c = meshgen.naca0012_ogrid(32, 8, split=0.5, seed=5)
    assert np.array_equal(a.faces, b.faces) and a.chains == b.chains
    assert not np.array_equal(a.conn, c.conn)


def test_split_probability():
    m = meshgen.naca0012_ogrid(256, 64, split=0.3, seed=0)
    frac = (m.conn[:, 2] == m.conn[:, 3]).sum() / 2 / (256 * 64)
    assert abs(frac - 0.3) < 0.02


def test_validate_catches_a_broken_mesh():
    m = meshgen.naca0012_ogrid(24, 8, split=0.5, seed=1)
    m.chains[3] = list(m.chains[3])[:-1]      # drop a chain's last face
    with pytest.raises(ValueError):
        meshgen.validate(m)


def test_cell_zero_avoids_the_ghost_quirk():
    # split meshes put cell 0 where computeRHS.cpp:158,170's id-0 test is harmless
    m = meshgen.naca0012_ogrid(24, 8, split=0.5, seed=1)
    left = m.faces[:, 2]
    for ch in m.chains:
        closed = ch[0] == ch[-1]
        cells = [int(left[f]) for f in (ch[:-1] if closed else ch[:-1])]
        n = len(cells)
        if 0 not in cells:
            continue
        k = cells.index(0)
        bad = {0, 1, 2, n - 3, n - 2, n - 1} if closed else {1, 2, n - 2, n - 3}
        assert k not in bad


def _march(oracle_lib, case, rule, n, kind="port"):
    o = oracle_lib.OracleCase(case, kind)
    o.set_option("chain_end_rule", rule)
    return o.march(n), o.get("q")


@pytest.mark.parametrize("order", [1, 3, 5])
def test_extended_rule_is_the_reference_rule_on_quad_meshes(make_case, oracle_lib, order):
    case = make_case(24, 8, order=order, CFL=10.0, msweep=2)
    h0, q0 = _march(oracle_lib, case, 0, 6)
    h1, q1 = _march(oracle_lib, case, 1, 6)
    assert np.array_equal(h0, h1) and np.array_equal(q0, q1)


@pytest.mark.parametrize("order", [1, 3, 5])
def test_reference_rule_matches_the_reference_on_a_mixed_mesh(make_case, oracle_lib, order):
    from conftest import has_reference_sources
    if not has_reference_sources():
        pytest.skip("reference sources not present")
    case = make_case(LIGHT["ni"], LIGHT["nj"], split=LIGHT["split"], seed=LIGHT["seed"],
                     order=order, CFL=2.0, msweep=2)
    h0, q0 = _march(oracle_lib, case, 0, 5)
    hr, qr = _march(oracle_lib, case, 0, 5, kind="reference")
    assert np.array_equal(h0, hr) and np.array_equal(q0, qr)


def test_extended_rule_converges_on_a_half_split_mesh(make_case, oracle_lib):
    # the reference's rule puts freestream ghosts inside the domain here;
    # the extended rule converges (first order, CFL 10)
    case = make_case(24, 8, split=0.5, seed=1, order=1, CFL=10.0, msweep=2)
    h, _ = _march(oracle_lib, case, 1, 1500)
    assert h[-1, 0] < 1e-9 * 1.0 and np.all(np.isfinite(h))


def test_reference_rule_rejects_short_open_chains(make_case, native_lib):
    from hamstr_oop_gb300 import native
    case = make_case(24, 8, split=0.5, seed=1, order=3)
    c = native.Case(case)
    with pytest.raises(native.HamstrError) as ei:
        native.GpuSolver(c)
    assert ei.value.status == -2 and "extended" in str(ei.value)


def test_case_option_validation(make_case, native_lib):
    from hamstr_oop_gb300 import native
    c = native.Case(make_case(16, 4))
    with pytest.raises(native.HamstrError):
        c.set_option("chain_end_rule", 7)
    with pytest.raises(native.HamstrError):
        c.set_option("no_such_option", 1)
    c.set_option("chain_end_rule", native.END_RULE_EXTENDED)
