"""The case generator writes meshes in the reference's conventions."""
import numpy as np

from hamstr_oop_gb300 import meshgen


def test_counts_and_chain_convention():
    m = meshgen.naca0012_ogrid(16, 4)
    assert m.n_cell == 64 and m.n_face == 16 * 4 + 16 * 5
    assert len(m.chains) == 4 + 16 and m.colors == [4, 16]
    f = m.faces
    # closed loops: first face repeated, face k left = cell k, right = cell k-1
    for ch in m.chains[:4]:
        assert ch[0] == ch[-1]
        cells = [f[x, 2] for x in ch[:-1]]
        for k, x in enumerate(ch[:-1]):
            assert f[x, 3] == cells[k - 1]
    # open lines: wall face, interior faces, far-field face
    for ch in m.chains[4:]:
        assert f[ch[0], 3] == -1 and f[ch[-1], 3] == -1
        assert f[ch[-1], 2] == f[ch[-2], 2]


def test_normals_point_left_to_right():
    m = meshgen.naca0012_ogrid(24, 6)
    cent = m.nodes[m.conn].mean(axis=1)
    for a, b, l, r, _, _ in m.faces:
        (x1, y1), (x2, y2) = m.nodes[a], m.nodes[b]
        n = np.array([y2 - y1, -(x2 - x1)])
        mid = 0.5 * (m.nodes[a] + m.nodes[b])
        assert n @ (mid - cent[l]) > 0
        if r >= 0:
            assert n @ (cent[r] - mid) > 0


def test_wall_and_farfield_radii():
    m = meshgen.naca0012_ogrid(32, 8)
    r = np.hypot(m.nodes[:, 0], m.nodes[:, 1])
    wall = [x for ch in m.chains[8:] for x in ch[:1]]
    far = [x for ch in m.chains[8:] for x in ch[-1:]]
    assert all(0.5 * (r[m.faces[x, 0]] + r[m.faces[x, 1]]) < 3.0 for x in wall)
    assert all(0.5 * (r[m.faces[x, 0]] + r[m.faces[x, 1]]) > 3.0 for x in far)
