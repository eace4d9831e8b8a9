"""NACA 0012 O-grid generator that writes HAMSTR's on-disk case format.

The reference ships no meshes and no line/chain generator, so every case used by
the tests and the benchmark is generated here, seeded and reproducible, in
exactly the file formats that the reference reader parses:

* ``input/domain000/coord.dat``   -- ``nNode`` then ``x y z`` rows (io.cpp:144-156)
* ``input/domain000/conn.dat``    -- ``nCell`` then 4 node ids per cell (io.cpp:171-188)
* ``input/domain000/ncolors.dat`` -- ``nColor`` then chains per colour (io.cpp:205-208)
* ``input/domain000/iqloops.dat`` -- K, then K chain start offsets (io.cpp:223-245)
* ``input/domain000/qloops.dat``  -- ``nChainFace`` then face ids (io.cpp:259-264)
* ``input/domain000/qedges.dat``  -- ``nFace`` then ``n1 n2 cL cR eL eR`` (io.cpp:344-365)
* ``input.hamstr``                -- 16 ``key=value`` lines in fixed order (io.cpp:26-41)

Chain convention (the one computeRHS.cpp:62-133 and ADI.cpp:85-190 assume):

* closed loop of M cells: faces 0..M-1, face k has left = cell k and
  right = cell k-1 (mod M); face 0 is repeated at the end of the chain;
* open line of N cells: N+1 faces; face 0 (wall) has left = cell 0 and right
  = -1; interior face k has left = cell k, right = cell k-1; face N (far
  field) has left = cell N-1 and right = -1.

The face normal (dy, -dx) taken from n1 to n2 points from the left to the
right cell (preprocess.cpp:86-87).  Boundary faces whose mean node radius is
below 3.0 become walls in preprocessing (preprocess.cpp:169-190), so the
aerofoil sits with its chord on [0, 1] and the far field at radius ``rfar``
about (0.5, 0).
"""
from __future__ import annotations

import dataclasses
import math
import os

import numpy as np

INPUT_KEYS = ("Mach", "alpha", "beta", "rey", "scheme", "time integration",
              "order", "timeacc", "nsteps", "nwrite", "dt", "CFL", "msweep",
              "visc", "testcase", "output")


@dataclasses.dataclass
class Mesh:
    """A 2D mesh plus its line chains, in the reference's integer conventions."""
    nodes: np.ndarray          # (nNode, 2) float64
    conn: np.ndarray           # (nCell, 4) int, node ids (triangles repeat a node)
    faces: np.ndarray          # (nFace, 6) int: n1 n2 cL cR eL eR (file order)
    chains: list               # list of lists of face ids (closed chains repeat face 0)
    colors: list               # chains per colour, in file order
    ni: int = 0
    nj: int = 0

    @property
    def n_cell(self) -> int:
        return int(self.conn.shape[0])

    @property
    def n_face(self) -> int:
        return int(self.faces.shape[0])


def naca0012_half_thickness(x):
    """Closed-trailing-edge NACA 0012 half thickness (coefficient -0.1036)."""
    x = np.asarray(x, dtype=np.float64)
    return 0.6 * (0.2969 * np.sqrt(x) - 0.1260 * x - 0.3516 * x ** 2
                  + 0.2843 * x ** 3 - 0.1036 * x ** 4)


def _stretch_ratio(ds1: float, n: int, total: float) -> float:
    """Geometric ratio r with ds1 * (r**n - 1) / (r - 1) == total (bisection)."""
    lo, hi = 1.0 + 1e-12, 4.0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        s = ds1 * (mid ** n - 1.0) / (mid - 1.0)
        if s < total:
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi)


def naca0012_ogrid(ni: int, nj: int, ds1: float = 2e-3, rfar: float = 20.0,
                   loop_start: int | None = None) -> Mesh:
    """Structured NACA 0012 O-grid with ``ni`` wrap-around x ``nj`` wall-normal quads.

    Surface points use cosine clustering in x (dense at the leading and
    trailing edges).  Grid lines are straight rays from the surface point to
    the far-field circle at the same polar angle about (0.5, 0); the aerofoil
    is star-shaped about that point so the rays never cross.  Wall-normal
    spacing starts at ``ds1`` chords and grows geometrically to the far field.

    Cells are numbered ``j * ni + i``.  Colour 0 holds the ``nj`` closed loops
    (one per wall-normal layer), colour 1 the ``ni`` open wall-to-far-field
    lines.  Each loop starts at index ``loop_start`` (default ``ni // 2``, the
    leading edge) so that cell 0 is never the first or last cell of a loop;
    the reference's ghost test treats cell id 0 specially at those stencil
    positions (computeRHS.cpp:158,170), and starting loops at 0 would make the
    wall loop read a freestream ghost.  ``loop_start=0`` reproduces that case
    on purpose for parity tests.
    """
    if ni < 4 or nj < 2:
        raise ValueError("ogrid needs ni >= 4 and nj >= 2")
    if loop_start is None:
        loop_start = ni // 2
    theta = 2.0 * math.pi * np.arange(ni) / ni
    sx = 0.5 * (1.0 + np.cos(theta))
    sy = naca0012_half_thickness(sx) * np.where(theta <= math.pi, 1.0, -1.0)
    ang = np.arctan2(sy, sx - 0.5)
    fx = 0.5 + rfar * np.cos(ang)
    fy = rfar * np.sin(ang)
    dist = np.hypot(fx - sx, fy - sy)
    # geometric spacing in physical distance, normalised per ray
    r = _stretch_ratio(ds1, nj, float(dist.mean()))
    s = np.concatenate([[0.0], np.cumsum(ds1 * r ** np.arange(nj))])
    s = s / s[-1]
    nodes = np.empty(((nj + 1) * ni, 2), dtype=np.float64)
    for j in range(nj + 1):
        nodes[j * ni:(j + 1) * ni, 0] = sx + s[j] * (fx - sx)
        nodes[j * ni:(j + 1) * ni, 1] = sy + s[j] * (fy - sy)

    def nid(i, j):
        return j * ni + (i % ni)

    def cid(i, j):
        return j * ni + (i % ni)

    conn = np.empty((ni * nj, 4), dtype=np.int64)
    for j in range(nj):
        for i in range(ni):
            conn[cid(i, j)] = (nid(i, j), nid(i + 1, j), nid(i + 1, j + 1), nid(i, j + 1))
    centroid = nodes[conn].mean(axis=1)

    faces = []

    def add_face(a, b, left, right, el, er):
        (x1, y1), (x2, y2) = nodes[a], nodes[b]
        nx, ny = (y2 - y1), -(x2 - x1)
        mx, my = 0.5 * (x1 + x2), 0.5 * (y1 + y2)
        cx, cy = centroid[left]
        if nx * (mx - cx) + ny * (my - cy) < 0.0:
            a, b = b, a
        faces.append((a, b, left, right, el, er))
        return len(faces) - 1

    chains = []
    # colour 0: closed loops; local edges 0 bottom, 1 right, 2 top, 3 left
    for j in range(nj):
        ch = []
        for k in range(ni):
            i = (loop_start + k) % ni
            ch.append(add_face(nid(i, j), nid(i, j + 1), cid(i, j), cid(i - 1, j), 3, 1))
        chains.append(ch + [ch[0]])
    # colour 1: open wall-normal lines
    for i in range(ni):
        ch = [add_face(nid(i, 0), nid(i + 1, 0), cid(i, 0), -1, 0, -1)]
        for j in range(1, nj):
            ch.append(add_face(nid(i, j), nid(i + 1, j), cid(i, j), cid(i, j - 1), 0, 2))
        ch.append(add_face(nid(i, nj), nid(i + 1, nj), cid(i, nj - 1), -1, 2, -1))
        chains.append(ch)
    return Mesh(nodes=nodes, conn=conn, faces=np.asarray(faces, dtype=np.int64),
                chains=chains, colors=[nj, ni], ni=ni, nj=nj)


def default_inputs(**over) -> dict:
    """``input.hamstr`` values for the steady ADI path (io.cpp:26-41)."""
    d = {"Mach": 0.5, "alpha": 1.25, "beta": 0.0, "rey": 1.0e6, "scheme": "ADI",
         "time integration": "euler", "order": 3, "timeacc": 0, "nsteps": 100,
         "nwrite": 100, "dt": 0.01, "CFL": 10.0, "msweep": 2, "visc": 0,
         "testcase": 0, "output": 0}
    d.update(over)
    return d


def _fmt(v) -> str:
    if isinstance(v, float):
        return repr(float(v))
    return str(v)


def write_case(case_dir: str, mesh: Mesh, inputs: dict | None = None,
               domain: int = 0) -> str:
    """Write ``mesh`` and ``inputs`` under ``case_dir`` in the reference formats."""
    inputs = default_inputs(**(inputs or {}))
    d = os.path.join(case_dir, "input", "domain%03d" % domain)
    os.makedirs(d, exist_ok=True)
    with open(os.path.join(d, "coord.dat"), "w") as f:
        f.write("%d\n" % len(mesh.nodes))
        f.write("".join("%.17e %.17e 0.0\n" % (x, y) for x, y in mesh.nodes))
    with open(os.path.join(d, "conn.dat"), "w") as f:
        f.write("%d\n" % mesh.n_cell)
        f.write("".join("%d %d %d %d\n" % tuple(c) for c in mesh.conn))
    with open(os.path.join(d, "ncolors.dat"), "w") as f:
        f.write("%d\n" % len(mesh.colors))
        f.write("".join("%d\n" % c for c in mesh.colors))
    offsets = [0]
    for ch in mesh.chains:
        offsets.append(offsets[-1] + len(ch))
    with open(os.path.join(d, "iqloops.dat"), "w") as f:
        f.write("%d\n" % len(offsets))
        f.write("".join("%d\n" % o for o in offsets))
    with open(os.path.join(d, "qloops.dat"), "w") as f:
        f.write("%d\n" % offsets[-1])
        f.write("".join("%d\n" % x for ch in mesh.chains for x in ch))
    with open(os.path.join(d, "qedges.dat"), "w") as f:
        f.write("%d\n" % mesh.n_face)
        f.write("".join("%d %d %d %d %d %d\n" % tuple(r) for r in mesh.faces))
    with open(os.path.join(case_dir, "input.hamstr"), "w") as f:
        for k in INPUT_KEYS:
            f.write("%s=%s\n" % (k, _fmt(inputs[k])))
    return case_dir


def make_case(case_dir: str, ni: int, nj: int, **inputs) -> str:
    """Generate an O-grid case directory in one call (keyword args are inputs)."""
    loop_start = inputs.pop("loop_start", None)
    mesh = naca0012_ogrid(ni, nj, loop_start=loop_start)
    return write_case(case_dir, mesh, inputs)
