"""Seeded inputs of the function-level checks (Roe flux and Jacobian per
face, reconstructions per line), shared by the CPU and GPU tests."""
import numpy as np

GAMMA = 1.4


def faces(n: int, seed: int):
    """n faces: normals (dy, -dx) of lengths 1e-3..1 in every direction and
    physical left/right states (density, momentum, total energy), some pairs
    nearly equal so the Roe averages' small-difference branches are taken."""
    rng = np.random.default_rng(seed)
    ang = rng.uniform(0.0, 2.0 * np.pi, n)
    mag = 10.0 ** rng.uniform(-3.0, 0.0, n)
    nxy = np.stack([mag * np.cos(ang), mag * np.sin(ang)], axis=1)

    def states():
        rho = rng.uniform(0.4, 1.6, n)
        u, v = rng.uniform(-0.9, 0.9, n), rng.uniform(-0.9, 0.9, n)
        p = rng.uniform(0.3, 1.3, n)
        return np.stack([rho, rho * u, rho * v, p / (GAMMA - 1.0) + 0.5 * rho * (u * u + v * v)], axis=1)
    ql, qr = states(), states()
    near = rng.random(n) < 0.25
    qr[near] = ql[near] * (1.0 + 1e-9 * rng.standard_normal((int(near.sum()), 4)))
    return nxy, ql, qr


def lines(nlines: int, imax: int, nq: int, seed: int):
    """nlines lines of imax entries: smooth profiles with a jump and noise
    (f), increments (dq), and prior contents of the output arrays."""
    rng = np.random.default_rng(seed)
    x = np.linspace(0.0, 1.0, imax)[None, :, None]
    f = 1.0 + 0.3 * np.sin(6.0 * x + rng.uniform(0, 6, (nlines, 1, nq)))
    f = f + 0.2 * (x > rng.uniform(0.2, 0.8, (nlines, 1, nq)))
    f = f + 1e-3 * rng.standard_normal((nlines, imax, nq))
    f[:, imax // 3, :] = f[:, imax // 3 - 1, :]          # a zero difference
    dq = 1e-3 * rng.standard_normal((nlines, imax, nq))
    prior = rng.standard_normal((3, nlines, imax, nq))
    return f, dq, prior


def faces3d(n: int, seed: int):
    """n faces of the 5-variable (3D) form: normals in every direction with
    lengths 1e-3..1 and physical states rho, rho u, rho v, rho w, E."""
    rng = np.random.default_rng(seed)
    v = rng.standard_normal((n, 3))
    v /= np.linalg.norm(v, axis=1)[:, None]
    nxyz = v * (10.0 ** rng.uniform(-3.0, 0.0, n))[:, None]

    def states():
        rho = rng.uniform(0.4, 1.6, n)
        u = rng.uniform(-0.8, 0.8, (n, 3))
        p = rng.uniform(0.3, 1.3, n)
        e = p / (GAMMA - 1.0) + 0.5 * rho * (u * u).sum(axis=1)
        return np.column_stack([rho, rho[:, None] * u, e])
    ql, qr = states(), states()
    near = rng.random(n) < 0.25
    qr[near] = ql[near] * (1.0 + 1e-9 * rng.standard_normal((int(near.sum()), 5)))
    return nxyz, ql, qr


def blocks5(nlines: int, n: int, seed: int, dominance: float = 8.0):
    """nlines systems of n 5x5 block rows, diagonally dominant."""
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((nlines, n, 5, 5))
    b = rng.standard_normal((nlines, n, 5, 5)) + dominance * np.eye(5)
    c = rng.standard_normal((nlines, n, 5, 5))
    f = rng.standard_normal((nlines, n, 5))
    return a, b, c, f
