"""ctypes driver for the two CPU oracles (TEST INFRASTRUCTURE ONLY).

* ``kind="port"``      -- oracle/_ref/libhamstr_oracle.so, the C restatement
  (hamstr_oracle.c); builds everywhere, including the GPU host.
* ``kind="reference"`` -- oracle/_ref/libhamstr_ref.so, the reference's own
  sources compiled with ref_harness.cpp; only where the reference sources
  are present.

Both expose the same handle API, so tests compare them array by array.  Only
tests/, the smoke check and the CPU-baseline leg of bench.py import this.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
PORT_LIB = os.path.join(REF_DIR, "libhamstr_oracle.so")
REF_LIB = os.path.join(REF_DIR, "libhamstr_ref.so")
REFERENCE_SOURCES = os.environ.get("HAMSTR_REFERENCE_DIR", "/root/reference")

SIZE_NAMES = ("nCell", "nFace", "nChain", "nChainFace", "nMaxChain", "order",
              "msweep", "nGhost", "nNode", "nColor")
PARAM_NAMES = ("Mach", "alpha", "CFL", "gamma", "rinf", "uinf", "vinf", "einf", "pinf")


def build(reference: bool | None = None) -> None:
    """Compile the port (always) and the reference library (when its sources exist)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if reference is None:
        reference = os.path.isdir(REFERENCE_SOURCES)
    if reference:
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REFDIR=" + REFERENCE_SOURCES], check=True)


_LIBS: dict = {}


def _lib(kind: str):
    if kind in _LIBS:
        return _LIBS[kind]
    path = PORT_LIB if kind == "port" else REF_LIB
    if not os.path.exists(path):
        build(reference=(kind == "reference"))
    lib = ctypes.CDLL(path)
    p = "ho_" if kind == "port" else "ref_"
    vp, dp, ip, i, d = ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    fns = {
        "open": (vp, [ctypes.c_char_p] + ([ctypes.c_char_p, i] if kind == "port" else [])),
        "close": (None, [vp]),
        "sizes": (None, [vp, ip]),
        "params": (None, [vp, dp]),
        "set_freestream": (None, [vp, d, d, d]),
        "set_run": (None, [vp, i, i, d]),
        "compute_rhs": (i if kind == "port" else None, [vp, i, dp, dp]),
        "adi": (i if kind == "port" else None, [vp, dp, dp]),
        "linear_rhs": (i if kind == "port" else None, [vp, dp, dp]),
        "step": (i if kind == "port" else None, [vp, dp]),
        "march": (i if kind == "port" else None, [vp, i, dp]),
        "get": (i, [vp, ctypes.c_char_p, dp]),
        "set": (i, [vp, ctypes.c_char_p, dp]),
        "get_int": (i, [vp, ctypes.c_char_p, ip]),
    }
    for name, (res, args) in fns.items():
        fn = getattr(lib, p + name)
        fn.restype, fn.argtypes = res, args
    if kind == "port":
        lib.ho_clone.restype, lib.ho_clone.argtypes = vp, [vp]
        lib.ho_march_replicas.restype = i
        lib.ho_march_replicas.argtypes = [ctypes.POINTER(vp), i, i]
    _LIBS[kind] = (lib, p)
    return _LIBS[kind]


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


class OracleCase:
    """One case directory driven through either CPU oracle."""

    def __init__(self, case_dir: str, kind: str = "port", _handle=None):
        self.kind = kind
        self.lib, self.p = _lib(kind)
        self.case_dir = case_dir
        if _handle is not None:
            self.h = _handle
        elif kind == "port":
            err = ctypes.create_string_buffer(512)
            self.h = self._fn("open")(case_dir.encode(), err, 512)
            if not self.h:
                raise RuntimeError("oracle open failed: " + err.value.decode())
        else:
            self.h = self._fn("open")(os.path.abspath(case_dir).encode())
            if not self.h:
                raise RuntimeError("reference open failed for " + case_dir)
        s = np.zeros(10, dtype=np.int32)
        self._fn("sizes")(self.h, _ptr(s))
        self.sizes = dict(zip(SIZE_NAMES, (int(v) for v in s)))

    def _fn(self, name):
        return getattr(self.lib, self.p + name)

    def close(self):
        if self.h:
            self._fn("close")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def clone(self) -> "OracleCase":
        assert self.kind == "port"
        return OracleCase(self.case_dir, "port", _handle=self.lib.ho_clone(self.h))

    @property
    def params(self) -> dict:
        v = np.zeros(9)
        self._fn("params")(self.h, _ptr(v))
        return dict(zip(PARAM_NAMES, (float(x) for x in v)))

    def set_freestream(self, uinf, vinf, einf):
        self._fn("set_freestream")(self.h, uinf, vinf, einf)

    def set_run(self, order, msweep, cfl):
        self._fn("set_run")(self.h, order, msweep, cfl)

    def set_option(self, name: str, value: int) -> None:
        """Project options of the restatement (``chain_end_rule``); the
        reference build has none and accepts only the reference values."""
        if self.kind != "port":
            if value != 0:
                raise ValueError("the reference has no option %s=%d" % (name, value))
            return
        fn = self.lib.ho_set_option
        fn.restype, fn.argtypes = ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int]
        if fn(self.h, name.encode(), int(value)) != 0:
            raise ValueError("bad oracle option %s=%r" % (name, value))

    def forces(self) -> dict:
        """Wall pressure force (project addition, restated by ho_forces)."""
        if self.kind != "port":
            raise ValueError("the reference computes no forces")
        fn = self.lib.ho_forces
        fn.restype, fn.argtypes = ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]
        out = np.zeros(6)
        self._check(fn(self.h, _ptr(out)))
        return dict(zip(("Fx", "Fy", "M", "CL", "CD", "CM"), (float(v) for v in out)))

    def _check(self, rc):
        if rc is not None and rc != 0:
            raise RuntimeError("oracle returned status %d" % rc)

    def compute_rhs(self, implicit=True):
        a, b = ctypes.c_double(), ctypes.c_double()
        self._check(self._fn("compute_rhs")(self.h, int(implicit), ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def adi(self):
        a, b = ctypes.c_double(), ctypes.c_double()
        self._check(self._fn("adi")(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def linear_rhs(self):
        a, b = ctypes.c_double(), ctypes.c_double()
        self._check(self._fn("linear_rhs")(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def step(self):
        out = np.zeros(4)
        self._check(self._fn("step")(self.h, _ptr(out)))
        return out

    def march(self, n):
        hist = np.zeros((n, 4))
        self._check(self._fn("march")(self.h, n, _ptr(hist)))
        return hist

    def step_explicit(self, scheme: str):
        out = np.zeros(2)
        if self.kind == "port":
            fn = self.lib.ho_step_explicit
            fn.restype, fn.argtypes = ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
            self._check(fn(self.h, {"euler": 0, "rk3": 1}[scheme], _ptr(out)))
        else:
            fn = self.lib.ref_step_scheme
            fn.restype, fn.argtypes = None, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p]
            fn(self.h, scheme.encode(), _ptr(out))
        return out

    _DSIZE = {"q": ("nCell", 4), "qt": ("nCell", 4), "r": ("nCell", 4), "r0": ("nCell", 4), "dq": ("nCell", 4),
              "sigma": ("nCell", 1), "ff": ("nFace", 32), "x": ("nNode", 2), "vol": ("nCell", 1),
              "normVec": ("nFace", 2), "refMtx": ("nFace", 4)}

    def get(self, name) -> np.ndarray:
        key, w = self._DSIZE[name]
        out = np.zeros(self.sizes[key] * w)
        rc = self._fn("get")(self.h, name.encode(), _ptr(out))
        if rc != 0:
            raise KeyError(name)
        return out

    def set(self, name, arr):
        arr = np.ascontiguousarray(arr, dtype=np.float64).ravel()
        key, w = self._DSIZE[name]
        assert arr.size == self.sizes[key] * w
        rc = self._fn("set")(self.h, name.encode(), _ptr(arr))
        if rc != 0:
            raise KeyError(name)

    _ISIZE = {"faces": ("nFace", 6), "chainConn": ("nChainFace", 1),
              "faceStartPerChain": ("nChain", 1), "c2chain": ("nCell", 2),
              "bFaces": ("nFace", 1), "chainsPerColor": ("nColor", 1)}

    def get_int(self, name) -> np.ndarray:
        key, w = self._ISIZE[name]
        n = self.sizes[key] * w + (1 if name == "faceStartPerChain" else 0)
        out = np.zeros(n, dtype=np.int32)
        rc = self._fn("get_int")(self.h, name.encode(), _ptr(out))
        if rc < 0:
            raise KeyError(name)
        if name == "bFaces":
            out = out[:rc]
        return out


def block_tridag4(a, b, c, f, periodic: bool, kind: str = "port"):
    """In-place 4x4 block-tridiagonal solve of one line (copies are made)."""
    lib, p = _lib(kind)
    fn = getattr(lib, p + "block_tridag4")
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_int, ctypes.c_int]
    a, b, c, f = (np.array(x, dtype=np.float64, order="C", copy=True) for x in (a, b, c, f))
    if fn(_ptr(a), _ptr(b), _ptr(c), _ptr(f), int(f.shape[0]), int(periodic)) != 0:
        raise ValueError("bad block_tridag4 arguments")
    return f


def mlp_nparams() -> int:
    lib, _ = _lib("port")
    lib.mo_nparams.restype = ctypes.c_int
    return int(lib.mo_nparams())


def mlp_loss_grad(params, feat, targ, bf16: bool = True, grad: bool = True):
    """Loss, gradient (or None) and outputs of the warm-start network
    restated in FP64 (oracle/mlp_oracle.c); bf16 rounds what the GPU holds
    in BF16."""
    lib, _ = _lib("port")
    fn = lib.mo_loss_grad
    fn.restype = ctypes.c_double
    fn.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    p = np.ascontiguousarray(params, dtype=np.float64)
    f = np.ascontiguousarray(feat, dtype=np.float64)
    t = np.ascontiguousarray(targ, dtype=np.float64)
    n = f.shape[0]
    g = np.zeros(p.shape[0]) if grad else None
    y = np.zeros((n, 4))
    loss = fn(_ptr(p), _ptr(f), _ptr(t), n, int(bf16), _ptr(g) if grad else None, _ptr(y))
    return loss, g, y


def march_replicas(cases, iters: int) -> None:
    """Run ``iters`` steps on each port case, one OpenMP thread per case."""
    lib, _ = _lib("port")
    arr = (ctypes.c_void_p * len(cases))(*[c.h for c in cases])
    rc = lib.ho_march_replicas(arr, len(cases), iters)
    if rc != 0:
        raise RuntimeError("oracle replica march failed")


# ---------------------------------------------------------------------------
# The reference's per-face and per-line functions (checkers of the library's
# function-level entry points).  Arrays are numpy float64; "reference" needs
# an open reference case handle for the SOLVER methods.
# ---------------------------------------------------------------------------

def flux_roe2d(nxy, ql, qr, gamma: float = 1.4, kind: str = "port", case: "OracleCase" = None):
    """SOLVER::fluxRoe2D face by face: (flux [n][4], spec [n])."""
    lib, p = _lib(kind)
    nxy, ql, qr = (np.ascontiguousarray(a, dtype=np.float64) for a in (nxy, ql, qr))
    n = nxy.shape[0]
    flux, spec = np.zeros((n, 4)), np.zeros(n)
    if kind == "port":
        fn = lib.ho_flux_roe2d
        fn.restype, fn.argtypes = ctypes.c_int, [ctypes.c_void_p] * 5 + [ctypes.c_double]
    else:
        fn = lib.ref_flux_roe2d
        fn.restype, fn.argtypes = None, [ctypes.c_void_p] * 6 + [ctypes.c_double]
    for k in range(n):
        s = np.array(nxy[k])
        a, b = np.array(ql[k]), np.array(qr[k])
        fl, sp = np.zeros(4), np.zeros(1)
        if kind == "port":
            fn(_ptr(s), _ptr(a), _ptr(b), _ptr(fl), _ptr(sp), gamma)
        else:
            fn(case.h, _ptr(s), _ptr(a), _ptr(b), _ptr(fl), _ptr(sp), gamma)
        flux[k], spec[k] = fl, sp[0]
    return flux, spec


def jacobian_roe2d(nxy, ql, qr, gamma: float = 1.4, kind: str = "port", case: "OracleCase" = None):
    """SOLVER::jacobianRoe2D face by face: (lmat [n][4][4], rmat [n][4][4])."""
    lib, p = _lib(kind)
    nxy, ql, qr = (np.ascontiguousarray(a, dtype=np.float64) for a in (nxy, ql, qr))
    n = nxy.shape[0]
    lm, rm = np.zeros((n, 4, 4)), np.zeros((n, 4, 4))
    if kind == "port":
        fn = lib.ho_jacobian_roe2d
        fn.restype, fn.argtypes = None, [ctypes.c_void_p] * 5 + [ctypes.c_double]
    else:
        fn = lib.ref_jacobian_roe2d
        fn.restype, fn.argtypes = None, [ctypes.c_void_p] * 6 + [ctypes.c_double]
    for k in range(n):
        s = np.array(nxy[k])
        a, b = np.array(ql[k]), np.array(qr[k])
        l4, r4 = np.zeros(16), np.zeros(16)
        if kind == "port":
            fn(_ptr(s), _ptr(a), _ptr(b), _ptr(l4), _ptr(r4), gamma)
        else:
            fn(case.h, _ptr(s), _ptr(a), _ptr(b), _ptr(l4), _ptr(r4), gamma)
        lm[k], rm[k] = l4.reshape(4, 4), r4.reshape(4, 4)
    return lm, rm


def recon_line(name: str, f, is_: int, ie: int, *, dq=None, th: float = 1.0 / 3.0, qt: float = 0.25,
               eps: float = 1e-10, ql=None, qr=None, f2=None, kind: str = "port"):
    """RECONSTRUCTION::MUSCL / MUSCL_DERIV / WENO / WENO_DERIV on one line
    f [imax][nq] (name "muscl", "muscl_deriv", "weno", "weno_deriv").
    ql, qr, f2 give the arrays' prior contents (entries the function does
    not write keep them); returns (ql, qr, f2)."""
    lib, p = _lib(kind)
    f = np.array(f, dtype=np.float64, order="C", copy=True)
    imax, nq = f.shape
    ql = np.zeros_like(f) if ql is None else np.array(ql, dtype=np.float64, order="C", copy=True)
    qr = np.zeros_like(f) if qr is None else np.array(qr, dtype=np.float64, order="C", copy=True)
    f2 = np.zeros_like(f) if f2 is None else np.array(f2, dtype=np.float64, order="C", copy=True)
    vp, i, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    fn = getattr(lib, p + name + "_line")
    fn.restype = None
    if name == "muscl":
        fn.argtypes = [vp] * 4 + [i, i, d, d, d, i, i]
        fn(_ptr(f), _ptr(ql), _ptr(qr), _ptr(f2), is_, ie, th, qt, eps, imax, nq)
    elif name == "muscl_deriv":
        dqa = np.array(dq, dtype=np.float64, order="C", copy=True)
        fn.argtypes = [vp] * 5 + [i, i, d, d, d, i, i]
        fn(_ptr(f), _ptr(ql), _ptr(qr), _ptr(f2), _ptr(dqa), is_, ie, th, qt, eps, imax, nq)
    elif name == "weno":
        fn.argtypes = [vp] * 3 + [i, i, d, i, i]
        fn(_ptr(f), _ptr(ql), _ptr(qr), is_, ie, eps, imax, nq)
    elif name == "weno_deriv":
        dqa = np.array(dq, dtype=np.float64, order="C", copy=True)
        fn.argtypes = [vp] * 4 + [i, i, d, i, i]
        fn(_ptr(f), _ptr(ql), _ptr(qr), _ptr(dqa), is_, ie, eps, imax, nq)
    else:
        raise ValueError(name)
    return ql, qr, f2


def _face_loop(fn_port, fn_ref, nq: int, nout: int, nxyz, ql, qr, gamma, kind, case):
    """Calls a per-face function face by face: returns its two outputs."""
    lib, p = _lib(kind)
    nxyz, ql, qr = (np.ascontiguousarray(a, dtype=np.float64) for a in (nxyz, ql, qr))
    n = nxyz.shape[0]
    fn = getattr(lib, fn_port if kind == "port" else fn_ref)
    if kind == "port":
        fn.restype, fn.argtypes = None, [ctypes.c_void_p] * 5 + [ctypes.c_double]
    else:
        fn.restype, fn.argtypes = None, [ctypes.c_void_p] * 6 + [ctypes.c_double]
    o1, o2 = np.zeros((n, nout[0])), np.zeros((n, nout[1]))
    for k in range(n):
        s, a, b = np.array(nxyz[k]), np.array(ql[k]), np.array(qr[k])
        x, y = np.zeros(nout[0]), np.zeros(nout[1])
        if kind == "port":
            fn(_ptr(s), _ptr(a), _ptr(b), _ptr(x), _ptr(y), gamma)
        else:
            fn(case.h, _ptr(s), _ptr(a), _ptr(b), _ptr(x), _ptr(y), gamma)
        o1[k], o2[k] = x, y
    return o1, o2


def flux_roe3d(nxyz, ql, qr, gamma: float = 1.4, kind: str = "port", case: "OracleCase" = None):
    """SOLVER::fluxRoe3D face by face: (flux [n][5], spec [n])."""
    flux, spec = _face_loop("ho_flux_roe3d", "ref_flux_roe3d", 5, (5, 1), nxyz, ql, qr, gamma, kind, case)
    return flux, spec[:, 0]


def jacobian_roe3d(nxyz, ql, qr, gamma: float = 1.4, kind: str = "port", case: "OracleCase" = None):
    """SOLVER::jacobianRoe3D face by face: (lmat [n][5][5], rmat [n][5][5])."""
    lm, rm = _face_loop("ho_jacobian_roe3d", "ref_jacobian_roe3d", 5, (25, 25), nxyz, ql, qr, gamma, kind, case)
    return lm.reshape(-1, 5, 5), rm.reshape(-1, 5, 5)


def block_tridag5(a, b, c, f, periodic: bool, kind: str = "port"):
    """TRISOLVER::blockTridag / blockTridagPeriodic (nq = 5) on copies of one
    line: returns (a, b, c, f) after the call (a, b, c are its scratch)."""
    lib, p = _lib(kind)
    fn = getattr(lib, p + "block_tridag5")
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_int, ctypes.c_int]
    a, b, c, f = (np.array(x, dtype=np.float64, order="C", copy=True) for x in (a, b, c, f))
    if fn(_ptr(a), _ptr(b), _ptr(c), _ptr(f), int(f.shape[0]), int(periodic)) != 0:
        raise ValueError("bad block_tridag5 arguments")
    return a, b, c, f
