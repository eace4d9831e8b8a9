"""ctypes bindings of the C ABI in include/hamstr_gpu.h.

The library is ``hamstr_oop_gb300/lib/libhamstr_gb300.so`` built by
``hamstr_oop_gb300.build``.  There is no CPU fallback: if the library is
missing, loading raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libhamstr_gb300.so")
HEADER = os.path.join(os.path.dirname(PKG), "include", "hamstr_gpu.h")

SIZE_NAMES = ("nCell", "nFace", "nChain", "nChainFace", "nMaxChain", "order",
              "msweep", "nGhost", "nNode", "nColor")
PARAM_NAMES = ("Mach", "alpha", "CFL", "gamma", "rinf", "uinf", "vinf", "einf", "pinf")

_lib = None


class HamstrError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("%s (status %d)" % (msg, status))
        self.status = status


class Params(ctypes.Structure):
    _fields_ = [("order", ctypes.c_int), ("msweep", ctypes.c_int), ("CFL", ctypes.c_double),
                ("gamma", ctypes.c_double), ("rinf", ctypes.c_double), ("uinf", ctypes.c_double),
                ("vinf", ctypes.c_double), ("einf", ctypes.c_double), ("chain_end_rule", ctypes.c_int),
                ("limiter", ctypes.c_int)]

END_RULE_REFERENCE = 0
END_RULE_EXTENDED = 1
LIMITER_REFERENCE = 0
LIMITER_MINMOD = 1
LIMITER_VANALBADA = 2


def lib_path() -> str:
    return LIB_PATH


def load(build_if_missing: bool = False):
    """Load the native library (optionally building it first)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise RuntimeError("libhamstr_gb300.so is not built; run `python -m hamstr_oop_gb300.build`")
        from . import build
        build.build()
    L = ctypes.CDLL(LIB_PATH)
    vp, i, d, cp = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_char_p
    pp = ctypes.POINTER(ctypes.c_void_p)
    sig = {
        "hamstr_case_open": (i, [cp, pp, cp, i]),
        "hamstr_case_close": (None, [vp]),
        "hamstr_case_sizes": (i, [vp, vp]),
        "hamstr_case_params": (i, [vp, vp]),
        "hamstr_case_get_int": (i, [vp, cp, vp, ctypes.POINTER(i)]),
        "hamstr_case_get": (i, [vp, cp, vp]),
        "hamstr_case_set_run": (i, [vp, i, i, d]),
        "hamstr_case_set_freestream": (i, [vp, d, d, d]),
        "hamstr_case_set_option": (i, [vp, ctypes.c_char_p, i]),
        "hamstr_case_clone": (i, [vp, pp]),
        "hamstr_case_set_flow": (i, [vp, d, d]),
        "hamstr_gpu_set_cfl": (i, [vp, d]),
        "hamstr_mlp_gemm": (i, [vp, vp, i, i, i, i, vp, vp, vp]),
        "hamstr_mlp_nparams": (i, []),
        "hamstr_mlp_create": (i, [i, ctypes.c_ulonglong, pp]),
        "hamstr_mlp_destroy": (i, [vp]),
        "hamstr_mlp_set_params": (i, [vp, vp]),
        "hamstr_mlp_get_params": (i, [vp, vp]),
        "hamstr_mlp_get_grads": (i, [vp, vp]),
        "hamstr_mlp_forward": (i, [vp, vp, i, vp]),
        "hamstr_mlp_grad": (i, [vp, vp, vp, i, ctypes.POINTER(d)]),
        "hamstr_mlp_train_step": (i, [vp, vp, vp, ctypes.c_longlong, i, ctypes.c_ulonglong, ctypes.c_ulonglong,
                                      ctypes.c_float, ctypes.POINTER(d)]),
        "hamstr_gpu_autotune": (i, [vp, i, ctypes.c_char_p, i]),
        "hamstr_gpu_get_shape": (i, [vp, vp]),
        "hamstr_gpu_set_shape": (i, [vp, vp]),
        "hamstr_gpu_set_geometry": (i, [vp, i, vp]),
        "hamstr_gpu_forces": (i, [vp, vp]),
        "hamstr_gpu_create": (i, [ctypes.POINTER(Params), i, i, vp, vp, vp, i, vp, vp, pp]),
        "hamstr_gpu_create_from_case": (i, [vp, pp]),
        "hamstr_gpu_create_batch": (i, [vp, i, pp]),
        "hamstr_gpu_instances": (i, [vp, ctypes.POINTER(i), vp]),
        "hamstr_gpu_instance_norms": (i, [vp, vp]),
        "hamstr_gpu_batch_forces": (i, [vp, vp]),
        "hamstr_gpu_destroy": (i, [vp]),
        "hamstr_gpu_strerror": (cp, [i]),
        "hamstr_gpu_last_error": (cp, []),
        "hamstr_gpu_get": (i, [vp, cp, vp]),
        "hamstr_gpu_set": (i, [vp, cp, vp]),
        "hamstr_gpu_compute_rhs": (i, [vp, i, ctypes.POINTER(d), ctypes.POINTER(d)]),
        "hamstr_gpu_adi": (i, [vp, ctypes.POINTER(d), ctypes.POINTER(d)]),
        "hamstr_gpu_linear_rhs": (i, [vp, ctypes.POINTER(d), ctypes.POINTER(d)]),
        "hamstr_gpu_step": (i, [vp, vp]),
        "hamstr_gpu_step_host": (i, [vp, vp, vp, vp]),
        "hamstr_gpu_march": (i, [vp, i, d, vp, ctypes.POINTER(i), ctypes.POINTER(i)]),
        "hamstr_gpu_stream": (vp, [vp]),
        "hamstr_gpu_step_explicit": (i, [vp, i, vp]),
        "hamstr_gpu_set_precision": (i, [vp, i]),
        "hamstr_gpu_set_sweep_order": (i, [vp, i]),
        "hamstr_gpu_update_solution": (i, [vp, cp, cp, d]),
        "hamstr_gpu_enqueue_steps": (i, [vp, i]),
        "hamstr_gpu_sync": (i, [vp]),
        "hamstr_gpu_layout": (i, [vp, vp]),
        "hamstr_gpu_profile_step": (i, [vp, i, ctypes.POINTER(cp), vp, vp, ctypes.POINTER(i)]),
        "hamstr_gpu_launches_per_step": (i, [vp]),
        "hamstr_gpu_block_tridag4": (i, [i, i, i, vp, vp, vp, vp, vp]),
        "hamstr_gpu_block_tridag4_noalloc": (i, [i, i, i, vp, vp, vp, vp, vp]),
        "hamstr_gpu_flux_roe2d": (i, [i, vp, vp, vp, vp, vp, d, vp]),
        "hamstr_gpu_jacobian_roe2d": (i, [i, vp, vp, vp, vp, vp, d, vp]),
        "hamstr_gpu_muscl": (i, [i, i, i, vp, vp, vp, vp, i, i, d, d, d, vp]),
        "hamstr_gpu_muscl_deriv": (i, [i, i, i, vp, vp, vp, vp, vp, i, i, d, d, d, vp]),
        "hamstr_gpu_weno": (i, [i, i, i, vp, vp, vp, i, i, d, vp]),
        "hamstr_gpu_weno_deriv": (i, [i, i, i, vp, vp, vp, vp, i, i, d, vp]),
        "hamstr_gpu_flux_roe3d": (i, [i, vp, vp, vp, vp, vp, d, vp]),
        "hamstr_gpu_jacobian_roe3d": (i, [i, vp, vp, vp, vp, vp, d, vp]),
        "hamstr_gpu_block_tridag5": (i, [i, i, i, vp, vp, vp, vp, vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype, fn.argtypes = res, args
    _lib = L
    return L


def declared_symbols() -> list:
    """Function names declared in include/hamstr_gpu.h."""
    import re
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(hamstr_[a-z_0-9]+)\s*\(", txt)))


def _tridag_operands(name: str, A, B, C, F):
    """(nlines, N) of a batched block-tridiagonal system after checking that
    A, B, C are (nlines, N, 4, 4) and F is (nlines, N, 4), all contiguous
    float64 CUDA tensors on one device: the kernel reads every block of
    every line, so a smaller operand would be read past its end."""
    import torch
    if F.dim() != 3 or F.shape[2] != 4:
        raise ValueError("%s: F must be (nlines, N, 4), got %s" % (name, tuple(F.shape)))
    nl, n = int(F.shape[0]), int(F.shape[1])
    for t in (A, B, C, F):
        if not (t.is_cuda and t.is_contiguous() and t.dtype == torch.float64):
            raise ValueError("%s needs contiguous float64 CUDA tensors" % name)
        if t.device != F.device:
            raise ValueError("%s: every operand must be on %s" % (name, F.device))
    for label, t in (("A", A), ("B", B), ("C", C)):
        if tuple(t.shape) != (nl, n, 4, 4):
            raise ValueError("%s: %s must be %s, got %s" % (name, label, (nl, n, 4, 4), tuple(t.shape)))
    return nl, n


def block_tridag4(A, B, C, F, periodic: bool, stream: int = 0):
    """Batched block-tridiagonal solve on device memory (torch CUDA tensors).

    A, B, C: (nlines, N, 4, 4) float64; F: (nlines, N, 4) float64, solved in
    place.  Runs on the operands' device."""
    import torch
    nl, n = _tridag_operands("block_tridag4", A, B, C, F)
    with torch.cuda.device(F.device):
        _check(load().hamstr_gpu_block_tridag4(nl, n, int(periodic), A.data_ptr(), B.data_ptr(), C.data_ptr(),
                                               F.data_ptr(), stream or None))


def block_tridag4_noalloc(A, B, C, F, periodic: bool, stream: int = 0):
    """block_tridag4 without device allocation (fixed 8 MiB scratch in the
    library; nlines*(80*N+16) <= 1048576).  Only enqueues on `stream`: the
    caller synchronises before reading F.  For callers that cannot allocate
    device memory per call (loops beside other streams, pool-owned memory).
    Runs on the operands' device, with that device's scratch."""
    import torch
    nl, n = _tridag_operands("block_tridag4_noalloc", A, B, C, F)
    with torch.cuda.device(F.device):
        _check(load().hamstr_gpu_block_tridag4_noalloc(nl, n, int(periodic), A.data_ptr(), B.data_ptr(),
                                                       C.data_ptr(), F.data_ptr(), stream or None))


def _f64_cuda(name: str, shape: tuple, *ts):
    """Check that every tensor is a contiguous float64 CUDA tensor of `shape`
    on the first one's device (the kernels index them by that shape)."""
    import torch
    dev = ts[0].device
    for t in ts:
        if not (t.is_cuda and t.is_contiguous() and t.dtype == torch.float64):
            raise ValueError("%s needs contiguous float64 CUDA tensors" % name)
        if t.device != dev:
            raise ValueError("%s: every operand must be on %s" % (name, dev))
        if tuple(t.shape) != tuple(shape):
            raise ValueError("%s: operand of shape %s, expected %s" % (name, tuple(t.shape), tuple(shape)))
    return dev


def flux_roe2d(nxy, ql, qr, gamma: float = 1.4):
    """SOLVER::fluxRoe2D over n faces (hamstr_gpu_flux_roe2d) on torch CUDA
    tensors nxy (n, 2), ql, qr (n, 4): returns (flux (n, 4), spec (n,))."""
    import torch
    n = int(nxy.shape[0])
    dev = _f64_cuda("flux_roe2d", (n, 2), nxy)
    _f64_cuda("flux_roe2d", (n, 4), ql, qr)
    flux = torch.empty((n, 4), dtype=torch.float64, device=dev)
    spec = torch.empty((n,), dtype=torch.float64, device=dev)
    with torch.cuda.device(dev):
        _check(load().hamstr_gpu_flux_roe2d(n, nxy.data_ptr(), ql.data_ptr(), qr.data_ptr(), flux.data_ptr(),
                                            spec.data_ptr(), float(gamma), torch.cuda.current_stream().cuda_stream))
    return flux, spec


def jacobian_roe2d(nxy, ql, qr, gamma: float = 1.4):
    """SOLVER::jacobianRoe2D over n faces (hamstr_gpu_jacobian_roe2d):
    returns (lmat (n, 4, 4), rmat (n, 4, 4)), times the face area."""
    import torch
    n = int(nxy.shape[0])
    dev = _f64_cuda("jacobian_roe2d", (n, 2), nxy)
    _f64_cuda("jacobian_roe2d", (n, 4), ql, qr)
    lm = torch.empty((n, 4, 4), dtype=torch.float64, device=dev)
    rm = torch.empty((n, 4, 4), dtype=torch.float64, device=dev)
    with torch.cuda.device(dev):
        _check(load().hamstr_gpu_jacobian_roe2d(n, nxy.data_ptr(), ql.data_ptr(), qr.data_ptr(), lm.data_ptr(),
                                                rm.data_ptr(), float(gamma), torch.cuda.current_stream().cuda_stream))
    return lm, rm


def flux_roe3d(nxyz, ql, qr, gamma: float = 1.4):
    """SOLVER::fluxRoe3D over n faces (hamstr_gpu_flux_roe3d): nxyz (n, 3),
    ql, qr (n, 5) -> (flux (n, 5), spec (n,)), not scaled by the area."""
    import torch
    n = int(nxyz.shape[0])
    dev = _f64_cuda("flux_roe3d", (n, 3), nxyz)
    _f64_cuda("flux_roe3d", (n, 5), ql, qr)
    flux = torch.empty((n, 5), dtype=torch.float64, device=dev)
    spec = torch.empty((n,), dtype=torch.float64, device=dev)
    with torch.cuda.device(dev):
        _check(load().hamstr_gpu_flux_roe3d(n, nxyz.data_ptr(), ql.data_ptr(), qr.data_ptr(), flux.data_ptr(),
                                            spec.data_ptr(), float(gamma), torch.cuda.current_stream().cuda_stream))
    return flux, spec


def jacobian_roe3d(nxyz, ql, qr, gamma: float = 1.4):
    """SOLVER::jacobianRoe3D over n faces (hamstr_gpu_jacobian_roe3d):
    returns (lmat (n, 5, 5), rmat (n, 5, 5))."""
    import torch
    n = int(nxyz.shape[0])
    dev = _f64_cuda("jacobian_roe3d", (n, 3), nxyz)
    _f64_cuda("jacobian_roe3d", (n, 5), ql, qr)
    lm = torch.empty((n, 5, 5), dtype=torch.float64, device=dev)
    rm = torch.empty((n, 5, 5), dtype=torch.float64, device=dev)
    with torch.cuda.device(dev):
        _check(load().hamstr_gpu_jacobian_roe3d(n, nxyz.data_ptr(), ql.data_ptr(), qr.data_ptr(), lm.data_ptr(),
                                                rm.data_ptr(), float(gamma), torch.cuda.current_stream().cuda_stream))
    return lm, rm


def block_tridag5(A, B, C, F, periodic: bool) -> None:
    """TRISOLVER::blockTridag / blockTridagPeriodic (nq = 5) over lines
    (hamstr_gpu_block_tridag5), in place on torch CUDA tensors: A, B, C
    (nlines, N, 5, 5) become the reference's scratch, F (nlines, N, 5) the
    solution; on the current stream."""
    import torch
    if F.dim() != 3 or F.shape[2] != 5:
        raise ValueError("block_tridag5: F must be (nlines, N, 5), got %s" % (tuple(F.shape),))
    nl, n = int(F.shape[0]), int(F.shape[1])
    dev = _f64_cuda("block_tridag5", (nl, n, 5, 5), A, B, C)
    _f64_cuda("block_tridag5", (nl, n, 5), F)
    if F.device != dev:
        raise ValueError("block_tridag5: every operand must be on %s" % dev)
    with torch.cuda.device(dev):
        _check(load().hamstr_gpu_block_tridag5(nl, n, int(periodic), A.data_ptr(), B.data_ptr(), C.data_ptr(),
                                               F.data_ptr(), torch.cuda.current_stream().cuda_stream))


def reconstruct(name: str, f, ql, qr, is_: int, ie: int, *, dq=None, f2=None, th: float = 1.0 / 3.0,
                qt: float = 0.25, eps: float = 1e-10) -> None:
    """RECONSTRUCTION::MUSCL / MUSCL_DERIV / WENO / WENO_DERIV over lines
    (hamstr_gpu_muscl etc.): f, ql, qr (and dq, f2) are (nlines, imax, nq)
    torch CUDA tensors; ql, qr (and f2) are written in place on the entries
    the reference writes, on the current stream."""
    import torch
    nl, imax, nq = (int(x) for x in f.shape)
    shape = (nl, imax, nq)
    ops = [f, ql, qr] + ([dq] if name in ("muscl_deriv", "weno_deriv") else []) + \
        ([f2] if name in ("muscl", "muscl_deriv") else [])
    dev = _f64_cuda(name, shape, *ops)
    L = load()
    with torch.cuda.device(dev):
        st = torch.cuda.current_stream().cuda_stream
        if name == "muscl":
            rc = L.hamstr_gpu_muscl(nl, imax, nq, f.data_ptr(), ql.data_ptr(), qr.data_ptr(), f2.data_ptr(), is_, ie,
                                    th, qt, eps, st)
        elif name == "muscl_deriv":
            rc = L.hamstr_gpu_muscl_deriv(nl, imax, nq, f.data_ptr(), dq.data_ptr(), ql.data_ptr(), qr.data_ptr(),
                                          f2.data_ptr(), is_, ie, th, qt, eps, st)
        elif name == "weno":
            rc = L.hamstr_gpu_weno(nl, imax, nq, f.data_ptr(), ql.data_ptr(), qr.data_ptr(), is_, ie, eps, st)
        elif name == "weno_deriv":
            rc = L.hamstr_gpu_weno_deriv(nl, imax, nq, f.data_ptr(), dq.data_ptr(), ql.data_ptr(), qr.data_ptr(),
                                         is_, ie, eps, st)
        else:
            raise ValueError(name)
    _check(rc)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _check(st: int):
    if st != 0:
        L = load()
        msg = L.hamstr_gpu_strerror(st).decode()
        det = L.hamstr_gpu_last_error()
        if det:
            msg += ": " + det.decode()
        raise HamstrError(st, msg)


class Case:
    """Host-side case: the reference reader + preprocessing + initial state."""

    def __init__(self, case_dir: str):
        L = load()
        h = ctypes.c_void_p()
        err = ctypes.create_string_buffer(1024)
        st = L.hamstr_case_open(case_dir.encode(), ctypes.byref(h), err, 1024)
        if st != 0:
            raise HamstrError(st, err.value.decode())
        self.h = h
        self.case_dir = case_dir
        s = np.zeros(10, dtype=np.int32)
        _check(L.hamstr_case_sizes(self.h, _ptr(s)))
        self.sizes = dict(zip(SIZE_NAMES, (int(v) for v in s)))

    def close(self):
        if self.h:
            load().hamstr_case_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def params(self) -> dict:
        v = np.zeros(9)
        _check(load().hamstr_case_params(self.h, _ptr(v)))
        return dict(zip(PARAM_NAMES, (float(x) for x in v)))

    def get_int(self, name: str) -> np.ndarray:
        L = load()
        n = ctypes.c_int(0)
        _check(L.hamstr_case_get_int(self.h, name.encode(), None, ctypes.byref(n)))
        out = np.zeros(max(n.value, 1), dtype=np.int32)
        _check(L.hamstr_case_get_int(self.h, name.encode(), _ptr(out), ctypes.byref(n)))
        return out[:n.value]

    _DW = {"x": ("nNode", 2), "vol": ("nCell", 1), "normVec": ("nFace", 2), "refMtx": ("nFace", 4),
           "q": ("nCell", 4)}

    def get(self, name: str) -> np.ndarray:
        key, w = self._DW[name]
        out = np.zeros(self.sizes[key] * w)
        _check(load().hamstr_case_get(self.h, name.encode(), _ptr(out)))
        return out

    def set_run(self, order: int, msweep: int, cfl: float):
        _check(load().hamstr_case_set_run(self.h, order, msweep, cfl))
        self.sizes = dict(self.sizes, order=order, msweep=msweep, nGhost=3 if order == 5 else 2)

    def set_freestream(self, uinf: float, vinf: float, einf: float):
        _check(load().hamstr_case_set_freestream(self.h, uinf, vinf, einf))

    def set_option(self, name: str, value: int) -> None:
        """Project options: ``chain_end_rule`` (END_RULE_*), ``limiter`` (LIMITER_*)."""
        _check(load().hamstr_case_set_option(self.h, name.encode(), int(value)))

    def clone(self) -> "Case":
        h = ctypes.c_void_p()
        _check(load().hamstr_case_clone(self.h, ctypes.byref(h)))
        c = Case.__new__(Case)
        c.h, c.case_dir, c.sizes = h, self.case_dir, dict(self.sizes)
        return c

    def set_flow(self, mach: float, alpha_deg: float) -> None:
        """New flow condition: freestream and initial state from Mach and alpha."""
        _check(load().hamstr_case_set_flow(self.h, float(mach), float(alpha_deg)))


class GpuSolver:
    """Device solver handle (the SOLVER of the drop-in)."""

    def __init__(self, case: Case = None, *, _handle=None, _sizes=None):
        if _handle is None:
            h = ctypes.c_void_p()
            _check(load().hamstr_gpu_create_from_case(case.h, ctypes.byref(h)))
            self.h = h
            self.sizes = dict(case.sizes)
        else:
            self.h, self.sizes = _handle, _sizes
        n = ctypes.c_int(0)
        _check(load().hamstr_gpu_instances(self.h, ctypes.byref(n), None))
        self.n_instances = n.value

    @classmethod
    def batch(cls, cases: list) -> "GpuSolver":
        """The batched form: all cases in one handle (hamstr_gpu_create_batch)."""
        arr = (ctypes.c_void_p * len(cases))(*[c.h for c in cases])
        h = ctypes.c_void_p()
        _check(load().hamstr_gpu_create_batch(arr, len(cases), ctypes.byref(h)))
        sizes = dict(cases[0].sizes)
        for k in ("nCell", "nFace", "nChain", "nChainFace", "nNode"):
            sizes[k] = sum(c.sizes[k] for c in cases)
        return cls(_handle=h, _sizes=sizes)

    def instance_cells(self) -> np.ndarray:
        """Cell offsets of the instances (n+1 entries)."""
        n = ctypes.c_int(0)
        out = np.zeros(self.n_instances + 1, dtype=np.int32)
        _check(load().hamstr_gpu_instances(self.h, ctypes.byref(n), _ptr(out)))
        return out

    def instance_norms(self) -> np.ndarray:
        """[n][4] last computeRHS L2, Linf and linear L2, Linf of every instance."""
        out = np.zeros((self.n_instances, 4))
        _check(load().hamstr_gpu_instance_norms(self.h, _ptr(out)))
        return out

    def batch_forces(self) -> np.ndarray:
        """[n][6] Fx, Fy, M, CL, CD, CM of every instance."""
        out = np.zeros((self.n_instances, 6))
        _check(load().hamstr_gpu_batch_forces(self.h, _ptr(out)))
        return out

    def close(self):
        if self.h:
            load().hamstr_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    _DW = {"q": ("nCell", 4), "qt": ("nCell", 4), "r": ("nCell", 4), "r0": ("nCell", 4), "dq": ("nCell", 4),
           "sigma": ("nCell", 1), "ff": ("nFace", 32)}

    def set_precision(self, mixed: bool) -> None:
        """False: plain FP64 (bit-identical); True: FP64 residual with an FP32
        Jacobian/ADI operator (defect correction)."""
        _check(load().hamstr_gpu_set_precision(self.h, int(bool(mixed))))

    def set_sweep_order(self, order: int) -> None:
        """0: the reference's sweeps (linearised residual at the scheme's
        order); 1: first-order linearised residual (same converged state)."""
        _check(load().hamstr_gpu_set_sweep_order(self.h, int(order)))

    def forces(self) -> dict:
        """Wall pressure force of the current state: Fx, Fy, M (about x=0.25), CL, CD, CM."""
        out = np.zeros(6)
        _check(load().hamstr_gpu_forces(self.h, _ptr(out)))
        return dict(zip(("Fx", "Fy", "M", "CL", "CD", "CM"), (float(v) for v in out)))

    def autotune(self, reps: int = 3) -> dict:
        """Pick the fastest launch shapes for the current precision (hamstr_gpu_autotune)."""
        import json
        buf = ctypes.create_string_buffer(131072)
        _check(load().hamstr_gpu_autotune(self.h, int(reps), buf, 131072))
        return json.loads(buf.value.decode())

    SHAPE_KEYS = ("face_block", "adi_warps_per_sm", "mx_block", "mx_fused", "face_softdiv", "pivot_softdiv",
                  "adi_open_lanes", "weno_keep", "adi_bundle_rows", "mx_chunk", "mx_spike", "adi_fuse",
                  "adi_factor_warps_per_sm")

    def shape(self) -> dict:
        """The launch shape in use (hamstr_gpu_get_shape), keyed as the autotuner's report."""
        v = (ctypes.c_int * len(self.SHAPE_KEYS))()
        _check(load().hamstr_gpu_get_shape(self.h, v))
        return dict(zip(self.SHAPE_KEYS, list(v)))

    def set_shape(self, **kw) -> None:
        """Change some launch-shape values (hamstr_gpu_set_shape); results do not depend on them."""
        cur = self.shape()
        for k, val in kw.items():
            if k not in cur:
                raise KeyError(k)
            cur[k] = int(val)
        v = (ctypes.c_int * len(self.SHAPE_KEYS))(*[cur[k] for k in self.SHAPE_KEYS])
        _check(load().hamstr_gpu_set_shape(self.h, v))

    def set_cfl(self, cfl: float) -> None:
        """CFL of later steps (a project addition for CFL ramping)."""
        _check(load().hamstr_gpu_set_cfl(self.h, float(cfl)))

    def step_explicit(self, scheme: str) -> np.ndarray:
        out = np.zeros(2)
        _check(load().hamstr_gpu_step_explicit(self.h, {"euler": 0, "rk3": 1}[scheme], _ptr(out)))
        return out

    def update_solution(self, qold: str, qnew: str, coef: float) -> None:
        _check(load().hamstr_gpu_update_solution(self.h, qold.encode(), qnew.encode(), coef))

    def get(self, name: str, out: np.ndarray = None) -> np.ndarray:
        """Copy a device array to the host; `out` (contiguous float64 of the
        right size, e.g. a pinned buffer) receives it in place of a new array."""
        key, w = self._DW[name]
        n = self.sizes[key] * w
        if out is None:
            out = np.zeros(n)
        elif out.dtype != np.float64 or out.size != n or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("%s needs a contiguous float64 array of %d values" % (name, n))
        _check(load().hamstr_gpu_get(self.h, name.encode(), _ptr(out)))
        return out

    def set(self, name: str, arr) -> None:
        key, w = self._DW[name]
        a = np.ascontiguousarray(arr, dtype=np.float64).ravel()
        if a.size != self.sizes[key] * w:
            raise ValueError("%s needs %d values" % (name, self.sizes[key] * w))
        _check(load().hamstr_gpu_set(self.h, name.encode(), _ptr(a)))

    def compute_rhs(self, implicit: bool = True):
        a, b = ctypes.c_double(), ctypes.c_double()
        _check(load().hamstr_gpu_compute_rhs(self.h, int(implicit), ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def adi(self):
        a, b = ctypes.c_double(), ctypes.c_double()
        _check(load().hamstr_gpu_adi(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def linear_rhs(self):
        a, b = ctypes.c_double(), ctypes.c_double()
        _check(load().hamstr_gpu_linear_rhs(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def step(self) -> np.ndarray:
        out = np.zeros(4)
        _check(load().hamstr_gpu_step(self.h, _ptr(out)))
        return out

    def step_host(self, q_in: np.ndarray = None, q_out: np.ndarray = None) -> np.ndarray:
        """One step on a host-resident solution (hamstr_gpu_step_host): q_in
        (or None: keep the device state) in, q_out (or None) out, one
        synchronisation.  Both are contiguous float64 arrays of 4*nCell
        values; page-locked ones (e.g. a pinned torch tensor's numpy view)
        copy at full speed."""
        n = 4 * self.sizes["nCell"]
        for a in (q_in, q_out):
            if a is not None and (a.dtype != np.float64 or a.size != n or not a.flags["C_CONTIGUOUS"]):
                raise ValueError("q needs a contiguous float64 array of %d values" % n)
        out = np.zeros(4)
        _check(load().hamstr_gpu_step_host(self.h, None if q_in is None else _ptr(q_in),
                                           None if q_out is None else _ptr(q_out), _ptr(out)))
        return out

    def march(self, nsteps: int, tol: float = 0.0):
        """(hist, converged): hist is [rows][4], or [rows][n][4] on a batched handle."""
        hist = np.zeros((max(nsteps, 1), self.n_instances, 4))
        ev, conv = ctypes.c_int(0), ctypes.c_int(0)
        _check(load().hamstr_gpu_march(self.h, nsteps, tol, _ptr(hist), ctypes.byref(ev), ctypes.byref(conv)))
        hist = hist[:ev.value]
        return (hist[:, 0, :] if self.n_instances == 1 else hist), bool(conv.value)

    def enqueue_steps(self, n: int) -> None:
        _check(load().hamstr_gpu_enqueue_steps(self.h, n))

    def sync(self) -> None:
        _check(load().hamstr_gpu_sync(self.h))

    def layout(self) -> dict:
        v = np.zeros(8, dtype=np.int32)
        _check(load().hamstr_gpu_layout(self.h, _ptr(v)))
        return dict(zip(("nSlot", "nSten", "nRow", "nChain", "nWave", "nPeriodicChains",
                         "nPeriodicRows", "maxRows"), (int(x) for x in v)))

    @property
    def stream(self) -> int:
        return int(load().hamstr_gpu_stream(self.h) or 0)

    def launches_per_step(self) -> int:
        n = load().hamstr_gpu_launches_per_step(self.h)
        if n < 0:
            _check(n)
        return n

    def profile_step(self, reps: int = 3) -> dict:
        names = (ctypes.c_char_p * 16)()
        ms = np.zeros(16)
        cnt = np.zeros(16, dtype=np.int32)
        n = ctypes.c_int(16)
        _check(load().hamstr_gpu_profile_step(self.h, reps, names, _ptr(ms), _ptr(cnt), ctypes.byref(n)))
        return {names[k].decode(): (float(ms[k]), int(cnt[k])) for k in range(n.value)}


class Mlp:
    """The warm-start network on the tensor cores (hamstr_mlp_*).  Device
    arrays are torch CUDA tensors (float32, contiguous): features [n][5],
    targets / outputs [n][4]."""

    def __init__(self, batch_capacity: int = 65536, seed: int = 1):
        h = ctypes.c_void_p()
        _check(load().hamstr_mlp_create(int(batch_capacity), int(seed), ctypes.byref(h)))
        self.h = h
        self.nparams = int(load().hamstr_mlp_nparams())

    def close(self):
        if self.h:
            load().hamstr_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.nparams, dtype=np.float32)
        _check(load().hamstr_mlp_get_params(self.h, _ptr(out)))
        return out

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        _check(load().hamstr_mlp_set_params(self.h, _ptr(p)))

    def get_grads(self) -> np.ndarray:
        out = np.zeros(self.nparams, dtype=np.float32)
        _check(load().hamstr_mlp_get_grads(self.h, _ptr(out)))
        return out

    def forward(self, feat):
        import torch
        y = torch.empty((feat.shape[0], 4), dtype=torch.float32, device=feat.device)
        _check(load().hamstr_mlp_forward(self.h, feat.data_ptr(), int(feat.shape[0]), y.data_ptr()))
        return y

    def grad(self, feat, targ) -> float:
        loss = ctypes.c_double(0.0)
        _check(load().hamstr_mlp_grad(self.h, feat.data_ptr(), targ.data_ptr(), int(feat.shape[0]),
                                      ctypes.byref(loss)))
        return loss.value

    def train_step(self, feat, targ, batch: int, seed: int, step: int, lr: float) -> float:
        loss = ctypes.c_double(0.0)
        _check(load().hamstr_mlp_train_step(self.h, feat.data_ptr(), targ.data_ptr(), int(feat.shape[0]), int(batch),
                                            int(seed), int(step), float(lr), ctypes.byref(loss)))
        return loss.value
