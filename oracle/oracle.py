"""ctypes binding of the CPU oracle (oracle/mpm_oracle.cpp) and of its
dual-number restatement for gradients (oracle/mpm_dual.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and bench.py's
CPU-baseline leg, never by the jump_gb300 package.  It consumes the same
descriptors as the CUDA library (jump_gb300.engine.Descriptors) so both run
on identical inputs.  Parity status: not pinned to reference outputs (the
Julia reference cannot run here and ships no golden data); pinned instead by
known answers (tests/test_oracle_pins.py) and by an independent Python
restatement (tests/golden/).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from jump_gb300 import _capi
from jump_gb300.engine import BodyState, Descriptors, _ContextBase

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "mpm_oracle.cpp")
LIB = os.path.join(HERE, "_build", "libmpm_oracle.so")
DUAL_SRC = os.path.join(HERE, "mpm_dual.cpp")
DUAL_LIB = os.path.join(HERE, "_build", "libmpm_dual.so")

_lib = None
_dual = None


def _compile(src: str, out: str, force: bool, openmp: bool) -> str:
    hdr = os.path.join(HERE, "..", "include", "jump_mpm.h")
    if (not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src)
            and os.path.getmtime(out) >= os.path.getmtime(hdr)):
        return out
    base = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", src, "-o", out]
    r = subprocess.run(base[:6] + ["-fopenmp"] + base[6:], capture_output=True, text=True) if openmp else None
    if r is None or r.returncode != 0:
        r = subprocess.run(base, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed ({os.path.basename(src)}):\n" + r.stderr)
    return out


def build(force: bool = False) -> str:
    """g++ -O3 -ffp-contract=off (no FMA contraction), OpenMP when available; both the
    oracle and its dual-number (forward-mode gradient) restatement."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    _compile(DUAL_SRC, DUAL_LIB, force, openmp=False)
    return _compile(SRC, LIB, force, openmp=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        vp = C.c_void_p
        L.oracle_create.argtypes = [C.POINTER(_capi.GridDesc), C.POINTER(_capi.BodyDesc), C.c_int32,
                                    C.POINTER(_capi.Params), C.POINTER(vp)]
        L.oracle_step.argtypes = [vp, C.c_int64, C.POINTER(C.c_double)]
        L.oracle_download.argtypes = [vp, C.c_int32, C.POINTER(_capi.BodyView)]
        L.oracle_download_grid.argtypes = [vp] + [C.POINTER(C.c_double)] * 4
        L.oracle_energies.argtypes = [vp] + [C.POINTER(C.c_double)] * 3
        L.oracle_destroy.argtypes = [vp]
        L.oracle_set_threads.argtypes = [vp, C.c_int32]
        L.oracle_last_error.restype = C.c_char_p
        L.oracle_max_threads.restype = C.c_int
        L.oracle_shape.argtypes = [C.POINTER(_capi.GridDesc), C.c_int32, C.POINTER(C.c_double),
                                   C.POINTER(C.c_int64), C.POINTER(C.c_double), C.POINTER(C.c_double)]
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise _capi.MPMError(rc, lib().oracle_last_error().decode())


class OracleContext(_ContextBase):
    """Same driver surface as jump_gb300.engine.MPMContext, on the CPU restatement."""

    def __init__(self, desc: Descriptors, threads: int = 1):
        super().__init__(desc)
        self.L = lib()
        h = C.c_void_p()
        _check(self.L.oracle_create(C.byref(desc.grid), desc.bodies, desc.nbodies,
                                    C.byref(desc.params), C.byref(h)))
        self.h = h
        self.L.oracle_set_threads(self.h, int(threads))

    def step(self, nsteps: int, t: float | None = None, check: bool = True):
        tt = C.c_double(0.0 if t is None else t)
        rc = self.L.oracle_step(self.h, int(nsteps), C.byref(tt))
        if check:
            _check(rc)
        return tt.value if t is not None else rc

    def _download(self, s, view):
        _check(self.L.oracle_download(self.h, int(s), C.byref(view)))

    def download_grid(self, nn: int):
        d = self.dim
        m, p0, p, f = np.zeros(nn), np.zeros((nn, d)), np.zeros((nn, d)), np.zeros((nn, d))
        _check(self.L.oracle_download_grid(self.h, _capi.dptr(m), _capi.dptr(p0), _capi.dptr(p),
                                           _capi.dptr(f)))
        return m, p0, p, f

    def energies(self):
        ke, se = C.c_double(), C.c_double()
        mom = np.zeros(3)
        _check(self.L.oracle_energies(self.h, C.byref(ke), C.byref(se), _capi.dptr(mom)))
        return ke.value, se.value, mom[: self.dim]

    def close(self):
        if getattr(self, "h", None):
            self.L.oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def shape(grid_desc, basis: int, x):
    """(node ids, N, dN (support x dim)) of point x: the oracle's shape functions
    (Basis.jl getShapeAndGradient) for known-answer tests; None outside the grid."""
    d = int(grid_desc.dim)
    xp = np.ascontiguousarray(x, dtype=np.float64)
    near = np.zeros(64, dtype=np.int64)
    N = np.zeros(64)
    dN = np.zeros(64 * d)
    n = lib().oracle_shape(C.byref(grid_desc), int(basis), _capi.dptr(xp), near.ctypes.data_as(C.POINTER(C.c_int64)),
                           _capi.dptr(N), _capi.dptr(dN))
    if n <= 0:
        return None
    return near[:n].copy(), N[:n].copy(), dN[: n * d].reshape(n, d).copy()


def dual_lib():
    global _dual
    if _dual is None:
        if not os.path.exists(DUAL_LIB):
            build()
        L = C.CDLL(DUAL_LIB)
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int64)
        L.dual_grad.argtypes = [C.POINTER(_capi.GridDesc), C.POINTER(_capi.BodyDesc), C.c_int32,
                                C.POINTER(_capi.Params), C.c_int64, C.c_int32, ip, C.c_int32, dp, dp]
        L.dual_run.argtypes = [C.POINTER(_capi.GridDesc), C.POINTER(_capi.BodyDesc), C.c_int32,
                               C.POINTER(_capi.Params), C.c_int64, dp, dp]
        _dual = L
    return _dual


def dual_gradient(desc: Descriptors, nsteps: int, kind: str, ids, xbar) -> np.ndarray:
    """d(xbar . x_final)/d(parameter) by forward-mode dual numbers through the
    templated restatement (oracle/mpm_dual.cpp): kind "E" (ids: particles, their
    Young's modulus) or "v0" (ids: particle * dim + component of the initial
    velocity).  USL, linear basis, one velocity field; elastic, neo-Hookean, J2."""
    ids = np.ascontiguousarray(ids, dtype=np.int64)
    xb = np.ascontiguousarray(xbar, dtype=np.float64).ravel()
    out = np.zeros(len(ids))
    rc = dual_lib().dual_grad(C.byref(desc.grid), desc.bodies, desc.nbodies, C.byref(desc.params), int(nsteps),
                              {"E": 0, "v0": 1}[kind], ids.ctypes.data_as(C.POINTER(C.c_int64)), len(ids),
                              _capi.dptr(xb), _capi.dptr(out))
    if rc != 0:
        raise _capi.MPMError(rc, "dual_grad failed")
    return out


def dual_values(desc: Descriptors, nsteps: int):
    """(positions, stresses) of the templated restatement run with plain doubles."""
    n = sum(desc.bodies[s].count for s in range(desc.nbodies))
    d = desc.dim
    pos, sig = np.zeros(n * d), np.zeros(n * d * d)
    rc = dual_lib().dual_run(C.byref(desc.grid), desc.bodies, desc.nbodies, C.byref(desc.params), int(nsteps),
                             _capi.dptr(pos), _capi.dptr(sig))
    if rc != 0:
        raise _capi.MPMError(rc, "dual_run failed")
    return pos.reshape(n, d), sig


def max_threads() -> int:
    return int(lib().oracle_max_threads())


__all__ = ["OracleContext", "BodyState", "build", "lib", "max_threads", "shape", "dual_gradient", "dual_values"]
