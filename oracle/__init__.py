"""CPU ORACLE -- test infrastructure only.

ctypes binding of the plain-C restatement in this folder (liboracle.so). Only
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import it,
and only as the checker; the product package never does.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None
dp = C.POINTER(C.c_double)


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = C.CDLL(path)
        _declare(_lib)
    return _lib


def _declare(l):
    vp, d, i = C.c_void_p, C.c_double, C.c_int
    l.oracle_tridiag_run.argtypes = [i, vp, vp, vp, vp, vp, d, d, d, i, vp, vp]
    l.oracle_tridiag_run.restype = None
    l.oracle_diffusion_matrix.argtypes = [i, vp, i, i, i, vp, vp, vp, d, d, vp, vp, vp, vp]
    l.oracle_diffusion_matrix.restype = None
    l.oracle_diffusion_step_size.argtypes = [i, vp, vp, vp, d, d]
    l.oracle_diffusion_step_size.restype = d
    l.oracle_diffusion_system.argtypes = [i, vp, i, i, i, vp, vp, vp, d, d, d, d, d, d, d, vp]
    l.oracle_diffusion_system.restype = None
    from . import chem as _chem
    _chem.declare(l)


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def tridiag_run(a, b, c, k, y0, t0, h, t_end=None, n_steps=0):
    """One TridiagonalIntegrator: initialize(t0, h) then n_steps step() calls
    (n_steps > 0) or integrateToTime(t_end). Returns (y, t, h)."""
    a, b, c, k = _f(a), _f(b), _f(c), _f(k)
    y = _f(y0).copy()
    t_out, h_out = C.c_double(), C.c_double()
    lib().oracle_tridiag_run(len(y), a.ctypes.data, b.ctypes.data, c.ctypes.data, k.ctypes.data, y.ctypes.data,
                             float(t0), float(h), float(t_end if t_end is not None else 0.0), int(n_steps),
                             C.addressof(t_out), C.addressof(h_out))
    return y, t_out.value, h_out.value


def diffusion_matrix(x, B, D, split_const=None, alpha=0, left_bc=0, right_bc=0, wall_const=0.0, y_inf=0.0):
    x, B, D = _f(x), _f(B), _f(D)
    N = len(x)
    s = _f(split_const) if split_const is not None else None
    a, b, c, k = (np.empty(N) for _ in range(4))
    lib().oracle_diffusion_matrix(N, x.ctypes.data, alpha, left_bc, right_bc, B.ctypes.data, D.ctypes.data,
                                  s.ctypes.data if s is not None else None, wall_const, y_inf, a.ctypes.data,
                                  b.ctypes.data, c.ctypes.data, k.ctypes.data)
    return a, b, c, k


def diffusion_step_size(x, B, D, mult, gdt):
    x, B, D = _f(x), _f(B), _f(D)
    return lib().oracle_diffusion_step_size(len(x), x.ctypes.data, B.ctypes.data, D.ctypes.data, mult, gdt)


def diffusion_system(x, B, D, y, t0, t1, split_const=None, alpha=0, left_bc=0, right_bc=0, wall_const=0.0,
                     y_inf=0.0, h=0.0, mult=10.0, gdt=2e-5):
    """One DiffusionSystem + TridiagonalIntegrator through one stage."""
    x, B, D = _f(x), _f(B), _f(D)
    y = _f(y).copy()
    s = _f(split_const) if split_const is not None else None
    lib().oracle_diffusion_system(len(x), x.ctypes.data, alpha, left_bc, right_bc, B.ctypes.data, D.ctypes.data,
                                  s.ctypes.data if s is not None else None, wall_const, y_inf, h, mult, gdt,
                                  t0, t1, y.ctypes.data)
    return y
