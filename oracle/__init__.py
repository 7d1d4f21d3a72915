"""CPU ORACLE -- test infrastructure only.

ctypes binding of the plain-C restatement in this folder (liboracle.so). Only
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import it,
and only to compare the GPU results with; the product package never does.
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
    l.oracle_diffusion_batch.argtypes = [i, i, vp, vp, vp, vp, vp, vp, vp, vp, vp, d, d, d, d, vp, i]
    l.oracle_diffusion_batch.restype = None
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


def diffusion_batch(grids, B, D, S, Y, t0, t1, h=None, mult=10.0, gdt=2e-5, n_threads=None):
    """Every (flame, variable) system of a diffusion stage, threaded over
    systems (flat arrays in the layout of ember_diffusion_integrate)."""
    import os as _os
    nf = len(grids)
    npts = np.array([g.n_points for g in grids], dtype=np.int32)
    n_vars = np.asarray(Y).size // int(npts.sum())
    ci = lambda v: np.ascontiguousarray(v, dtype=np.int32)
    lb, rb, al = ci([g.left_bc for g in grids]), ci([g.right_bc for g in grids]), ci([g.alpha for g in grids])
    x = _f(np.concatenate([np.asarray(g.x, dtype=np.float64) for g in grids]))
    B, D = _f(B), _f(D)
    S = _f(S) if S is not None else None
    hh = _f(h) if h is not None else None
    y = _f(Y).copy()
    lib().oracle_diffusion_batch(nf, n_vars, npts.ctypes.data, lb.ctypes.data, rb.ctypes.data, al.ctypes.data,
                                 x.ctypes.data, B.ctypes.data, D.ctypes.data, S.ctypes.data if S is not None else None,
                                 hh.ctypes.data if hh is not None else None, mult, gdt, t0, t1, y.ctypes.data,
                                 int(n_threads or _os.cpu_count() or 1))
    return y
