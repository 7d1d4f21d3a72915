"""CPU ORACLE -- test infrastructure only.

ctypes binding of the convection-stage restatement (oracle_convection.c): the
UTW right-hand side, the Adams coefficients and one flame's whole stage.
"""
from __future__ import annotations

import ctypes as C

import numpy as np


class OracleConvFlame(C.Structure):
    _fields_ = [("n_points", C.c_int), ("left_bc", C.c_int), ("right_bc", C.c_int), ("alpha", C.c_int),
                ("continuity_bc", C.c_int), ("j_cont", C.c_int),
                ("beta", C.c_double), ("x_vzero", C.c_double), ("rv_zero", C.c_double), ("rv_cont", C.c_double),
                ("t_left", C.c_double), ("w_left", C.c_double), ("rhou", C.c_double), ("pressure", C.c_double),
                ("strain_initial", C.c_double), ("strain_final", C.c_double), ("strain_t0", C.c_double),
                ("strain_dt", C.c_double), ("strain_type", C.c_int), ("n_cheb", C.c_int), ("cheb_t0", C.c_double),
                ("cheb_t1", C.c_double), ("cheb", C.c_double * 16)]


class OracleConvOptions(C.Structure):
    _fields_ = [("reltol", C.c_double), ("abstol_u", C.c_double), ("abstol_t", C.c_double),
                ("abstol_y", C.c_double), ("min_step", C.c_double), ("max_steps", C.c_int),
                ("max_history", C.c_int)]


def _lib():
    import oracle
    l = oracle.lib()
    vp, d, i = C.c_void_p, C.c_double, C.c_int
    l.oracle_convection_strain.argtypes = [vp, d, vp, vp]
    l.oracle_convection_strain.restype = None
    l.oracle_adams_gammas.argtypes = [vp]
    l.oracle_adams_gammas.restype = None
    l.oracle_adams_l.argtypes = [i, vp]
    l.oracle_adams_l.restype = None
    l.oracle_convection_grid.argtypes = [i, vp, i, vp, vp]
    l.oracle_convection_grid.restype = None
    l.oracle_convection_prepare.argtypes = [i, i, vp, vp, vp, vp, vp]
    l.oracle_convection_prepare.restype = None
    l.oracle_convection_utw_rhs.argtypes = [vp, vp, vp, vp, d, vp, vp, vp, vp, vp, vp, vp, vp, vp]
    l.oracle_convection_utw_rhs.restype = None
    l.oracle_convection_interval.argtypes = [vp, i, d, vp]
    l.oracle_convection_interval.restype = i
    l.oracle_convection_flame.argtypes = [vp, i, vp, vp, vp, d, d, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]
    l.oracle_convection_flame.restype = i
    l.oracle_convection_drhodt.argtypes = [i, i, i, d, vp, vp, vp, vp, vp, vp, vp]
    l.oracle_convection_drhodt.restype = None
    return l


def density_derivative(state, W, pressure, ddt_conv, ddt_diff, ddt_prod, ddt_cross, balanced):
    """drho/dt per point of point-major arrays (prepareIntegrators)."""
    state = np.ascontiguousarray(state, dtype=np.float64)
    n_pts, n = state.shape
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (W, ddt_conv, ddt_diff, ddt_prod, ddt_cross)]
    out = np.zeros(n_pts)
    _lib().oracle_convection_drhodt(n_pts, n, int(bool(balanced)), float(pressure), _p(arrs[0]), _p(state),
                                    _p(arrs[1]), _p(arrs[2]), _p(arrs[3]), _p(arrs[4]), _p(out))
    return out


def _p(a):
    return a.ctypes.data if a is not None else None


def flame_struct(params) -> OracleConvFlame:
    """From any object with the ConvectionFlame attributes."""
    kw = {n: getattr(params, n) for n, _ in OracleConvFlame._fields_ if n != "cheb"}
    c = list(getattr(params, "cheb", ()) or ())
    kw["cheb"] = (C.c_double * 16)(*(c + [0.0] * (16 - len(c))))
    return OracleConvFlame(**kw)


def strain(params, t):
    """(a, da/dt) of a flame's strain function at t (oracle_convection_strain)."""
    a, d = C.c_double(), C.c_double()
    f = flame_struct(params)
    _lib().oracle_convection_strain(C.byref(f), float(t), C.byref(a), C.byref(d))
    return a.value, d.value


def adams_gammas():
    g = np.zeros(14)
    _lib().oracle_adams_gammas(_p(g))
    return g


def adams_l(q: int):
    l = np.zeros(14)
    _lib().oracle_adams_l(q, _p(l))
    return l


def utw_rhs(fl, x, t, y3, drhodt, sU, sT, sW):
    """ConvectionSystemUTW::f at (t, y3 = interleaved [U, T, W] per point).
    Returns (ydot3, rho, rV, V)."""
    N = fl.n_points
    f = flame_struct(fl)
    x = np.ascontiguousarray(x, dtype=np.float64)
    hh, rph = np.zeros(N), np.zeros(N)
    _lib().oracle_convection_grid(N, _p(x), fl.alpha, _p(hh), _p(rph))
    out = [np.zeros(3 * N), np.zeros(N), np.zeros(N), np.zeros(N)]
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (y3, drhodt, sU, sT, sW)]
    _lib().oracle_convection_utw_rhs(C.byref(f), _p(x), _p(hh), _p(rph), float(t), *[_p(a) for a in arrs],
                                     *[_p(a) for a in out])
    return tuple(out)


def interval(ht, t):
    s = C.c_double(0.0)
    ht = np.ascontiguousarray(ht, dtype=np.float64)
    i = _lib().oracle_convection_interval(_p(ht), len(ht), float(t), C.byref(s))
    return i, s.value


def convection_flame(fl, W, x, y_left, drhodt, split, state, t0, tf, opts, last=None):
    """One flame's stage: state (variable-major (S+2) x N) is copied and the
    result returned with (status [1+S], stats [4], history times, history
    values [H, N]). ``last``: a dict that receives V and rV of the UTW
    system's last right-hand side evaluation ("V", "rV")."""
    N = fl.n_points
    S = len(W)
    st = np.array(state, dtype=np.float64).reshape(-1).copy()
    status = np.zeros(1 + S, dtype=np.int32)
    stats = np.zeros(4, dtype=np.int32)
    H = C.c_int(0)
    ht = np.zeros(opts.max_history)
    hv = np.zeros(opts.max_history * N)
    o = OracleConvOptions(opts.reltol, opts.abstol_u, opts.abstol_t, opts.abstol_y, opts.min_step,
                          int(opts.max_steps), int(opts.max_history))
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (W, x, y_left, drhodt, split)]
    f = flame_struct(fl)
    vl, rvl = np.zeros(N), np.zeros(N)
    _lib().oracle_convection_flame(C.byref(f), S, _p(arrs[0]), _p(arrs[1]), _p(arrs[2]), float(t0), float(tf),
                                   _p(arrs[3]), _p(arrs[4]), _p(st), C.byref(o), _p(status), _p(stats), C.byref(H),
                                   _p(ht), _p(hv), _p(vl), _p(rvl))
    if last is not None:
        last["V"], last["rV"] = vl, rvl
    h = H.value
    return st, status, stats, ht[:h].copy(), hv[:h * N].reshape(h, N).copy()


def convection_batch(batch, W, t0, tf, opts):
    """Every flame of an ember_gb300.convection.ConvectionBatch-like batch;
    returns (state, status [n_flames, 1+S], stats [n_flames, 4])."""
    S = len(W)
    out = np.array(batch.state, dtype=np.float64).copy()
    status, stats = [], []
    v0 = 0
    for f, fl in enumerate(batch.flames):
        N = fl.n_points
        p0, p1 = batch.offsets[f], batch.offsets[f + 1]
        sl = slice(v0, v0 + (S + 2) * N)
        st, s, t, _, _ = convection_flame(fl, W, batch.x[p0:p1], batch.y_left[f], batch.drhodt[p0:p1],
                                          batch.split_const[sl], out[sl], t0, tf, opts)
        out[sl] = st
        status.append(s)
        stats.append(t)
        v0 += (S + 2) * N
    return out, np.array(status), np.array(stats)
