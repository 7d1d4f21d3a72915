"""CPU ORACLE -- test infrastructure only.

ctypes binding of the chemistry restatement (oracle_chem.c, oracle_bdf.c):
thermo/kinetics evaluation, the QSS integrator and the BDF integrator of the
source term, and a threaded batch driver used as the CPU baseline.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

KINETICS_STANDARD, KINETICS_INTERP = 0, 1
STATE_NORMALIZED, STATE_NO_NORM = 0, 1
QSS, BDF = 0, 1


def declare(l):
    vp, d, i = C.c_void_p, C.c_double, C.c_int
    l.oracle_mech_create.argtypes = [vp]
    l.oracle_mech_create.restype = vp
    l.oracle_mech_destroy.argtypes = [vp]
    l.oracle_mech_destroy.restype = None
    l.oracle_mech_set_multipliers.argtypes = [vp, vp]
    l.oracle_mech_set_multipliers.restype = None
    l.oracle_gas_eval.argtypes = [vp, d, i, i, i, vp, vp, vp, vp, vp, vp, vp, vp]
    l.oracle_gas_eval.restype = None
    l.oracle_source_batch.argtypes = [vp, i, i, vp, vp, vp, d, vp, vp, vp, vp, vp, i]
    l.oracle_source_batch.restype = None
    l.oracle_qss_adjoint_batch.argtypes = [vp, i, vp, vp, vp, d, vp, vp, vp, vp, vp, vp, vp, vp, i]
    l.oracle_qss_adjoint_batch.restype = None
    l.oracle_exp.argtypes = [d]
    l.oracle_exp.restype = d
    l.oracle_log.argtypes = [d]
    l.oracle_log.restype = d


def _lib():
    import oracle
    return oracle.lib()


def _p(a):
    return a.ctypes.data if a is not None else None


class OracleMech:
    """The oracle's copy of a mechanism (built from ember_gb300.mechanism.Mechanism)."""

    def __init__(self, mech):
        self.mech = mech
        desc = mech.desc()
        self._h = _lib().oracle_mech_create(C.addressof(desc))
        self.S = mech.n_species
        self.R = mech.n_reactions

    def __del__(self):
        try:
            if self._h:
                _lib().oracle_mech_destroy(self._h)
        except Exception:
            pass

    def set_multipliers(self, mult=None):
        m = np.ascontiguousarray(mult, dtype=np.float64) if mult is not None else None
        _lib().oracle_mech_set_multipliers(self._h, _p(m))

    def gas_eval(self, T, Y, pressure=101325.0, model=KINETICS_STANDARD, mode=STATE_NORMALIZED):
        T = np.ascontiguousarray(np.atleast_1d(T), dtype=np.float64)
        Y = np.ascontiguousarray(Y, dtype=np.float64).reshape(T.size, self.S)
        n = T.size
        out = {k: np.empty((n, self.S)) for k in ("creation", "destruction", "net", "hk")}
        cp = np.empty(n)
        rho = np.empty(n)
        _lib().oracle_gas_eval(self._h, pressure, model, mode, n, _p(T), _p(Y), _p(out["creation"]),
                               _p(out["destruction"]), _p(out["net"]), _p(out["hk"]), _p(cp), _p(rho))
        out["cp_mass"] = cp
        out["density"] = rho
        return out

    def integrate(self, method, state, dt, opts, split_const=None, t_start=0.0, x=None, n_threads=None):
        """Batch of source-term integrations; returns (state_out, status, stats)."""
        state = np.ascontiguousarray(state, dtype=np.float64)
        n = state.shape[0]
        dt = np.ascontiguousarray(np.broadcast_to(np.asarray(dt, dtype=np.float64), (n,)))
        sc = np.ascontiguousarray(split_const, dtype=np.float64) if split_const is not None else None
        xx = np.ascontiguousarray(x, dtype=np.float64) if x is not None else None
        out = np.empty_like(state)
        status = np.zeros(n, dtype=np.int32)
        stats = np.zeros((n, 4), dtype=np.int32)
        nt = n_threads or os.cpu_count() or 1
        _lib().oracle_source_batch(self._h, method, n, _p(state), _p(sc), _p(dt), float(t_start), _p(xx),
                                   C.addressof(opts), _p(out), _p(status), _p(stats), int(nt))
        return out, status, stats


def qss_adjoint(om: OracleMech, state, dt, opts, state_bar, split_const=None, t_start=0.0, x=None, n_threads=None):
    """Discrete adjoint of the QSS integration of a batch of points
    (oracle_qss_adjoint.c): for phi = sum state_bar . state_out, returns
    (state_out, d phi / d state_in, d phi / d ln(multiplier) per point
    [n, R], status, steps)."""
    state = np.ascontiguousarray(state, dtype=np.float64)
    n = state.shape[0]
    dt = np.ascontiguousarray(np.broadcast_to(np.asarray(dt, dtype=np.float64), (n,)))
    sc = np.ascontiguousarray(split_const, dtype=np.float64) if split_const is not None else None
    xx = np.ascontiguousarray(x, dtype=np.float64) if x is not None else None
    bar = np.ascontiguousarray(np.broadcast_to(state_bar, state.shape), dtype=np.float64)
    out = np.empty_like(state)
    ybar = np.zeros_like(state)
    pbar = np.zeros((n, om.R))
    status = np.zeros(n, dtype=np.int32)
    steps = np.zeros(n, dtype=np.int32)
    nt = n_threads or os.cpu_count() or 1
    _lib().oracle_qss_adjoint_batch(om._h, n, _p(state), _p(sc), _p(dt), float(t_start), _p(xx), C.addressof(opts),
                                    _p(bar), _p(out), _p(ybar), _p(pbar), _p(status), _p(steps), int(nt))
    return out, ybar, pbar, status, steps


def exp(x):
    return _lib().oracle_exp(float(x))


def log(x):
    return _lib().oracle_log(float(x))


class QssParams(C.Structure):
    _fields_ = [("epsmin", C.c_double), ("epsmax", C.c_double), ("dtmin", C.c_double), ("dtmax", C.c_double),
                ("abstol", C.c_double), ("itermax", C.c_int), ("stability_check", C.c_int)]


def qss_cesium(y0, tf, epsmin, itermax=5, epsmax=20.0, dtmin=1e-15, dtmax=1e300, abstol=1e-8,
               stability_check=1, max_steps=10_000_000):
    """The cesium KAT problem through the oracle's QSS integrator."""
    l = _lib()
    l.oracle_qss_cesium.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_int, C.c_void_p]
    l.oracle_qss_cesium.restype = C.c_int
    P = QssParams(epsmin, epsmax, dtmin, dtmax, abstol, itermax, stability_check)
    y = np.ascontiguousarray(y0, dtype=np.float64).copy()
    stats = np.zeros(4, dtype=np.int32)
    r = l.oracle_qss_cesium(C.addressof(P), y.ctypes.data, float(tf), int(max_steps), stats.ctypes.data)
    return y, r, stats


def transport_eval(om: OracleMech, data, T, Y, pressure=101325.0, threshold=1e-5, n_threads=1):
    """The oracle's thermo and mixture-averaged transport properties
    (oracle_transport.c) of the states T [n], Y [n, S], with the fits of a
    ember_gb300.transport.TransportData; n_threads > 1 splits the points."""
    l = _lib()
    if not getattr(l, "_transport_declared", False):
        vp = C.c_void_p
        l.oracle_transport_eval_threads.argtypes = ([vp, vp, vp, vp, C.c_int, C.c_double, C.c_double, vp, vp]
                                                    + [vp] * 8 + [C.c_int])
        l.oracle_transport_eval_threads.restype = None
        l._transport_declared = True
    T = np.ascontiguousarray(np.atleast_1d(T), dtype=np.float64)
    n, S = T.size, om.S
    Y = np.ascontiguousarray(Y, dtype=np.float64).reshape(n, S)
    fits = [np.ascontiguousarray(a, dtype=np.float64) for a in (data.visc_fit, data.cond_fit, data.diff_fit)]
    out = {"density": np.empty(n), "mean_mol_weight": np.empty(n), "cp_mass": np.empty(n),
           "cp_species": np.empty((n, S)), "h_species": np.empty((n, S)), "conductivity": np.empty(n),
           "viscosity": np.empty(n), "rho_d": np.empty((n, S))}
    l.oracle_transport_eval_threads(om._h, *(_p(f) for f in fits), n, float(pressure), float(threshold), _p(T),
                                    _p(Y), *(_p(out[k]) for k in ("density", "mean_mol_weight", "cp_mass",
                                                                  "cp_species", "h_species", "conductivity",
                                                                  "viscosity", "rho_d")), int(n_threads))
    return out
