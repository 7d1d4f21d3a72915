"""Host-side mirror of the reference's production-stage interface.

``GpuMechanism`` holds a mechanism compiled into device tables
(``ember_mech_create``). ``integrate_production_terms`` is
``FlameSolver::integrateProductionTerms`` (src/flameSolver.cpp:754-836) for
a batch of grid points: every point's SourceSystem (QSS or the CVODE-path
BDF) integrated over its own interval in one call. ``gas_eval`` exposes the
CanteraGas rate/thermo calls the source systems make.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .mechanism import Mechanism

QSS, BDF = 0, 1
KINETICS_STANDARD, KINETICS_INTERP = 0, 1
STATE_NORMALIZED, STATE_NO_NORM = 0, 1
STATS_WIDTH = 4

SRC_OK, SRC_DTMIN, SRC_TOO_MUCH_WORK, SRC_ERR_FAILURE, SRC_CONV_FAILURE = 0, -1, -11, -13, -14
SRC_STEP_LIMIT, SRC_NONFINITE = -20, -21


class SourceOptions(C.Structure):
    """ember_source_options; defaults are the reference's (python/ember/input.py)."""
    _fields_ = [
        ("pressure", C.c_double), ("kinetics_model", C.c_int), ("max_steps", C.c_int),
        ("qss_epsmin", C.c_double), ("qss_epsmax", C.c_double), ("qss_dtmin", C.c_double),
        ("qss_dtmax", C.c_double), ("qss_abstol", C.c_double), ("qss_minval", C.c_double),
        ("qss_iteration_count", C.c_int), ("qss_stability_check", C.c_int),
        ("bdf_reltol", C.c_double), ("bdf_abstol_momentum", C.c_double), ("bdf_abstol_energy", C.c_double),
        ("bdf_abstol_species", C.c_double), ("bdf_min_step", C.c_double), ("bdf_max_num_steps", C.c_int),
        ("threads_per_point", C.c_int),
        ("ignition_tstart", C.c_double), ("ignition_duration", C.c_double), ("ignition_energy", C.c_double),
        ("ignition_center", C.c_double), ("ignition_stddev", C.c_double),
        ("qss_tail_steps", C.c_int), ("qss_tail_threads", C.c_int), ("bdf_layout", C.c_int),
    ]

    @classmethod
    def defaults(cls, **kw):
        o = cls()
        o.pressure = 101325.0
        o.kinetics_model = KINETICS_INTERP
        o.max_steps = 1_000_000
        o.qss_epsmin, o.qss_epsmax, o.qss_dtmin, o.qss_dtmax = 2e-2, 10.0, 1e-16, 1e-6
        o.qss_abstol, o.qss_minval = 1e-11, 1e-60
        o.qss_iteration_count, o.qss_stability_check = 1, 0
        o.bdf_reltol, o.bdf_abstol_momentum, o.bdf_abstol_energy = 1e-6, 1e-7, 1e-8
        o.bdf_abstol_species, o.bdf_min_step, o.bdf_max_num_steps = 1e-13, 1e-18, 1_000_000
        o.ignition_tstart, o.ignition_duration, o.ignition_energy = 0.0, 1e-3, 0.0
        o.ignition_center, o.ignition_stddev = 0.0, 1e-4
        o.threads_per_point = 0  # the mechanism's autotuned width, else the default for its size
        o.qss_tail_steps, o.qss_tail_threads = 0, 0  # the mechanism's autotuned schedule, else one pass
        o.bdf_layout = 0  # the mechanism's autotuned matrix placement, else the first that fits
        for k, v in kw.items():
            if not hasattr(o, k):
                raise AttributeError(k)
            setattr(o, k, v)
        return o


class GpuMechanism:
    """A mechanism uploaded to the GPU (ember_mech handle)."""

    def __init__(self, mech: Mechanism):
        self.mech = mech
        desc = mech.desc()
        h = C.c_void_p()
        L.check(L.lib().ember_mech_create(C.byref(desc), C.byref(h)), "ember_mech_create")
        self._h = h

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            L.lib().ember_mech_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_multipliers(self, mult=None):
        """Per-reaction rate multipliers (numpy, or a torch CUDA tensor used in
        place); None resets them to 1."""
        if mult is not None and L.mem_of(mult) == L.MEM_DEVICE:
            m, mem = mult.contiguous(), L.MEM_DEVICE
        else:
            m = np.ascontiguousarray(mult, dtype=np.float64) if mult is not None else None
            mem = L.MEM_HOST
        L.check(L.lib().ember_mech_set_multipliers(self._h, L.ptr(m), mem, None), "set_multipliers")

    def gas_eval(self, T, Y, pressure=101325.0, model=KINETICS_STANDARD, mode=STATE_NORMALIZED):
        S = self.mech.n_species
        T = np.ascontiguousarray(np.atleast_1d(T), dtype=np.float64)
        Y = np.ascontiguousarray(Y, dtype=np.float64).reshape(T.size, S)
        n = T.size
        out = {k: np.empty((n, S)) for k in ("creation", "destruction", "net", "hk")}
        cp, rho = np.empty(n), np.empty(n)
        L.check(L.lib().ember_gas_eval(self._h, n, float(pressure), model, mode, L.ptr(T), L.ptr(Y),
                                       L.ptr(out["creation"]), L.ptr(out["destruction"]), L.ptr(out["net"]),
                                       L.ptr(out["hk"]), L.ptr(cp), L.ptr(rho), L.MEM_HOST, None), "ember_gas_eval")
        out["cp_mass"] = cp
        out["density"] = rho
        return out


THREAD_CHOICES = (32, 64, 96, 128, 160, 192, 256)


def autotune(gmech: GpuMechanism, method: int, state, dt, opts: SourceOptions | None = None, split_const=None,
             t_start: float = 0.0, x=None, stream=None):
    """``ember_source_autotune``: time the QSS kernel at every width of
    THREAD_CHOICES on these points, keep the fastest in the mechanism handle
    (used by later calls whose threads_per_point is 0) and return
    (width, {width: ms}). Host (numpy) arrays or torch CUDA tensors."""
    opts = opts or SourceOptions.defaults()
    mem = L.mem_of(state)
    n = int(state.shape[0])
    if mem == L.MEM_HOST:
        state = np.ascontiguousarray(state, dtype=np.float64)
        dt = np.ascontiguousarray(np.broadcast_to(np.asarray(dt, dtype=np.float64), (n,)))
        split_const = np.ascontiguousarray(split_const, dtype=np.float64) if split_const is not None else None
        x = np.ascontiguousarray(x, dtype=np.float64) if x is not None else None
    width = C.c_int(0)
    ms = (C.c_double * len(THREAD_CHOICES))()
    L.check(L.lib().ember_source_autotune(gmech.handle, method, n, L.ptr(state), L.ptr(split_const), L.ptr(dt),
                                          float(t_start), L.ptr(x), C.byref(opts), C.byref(width), ms, mem,
                                          L.stream_ptr(stream)), "ember_source_autotune")
    return width.value, {c: ms[i] for i, c in enumerate(THREAD_CHOICES) if ms[i] > 0}


def tuning(gmech: GpuMechanism) -> dict:
    """The launch configuration ember_source_autotune stored in the mechanism."""
    v = [C.c_int() for _ in range(6)]
    L.check(L.lib().ember_mech_get_tuning(gmech.handle, *(C.byref(x) for x in v)), "ember_mech_get_tuning")
    keys = ("qss_threads", "qss_tail_steps", "qss_tail_threads", "qss_chunk", "bdf_threads", "bdf_layout")
    return {k: x.value for k, x in zip(keys, v)}


def integrate_production_terms(gmech: GpuMechanism, method: int, state, dt, opts: SourceOptions | None = None,
                               split_const=None, t_start: float = 0.0, x=None, stream=None, out=None,
                               status=None, stats=None):
    """Source-term stage for a batch of points.

    state: [n, S+2] (U, T, Y...) as a numpy array (host) or a contiguous torch
    CUDA tensor (device, no copies). Returns (state_out, status, stats).
    """
    opts = opts or SourceOptions.defaults()
    mem = L.mem_of(state)
    n = int(state.shape[0])
    if mem == L.MEM_HOST:
        state = np.ascontiguousarray(state, dtype=np.float64)
        dt = np.ascontiguousarray(np.broadcast_to(np.asarray(dt, dtype=np.float64), (n,)))
        split_const = np.ascontiguousarray(split_const, dtype=np.float64) if split_const is not None else None
        x = np.ascontiguousarray(x, dtype=np.float64) if x is not None else None
        out = np.empty_like(state) if out is None else out
        status = np.zeros(n, dtype=np.int32) if status is None else status
        stats = np.zeros((n, STATS_WIDTH), dtype=np.int32) if stats is None else stats
    else:
        import torch
        out = torch.empty_like(state) if out is None else out
        status = torch.zeros(n, dtype=torch.int32, device=state.device) if status is None else status
        stats = torch.zeros((n, STATS_WIDTH), dtype=torch.int32, device=state.device) if stats is None else stats
    rc = L.lib().ember_source_integrate(gmech.handle, method, n, L.ptr(state), L.ptr(split_const), L.ptr(dt),
                                        float(t_start), L.ptr(x), C.byref(opts), L.ptr(out), L.ptr(status),
                                        L.ptr(stats), mem, L.stream_ptr(stream))
    if rc not in (L.OK, L.EFAIL):
        L.check(rc, "ember_source_integrate")
    return out, status, stats


def source_adjoint(gmech: GpuMechanism, state, dt, opts: SourceOptions, state_bar, split_const=None, t_start=0.0,
                   x=None, tape_cap: int = 0, method: int = BDF):
    """Discrete adjoint of a source-term integration (``ember_source_adjoint``
    for BDF, ``ember_source_adjoint_qss`` for QSS): for phi = sum(state_bar *
    state_out), returns (state_out, status, d phi / d state, d phi / d
    ln(multiplier) per reaction). Host (numpy) arrays."""
    state = np.ascontiguousarray(state, dtype=np.float64)
    n = state.shape[0]
    dt = np.ascontiguousarray(np.broadcast_to(np.asarray(dt, dtype=np.float64), (n,)))
    bar = np.ascontiguousarray(state_bar, dtype=np.float64).reshape(state.shape)
    sc = np.ascontiguousarray(split_const, dtype=np.float64) if split_const is not None else None
    xx = np.ascontiguousarray(x, dtype=np.float64) if x is not None else None
    out = np.empty_like(state)
    status = np.zeros(n, dtype=np.int32)
    gin = np.empty_like(state)
    glnk = np.zeros(max(gmech.mech.n_reactions, 1))
    name = "ember_source_adjoint_qss" if method == QSS else "ember_source_adjoint"
    rc = getattr(L.lib(), name)(gmech.handle, n, L.ptr(state), L.ptr(sc), L.ptr(dt), float(t_start), L.ptr(xx),
                                C.byref(opts), L.ptr(bar), int(tape_cap), L.ptr(out), L.ptr(status),
                                L.ptr(gin), L.ptr(glnk), L.MEM_HOST, None)
    if rc not in (L.OK, L.EFAIL):
        L.check(rc, name)
    return out, status, gin, glnk[:gmech.mech.n_reactions]
