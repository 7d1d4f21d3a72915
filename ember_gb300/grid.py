"""Adaptive flame grid (host code of libember_gpu, no device needed).

``AdaptiveGrid`` wraps ``ember_grid_*``: the regrid block of
FlameSolver::finishStep (src/flameSolver.cpp:279-352) with OneDimGrid's
boundary regrid and interior adaptation (src/grid.cpp). ``regrid_batch``
applies it to every flame of a split batch: the state and the three time
derivative arrays are regridded together (the state rows drive the
criteria), the damping length comes from the transport properties of the
state, and the mass fractions are renormalised afterwards
(correctMassFractions), as the reference does when the grid changed.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from .diffusion import FlameGrid


class GridOptions(C.Structure):
    """ember_grid_options; ``defaults()`` are the reference's."""
    _fields_ = [("vtol", C.c_double), ("dvtol", C.c_double), ("absvtol", C.c_double), ("rm_tol", C.c_double),
                ("uniformity_tol", C.c_double), ("grid_min", C.c_double), ("grid_max", C.c_double),
                ("damp_const", C.c_double), ("center_grid_min", C.c_double), ("boundary_tol", C.c_double),
                ("boundary_tol_rm", C.c_double), ("unstrained_downstream_width", C.c_double),
                ("add_point_count", C.c_int), ("fixed_burned_val", C.c_int), ("unburned_left", C.c_int),
                ("fixed_left_loc", C.c_int), ("twin_flame", C.c_int), ("cylindrical_flame", C.c_int),
                ("left_bc", C.c_int), ("right_bc", C.c_int)]

    @classmethod
    def defaults(cls, **kw):
        o = cls()
        L.check(_lib().ember_grid_options_default(C.byref(o)), "ember_grid_options_default")
        for k, v in kw.items():
            if not hasattr(o, k):
                raise AttributeError(k)
            setattr(o, k, v)
        return o


_declared = False


def _lib():
    global _declared
    lib = L.lib()
    if not _declared:
        vp, d, i = C.c_void_p, C.c_double, C.c_int
        for name, res, args in (
                ("ember_grid_options_default", i, [vp]),
                ("ember_grid_create", i, [vp, i, vp, C.POINTER(vp)]),
                ("ember_grid_destroy", i, [vp]),
                ("ember_grid_regrid", i, [vp, i, i, vp, vp, vp, d, i, C.POINTER(i), C.POINTER(i)]),
                ("ember_grid_get", i, [vp, vp, vp, C.POINTER(i), C.POINTER(i)]),
                ("ember_grid_damping", i, [i, i, vp, vp, vp, vp, vp, d, vp])):
            fn = getattr(lib, name)
            fn.restype, fn.argtypes = res, args
        _declared = True
    return lib


class AdaptiveGrid:
    """One flame's adaptive grid (``ember_grid`` handle)."""

    def __init__(self, x, options: GridOptions | None = None):
        self.options = options or GridOptions.defaults()
        x = np.ascontiguousarray(x, dtype=np.float64)
        h = C.c_void_p()
        L.check(_lib().ember_grid_create(C.byref(self.options), x.size, x.ctypes.data, C.byref(h)),
                "ember_grid_create")
        self._h = h
        self.x = x.copy()
        self.n_rows = 0

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib().ember_grid_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def regrid(self, rows, n_adapt: int, damp_val, qdot=None, strain_rate: float = 1.0, boundaries: bool = True):
        """Regrid with ``rows`` [n_rows, N] (the first ``n_adapt`` drive the
        criteria). Returns (x, rows, updated) on the new grid."""
        rows = np.ascontiguousarray(rows, dtype=np.float64)
        n_rows, N = rows.shape
        if N != self.x.size:
            raise ValueError(f"rows have {N} points, the grid {self.x.size}")
        damp = np.ascontiguousarray(damp_val, dtype=np.float64)
        q = np.ascontiguousarray(qdot, dtype=np.float64) if qdot is not None else None
        n_out, upd = C.c_int(), C.c_int()
        L.check(_lib().ember_grid_regrid(self._h, n_rows, int(n_adapt), rows.ctypes.data, damp.ctypes.data, L.ptr(q),
                                         float(strain_rate), int(bool(boundaries)), C.byref(n_out), C.byref(upd)),
                "ember_grid_regrid")
        x = np.empty(n_out.value)
        out = np.empty((n_rows, n_out.value))
        ju, jb = C.c_int(), C.c_int()
        L.check(_lib().ember_grid_get(self._h, x.ctypes.data, out.ctypes.data, C.byref(ju), C.byref(jb)),
                "ember_grid_get")
        self.x = x
        self.ju, self.jb = ju.value, jb.value
        return x, out, bool(upd.value)


def damping(props: dict, n_species: int, strain_rate: float):
    """ember_grid_damping from transport properties (GpuTransport.eval keys)."""
    mu = np.ascontiguousarray(props["viscosity"], dtype=np.float64)
    n = mu.size
    out = np.empty(n)
    arrs = [np.ascontiguousarray(props[k], dtype=np.float64) for k in ("conductivity", "cp_mass", "rho_d", "density")]
    L.check(_lib().ember_grid_damping(n, int(n_species), mu.ctypes.data, arrs[0].ctypes.data, arrs[1].ctypes.data,
                                      arrs[2].ctypes.data, arrs[3].ctypes.data, float(strain_rate), out.ctypes.data),
            "ember_grid_damping")
    return out


@dataclass
class RegridResult:
    grids: list
    state: np.ndarray          # point-major [n_points, S+2]
    ddt: tuple                 # (ddt_conv, ddt_diff, ddt_prod), point-major
    updated: list              # per flame


def regrid_batch(grids, state, ddt, props, strain_rates, options: GridOptions | None = None, qdot=None):
    """Regrid every flame of a batch as FlameSolver::finishStep does.

    grids: FlameGrid per flame; state: point-major [n_points, S+2]; ddt:
    (ddt_conv, ddt_diff, ddt_prod) point-major (None entries count as zero);
    props: transport properties of ``state`` (GpuTransport.eval output);
    strain_rates: per flame (0: unstrained, then ``qdot`` per point is
    needed). Returns a RegridResult with the new grids, the state (mass
    fractions renormalised where a flame's grid changed) and the derivatives
    on the new grids."""
    state = np.asarray(state, dtype=np.float64)
    n = state.shape[1]
    S = n - 2
    ddt = tuple(np.zeros_like(state) if d is None else np.asarray(d, dtype=np.float64) for d in ddt)
    offs = np.cumsum([0] + [g.n_points for g in grids])
    new_grids, states, derivs, updated = [], [], ([], [], []), []
    for f, g in enumerate(grids):
        a, b = offs[f], offs[f + 1]
        base = options or GridOptions.defaults()
        opts = GridOptions.from_buffer_copy(base)
        opts.left_bc, opts.right_bc = g.left_bc, g.right_bc
        opts.cylindrical_flame = int(g.alpha == 1)
        sub = {k: np.asarray(v)[a:b] for k, v in props.items()}
        damp = damping(sub, S, float(strain_rates[f]))
        rows = np.concatenate([state[a:b].T] + [d[a:b].T for d in ddt])
        grid = AdaptiveGrid(g.x, opts)
        x, out, upd = grid.regrid(rows, n, damp, qdot=None if qdot is None else np.asarray(qdot)[a:b],
                                  strain_rate=float(strain_rates[f]))
        st = out[:n].T.copy()
        if upd:
            y = np.where(st[:, 2:] < 0.0, 0.0, st[:, 2:])
            st[:, 2:] = y * (1.0 / np.cumsum(y, axis=1)[:, -1])[:, None]
        new_grids.append(FlameGrid(x=x, left_bc=g.left_bc, right_bc=g.right_bc, alpha=g.alpha))
        states.append(st)
        for i in range(3):
            derivs[i].append(out[n * (i + 1):n * (i + 2)].T.copy())
        updated.append(upd)
    return RegridResult(new_grids, np.concatenate(states),
                        tuple(np.concatenate(d) for d in derivs), updated)
