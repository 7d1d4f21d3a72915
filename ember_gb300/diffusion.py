"""Host-side mirror of the reference's diffusion-stage interface.

``TridiagonalIntegratorBatch`` mirrors ``TridiagonalIntegrator``
(src/integrator.h:106-133): set_y0 / initialize / step / integrateToTime /
get_y / get_ydot / t / h, for many independent systems at once, on the GPU.

``integrate_diffusion_terms`` is ``FlameSolver::integrateDiffusionTerms``
(src/flameSolver.cpp:838-854, with setDiffusionSolverState 702-718) for a
batch of flames: it builds every DiffusionSystem matrix on the device and
integrates all (flame, variable) systems in one call.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L


def _f64(a, n=None, name="array"):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if n is not None and a.size != n:
        raise ValueError(f"{name}: expected {n} values, got {a.size}")
    return a


class TridiagonalIntegratorBatch:
    """A batch of TridiagonalIntegrator objects whose state lives on the GPU.

    ``sizes`` gives the number of points of each system; per-point arrays are
    the concatenation of the systems (CSR layout).
    """

    def __init__(self, sizes):
        sizes = [int(n) for n in sizes]
        self.offsets = np.zeros(len(sizes) + 1, dtype=np.int64)
        self.offsets[1:] = np.cumsum(sizes)
        self.n_systems = len(sizes)
        self.n_total = int(self.offsets[-1])
        h = C.c_void_p()
        lib = L.lib()
        L.check(lib.ember_tridiag_create(self.n_systems, self.offsets.ctypes.data_as(L.i64p), C.byref(h)),
                "ember_tridiag_create")
        self._h = h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            L.lib().ember_tridiag_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_coefficients(self, a, b, c, k):
        """Constant ODE y' = A y + k (TridiagonalODE::get_A / get_k)."""
        n = self.n_total
        a, b, c, k = (_f64(v, n, nm) for v, nm in zip((a, b, c, k), "abck"))
        L.check(L.lib().ember_tridiag_set_coefficients(self._h, a.ctypes.data, b.ctypes.data, c.ctypes.data,
                                                       k.ctypes.data, L.MEM_HOST, None), "set_coefficients")

    def set_y0(self, y0):
        y0 = _f64(y0, self.n_total, "y0")
        L.check(L.lib().ember_tridiag_set_y0(self._h, y0.ctypes.data, L.MEM_HOST, None), "set_y0")

    def initialize(self, t0, h):
        t0 = _f64(np.broadcast_to(np.asarray(t0, dtype=np.float64), (self.n_systems,)))
        h = _f64(np.broadcast_to(np.asarray(h, dtype=np.float64), (self.n_systems,)))
        L.check(L.lib().ember_tridiag_initialize(self._h, t0.ctypes.data, h.ctypes.data, L.MEM_HOST, None),
                "initialize")

    def step(self):
        L.check(L.lib().ember_tridiag_step(self._h, None), "step")

    def integrate_to_time(self, t_end):
        t_end = _f64(np.broadcast_to(np.asarray(t_end, dtype=np.float64), (self.n_systems,)))
        L.check(L.lib().ember_tridiag_integrate_to_time(self._h, t_end.ctypes.data, L.MEM_HOST, None),
                "integrate_to_time")

    def state(self):
        y = np.empty(self.n_total)
        t = np.empty(self.n_systems)
        h = np.empty(self.n_systems)
        L.check(L.lib().ember_tridiag_get_state(self._h, y.ctypes.data, t.ctypes.data, h.ctypes.data,
                                                L.MEM_HOST, None), "get_state")
        return y, t, h

    @property
    def y(self):
        return self.state()[0]

    @property
    def t(self):
        return self.state()[1]

    @property
    def h(self):
        return self.state()[2]

    def get_ydot(self):
        ydot = np.empty(self.n_total)
        L.check(L.lib().ember_tridiag_get_ydot(self._h, ydot.ctypes.data, L.MEM_HOST, None), "get_ydot")
        return ydot

    def split(self, v):
        return [v[self.offsets[i]:self.offsets[i + 1]] for i in range(self.n_systems)]


@dataclass
class FlameGrid:
    """One flame's grid (OneDimGrid: x, alpha, leftBC, rightBC)."""
    x: np.ndarray
    left_bc: int = L.BC_FIXED_VALUE
    right_bc: int = L.BC_FIXED_VALUE
    alpha: int = 0

    @property
    def n_points(self) -> int:
        return int(np.asarray(self.x).size)


def integrate_diffusion_terms(grids, B, D, split_const, y, t_start, t_end, *, h=None, dt_multiplier=10.0,
                              global_timestep=2e-5, wall_const=None, y_inf=None, stream=None, x=None,
                              algorithm=L.DIFFUSION_PARALLEL):
    """One diffusion stage for a batch of flames.

    ``B``, ``D``, ``split_const`` and ``y`` are either lists with one
    (n_vars, N_f) array per flame, or flat arrays in the C ABI layout
    (variable-major per flame, flames concatenated); flat torch CUDA tensors
    are used in place on the device. Returns the integrated state in the same
    form as ``y`` (lists are returned as new arrays; flat arrays in place)
    and the per-(flame, variable) status array. ``algorithm`` selects the
    warp-parallel solver (default) or the serial one that reproduces the
    reference bit for bit. ``x`` may pass the
    concatenated grid coordinates (e.g. already on the device); per-system
    arrays (h, wall_const, y_inf) may be device tensors for device calls.
    """
    n_flames = len(grids)
    as_list = isinstance(y, (list, tuple))
    if as_list:
        n_vars = int(np.asarray(y[0]).shape[0])
        flat = lambda arrs: np.concatenate([_f64(a).reshape(-1) for a in arrs]) if arrs is not None else None
        B_, D_, S_, Y_ = flat(B), flat(D), flat(split_const), flat(y)
    else:
        total_pts = sum(g.n_points for g in grids)
        n_vars = int(y.numel() if hasattr(y, "numel") else np.asarray(y).size) // total_pts
        B_, D_, S_, Y_ = B, D, split_const, y
    mem = L.mem_of(Y_)
    if mem == L.MEM_HOST:
        B_, D_, Y_ = _f64(B_), _f64(D_), _f64(Y_)
        S_ = _f64(S_) if S_ is not None else None
        x_ = np.concatenate([_f64(g.x) for g in grids])
        status = np.zeros(n_flames * n_vars, dtype=np.int32)
        per_sys = lambda v: _f64(np.broadcast_to(np.asarray(v, dtype=np.float64), (n_flames * n_vars,))) \
            if v is not None else None
    else:
        import torch
        dev = Y_.device
        x_ = x if x is not None else torch.as_tensor(np.concatenate([_f64(g.x) for g in grids]), device=dev)
        status = torch.zeros(n_flames * n_vars, dtype=torch.int32, device=dev)
        per_sys = lambda v: v if (v is None or hasattr(v, "data_ptr")) else torch.as_tensor(
            np.broadcast_to(np.asarray(v, dtype=np.float64), (n_flames * n_vars,)).copy(), device=dev)
    h_, wc_, yi_ = per_sys(h), per_sys(wall_const), per_sys(y_inf)
    garr = (L.DiffusionGrid * n_flames)(*[L.DiffusionGrid(g.n_points, g.left_bc, g.right_bc, g.alpha)
                                          for g in grids])
    opts = L.DiffusionOptions(float(t_start), float(t_end), float(dt_multiplier), float(global_timestep),
                              L.ptr(h_), L.ptr(wc_), L.ptr(yi_), int(algorithm))
    rc = L.lib().ember_diffusion_integrate(n_flames, garr, n_vars, L.ptr(x_), L.ptr(B_), L.ptr(D_), L.ptr(S_),
                                           L.ptr(Y_), C.byref(opts), L.ptr(status), mem, L.stream_ptr(stream))
    if rc not in (L.OK, L.EFAIL):
        L.check(rc, "ember_diffusion_integrate")
    if as_list:
        out, o = [], 0
        for g in grids:
            n = n_vars * g.n_points
            out.append(Y_[o:o + n].reshape(n_vars, g.n_points))
            o += n
        return out, status
    return Y_, status


def diffusion_adjoint(grids, B, D, ybar, t_start, t_end, *, h=None, dt_multiplier=10.0, global_timestep=2e-5,
                      wall_const=None):
    """Gradient of phi = ybar . y_out of one diffusion stage with respect to
    its start state (``ember_diffusion_adjoint``): flat host arrays in the
    layout of ``integrate_diffusion_terms``; returns (ybar_in, status)."""
    n_flames = len(grids)
    total_pts = sum(g.n_points for g in grids)
    y = _f64(ybar).copy()
    n_vars = y.size // total_pts
    B_, D_ = _f64(B), _f64(D)
    x_ = np.concatenate([_f64(g.x) for g in grids])
    per_sys = lambda v: _f64(np.broadcast_to(np.asarray(v, dtype=np.float64), (n_flames * n_vars,))) \
        if v is not None else None
    h_, wc_ = per_sys(h), per_sys(wall_const)
    status = np.zeros(n_flames * n_vars, dtype=np.int32)
    garr = (L.DiffusionGrid * n_flames)(*[L.DiffusionGrid(g.n_points, g.left_bc, g.right_bc, g.alpha)
                                          for g in grids])
    opts = L.DiffusionOptions(float(t_start), float(t_end), float(dt_multiplier), float(global_timestep),
                              L.ptr(h_), L.ptr(wc_), None, L.DIFFUSION_SERIAL)
    L.check(L.lib().ember_diffusion_adjoint(n_flames, garr, n_vars, L.ptr(x_), L.ptr(B_), L.ptr(D_), L.ptr(y),
                                            C.byref(opts), L.ptr(status), L.MEM_HOST, None), "ember_diffusion_adjoint")
    return y, status


def synthetic_flames(n_flames: int = 64, n_vars: int = 55, n_min: int = 100, n_max: int = 4000, seed: int = 6455,
                     dt: float = 1e-5):
    """Seeded batch of diffusion stages with uneven grids: N_f uniform in
    [n_min, n_max]; a non-uniform grid whose neighbouring spacings differ by
    at most a factor 1.5 (log-ratio random walk, base spacing 2e-5 m);
    D log-uniform in [1e-6, 1e-3] m^2/s per (variable, point); B = 1 (the
    equations of the variables are scaled as DiffusionSystem's B = 1/rho
    with rho = 1); split constant 0; smooth initial profiles; both boundary
    conditions FixedValue; an explicit step h = dt so that one stage is one
    BDF1 x 8 step (TridiagonalIntegrator::initialize(0, dt) then
    integrateToTime(dt)). Returns (grids, B, D, split, y, h) with the flat
    arrays in the layout of ember_diffusion_integrate."""
    rng = np.random.default_rng(seed)
    grids, Bs, Ds, Ys = [], [], [], []
    for f in range(n_flames):
        n = int(rng.integers(n_min, n_max + 1))
        steps = np.clip(np.cumsum(rng.uniform(-0.3, 0.3, n - 1)), np.log(1 / 20), np.log(20))
        dx = 2e-5 * np.exp(steps)
        ratio = dx[1:] / dx[:-1]
        assert ratio.max() <= 1.5 and ratio.min() >= 1 / 1.5
        x = np.concatenate([[0.0], np.cumsum(dx)])
        grids.append(FlameGrid(x=x))
        Bs.append(np.ones((n_vars, n)))
        Ds.append(np.exp(rng.uniform(np.log(1e-6), np.log(1e-3), (n_vars, n))))
        xs = (x - x[0]) / (x[-1] - x[0])
        phase = rng.uniform(0, 2 * np.pi, (n_vars, 1))
        Ys.append(1.0 + 0.5 * np.tanh(8 * (xs[None, :] - 0.5)) + 0.1 * np.sin(6 * np.pi * xs[None, :] + phase))
    flat = lambda arrs: np.concatenate([a.reshape(-1) for a in arrs])
    B, D, Y = flat(Bs), flat(Ds), flat(Ys)
    return grids, B, D, np.zeros_like(B), Y, np.full(n_flames * n_vars, dt)
