"""Split step of a batch of flames on the GPU.

``FlameBatchSplitSolver`` is ``SplitSolver::step`` (src/splitSolver.cpp:
34-121) with FlameSolver's stage hooks (src/flameSolver.cpp:702-854) and
mass-fraction correction (src/flameSolver.cpp:219-224, 942-949), for many
flames at once, every array resident on the device (``ember_split_*`` in the
C ABI). Convection is not integrated (its rate can enter through
``ddt_cross``); see include/ember_gpu.h for the split constants used.

``flame_batch`` builds the seeded flame-like inputs of the strain-sweep proxy
(flame-shaped profiles with synthetic transport coefficients).
"""
from __future__ import annotations

import copy
import ctypes as C

import numpy as np

from . import _lib as L
from .diffusion import FlameGrid
from .mechanism import GAS_CONSTANT, Mechanism, nasa_cp_R, stoichiometric_ch4_air
from .source import BDF, QSS, SourceOptions, GpuMechanism, STATS_WIDTH


class SplitOptions(C.Structure):
    _fields_ = [("method", C.c_int), ("diffusion_algorithm", C.c_int), ("balanced", C.c_int), ("dt", C.c_double),
                ("dt_multiplier", C.c_double), ("source", SourceOptions)]


def _declare(lib):
    vp = C.c_void_p
    sig = {
        "ember_split_create": (C.c_int, [vp, C.c_int, C.POINTER(L.DiffusionGrid), vp, C.POINTER(SplitOptions),
                                         C.POINTER(vp)]),
        "ember_split_destroy": (C.c_int, [vp]),
        "ember_split_set_state": (C.c_int, [vp, C.c_double, vp, C.c_int, vp]),
        "ember_split_set_transport": (C.c_int, [vp, vp, vp, vp, C.c_int, vp]),
        "ember_split_step": (C.c_int, [vp, C.c_int, C.c_int, vp]),
        "ember_split_get_state": (C.c_int, [vp, vp, vp, C.c_int, vp]),
        "ember_split_get_derivatives": (C.c_int, [vp, vp, vp, C.c_int, vp]),
        "ember_split_set_derivatives": (C.c_int, [vp, vp, vp, vp, C.c_int, vp]),
        "ember_split_source_status": (C.c_int, [vp, vp, vp, C.c_int, vp]),
        "ember_split_failures": (C.c_int, [vp, vp, vp, vp]),
        "ember_split_objectives": (C.c_int, [vp, vp, vp, vp, vp, vp, vp, C.c_int, vp]),
        "ember_split_adjoint": (C.c_int, [vp, vp, vp, vp, vp, vp, C.c_int, vp, vp, vp, vp, C.c_int, vp]),
        "ember_split_set_convection": (C.c_int, [vp, vp, vp, vp]),
        "ember_split_set_strain": (C.c_int, [vp, C.c_int, vp, vp]),
        "ember_split_get_convection_derivative": (C.c_int, [vp, vp, C.c_int, vp]),
        "ember_split_get_velocity": (C.c_int, [vp, vp, C.c_int, vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


_declared = False


def _lib():
    global _declared
    lib = L.lib()
    if not _declared:
        _declare(lib)
        _declared = True
    return lib


class FlameBatchSplitSolver:
    """Split steps of a batch of flames on the GPU.

    State arrays are point-major ``[n_points, S+2]`` (U, T, Y), flames
    concatenated; ``B`` and ``D`` are variable-major per flame (as
    ``integrate_diffusion_terms``). numpy arrays are copied from/to the host;
    torch CUDA tensors are used on the device.
    """

    def __init__(self, gmech: GpuMechanism, grids, dt: float, *, method: int = QSS, source_options=None,
                 balanced: bool = True, diffusion_algorithm: int = L.DIFFUSION_PARALLEL, dt_multiplier: float = 10.0):
        self.gmech = gmech
        self.grids = list(grids)
        self.n_vars = gmech.mech.n_vars
        self.n_points = sum(g.n_points for g in self.grids)
        self.dt = float(dt)
        opts = SplitOptions()
        opts.method = int(method)
        opts.diffusion_algorithm = int(diffusion_algorithm)
        opts.balanced = int(bool(balanced))
        opts.dt = float(dt)
        opts.dt_multiplier = float(dt_multiplier)
        opts.source = source_options if source_options is not None else SourceOptions.defaults()
        self.options = opts
        garr = (L.DiffusionGrid * len(self.grids))(*[L.DiffusionGrid(g.n_points, g.left_bc, g.right_bc, g.alpha)
                                                     for g in self.grids])
        x = np.ascontiguousarray(np.concatenate([np.asarray(g.x, dtype=np.float64) for g in self.grids]))
        h = C.c_void_p()
        L.check(_lib().ember_split_create(gmech.handle, len(self.grids), garr, x.ctypes.data, C.byref(opts),
                                          C.byref(h)), "ember_split_create")
        self._h = h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib().ember_split_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _arr(self, a, shape):
        if hasattr(a, "data_ptr"):
            return a, L.mem_of(a)
        a = np.ascontiguousarray(a, dtype=np.float64)
        if a.size != int(np.prod(shape)):
            raise ValueError(f"expected {int(np.prod(shape))} values, got {a.size}")
        return a, L.MEM_HOST

    def set_state(self, t: float, state):
        a, mem = self._arr(state, (self.n_points, self.n_vars))
        L.check(_lib().ember_split_set_state(self._h, float(t), L.ptr(a), mem, None), "ember_split_set_state")

    def load_state(self, state, stream=None):
        """ember_split_load_state: new state values, same time and split history."""
        a, mem = self._arr(state, (self.n_points, self.n_vars))
        L.check(_lib().ember_split_load_state(self._h, L.ptr(a), mem, L.stream_ptr(stream)), "ember_split_load_state")

    def set_transport(self, B, D, ddt_cross=None, stream=None):
        n = self.n_points * self.n_vars
        b, mem = self._arr(B, (n,))
        d, _ = self._arr(D, (n,))
        x = self._arr(ddt_cross, (n,))[0] if ddt_cross is not None else None
        L.check(_lib().ember_split_set_transport(self._h, L.ptr(b), L.ptr(d), L.ptr(x), mem, L.stream_ptr(stream)),
                "ember_split_set_transport")

    def set_transport_model(self, transport=None, threshold: float = 1e-5, cross_terms: bool = True):
        """ember_split_set_transport_model: B, D (and with cross_terms the
        cross terms) from a GpuTransport at the start of every step; None
        detaches."""
        self._transport = transport  # keeps the handle alive
        L.check(_lib().ember_split_set_transport_model(self._h, transport.handle if transport is not None else None,
                                                       float(threshold), int(bool(cross_terms))),
                "ember_split_set_transport_model")

    def set_convection(self, flames=None, y_left=None, opts=None):
        """ember_split_set_convection: every step becomes D C D S D C D with
        the convection stage of ``flames`` (ember_gb300.convection.
        ConvectionFlame, one per flame; y_left [n_flames, S]; opts a
        ConvectionOptions); None detaches."""
        if flames is None:
            L.check(_lib().ember_split_set_convection(self._h, None, None, None), "ember_split_set_convection")
            self._convection = None
            return
        from .convection import ConvectionFlameC, ConvectionOptions, ConvectionOptionsC
        opts = opts or ConvectionOptions()
        arr = (ConvectionFlameC * len(flames))(*[f.as_c() for f in flames])
        o = ConvectionOptionsC(0.0, 0.0, opts.reltol, opts.abstol_u, opts.abstol_t, opts.abstol_y, opts.min_step,
                               int(opts.max_steps), int(opts.max_history), int(opts.species_threads))
        yl = np.ascontiguousarray(y_left, dtype=np.float64)
        L.check(_lib().ember_split_set_convection(self._h, C.addressof(arr), yl.ctypes.data, C.byref(o)),
                "ember_split_set_convection")
        # the handle's view of the flames' strain functions, for the output writers (copies: the
        # caller's objects are left as given)
        self._convection = [copy.copy(f) for f in flames]

    def set_strain_chebyshev(self, coeffs, stream=None):
        """ember_split_set_strain: per flame a row {t0, t1, c_0, ..., c_{n-1}}
        (the ChebyshevFunction coefficients of [t0, t1]); from the next step
        every flame's strain rate is that series."""
        c = np.ascontiguousarray(coeffs, dtype=np.float64)
        if c.ndim != 2 or c.shape[0] != len(self.grids) or c.shape[1] < 2:
            raise ValueError("coeffs must be [n_flames, 2 + n]")
        L.check(_lib().ember_split_set_strain(self._h, c.shape[1] - 2, c.ctypes.data, L.stream_ptr(stream)),
                "ember_split_set_strain")
        from .convection import STRAIN_CHEBYSHEV
        for fl, row in zip(getattr(self, "_convection", None) or [], c):
            fl.strain_type, fl.cheb_t0, fl.cheb_t1, fl.cheb = STRAIN_CHEBYSHEV, float(row[0]), float(row[1]), \
                tuple(float(v) for v in row[2:])

    def step(self, n_steps: int = 1, graph: bool = False, stream=None):
        L.check(_lib().ember_split_step(self._h, int(n_steps), int(bool(graph)), L.stream_ptr(stream)),
                "ember_split_step")

    def state(self, out=None):
        """(state, t); ``out`` may be a device tensor to fill on the device."""
        t = C.c_double()
        if out is not None and hasattr(out, "data_ptr") and L.mem_of(out) == L.MEM_DEVICE:
            L.check(_lib().ember_split_get_state(self._h, L.ptr(out), None, L.MEM_DEVICE, None), "get_state")
            L.check(_lib().ember_split_get_state(self._h, None, C.addressof(t), L.MEM_HOST, None), "get_state")
            return out, t.value
        s = np.empty((self.n_points, self.n_vars))
        L.check(_lib().ember_split_get_state(self._h, s.ctypes.data, C.addressof(t), L.MEM_HOST, None), "get_state")
        return s, t.value

    def derivatives(self):
        dd = np.empty((self.n_points, self.n_vars))
        dp = np.empty((self.n_points, self.n_vars))
        L.check(_lib().ember_split_get_derivatives(self._h, dd.ctypes.data, dp.ctypes.data, L.MEM_HOST, None),
                "get_derivatives")
        return dd, dp

    def convection_derivative(self):
        """ddtConv of the last step (convection stage attached)."""
        dc = np.empty((self.n_points, self.n_vars))
        L.check(_lib().ember_split_get_convection_derivative(self._h, dc.ctypes.data, L.MEM_HOST, None),
                "get_convection_derivative")
        return dc

    def velocity(self):
        """V per point at the UTW systems' last evaluation (convection stage attached)."""
        v = np.empty(self.n_points)
        L.check(_lib().ember_split_get_velocity(self._h, v.ctypes.data, L.MEM_HOST, None), "get_velocity")
        return v

    def set_derivatives(self, ddt_diff, ddt_prod, ddt_conv=None):
        """ember_split_set_derivatives: the time derivatives behind the next
        step's split constants (e.g. interpolated onto a new grid)."""
        shape = (self.n_points, self.n_vars)
        dd, mem = self._arr(ddt_diff, shape)
        dp, _ = self._arr(ddt_prod, shape)
        dc = self._arr(ddt_conv, shape)[0] if ddt_conv is not None else None
        L.check(_lib().ember_split_set_derivatives(self._h, L.ptr(dd), L.ptr(dp), L.ptr(dc), mem, None),
                "ember_split_set_derivatives")

    def source_status(self):
        st = np.empty(self.n_points, dtype=np.int32)
        stats = np.empty((self.n_points, STATS_WIDTH), dtype=np.int32)
        L.check(_lib().ember_split_source_status(self._h, st.ctypes.data, stats.ctypes.data, L.MEM_HOST, None),
                "source_status")
        return st, stats

    def failures(self):
        a, b = C.c_int64(), C.c_int64()
        L.check(_lib().ember_split_failures(self._h, C.addressof(a), C.addressof(b), None), "failures")
        return a.value, b.value

    def objectives(self, rho_u=None, ju=None, jb=None, device=None):
        """(qdot [n_points], heat release rate [n_flames], consumption speed
        [n_flames] or None) of the current state. With ``device`` (a torch
        device) the inputs may be tensors there and the outputs are tensors
        on it, with no host round trip."""
        nf = len(self.grids)
        if device is not None:
            import torch
            f64 = lambda v: torch.as_tensor(v, dtype=torch.float64, device=device).contiguous() \
                if v is not None else None
            i32 = lambda v: torch.as_tensor(v, dtype=torch.int32, device=device).contiguous() \
                if v is not None else None
            q = torch.empty(self.n_points, dtype=torch.float64, device=device)
            hr = torch.empty(nf, dtype=torch.float64, device=device)
            cs = torch.empty(nf, dtype=torch.float64, device=device) if rho_u is not None else None
            r, a, b, mem = f64(rho_u), i32(ju), i32(jb), L.MEM_DEVICE
        else:
            q = np.empty(self.n_points)
            hr = np.empty(nf)
            cs = np.empty(nf) if rho_u is not None else None
            r = np.ascontiguousarray(rho_u, dtype=np.float64) if rho_u is not None else None
            a = np.ascontiguousarray(ju, dtype=np.int32) if ju is not None else None
            b = np.ascontiguousarray(jb, dtype=np.int32) if jb is not None else None
            mem = L.MEM_HOST
        L.check(_lib().ember_split_objectives(self._h, L.ptr(r), L.ptr(a), L.ptr(b), L.ptr(q), L.ptr(hr),
                                              L.ptr(cs), mem, None), "objectives")
        return q, hr, cs

    def adjoint(self, w_heat_release=None, w_consumption_speed=None, rho_u=None, ju=None, jb=None,
                tape_cap: int = 0, device=None):
        """One split step from the current state and the gradient of
        J = sum_f w_heat_release[f] Q_f + w_consumption_speed[f] S_c,f at its end
        with respect to the state at its start and ln(multiplier) of every
        reaction (``ember_split_adjoint``; BDF or QSS source). Returns (Q, S_c or None,
        d J / d state [n_points, S+2], d J / d ln multiplier [R]); with
        ``device`` (a torch device) as tensors there, computed without a host
        round trip."""
        nf = len(self.grids)
        R = self.gmech.mech.n_reactions
        if device is not None:
            import torch
            f64 = lambda v: torch.as_tensor(v, dtype=torch.float64, device=device).contiguous() \
                if v is not None else None
            i32 = lambda v: torch.as_tensor(v, dtype=torch.int32, device=device).contiguous() \
                if v is not None else None
            wq, ws, r, a, b = f64(w_heat_release), f64(w_consumption_speed), f64(rho_u), i32(ju), i32(jb)
            hr = torch.empty(nf, dtype=torch.float64, device=device)
            cs = torch.empty(nf, dtype=torch.float64, device=device) if ws is not None else None
            sbar = torch.empty((self.n_points, self.n_vars), dtype=torch.float64, device=device)
            lbar = torch.empty(max(R, 1), dtype=torch.float64, device=device)
            mem = L.MEM_DEVICE
        else:
            f64 = lambda v: np.ascontiguousarray(v, dtype=np.float64) if v is not None else None
            i32 = lambda v: np.ascontiguousarray(v, dtype=np.int32) if v is not None else None
            wq, ws, r = f64(w_heat_release), f64(w_consumption_speed), f64(rho_u)
            a, b = i32(ju), i32(jb)
            hr = np.empty(nf)
            cs = np.empty(nf) if ws is not None else None
            sbar = np.empty((self.n_points, self.n_vars))
            lbar = np.empty(max(R, 1))
            mem = L.MEM_HOST
        L.check(_lib().ember_split_adjoint(self._h, L.ptr(wq), L.ptr(ws), L.ptr(r), L.ptr(a), L.ptr(b), int(tape_cap),
                                           L.ptr(hr), L.ptr(cs), L.ptr(sbar), L.ptr(lbar), mem, None),
                "ember_split_adjoint")
        return hr, cs, sbar, lbar[:R]


def mixture_properties(mech: Mechanism, state, pressure: float = 101325.0):
    """Density, cp (J/kg/K) of point-major states from the mechanism's NASA7
    thermo (ideal gas)."""
    T = state[:, 1]
    Y = state[:, 2:]
    W = mech.mol_weight
    wmix = 1.0 / (Y / W[None, :]).sum(axis=1)
    rho = pressure * wmix / (GAS_CONSTANT * T)
    cp = np.zeros_like(T)
    for k in range(mech.n_species):
        lo = mech.nasa_coeffs[k, 0:7]
        hi = mech.nasa_coeffs[k, 7:14]
        a_lo, a_hi = nasa_cp_R(lo, T), nasa_cp_R(hi, T)
        cpk = np.where(T <= mech.nasa_tmid[k], a_lo, a_hi) * GAS_CONSTANT / W[k]
        cp += Y[:, k] * cpk
    return rho, cp


def flame_batch(mech: Mechanism, n_flames: int = 32, n_min: int = 150, n_max: int = 700, seed: int = 3232,
                width: float = 0.02, thickness: float = 5e-4, T_u: float = 300.0, T_b: float = 2000.0,
                pressure: float = 101325.0):
    """Seeded flame-like batch (the strain-sweep proxy): flame f has N_f
    points (uniform in [n_min, n_max]) on [-width/2, width/2] clustered at
    the flame (x = sinh map), a progress variable c = (1 + tanh(x/thickness))
    / 2 with a seeded flame-position shift, T = T_u + (T_b - T_u) c, Y the
    blend of stoichiometric CH4/air and its complete-combustion products.
    Transport coefficients are synthetic power laws (transport is not part of
    this library): mu = 1.8e-5 (T/300)^0.7, lambda = 0.026 (T/300)^0.8,
    rho D_k = rho 2e-5 (T/300)^1.75 (W_N2 / W_k)^0.5; B = 1/rho (U, Y_k) and
    1/(rho cp) (T). Both boundaries FixedValue, planar. Returns (grids,
    state [n_points, S+2], B, D) with B, D variable-major per flame, and the
    per-flame unburned density and (ju, jb) indices."""
    rng = np.random.default_rng(seed)
    y_r, y_p = stoichiometric_ch4_air(mech)
    W = mech.mol_weight
    try:
        w_n2 = W[mech.species_index("N2")]
    except ValueError:
        w_n2 = 28.0
    grids, states, Bs, Ds, rho_u = [], [], [], [], []
    for f in range(n_flames):
        n = int(rng.integers(n_min, n_max + 1))
        s = np.linspace(-1.0, 1.0, n)
        x = 0.5 * width * np.sinh(3.0 * s) / np.sinh(3.0)
        x0 = rng.uniform(-0.1, 0.1) * width
        c = 0.5 * (1.0 + np.tanh((x - x0) / thickness))
        T = T_u + (T_b - T_u) * c
        Y = (1.0 - c)[:, None] * y_r[None, :] + c[:, None] * y_p[None, :]
        Y /= Y.sum(axis=1, keepdims=True)
        st = np.zeros((n, mech.n_vars))
        st[:, 1] = T
        st[:, 2:] = Y
        rho, cp = mixture_properties(mech, st, pressure)
        th = T / 300.0
        B = np.empty((mech.n_vars, n))
        D = np.empty((mech.n_vars, n))
        B[0], D[0] = 1.0 / rho, 1.8e-5 * th ** 0.7
        B[1], D[1] = 1.0 / (rho * cp), 0.026 * th ** 0.8
        B[2:] = (1.0 / rho)[None, :]
        D[2:] = (rho * 2e-5 * th ** 1.75)[None, :] * np.sqrt(w_n2 / W)[:, None]
        grids.append(FlameGrid(x=x))
        states.append(st)
        Bs.append(B.reshape(-1))
        Ds.append(D.reshape(-1))
        rho_u.append(rho[0])
    ju = np.zeros(n_flames, dtype=np.int32)
    jb = np.array([g.n_points - 1 for g in grids], dtype=np.int32)
    return grids, np.concatenate(states), np.concatenate(Bs), np.concatenate(Ds), np.array(rho_u), ju, jb
