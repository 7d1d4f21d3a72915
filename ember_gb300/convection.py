"""Convection stage on the GPU (``ember_convection_integrate``):
ConvectionSystemSplit::integrateToTime (src/convectionSystem.cpp:588-627) for
a batch of flames -- the UTW system (continuity, upwinded convection of U, T
and the mean molecular weight) stepped to the stage end with V / rho recorded
after every step, then one convection system per species with v(t)
interpolated from that record. Adams integrators with a diagonal
difference-quotient Jacobian, one 256-thread CTA per system.

``convection_batch`` builds a seeded flame-like batch (the strained-flame
profiles of ``split.flame_batch`` with a strained-flow velocity profile).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field, fields

import numpy as np

from . import _lib as L
from .mechanism import GAS_CONSTANT, Mechanism

BC_FIXED_VALUE, BC_ZERO_GRADIENT, BC_CONTROL_VOLUME, BC_WALL_FLUX = 0, 1, 2, 3
CONT_LEFT, CONT_RIGHT, CONT_ZERO, CONT_QDOT, CONT_TEMP = 0, 1, 2, 3, 4
STRAIN_LINEAR, STRAIN_CHEBYSHEV = 0, 1
CHEBYSHEV_MAX = 16
STATUS_RECORD_FULL = -20


class ConvectionFlameC(C.Structure):
    _fields_ = [("n_points", C.c_int), ("left_bc", C.c_int), ("right_bc", C.c_int), ("alpha", C.c_int),
                ("continuity_bc", C.c_int), ("j_cont", C.c_int),
                ("beta", C.c_double), ("x_vzero", C.c_double), ("rv_zero", C.c_double), ("rv_cont", C.c_double),
                ("t_left", C.c_double), ("w_left", C.c_double), ("rhou", C.c_double), ("pressure", C.c_double),
                ("strain_initial", C.c_double), ("strain_final", C.c_double), ("strain_t0", C.c_double),
                ("strain_dt", C.c_double), ("strain_type", C.c_int), ("n_cheb", C.c_int), ("cheb_t0", C.c_double),
                ("cheb_t1", C.c_double), ("cheb", C.c_double * CHEBYSHEV_MAX)]


class ConvectionOptionsC(C.Structure):
    _fields_ = [("t_start", C.c_double), ("t_end", C.c_double), ("reltol", C.c_double), ("abstol_u", C.c_double),
                ("abstol_t", C.c_double), ("abstol_y", C.c_double), ("min_step", C.c_double),
                ("max_steps", C.c_int), ("max_history", C.c_int), ("species_threads", C.c_int)]


@dataclass
class ConvectionFlame:
    """Per-flame parameters of the convection stage (the members of
    ConvectionSystemUTW / ConvectionSystemY that are not state)."""
    n_points: int
    left_bc: int = BC_CONTROL_VOLUME
    right_bc: int = BC_ZERO_GRADIENT
    alpha: int = 0
    continuity_bc: int = CONT_LEFT
    j_cont: int = 0
    beta: float = 1.0
    x_vzero: float = 0.0
    rv_zero: float = 0.0
    rv_cont: float = 0.0
    t_left: float = 300.0
    w_left: float = 28.0
    rhou: float = 1.0
    pressure: float = 101325.0
    strain_initial: float = 100.0
    strain_final: float = 100.0
    strain_t0: float = 0.0
    strain_dt: float = 0.0
    # ChebyshevFunction (strain_type STRAIN_CHEBYSHEV): the interval mapped
    # onto [-1, 1] and the coefficients (setCoefficients(2 + n, {t0, t1, c...}))
    strain_type: int = STRAIN_LINEAR
    cheb_t0: float = 0.0
    cheb_t1: float = 1.0
    cheb: tuple = ()

    @property
    def n_cheb(self) -> int:
        return len(self.cheb)

    def as_c(self) -> ConvectionFlameC:
        if len(self.cheb) > CHEBYSHEV_MAX:
            raise ValueError(f"at most {CHEBYSHEV_MAX} Chebyshev coefficients")
        kw = {f.name: getattr(self, f.name) for f in fields(self) if f.name != "cheb"}
        c = [float(v) for v in self.cheb]
        kw["n_cheb"] = len(c)
        kw["cheb"] = (C.c_double * CHEBYSHEV_MAX)(*(c + [0.0] * (CHEBYSHEV_MAX - len(c))))
        return ConvectionFlameC(**kw)


@dataclass
class ConvectionOptions:
    reltol: float = 1e-6        # integratorRelTol
    abstol_u: float = 1e-7      # integratorMomentumAbsTol
    abstol_t: float = 1e-8      # integratorEnergyAbsTol
    abstol_y: float = 1e-13     # integratorSpeciesAbsTol (W: 20 times it)
    min_step: float = 1e-16     # SundialsCvode::minStep as set by setState
    max_steps: int = 100000
    max_history: int = 4096
    species_threads: int = 0    # CTA width of a species system: 0 or 32 (one warp)


def mean_molecular_weight(Y, W):
    """1 / sum_k (max(Y_k, 0) / sum max(Y, 0)) / W_k, summed in species order
    (the W initial condition of ConvectionSystemSplit::setState)."""
    Y = np.atleast_2d(np.asarray(Y, dtype=np.float64))
    out = np.empty(Y.shape[0])
    for j, y in enumerate(Y):
        ysum = 0.0
        for v in y:
            ysum = ysum + max(v, 0.0)
        rn = 1.0 / ysum
        acc = 0.0
        for v, w in zip(y, W):
            acc = acc + (max(v, 0.0) * rn) / w
        out[j] = 1.0 / acc
    return out


def integrate_convection_terms(flames, mol_weight, x, y_left, drhodt, split_const, state, t_start: float,
                               t_end: float, opts: ConvectionOptions | None = None, stream=None):
    """One convection stage for a batch of flames. ``state`` (U, T, Y rows,
    variable-major per flame, numpy array or torch CUDA tensor) is replaced
    by the result in place. Returns (state, status [n_flames, 1+S], stats
    [n_flames, 4])."""
    opts = opts or ConvectionOptions()
    nf = len(flames)
    S = int(len(mol_weight))
    mem = L.mem_of(state)
    arr = (ConvectionFlameC * max(nf, 1))(*[f.as_c() for f in flames])
    o = ConvectionOptionsC(float(t_start), float(t_end), opts.reltol, opts.abstol_u, opts.abstol_t, opts.abstol_y,
                           opts.min_step, int(opts.max_steps), int(opts.max_history), int(opts.species_threads))
    if mem == L.MEM_HOST:
        conv = lambda a: np.ascontiguousarray(a, dtype=np.float64)  # noqa: E731
        W, x, y_left, drhodt, split_const = map(conv, (mol_weight, x, y_left, drhodt, split_const))
        if not (isinstance(state, np.ndarray) and state.dtype == np.float64 and state.flags.c_contiguous):
            raise TypeError("state must be a C-contiguous float64 numpy array (updated in place)")
        status = np.zeros((nf, 1 + S), dtype=np.int32)
        stats = np.zeros((nf, 4), dtype=np.int32)
    else:
        import torch
        dev = state.device
        conv = lambda a: torch.as_tensor(a, dtype=torch.float64, device=dev).contiguous()  # noqa: E731
        W, x, y_left, drhodt, split_const = map(conv, (mol_weight, x, y_left, drhodt, split_const))
        status = torch.zeros((nf, 1 + S), dtype=torch.int32, device=dev)
        stats = torch.zeros((nf, 4), dtype=torch.int32, device=dev)
    L.check(L.lib().ember_convection_integrate(nf, C.addressof(arr), S, L.ptr(W), L.ptr(x), L.ptr(y_left),
                                               L.ptr(drhodt), L.ptr(split_const), L.ptr(state), C.byref(o),
                                               L.ptr(status), L.ptr(stats), mem, L.stream_ptr(stream)),
            "ember_convection_integrate")
    return state, status, stats


@dataclass
class ConvectionBatch:
    flames: list
    x: np.ndarray            # concatenated grid
    state: np.ndarray        # variable-major per flame, (S + 2) * sum N
    split_const: np.ndarray  # same layout
    drhodt: np.ndarray       # concatenated
    y_left: np.ndarray       # [n_flames, S]
    offsets: np.ndarray = field(default=None)   # flame f: points [offsets[f], offsets[f+1])


def convection_batch(mech: Mechanism, n_flames: int = 32, n_min: int = 150, n_max: int = 700, seed: int = 3232,
                     strain_range=(100.0, 2000.0), split_scale: float = 0.0, drhodt_scale: float = 0.0,
                     pressure: float = 101325.0) -> ConvectionBatch:
    """Seeded strained-flame-like batch: the profiles of split.flame_batch,
    strain rates log-spaced over ``strain_range``, U = (a / beta) sqrt(rho_u /
    rho) (the potential-flow profile the reference starts from), a left
    control-volume boundary fed with the unburned mixture at rVzero = rho_u
    S_u (S_u = 0.4 m/s), an outflow right boundary, the continuity integral
    from the left. ``split_scale`` / ``drhodt_scale`` add seeded split
    constants and density derivatives of that relative size."""
    from .split import flame_batch
    grids, st_pm, _, _, rho_u, _, _ = flame_batch(mech, n_flames=n_flames, n_min=n_min, n_max=n_max, seed=seed,
                                                  pressure=pressure)
    rng = np.random.default_rng(seed + 1)
    S, W = mech.n_species, mech.mol_weight
    strains = np.geomspace(strain_range[0], strain_range[1], n_flames)
    flames, xs, states, splits, drs, yls = [], [], [], [], [], []
    p = 0
    offsets = [0]
    for f, g in enumerate(grids):
        N = g.n_points
        st = st_pm[p:p + N]
        p += N
        T = st[:, 1]
        Y = st[:, 2:]
        wmix = 1.0 / (Y / W[None, :]).sum(axis=1)
        rho = pressure * wmix / (GAS_CONSTANT * T)
        a = float(strains[f])
        U = a * np.sqrt(rho_u[f] / rho)
        sv = np.empty((S + 2, N))
        sv[0] = U
        sv[1] = T
        sv[2:] = Y.T
        sc = np.zeros_like(sv)
        if split_scale:
            sc[0] = split_scale * a * a * rng.standard_normal(N)
            sc[1] = split_scale * 1e5 * rng.standard_normal(N)
            sc[2:] = split_scale * 10.0 * rng.standard_normal((S, N)) * np.maximum(Y.T, 1e-6)
        dr = drhodt_scale * rho * 100.0 * rng.standard_normal(N) if drhodt_scale else np.zeros(N)
        y_left = Y[0].copy()
        flames.append(ConvectionFlame(n_points=N, rhou=float(rho_u[f]), rv_zero=float(rho_u[f] * 0.4),
                                      t_left=float(T[0]), w_left=float(mean_molecular_weight(y_left, W)[0]),
                                      pressure=pressure, strain_initial=a, strain_final=a))
        xs.append(g.x)
        states.append(sv.reshape(-1))
        splits.append(sc.reshape(-1))
        drs.append(dr)
        yls.append(y_left)
        offsets.append(offsets[-1] + N)
    return ConvectionBatch(flames=flames, x=np.concatenate(xs), state=np.concatenate(states),
                           split_const=np.concatenate(splits), drhodt=np.concatenate(drs), y_left=np.array(yls),
                           offsets=np.array(offsets, dtype=np.int64))
