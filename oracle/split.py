"""CPU ORACLE -- test infrastructure only.

Restatement of the split step of a batch of flames in the reference's
operation order, built from the oracle's diffusion systems (oracle_tridiag.c)
and source-term integrators (oracle_chem.c / oracle_bdf.c):

  SplitSolver::step / integrateSplitTerms / calculateTimeDerivatives
      src/splitSolver.cpp:27-121 (convection stages not integrated; the
      two-operator balanced split constants of the device split step)
  FlameSolver::setDiffusionSolverState / integrateDiffusionTerms
      src/flameSolver.cpp:702-718, 838-854
  FlameSolver::setProductionSolverState / integrateProductionTerms
      src/flameSolver.cpp:727-836
  FlameSolver::finishStep -> correctMassFractions
      src/flameSolver.cpp:219-224, 942-949
  FlameSolver::calculateQdot / getHeatReleaseRate / getConsumptionSpeed,
  mathUtils::integrate / computeSplines
      src/flameSolver.cpp:926-961, src/mathUtils.h:189-237, 338-358
"""
from __future__ import annotations

import numpy as np

import oracle


def _seq_sum(a, axis=-1):
    """Sum in index order (np.cumsum accumulates sequentially)."""
    return np.cumsum(a, axis=axis).take(-1, axis=axis)


def correct_mass_fractions(state):
    Y = state[:, 2:]
    Yc = np.where(Y < 0.0, 0.0, Y)
    r = 1.0 / _seq_sum(Yc, axis=1)
    state[:, 2:] = Yc * r[:, None]


def split_steps(omech, grids, state, t, B, D, dt, n_steps, method, opts, ddt_cross=None, balanced=True,
                mult=10.0, ddt=None):
    """n_steps split steps of a batch of flames. state: point-major [n_pts, n]
    (copied); B, D: variable-major per flame (flat). Returns (state, t,
    ddt_diff, ddt_prod, source_status_of_last_step)."""
    state = np.array(state, dtype=np.float64, copy=True)
    n_pts, n = state.shape
    offs = np.cumsum([0] + [g.n_points for g in grids])
    voffs = offs * n
    xs = np.concatenate([np.asarray(g.x, dtype=np.float64) for g in grids])
    cross = np.zeros_like(state) if ddt_cross is None else np.asarray(ddt_cross, dtype=np.float64).reshape(n_pts, n)
    ddt_diff = np.zeros_like(state) if ddt is None else ddt[0].copy()
    ddt_prod = np.zeros_like(state) if ddt is None else ddt[1].copy()
    status = None
    for _ in range(n_steps):
        if balanced:
            sc_diff = 0.5 * ((ddt_prod + cross) - ddt_diff)
            sc_prod = 0.5 * ((ddt_diff + cross) - ddt_prod)
        else:
            sc_diff = cross.copy()
            sc_prod = np.zeros_like(state)
        delta = np.zeros_like(state)

        def diffusion(f0, f1):
            t0 = t if f0 == 0.0 else t + f0 * dt
            t1 = t + f1 * dt
            for f, g in enumerate(grids):
                a, b = offs[f], offs[f + 1]
                N = b - a
                for v in range(n):
                    row = slice(voffs[f] + v * N, voffs[f] + (v + 1) * N)
                    y0 = state[a:b, v].copy()
                    y1 = oracle.diffusion_system(g.x, B[row], D[row], y0, t0, t1, split_const=sc_diff[a:b, v].copy(),
                                                 alpha=g.alpha, left_bc=g.left_bc, right_bc=g.right_bc, h=0.0,
                                                 mult=mult, gdt=dt)
                    delta[a:b, v] = delta[a:b, v] + (y1 - y0)
                    state[a:b, v] = y1

        diffusion(0.0, 0.25)
        diffusion(0.25, 0.5)
        xD2 = state.copy()
        dtp = np.full(n_pts, (t + dt) - t)
        out, status, _ = omech.integrate(method, state, dtp, opts, split_const=sc_prod, t_start=t, x=xs)
        state[:] = out
        xS = state.copy()
        diffusion(0.5, 0.75)
        diffusion(0.75, 1.0)
        ddt_diff = delta / dt - sc_diff
        ddt_prod = (xS - xD2) / dt - sc_prod
        correct_mass_fractions(state)
        t = t + dt
    return state, t, ddt_diff, ddt_prod, status


def spline_integral(x, y):
    """mathUtils::integrate: integral of the natural cubic spline through (x, y)."""
    x = [float(v) for v in x]
    y = [float(v) for v in y]
    n = len(x)
    hh = lambda i: x[i + 1] - x[i]
    bb = lambda i: (y[i + 1] - y[i]) / hh(i)
    u = [0.0] * n
    v = [0.0] * n
    z = [0.0] * n
    u[1] = 2 * (hh(0) + hh(1))
    v[1] = 6 * (bb(1) - bb(0))
    for i in range(2, n - 1):
        u[i] = 2 * (hh(i - 1) + hh(i)) - hh(i - 1) * hh(i - 1) / u[i - 1]
        v[i] = 6 * (bb(i) - bb(i - 1)) - hh(i - 1) * v[i - 1] / u[i - 1]
    for i in range(n - 2, 0, -1):
        z[i] = (v[i] - hh(i) * z[i + 1]) / u[i]
    total = 0.0
    for i in range(n - 1):
        h = hh(i)
        c0 = y[i]
        c1 = -h / 6 * z[i + 1] - h / 3 * z[i] + (y[i + 1] - y[i]) / h
        c2 = 0.5 * z[i]
        c3 = (z[i + 1] - z[i]) / (6 * h)
        dx = x[i + 1] - x[i]
        total += dx * (c0 + dx * (c1 / 2 + dx * (c2 / 3 + dx * c3 / 4)))
    return total


def objectives(omech, grids, state, pressure, kinetics_model, rho_u=None, ju=None, jb=None):
    """(qdot, heat release per flame, consumption speed per flame or None)."""
    from ember_gb300.source import STATE_NORMALIZED
    g = omech.gas_eval(state[:, 1], state[:, 2:], pressure=pressure, model=kinetics_model, mode=STATE_NORMALIZED)
    qdot = -_seq_sum(g["net"] * g["hk"], axis=1)
    qcp = qdot / g["cp_mass"]
    offs = np.cumsum([0] + [gr.n_points for gr in grids])
    hr = np.array([spline_integral(gr.x, qdot[offs[f]:offs[f + 1]]) for f, gr in enumerate(grids)])
    cs = None
    if rho_u is not None:
        cs = np.empty(len(grids))
        for f, gr in enumerate(grids):
            T = state[offs[f]:offs[f + 1], 1]
            cs[f] = spline_integral(gr.x, qcp[offs[f]:offs[f + 1]]) / (rho_u[f] * (T[jb[f]] - T[ju[f]]))
    return qdot, hr, cs
