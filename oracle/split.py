"""CPU ORACLE -- test infrastructure only.

Restatement of the split step of a batch of flames in the reference's
operation order, built from the oracle's diffusion systems (oracle_tridiag.c)
and source-term integrators (oracle_chem.c / oracle_bdf.c):

  SplitSolver::step / integrateSplitTerms / calculateTimeDerivatives
      src/splitSolver.cpp:27-121: D-S-D with the two-operator balanced
      split constants of the device split step, or, with a convection stage
      (oracle_convection.c), the reference's D C D S D C D with its
      three-operator constants and prepareIntegrators' density derivative
      (src/flameSolver.cpp:208-213)
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


def step_properties(omech, tdata, grids, state, pressure, threshold, mult, gdt, cross_terms, props_out=None):
    """Start of FlameSolver::step for a batch of flames: updateChemicalProperties
    (src/flameSolver.cpp:652-699, thermo and "Approx" transport from
    oracle_transport.c), prepareIntegrators' diffusion coefficients
    (src/flameSolver.cpp:156-172: B = 1/rho, D = mu for U; 1/(rho cp), lambda
    for T; 1/rho, rho D_k for Y_k) and, with cross_terms, updateCrossTerms
    (src/flameSolver.cpp:551-617) without thermal diffusion: Fick fluxes,
    the correction flux jCorr smoothed by a tridiagonal integration with
    B = lambda/(rho cp), D = 1 over [0, globalTimestep], and the species and
    temperature cross terms. Returns (B, D, ddt_cross) in the layouts of
    split_steps; the properties go into props_out (a dict) when given."""
    from oracle import chem
    n_pts, n = state.shape
    S = n - 2
    props = chem.transport_eval(omech, tdata, state[:, 1], state[:, 2:], pressure, threshold)
    if props_out is not None:
        props_out.update(props)
    rho, cp, lam, mu = props["density"], props["cp_mass"], props["conductivity"], props["viscosity"]
    rhoD, cpS = props["rho_d"], props["cp_species"]
    W = [float(w) for w in omech.mech.mol_weight]
    offs = np.cumsum([0] + [g.n_points for g in grids])
    B = np.empty(n_pts * n)
    D = np.empty(n_pts * n)
    for f in range(len(grids)):
        a, b = offs[f], offs[f + 1]
        N = b - a
        base = a * n
        B[base:base + N] = 1.0 / rho[a:b]
        D[base:base + N] = mu[a:b]
        B[base + N:base + 2 * N] = 1.0 / (rho[a:b] * cp[a:b])
        D[base + N:base + 2 * N] = lam[a:b]
        for k in range(S):
            B[base + (2 + k) * N:base + (3 + k) * N] = 1.0 / rho[a:b]
            D[base + (2 + k) * N:base + (3 + k) * N] = rhoD[a:b, k]
    cross = np.zeros((n_pts, n))
    if not cross_terms:
        return B, D, cross
    for f, g in enumerate(grids):
        a, b = offs[f], offs[f + 1]
        N = b - a
        x = [float(v) for v in g.x]
        Y = state[a:b, 2:]
        T = state[a:b, 1]
        rd = rhoD[a:b]
        jc = [0.0] * N
        for i in range(N - 1):
            hh = x[i + 1] - x[i]
            s = 0.0
            for k in range(S):
                F = (-0.5 * (rd[i, k] + rd[i + 1, k])) * ((Y[i + 1, k] - Y[i, k]) / hh)
                s = s - F
            jc[i] = s
        jB = lam[a:b] / (rho[a:b] * cp[a:b])
        h = gdt
        for i in range(1, N - 1):
            dlj = 0.5 * (x[i + 1] - x[i - 1])
            cand = ((mult * dlj) * dlj) / jB[i]
            h = cand if cand < h else h
        jc = oracle.diffusion_system(g.x, jB, np.ones(N), np.array(jc), 0.0, gdt, split_const=np.zeros(N),
                                     alpha=g.alpha, left_bc=g.left_bc, right_bc=g.right_bc, h=h, mult=mult, gdt=gdt)
        jc = [float(v) for v in jc]
        sumcpj = [0.0] * N
        for i in range(1, N - 1):
            r = x[i] ** g.alpha
            rph = (0.5 * (x[i] + x[i + 1])) ** g.alpha
            rphm = (0.5 * (x[i - 1] + x[i])) ** g.alpha
            dlj = 0.5 * (x[i + 1] - x[i - 1])
            hh = x[i + 1] - x[i]
            c = -0.5 / ((r * float(rho[a + i])) * dlj)
            s = 0.0
            for k in range(S):
                yk, yk1, ykm = float(Y[i, k]), float(Y[i + 1, k]), float(Y[i - 1, k])
                cross[a + i, 2 + k] = c * ((rph * (yk + yk1)) * jc[i] - (rphm * (ykm + yk)) * jc[i - 1])
                F = (-0.5 * (float(rd[i, k]) + float(rd[i + 1, k]))) * ((yk1 - yk) / hh)
                s = s + ((0.5 * (float(cpS[a + i, k]) + float(cpS[a + i + 1, k]))) / W[k]) * (
                    F + ((0.5 * (yk + yk1)) * jc[i]))
            sumcpj[i] = s
        for i in range(1, N - 1):
            hh, hm = x[i + 1] - x[i], x[i] - x[i - 1]
            cfp = hm / (hh * (hh + hm))
            cf = (hh - hm) / (hh * hm)
            cfm = -hh / (hm * (hh + hm))
            dTdx = (cfm * float(T[i - 1]) + cf * float(T[i])) + cfp * float(T[i + 1])
            cross[a + i, 1] = ((-0.5 * (sumcpj[i] + sumcpj[i - 1])) * dTdx) / (float(cp[a + i]) * float(rho[a + i]))
    return B, D, cross


def _sign(v):
    return 1 if v > 0 else (-1 if v < 0 else 0)


def continuity_point(fl, x, T, qdot, V, rV):
    """ConvectionSystemUTW::updateContinuityBoundaryCondition
    (src/convectionSystem.cpp:196-277) at the start of a step: the continuity
    point j_cont of the flame's condition from the step-start temperature, its
    heat release rate and V of the UTW system's last evaluation; x_vzero for
    the stagnation-point condition; and rv_cont, the value rV[j_cont] keeps
    (the reference's right-hand side never writes it for the fixedRight and
    fixedQdot conditions). Updates fl in place."""
    N = len(x)
    jj = N - 1
    bc = fl.continuity_bc
    if bc == 0:        # fixedLeft
        jc = 0
    elif bc == 1:      # fixedRight
        jc = jj
    elif bc == 3:      # fixedQdot: the first maximum of positive qdot
        jc, qmax = 0, 0.0
        for j in range(N):
            if qdot[j] > qmax:
                qmax, jc = qdot[j], j
    elif bc == 2:      # stagnationPoint: the sign change of V nearest the old x_vzero
        if x[jj] > fl.x_vzero:
            js = next(j for j in range(N) if x[j] > fl.x_vzero)
        else:
            js = jj
        jc = js
        i = 1
        while js + i <= jj or js >= i:
            if js + i <= jj and _sign(V[js + i]) != _sign(V[js]):
                jc = js + i
                break
            if js >= i and _sign(V[js - i]) != _sign(V[js]):
                jc = js - i + 1
                break
            i += 1
        if jc == 0:
            fl.x_vzero = x[0] - V[0] * (x[1] - x[0]) / (V[1] - V[0])
        elif jc == jj:
            fl.x_vzero = x[jj] - V[jj] * (x[jj] - x[jj - 1]) / (V[jj] - V[jj - 1])
        else:
            fl.x_vzero = x[jc] - V[jc] * (x[jc] - x[jc - 1]) / (V[jc] - V[jc - 1])
    else:              # fixedTemperature: the first crossing of the mid temperature
        Tmid = 0.5 * (max(T) + min(T))
        jc = 0
        for j in range(1, N):
            if (T[j] - Tmid) * (T[j - 1] - Tmid) <= 0:
                jc = j
                break
    fl.j_cont = jc
    if bc in (1, 3):
        fl.rv_cont = float(rV[jc])


def split_constants(ddt_diff, ddt_prod, cross, balanced, ddt_conv=None):
    """SplitSolver::step's split constants (src/splitSolver.cpp:38-46):
    (sc_diff, sc_prod, sc_conv). Without convection (ddt_conv None) the
    two-operator balanced constants of the device split step; with it the
    reference's three-operator ones. sc_conv is None without convection."""
    if ddt_conv is not None:
        if balanced:
            sc_diff = 0.25 * (((ddt_prod + ddt_conv) + cross) - 3.0 * ddt_diff)
            sc_conv = 0.25 * (((ddt_prod + ddt_diff) + cross) - 3.0 * ddt_conv)
            sc_prod = 0.5 * (((ddt_conv + ddt_diff) + cross) - ddt_prod)
        else:
            sc_diff = cross.copy()
            sc_conv = np.zeros_like(cross)
            sc_prod = np.zeros_like(cross)
        return sc_diff, sc_prod, sc_conv
    if balanced:
        return 0.5 * ((ddt_prod + cross) - ddt_diff), 0.5 * ((ddt_diff + cross) - ddt_prod), None
    return cross.copy(), np.zeros_like(cross), None


def split_steps(omech, grids, state, t, B, D, dt, n_steps, method, opts, ddt_cross=None, balanced=True,
                mult=10.0, ddt=None, transport=None, convection=None, props_out=None):
    """n_steps split steps of a batch of flames. state: point-major [n_pts, n]
    (copied); B, D: variable-major per flame (flat). transport: None, or
    (TransportData, threshold, cross_terms): B, D (and the cross terms) are
    then recomputed from the state at the start of every step
    (step_properties). convection: None, or (flames, y_left, options) of
    the convection stage (ConvectionFlame-like objects, [n_flames, S], a
    ConvectionOptions): the step is then D C D S D C D. ddt: None, or the
    time derivatives (ddt_diff, ddt_prod[, ddt_conv]) of the previous step.
    Returns (state, t,
    ddt_diff, ddt_prod, source_status_of_last_step); with a transport model
    the last step's properties go into props_out (a dict) when given."""
    state = np.array(state, dtype=np.float64, copy=True)
    n_pts, n = state.shape
    offs = np.cumsum([0] + [g.n_points for g in grids])
    voffs = offs * n
    xs = np.concatenate([np.asarray(g.x, dtype=np.float64) for g in grids])
    cross = np.zeros_like(state) if ddt_cross is None else np.asarray(ddt_cross, dtype=np.float64).reshape(n_pts, n)
    ddt_diff = np.zeros_like(state) if ddt is None else ddt[0].copy()
    ddt_prod = np.zeros_like(state) if ddt is None else ddt[1].copy()
    ddt_conv = np.zeros_like(state) if ddt is None or len(ddt) < 3 or ddt[2] is None else ddt[2].copy()
    W = np.asarray(omech.mech.mol_weight, dtype=np.float64)
    status = None
    if convection is not None:
        import copy
        # the flames' continuity points move every step after the first
        # (continuity_point); the caller's objects are left as given
        convection = ([copy.copy(f) for f in convection[0]],) + tuple(convection[1:])
        last_eval = [None] * len(grids)
    for step_no in range(n_steps):
        if transport is not None:
            tdata, thr, with_cross = transport
            B, D, c = step_properties(omech, tdata, grids, state, opts.pressure, thr, mult, dt, with_cross,
                                      props_out)
            if with_cross:
                cross = c
        if convection is not None:
            from oracle import convection as oconv
            drhodt = oconv.density_derivative(state, W, opts.pressure, ddt_conv, ddt_diff, ddt_prod, cross, balanced)
            if step_no > 0:
                qdot = None
                if any(f.continuity_bc == 3 for f in convection[0]):
                    qdot, _, _ = objectives(omech, grids, state, opts.pressure, opts.kinetics_model)
                for f, g in enumerate(grids):
                    a, b = offs[f], offs[f + 1]
                    ev = last_eval[f]
                    continuity_point(convection[0][f], xs[a:b], state[a:b, 1],
                                     None if qdot is None else qdot[a:b], ev["V"], ev["rV"])
        sc_diff, sc_prod, sc_conv = split_constants(ddt_diff, ddt_prod, cross, balanced,
                                                    ddt_conv if convection is not None else None)
        delta = np.zeros_like(state)
        delta_conv = np.zeros_like(state)

        def convection_stage(f0, f1):
            from oracle import convection as oconv
            cflames, y_left, copts = convection
            t0 = t if f0 == 0.0 else t + f0 * dt
            t1 = t + f1 * dt
            for f, g in enumerate(grids):
                a, b = offs[f], offs[f + 1]
                y0 = state[a:b].T.copy()
                last_eval[f] = {}
                y1, _, _, _, _ = oconv.convection_flame(cflames[f], W, xs[a:b], y_left[f], drhodt[a:b],
                                                        sc_conv[a:b].T.copy().reshape(-1), y0.reshape(-1), t0, t1,
                                                        copts, last=last_eval[f])
                y1 = y1.reshape(y0.shape)
                delta_conv[a:b] = delta_conv[a:b] + (y1 - y0).T
                state[a:b] = y1.T

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
        if convection is not None:
            convection_stage(0.0, 0.5)
        diffusion(0.25, 0.5)
        xD2 = state.copy()
        dtp = np.full(n_pts, (t + dt) - t)
        out, status, _ = omech.integrate(method, state, dtp, opts, split_const=sc_prod, t_start=t, x=xs)
        state[:] = out
        xS = state.copy()
        diffusion(0.5, 0.75)
        if convection is not None:
            convection_stage(0.5, 1.0)
        diffusion(0.75, 1.0)
        ddt_diff = delta / dt - sc_diff
        ddt_prod = (xS - xD2) / dt - sc_prod
        if convection is not None:
            ddt_conv = delta_conv / dt - sc_conv
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


def objectives(omech, grids, state, pressure, kinetics_model, rho_u=None, ju=None, jb=None, cp=None):
    """(qdot, heat release per flame, consumption speed per flame or None).
    The consumption speed divides qdot by cp: that of the last property
    update when given (FlameSolver's cp array, src/flameSolver.cpp:956-961),
    else the current state's."""
    from ember_gb300.source import STATE_NORMALIZED
    g = omech.gas_eval(state[:, 1], state[:, 2:], pressure=pressure, model=kinetics_model, mode=STATE_NORMALIZED)
    qdot = -_seq_sum(g["net"] * g["hk"], axis=1)
    qcp = qdot / (g["cp_mass"] if cp is None else np.asarray(cp, dtype=np.float64))
    offs = np.cumsum([0] + [gr.n_points for gr in grids])
    hr = np.array([spline_integral(gr.x, qdot[offs[f]:offs[f + 1]]) for f, gr in enumerate(grids)])
    cs = None
    if rho_u is not None:
        cs = np.empty(len(grids))
        for f, gr in enumerate(grids):
            T = state[offs[f]:offs[f + 1], 1]
            cs[f] = spline_integral(gr.x, qcp[offs[f]:offs[f + 1]]) / (rho_u[f] * (T[jb[f]] - T[ju[f]]))
    return qdot, hr, cs
