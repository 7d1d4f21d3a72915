"""CPU ORACLE -- test infrastructure only.

Extended-precision (numpy longdouble: 80-bit x87 on x86-64, IEEE binary128 on
AArch64) restatement of one diffusion stage, used to measure how close a
double-precision result is to the exact solution of the same discrete
problem. The matrix rows are formed exactly as DiffusionSystem::get_A /
get_k do (src/diffusionSystem.cpp:10-76), but in extended precision, so that
b = -(a + c) holds to ~1e-19 (in double it holds only to the rounding of the
largest coefficient, which can exceed the BDF shift on strongly refined
grids); the integration is TridiagonalIntegrator's first step of 8 BDF1
sub-steps and BDF2 later steps (src/integrator.cpp:133-204) with the step
count of Integrator::integrateToTime (src/integrator.cpp:37-47).
"""
from __future__ import annotations

import numpy as np

LD = np.longdouble


def diffusion_rows(x, B, D, split_const=None, alpha=0, left_bc=0, right_bc=0, wall_const=0.0, y_inf=0.0):
    """Rows (a, b, c, k) of one DiffusionSystem in extended precision."""
    x = np.asarray(x, dtype=LD)
    B = np.asarray(B, dtype=LD)
    D = np.asarray(D, dtype=LD)
    N = x.size
    a = np.zeros(N, dtype=LD)
    b = np.zeros(N, dtype=LD)
    c = np.zeros(N, dtype=LD)
    k = np.zeros(N, dtype=LD) if split_const is None else np.asarray(split_const, dtype=LD).copy()
    wc, yi = LD(wall_const), LD(y_inf)

    def rp(v):
        return LD(1) if alpha == 0 else v ** alpha

    def c1(j):
        if j < 1 or j > N - 2:
            return LD(0)
        return LD(0.5) * B[j] / (LD(0.5) * (x[j + 1] - x[j - 1]) * rp(x[j]))

    def c2(j):
        if j < 1 or j > N - 2:
            return LD(0)
        return rp(LD(0.5) * (x[j] + x[j + 1])) * (D[j] + D[j + 1]) / (x[j + 1] - x[j])

    j_start = 1
    if left_bc == 2:    # ControlVolume
        hh0 = x[1] - x[0]
        c0 = B[0] * (alpha + 1) * (D[0] + D[1]) / (2 * hh0 * hh0)
        b[0], c[0] = -c0, c0
    elif left_bc == 3:  # WallFlux
        hh0 = x[1] - x[0]
        c0 = B[0] * (alpha + 1) / hh0
        d = LD(0.5) * (D[0] + D[1])
        b[0], c[0] = -c0 * (d / hh0 + wc), d * c0 / hh0
        k[0] += c0 * wc * yi
    elif left_bc != 0:  # ZeroGradient and the rest
        j_start = 2
        b[1], c[1] = -c1(1) * c2(1), c1(1) * c2(1)
    if right_bc == 0:
        j_stop = N - 1
    else:
        j_stop = N - 2
        a[N - 2], b[N - 2] = c1(N - 2) * c2(N - 3), -c1(N - 2) * c2(N - 3)
    for j in range(j_start, j_stop):
        a[j], b[j], c[j] = c1(j) * c2(j - 1), -c1(j) * (c2(j - 1) + c2(j)), c1(j) * c2(j)
    return a, b, c, k


def tridiag_integrate(a, b, c, k, y0, t0, t1, h):
    """initialize(t0, h) then integrateToTime(t1) of one system, in extended
    precision (h is the double step the reference would use)."""
    a, b, c, k = (np.asarray(v, dtype=LD) for v in (a, b, c, k))
    y = np.asarray(y0, dtype=LD).copy()
    N = y.size
    q = (float(t1) - float(t0)) / float(h) + 1e-5
    n_steps = int(q) if q >= 1.0 else 1
    h = (LD(t1) - LD(t0)) / n_steps

    def factor(shift):
        luc = np.zeros(N, dtype=LD)
        inv = np.zeros(N, dtype=LD)
        inv[0] = 1 / (b[0] - shift)
        luc[0] = c[0] * inv[0]
        for i in range(1, N):
            inv[i] = 1 / ((b[i] - shift) - luc[i - 1] * a[i])
            luc[i] = c[i] * inv[i]
        return luc, inv

    def solve(r, luc, inv):
        d = np.empty(N, dtype=LD)
        d[0] = r[0] * inv[0]
        for i in range(1, N):
            d[i] = (r[i] - d[i - 1] * a[i]) * inv[i]
        for i in range(N - 2, -1, -1):
            d[i] = d[i] - luc[i] * d[i + 1]
        return d

    yprev = y.copy()
    h8 = h / 8
    luc, inv = factor(1 / h8)
    for _ in range(8):
        y = solve(-y / h8 - k, luc, inv)
    if n_steps > 1:
        luc, inv = factor(3 / (2 * h))
        for _ in range(1, n_steps):
            r = -2 * y / h + yprev / (2 * h) - k
            yprev = y
            y = solve(r, luc, inv)
    return y


def diffusion_system(x, B, D, y, t0, t1, h, split_const=None, alpha=0, left_bc=0, right_bc=0, wall_const=0.0,
                     y_inf=0.0):
    """One DiffusionSystem through one stage in extended precision; returns
    the state rounded to double."""
    a, b, c, k = diffusion_rows(x, B, D, split_const, alpha, left_bc, right_bc, wall_const, y_inf)
    return tridiag_integrate(a, b, c, k, y, t0, t1, h).astype(np.float64)
