"""Algorithmic work model of the hot-path kernels (roofline numerators).

Counts each +, -, *, /, exp, log and pow as one flop, over the formulas the
reference evaluates, so the figures do not depend on how the GPU code is
written. Per-point call counts come from the integrator statistics (steps and
right-hand-side calls), which are identical on the GPU and in the CPU oracle.
"""
from __future__ import annotations

import numpy as np

from .mechanism import Mechanism, RXN_ELEMENTARY, RXN_THREE_BODY, RXN_TROE


def _occurrences(mech: Mechanism):
    nr = (mech.reactants >= 0).sum(axis=1)
    npr = (mech.products >= 0).sum(axis=1)
    return nr, npr


def rhs_flops(mech: Mechanism, kinetics_model: int):
    """(flops of the temperature-dependent part, flops of the
    composition-dependent part) of one source-term right-hand side."""
    S = mech.n_species
    nr, npr = _occurrences(mech)
    ty = mech.rxn_type
    n_eff = np.diff(mech.efficiency_offsets)
    falloff = (ty == 2) | (ty == 3)
    # thermo per species: cp/R 8, h/RT 10, s/R 9, g 1
    f_T = 28 * S + 3  # + log T, 1/T, log(RT/p0)
    arr = ~falloff
    if kinetics_model == 0:
        f_T += int(np.sum(np.where(arr, 5, 0)))                             # A exp(b lnT - Ea/(RT))
        f_T += int(np.sum(np.where(mech.reversible != 0, nr + npr + 4, 0)))  # dG, exp, cap
    else:
        f_T += int(np.sum(np.where(arr, 2, 0)))                             # table lookups
        f_T += int(np.sum(np.where(mech.reversible != 0, 2, 0)))
        f_T += 4                                                            # table index
    # composition: clip/normalise 4/species, concentration 1, mean weight 1
    f_c = 6 * S + 4
    f_rop = np.zeros(mech.n_reactions)
    f_rop += np.where(ty != RXN_ELEMENTARY, 1 + 2 * n_eff, 0)               # [M]
    f_rop += np.where(falloff, 10 + 5, 0)                                   # k0, kinf, Pr, blend
    f_rop += np.where(ty == RXN_TROE, 24, 0)                                # Fcent, F
    f_rop += 1 + np.where(ty == RXN_THREE_BODY, 1, 0)                        # multiplier, [M]
    f_rop += nr + np.where(mech.reversible != 0, npr + 1, 0)                # mass action
    f_acc = 2 * int(np.sum(nr + npr))                                       # creation + destruction
    f_src = 8 * S + 4                                                       # q, d, qdot, cp
    return float(f_T), float(f_c + f_rop.sum() + f_acc + f_src)


def qss_point_flops(mech: Mechanism, kinetics_model: int, steps, rhs_calls):
    """Flops of QSS integrations given per-point step and RHS-call counts:
    every step re-evaluates the temperature-dependent part once (predictor
    call); every call evaluates the composition part; the integrator does
    about 40 flops per component per call (Pade predictor, corrector, error
    test)."""
    f_T, f_rhs = rhs_flops(mech, kinetics_model)
    n = mech.n_vars
    steps = np.asarray(steps, dtype=float)
    calls = np.asarray(rhs_calls, dtype=float)
    return steps * f_T + calls * (f_rhs + 40.0 * n)


def bdf_point_flops(mech: Mechanism, kinetics_model: int, steps, rhs_calls, jacobians):
    """Flops of BDF (CVODE-path) integrations given per-point counts of steps,
    right-hand-side calls and Jacobian evaluations. Every call evaluates the
    whole right-hand side (temperature changes between Newton iterations) and
    is followed by one Newton correction (solve with the LU factors, 2 n^2,
    plus about 12 n for the update, weights and norms); every Jacobian costs
    the analytic species part (per reaction, the derivatives of the rate of
    progress with respect to each participating species and the third-body
    sum, scattered to every participating species), the finite-difference
    temperature column (one right-hand side, not in the call count), the
    iteration matrix I - gamma J (n^2) and its LU factorisation (2 n^3 / 3).
    A lower bound: factorisations that reuse a Jacobian after a step-size
    change are not counted."""
    f_T, f_rhs = rhs_flops(mech, kinetics_model)
    n = float(mech.n_vars)
    nr, npr = _occurrences(mech)
    n_eff = np.diff(mech.efficiency_offsets)
    occ = (nr + npr).astype(float)
    f_jac_species = float(np.sum(2.0 * occ * occ + 2.0 * n_eff * occ))
    f_jac = f_jac_species + (f_T + f_rhs) + n * n + 2.0 * n ** 3 / 3.0
    steps = np.asarray(steps, dtype=float)
    calls = np.asarray(rhs_calls, dtype=float)
    jac = np.asarray(jacobians, dtype=float)
    return calls * (f_T + f_rhs + 2.0 * n * n + 12.0 * n) + jac * f_jac + steps * 20.0 * n


# DRAM bytes of one k_source_qss launch per integrated point, from the ncu
# capture of the 4096-point step at 64 threads per point (dram__bytes_read.sum
# 8,559,872 + dram__bytes_write.sum 823,552 bytes): state in and out plus the
# per-CTA rate-constant cache.
QSS_DRAM_BYTES_PER_POINT = (8559872 + 823552) / 4096
# The same for k_source_bdf with 152 variables, from the capture of 608 points
# at 128 threads (5,883,392 + 14,031,104 bytes): the LU factors in shared
# memory, the Jacobian, rates of progress and saved Nordsieck array in a
# global slice.
BDF_DRAM_BYTES_PER_POINT = (5883392 + 14031104) / 608


def tridiag_flops_per_point() -> float:
    """Diffusion system per point for one BDF1x8 step: matrix rows ~12,
    factorisation ~5, 8 sub-steps x (2 right-hand side + 3 forward + 2 back)."""
    return 12.0 + 5.0 + 8 * 7.0


def transport_point_flops(n_species: int, n_major=None, cross_terms: bool = True):
    """Thermo, "Approx" transport and cross terms of one grid point
    (ember_transport_eval / the split step's property update) with n_major
    species at or above the threshold (default: all; scalar or array): per
    species the NASA7 cp and h (~20) and three fits (3 x 11); per major pair
    the Wilke term (~10); per pair of the mixture diffusion sums (a major
    species with every other, a minor one with the major ones) the binary
    diffusion fit and the two sums (~15); the cross terms ~20 per species
    (Fick flux twice, species and heat-capacity terms)."""
    S = float(n_species)
    K = S if n_major is None else np.asarray(n_major, dtype=float)
    pairs = K * (S - 1.0) + (S - K) * K
    return 53.0 * S + 10.0 * K * K + 15.0 * pairs + (20.0 * S if cross_terms else 0.0)


def tridiag_bytes_per_point() -> float:
    """B, D, split constant and y read, y written (8 bytes each)."""
    return 40.0


def convection_flame_flops(n_points, stats):
    """Flops of one convection stage per flame from its counters (stats rows:
    UTW steps, UTW right-hand sides, species steps and right-hand sides
    summed over species). A UTW right-hand side costs about 30 flops per point
    (density, continuity increment, V, three upwinded differences and the
    three derivatives with the strain term), a species one about 8 (the
    interpolated v, one upwinded difference, the derivative); an Adams step
    about 35 per value (prediction, on average 1.5 Newton corrections with
    their norms, the Nordsieck update, weights, the error and order tests)."""
    N = np.asarray(n_points, dtype=float)
    st = np.asarray(stats, dtype=float).reshape(-1, 4)
    return st[:, 1] * 30.0 * N + st[:, 0] * 35.0 * 3.0 * N + st[:, 3] * 8.0 * N + st[:, 2] * 35.0 * N


# (name, op, chains, warps per SM, active lanes) of the FP64 issue probe
FP64_ISSUE_CASES = (
    ("DFMA latency, 1 warp", 0, 1, 1, 32),
    ("DFMA latency, 1 warp, 1 lane", 0, 1, 1, 1),
    ("DADD latency, 1 warp", 1, 1, 1, 32),
    ("DMUL latency, 1 warp", 2, 1, 1, 32),
    ("division latency, 1 warp", 3, 1, 1, 32),
    ("DFMA issue, 1 warp/SM", 0, 8, 1, 32),
    ("DFMA issue, 2 warps/SM", 0, 8, 2, 32),
    ("DFMA issue, 4 warps/SM", 0, 8, 4, 32),
    ("DFMA issue, 8 warps/SM", 0, 8, 8, 32),
    ("DFMA issue, 16 warps/SM", 0, 8, 16, 32),
    ("DFMA issue, 8 warps/SM, 1 lane", 0, 8, 8, 1),
    ("DFMA issue, 8 warps/SM, 8 lanes", 0, 8, 8, 8),
    ("DFMA issue, 8 warps/SM, 16 lanes", 0, 8, 8, 16),
    ("DADD issue, 8 warps/SM", 1, 8, 8, 32),
    ("DMUL issue, 8 warps/SM", 2, 8, 8, 32),
    ("division issue, 8 warps/SM", 3, 8, 8, 32),
    ("fmax + DADD issue, 8 warps/SM", 4, 8, 8, 32),
    ("compare-select + DADD issue, 8 warps/SM", 5, 8, 8, 32),
    ("reciprocal 1.0/x latency, 1 warp", 6, 1, 1, 32),
    ("reciprocal __drcp_rn latency, 1 warp", 7, 1, 1, 32),
    ("reciprocal 1.0/x issue, 8 warps/SM", 6, 8, 8, 32),
    ("reciprocal __drcp_rn issue, 8 warps/SM", 7, 8, 8, 32),
)


def fp64_issue_table():
    """ember_probe_fp64_issue over FP64_ISSUE_CASES on the current device:
    [(name, warps per SM, active lanes, cycles per instruction per warp,
    SM cycles per warp instruction, FP64 lane operations per SM cycle)]."""
    import ctypes as C
    from . import _lib as L
    rows = []
    for name, op, chains, warps, lanes in FP64_ISSUE_CASES:
        c = C.c_double()
        L.check(L.lib().ember_probe_fp64_issue(op, chains, warps, lanes, C.byref(c)), "probe")
        per_sm = c.value / warps
        rows.append((name, warps, lanes, c.value, per_sm, lanes / per_sm))
    return rows


if __name__ == "__main__":
    print(f"{'case':36s} {'warps':>5s} {'lanes':>5s} {'cyc/inst/warp':>13s} {'SM cyc/inst':>11s} {'lane ops/SM cyc':>15s}")
    for name, w, ln, c, s, r in fp64_issue_table():
        print(f"{name:36s} {w:5d} {ln:5d} {c:13.1f} {s:11.2f} {r:15.3f}")
