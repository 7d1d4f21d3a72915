"""FlameBatchRun: FlameSolver's step loop for a batch (termination test,
regrid, re-batching). CPU: the termination test against a literal
restatement of checkTerminationCondition; GPU: a short run of two flames with
regrids and terminations."""
import math

import numpy as np
import pytest

from ember_gb300.sweep import TerminationOptions, heat_release_steady


def _reference_check(t, q, t_now, o):
    """checkTerminationCondition, "Q" (src/flameSolver.cpp:377-412), as loops."""
    if t_now < o.t_min:
        return False
    j1 = None
    for j in range(len(t)):
        if t[j] < t_now - o.steady_period:
            j1 = j
    if j1 is None:
        return False
    j2 = len(t) - 1
    mean = sum(q[j1:j2 + 1]) / (j2 - j1 + 1)
    err = math.sqrt(sum((q[j] - mean) ** 2 for j in range(j1, j2 + 1))) / (j2 - j1 + 1)
    return err / abs(mean) < o.tolerance or err < o.abstol


def test_termination_test_matches_the_reference_loop():
    rng = np.random.default_rng(3)
    o = TerminationOptions(tolerance=1e-3, abstol=1e-9, steady_period=1e-3, t_min=2e-4)
    for trial in range(200):
        n = int(rng.integers(1, 60))
        t = np.cumsum(rng.uniform(1e-5, 1e-4, n))
        q = 1e6 * (1 + rng.normal(scale=10 ** rng.uniform(-6, -1), size=n))
        t_now = t[-1]
        got = heat_release_steady(t, q, t_now, o)[0]
        assert got == _reference_check(list(t), list(q), t_now, o), trial
    # shorter than the steady period: never terminates
    assert heat_release_steady([0.0, 1e-4], [1.0, 1.0], 1e-4, o) == (False, None, None)
    # a constant heat release rate over more than the period terminates
    t = np.linspace(0, 3e-3, 31)
    assert heat_release_steady(t, np.full(31, 5e5), t[-1], o)[0]


@pytest.mark.gpu
@pytest.mark.parametrize("with_convection", [False, True])
def test_batch_run_regrids_and_terminates(gpu_lib, with_convection):
    from ember_gb300 import _lib as L
    from ember_gb300.convection import ConvectionFlame, ConvectionOptions, mean_molecular_weight
    from ember_gb300.mechanism import synthetic_mechanism
    from ember_gb300.source import GpuMechanism, KINETICS_STANDARD, QSS, SourceOptions
    from ember_gb300.split import flame_batch, mixture_properties
    from ember_gb300.sweep import FlameBatchRun
    from ember_gb300.transport import GpuTransport, synthetic_transport
    mech = synthetic_mechanism(n_species=20, n_reactions=60, seed=3)
    td = synthetic_transport(mech, seed=4)
    grids, state, B, D, rho_u, ju, jb = flame_batch(mech, n_flames=2, n_min=30, n_max=50, seed=5, width=2e-3,
                                                    thickness=3e-4)
    dt = 5e-7
    conv = None
    if with_convection:
        rho, _ = mixture_properties(mech, state)
        flames, y_left, p = [], [], 0
        for f, g in enumerate(grids):
            N = g.n_points
            a = 200.0 + 100.0 * f
            state[p:p + N, 0] = a * np.sqrt(rho_u[f] / rho[p:p + N])
            y0 = state[p, 2:].copy()
            flames.append(ConvectionFlame(n_points=N, left_bc=g.left_bc, right_bc=g.right_bc, alpha=g.alpha,
                                          rv_zero=0.4 * rho_u[f], t_left=float(state[p, 1]),
                                          w_left=float(mean_molecular_weight(y0, mech.mol_weight)[0]),
                                          rhou=float(rho_u[f]), strain_initial=a, strain_final=a))
            y_left.append(y0)
            p += N
        conv = (flames, np.array(y_left), ConvectionOptions())
    gm = GpuMechanism(mech)
    gt = GpuTransport(gm, td)
    # No tolerance at first (nothing terminates), regrids every second step.
    # The seeded profiles are not converged flames. With the convection stage
    # attached, their first step after a regrid stays bounded, but the
    # convection systems of a flame fail within two steps of the second regrid
    # (the oracle, stepped through the same sequence of split steps and
    # regrids, fails in the same steps). The convection variant therefore
    # regrids once and terminates at the step after it.
    n_first = 2 if with_convection else 4
    term = TerminationOptions(tolerance=0.0, abstol=0.0, steady_period=(1.5 if with_convection else 4.0) * dt,
                              terminate_step_interval=3, regrid_step_interval=2)
    run = FlameBatchRun(gm, gt, grids, state, dt, rho_u, method=QSS,
                        source_options=SourceOptions.defaults(kinetics_model=KINETICS_STANDARD),
                        convection=conv, strain_rates=[200.0, 500.0], termination=term,
                        diffusion_algorithm=L.DIFFUSION_SERIAL)
    recs = run.run(n_first)
    assert run.n_steps == n_first and len(recs[0].t) == n_first
    assert run.n_rebuilds >= 1                      # the regrids changed the grids
    assert run.grids[0].n_points != grids[0].n_points or run.grids[1].n_points != grids[1].n_points
    # an absolute tolerance that any variation meets: both flames terminate at the next test
    run.termination.abstol = 1e30
    recs = run.run(6)
    assert all(r.terminated for r in recs)          # both terminate at the next test
    assert recs[0].t_terminated == recs[1].t_terminated
    for r in recs:
        assert np.isfinite(r.Q).all() and np.isfinite(r.Sc).all()
        assert r.t == sorted(r.t)
