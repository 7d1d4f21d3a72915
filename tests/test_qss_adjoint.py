"""Gradients of the QSS source-term integration (the reference's default
integrator, QssIntegrator with SourceSystemQSS).

The discrete adjoint differentiates the integrator exactly as it runs: every
attempt of every step (a retried attempt starts from the rejected one's last
corrector rates) and the step sizes as functions of the state (initial step
size, the error-estimate rule, the clip to the end time). With the step-size
decisions differentiated, central differences of the adaptive forward map
agree with it to the level of their own rounding noise at the reference's
default epsmin = 0.02, with perturbations of 1e-6.

CPU: the oracle's adjoint (oracle/oracle_qss_adjoint.c) against central
differences of the oracle's forward integration. GPU: the device adjoint
(ember_source_adjoint_qss) against the oracle's adjoint on the same inputs.
"""
import numpy as np
import pytest

from ember_gb300.mechanism import reactor_states, synthetic_mechanism
from ember_gb300.source import KINETICS_INTERP, KINETICS_STANDARD, QSS, SourceOptions


def _case(kinetics=KINETICS_STANDARD, n=3, seed=11):
    mech = synthetic_mechanism(n_species=20, n_reactions=60, seed=3)
    st, dt = reactor_states(mech, n, seed=seed, T_range=(1100.0, 1600.0), dt_range=(2e-5, 5e-5))
    opts = SourceOptions.defaults(kinetics_model=kinetics)
    rng = np.random.default_rng(1)
    bar = rng.normal(size=st.shape)
    bar[:, 0] = 0.0
    bar[:, 1] *= 1e-3
    return mech, st, dt, opts, bar


def test_oracle_qss_adjoint_matches_central_differences():
    from oracle import chem
    mech, st, dt, opts, bar = _case()
    om = chem.OracleMech(mech)
    out, g_state, g_pts, status, steps = chem.qss_adjoint(om, st, dt, opts, bar, n_threads=1)
    ref, ref_status, ref_stats = om.integrate(QSS, st, dt, opts, n_threads=1)
    assert (status == 0).all() and (ref_status == 0).all()
    assert np.array_equal(out, ref)                     # the adjoint's forward pass is the integrator's
    assert np.array_equal(steps, ref_stats[:, 0])
    assert steps.min() > 300                            # many steps, with rejected attempts among them
    assert ref_stats[:, 2].sum() > 0

    def phi(s, mult=None):
        om.set_multipliers(mult)
        o, stt, _ = om.integrate(QSS, s, dt, opts, n_threads=1)
        assert (stt == 0).all()
        return float((bar * o).sum())

    # state entries (T and mass fractions present in the mixture; entries at
    # zero sit on the setState clip, where the derivative is one-sided)
    for (j, k) in [(0, 1), (1, 1), (2, 1), (0, 2), (1, 3), (2, 4), (0, 6)]:
        assert st[j, k] > 0
        h = 1e-6 * abs(st[j, k])
        e = np.zeros_like(st)
        e[j, k] = h
        fd = (phi(st + e) - phi(st - e)) / (2 * h)
        assert abs(g_state[j, k] - fd) <= 1e-5 * abs(fd), (j, k, g_state[j, k], fd)
    g = g_pts.sum(axis=0)
    R = mech.n_reactions
    rng = np.random.default_rng(7)
    picks = list(np.argsort(-np.abs(g))[:3]) + list(rng.choice(R, 3, replace=False))
    for i in picks:
        mp, mm = np.ones(R), np.ones(R)
        mp[i], mm[i] = np.exp(1e-6), np.exp(-1e-6)
        fd = (phi(st, mp) - phi(st, mm)) / 2e-6
        assert abs(g[i] - fd) <= 1e-5 * abs(fd) + 1e-7 * np.abs(g).max(), (i, g[i], fd)
    om.set_multipliers(None)
