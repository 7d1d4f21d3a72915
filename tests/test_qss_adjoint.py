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


@pytest.mark.gpu
@pytest.mark.parametrize("kinetics,iterations", [(KINETICS_STANDARD, 1), (KINETICS_INTERP, 1), (KINETICS_STANDARD, 2)])
def test_gpu_qss_adjoint_matches_the_oracle_adjoint(gpu_lib, kinetics, iterations):
    # the device adjoint (its forward replay and its backward pass) against
    # the CPU restatement, with split constants and the igniter on; also with
    # two corrector iterations per attempt (qss_iteration_count)
    from oracle import chem
    from ember_gb300.source import GpuMechanism, integrate_production_terms, source_adjoint
    mech, st, dt, opts, bar = _case(kinetics, n=8, seed=12)
    opts.qss_iteration_count = iterations
    opts.ignition_energy, opts.ignition_duration, opts.ignition_stddev = 2e6, 1.0, 5e-4
    rng = np.random.default_rng(3)
    sc = rng.normal(scale=1e-2, size=st.shape) * np.abs(st).clip(1e-3)
    sc[:, 1] = rng.normal(scale=2e3, size=len(st))
    x = rng.uniform(-1e-3, 1e-3, size=len(st))
    gm = GpuMechanism(mech)
    out, status, g_state, g_lnk = source_adjoint(gm, st, dt, opts, bar, split_const=sc, x=x, method=QSS)
    om = chem.OracleMech(mech)
    ref_out, ref_g, ref_p, ref_status, _ = chem.qss_adjoint(om, st, dt, opts, bar, split_const=sc, x=x)
    assert (status == 0).all() and (ref_status == 0).all()
    assert np.array_equal(out, ref_out)                  # the replayed forward pass is the integrator's
    fwd, fstatus, _ = integrate_production_terms(gm, QSS, st, dt, opts, split_const=sc, x=x)
    assert np.array_equal(out, np.asarray(fwd))
    np.testing.assert_allclose(g_state, ref_g, rtol=1e-9, atol=1e-12 * np.abs(ref_g).max())
    ref_lnk = ref_p.sum(axis=0)
    np.testing.assert_allclose(g_lnk, ref_lnk, rtol=1e-9, atol=1e-12 * np.abs(ref_lnk).max())
    # a forward record too short for any point (16 step starts): the adjoint
    # integrates every point again itself, with the same result
    out2, status2, g2, l2 = source_adjoint(gm, st, dt, opts, bar, split_const=sc, x=x, method=QSS, tape_cap=16)
    assert (status2 == 0).all()
    assert np.array_equal(out2, out)
    np.testing.assert_allclose(g2, ref_g, rtol=1e-9, atol=1e-12 * np.abs(ref_g).max())
    np.testing.assert_allclose(l2, ref_lnk, rtol=1e-9, atol=1e-12 * np.abs(ref_lnk).max())


@pytest.mark.gpu
def test_split_step_qss_gradients_match_central_differences_of_the_oracle(gpu_lib):
    # Heat release and consumption speed after one balanced D-S-D split step
    # with the QSS source at its default options (serial diffusion): the
    # discrete adjoint of the step through torch.autograd against central
    # differences of the oracle's step, perturbations 1e-6.
    torch = pytest.importorskip("torch")
    from oracle import split as osplit
    from oracle.chem import OracleMech
    from ember_gb300 import _lib as L
    from ember_gb300.autograd import split_step_objectives
    from ember_gb300.source import GpuMechanism
    from ember_gb300.split import FlameBatchSplitSolver, flame_batch
    mech = synthetic_mechanism(n_species=20, n_reactions=60, seed=3)
    grids, state, B, D, rho_u, ju, jb = flame_batch(mech, n_flames=2, n_min=10, n_max=12, seed=5, width=2e-3,
                                                    thickness=3e-4, T_b=1500.0)
    opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD)
    dt = 1e-6
    gm = GpuMechanism(mech)
    solver = FlameBatchSplitSolver(gm, grids, dt, method=QSS, source_options=opts,
                                   diffusion_algorithm=L.DIFFUSION_SERIAL)
    solver.set_transport(B, D)
    R = mech.n_reactions
    s0 = torch.tensor(state, dtype=torch.float64, requires_grad=True)
    lk = torch.zeros(R, dtype=torch.float64, requires_grad=True)
    out = split_step_objectives(solver, s0, lk, 0.0, rho_u, ju, jb, 4096)
    w = torch.tensor([1.0, -0.5, 2e3, 1e3], dtype=torch.float64)  # Q_0, Q_1, S_c,0, S_c,1
    (out * w).sum().backward()
    g_state = s0.grad.numpy()
    g_lnk = lk.grad.numpy()
    om = OracleMech(mech)

    def J(st, mult=None):
        om.set_multipliers(mult)
        y, *_ = osplit.split_steps(om, grids, st, 0.0, B, D, dt, 1, QSS, opts)
        _, hr, cs = osplit.objectives(om, grids, y, opts.pressure, opts.kinetics_model, rho_u, ju, jb)
        return float(np.dot(w.numpy(), np.concatenate([hr, cs])))

    om.set_multipliers(None)
    y_ref, *_ = osplit.split_steps(om, grids, state, 0.0, B, D, dt, 1, QSS, opts)
    _, hr_ref, cs_ref = osplit.objectives(om, grids, y_ref, opts.pressure, opts.kinetics_model, rho_u, ju, jb)
    assert np.array_equal(out.detach().numpy(), np.concatenate([hr_ref, cs_ref]))
    n0 = grids[0].n_points
    for (p, k) in [(3, 1), (n0 + 5, 1), (4, 2), (n0 + 6, 3), (2, 4), (n0 - 2, 5)]:
        assert state[p, k] > 1e-6
        hstep = 1e-6 * abs(state[p, k])
        e = np.zeros_like(state)
        e[p, k] = hstep
        fd = (J(state + e) - J(state - e)) / (2 * hstep)
        assert abs(g_state[p, k] - fd) <= 1e-4 * abs(fd) + 1e-9 * np.abs(g_state).max(), (p, k, g_state[p, k], fd)
    rng = np.random.default_rng(5)
    for i in list(np.argsort(-np.abs(g_lnk))[:3]) + list(rng.choice(R, 3, replace=False)):
        mp, mm = np.ones(R), np.ones(R)
        mp[i], mm[i] = np.exp(1e-6), np.exp(-1e-6)
        fd = (J(state, mp) - J(state, mm)) / 2e-6
        assert abs(g_lnk[i] - fd) <= 1e-4 * abs(fd) + 1e-7 * np.abs(g_lnk).max(), (i, g_lnk[i], fd)
    om.set_multipliers(None)


@pytest.mark.gpu
def test_gpu_qss_adjoint_at_the_c4_size(gpu_lib):
    # The C4 sizes: the 400-point flame profile of the 53-species / 325-reaction
    # mechanism, one 2e-5 s source stage at the default options (interpolated
    # kinetics), 150 QSS steps per point on average and 475 at most. The device
    # adjoint against the oracle's. (Central differences are no check at this
    # size: with 400 points a perturbation of 1e-6 already flips some accept /
    # reject decisions, and the quotients of the large gradients vary by tens of
    # per cent between steps of 1e-4, 1e-5 and 1e-6.)
    from oracle import chem
    from ember_gb300.source import GpuMechanism, source_adjoint
    from ember_gb300.split import flame_batch
    mech = synthetic_mechanism(n_species=53, n_reactions=325, seed=53325)
    grids, state, B, D, rho_u, ju, jb = flame_batch(mech, n_flames=1, n_min=400, n_max=400, seed=4000)
    opts = SourceOptions.defaults()
    rng = np.random.default_rng(7)
    bar = rng.normal(size=state.shape)
    bar[:, 1] *= 1e-3
    gm = GpuMechanism(mech)
    out, status, g_state, g_lnk = source_adjoint(gm, state, 2e-5, opts, bar, method=QSS)
    om = chem.OracleMech(mech)
    ref_out, ref_g, ref_p, ref_status, steps = chem.qss_adjoint(om, state, 2e-5, opts, bar)
    assert (status == 0).all() and (ref_status == 0).all()
    assert steps.max() > 300
    assert np.array_equal(out, ref_out)
    np.testing.assert_allclose(g_state, ref_g, rtol=1e-9, atol=1e-12 * np.abs(ref_g).max())
    ref_lnk = ref_p.sum(axis=0)
    np.testing.assert_allclose(g_lnk, ref_lnk, rtol=1e-9, atol=1e-12 * np.abs(ref_lnk).max())
