"""Gradients: the discrete adjoint of the BDF source-term integration on the
GPU against central finite differences of the CPU restatement of the
reference's solver (the oracle), on stiff reactor states of a small
synthetic mechanism with tight tolerances.

Finite differences of an adaptive integrator carry noise from its step-size
decisions (about 1e-9 of the solution with these tolerances), so the
perturbations are 1e-4 of the state entry and 1e-3 in ln(multiplier)
(central differences), and the rate-multiplier checks use the reactions with
the largest gradients."""
import numpy as np
import pytest

from ember_gb300.mechanism import reactor_states, synthetic_mechanism
from ember_gb300.source import BDF, KINETICS_STANDARD, SourceOptions

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case():
    mech = synthetic_mechanism(n_species=20, n_reactions=60, seed=3)
    st, dt = reactor_states(mech, 3, seed=11, T_range=(1100.0, 1600.0), dt_range=(2e-5, 5e-5))
    opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD, bdf_reltol=1e-9, bdf_abstol_momentum=1e-9,
                                  bdf_abstol_energy=1e-9, bdf_abstol_species=1e-15)
    rng = np.random.default_rng(1)
    bar = rng.normal(size=st.shape)
    bar[:, 0] = 0.0
    bar[:, 1] *= 1e-3
    return mech, st, dt, opts, bar


def _phi(om, st, dt, opts, bar, mult=None):
    from ember_gb300.source import BDF as _BDF
    om.set_multipliers(mult)
    out, status, _ = om.integrate(_BDF, st, dt, opts, n_threads=1)
    assert (status == 0).all(), status
    return float((bar * out).sum())


def test_bdf_adjoint_matches_central_differences_of_the_oracle(gpu_lib, case):
    from oracle.chem import OracleMech
    from ember_gb300.source import GpuMechanism, source_adjoint
    mech, st, dt, opts, bar = case
    gm = GpuMechanism(mech)
    out, status, g_state, g_lnk = source_adjoint(gm, st, dt, opts, bar, tape_cap=4096)
    assert (status == 0).all(), status
    om = OracleMech(mech)
    ref_out, _, _ = om.integrate(BDF, st, dt, opts, n_threads=1)
    assert np.array_equal(out, ref_out)  # the taped forward pass is the ordinary one
    checked = 0
    for (j, k) in [(0, 1), (1, 1), (2, 1), (0, 2), (1, 3), (2, 4), (0, 6)]:
        hstep = 1e-4 * max(abs(st[j, k]), 1e-6)
        e = np.zeros_like(st)
        e[j, k] = hstep
        fd = (_phi(om, st + e, dt, opts, bar) - _phi(om, st - e, dt, opts, bar)) / (2 * hstep)
        assert abs(g_state[j, k] - fd) <= 1e-4 * abs(fd) + 1e-9, (j, k, g_state[j, k], fd)
        checked += 1
    R = mech.n_reactions
    rel = 1e-3
    for i in np.argsort(-np.abs(g_lnk))[:4]:
        mp, mm = np.ones(R), np.ones(R)
        mp[i], mm[i] = np.exp(rel), np.exp(-rel)
        fd = (_phi(om, st, dt, opts, bar, mp) - _phi(om, st, dt, opts, bar, mm)) / (2 * rel)
        assert abs(g_lnk[i] - fd) <= 1e-3 * abs(fd) + 1e-8, (i, g_lnk[i], fd)
        checked += 1
    om.set_multipliers(None)
    assert checked == 11


@pytest.mark.parametrize("explicit_h", [False, True])
def test_diffusion_adjoint_is_the_transpose_of_the_stage(gpu_lib, explicit_h):
    # The stage is linear in y (zero split constants, y_inf = 0): its matrix M
    # has columns M e_i (the serial stage applied to unit vectors), and the
    # adjoint must return M^T ybar, for every boundary condition and for both
    # the single BDF1 x 8 step and multi-step (BDF2) stages.
    from ember_gb300 import _lib as L
    from ember_gb300.diffusion import FlameGrid, diffusion_adjoint, integrate_diffusion_terms
    rng = np.random.default_rng(8 + explicit_h)
    grids = []
    for left, right, alpha in [(0, 0, 0), (1, 1, 1), (2, 4, 0), (3, 0, 1), (4, 4, 0)]:
        n = int(rng.integers(6, 14))
        x = np.cumsum(np.full(n, 2e-5) * np.exp(rng.uniform(-0.3, 0.3, n))) + (1e-4 if alpha else 0.0)
        grids.append(FlameGrid(x=x, left_bc=left, right_bc=right, alpha=alpha))
    n_vars = 2
    tot = sum(g.n_points for g in grids) * n_vars
    B = np.exp(rng.uniform(-1, 1, tot))
    D = np.exp(rng.uniform(np.log(1e-6), np.log(1e-4), tot))
    nsys = len(grids) * n_vars
    h = np.full(nsys, 2e-6) if explicit_h else None
    wall = rng.uniform(0.0, 3.0, nsys)
    ybar = rng.normal(size=tot)
    got, status = diffusion_adjoint(grids, B, D, ybar, 0.0, 1e-5, h=h, wall_const=wall)
    assert (status == 0).all()
    M = np.zeros((tot, tot))
    for i in range(tot):
        e = np.zeros(tot)
        e[i] = 1.0
        out, st = integrate_diffusion_terms(grids, B, D, np.zeros(tot), e, 0.0, 1e-5, h=h, wall_const=wall,
                                            algorithm=L.DIFFUSION_SERIAL)
        M[:, i] = out
    ref = M.T @ ybar
    np.testing.assert_allclose(got, ref, rtol=1e-11, atol=1e-12 * np.abs(ref).max())


def test_split_step_gradients_match_central_differences_of_the_oracle(gpu_lib):
    # Heat release and consumption speed after one balanced D-S-D split step
    # (BDF source, serial diffusion): gradients through torch.autograd (the
    # discrete adjoint of the step) against central differences of the CPU
    # restatement of the same step.
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
    opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD, bdf_reltol=1e-9, bdf_abstol_momentum=1e-9,
                                  bdf_abstol_energy=1e-9, bdf_abstol_species=1e-15)
    dt = 1e-6
    gm = GpuMechanism(mech)
    solver = FlameBatchSplitSolver(gm, grids, dt, method=BDF, source_options=opts,
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
        y, *_ = osplit.split_steps(om, grids, st, 0.0, B, D, dt, 1, BDF, opts)
        _, hr, cs = osplit.objectives(om, grids, y, opts.pressure, opts.kinetics_model, rho_u, ju, jb)
        return float(np.dot(w.numpy(), np.concatenate([hr, cs])))

    # the forward values are the oracle's (serial diffusion, bitwise source and objectives)
    om.set_multipliers(None)
    y_ref, *_ = osplit.split_steps(om, grids, state, 0.0, B, D, dt, 1, BDF, opts)
    _, hr_ref, cs_ref = osplit.objectives(om, grids, y_ref, opts.pressure, opts.kinetics_model, rho_u, ju, jb)
    assert np.array_equal(out.detach().numpy(), np.concatenate([hr_ref, cs_ref]))
    n0 = grids[0].n_points
    # state entries away from Y = 0, where the clipping of setState_TPY makes J one-sided.
    # Difference step 1e-3 of the entry: below it the adaptive integrator's
    # step-size decisions make the quotients noisy (for (4, 2): -8.0542e5,
    # -8.0549e5, -8.0447e5, -8.0706e5, -8.1672e5 at 1e-3, 3e-4, 1e-4, 3e-5,
    # 1e-5 of the entry), while at 1e-3 and 3e-4 they agree to 1e-4.
    for (p, k) in [(3, 1), (n0 + 5, 1), (4, 2), (n0 + 6, 3), (2, 4), (n0 - 2, 5)]:
        assert state[p, k] > 1e-6
        hstep = 1e-3 * max(abs(state[p, k]), 1e-6)
        e = np.zeros_like(state)
        e[p, k] = hstep
        fd = (J(state + e) - J(state - e)) / (2 * hstep)
        assert abs(g_state[p, k] - fd) <= 2e-3 * abs(fd) + 1e-9 * np.abs(g_state).max(), (p, k, g_state[p, k], fd)
    for i in np.argsort(-np.abs(g_lnk))[:3]:
        mp, mm = np.ones(R), np.ones(R)
        mp[i], mm[i] = np.exp(1e-3), np.exp(-1e-3)
        fd = (J(state, mp) - J(state, mm)) / 2e-3
        assert abs(g_lnk[i] - fd) <= 2e-3 * abs(fd), (i, g_lnk[i], fd)
    om.set_multipliers(None)


def test_split_step_adjoint_at_the_c4_size(gpu_lib):
    # The C4 configuration: one 400-point flame-like profile of the 53-species /
    # 325-reaction mechanism, one balanced D-S-D split step of 2e-5 s with the
    # BDF source; J = Q + 1e3 S_c. Gradients of the discrete adjoint against
    # central differences of the oracle for 20 random reactions and 20 random
    # state entries (T and mass fractions above 1e-6).
    #
    # Step size of the differences: the benchmark spec names 1e-6 in ln A, but the
    # adaptive integrator's step-size decisions make J noisy at the level of
    # its tolerance (|J| = 3.8e5; at reltol 1e-10 the central differences of one
    # reaction vary from 405 to -0.24 between h = 1e-6 and 1e-3, and most
    # reactions' true sensitivities here are below 0.1). The test therefore uses
    # reltol 1e-10 and h = 1e-3 (noise about 0.02), and holds each gradient to
    # 2e-3 of the difference quotient plus 1e-4 of the largest gradient.
    from oracle import split as osplit
    from oracle.chem import OracleMech
    from ember_gb300 import _lib as L
    from ember_gb300.source import GpuMechanism
    from ember_gb300.split import FlameBatchSplitSolver, flame_batch
    mech = synthetic_mechanism(n_species=53, n_reactions=325, seed=53325)   # the benchmark's C4 inputs
    grids, state, B, D, rho_u, ju, jb = flame_batch(mech, n_flames=1, n_min=400, n_max=400, seed=4000)
    rt = 1e-10
    opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD, bdf_reltol=rt, bdf_abstol_momentum=rt,
                                  bdf_abstol_energy=rt, bdf_abstol_species=rt * 1e-6)
    dt = 2e-5
    gm = GpuMechanism(mech)
    solver = FlameBatchSplitSolver(gm, grids, dt, method=BDF, source_options=opts,
                                   diffusion_algorithm=L.DIFFUSION_SERIAL)
    solver.set_state(0.0, state)
    solver.set_transport(B, D)
    hr, cs, g_state, g_lnk = solver.adjoint(np.ones(1), np.full(1, 1e3), rho_u, ju, jb, tape_cap=8192)
    om = OracleMech(mech)
    R = mech.n_reactions

    def J(st, mult=None):
        om.set_multipliers(mult)
        y, _, _, _, status = osplit.split_steps(om, grids, st, 0.0, B, D, dt, 1, BDF, opts)
        assert (status == 0).all()
        _, q, c = osplit.objectives(om, grids, y, opts.pressure, opts.kinetics_model, rho_u, ju, jb)
        return q[0] + 1e3 * c[0]

    # the taped forward step is the oracle's step
    assert hr[0] + 1e3 * cs[0] == J(state)
    rng = np.random.default_rng(2024)
    gmax = np.abs(g_lnk).max()
    assert gmax > 0
    for i in rng.choice(R, 20, replace=False):
        mp, mm = np.ones(R), np.ones(R)
        mp[i], mm[i] = np.exp(1e-3), np.exp(-1e-3)
        fd = (J(state, mp) - J(state, mm)) / 2e-3
        assert abs(g_lnk[i] - fd) <= 2e-3 * abs(fd) + 1e-4 * gmax, (i, g_lnk[i], fd, gmax)
    om.set_multipliers(None)
    # State entries: steps of 1e-3 of the entry. Smaller steps reach the
    # integrator's step-size noise: for entry (294, 3) the quotients are
    # -63482, -63466, -63496, -63508 at 1e-2, 3e-3, 1e-3, 3e-4 of the entry,
    # then -63017, -63949, -59702 at 1e-4, 3e-5, 1e-5 (and the noisy ones
    # differ between hosts).
    pts = rng.choice(len(state), 20, replace=False)
    for p in pts:
        ks = [1] + [2 + k for k in np.flatnonzero(state[p, 2:] > 1e-6)]
        k = int(rng.choice(ks))
        hstep = 1e-3 * abs(state[p, k])
        e = np.zeros_like(state)
        e[p, k] = hstep
        fd = (J(state + e) - J(state - e)) / (2 * hstep)
        scale = np.abs(g_state[:, k]).max()
        assert abs(g_state[p, k] - fd) <= 2e-3 * abs(fd) + 1e-4 * scale, (p, k, g_state[p, k], fd, scale)


def test_autograd_on_cuda_tensors_matches_the_host_path(gpu_lib):
    # CUDA inputs stay on the device (multipliers, state, objectives, gradients
    # through device pointers); the numbers are those of the host path
    torch = pytest.importorskip("torch")
    from ember_gb300 import _lib as L
    from ember_gb300.autograd import split_step_objectives
    from ember_gb300.source import GpuMechanism
    from ember_gb300.split import FlameBatchSplitSolver, flame_batch
    mech = synthetic_mechanism(n_species=20, n_reactions=60, seed=3)
    grids, state, B, D, rho_u, ju, jb = flame_batch(mech, n_flames=2, n_min=10, n_max=12, seed=5, width=2e-3,
                                                    thickness=3e-4, T_b=1500.0)
    opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD)
    gm = GpuMechanism(mech)
    solver = FlameBatchSplitSolver(gm, grids, 1e-6, method=BDF, source_options=opts,
                                   diffusion_algorithm=L.DIFFUSION_SERIAL)
    solver.set_transport(B, D)
    w = np.array([1.0, -0.5, 2e3, 1e3])
    res = []
    for dev in ("cpu", "cuda"):
        s0 = torch.tensor(state, dtype=torch.float64, device=dev, requires_grad=True)
        lk = torch.zeros(mech.n_reactions, dtype=torch.float64, device=dev, requires_grad=True)
        out = split_step_objectives(solver, s0, lk, 0.0, rho_u, ju, jb, 4096)
        assert out.device.type == dev
        (out * torch.as_tensor(w, device=dev)).sum().backward()
        assert s0.grad.device.type == dev and lk.grad.device.type == dev
        res.append((out.detach().cpu().numpy(), s0.grad.cpu().numpy(), lk.grad.cpu().numpy()))
    for a, b in zip(*res):
        np.testing.assert_array_equal(a, b)
