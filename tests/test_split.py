"""Split step of a batch of flames (SplitSolver::step, src/splitSolver.cpp:
34-121): the GPU path (ember_split_*) against the CPU restatement in
oracle/split.py, which strings together the oracle's diffusion systems and
source-term integrators in the reference's stage order."""
import numpy as np
import pytest

import oracle
from oracle import split as osplit
from ember_gb300 import _lib as L
from ember_gb300.mechanism import synthetic_mechanism
from ember_gb300.source import BDF, KINETICS_STANDARD, QSS, SourceOptions
from ember_gb300.split import flame_batch


@pytest.fixture(scope="module")
def mech():
    return synthetic_mechanism(n_species=20, n_reactions=60, seed=3)


def _case(mech, n_flames=2, n_min=9, n_max=14, seed=5):
    return flame_batch(mech, n_flames=n_flames, n_min=n_min, n_max=n_max, seed=seed, width=2e-3, thickness=3e-4)


def test_oracle_split_keeps_mass_fractions_normalised_and_uniform_states_uniform(mech):
    from oracle.chem import OracleMech
    om = OracleMech(mech)
    grids, state, B, D, rho_u, ju, jb = _case(mech)
    opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD)
    out, t, dd, dp, st = osplit.split_steps(om, grids, state, 0.0, B, D, 1e-6, 2, QSS, opts)
    assert t == 2e-6
    np.testing.assert_allclose(out[:, 2:].sum(axis=1), 1.0, rtol=0, atol=1e-12)
    assert (out[:, 2:] >= 0).all()
    # every point of one flame in the same state: diffusion leaves the
    # profile flat (up to the rounding of b = -(a + c)), the source acts alike
    uni = np.repeat(state[len(state) // 2][None, :], grids[0].n_points, axis=0)
    n0 = grids[0].n_points
    Bu = B[:mech.n_vars * n0]
    Du = D[:mech.n_vars * n0]
    out, *_ = osplit.split_steps(om, grids[:1], uni, 0.0, Bu, Du, 1e-6, 1, QSS, opts)
    np.testing.assert_allclose(out, np.repeat(out[:1], n0, axis=0), rtol=1e-12, atol=1e-15)


def _gpu_solver(mech, grids, dt, method, opts, algorithm, balanced=True):
    from ember_gb300.source import GpuMechanism
    from ember_gb300.split import FlameBatchSplitSolver
    gm = GpuMechanism(mech)
    s = FlameBatchSplitSolver(gm, grids, dt, method=method, source_options=opts, balanced=balanced,
                              diffusion_algorithm=algorithm)
    return gm, s


@pytest.mark.gpu
@pytest.mark.parametrize("method,n_steps", [(QSS, 3), (BDF, 2)])
def test_split_serial_bitwise_vs_oracle(gpu_lib, mech, method, n_steps):
    from oracle.chem import OracleMech
    grids, state, B, D, rho_u, ju, jb = _case(mech)
    opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD)
    dt = 2e-6
    gm, s = _gpu_solver(mech, grids, dt, method, opts, L.DIFFUSION_SERIAL)
    s.set_state(1e-3, state)
    s.set_transport(B, D)
    s.step(n_steps)
    out, t = s.state()
    dd, dp = s.derivatives()
    ref, rt, rdd, rdp, rst = osplit.split_steps(OracleMech(mech), grids, state, 1e-3, B, D, dt, n_steps, method, opts)
    st, _ = s.source_status()
    assert t == rt
    np.testing.assert_array_equal(st, rst)
    assert np.array_equal(out, ref), np.abs(out - ref).max()
    assert np.array_equal(dd, rdd) and np.array_equal(dp, rdp)
    np.testing.assert_allclose(out[:, 2:].sum(axis=1), 1.0, rtol=0, atol=1e-12)
    # this small synthetic mechanism runs away to ~5000 K: a few points fail
    # (QSS dtmin) in the later steps, on the GPU as in the oracle
    assert s.failures()[1] == 0


@pytest.mark.gpu
def test_split_graph_replay_equals_stream_steps(gpu_lib, mech):
    grids, state, B, D, rho_u, ju, jb = _case(mech, n_flames=3, n_min=20, n_max=60)
    opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD)
    outs = []
    for graph in (False, True):
        gm, s = _gpu_solver(mech, grids, 2e-6, QSS, opts, L.DIFFUSION_PARALLEL)
        s.set_state(0.0, state)
        s.set_transport(B, D)
        s.step(2, graph=graph)
        s.step(2, graph=graph)  # the graph is captured once and replayed
        outs.append((s.state(), s.derivatives()))
    (a, ta), (da, pa) = outs[0]
    (b, tb), (db, pb) = outs[1]
    assert ta == tb and abs(ta - 8e-6) < 1e-18
    assert np.array_equal(a, b) and np.array_equal(da, db) and np.array_equal(pa, pb)


@pytest.mark.gpu
def test_split_parallel_diffusion_close_to_oracle(gpu_lib, mech):
    # The warp-parallel diffusion solver agrees with the reference's Thomas
    # algorithm to rounding (1e-12 of max|y| per system); through the source
    # stage and the mass-fraction correction the step stays within 1e-9 of
    # the largest value of each variable.
    from oracle.chem import OracleMech
    grids, state, B, D, rho_u, ju, jb = _case(mech, n_flames=2, n_min=40, n_max=90)
    opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD)
    gm, s = _gpu_solver(mech, grids, 2e-6, QSS, opts, L.DIFFUSION_PARALLEL)
    s.set_state(0.0, state)
    s.set_transport(B, D)
    s.step(2)
    out, _ = s.state()
    ref, *_ = osplit.split_steps(OracleMech(mech), grids, state, 0.0, B, D, 2e-6, 2, QSS, opts)
    scale = np.abs(ref).max(axis=0)
    err = (np.abs(out - ref) / np.where(scale > 0, scale, 1.0)).max()
    assert err <= 1e-9, err


@pytest.mark.gpu
def test_split_objectives_bitwise_vs_oracle(gpu_lib, mech):
    from oracle.chem import OracleMech
    grids, state, B, D, rho_u, ju, jb = _case(mech, n_flames=3, n_min=12, n_max=30)
    opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD)
    gm, s = _gpu_solver(mech, grids, 2e-6, QSS, opts, L.DIFFUSION_SERIAL)
    s.set_state(0.0, state)
    s.set_transport(B, D)
    s.step(1)
    out, _ = s.state()
    q, hr, cs = s.objectives(rho_u, ju, jb)
    rq, rhr, rcs = osplit.objectives(OracleMech(mech), grids, out, opts.pressure, opts.kinetics_model, rho_u, ju, jb)
    assert np.array_equal(q, rq)
    assert np.array_equal(hr, rhr) and np.array_equal(cs, rcs)
    assert (hr != 0).all()


@pytest.mark.gpu
def test_consumption_speed_uses_the_property_update_cp(gpu_lib, mech):
    # with the transport model the step starts with a property update, and the
    # consumption speed divides by that cp (FlameSolver::getConsumptionSpeed)
    from oracle.chem import OracleMech
    from ember_gb300.transport import GpuTransport, synthetic_transport
    td = synthetic_transport(mech, seed=4)
    grids, state, B, D, rho_u, ju, jb = _case(mech, n_flames=2, n_min=12, n_max=20)
    opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD)
    gm, s = _gpu_solver(mech, grids, 2e-6, QSS, opts, L.DIFFUSION_SERIAL)
    gt = GpuTransport(gm, td)
    s.set_state(0.0, state)
    s.set_transport(B, D)
    s.set_transport_model(gt, 1e-5, True)
    s.step(2)
    out, _ = s.state()
    q, hr, cs = s.objectives(rho_u, ju, jb)
    om = OracleMech(mech)
    props = {}
    ref, *_ = osplit.split_steps(om, grids, state, 0.0, B, D, 2e-6, 2, QSS, opts, transport=(td, 1e-5, True),
                                 props_out=props)
    assert np.array_equal(out, ref)
    rq, rhr, rcs = osplit.objectives(om, grids, ref, opts.pressure, opts.kinetics_model, rho_u, ju, jb,
                                     cp=props["cp_mass"])
    assert np.array_equal(q, rq) and np.array_equal(hr, rhr)
    assert np.array_equal(cs, rcs)
    _, _, cs_now = osplit.objectives(om, grids, ref, opts.pressure, opts.kinetics_model, rho_u, ju, jb)
    assert not np.array_equal(cs, cs_now)   # the start-of-step cp differs from the end state's


def _cross_numpy(om, td, grids, state, pressure, thr, mult, gdt):
    """Vectorised restatement of updateCrossTerms (src/flameSolver.cpp:551-617,
    no thermal diffusion) for checking oracle/split.py's loops."""
    import oracle
    from oracle import chem
    props = chem.transport_eval(om, td, state[:, 1], state[:, 2:], pressure, thr)
    n_pts, n = state.shape
    cross = np.zeros((n_pts, n))
    offs = np.cumsum([0] + [g.n_points for g in grids])
    W = om.mech.mol_weight
    for f, g in enumerate(grids):
        a, b = offs[f], offs[f + 1]
        N = b - a
        x = np.asarray(g.x, float)
        Y = state[a:b, 2:]
        T = state[a:b, 1]
        rd = props["rho_d"][a:b]
        cs = props["cp_species"][a:b]
        rho, cp, lam = props["density"][a:b], props["cp_mass"][a:b], props["conductivity"][a:b]
        hh = np.diff(x)
        jF = -0.5 * (rd[:-1] + rd[1:]) * (np.diff(Y, axis=0) / hh[:, None])
        jc = np.append(-jF.sum(axis=1), 0.0)
        jB = lam / (rho * cp)
        dlj = 0.5 * (x[2:] - x[:-2])
        h = min(gdt, (mult * dlj * dlj / jB[1:-1]).min())
        jc = oracle.diffusion_system(x, jB, np.ones(N), jc, 0.0, gdt, split_const=np.zeros(N), alpha=g.alpha,
                                     left_bc=g.left_bc, right_bc=g.right_bc, h=h, mult=mult, gdt=gdt)
        r = x ** g.alpha
        rph = (0.5 * (x[:-1] + x[1:])) ** g.alpha
        i = np.arange(1, N - 1)
        c = -0.5 / (r[i] * rho[i] * dlj)
        dY = c[:, None] * (rph[i, None] * (Y[i] + Y[i + 1]) * jc[i, None]
                           - rph[i - 1, None] * (Y[i - 1] + Y[i]) * jc[i - 1, None])
        cross[a + 1:b - 1, 2:] = dY
        s = np.zeros(N)
        s[i] = (0.5 * (cs[i] + cs[i + 1]) / W * (jF[i] + 0.5 * (Y[i] + Y[i + 1]) * jc[i, None])).sum(axis=1)
        hm = hh[:-1]
        hp = hh[1:]
        dTdx = (-hp / (hm * (hp + hm))) * T[:-2] + ((hp - hm) / (hp * hm)) * T[1:-1] + (hm / (hp * (hp + hm))) * T[2:]
        cross[a + 1:b - 1, 1] = -0.5 * (s[i] + s[i - 1]) * dTdx / (cp[i] * rho[i])
    return props, cross


def test_oracle_step_properties_match_vectorised_restatement(mech):
    from oracle.chem import OracleMech
    from ember_gb300.transport import synthetic_transport
    om = OracleMech(mech)
    td = synthetic_transport(mech, seed=4)
    grids, state, B, D, rho_u, ju, jb = _case(mech, n_flames=2, n_min=12, n_max=20)
    Bo, Do, co = osplit.step_properties(om, td, grids, state, 101325.0, 1e-5, 10.0, 2e-6, True)
    props, cr = _cross_numpy(om, td, grids, state, 101325.0, 1e-5, 10.0, 2e-6)
    scale = np.abs(cr).max(axis=0)
    np.testing.assert_allclose(co, cr, rtol=0, atol=1e-10 * scale.max())
    assert np.abs(co[:, 2:]).max() > 0 and np.abs(co[:, 1]).max() > 0
    assert (co[:, 0] == 0).all()
    # B, D of the first flame's T and Y_0 rows
    N = grids[0].n_points
    np.testing.assert_array_equal(Bo[N:2 * N], 1.0 / (props["density"][:N] * props["cp_mass"][:N]))
    np.testing.assert_array_equal(Do[2 * N:3 * N], props["rho_d"][:N, 0])
    # a spatially uniform state has no cross terms
    uni = np.repeat(state[N // 2][None, :], N, axis=0)
    _, _, cu = osplit.step_properties(om, td, grids[:1], uni, 101325.0, 1e-5, 10.0, 2e-6, True)
    assert (cu == 0).all()


@pytest.mark.gpu
@pytest.mark.parametrize("cross", [False, True])
def test_split_transport_model_bitwise_vs_oracle(gpu_lib, mech, cross):
    from oracle.chem import OracleMech
    from ember_gb300.transport import GpuTransport, synthetic_transport
    td = synthetic_transport(mech, seed=4)
    grids, state, B, D, rho_u, ju, jb = _case(mech, n_flames=2, n_min=10, n_max=16)
    opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD)
    dt = 2e-6
    gm, s = _gpu_solver(mech, grids, dt, QSS, opts, L.DIFFUSION_SERIAL)
    gt = GpuTransport(gm, td)
    s.set_state(0.0, state)
    s.set_transport(B * 0.0, D * 0.0)   # replaced by the model at every step
    s.set_transport_model(gt, 1e-5, cross)
    s.step(2)
    out, t = s.state()
    dd, dp = s.derivatives()
    ref, rt, rdd, rdp, rst = osplit.split_steps(OracleMech(mech), grids, state, 0.0, B, D, dt, 2, QSS, opts,
                                                transport=(td, 1e-5, cross))
    assert t == rt
    assert np.array_equal(out, ref), np.abs(out - ref).max()
    assert np.array_equal(dd, rdd) and np.array_equal(dp, rdp)
    assert s.failures()[1] == 0
    # the captured graph replays the same step
    gm2, s2 = _gpu_solver(mech, grids, dt, QSS, opts, L.DIFFUSION_SERIAL)
    gt2 = GpuTransport(gm2, td)
    s2.set_state(0.0, state)
    s2.set_transport(B, D)
    s2.set_transport_model(gt2, 1e-5, cross)
    s2.step(2, graph=True)
    assert np.array_equal(s2.state()[0], out)


@pytest.mark.gpu
def test_split_transport_model_parallel_diffusion_close_to_oracle(gpu_lib, mech):
    # the warp-parallel integrator (diffusion stages and the jCorr smoothing)
    # agrees with the reference's Thomas algorithm to rounding
    from oracle.chem import OracleMech
    from ember_gb300.transport import GpuTransport, synthetic_transport
    td = synthetic_transport(mech, seed=4)
    grids, state, B, D, rho_u, ju, jb = _case(mech, n_flames=2, n_min=40, n_max=90)
    opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD)
    gm, s = _gpu_solver(mech, grids, 2e-6, QSS, opts, L.DIFFUSION_PARALLEL)
    gt = GpuTransport(gm, td)
    s.set_state(0.0, state)
    s.set_transport(B, D)
    s.set_transport_model(gt, 1e-5, True)
    s.step(2, graph=True)
    out, _ = s.state()
    ref, *_ = osplit.split_steps(OracleMech(mech), grids, state, 0.0, B, D, 2e-6, 2, QSS, opts,
                                 transport=(td, 1e-5, True))
    scale = np.abs(ref).max(axis=0)
    err = (np.abs(out - ref) / np.where(scale > 0, scale, 1.0)).max()
    assert err <= 1e-9, err


@pytest.mark.gpu
def test_load_state_keeps_time_and_split_history(gpu_lib, mech):
    grids, state, B, D, rho_u, ju, jb = _case(mech, n_flames=2, n_min=12, n_max=20)
    opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD)
    gm, a = _gpu_solver(mech, grids, 2e-6, QSS, opts, L.DIFFUSION_SERIAL)
    a.set_state(0.0, state)
    a.set_transport(B, D)
    a.step(2)
    _, b = _gpu_solver(mech, grids, 2e-6, QSS, opts, L.DIFFUSION_SERIAL)
    b.set_state(0.0, state)
    b.set_transport(B, D)
    b.step(1)
    mid, _ = b.state()
    b.load_state(mid)   # a host round trip of the state between steps
    b.step(1)
    (sa, ta), (sb, tb) = a.state(), b.state()
    assert ta == tb and np.array_equal(sa, sb)
    assert all(np.array_equal(x, y) for x, y in zip(a.derivatives(), b.derivatives()))


def _convection_case(mech, n_flames=2, n_min=12, n_max=18, seed=5):
    """A split case with the convection stage: the strained-flow velocity
    U = a sqrt(rho_u / rho), inflow through the left boundary."""
    from ember_gb300.convection import ConvectionFlame, mean_molecular_weight
    from ember_gb300.split import mixture_properties
    grids, state, B, D, rho_u, ju, jb = _case(mech, n_flames=n_flames, n_min=n_min, n_max=n_max, seed=seed)
    state = state.copy()
    rho, _ = mixture_properties(mech, state)
    flames, y_left = [], []
    p = 0
    for f, g in enumerate(grids):
        N = g.n_points
        a = 200.0 + 300.0 * f
        state[p:p + N, 0] = a * np.sqrt(rho_u[f] / rho[p:p + N])
        y0 = state[p, 2:].copy()
        flames.append(ConvectionFlame(n_points=N, left_bc=g.left_bc, right_bc=g.right_bc, alpha=g.alpha,
                                      rv_zero=0.4 * rho_u[f], t_left=float(state[p, 1]),
                                      w_left=float(mean_molecular_weight(y0, mech.mol_weight)[0]),
                                      rhou=float(rho_u[f]), strain_initial=a, strain_final=a))
        y_left.append(y0)
        p += N
    return grids, state, B, D, flames, np.array(y_left)


def test_oracle_split_with_convection_runs_the_full_sequence(mech):
    from oracle.chem import OracleMech
    from ember_gb300.convection import ConvectionOptions
    grids, state, B, D, flames, y_left = _convection_case(mech)
    opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD)
    om = OracleMech(mech)
    conv = (flames, y_left, ConvectionOptions())
    out, t, dd, dp, st = osplit.split_steps(om, grids, state, 0.0, B, D, 2e-6, 2, QSS, opts, convection=conv)
    assert t == 4e-6 and np.isfinite(out).all()
    np.testing.assert_allclose(out[:, 2:].sum(axis=1), 1.0, rtol=0, atol=1e-12)
    ref, *_ = osplit.split_steps(om, grids, state, 0.0, B, D, 2e-6, 2, QSS, opts)
    assert not np.array_equal(out[:, 0], ref[:, 0])      # the convection stage moved U


@pytest.mark.gpu
@pytest.mark.parametrize("graph", [False, True])
def test_split_with_convection_bitwise_vs_oracle(gpu_lib, mech, graph):
    from oracle.chem import OracleMech
    from ember_gb300.convection import ConvectionOptions
    grids, state, B, D, flames, y_left = _convection_case(mech)
    opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD)
    dt = 2e-6
    copts = ConvectionOptions()
    gm, s = _gpu_solver(mech, grids, dt, QSS, opts, L.DIFFUSION_SERIAL)
    s.set_state(1e-3, state)
    s.set_transport(B, D)
    s.set_convection(flames, y_left, copts)
    s.step(3, graph=graph)
    out, t = s.state()
    dd, dp = s.derivatives()
    ref, rt, rdd, rdp, rst = osplit.split_steps(OracleMech(mech), grids, state, 1e-3, B, D, dt, 3, QSS, opts,
                                                convection=(flames, y_left, copts))
    assert t == rt
    assert np.array_equal(out, ref), np.abs(out - ref).max()
    assert np.array_equal(dd, rdd) and np.array_equal(dp, rdp)
    assert s.failures()[1] == 0
    # detached: the step is D-S-D again
    s.set_convection(None)
    s.set_state(1e-3, state)
    s.step(1)
    ref2, *_ = osplit.split_steps(OracleMech(mech), grids, state, 1e-3, B, D, dt, 1, QSS, opts)
    assert np.array_equal(s.state()[0], ref2)


@pytest.mark.gpu
@pytest.mark.parametrize("algorithm", [L.DIFFUSION_SERIAL, L.DIFFUSION_PARALLEL], ids=["serial", "parallel"])
def test_split_with_convection_and_transport_model_vs_oracle(gpu_lib, mech, algorithm):
    # the configuration the split benchmark runs: D C D S D C D with the device
    # transport model and cross terms (properties, B/D, jCorr smoothing) at the
    # start of every step; the serial diffusion algorithm is bitwise. With the
    # warp-parallel one the rounding-level differences reach the convection
    # stage, whose adaptive Adams integrator (reltol 1e-6) can then take other
    # steps: the two agree within the convection tolerances, |error| <=
    # reltol |y| + abstol per variable (measured: 5e-5 of a variable's largest
    # value, for a minor species near its abstol)
    from oracle.chem import OracleMech
    from ember_gb300.convection import ConvectionOptions
    from ember_gb300.transport import GpuTransport, synthetic_transport
    td = synthetic_transport(mech, seed=4)
    grids, state, B, D, flames, y_left = _convection_case(mech)
    opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD)
    # this small synthetic mechanism runs away within a few steps of 2e-6 s
    # (points fail at the QSS dtmin, on the GPU as in the oracle); two steps
    # of 5e-7 s stay clear of that
    dt = 5e-7
    copts = ConvectionOptions()
    gm, s = _gpu_solver(mech, grids, dt, QSS, opts, algorithm)
    gt = GpuTransport(gm, td)
    s.set_state(0.0, state)
    s.set_transport(B, D)
    s.set_transport_model(gt, 1e-5, True)
    s.set_convection(flames, y_left, copts)
    s.step(2, graph=True)
    out, t = s.state()
    ref, rt, _, _, rst = osplit.split_steps(OracleMech(mech), grids, state, 0.0, B, D, dt, 2, QSS, opts,
                                            transport=(td, 1e-5, True), convection=(flames, y_left, copts))
    assert t == rt
    assert (rst == 0).all()
    assert s.failures() == (0, 0)
    if algorithm == L.DIFFUSION_SERIAL:
        assert np.array_equal(out, ref), np.abs(out - ref).max()
    else:
        atol = np.full(out.shape[1], copts.abstol_y)
        atol[0], atol[1] = copts.abstol_u, copts.abstol_t
        units = np.abs(out - ref) / (copts.reltol * np.abs(ref) + atol)
        assert units.max() <= 1.0, units.max()


@pytest.mark.gpu
@pytest.mark.parametrize("bc", ["temperature", "stagnation", "qdot", "right"])
def test_continuity_point_moves_every_step_like_the_oracle(gpu_lib, mech, bc):
    # updateContinuityBoundaryCondition at the start of every step after the
    # first: the continuity point follows the mid-temperature crossing, the
    # stagnation point of V, the heat-release peak; rV[j_cont] is carried from
    # the last evaluation (fixedRight, fixedQdot). Start values deliberately
    # off, so that the update moves them; bitwise against the oracle, stream
    # launches and graph replay.
    from oracle.chem import OracleMech
    from ember_gb300.convection import CONT_QDOT, CONT_RIGHT, CONT_TEMP, CONT_ZERO, ConvectionOptions
    grids, state, B, D, flames, y_left = _convection_case(mech)
    for fl, g in zip(flames, grids):
        N = g.n_points
        if bc == "temperature":
            fl.continuity_bc, fl.j_cont = CONT_TEMP, 1
        elif bc == "stagnation":
            fl.continuity_bc, fl.j_cont, fl.x_vzero = CONT_ZERO, 2, float(g.x[2])
        elif bc == "qdot":
            fl.continuity_bc, fl.j_cont, fl.rv_cont = CONT_QDOT, 1, 0.1
        else:
            fl.continuity_bc, fl.j_cont, fl.rv_cont = CONT_RIGHT, N - 1, -0.05
    opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD)
    dt = 5e-7
    copts = ConvectionOptions()
    ref, rt, *_ = osplit.split_steps(OracleMech(mech), grids, state, 0.0, B, D, dt, 3, QSS, opts,
                                     convection=(flames, y_left, copts))
    for graph in (False, True):
        gm, s = _gpu_solver(mech, grids, dt, QSS, opts, L.DIFFUSION_SERIAL)
        s.set_state(0.0, state)
        s.set_transport(B, D)
        s.set_convection(flames, y_left, copts)
        s.step(3, graph=graph)
        out, t = s.state()
        assert t == rt
        assert np.array_equal(out, ref), (graph, np.abs(out - ref).max())
    if bc == "temperature":
        # the start value was not the crossing: the update moved it
        from copy import copy
        fl = copy(flames[0])
        n0 = grids[0].n_points
        osplit.continuity_point(fl, grids[0].x, state[:n0, 1], None, None, None)
        assert fl.j_cont != 1


@pytest.mark.gpu
def test_captured_step_survives_a_later_call_for_smaller_flames(gpu_lib, mech):
    # the UTW kernel stages 3N doubles of shared memory per flame; a later
    # convection call for small flames must not lower the kernel's limit
    # below what a captured step of a 2100-point flame (50 KB) needs
    from ember_gb300.convection import ConvectionOptions, convection_batch, integrate_convection_terms
    grids, state, B, D, flames, y_left = _convection_case(mech, n_flames=1, n_min=2100, n_max=2100)
    opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD)
    copts = ConvectionOptions()
    gm, s = _gpu_solver(mech, grids, 2e-7, QSS, opts, L.DIFFUSION_PARALLEL)
    s.set_state(0.0, state)
    s.set_transport(B, D)
    s.set_convection(flames, y_left, copts)
    s.step(1, graph=True)
    cb = convection_batch(mech, n_flames=2, n_min=40, n_max=60, seed=17)
    integrate_convection_terms(cb.flames, mech.mol_weight, cb.x, cb.y_left, cb.drhodt, cb.split_const,
                               cb.state.copy(), 0.0, 1e-6, copts)
    s.step(1, graph=True)   # replays the captured step
    out, t = s.state()
    gm2, r = _gpu_solver(mech, grids, 2e-7, QSS, opts, L.DIFFUSION_PARALLEL)
    r.set_state(0.0, state)
    r.set_transport(B, D)
    r.set_convection(flames, y_left, copts)
    r.step(2)
    assert np.array_equal(out, r.state()[0])


@pytest.mark.gpu
def test_split_rejects_convection_flames_at_another_pressure(gpu_lib, mech):
    # the reference has one gas pressure for every stage of the step
    from ember_gb300.convection import ConvectionOptions
    grids, state, B, D, flames, y_left = _convection_case(mech)
    opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD)
    gm, s = _gpu_solver(mech, grids, 2e-6, QSS, opts, L.DIFFUSION_SERIAL)
    flames[1].pressure = 2.0 * opts.pressure
    with pytest.raises(L.EmberGpuError):
        s.set_convection(flames, y_left, ConvectionOptions())


@pytest.mark.parametrize("with_convection", [False, True])
def test_balanced_split_constants_add_up_to_the_cross_rate(with_convection):
    """Balanced splitting redistributes the rates between the operators: the
    split constants of all operators sum to the cross-term rate (two operators:
    c_D + c_S = f_X; three: c_D + c_C + c_S = f_X), and each operator's
    constant plus its own rate is the same total rate share."""
    rng = np.random.default_rng(7)
    shape = (13, 9)
    fd, fs, fc, fx = (rng.standard_normal(shape) * 1e3 for _ in range(4))
    sd, ss, sc = osplit.split_constants(fd, fs, fx, True, fc if with_convection else None)
    total = sd + ss + (sc if with_convection else 0.0)
    np.testing.assert_allclose(total, fx, rtol=0, atol=1e-9)
    if with_convection:
        rate = (fd + fs + fc + fx) / 4.0
        np.testing.assert_allclose(sd + fd, rate, atol=1e-9)
        np.testing.assert_allclose(sc + fc, rate, atol=1e-9)
        np.testing.assert_allclose(ss + fs, 2.0 * rate, atol=1e-9)
    sd, ss, sc = osplit.split_constants(fd, fs, fx, False, fc if with_convection else None)
    np.testing.assert_array_equal(sd, fx)


@pytest.mark.gpu
def test_split_with_chebyshev_strain_vs_oracle(gpu_lib, mech):
    # ember_split_set_strain: every flame's strain rate becomes a Chebyshev
    # series (the reference's strainfunc after setCoefficients); bitwise
    # against the oracle with the same series attached from the start, and
    # an update between captured-graph replays reaches the graph
    from dataclasses import replace
    from oracle.chem import OracleMech
    from ember_gb300.convection import STRAIN_CHEBYSHEV, ConvectionOptions
    grids, state, B, D, flames, y_left = _convection_case(mech)
    opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD)
    dt = 5e-7
    copts = ConvectionOptions()
    coeffs = np.array([[0.0, 3 * dt, a, 0.3 * a, -0.1 * a, 0.05 * a] for a in (200.0, 500.0)])
    cheb = [replace(fl, strain_type=STRAIN_CHEBYSHEV, cheb_t0=c[0], cheb_t1=c[1], cheb=tuple(c[2:]))
            for fl, c in zip(flames, coeffs)]
    ref, rt, *_ = osplit.split_steps(OracleMech(mech), grids, state, 0.0, B, D, dt, 3, QSS, opts,
                                     convection=(cheb, y_left, copts))
    outs = {}
    for graph in (False, True):
        gm, s = _gpu_solver(mech, grids, dt, QSS, opts, L.DIFFUSION_SERIAL)
        s.set_state(0.0, state)
        s.set_transport(B, D)
        s.set_convection(flames, y_left, copts)
        s.set_strain_chebyshev(coeffs)
        s.step(3, graph=graph)
        out, t = s.state()
        assert t == rt
        assert np.array_equal(out, ref), (graph, np.abs(out - ref).max())
        # linear strain for one captured step, then the series
        s.set_state(0.0, state)
        s.set_convection(flames, y_left, copts)
        s.step(1, graph=graph)
        s.set_strain_chebyshev(coeffs)
        s.step(2, graph=graph)
        outs[graph] = s.state()[0]
    assert np.array_equal(outs[False], outs[True])
    assert not np.array_equal(outs[False], ref)
    # a one-coefficient series is a constant strain: LinearFunction's bits
    const = np.array([[0.0, 3 * dt, fl.strain_initial] for fl in flames])
    res = []
    for use_cheb in (False, True):
        gm, s = _gpu_solver(mech, grids, dt, QSS, opts, L.DIFFUSION_SERIAL)
        s.set_state(0.0, state)
        s.set_transport(B, D)
        s.set_convection(flames, y_left, copts)
        if use_cheb:
            s.set_strain_chebyshev(const)
        s.step(2)
        res.append(s.state()[0])
    assert np.array_equal(res[0], res[1])
