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
