"""Adaptive flame grid (ember_grid_*, host code): OneDimGrid's rules
(src/grid.cpp) on hand-worked cases, each isolating one criterion by
disabling the others through the options, and FlameSolver's regrid block on
a split batch (the regridded batch then steps on the GPU bit for bit like
the oracle)."""
import numpy as np
import pytest

from ember_gb300 import _lib as L
from ember_gb300.grid import AdaptiveGrid, GridOptions, damping

OFF = 1e30   # a tolerance that never triggers


def _quiet(**kw):
    """Options with every criterion off, then the ones under test. rm_tol = 0
    keeps every interior point (the damping test of the removal sweep,
    hh[j] + hh[j-1] >= rm_tol * damp_const * damp[j], always holds);
    boundary_tol_rm = -1 keeps both ends."""
    o = GridOptions.defaults(vtol=OFF, dvtol=OFF, absvtol=1e-8, rm_tol=0.0, uniformity_tol=OFF, grid_min=0.0,
                             grid_max=OFF, damp_const=OFF, boundary_tol=OFF, boundary_tol_rm=-1.0)
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def _natural_spline(x, y, xo):
    """Value at xo of the natural cubic spline through (x, y): the second
    derivatives m solve the tridiagonal system of the standard derivation
    (m_0 = m_{n-1} = 0), solved here densely."""
    x, y = np.asarray(x, float), np.asarray(y, float)
    n = len(x)
    h = np.diff(x)
    A = np.zeros((n, n))
    r = np.zeros(n)
    A[0, 0] = A[-1, -1] = 1.0
    for i in range(1, n - 1):
        A[i, i - 1], A[i, i], A[i, i + 1] = h[i - 1], 2 * (h[i - 1] + h[i]), h[i]
        r[i] = 6 * ((y[i + 1] - y[i]) / h[i] - (y[i] - y[i - 1]) / h[i - 1])
    m = np.linalg.solve(A, r)
    j = int(np.searchsorted(x, xo)) - 1
    t = xo - x[j]
    return (y[j] + t * ((y[j + 1] - y[j]) / h[j] - h[j] * (2 * m[j] + m[j + 1]) / 6)
            + t * t * m[j] / 2 + t ** 3 * (m[j + 1] - m[j]) / (6 * h[j]))


def test_value_criterion_inserts_one_midpoint_per_pass():
    # a step between x = 4 and x = 5: |v[j+1] - v[j]| = range > vtol * range
    # inserts the midpoint 4.5 with the spline value; the insertion sweep then
    # moves past both new intervals
    x = np.arange(11.0)
    v = (x >= 5).astype(float)
    g = AdaptiveGrid(x, _quiet(vtol=0.12))
    xn, rows, upd = g.regrid(v[None, :], 1, np.ones(11), boundaries=False)
    assert upd
    np.testing.assert_array_equal(xn, np.concatenate([x[:5], [4.5], x[5:]]))
    assert abs(rows[0, 5] - _natural_spline(x, v, 4.5)) < 1e-14
    np.testing.assert_array_equal(np.delete(rows[0], 5), v)


def test_max_spacing_splits_every_interval_once():
    x = np.arange(11.0)
    v = np.sin(x)
    g = AdaptiveGrid(x, _quiet(grid_max=0.8))
    xn, rows, upd = g.regrid(v[None, :], 1, np.ones(11), boundaries=False)
    np.testing.assert_array_equal(xn, np.arange(21.0) * 0.5)
    np.testing.assert_array_equal(rows[0, ::2], v)   # old points keep their values
    for j in (1, 7, 19):
        assert abs(rows[0, j] - _natural_spline(x, v, xn[j])) < 1e-13


def test_uniformity_splits_the_long_interval():
    # spacings 1, 1, 3, 1, 1: 3/1 > 2.5 inserts x = 3.5 in [2, 5]; the new
    # spacings 1.5 / 1 pass the test, and the sweep skips past them
    x = np.array([0.0, 1.0, 2.0, 5.0, 6.0, 7.0])
    g = AdaptiveGrid(x, _quiet(uniformity_tol=2.5))
    xn, rows, _ = g.regrid(np.zeros((1, 6)), 1, np.ones(6), boundaries=False)
    np.testing.assert_array_equal(xn, [0.0, 1.0, 2.0, 3.5, 5.0, 6.0, 7.0])


def test_damping_length_criterion():
    # hh[j] > damp_const * damp[j] only in the interval starting at x = 3
    x = np.arange(8.0)
    damp = np.full(8, 1.0)
    damp[3] = 0.1
    g = AdaptiveGrid(x, _quiet(damp_const=2.0))
    xn, _, _ = g.regrid(np.zeros((1, 8)), 1, damp, boundaries=False)
    np.testing.assert_array_equal(xn, [0, 1, 2, 3, 3.5, 4, 5, 6, 7])


def test_minimum_spacing_cancels_an_insertion():
    x = np.arange(11.0)
    v = (x >= 5).astype(float)
    g = AdaptiveGrid(x, _quiet(vtol=0.12, grid_min=0.6))   # hh = 1 < 2 * grid_min
    xn, _, upd = g.regrid(v[None, :], 1, np.ones(11), boundaries=False)
    assert not upd
    np.testing.assert_array_equal(xn, x)


def test_removal_sweep_of_a_flat_profile():
    # constant rows (range < absvtol: no value criteria); with uniformity 2.5
    # the greedy sweep removes x = 1 (2 <= 2.5 hh[2]), keeps x = 2 (3 > 2.5),
    # removes x = 3, then x = 4 (its right test no longer applies): [0, 2, 5]
    x = np.arange(6.0)
    g = AdaptiveGrid(x, _quiet(uniformity_tol=2.5, rm_tol=0.6))
    xn, rows, upd = g.regrid(np.ones((2, 6)), 1, np.ones(6), boundaries=False)
    assert upd
    np.testing.assert_array_equal(xn, [0.0, 2.0, 5.0])
    np.testing.assert_array_equal(rows, np.ones((2, 3)))


def test_pinned_left_boundary_keeps_its_first_interior_point():
    # as the flat-profile sweep, but j = 1 stays: x = 2 goes, x = 3 stays
    # (3 > 2.5 hh[0]), x = 4 goes: [0, 1, 3, 5]
    x = np.arange(6.0)
    g = AdaptiveGrid(x, _quiet(uniformity_tol=2.5, rm_tol=0.6, left_bc=L.BC_CONTROL_VOLUME))
    xn, _, _ = g.regrid(np.ones((1, 6)), 1, np.ones(6), boundaries=False)
    np.testing.assert_array_equal(xn, [0.0, 1.0, 3.0, 5.0])


def test_right_boundary_extension_and_left_extension():
    # T (row 1) still rising at the right end: three points added with the
    # spacing ratio uniformityTol^(1/4); U (row 0, momentum) not flat at the
    # left end: three points added at sqrt(uniformityTol) times the first spacing
    x = np.arange(8.0)
    U = np.array([2.0, 1.0, 1, 1, 1, 1, 1, 1])
    T = np.linspace(300.0, 2000.0, 8)
    o = _quiet(boundary_tol=5e-5, boundary_tol_rm=1e-5, uniformity_tol=2.5)
    g = AdaptiveGrid(x, o)
    xn, rows, upd = g.regrid(np.vstack([U, T]), 2, np.ones(8))
    r, s = 2.5 ** 0.25, np.sqrt(2.5)
    right = [7 + r, 7 + r + r * r, 7 + r + r * r + r ** 3]
    left = [-(s + s * s + s ** 3), -(s + s * s), -s]
    assert upd
    np.testing.assert_allclose(xn, left + list(x) + right, rtol=0, atol=1e-12)
    np.testing.assert_array_equal(rows[1], np.concatenate([[300.0] * 3, T, [2000.0] * 3]))
    np.testing.assert_array_equal(rows[0], np.concatenate([[2.0] * 3, U, [1.0] * 3]))
    assert g.ju == 0 and g.jb == len(xn) - 1


def test_flat_right_end_is_trimmed():
    # the last five points are flat in every row: removeRight compares T[jj]
    # with T[jj - 2] (fixedBurnedVal) and takes points off the right end until
    # T[jj - 2] = 1500 differs from the boundary value, at jj = 6
    x = np.arange(10.0)
    T = np.array([300, 600, 900, 1200, 1500, 1800, 1800, 1800, 1800, 1800.0])
    g = AdaptiveGrid(x, _quiet(boundary_tol=OFF, boundary_tol_rm=1e-5))
    xn, rows, upd = g.regrid(np.vstack([np.ones(10), T]), 2, np.ones(10))
    assert upd
    np.testing.assert_array_equal(xn, np.arange(7.0))
    np.testing.assert_array_equal(rows[1], T[:7])


def test_unstrained_right_end_follows_the_reaction_zone():
    # heat release peak at x = 3 falling below 1 % at x = 2 and x = 4: width 2;
    # downstream width 5: the domain must reach 3 + 5 * 2 = 13 > 9
    x = np.arange(10.0)
    q = np.array([0, 0, 0.001, 1.0, 0.001, 0, 0, 0, 0, 0])
    g = AdaptiveGrid(x, _quiet(unstrained_downstream_width=5.0, uniformity_tol=2.5))
    xn, rows, upd = g.regrid(np.ones((1, 10)), 1, np.ones(10), qdot=q, strain_rate=0.0)
    assert upd and len(xn) == 13
    r = 2.5 ** 0.25
    assert xn[10] == pytest.approx(9 + r)


def test_damping_from_properties():
    props = {"viscosity": np.array([2e-5, 3e-5]), "conductivity": np.array([0.05, 0.1]),
             "cp_mass": np.array([1000.0, 2000.0]), "density": np.array([1.0, 0.5]),
             "rho_d": np.array([[1e-5, -1.0], [4e-5, 6e-5]])}
    d = damping(props, 2, 100.0)
    expect = [np.sqrt(min(2e-5, 0.05 / 1000.0, 1e-5) / 100.0), np.sqrt(min(3e-5, 0.1 / 2000.0, 4e-5, 6e-5) / 50.0)]
    np.testing.assert_allclose(d, expect, rtol=1e-15)


def test_bad_arguments():
    with pytest.raises(L.EmberGpuError):
        AdaptiveGrid(np.array([0.0, 1.0]))
    with pytest.raises(L.EmberGpuError):
        AdaptiveGrid(np.array([0.0, 2.0, 1.0]))
    g = AdaptiveGrid(np.arange(5.0))
    with pytest.raises(L.EmberGpuError):
        g.regrid(np.ones((1, 5)), 1, np.zeros(5))      # damping lengths must be positive
    with pytest.raises(L.EmberGpuError):
        g.regrid(np.ones((1, 5)), 1, np.ones(5), strain_rate=0.0)   # unstrained needs qdot


def _flame_case():
    from ember_gb300.mechanism import synthetic_mechanism
    from ember_gb300.split import flame_batch
    from ember_gb300.transport import synthetic_transport
    mech = synthetic_mechanism(n_species=20, n_reactions=60, seed=3)
    td = synthetic_transport(mech, seed=4)
    grids, state, B, D, rho_u, ju, jb = flame_batch(mech, n_flames=2, n_min=30, n_max=50, seed=5, width=2e-3,
                                                    thickness=3e-4)
    return mech, td, grids, state, B, D


def test_regrid_batch_keeps_surviving_points_and_renormalises():
    # FlameSolver's regrid block on a two-flame batch: the flame profiles do
    # not reach flat ends on this domain, so both ends are extended, and the
    # interior is refined and coarsened; points that stay keep their values
    # bit for bit, the mass fractions are renormalised where the grid changed
    from oracle import chem
    from ember_gb300.grid import regrid_batch
    mech, td, grids, state, B, D = _flame_case()
    om = chem.OracleMech(mech)
    props = chem.transport_eval(om, td, state[:, 1], state[:, 2:], 101325.0, 1e-5)
    rng = np.random.default_rng(1)
    ddt = tuple(rng.normal(size=state.shape) for _ in range(3))
    res = regrid_batch(grids, state, ddt, props, strain_rates=[200.0, 200.0])
    assert all(res.updated)
    offs = np.cumsum([0] + [g.n_points for g in grids])
    noffs = np.cumsum([0] + [g.n_points for g in res.grids])
    for f, (g, ng) in enumerate(zip(grids, res.grids)):
        assert (np.diff(ng.x) > 0).all() and ng.x[0] < g.x[0] and ng.x[-1] > g.x[-1]   # ends extended
        old = state[offs[f]:offs[f + 1]]
        new = res.state[noffs[f]:noffs[f + 1]]
        for j, xj in enumerate(g.x):
            k = np.flatnonzero(ng.x == xj)
            if k.size:
                np.testing.assert_array_equal(new[k[0], :2], old[j, :2])
                np.testing.assert_array_equal(res.ddt[1][noffs[f] + k[0]], ddt[1][offs[f] + j])
    np.testing.assert_allclose(res.state[:, 2:].sum(axis=1), 1.0, rtol=0, atol=1e-12)
    assert (res.state[:, 2:] >= 0).all()


@pytest.mark.gpu
def test_regridded_batch_steps_like_the_oracle(gpu_lib):
    # a regrid between steps: new grids, state and time derivatives; the GPU
    # split handle created on the new grids (with the time derivatives carried
    # over) steps bit for bit like the oracle
    from oracle import chem
    from oracle import split as osplit
    from ember_gb300.grid import regrid_batch
    from ember_gb300.source import GpuMechanism, KINETICS_STANDARD, QSS, SourceOptions
    from ember_gb300.split import FlameBatchSplitSolver
    from ember_gb300.transport import GpuTransport
    mech, td, grids, state, B, D = _flame_case()
    opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD)
    dt = 5e-7
    om = chem.OracleMech(mech)
    st1, t1, dd, dp, _ = osplit.split_steps(om, grids, state, 0.0, B, D, dt, 1, QSS, opts, transport=(td, 1e-5, True))
    props = chem.transport_eval(om, td, st1[:, 1], st1[:, 2:], opts.pressure, 1e-5)
    res = regrid_batch(grids, st1, (None, dd, dp), props, strain_rates=[200.0, 200.0])
    assert any(res.updated)
    n = mech.n_vars * len(res.state)
    gm = GpuMechanism(mech)
    s = FlameBatchSplitSolver(gm, res.grids, dt, method=QSS, source_options=opts, diffusion_algorithm=L.DIFFUSION_SERIAL)
    gt = GpuTransport(gm, td)
    s.set_state(t1, res.state)
    s.set_transport(np.zeros(n), np.zeros(n))   # replaced by the transport model at every step
    s.set_transport_model(gt, 1e-5, True)
    s.set_derivatives(res.ddt[1], res.ddt[2])
    s.step(2, graph=True)
    out, t = s.state()
    ref, rt, *_ = osplit.split_steps(om, res.grids, res.state, t1, np.zeros(n), np.zeros(n), dt, 2, QSS, opts,
                                     transport=(td, 1e-5, True), ddt=(res.ddt[1], res.ddt[2]))
    assert t == rt
    assert np.array_equal(out, ref), np.abs(out - ref).max()
