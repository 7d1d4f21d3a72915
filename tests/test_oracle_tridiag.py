"""The CPU oracle's tridiagonal integrator and diffusion system, pinned to the
reference's own tests: the golden table of test/tridiagonalIntegrator.cpp
(generated by test/reference/bdf.py) and the analytic/property tests of
test/test_diffusionSystem.cpp."""
import json
import os

import numpy as np
import pytest

import oracle


@pytest.fixture(scope="module")
def golden(golden_dir):
    with open(os.path.join(golden_dir, "tridiag_bdf.json")) as f:
        return json.load(f)


def test_golden_table_matches_generator(golden):
    # The committed table and a fresh run of bdf.py agree (fixture sanity).
    np.testing.assert_allclose(golden["table_cpp"], golden["bdf_dt0.2"], rtol=0, atol=1e-13)


def test_stepwise(golden):
    # TridiagonalIntegratorTest.Stepwise (test/tridiagonalIntegrator.cpp:64-76)
    g = golden
    for j, row in enumerate(g["table_cpp"]):
        y, t, h = oracle.tridiag_run(g["a"], g["b"], g["c"], g["k"], g["y0"], 0.0, 0.2, n_steps=j)
        if j == 0:
            y = np.array(g["y0"], dtype=float)
        np.testing.assert_allclose(y, row, rtol=0, atol=1e-10)


def test_full_integration(golden):
    # TridiagonalIntegratorTest.FullIntegration (79-90)
    g = golden
    y, t, h = oracle.tridiag_run(g["a"], g["b"], g["c"], g["k"], g["y0"], 0.0, 0.2, t_end=1.0)
    assert abs(h - 0.2) < 1e-10 and abs(t - 1.0) < 1e-10
    np.testing.assert_allclose(y, g["table_cpp"][5], rtol=0, atol=1e-10)


def test_short_integration(golden):
    # TridiagonalIntegratorTest.ShortIntegration (93-102)
    g = golden
    y, t, h = oracle.tridiag_run(g["a"], g["b"], g["c"], g["k"], g["y0"], 0.0, 1.3, t_end=0.2)
    assert abs(t - 0.2) < 1e-10
    np.testing.assert_allclose(y, g["table_cpp"][1], rtol=0, atol=1e-10)


def test_finer_steps_converge_to_exact(golden):
    # bdf.py's dt=0.05 and dt=0.0125 runs and the matrix-exponential solution.
    g = golden
    for dt, key in ((0.05, "bdf_dt0.05_t1"), (0.0125, "bdf_dt0.0125_t1")):
        y, t, h = oracle.tridiag_run(g["a"], g["b"], g["c"], g["k"], g["y0"], 0.0, dt, t_end=1.0)
        np.testing.assert_allclose(y, g[key], rtol=0, atol=1e-12)
    err1 = np.linalg.norm(np.array(g["bdf_dt0.05_t1"]) - g["exact_t1"])
    err2 = np.linalg.norm(np.array(g["bdf_dt0.0125_t1"]) - g["exact_t1"])
    assert 1.8 < np.log(err1 / err2) / np.log(4.0) < 2.2  # second order


# ---- test/test_diffusionSystem.cpp ---------------------------------------

NP = 401
DCOEF = 0.1


def _run(x, B, D, y0, t0, h, t1, alpha=0):
    return oracle.diffusion_system(x, B, D, y0, t0, t1, alpha=alpha, h=h)


def test_constant():
    x = np.linspace(-2, 2, NP)
    B, D = np.ones(NP), np.full(NP, DCOEF)
    y0 = np.full(NP, 5.0)
    a, b, c, k = oracle.diffusion_matrix(x, B, D)
    ydot = np.zeros(NP)
    ydot[0] = b[0] * y0[0] + c[0] * y0[1] + k[0]
    ydot[1:-1] = a[1:-1] * y0[:-2] + b[1:-1] * y0[1:-1] + c[1:-1] * y0[2:] + k[1:-1]
    ydot[-1] = a[-1] * y0[-2] + b[-1] * y0[-1] + k[-1]
    np.testing.assert_allclose(ydot, 0.0, atol=1e-11)
    y1 = _run(x, B, D, y0, 0.0, 0.01, 1.0)
    np.testing.assert_allclose(y1, y0, atol=1e-11)


def test_gaussian():
    x = np.linspace(-2, 2, NP)
    t0, t = 0.2, 0.3
    y0 = np.exp(-x * x / (4 * DCOEF * t0))
    y1 = _run(x, np.ones(NP), np.full(NP, DCOEF), y0, t0, 0.001, t)
    exact = np.sqrt(t0 / t) * np.exp(-x * x / (4 * DCOEF * t))
    np.testing.assert_allclose(y1, exact, atol=1e-4)


def test_cylindrical():
    x = np.linspace(0, 2, NP)
    t0, t = 0.7, 0.8
    y0 = np.exp(-x * x / (4 * DCOEF * t0))
    y1 = _run(x, np.ones(NP), np.full(NP, DCOEF), y0, t0, 0.001, t, alpha=1)
    exact = t0 / t * np.exp(-x * x / (4 * DCOEF * t))
    np.testing.assert_allclose(y1[1:], exact[1:], atol=2e-4)


@pytest.mark.parametrize("variable", [False, True])
def test_superposition(variable):
    x = np.linspace(-2, 2, NP)
    if variable:
        D, B = 0.1 + 0.02 * x, 1 + 0.5 * x * x
    else:
        D, B = np.full(NP, DCOEF), np.ones(NP)
    ya, yb = np.cos(np.pi * x), np.sin(np.pi * x / 4.0)
    ra = _run(x, B, D, ya, 0, 0.001, 0.1)
    rb = _run(x, B, D, yb, 0, 0.001, 0.1)
    r = _run(x, B, D, ya + yb, 0, 0.001, 0.1)
    np.testing.assert_allclose(ra + rb, r, atol=1e-12)


def test_timestep_independence():
    x = np.linspace(-2, 2, NP)
    D, B = 0.1 + 0.02 * x, 1 + 0.5 * x * x
    y0 = np.cos(np.pi * x) + np.exp(-x * x / (4 * DCOEF * 0.2))
    ra = _run(x, B, D, y0, 0, 0.001, 0.1)
    rb = _run(x, B, D, y0, 0, 0.0005, 0.1)
    np.testing.assert_allclose(ra, rb, atol=5e-6)


def test_step_size_rule():
    rng = np.random.default_rng(3)
    x = np.cumsum(rng.uniform(1e-5, 3e-5, 50))
    B, D = rng.uniform(0.5, 2, 50), rng.uniform(1e-5, 1e-4, 50)
    dlj = 0.5 * (x[2:] - x[:-2])
    expect = min(10 * np.min(dlj ** 2 / (B[1:-1] * D[1:-1])), 2e-5)
    assert oracle.diffusion_step_size(x, B, D, 10.0, 2e-5) == pytest.approx(expect, rel=1e-15)


def test_extended_precision_restatement_matches_oracle():
    # The extended-precision diffusion stage (used to measure accuracy on
    # badly scaled grids) agrees with the double-precision restatement to the
    # latter's rounding on a moderate grid, for every boundary condition.
    from oracle import extended
    rng = np.random.default_rng(5)
    for left in range(5):
        for right in (0, 1, 4):
            n = 60
            x = np.cumsum(np.full(n, 3e-5) * np.exp(rng.uniform(-0.2, 0.2, n)))
            B = np.exp(rng.uniform(-1, 1, n))
            D = np.exp(rng.uniform(np.log(1e-6), np.log(1e-3), n))
            S = rng.normal(size=n)
            y0 = np.cumsum(rng.normal(size=n))
            alpha = left % 2
            kw = dict(split_const=S, alpha=alpha, left_bc=left, right_bc=right, wall_const=1.5, y_inf=0.3)
            ref = oracle.diffusion_system(x, B, D, y0, 0.0, 1e-5, h=2e-6, **kw)
            ext = extended.diffusion_system(x, B, D, y0, 0.0, 1e-5, 2e-6, **kw)
            assert np.abs(ext - ref).max() <= 1e-13 * np.abs(ref).max(), (left, right)
