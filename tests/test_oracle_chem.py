"""The CPU oracle's chemistry: its exp/log against the C library, its
kinetics against an independent numpy restatement of the same published
formulas, conservation properties, and its QSS integrator against the
reference's CHEMEQ2 cesium known-answer test
(test/old/test_qssintegrator.cpp)."""
import json
import os

import numpy as np
import pytest

from oracle import chem
from ember_gb300.mechanism import synthetic_mechanism, reactor_states
from ember_gb300.source import SourceOptions
import chem_numpy


@pytest.fixture(scope="module")
def mech():
    return synthetic_mechanism(n_species=40, n_reactions=200, seed=7)


@pytest.fixture(scope="module")
def omech(mech):
    return chem.OracleMech(mech)


def _ulps(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b) / np.spacing(np.abs(b))


def test_exp_log_accuracy():
    rng = np.random.default_rng(0)
    xs = np.concatenate([rng.uniform(-700, 700, 4000), rng.uniform(-1, 1, 2000), [0.0, 1e-300, -1e-20]])
    e = np.array([chem.exp(x) for x in xs])
    assert _ulps(e, np.exp(xs)).max() <= 2.0
    ys = np.exp(rng.uniform(-700, 700, 4000))
    ys = np.concatenate([ys, rng.uniform(0.5, 2.0, 2000), [1.0, 2.0, 1e-310, 5e-324]])
    lg = np.array([chem.log(y) for y in ys])
    ref = np.log(ys)
    nz = ref != 0
    assert _ulps(lg[nz], ref[nz]).max() <= 2.0
    assert chem.log(1.0) == 0.0
    assert chem.exp(-800.0) == 0.0 and np.isinf(chem.exp(710.0))


def test_kinetics_matches_numpy_restatement(mech, omech):
    st, _ = reactor_states(mech, 12, seed=3)
    T, Y = st[:, 1], st[:, 2:]
    # perturb compositions so every species is present
    Y = Y + 1e-4 * np.random.default_rng(1).uniform(0, 1, Y.shape)
    out = omech.gas_eval(T, Y, model=chem.KINETICS_STANDARD)
    for j in range(len(T)):
        ref = chem_numpy.rates(mech, T[j], Y[j])
        for key in ("creation", "destruction", "hk"):
            np.testing.assert_allclose(out[key][j], ref[key], rtol=1e-10, atol=1e-12 * np.abs(ref[key]).max())
        np.testing.assert_allclose(out["net"][j], ref["net"], rtol=1e-8,
                                   atol=1e-10 * np.abs(ref["creation"]).max())
        assert out["density"][j] == pytest.approx(ref["density"], rel=1e-14)
        assert out["cp_mass"][j] == pytest.approx(ref["cp_mass"], rel=1e-13)


def test_mass_and_element_conservation(mech, omech):
    st, _ = reactor_states(mech, 8, seed=4)
    Y = st[:, 2:] + 1e-5
    out = omech.gas_eval(st[:, 1], Y, model=chem.KINETICS_STANDARD)
    elems, E = mech.element_matrix()
    for j in range(8):
        net = out["net"][j]
        scale = np.abs(out["creation"][j]).max()
        assert abs(net @ mech.mol_weight) <= 1e-12 * scale * mech.mol_weight.max()
        assert np.abs(E @ net).max() <= 1e-11 * scale


def test_interp_model_close_to_standard(mech, omech):
    st, _ = reactor_states(mech, 8, seed=5)
    Y = st[:, 2:] + 1e-5
    a = omech.gas_eval(st[:, 1], Y, model=chem.KINETICS_STANDARD)
    b = omech.gas_eval(st[:, 1], Y, model=chem.KINETICS_INTERP)
    rel = np.abs(a["creation"] - b["creation"]) / (np.abs(a["creation"]) + 1e-30 * np.abs(a["creation"]).max())
    assert np.median(rel) < 1e-3
    # outside the table range (T > 3500 K) the interp model falls back to the formulas
    c = omech.gas_eval(np.full(2, 3600.0), Y[:2], model=chem.KINETICS_STANDARD)
    d = omech.gas_eval(np.full(2, 3600.0), Y[:2], model=chem.KINETICS_INTERP)
    np.testing.assert_array_equal(c["creation"], d["creation"])


def test_negative_mass_fractions_clipped_in_normalized_mode(mech, omech):
    st, _ = reactor_states(mech, 2, seed=6)
    Y = st[:, 2:].copy()
    Y[:, 5] = -1e-3
    a = omech.gas_eval(st[:, 1], Y, mode=chem.STATE_NORMALIZED)
    Yc = np.maximum(Y, 0)
    Yc /= Yc.sum(axis=1, keepdims=True)
    b = omech.gas_eval(st[:, 1], Yc, mode=chem.STATE_NORMALIZED)
    np.testing.assert_allclose(a["creation"], b["creation"], rtol=1e-13)


@pytest.fixture(scope="module")
def cesium(golden_dir):
    with open(os.path.join(golden_dir, "qss_cesium.json")) as f:
        return json.load(f)


def test_qss_cesium_known_answer(cesium):
    """CHEMEQ2 cesium problem: the error against the reference's converged
    final values shrinks with epsmin (first order) and is small in absolute
    terms; settings of test/old/test_qssintegrator.cpp (itermax 5, ymin 1e-20)
    with the QssIntegrator constructor defaults for the rest."""
    yi, yf = np.array(cesium["YI"]), np.array(cesium["YF"])
    errs = []
    for eps in cesium["eps_cases"]:
        y, r, stats = chem.qss_cesium(yi, cesium["t_final"], eps, itermax=cesium["itermax"])
        assert r == 0
        rel = np.abs(y - yf) / np.minimum(y, yf)
        errs.append(np.sqrt(np.sum(rel ** 2) / 6))
        assert errs[-1] < 0.1 * eps, (eps, errs[-1])
    assert errs[-1] < 2e-7
    assert all(b < a for a, b in zip(errs, errs[1:]))


def test_qss_source_points_run(mech, omech):
    st, dt = reactor_states(mech, 16, seed=8)
    opts = SourceOptions.defaults(kinetics_model=chem.KINETICS_STANDARD)
    out, status, stats = omech.integrate(chem.QSS, st, dt, opts, n_threads=4)
    assert (status == 0).all(), status
    assert np.isfinite(out).all()
    assert (stats[:, 0] > 0).all()
    np.testing.assert_allclose(out[:, 2:].sum(axis=1), 1.0, atol=1e-3)
    # U has no source without a split constant
    np.testing.assert_array_equal(out[:, 0], st[:, 0])


def test_qss_dtmin_failure_reported(mech, omech):
    st, dt = reactor_states(mech, 2, seed=9)
    opts = SourceOptions.defaults(kinetics_model=chem.KINETICS_STANDARD, qss_dtmin=1.0)
    out, status, stats = omech.integrate(chem.QSS, st, dt, opts, n_threads=1)
    assert (status == -1).all()


def test_bdf_matches_tight_radau(mech, omech):
    """The oracle's CVODE-path integrator against a converged implicit
    Runge-Kutta solution (scipy Radau, rtol 1e-11) of the same right-hand side
    (SourceSystemCVODE::f): final states within a small multiple of the
    configured tolerances (CvodeTolerances defaults: rtol 1e-6, atol U 1e-7,
    T 1e-8, Y 1e-13)."""
    from scipy.integrate import solve_ivp
    S = mech.n_species
    st, dt = reactor_states(mech, 4, seed=21)
    opts = SourceOptions.defaults(kinetics_model=chem.KINETICS_STANDARD)
    out, status, stats = omech.integrate(chem.BDF, st, dt, opts, n_threads=4)
    assert (status == 0).all(), status

    def f(t, y):
        r = omech.gas_eval(np.array([y[1]]), y[None, 2:], model=chem.KINETICS_STANDARD, mode=chem.STATE_NO_NORM)
        wn, hk, cp, rho = r["net"][0], r["hk"][0], r["cp_mass"][0], r["density"][0]
        yd = np.zeros_like(y)
        yd[1] = -(wn @ hk) / (rho * cp)
        yd[2:] = wn * mech.mol_weight / rho
        return yd

    tol = np.r_[1e-7, 1e-8, np.full(S, 1e-13)]
    for j in range(len(st)):
        ref = solve_ivp(f, (0, dt[j]), st[j], method="Radau", rtol=1e-11, atol=1e-18).y[:, -1]
        err = np.abs(out[j] - ref) / (1e-6 * np.abs(ref) + tol)
        assert err.max() < 50.0, (j, err.max())
        assert abs(out[j, 1] - ref[1]) < 1e-4 * ref[1]


def test_bdf_split_constants_and_failures(mech, omech):
    st, dt = reactor_states(mech, 3, seed=22)
    split = np.zeros_like(st)
    split[:, 0] = 5.0
    opts = SourceOptions.defaults(kinetics_model=chem.KINETICS_INTERP)
    out, status, stats = omech.integrate(chem.BDF, st, dt, opts, split_const=split, n_threads=1)
    assert (status == 0).all()
    np.testing.assert_allclose(out[:, 0], st[:, 0] + 5.0 * dt, rtol=1e-6)
    opts = SourceOptions.defaults(bdf_max_num_steps=3)
    out, status, stats = omech.integrate(chem.BDF, st, dt, opts, n_threads=1)
    assert (status == -11).all()
