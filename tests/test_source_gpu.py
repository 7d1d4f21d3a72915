"""GPU parity of the chemistry source term through the C ABI: thermo/rates
(ember_gas_eval) and the QSS source-term integrator (ember_source_integrate)
against the CPU oracle, bit for bit, plus the device QSS integrator on the
reference's CHEMEQ2 cesium known-answer test."""
import ctypes as C
import json
import os

import numpy as np
import pytest

from oracle import chem
from ember_gb300 import _lib as L
from ember_gb300.mechanism import synthetic_mechanism, reactor_states
from ember_gb300.source import (GpuMechanism, SourceOptions, integrate_production_terms, QSS,
                                KINETICS_STANDARD, KINETICS_INTERP, STATE_NORMALIZED, STATE_NO_NORM)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small_mech():
    return synthetic_mechanism(n_species=40, n_reactions=200, seed=7)


@pytest.fixture(scope="module")
def big_mech():
    return synthetic_mechanism()  # 150 species, 1000 reactions


@pytest.fixture(scope="module")
def pair_small(gpu_lib, small_mech):
    return GpuMechanism(small_mech), chem.OracleMech(small_mech)


@pytest.fixture(scope="module")
def pair_big(gpu_lib, big_mech):
    return GpuMechanism(big_mech), chem.OracleMech(big_mech)


def _states(mech, n, seed):
    st, dt = reactor_states(mech, n, seed=seed)
    rng = np.random.default_rng(seed)
    st[:, 2:] += 1e-6 * rng.uniform(0, 1, st[:, 2:].shape)
    return st, dt


@pytest.mark.parametrize("model", [KINETICS_STANDARD, KINETICS_INTERP])
@pytest.mark.parametrize("mode", [STATE_NORMALIZED, STATE_NO_NORM])
def test_gas_eval_bitwise(pair_small, small_mech, model, mode):
    g, o = pair_small
    st, _ = _states(small_mech, 48, seed=11)
    T = st[:, 1].copy()
    T[:3] = [250.0, 3500.0, 3900.0]  # below / at / above the table range
    Y = st[:, 2:].copy()
    Y[5, 3] = -1e-4  # a negative mass fraction
    a = g.gas_eval(T, Y, model=model, mode=mode)
    b = o.gas_eval(T, Y, model=model, mode=mode)
    for key in ("creation", "destruction", "net", "hk", "cp_mass", "density"):
        np.testing.assert_array_equal(a[key], b[key], err_msg=key)


def test_gas_eval_big_mechanism_bitwise(pair_big, big_mech):
    g, o = pair_big
    st, _ = _states(big_mech, 64, seed=12)
    for model in (KINETICS_STANDARD, KINETICS_INTERP):
        a = g.gas_eval(st[:, 1], st[:, 2:], model=model)
        b = o.gas_eval(st[:, 1], st[:, 2:], model=model)
        for key in ("creation", "destruction", "net", "hk", "cp_mass", "density"):
            np.testing.assert_array_equal(a[key], b[key], err_msg=key)


@pytest.mark.parametrize("model", [KINETICS_STANDARD, KINETICS_INTERP])
def test_qss_bitwise_vs_oracle(pair_small, small_mech, model):
    g, o = pair_small
    st, dt = _states(small_mech, 96, seed=13)
    opts = SourceOptions.defaults(kinetics_model=model)
    out, status, stats = integrate_production_terms(g, QSS, st, dt, opts)
    ro, rs, rst = o.integrate(chem.QSS, st, dt, opts)
    np.testing.assert_array_equal(status, rs)
    np.testing.assert_array_equal(stats, rst)
    np.testing.assert_array_equal(out, ro)


def test_qss_big_mechanism_bitwise(pair_big, big_mech):
    g, o = pair_big
    st, dt = _states(big_mech, 48, seed=14)
    opts = SourceOptions.defaults(kinetics_model=KINETICS_INTERP)
    out, status, stats = integrate_production_terms(g, QSS, st, dt, opts)
    ro, rs, rst = o.integrate(chem.QSS, st, dt, opts)
    assert (status == 0).all()
    np.testing.assert_array_equal(stats, rst)
    np.testing.assert_array_equal(out, ro)


def test_qss_split_constants_multipliers_igniter(pair_small, small_mech):
    g, o = pair_small
    st, dt = _states(small_mech, 32, seed=15)
    rng = np.random.default_rng(15)
    split = rng.normal(scale=1e-2, size=st.shape)
    split[:, 0] = rng.normal(scale=10.0, size=len(st))
    split[:, 1] = rng.normal(scale=1e4, size=len(st))
    x = rng.uniform(-1e-3, 1e-3, len(st))
    mult = np.exp(rng.normal(scale=0.3, size=small_mech.n_reactions))
    g.set_multipliers(mult)
    o.set_multipliers(mult)
    try:
        opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD, ignition_energy=5e6, ignition_tstart=0.0,
                                      ignition_duration=1e-3, ignition_center=0.0, ignition_stddev=3e-4)
        out, status, stats = integrate_production_terms(g, QSS, st, dt, opts, split_const=split, t_start=1e-4, x=x)
        ro, rs, rst = o.integrate(chem.QSS, st, dt, opts, split_const=split, t_start=1e-4, x=x)
        np.testing.assert_array_equal(status, rs)
        np.testing.assert_array_equal(out, ro)
    finally:
        g.set_multipliers(None)
        o.set_multipliers(None)


def test_qss_device_memory_path(pair_small, small_mech):
    torch = pytest.importorskip("torch")
    g, _ = pair_small
    st, dt = _states(small_mech, 40, seed=16)
    opts = SourceOptions.defaults()
    host, hs, _ = integrate_production_terms(g, QSS, st, dt, opts)
    dev, ds, _ = integrate_production_terms(g, QSS, torch.as_tensor(st, device="cuda"),
                                            torch.as_tensor(dt, device="cuda"), opts)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(dev.cpu().numpy(), host)
    np.testing.assert_array_equal(ds.cpu().numpy(), hs)


def test_qss_failures_reported(pair_small, small_mech):
    g, o = pair_small
    st, dt = _states(small_mech, 8, seed=17)
    opts = SourceOptions.defaults(qss_dtmin=1.0)
    out, status, _ = integrate_production_terms(g, QSS, st, dt, opts)
    assert (np.asarray(status) == -1).all()
    opts = SourceOptions.defaults(max_steps=3)
    out, status, stats = integrate_production_terms(g, QSS, st, dt, opts)
    ro, rs, _ = o.integrate(chem.QSS, st, dt, opts)
    np.testing.assert_array_equal(status, rs)
    assert (np.asarray(status) == -20).any()
    np.testing.assert_array_equal(out, ro)


def test_qss_cesium_known_answer_on_gpu(gpu_lib, golden_dir):
    with open(os.path.join(golden_dir, "qss_cesium.json")) as f:
        ces = json.load(f)
    yi, yf = np.array(ces["YI"]), np.array(ces["YF"])
    for eps in ces["eps_cases"]:
        y = yi.copy()
        stats = np.zeros(4, dtype=np.int32)
        r = gpu_lib.ember_selftest_qss_cesium(eps, 20.0, 1e-15, 1e300, 1e-8, ces["itermax"], 1, ces["t_final"],
                                              10_000_000, y.ctypes.data, stats.ctypes.data)
        assert r == 0
        yo, ro, so = chem.qss_cesium(yi, ces["t_final"], eps, itermax=ces["itermax"])
        np.testing.assert_array_equal(y, yo)
        np.testing.assert_array_equal(stats, so)
        rel = np.abs(y - yf) / np.minimum(y, yf)
        assert np.sqrt(np.sum(rel ** 2) / 6) < 0.1 * eps


@pytest.mark.parametrize("model", [KINETICS_STANDARD, KINETICS_INTERP])
def test_bdf_bitwise_vs_oracle(pair_small, small_mech, model):
    from ember_gb300.source import BDF
    g, o = pair_small
    st, dt = _states(small_mech, 24, seed=31)
    opts = SourceOptions.defaults(kinetics_model=model)
    out, status, stats = integrate_production_terms(g, BDF, st, dt, opts)
    ro, rs, rst = o.integrate(chem.BDF, st, dt, opts)
    np.testing.assert_array_equal(status, rs)
    np.testing.assert_array_equal(stats, rst)
    np.testing.assert_array_equal(out, ro)


def test_bdf_big_mechanism_bitwise(pair_big, big_mech):
    from ember_gb300.source import BDF
    g, o = pair_big
    st, dt = _states(big_mech, 8, seed=32)
    opts = SourceOptions.defaults(kinetics_model=KINETICS_INTERP)
    out, status, stats = integrate_production_terms(g, BDF, st, dt, opts)
    ro, rs, rst = o.integrate(chem.BDF, st, dt, opts)
    assert (status == 0).all()
    np.testing.assert_array_equal(stats, rst)
    np.testing.assert_array_equal(out, ro)


def test_bdf_split_igniter_failures(pair_small, small_mech):
    from ember_gb300.source import BDF
    g, o = pair_small
    st, dt = _states(small_mech, 12, seed=33)
    rng = np.random.default_rng(33)
    split = rng.normal(scale=1e-2, size=st.shape)
    split[:, 1] = rng.normal(scale=1e4, size=len(st))
    x = rng.uniform(-1e-3, 1e-3, len(st))
    opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD, ignition_energy=5e6, ignition_duration=1e-3,
                                  ignition_stddev=3e-4)
    out, status, stats = integrate_production_terms(g, BDF, st, dt, opts, split_const=split, t_start=1e-4, x=x)
    ro, rs, rst = o.integrate(chem.BDF, st, dt, opts, split_const=split, t_start=1e-4, x=x)
    np.testing.assert_array_equal(status, rs)
    np.testing.assert_array_equal(out, ro)
    opts = SourceOptions.defaults(bdf_max_num_steps=5)
    out, status, stats = integrate_production_terms(g, BDF, st, dt, opts)
    ro, rs, rst = o.integrate(chem.BDF, st, dt, opts)
    np.testing.assert_array_equal(status, rs)
    assert (np.asarray(status) == -11).any()
    np.testing.assert_array_equal(out, ro)


@pytest.mark.parametrize("method", ["qss", "bdf"])
def test_empty_and_single_point_batches(pair_small, small_mech, method):
    # Edge sizes: an empty batch is a no-op; one point alone gives the same
    # bits as that point inside a batch (no cross-point state).
    from ember_gb300.source import BDF
    m = QSS if method == "qss" else BDF
    g, o = pair_small
    st, dt = _states(small_mech, 5, seed=44)
    opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD)
    out0, status0, stats0 = integrate_production_terms(g, m, st[:0], dt[:0], opts)
    assert out0.shape == (0, st.shape[1]) and status0.size == 0
    full, fst, fstats = integrate_production_terms(g, m, st, dt, opts)
    for j in (0, 4):
        one, ost, ostats = integrate_production_terms(g, m, st[j:j + 1], dt[j:j + 1], opts)
        assert np.array_equal(one[0], full[j]) and ost[0] == fst[j]
        assert np.array_equal(ostats[0], fstats[j])


def test_qss_results_do_not_depend_on_the_launch_width(gpu_lib, big_mech):
    # every reduction runs in one 32-lane order, so each width gives the
    # oracle's bits
    from ember_gb300.source import THREAD_CHOICES
    g, o = GpuMechanism(big_mech), chem.OracleMech(big_mech)
    st, dt = _states(big_mech, 40, seed=21)
    opts = SourceOptions.defaults(kinetics_model=KINETICS_INTERP)
    ro, rs, rst = o.integrate(chem.QSS, st, dt, opts)
    for width in THREAD_CHOICES:
        out, status, stats = integrate_production_terms(g, QSS, st, dt,
                                                        SourceOptions.defaults(kinetics_model=KINETICS_INTERP,
                                                                               threads_per_point=width))
        np.testing.assert_array_equal(status, rs, err_msg=str(width))
        assert np.array_equal(out, ro), (width, np.abs(out - ro).max())
        np.testing.assert_array_equal(stats[:, :3], rst[:, :3], err_msg=str(width))


def test_autotune_keeps_the_fastest_width_and_the_results(gpu_lib, small_mech):
    from ember_gb300.source import THREAD_CHOICES, BDF, autotune
    g, o = GpuMechanism(small_mech), chem.OracleMech(small_mech)
    st, dt = _states(small_mech, 200, seed=22)
    opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD)
    width, ms = autotune(g, QSS, st, dt, opts)
    assert width in THREAD_CHOICES and width in ms
    assert set(ms) == set(THREAD_CHOICES) and all(v > 0 for v in ms.values())
    assert ms[width] == min(ms.values())
    out, status, _ = integrate_production_terms(g, QSS, st, dt, opts)  # threads_per_point 0: the tuned width
    ro, rs, _ = o.integrate(chem.QSS, st, dt, opts)
    np.testing.assert_array_equal(status, rs)
    assert np.array_equal(out, ro)
    # BDF: widths 32/64/128/160/256 x the matrix placements that fit
    bw, bms = autotune(g, BDF, st[:16], dt[:16], opts)
    assert bw in (32, 64, 128, 160, 256) and set(bms) == {32, 64, 128, 160, 256}
    with pytest.raises(L.EmberGpuError):
        integrate_production_terms(g, QSS, st, dt, SourceOptions.defaults(threads_per_point=48))


@pytest.mark.gpu
@pytest.mark.parametrize("n_species,n_reactions,seed", [(40, 200, 7), (150, 1000, 150_1000)])
def test_bdf_results_do_not_depend_on_width_or_matrix_placement(gpu_lib, n_species, n_reactions, seed):
    # every BDF launch configuration the autotuner can pick gives the oracle's bits
    import ctypes as C
    from ember_gb300.source import BDF, autotune
    m = synthetic_mechanism(n_species=n_species, n_reactions=n_reactions, seed=seed)
    g, o = GpuMechanism(m), chem.OracleMech(m)
    st, dt = _states(m, 12, seed=23)
    opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD)
    ro, rs, rst = o.integrate(chem.BDF, st, dt, opts)
    for width in (32, 64, 128, 160, 256):
        for layout in (0, 1, 2, 3, 4):
            try:
                out, status, stats = integrate_production_terms(
                    g, BDF, st, dt, SourceOptions.defaults(kinetics_model=KINETICS_STANDARD, threads_per_point=width,
                                                           bdf_layout=layout))
            except L.EmberGpuError:
                assert layout != 0    # a placement that does not fit this mechanism falls back or is refused
                continue
            np.testing.assert_array_equal(status, rs, err_msg=str((width, layout)))
            assert np.array_equal(out, ro), (width, layout, np.abs(out - ro).max())
    # the placement the autotuner keeps (it tries every one that fits)
    autotune(g, BDF, st, dt, opts)
    out, status, _ = integrate_production_terms(g, BDF, st, dt, opts)
    assert np.array_equal(out, ro)


@pytest.mark.gpu
@pytest.mark.parametrize("big", [False, True])
def test_qss_two_pass_schedule_gives_the_same_bits(gpu_lib, small_mech, big_mech, big):
    # points suspended after a few steps and resumed on wider CTAs reproduce
    # the one-pass integration (and the oracle) exactly, statistics included
    from ember_gb300.source import autotune, tuning
    m = big_mech if big else small_mech
    g, o = GpuMechanism(m), chem.OracleMech(m)
    st, dt = _states(m, 40, seed=31)
    base = dict(kinetics_model=KINETICS_INTERP)
    ro, rs, rst = o.integrate(chem.QSS, st, dt, SourceOptions.defaults(**base))
    for cap, tw in ((1, 256), (5, 128), (20, 32)):
        out, status, stats = integrate_production_terms(
            g, QSS, st, dt, SourceOptions.defaults(qss_tail_steps=cap, qss_tail_threads=tw, **base))
        np.testing.assert_array_equal(status, rs, err_msg=str(cap))
        assert np.array_equal(out, ro), (cap, np.abs(out - ro).max())
        np.testing.assert_array_equal(stats[:, :3], rst[:, :3])
    # whatever schedule the autotuner keeps
    autotune(g, QSS, st, dt, SourceOptions.defaults(**base))
    t = tuning(g)
    assert t["qss_threads"] in (32, 64, 96, 128, 160, 192, 256)
    out, status, _ = integrate_production_terms(g, QSS, st, dt, SourceOptions.defaults(**base))
    assert np.array_equal(out, ro)
    with pytest.raises(L.EmberGpuError):
        integrate_production_terms(g, QSS, st, dt, SourceOptions.defaults(qss_tail_steps=5, qss_stability_check=1))
