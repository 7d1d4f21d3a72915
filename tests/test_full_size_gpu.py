"""GPU parity at the full sizes of the benchmark configurations, through the
C ABI, against the CPU oracle on the same seeded inputs:

* the isolated source-term step: 4096 reactor states of the 150-species /
  1000-reaction synthetic mechanism and of the GRI-3.0-sized 53-species /
  325-reaction one, QSS and BDF, interp kinetics: every point bit for bit
  (end state, status and step / right-hand-side counters);
* the batched diffusion stage: 64 flames x 55 variables, N uniform in
  100..4000: the serial algorithm bit for bit, the warp-parallel one within
  1e-12 of each system's largest |y| (the tolerance of the tridiagonal path).

The states and flames are those bench.py times (same generators and seeds).
"""
import numpy as np
import pytest

import oracle
from oracle import chem
from ember_gb300 import _lib as L
from ember_gb300.diffusion import integrate_diffusion_terms, synthetic_flames
from ember_gb300.mechanism import reactor_states, synthetic_mechanism
from ember_gb300.source import BDF, QSS, GpuMechanism, SourceOptions, integrate_production_terms, KINETICS_INTERP

pytestmark = pytest.mark.gpu

N_STATES = 4096


def _mechanism(size):
    if size == 53:
        return synthetic_mechanism(n_species=53, n_reactions=325, seed=53325)
    return synthetic_mechanism(seed=150_1000)


@pytest.mark.parametrize("size", [150, 53])
@pytest.mark.parametrize("method", [QSS, BDF], ids=["qss", "bdf"])
def test_full_source_batch_bitwise(gpu_lib, size, method):
    mech = _mechanism(size)
    state, dt = reactor_states(mech, N_STATES, seed=4096)
    opts = SourceOptions.defaults(kinetics_model=KINETICS_INTERP)
    out, status, stats = integrate_production_terms(GpuMechanism(mech), method, state, dt, opts)
    ro, rs, rst = chem.OracleMech(mech).integrate(chem.QSS if method == QSS else chem.BDF, state, dt, opts)
    np.testing.assert_array_equal(status, rs)
    np.testing.assert_array_equal(stats, rst)
    same = np.all(out.view(np.int64) == ro.view(np.int64), axis=1)
    assert same.all(), f"{int((~same).sum())} of {N_STATES} points differ; max |diff| {np.abs(out - ro).max()}"
    # every point of these batches integrates without failure
    assert (status == 0).all()


def test_full_diffusion_batch(gpu_lib):
    grids, B, D, S, Y, h = synthetic_flames(seed=6455)
    ref = oracle.diffusion_batch(grids, B, D, S, Y, 0.0, 1e-5, h=h)
    serial, st_s = integrate_diffusion_terms(grids, B, D, S, Y.copy(), 0.0, 1e-5, h=h,
                                             algorithm=L.DIFFUSION_SERIAL)
    par, st_p = integrate_diffusion_terms(grids, B, D, S, Y.copy(), 0.0, 1e-5, h=h)
    assert (np.asarray(st_s) == 0).all() and (np.asarray(st_p) == 0).all()
    flat = lambda a: np.concatenate([np.asarray(v).reshape(-1) for v in a]) if isinstance(a, list) else a
    serial, par = flat(serial), flat(par)
    np.testing.assert_array_equal(serial, ref)
    nv = Y.size // sum(g.n_points for g in grids)
    p, worst = 0, 0.0
    for g in grids:
        for _ in range(nv):
            r = ref[p:p + g.n_points]
            worst = max(worst, float(np.abs(par[p:p + g.n_points] - r).max() / np.abs(r).max()))
            p += g.n_points
    assert worst <= 1e-12, worst
