"""Profile and time-series writers of a flame batch (python/ember/output.py:
33-130): file layout, key names and shapes, the strain function and the
flame position, on a stand-in solver (no GPU)."""
import os

import numpy as np
import pytest

from ember_gb300.convection import ConvectionFlame
from ember_gb300.diffusion import FlameGrid
from ember_gb300.mechanism import synthetic_mechanism
from ember_gb300.output import StateWriter, TimeSeriesWriter, strain, trapz


class _Mech:
    def __init__(self, mech):
        self.mech = mech


class FakeSolver:
    """The parts of FlameBatchSplitSolver the writers read."""

    def __init__(self, mech, sizes, seed=0):
        rng = np.random.default_rng(seed)
        self.gmech = _Mech(mech)
        self.grids = [FlameGrid(x=np.sort(rng.uniform(-1e-2, 1e-2, n)), alpha=f % 2) for f, n in enumerate(sizes)]
        S = mech.n_species
        n = sum(sizes)
        st = np.empty((n, S + 2))
        st[:, 0] = rng.uniform(0, 5, n)
        st[:, 1] = rng.uniform(300, 2000, n)
        y = rng.uniform(0, 1, (n, S))
        st[:, 2:] = y / y.sum(axis=1, keepdims=True)
        self._state, self.t, self.dt = st, 1.5e-3, 2e-5
        self._qdot = rng.uniform(0, 1e8, n)
        self._convection = [ConvectionFlame(n_points=m, strain_initial=100.0 * (f + 1), strain_final=400.0,
                                            strain_t0=1e-3, strain_dt=1e-3) for f, m in enumerate(sizes)]

    def state(self):
        return self._state.copy(), self.t

    def objectives(self, rho_u=None, ju=None, jb=None):
        offs = np.cumsum([0] + [g.n_points for g in self.grids])
        hr = np.array([trapz(g.x, self._qdot[offs[f]:offs[f + 1]]) for f, g in enumerate(self.grids)])
        sc = hr * 1e-6 if rho_u is not None else None
        return self._qdot.copy(), hr, sc

    def derivatives(self):
        return self._state * 2.0, self._state * 3.0


def test_strain_is_the_linear_function():
    fl = ConvectionFlame(n_points=3, strain_initial=100.0, strain_final=300.0, strain_t0=1.0, strain_dt=2.0)
    assert strain(fl, 0.5) == (100.0, 0.0)
    assert strain(fl, 1.0) == (100.0, 100.0)
    assert strain(fl, 2.0) == (200.0, 100.0)
    assert strain(fl, 3.0) == (300.0, 0.0)
    assert strain(fl, 5.0) == (300.0, 0.0)


def test_state_writer_writes_one_profile_per_flame(tmp_path):
    mech = synthetic_mechanism(n_species=12, n_reactions=30, seed=1)
    s = FakeSolver(mech, [9, 14])
    w = StateWriter(s, str(tmp_path), first_file_number=1)
    names = w()
    assert [os.path.relpath(n, tmp_path) for n in names] == [os.path.join("flame000", "prof000001.npz"),
                                                             os.path.join("flame001", "prof000001.npz")]
    assert os.path.basename(w()[0]) == "prof000002.npz"
    assert os.path.basename(w("postAdapt")[1]) == "postAdapt.npz"
    d = np.load(names[1])
    st, _ = s.state()
    sl = slice(9, 23)
    assert float(d["t"]) == s.t and float(d["P"]) == 101325.0 and int(d["fileNumber"]) == 1
    np.testing.assert_array_equal(d["x"], s.grids[1].x)
    np.testing.assert_array_equal(d["T"], st[sl, 1])
    np.testing.assert_array_equal(d["U"], st[sl, 0])
    assert d["Y"].shape == (12, 14)
    np.testing.assert_array_equal(d["Y"], st[sl, 2:].T)
    assert int(d["gridAlpha"]) == 1
    assert (float(d["a"]), float(d["dadt"])) == strain(s._convection[1], s.t)
    np.testing.assert_array_equal(d["q"], s._qdot[sl])
    assert d["rho"].shape == (14,) and (d["rho"] > 0).all()
    np.testing.assert_array_equal(d["dTdtDiff"], 2.0 * st[sl, 1])
    np.testing.assert_array_equal(d["dYdtProd"], 3.0 * st[sl, 2:].T)


def test_time_series_records_each_time_once(tmp_path):
    mech = synthetic_mechanism(n_species=12, n_reactions=30, seed=1)
    s = FakeSolver(mech, [9, 14])
    w = TimeSeriesWriter(s, str(tmp_path), rho_u=np.ones(2), ju=np.zeros(2, int), jb=np.ones(2, int))
    w("out", flag=False)
    w("out", flag=False)          # same time: not recorded again
    s.t += s.dt
    names = w("out")
    d = np.load(names[0])
    assert list(d["t"]) == [1.5e-3, 1.5e-3 + 2e-5]
    x, q = s.grids[0].x, s._qdot[:9]
    assert d["xFlame"][0] == pytest.approx(np.trapezoid(x * q, x) / np.trapezoid(q, x), rel=1e-12)
    assert d["Q"][0] == pytest.approx(np.trapezoid(q, x), rel=1e-12)
    assert d["Sc"][0] == pytest.approx(1e-6 * d["Q"][0])
    assert d["a"][1] == strain(s._convection[0], s.t)[0]


@pytest.mark.gpu
def test_writers_on_a_gpu_batch(gpu_lib, tmp_path):
    # the real batch solver: profiles hold its state, the time series its objectives
    from ember_gb300 import _lib as L
    from ember_gb300.source import GpuMechanism, QSS, KINETICS_STANDARD, SourceOptions
    from ember_gb300.split import FlameBatchSplitSolver, flame_batch
    mech = synthetic_mechanism(n_species=20, n_reactions=60, seed=3)
    grids, state, B, D, rho_u, ju, jb = flame_batch(mech, n_flames=2, n_min=9, n_max=14, seed=5, width=2e-3,
                                                    thickness=3e-4)
    gm = GpuMechanism(mech)
    s = FlameBatchSplitSolver(gm, grids, 1e-6, method=QSS,
                              source_options=SourceOptions.defaults(kinetics_model=KINETICS_STANDARD),
                              diffusion_algorithm=L.DIFFUSION_SERIAL)
    s.set_state(0.0, state)
    s.set_transport(B, D)
    ts = TimeSeriesWriter(s, str(tmp_path), rho_u=rho_u, ju=ju, jb=jb)
    pw = StateWriter(s, str(tmp_path))
    for _ in range(3):
        s.step(1)
        ts("out", flag=False)
    names = pw()
    out, t = s.state()
    d = np.load(names[1])
    n0 = grids[0].n_points
    np.testing.assert_array_equal(d["T"], out[n0:, 1])
    assert float(d["t"]) == t
    q, hr, sc = s.objectives(rho_u, ju, jb)
    np.testing.assert_array_equal(d["q"], q[n0:])
    series = np.load(ts("out")[1])
    assert len(series["t"]) == 3 and series["Q"][-1] == hr[1] and series["Sc"][-1] == sc[1]
