"""Profile and time-series output of a batch of flames.

Host-side counterpart of the reference's ``StateWriter`` and
``TimeSeriesWriter`` (python/ember/output.py:7-130) for
:class:`~ember_gb300.split.FlameBatchSplitSolver`: every flame of the batch
gets its own directory ``<out_dir>/flame<NNN>/`` holding the files the
reference writes for one flame -- ``prof<NNNNNN>.<ext>`` profiles and a
time-series file -- with the reference's key names, in ``.npz`` (numpy) or
``.h5`` (h5py, where installed). Profiles carry what the batch solver holds:

* ``t``, ``P``, ``fileNumber``, ``x``, ``T``, ``U``, ``Y`` (species x points,
  as the reference), ``gridAlpha``, and with a convection stage attached the
  strain rate ``a`` and ``dadt`` (LinearFunction or ChebyshevFunction,
  src/scalarFunction.cpp);
* ``q`` (heat release rate per point) and ``rho`` (heatReleaseRate option);
* ``dUdtDiff``/``dTdtDiff``/``dYdtDiff`` and ``...Prod`` (timeDerivatives
  option): the time derivatives behind the next step's split constants.

The time series holds per flame ``t``, ``dt``, ``Q`` (integrated heat
release rate), ``Sc`` (consumption speed, when the unburned state is given),
``xFlame`` (the qdot-weighted flame position, FlameSolver::getFlamePosition,
src/flameSolver.cpp:963-966), ``a`` and ``dadt``.
"""
from __future__ import annotations

import os

import numpy as np


class OutputFile:
    """One output file (python/ember/output.py:7-30): a dict written as
    ``.npz`` on exit, or an h5py File for ``.h5``."""

    def __init__(self, filename: str):
        self.filename = filename

    def __enter__(self):
        if self.filename.endswith(".h5"):
            import h5py
            os.makedirs(os.path.dirname(self.filename) or ".", exist_ok=True)
            self.data = h5py.File(self.filename, mode="a")
        elif self.filename.endswith(".npz"):
            self.data = {}
        else:
            raise ValueError(f"unknown output file format for {self.filename!r}: expected .h5 or .npz")
        return self.data

    def __exit__(self, exc_type, exc_val, exc_tb):
        if self.filename.endswith(".h5"):
            self.data.close()
        elif exc_type is None:
            os.makedirs(os.path.dirname(self.filename) or ".", exist_ok=True)
            np.savez_compressed(self.filename, **self.data)


def strain(flame, t: float):
    """(a, da/dt) of a convection flame's strain function at time t:
    LinearFunction or ChebyshevFunction (src/scalarFunction.cpp:12-87; the
    Chebyshev derivative with the reference's recurrence, coefficient i
    weighted by i U_i(x))."""
    if getattr(flame, "strain_type", 0) == 1:
        c = [float(v) for v in flame.cheb] + [0.0, 0.0]
        n = max(len(flame.cheb), 2)
        x = (2 * (t - flame.cheb_t0)) / (flame.cheb_t1 - flame.cheb_t0) - 1
        cm, cn, y = 1.0, x, c[0] + x * c[1]
        for i in range(2, n):
            cp = (2 * x) * cn - cm
            y += cp * c[i]
            cm, cn = cn, cp
        cm, cn, dydx = 1.0, 2 * x, c[1]
        for i in range(2, n):
            cp = (2 * x) * cn - cm
            dydx += (i * cp) * c[i]
            cm, cn = cn, cp
        return y, dydx * (2.0 / (flame.cheb_t1 - flame.cheb_t0))
    a0, a1, t0, dt = flame.strain_initial, flame.strain_final, flame.strain_t0, flame.strain_dt
    if t <= t0:
        a = a0
    elif t >= t0 + dt:
        a = a1
    else:
        a = a0 + (a1 - a0) * (t - t0) / dt
    dadt = (a1 - a0) / dt if (t >= t0 and t < t0 + dt) else 0.0
    return a, dadt


def trapz(x, y):
    """mathUtils::trapz: the trapezoid rule over the grid."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    return float(np.sum(0.5 * (y[1:] + y[:-1]) * np.diff(x)))


class _BatchView:
    """The batch solver's current state split per flame."""

    def __init__(self, solver):
        self.solver = solver
        self.state, self.t = solver.state()
        self.offs = np.cumsum([0] + [g.n_points for g in solver.grids])
        self._qdot = None

    def flame(self, f):
        return self.state[self.offs[f]:self.offs[f + 1]]

    def qdot(self):
        if self._qdot is None:
            self._qdot = np.asarray(self.solver.objectives()[0])
        return self._qdot

    def flame_qdot(self, f):
        return self.qdot()[self.offs[f]:self.offs[f + 1]]


def _flame_dir(out_dir: str, f: int) -> str:
    return os.path.join(out_dir, f"flame{f:03d}")


class StateWriter:
    """Profiles of every flame of a batch (python/ember/output.py:71-130).

    ``writer()`` writes ``prof<N>.<ext>`` with the next file number into each
    flame's directory, ``writer(name)`` writes ``<name>.<ext>``; returns the
    file names."""

    def __init__(self, solver, out_dir: str, file_extension: str = "npz", first_file_number: int = 1,
                 pressure: float = 101325.0, heat_release_rate: bool = True, time_derivatives: bool = True):
        self.solver = solver
        self.out_dir = out_dir
        self.ext = file_extension
        self.file_number = first_file_number - 1
        self.pressure = float(pressure)
        self.heat_release_rate = heat_release_rate
        self.time_derivatives = time_derivatives

    def __call__(self, name: str | None = None):
        from .split import mixture_properties
        if not name:
            self.file_number += 1
            base = f"prof{self.file_number:06d}"
        else:
            base = name
        view = _BatchView(self.solver)
        mech = self.solver.gmech.mech
        flames = getattr(self.solver, "_convection", None)
        derivs = self.solver.derivatives() if self.time_derivatives else None
        names = []
        for f, g in enumerate(self.solver.grids):
            st = view.flame(f)
            filename = os.path.join(_flame_dir(self.out_dir, f), f"{base}.{self.ext}")
            if os.path.exists(filename):
                os.remove(filename)
            with OutputFile(filename) as data:
                data["t"] = view.t
                data["P"] = self.pressure
                data["fileNumber"] = self.file_number
                data["x"] = np.asarray(g.x, dtype=np.float64)
                data["T"] = st[:, 1].copy()
                data["U"] = st[:, 0].copy()
                data["Y"] = st[:, 2:].T.copy()
                data["gridAlpha"] = int(g.alpha)
                if flames is not None:
                    a, dadt = strain(flames[f], view.t)
                    data["a"] = a
                    data["dadt"] = dadt
                if self.heat_release_rate:
                    data["q"] = view.flame_qdot(f).copy()
                    data["rho"] = mixture_properties(mech, st, self.pressure)[0]
                if derivs is not None:
                    a, b = view.offs[f], view.offs[f + 1]
                    for label, d in (("Diff", derivs[0]), ("Prod", derivs[1])):
                        data[f"dUdt{label}"] = d[a:b, 0].copy()
                        data[f"dTdt{label}"] = d[a:b, 1].copy()
                        data[f"dYdt{label}"] = d[a:b, 2:].T.copy()
            names.append(filename)
        return names


class TimeSeriesWriter:
    """Integral flame properties over time for every flame of a batch
    (python/ember/output.py:33-69). Call after each step to record; with
    ``flag`` the series so far is written to ``<name>.<ext>`` in each flame's
    directory. ``rho_u``, ``ju``, ``jb`` (per flame: unburned density and the
    unburned / burned point) give the consumption speed."""

    def __init__(self, solver, out_dir: str, file_extension: str = "npz", rho_u=None, ju=None, jb=None):
        self.solver = solver
        self.out_dir = out_dir
        self.ext = file_extension
        self.rho_u, self.ju, self.jb = rho_u, ju, jb
        nf = len(solver.grids)
        self.series = [{k: [] for k in ("t", "dt", "Q", "Sc", "xFlame", "a", "dadt")} for _ in range(nf)]

    def record(self):
        view = _BatchView(self.solver)
        last = self.series[0]["t"]
        if last and last[-1] == view.t:
            return
        have_sc = self.rho_u is not None
        if have_sc:
            qdot, hr, sc = self.solver.objectives(self.rho_u, self.ju, self.jb)
        else:
            qdot, hr, sc = self.solver.objectives()
        qdot = np.asarray(qdot)
        flames = getattr(self.solver, "_convection", None)
        for f, g in enumerate(self.solver.grids):
            s = self.series[f]
            q = qdot[view.offs[f]:view.offs[f + 1]]
            x = np.asarray(g.x, dtype=np.float64)
            s["t"].append(view.t)
            s["dt"].append(self.solver.dt)
            s["Q"].append(float(hr[f]))
            s["Sc"].append(float(sc[f]) if have_sc else float("nan"))
            den = trapz(x, q)
            s["xFlame"].append(trapz(x, x * q) / den if den != 0.0 else float("nan"))
            a, dadt = strain(flames[f], view.t) if flames is not None else (0.0, 0.0)
            s["a"].append(a)
            s["dadt"].append(dadt)

    def __call__(self, name: str = "out", flag: bool = True):
        self.record()
        if not flag:
            return []
        names = []
        for f, s in enumerate(self.series):
            filename = os.path.join(_flame_dir(self.out_dir, f), f"{name}.{self.ext}")
            if os.path.exists(filename):
                os.remove(filename)
            with OutputFile(filename) as data:
                for k, v in s.items():
                    data[k] = np.asarray(v, dtype=np.float64)
            names.append(filename)
        return names
