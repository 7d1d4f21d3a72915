"""A batch of flames run to steady state: FlameSolver's step loop on the GPU.

:class:`FlameBatchRun` drives a :class:`~ember_gb300.split.FlameBatchSplitSolver`
the way FlameSolver::step / finishStep drive one flame
(src/flameSolver.cpp:240-365, checkTerminationCondition 377-425), for every
flame of a batch at once:

* each step: the split step on the GPU (one captured graph for the batch),
  then the heat release rate and consumption speed of every flame recorded
  (outputStepInterval = 1);
* every ``terminate_step_interval`` steps: the termination test of each
  flame -- the RMS variation of its heat release rate over the last
  ``steady_period`` against ``tolerance`` (relative) and ``abstol``
  (TerminationCondition, python/ember/input.py:864-874); flames that
  terminate leave the batch, which is rebuilt on the others;
* every ``regrid_step_interval`` steps: the regrid block of finishStep for
  every flame (:func:`~ember_gb300.grid.regrid_batch`: damping from the
  transport properties, boundary regrid or its unstrained form, interior
  adaptation, the state and the three time derivatives carried over, mass
  fractions renormalised), then the batch is rebuilt on the new grids. With
  the convection stage attached, the left mass flux rVzero and the continuity
  point follow the grid as in FlameSolver (V interpolated onto the new grid).

The batch is rebuilt (a new split handle, whose graph is captured at its
first step) only when grids or membership change.
"""
from __future__ import annotations

import copy
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from .grid import GridOptions, regrid_batch
from .output import strain
from .source import QSS
from .split import FlameBatchSplitSolver


class StepFailure(RuntimeError):
    """A split step whose diffusion or convection systems failed; ``run``
    is the FlameBatchRun (its solver holds the failed state, e.g. for a
    StateWriter error file)."""

    def __init__(self, message: str, run):
        super().__init__(message)
        self.run = run


@dataclass
class TerminationOptions:
    """TerminationCondition (python/ember/input.py:864-874) and the step
    intervals of the loop (python/ember/input.py:704-726)."""
    t_end: float = 0.8
    tolerance: float = 1e-4
    abstol: float = 0.5
    steady_period: float = 0.002
    t_min: float = 0.0
    terminate_step_interval: int = 10
    regrid_step_interval: int = 20


def heat_release_steady(t_hist, q_hist, t_now: float, opts: TerminationOptions):
    """FlameSolver::checkTerminationCondition for the "Q" measurement
    (src/flameSolver.cpp:377-412): (terminate, relative RMS variation,
    absolute RMS variation); the variations are None while the history is
    shorter than the steady period."""
    if t_now < opts.t_min:
        return False, None, None
    t = np.asarray(t_hist, dtype=np.float64)
    q = np.asarray(q_hist, dtype=np.float64)
    before = np.flatnonzero(t < t_now - opts.steady_period)
    if before.size == 0:
        return False, None, None
    j1, j2 = int(before[-1]), len(q) - 1
    seg = q[j1:j2 + 1]
    q_mean = float(np.mean(seg))
    err = float(np.sqrt(np.sum((seg - q_mean) ** 2)) / (j2 - j1 + 1))
    rel = err / abs(q_mean) if q_mean != 0.0 else float("inf")
    return (rel < opts.tolerance or err < opts.abstol), rel, err


@dataclass
class FlameRecord:
    """History and outcome of one flame of the batch."""
    t: list = field(default_factory=list)
    Q: list = field(default_factory=list)
    Sc: list = field(default_factory=list)
    steps: int = 0
    terminated: bool = False
    t_terminated: float | None = None
    rms_rel: float | None = None
    n_points: list = field(default_factory=list)


class FlameBatchRun:
    """Run a batch of flames towards steady state (see the module docstring).

    grids, state (point-major [n_points, S+2]), rho_u (unburned density per
    flame), unburned_left (per flame, default True: ju = 0, jb = N - 1),
    transport (GpuTransport: the device transport model of every step and
    the damping of the regrid), convection (flames, y_left, options) or
    None. strain_rates: per flame, for the damping and the choice between
    the strained and unstrained regrid when no convection stage is attached
    (with one, the flames' strain functions give them)."""

    def __init__(self, gmech, transport, grids, state, dt: float, rho_u, *, t_start: float = 0.0,
                 method: int = QSS, source_options=None, threshold: float = 1e-5, cross_terms: bool = True,
                 convection=None, unburned_left=None, strain_rates=None, termination: TerminationOptions | None = None,
                 grid_options: GridOptions | None = None, diffusion_algorithm: int = L.DIFFUSION_PARALLEL,
                 graph: bool = True, balanced: bool = True):
        self.gmech = gmech
        self.transport = transport
        self.dt = float(dt)
        self.method = method
        self.source_options = source_options
        self.threshold = threshold
        self.cross_terms = cross_terms
        self.termination = termination or TerminationOptions()
        self.grid_options = grid_options
        self.algorithm = diffusion_algorithm
        self.graph = graph
        self.balanced = balanced
        nf = len(grids)
        self.rho_u = np.asarray(rho_u, dtype=np.float64).reshape(nf)
        self.unburned_left = [True] * nf if unburned_left is None else [bool(u) for u in unburned_left]
        self.strain_rates = None if strain_rates is None else [float(a) for a in strain_rates]
        if convection is not None:
            flames, y_left, copts = convection
            self.conv_flames = [copy.copy(f) for f in flames]
            self.y_left = np.asarray(y_left, dtype=np.float64).reshape(nf, -1)
            self.conv_opts = copts
        else:
            self.conv_flames = None
        self.records = [FlameRecord() for _ in range(nf)]
        # the batch: flame indices and their grids, state, time, derivatives
        self.active = list(range(nf))
        self.grids = list(grids)
        self.t = float(t_start)
        self.solver = None
        self._build(np.asarray(state, dtype=np.float64), None)
        self.n_rebuilds = 0
        self.n_steps = 0
        self._since_term = self._since_regrid = 0   # steps since the last test / regrid (across run() calls)

    # -- the batch ---------------------------------------------------------
    def _offsets(self, grids):
        return np.cumsum([0] + [g.n_points for g in grids])

    def _ends(self, f, n):
        return (0, n - 1) if self.unburned_left[f] else (n - 1, 0)

    def _build(self, state, ddt):
        """A split handle on the active flames' grids."""
        grids = [self.grids[f] for f in self.active]
        if self.solver is not None:
            self.solver.close()
        s = FlameBatchSplitSolver(self.gmech, grids, self.dt, method=self.method,
                                  source_options=self.source_options, balanced=self.balanced,
                                  diffusion_algorithm=self.algorithm)
        n = s.n_points * s.n_vars
        s.set_state(self.t, state)
        s.set_transport(np.zeros(n), np.zeros(n))   # replaced by the transport model at every step
        s.set_transport_model(self.transport, self.threshold, self.cross_terms)
        if self.conv_flames is not None:
            s.set_convection([self.conv_flames[f] for f in self.active], self.y_left[self.active], self.conv_opts)
        if ddt is not None:
            s.set_derivatives(ddt[1], ddt[2], ddt[0] if self.conv_flames is not None else None)
        self.solver = s
        ends = [self._ends(f, g.n_points) for f, g in zip(self.active, grids)]
        self._ju = np.array([e[0] for e in ends], dtype=np.int32)
        self._jb = np.array([e[1] for e in ends], dtype=np.int32)

    def _strain_rate(self, f):
        if self.conv_flames is not None:
            return strain(self.conv_flames[f], self.t)[0]
        return self.strain_rates[f] if self.strain_rates is not None else 1.0

    def _record(self):
        _, hr, sc = self.solver.objectives(self.rho_u[self.active], self._ju, self._jb)
        for i, f in enumerate(self.active):
            r = self.records[f]
            r.t.append(self.t)
            r.Q.append(float(hr[i]))
            r.Sc.append(float(sc[i]))
            r.steps += 1
            r.n_points.append(self.grids[f].n_points)

    def _terminate(self):
        """Flames whose heat release rate is steady leave the batch."""
        keep = []
        for f in self.active:
            r = self.records[f]
            done, rel, _ = heat_release_steady(r.t, r.Q, self.t, self.termination)
            r.rms_rel = rel
            if done:
                r.terminated, r.t_terminated = True, self.t
            else:
                keep.append(f)
        if len(keep) == len(self.active):
            return
        state, _ = self.solver.state()
        ddt = self._derivatives()
        offs = self._offsets([self.grids[f] for f in self.active])
        sel = [i for i, f in enumerate(self.active) if f in keep]
        pick = lambda a: np.concatenate([a[offs[i]:offs[i + 1]] for i in sel]) if sel else a[:0]
        self.active = keep
        if keep:
            self._build(pick(state), tuple(None if d is None else pick(d) for d in ddt))
            self.n_rebuilds += 1

    def _derivatives(self):
        dd, dp = self.solver.derivatives()
        dc = self.solver.convection_derivative() if self.conv_flames is not None else None
        return dc, dd, dp

    def _regrid(self):
        """FlameSolver's regrid block for every active flame, then a new batch."""
        state, _ = self.solver.state()
        dc, dd, dp = self._derivatives()
        grids = [self.grids[f] for f in self.active]
        props = self.transport.eval(state[:, 1].copy(), state[:, 2:].copy(),
                                    self.source_options.pressure if self.source_options is not None else 101325.0,
                                    self.threshold)
        rates = [self._strain_rate(f) for f in self.active]
        qdot = None
        if any(a == 0.0 for a in rates):
            qdot = np.asarray(self.solver.objectives()[0])
        V = self.solver.velocity() if self.conv_flames is not None else None
        res = regrid_batch(grids, state, (dc, dd, dp), props, rates, self.grid_options, qdot=qdot)
        offs = self._offsets(grids)
        for i, f in enumerate(self.active):
            old, new = grids[i], res.grids[i]
            self.grids[f] = new
            if self.conv_flames is not None and res.updated[i]:
                # rVzero and the continuity point follow the grid (src/flameSolver.cpp:336-338)
                fl = self.conv_flames[f]
                xo, xn = np.asarray(old.x), np.asarray(new.x)
                v = V[offs[i]:offs[i + 1]]
                fl.n_points = new.n_points
                fl.rv_zero = float(np.interp(xn[0], xo, v))
                if fl.j_cont > 0:
                    fl.j_cont = int(min(np.searchsorted(xn, xo[min(fl.j_cont, old.n_points - 1)]),
                                        new.n_points - 1))
        if any(res.updated):
            self._build(res.state, res.ddt)
            self.n_rebuilds += 1

    # -- the loop ----------------------------------------------------------
    def run(self, max_steps: int, t_end: float | None = None):
        """Step until every flame has terminated, t_end (default the
        termination options' t_end) is reached, or max_steps steps. Returns
        the per-flame records."""
        t_end = self.termination.t_end if t_end is None else t_end
        opts = self.termination
        for _ in range(max_steps):
            if not self.active or self.t >= t_end:
                break
            self.solver.step(1, graph=self.graph)
            self.t = self.t + self.dt   # the device clock's own addition
            self.n_steps += 1
            # a failed diffusion or convection system ends the run, as FlameSolver throws when
            # convectionSystem.integrateToTime fails (src/flameSolver.cpp:736-752); failed source-term
            # points are counted and stepping continues, as there
            n_src, n_sys = self.solver.failures()
            if n_sys:
                raise StepFailure(f"t = {self.t:.6e}: {n_sys} diffusion / convection systems failed in the last step "
                                  f"({n_src} source-term points)", self)
            self._record()
            self._since_term += 1
            self._since_regrid += 1
            if self._since_term >= opts.terminate_step_interval:
                self._since_term = 0
                self._terminate()
                if not self.active:
                    break
            if self._since_regrid >= opts.regrid_step_interval:
                self._since_regrid = 0
                self._regrid()
        return self.records
