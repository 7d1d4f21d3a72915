"""Gradients: the discrete adjoint of the BDF source-term integration on the
GPU against central finite differences of the CPU restatement of the
reference's solver (the oracle), on stiff reactor states of a small
synthetic mechanism with tight tolerances.

Finite differences of an adaptive integrator carry noise from its step-size
decisions (about 1e-9 of the solution with these tolerances), so the
perturbations are 1e-4 of the state entry and 1e-3 in ln(multiplier)
(central differences), and the rate-multiplier checks use the reactions with
the largest gradients."""
import numpy as np
import pytest

from ember_gb300.mechanism import reactor_states, synthetic_mechanism
from ember_gb300.source import BDF, KINETICS_STANDARD, SourceOptions

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case():
    mech = synthetic_mechanism(n_species=20, n_reactions=60, seed=3)
    st, dt = reactor_states(mech, 3, seed=11, T_range=(1100.0, 1600.0), dt_range=(2e-5, 5e-5))
    opts = SourceOptions.defaults(kinetics_model=KINETICS_STANDARD, bdf_reltol=1e-9, bdf_abstol_momentum=1e-9,
                                  bdf_abstol_energy=1e-9, bdf_abstol_species=1e-15)
    rng = np.random.default_rng(1)
    bar = rng.normal(size=st.shape)
    bar[:, 0] = 0.0
    bar[:, 1] *= 1e-3
    return mech, st, dt, opts, bar


def _phi(om, st, dt, opts, bar, mult=None):
    from ember_gb300.source import BDF as _BDF
    om.set_multipliers(mult)
    out, status, _ = om.integrate(_BDF, st, dt, opts, n_threads=1)
    assert (status == 0).all(), status
    return float((bar * out).sum())


def test_bdf_adjoint_matches_central_differences_of_the_oracle(gpu_lib, case):
    from oracle.chem import OracleMech
    from ember_gb300.source import GpuMechanism, source_adjoint
    mech, st, dt, opts, bar = case
    gm = GpuMechanism(mech)
    out, status, g_state, g_lnk = source_adjoint(gm, st, dt, opts, bar, tape_cap=4096)
    assert (status == 0).all(), status
    om = OracleMech(mech)
    ref_out, _, _ = om.integrate(BDF, st, dt, opts, n_threads=1)
    assert np.array_equal(out, ref_out)  # the taped forward pass is the ordinary one
    checked = 0
    for (j, k) in [(0, 1), (1, 1), (2, 1), (0, 2), (1, 3), (2, 4), (0, 6)]:
        hstep = 1e-4 * max(abs(st[j, k]), 1e-6)
        e = np.zeros_like(st)
        e[j, k] = hstep
        fd = (_phi(om, st + e, dt, opts, bar) - _phi(om, st - e, dt, opts, bar)) / (2 * hstep)
        assert abs(g_state[j, k] - fd) <= 1e-4 * abs(fd) + 1e-9, (j, k, g_state[j, k], fd)
        checked += 1
    R = mech.n_reactions
    rel = 1e-3
    for i in np.argsort(-np.abs(g_lnk))[:4]:
        mp, mm = np.ones(R), np.ones(R)
        mp[i], mm[i] = np.exp(rel), np.exp(-rel)
        fd = (_phi(om, st, dt, opts, bar, mp) - _phi(om, st, dt, opts, bar, mm)) / (2 * rel)
        assert abs(g_lnk[i] - fd) <= 1e-3 * abs(fd) + 1e-8, (i, g_lnk[i], fd)
        checked += 1
    om.set_multipliers(None)
    assert checked == 11


@pytest.mark.parametrize("explicit_h", [False, True])
def test_diffusion_adjoint_is_the_transpose_of_the_stage(gpu_lib, explicit_h):
    # The stage is linear in y (zero split constants, y_inf = 0): its matrix M
    # has columns M e_i (the serial stage applied to unit vectors), and the
    # adjoint must return M^T ybar, for every boundary condition and for both
    # the single BDF1 x 8 step and multi-step (BDF2) stages.
    from ember_gb300 import _lib as L
    from ember_gb300.diffusion import FlameGrid, diffusion_adjoint, integrate_diffusion_terms
    rng = np.random.default_rng(8 + explicit_h)
    grids = []
    for left, right, alpha in [(0, 0, 0), (1, 1, 1), (2, 4, 0), (3, 0, 1), (4, 4, 0)]:
        n = int(rng.integers(6, 14))
        x = np.cumsum(np.full(n, 2e-5) * np.exp(rng.uniform(-0.3, 0.3, n))) + (1e-4 if alpha else 0.0)
        grids.append(FlameGrid(x=x, left_bc=left, right_bc=right, alpha=alpha))
    n_vars = 2
    tot = sum(g.n_points for g in grids) * n_vars
    B = np.exp(rng.uniform(-1, 1, tot))
    D = np.exp(rng.uniform(np.log(1e-6), np.log(1e-4), tot))
    nsys = len(grids) * n_vars
    h = np.full(nsys, 2e-6) if explicit_h else None
    wall = rng.uniform(0.0, 3.0, nsys)
    ybar = rng.normal(size=tot)
    got, status = diffusion_adjoint(grids, B, D, ybar, 0.0, 1e-5, h=h, wall_const=wall)
    assert (status == 0).all()
    M = np.zeros((tot, tot))
    for i in range(tot):
        e = np.zeros(tot)
        e[i] = 1.0
        out, st = integrate_diffusion_terms(grids, B, D, np.zeros(tot), e, 0.0, 1e-5, h=h, wall_const=wall,
                                            algorithm=L.DIFFUSION_SERIAL)
        M[:, i] = out
    ref = M.T @ ybar
    np.testing.assert_allclose(got, ref, rtol=1e-11, atol=1e-12 * np.abs(ref).max())
