"""Convection stage (ConvectionSystemSplit::integrateToTime,
src/convectionSystem.cpp:588-627; ConvectionSystemUTW::f 14-130;
ConvectionSystemY::f 307-359 and update_v 372-398).

CPU: the oracle's Adams coefficients against exact fractions, its UTW
right-hand side against an independent numpy restatement for every boundary
and continuity condition, its interpolation rule against std::map lower_bound
semantics, the whole stage against scipy at tight tolerance, and invariants
of the species stage. GPU: ember_convection_integrate against the oracle bit
for bit (states, statuses, step counts), host and device memory alike."""
from fractions import Fraction
import bisect

import numpy as np
import numpy.polynomial.chebyshev as npcheb
import pytest

from oracle import convection as oc
from ember_gb300.convection import (BC_CONTROL_VOLUME, BC_FIXED_VALUE, BC_WALL_FLUX, BC_ZERO_GRADIENT, CONT_LEFT,
                                    CONT_QDOT, CONT_RIGHT, CONT_TEMP, CONT_ZERO, STRAIN_CHEBYSHEV, ConvectionFlame,
                                    ConvectionOptions, convection_batch, mean_molecular_weight)
from ember_gb300.mechanism import GAS_CONSTANT, synthetic_mechanism


@pytest.fixture(scope="module")
def mech():
    return synthetic_mechanism(n_species=12, n_reactions=40, seed=1240)


def _profile(N, seed, alpha=0):
    rng = np.random.default_rng(seed)
    x = np.cumsum(rng.uniform(0.5, 1.5, N)) * 2e-5
    if alpha == 0:
        x = x - x[N // 3]
    c = 0.5 * (1 + np.tanh((x - x[N // 2]) / (5 * 2e-5)))
    T = 300 + 1700 * c + rng.uniform(-5, 5, N)
    U = 300 * (1 + 0.5 * c) + rng.uniform(-20, 20, N)
    Wm = 28.5 - 3 * c + rng.uniform(-0.1, 0.1, N)
    return x, U, T, Wm


# ---- coefficients --------------------------------------------------------

def test_adams_coefficients_are_the_exact_fractions():
    g = [Fraction(1)]
    for j in range(1, 14):
        g.append(1 - sum(g[i] / (j + 1 - i) for i in range(j)))
    assert [float(v) for v in g[:6]] == [1.0, 0.5, 5 / 12, 3 / 8, 251 / 720, 95 / 288]
    np.testing.assert_allclose(oc.adams_gammas(), [float(v) for v in g], rtol=1e-14)
    for q in range(1, 13):
        # Lambda(x) = int_{-1}^x prod_{i<q} (u+i) du / int_{-1}^0 ...
        p = [Fraction(1)]
        for i in range(1, q):
            p = [Fraction(0)] + p
            for j in range(len(p) - 1):
                p[j] += i * p[j + 1]
        integ = [Fraction(0)] + [p[j] / (j + 1) for j in range(len(p))]
        q0 = -sum(c * (-1) ** k for k, c in enumerate(integ))   # int_{-1}^0 P = -I(-1)
        lam = list(integ)
        lam[0] = q0
        exact = [float(c / q0) for c in lam]
        np.testing.assert_allclose(oc.adams_l(q)[:q + 1], exact, rtol=1e-13, err_msg=f"q={q}")


def test_adams_l_gives_backward_euler_and_trapezoid():
    assert list(oc.adams_l(1)[:2]) == [1.0, 1.0]
    assert list(oc.adams_l(2)[:3]) == [1.0, 2.0, 1.0]


# ---- the UTW right-hand side ------------------------------------------------

def _numpy_strain(fl, t):
    """LinearFunction, or ChebyshevFunction through numpy's Chebyshev series
    for a(t) and the closed form U_i(cos th) = sin((i+1) th) / sin th for the
    reference's derivative sum c_1 + sum_{i>=2} i U_i(x) c_i."""
    if fl.strain_type == STRAIN_CHEBYSHEV:
        c = np.array(list(fl.cheb) + [0.0] * max(0, 2 - len(fl.cheb)))
        x = 2 * (t - fl.cheb_t0) / (fl.cheb_t1 - fl.cheb_t0) - 1
        a = npcheb.chebval(x, c)
        th = np.arccos(np.clip(x, -1, 1))
        U = [np.sin((i + 1) * th) / np.sin(th) for i in range(len(c))]
        d = c[1] + sum(i * U[i] * c[i] for i in range(2, len(c)))
        return a, d * 2.0 / (fl.cheb_t1 - fl.cheb_t0)
    if t <= fl.strain_t0:
        a = fl.strain_initial
    elif t >= fl.strain_t0 + fl.strain_dt:
        a = fl.strain_final
    else:
        a = fl.strain_initial + (fl.strain_final - fl.strain_initial) * (t - fl.strain_t0) / fl.strain_dt
    dadt = (fl.strain_final - fl.strain_initial) / fl.strain_dt \
        if fl.strain_t0 <= t < fl.strain_t0 + fl.strain_dt else 0.0
    return a, dadt


def test_chebyshev_strain_matches_the_series():
    # ChebyshevFunction (src/scalarFunction.cpp:31-87): a(t) is the series;
    # da/dt follows the reference's recurrence (coefficient i weighted by
    # i U_i, where T'_i = i U_{i-1}); fewer than two coefficients are padded
    from ember_gb300.output import strain as out_strain
    rng = np.random.default_rng(7)
    for n in (0, 1, 2, 5, 16):
        fl = ConvectionFlame(n_points=5, strain_type=STRAIN_CHEBYSHEV, cheb_t0=1e-3, cheb_t1=1.2e-3,
                             cheb=tuple(rng.standard_normal(n) * 100.0))
        for t in np.linspace(1e-3, 1.2e-3, 7)[1:-1]:
            a, d = oc.strain(fl, t)
            ea, ed = _numpy_strain(fl, t)
            assert a == pytest.approx(ea, rel=1e-12, abs=1e-9)
            assert d == pytest.approx(ed, rel=1e-10, abs=1e-6)
            assert out_strain(fl, t) == (a, d)       # the output writer's restatement: same bits
    # one coefficient: a constant strain, as LinearFunction's
    fl = ConvectionFlame(n_points=5, strain_type=STRAIN_CHEBYSHEV, cheb_t0=0.0, cheb_t1=1.0, cheb=(350.0,))
    assert oc.strain(fl, 0.3) == (350.0, 0.0)


def _numpy_utw(fl, x, t, U, T, Wm, drhodt, sU, sT, sW):
    """Independent vectorised restatement of ConvectionSystemUTW::f."""
    N = len(x)
    jj = N - 1
    hh = np.diff(x)
    rph = np.ones(N - 1) if fl.alpha == 0 else 0.5 * (x[:-1] + x[1:])
    # one past the half points: the factor at the last point (read by fixedRight / stagnation point at jj)
    rph = np.append(rph, 1.0 if fl.alpha == 0 else x[-1])
    rho = fl.pressure * Wm / (GAS_CONSTANT * T)
    m = hh * rph[:-1] * (drhodt[:-1] + rho[:-1] * fl.beta * U[:-1])   # flux increment between j and j+1
    rV = np.zeros(N)
    jc = fl.j_cont
    if fl.continuity_bc == CONT_LEFT:
        rV[0] = fl.rv_zero
        rV[1:] = fl.rv_zero - np.cumsum(m)
    elif fl.continuity_bc == CONT_ZERO:
        d0 = -rph[jc] * (drhodt[jc] - rho[jc] * fl.beta * U[jc])
        if jc:
            d0 = 0.5 * d0 - 0.5 * rph[jc - 1] * (drhodt[jc - 1] + rho[jc - 1] * fl.beta * U[jc - 1])
        rV[jc] = (x[jc] - fl.x_vzero) * d0
        for j in range(jc, jj):
            rV[j + 1] = rV[j] - m[j]
        if jc:
            rV[jc - 1] = (x[jc - 1] - fl.x_vzero) * d0
            for j in range(jc - 1, 0, -1):
                rV[j - 1] = rV[j] + m[j - 1]
    else:
        if fl.continuity_bc == CONT_TEMP:
            # at the last point only the backward difference exists
            if jc == 0 or (jc < jj and sT[jc] / (T[jc + 1] - T[jc]) < 0):
                rV[jc] = rph[jc] * rho[jc] * sT[jc] * hh[jc] / (T[jc + 1] - T[jc])
            else:
                rV[jc] = rph[jc - 1] * rho[jc] * sT[jc] * hh[jc - 1] / (T[jc] - T[jc - 1])
        else:
            rV[jc] = fl.rv_cont
        for j in range(jc, jj):
            rV[j + 1] = rV[j] - m[j]
        for j in range(jc, 0, -1):
            rV[j - 1] = rV[j] + hh[j - 1] * rph[j] * (drhodt[j] + rho[j] * fl.beta * U[j])
    V = rV.copy()
    if fl.alpha:
        V[1:] = rV[1:] / x[1:]
    a, dadt = _numpy_strain(fl, t)
    src = fl.rhou / rho * (dadt / fl.beta + a * a / fl.beta ** 2)
    dU, dT, dW = np.zeros(N), np.zeros(N), np.zeros(N)
    fwd = rV[1:jj] < 0
    for arr, out in ((U, dU), (T, dT), (Wm, dW)):
        f_ = (arr[2:] - arr[1:-1]) / hh[1:]
        b_ = (arr[1:-1] - arr[:-2]) / hh[:-1]
        out[1:jj] = np.where(fwd, f_, b_)
    yU = -V * dU / rho - U * U + src + sU
    yT = -V * dT / rho + sT
    yW = -V * dW / rho - Wm * Wm * sW
    yU[0] = sU[0] - U[0] ** 2 + src[0]
    if fl.left_bc in (BC_CONTROL_VOLUME, BC_WALL_FLUX):
        cvol = x[1] if fl.alpha == 0 else x[1] ** 2 / 2
        r0 = max(rV[0], 0.0)
        yT[0] = -r0 * (T[0] - fl.t_left) / (rho[0] * cvol) + sT[0]
        yW[0] = -r0 * (Wm[0] - fl.w_left) / (rho[0] * cvol) - Wm[0] ** 2 * sW[0]
    else:
        yT[0] = sT[0]
        yW[0] = -Wm[0] ** 2 * sW[0]
    if rV[jj] < 0 or fl.right_bc == BC_FIXED_VALUE:
        yU[jj] = sU[jj] - U[jj] ** 2 + src[jj]
        yT[jj] = sT[jj]
        yW[jj] = -Wm[jj] ** 2 * sW[jj]
    else:
        hl = hh[jj - 1]
        yU[jj] = sU[jj] - V[jj] * (U[jj] - U[jj - 1]) / hl / rho[jj] - U[jj] ** 2 + src[jj]
        yT[jj] = sT[jj] - V[jj] * (T[jj] - T[jj - 1]) / hl / rho[jj]
        yW[jj] = -Wm[jj] ** 2 * sW[jj] - V[jj] * (Wm[jj] - Wm[jj - 1]) / hl / rho[jj]
    return yU, yT, yW, rho, rV


CASES = [
    dict(continuity_bc=CONT_LEFT, left_bc=BC_CONTROL_VOLUME, right_bc=BC_ZERO_GRADIENT, rv_zero=0.3),
    dict(continuity_bc=CONT_LEFT, left_bc=BC_FIXED_VALUE, right_bc=BC_FIXED_VALUE, rv_zero=-0.2),
    dict(continuity_bc=CONT_LEFT, left_bc=BC_WALL_FLUX, right_bc=BC_ZERO_GRADIENT, rv_zero=0.5, alpha=1),
    dict(continuity_bc=CONT_ZERO, j_cont=17, x_vzero=0.0),
    dict(continuity_bc=CONT_ZERO, j_cont=0, x_vzero=-1e-4),
    dict(continuity_bc=CONT_ZERO, j_cont=39, x_vzero=1e-3, alpha=1),
    dict(continuity_bc=CONT_TEMP, j_cont=20),
    dict(continuity_bc=CONT_TEMP, j_cont=0),
    dict(continuity_bc=CONT_TEMP, j_cont=39),   # the last point: backward difference only
    dict(continuity_bc=CONT_RIGHT, j_cont=39, rv_cont=-0.4),
    dict(continuity_bc=CONT_QDOT, j_cont=11, rv_cont=0.1, alpha=1, left_bc=BC_ZERO_GRADIENT),
    dict(continuity_bc=CONT_LEFT, rv_zero=0.3, strain_type=STRAIN_CHEBYSHEV, cheb_t0=0.0, cheb_t1=5e-5,
         cheb=(300.0, 120.0, -40.0, 15.0)),
]


@pytest.mark.parametrize("case", range(len(CASES)))
def test_utw_rhs_matches_numpy_restatement(case):
    kw = dict(CASES[case])
    alpha = kw.get("alpha", 0)
    N = 40
    x, U, T, Wm = _profile(N, seed=case, alpha=alpha)
    rng = np.random.default_rng(100 + case)
    fl = ConvectionFlame(n_points=N, beta=1.0 + alpha, rhou=1.17, pressure=101325.0, t_left=310.0, w_left=28.4,
                         strain_initial=200.0, strain_final=600.0, strain_t0=1e-5, strain_dt=2e-5, **kw)
    dr, sU, sT, sW = (rng.standard_normal(N) * s for s in (5.0, 1e4, 1e5, 1e-2))
    y3 = np.empty(3 * N)
    y3[0::3], y3[1::3], y3[2::3] = U, T, Wm
    for t in (0.0, 2e-5, 4e-5):
        yd, rho, rV, V = oc.utw_rhs(fl, x, t, y3, dr, sU, sT, sW)
        eU, eT, eW, erho, erV = _numpy_utw(fl, x, t, U, T, Wm, dr, sU, sT, sW)
        np.testing.assert_allclose(rho, erho, rtol=1e-14)
        np.testing.assert_allclose(rV, erV, rtol=1e-11, atol=1e-12 * np.abs(erV).max())
        for got, exp in ((yd[0::3], eU), (yd[1::3], eT), (yd[2::3], eW)):
            np.testing.assert_allclose(got, exp, rtol=1e-10, atol=1e-10 * np.abs(exp).max())


def test_interval_rule_is_lower_bound_then_next():
    ht = np.array([0.0, 1.0, 2.5, 4.0])
    for t in (-1.0, 0.0, 0.3, 1.0, 2.0, 2.5, 3.9, 4.0, 7.0):
        iL = bisect.bisect_left(list(ht), t)      # std::map::lower_bound
        if iL == len(ht):
            iL -= 1
        if iL + 1 == len(ht):
            iL -= 1
        i, s = oc.interval(ht, t)
        assert i == iL and s == pytest.approx((t - ht[iL]) / (ht[iL + 1] - ht[iL]), rel=1e-15), t
    assert oc.interval(np.array([3.0]), 5.0)[0] == -1


# ---- the stage ----------------------------------------------------------------

def _one_flame(mech, seed=5, **kw):
    b = convection_batch(mech, n_flames=1, n_min=60, n_max=80, seed=seed, **kw)
    return b


def test_stage_matches_scipy(mech):
    from scipy.integrate import solve_ivp
    S, Wt = mech.n_species, mech.mol_weight
    b = _one_flame(mech, split_scale=0.3, drhodt_scale=0.3)
    fl = b.flames[0]
    N = fl.n_points
    tf = 1e-5
    opts = ConvectionOptions()
    st, status, stats, ht, hv = oc.convection_flame(fl, Wt, b.x, b.y_left[0], b.drhodt, b.split_const, b.state,
                                                    0.0, tf, opts)
    assert (status == 0).all() and stats[0] > 3 and len(ht) == stats[0] + 1 and ht[-1] == tf
    sv = b.state.reshape(S + 2, N)
    sc = b.split_const.reshape(S + 2, N)
    out = st.reshape(S + 2, N)
    Wm = mean_molecular_weight(sv[2:].T, Wt)
    sW = (sc[2:] / Wt[:, None]).sum(axis=0)
    y3 = np.empty(3 * N)
    y3[0::3], y3[1::3], y3[2::3] = sv[0], sv[1], Wm
    r = solve_ivp(lambda t, y: oc.utw_rhs(fl, b.x, t, y, b.drhodt, sc[0], sc[1], sW)[0], (0, tf), y3,
                  method="LSODA", rtol=1e-10, atol=1e-12)
    ref = r.y[:, -1]
    assert np.abs(out[0] - ref[0::3]).max() < 1e-4 * np.abs(ref[0::3]).max()
    assert np.abs(out[1] - ref[1::3]).max() < 1e-4 * ref[1::3].max()
    # species with the recorded v(t) and the same interpolation rule
    hh = np.diff(b.x)

    def vel(t):
        i, s = oc.interval(ht, t)
        return hv[0] if i < 0 else hv[i] * (1 - s) + hv[i + 1] * s

    for k in (0, 3, S - 1):
        def f(t, y, k=k):
            v = vel(t)
            d = np.zeros(N)
            cvol = b.x[1]
            d[0] = -max(v[0], 0.0) * (y[0] - b.y_left[0][k]) / cvol + sc[2 + k][0]
            fw = (y[2:] - y[1:-1]) / hh[1:]
            bw = (y[1:-1] - y[:-2]) / hh[:-1]
            d[1:-1] = -v[1:-1] * np.where(v[1:-1] < 0, fw, bw) + sc[2 + k][1:-1]
            d[-1] = sc[2 + k][-1] if v[-1] < 0 else sc[2 + k][-1] - v[-1] * (y[-1] - y[-2]) / hh[-1]
            return d
        r = solve_ivp(f, (0, tf), sv[2 + k], method="LSODA", rtol=1e-10, atol=1e-15)
        scale = max(np.abs(sv[2 + k]).max(), 1e-8)
        assert np.abs(out[2 + k] - r.y[:, -1]).max() < 1e-4 * scale, k


def test_uniform_species_field_is_left_unchanged(mech):
    """Convection of a uniform field with the same inflow and no split
    constant has a zero right-hand side: the species come back bit for bit."""
    S, Wt = mech.n_species, mech.mol_weight
    b = _one_flame(mech, seed=9)
    fl = b.flames[0]
    N = fl.n_points
    sv = b.state.reshape(S + 2, N).copy()
    y0 = sv[2:, 0].copy()
    sv[2:] = y0[:, None]
    st, status, _, _, _ = oc.convection_flame(fl, Wt, b.x, y0, b.drhodt, b.split_const, sv.reshape(-1), 0.0,
                                              5e-6, ConvectionOptions())
    assert (status == 0).all()
    np.testing.assert_array_equal(st.reshape(S + 2, N)[2:], sv[2:])


def test_mass_fractions_still_sum_to_one(mech):
    S, Wt = mech.n_species, mech.mol_weight
    b = _one_flame(mech, seed=12)
    fl = b.flames[0]
    N = fl.n_points
    st, status, _, _, _ = oc.convection_flame(fl, Wt, b.x, b.y_left[0], b.drhodt, b.split_const, b.state, 0.0,
                                              1e-5, ConvectionOptions())
    assert (status == 0).all()
    tot = st.reshape(S + 2, N)[2:].sum(axis=0)
    assert np.abs(tot - 1.0).max() < 1e-5


def test_record_overflow_is_reported(mech):
    S, Wt = mech.n_species, mech.mol_weight
    b = _one_flame(mech, seed=5)
    fl = b.flames[0]
    st, status, _, ht, _ = oc.convection_flame(fl, Wt, b.x, b.y_left[0], b.drhodt, b.split_const, b.state, 0.0,
                                               1e-5, ConvectionOptions(max_history=3))
    assert status[0] == -20 and (status[1:] == -20).all() and len(ht) == 3


# ---- GPU ----------------------------------------------------------------------

def _mixed_batch(mech, seed):
    """Several flames with every continuity and boundary condition."""
    b = convection_batch(mech, n_flames=len(CASES), n_min=40, n_max=120, seed=seed, split_scale=0.2,
                         drhodt_scale=0.2)
    for fl, kw in zip(b.flames, CASES):
        for k, v in kw.items():
            setattr(fl, k, v)
        if fl.continuity_bc in (CONT_RIGHT, CONT_ZERO) and fl.j_cont == 39:
            fl.j_cont = fl.n_points - 1          # the last point (fixedRight; stagnation point past the end)
        elif fl.continuity_bc != CONT_LEFT:
            fl.j_cont = min(fl.j_cont, fl.n_points - 2)
        if fl.alpha == 1:
            fl.beta = 2.0
        fl.strain_final = fl.strain_initial * 1.5
        fl.strain_t0, fl.strain_dt = 2e-6, 4e-6
    # cylindrical flames need x > 0
    p = 0
    for f, fl in enumerate(b.flames):
        N = fl.n_points
        if fl.alpha == 1:
            seg = b.x[p:p + N]
            b.x[p:p + N] = seg - seg[0] + 1e-4
        p += N
    return b


@pytest.mark.gpu
@pytest.mark.parametrize("n_species,seed", [(12, 3), (53, 4)])
def test_gpu_convection_bitwise_vs_oracle(gpu_lib, n_species, seed):
    from ember_gb300.convection import integrate_convection_terms
    m = synthetic_mechanism(n_species=n_species, n_reactions=4 * n_species, seed=seed)
    b = _mixed_batch(m, seed)
    opts = ConvectionOptions()
    tf = 8e-6
    ref, rstatus, rstats = oc.convection_batch(b, m.mol_weight, 0.0, tf, opts)
    st = b.state.copy()
    _, status, stats = integrate_convection_terms(b.flames, m.mol_weight, b.x, b.y_left, b.drhodt, b.split_const, st,
                                                  0.0, tf, opts)
    np.testing.assert_array_equal(status, rstatus)
    np.testing.assert_array_equal(stats, rstats)
    assert np.array_equal(st, ref), np.abs(st - ref).max()
    assert (rstatus == 0).any()


@pytest.mark.gpu
def test_gpu_convection_device_memory_and_overflow(gpu_lib, mech):
    import torch
    from ember_gb300.convection import integrate_convection_terms
    b = convection_batch(mech, n_flames=5, n_min=30, n_max=90, seed=21)
    opts = ConvectionOptions()
    host = b.state.copy()
    _, s1, t1 = integrate_convection_terms(b.flames, mech.mol_weight, b.x, b.y_left, b.drhodt, b.split_const, host,
                                           1e-3, 1e-3 + 5e-6, opts)
    dev = torch.as_tensor(b.state, device="cuda").clone()
    _, s2, t2 = integrate_convection_terms(b.flames, mech.mol_weight, b.x, b.y_left, b.drhodt, b.split_const, dev,
                                           1e-3, 1e-3 + 5e-6, opts)
    assert np.array_equal(dev.cpu().numpy(), host)
    assert np.array_equal(s2.cpu().numpy(), s1) and np.array_equal(t2.cpu().numpy(), t1)
    st = b.state.copy()
    integrate_convection_terms(b.flames, mech.mol_weight, b.x, b.y_left, b.drhodt, b.split_const, st, 1e-3,
                               1e-3 + 5e-6, ConvectionOptions(species_threads=32))
    assert np.array_equal(st, host)
    # a record too short for the UTW steps: every system of the flame reports it, nothing faults
    small = ConvectionOptions(max_history=3)
    st = b.state.copy()
    _, s3, _ = integrate_convection_terms(b.flames, mech.mol_weight, b.x, b.y_left, b.drhodt, b.split_const, st,
                                          0.0, 5e-6, small)
    ref, rs, _ = oc.convection_batch(b, mech.mol_weight, 0.0, 5e-6, small)
    np.testing.assert_array_equal(s3, rs)
    assert (s3 == -20).any()
    assert np.array_equal(st, ref)


@pytest.mark.parametrize("balanced", [True, False])
def test_density_derivative_matches_numpy_restatement(mech, balanced):
    """prepareIntegrators' drho/dt (src/flameSolver.cpp:208-212) from the
    four time derivatives and the state, as the split step computes it."""
    rng = np.random.default_rng(31)
    S, W = mech.n_species, mech.mol_weight
    n_pts = 17
    state = np.empty((n_pts, S + 2))
    state[:, 0] = rng.uniform(0, 500, n_pts)
    state[:, 1] = rng.uniform(300, 2500, n_pts)
    Y = rng.uniform(0, 1, (n_pts, S))
    Y[3, 2] = -1e-4                                     # clipped
    state[:, 2:] = Y / Y.sum(axis=1, keepdims=True)
    ddt = [rng.standard_normal((n_pts, S + 2)) * 1e3 for _ in range(4)]
    got = oc.density_derivative(state, W, 101325.0, *ddt, balanced)
    yc = np.maximum(state[:, 2:], 0.0)
    wmx = 1.0 / ((yc / yc.sum(axis=1, keepdims=True)) / W[None, :]).sum(axis=1)
    rho = 101325.0 * wmx / (GAS_CONSTANT * state[:, 1])
    tot = ddt[0] + ddt[1] + ddt[2] + (ddt[3] if balanced else 0.0)
    exp = -rho * (tot[:, 1] / state[:, 1] + (tot[:, 2:] / W[None, :]).sum(axis=1) * wmx)
    np.testing.assert_allclose(got, exp, rtol=1e-12)
