"""Thermo and mixture-averaged transport properties (FlameSolver::
updateChemicalProperties with ApproxMixTransport, src/flameSolver.cpp:652-699,
src/chemistry0d.cpp:12-269, 583-591): the oracle against an independent numpy
restatement of the same model, the seeded fits against the kinetic-theory
curves they came from, and the GPU (ember_transport_eval) against the oracle
bit for bit."""
import numpy as np
import pytest

from oracle import chem
from ember_gb300.mechanism import GAS_CONSTANT, nasa_cp_R, reactor_states, synthetic_mechanism
from ember_gb300.transport import kinetic_theory, pair_index, synthetic_transport

KEYS = ("density", "mean_mol_weight", "cp_mass", "cp_species", "h_species", "conductivity", "viscosity", "rho_d")


@pytest.fixture(scope="module")
def mech():
    return synthetic_mechanism(n_species=40, n_reactions=200, seed=7)


@pytest.fixture(scope="module")
def tdata(mech):
    return synthetic_transport(mech, seed=11)


def _states(mech, n, seed):
    st, _ = reactor_states(mech, n, seed=seed)
    rng = np.random.default_rng(seed)
    Y = st[:, 2:] * rng.uniform(0.5, 1.5, st[:, 2:].shape) + 1e-7 * rng.uniform(0, 1, st[:, 2:].shape)
    Y[:, rng.integers(0, mech.n_species, 5)] = 0.0            # absent species
    Y[1, 3] = -1e-5                                            # a negative mass fraction (clipped)
    Y[2] = 0.0
    Y[2, 2] = 1.0                                              # a pure species (N2)
    T = rng.uniform(300.0, 2800.0, n)
    return T, Y


def _numpy_properties(mech, td, T, Y, p, thr):
    """Independent restatement: vectorised formulas, numpy's own sums, Wilke's
    phi from its direct formula for every pair."""
    S = mech.n_species
    W = mech.mol_weight
    out = {k: [] for k in KEYS}
    D = np.zeros((S, S, 5))
    for j in range(S):
        for k in range(j, S):
            D[j, k] = D[k, j] = td.diff_fit[pair_index(S, j, k)]
    for Tj, y in zip(T, Y):
        lnT = np.log(Tj)
        pw = lnT ** np.arange(5)
        a = np.where(Tj <= mech.nasa_tmid[:, None], mech.nasa_coeffs[:, :7], mech.nasa_coeffs[:, 7:])
        cpR = nasa_cp_R(a.T, Tj)
        hRT = (a[:, 0] + Tj * (a[:, 1] / 2 + Tj * (a[:, 2] / 3 + Tj * (a[:, 3] / 4 + Tj * a[:, 4] / 5)))
               + a[:, 5] / Tj)
        yc = np.maximum(y, 0.0)
        yc = yc / yc.sum()
        mmw = 1.0 / (yc / W).sum()
        X = yc / W * mmw
        rho = p * mmw / (GAS_CONSTANT * Tj)
        Xc = np.maximum(X, 1e-20)
        mu = (Tj ** 0.25 * (td.visc_fit @ pw)) ** 2
        lam = np.sqrt(Tj) * (td.cond_fit @ pw)
        bd = Tj ** 1.5 * (D @ pw)
        major = Xc >= thr
        phi = (1 + np.sqrt(mu[:, None] / mu[None, :]) * (W[None, :] / W[:, None]) ** 0.25) ** 2 / np.sqrt(
            8 * (1 + W[:, None] / W[None, :]))
        den = (phi[np.ix_(major, major)] * Xc[major][None, :]).sum(axis=1)
        vis = (Xc[major] * mu[major] / den).sum()
        rd = np.empty(S)
        for k in range(S):
            sel = np.ones(S, bool) if major[k] else major.copy()
            sel[k] = False
            s1 = p * (Xc[sel] / bd[k, sel]).sum()
            with np.errstate(divide="ignore"):
                s2 = p * Xc[k] / (mmw - W[k] * Xc[k]) * (Xc[sel] * W[sel] / bd[k, sel]).sum()
            rd[k] = rho / (s1 + s2)
        out["density"].append(rho)
        out["mean_mol_weight"].append(mmw)
        out["cp_mass"].append(GAS_CONSTANT * (cpR * yc / W).sum())
        out["cp_species"].append(cpR * GAS_CONSTANT)
        out["h_species"].append(hRT * GAS_CONSTANT * Tj)
        out["conductivity"].append(0.5 * ((Xc * lam).sum() + 1.0 / (Xc / lam).sum()))
        out["viscosity"].append(vis)
        out["rho_d"].append(rd)
    return {k: np.array(v) for k, v in out.items()}


@pytest.mark.parametrize("thr", [0.0, 1e-5])
def test_oracle_matches_independent_restatement(mech, tdata, thr):
    T, Y = _states(mech, 12, seed=3)
    om = chem.OracleMech(mech)
    o = chem.transport_eval(om, tdata, T, Y, 101325.0, thr)
    r = _numpy_properties(mech, tdata, T, Y, 101325.0, thr)
    for k in KEYS:
        np.testing.assert_allclose(o[k], r[k], rtol=1e-12, atol=0, err_msg=k)


def test_fits_reproduce_kinetic_theory(mech, tdata):
    Tg = np.geomspace(320.0, 3400.0, 23)
    mu, lam, pD = kinetic_theory(mech, tdata.sigma, tdata.eps_k, Tg)
    pw = np.log(Tg)[None, :] ** np.arange(5)[:, None]
    np.testing.assert_allclose((Tg ** 0.25 * (tdata.visc_fit @ pw)) ** 2, mu, rtol=1e-2)
    np.testing.assert_allclose(np.sqrt(Tg) * (tdata.cond_fit @ pw), lam, rtol=1e-2)
    np.testing.assert_allclose(Tg ** 1.5 * (tdata.diff_fit @ pw), pD, rtol=1e-2)
    # magnitudes of small gases at 1 atm, 1000 K
    i = np.searchsorted(Tg, 1000.0)
    assert 1e-5 < np.median(mu[:, i]) < 1e-4 and 0.02 < np.median(lam[:, i]) < 0.3
    assert 5e-5 < np.median(pD[:, i]) / 101325.0 < 1e-3


def test_approx_threshold_changes_little(mech, tdata):
    T, Y = _states(mech, 8, seed=5)
    om = chem.OracleMech(mech)
    mix = chem.transport_eval(om, tdata, T, Y, 101325.0, 0.0)
    approx = chem.transport_eval(om, tdata, T, Y, 101325.0, 1e-5)
    np.testing.assert_allclose(approx["viscosity"], mix["viscosity"], rtol=1e-3)
    ok = np.isfinite(mix["rho_d"]) & (mix["rho_d"] > 0)
    np.testing.assert_allclose(approx["rho_d"][ok], mix["rho_d"][ok], rtol=2e-2)
    np.testing.assert_array_equal(approx["conductivity"], mix["conductivity"])


@pytest.mark.gpu
@pytest.mark.parametrize("n_species,n_reactions,seed", [(40, 200, 7), (150, 1000, 150_1000)])
@pytest.mark.parametrize("thr", [0.0, 1e-5])
def test_gpu_transport_bitwise_vs_oracle(gpu_lib, n_species, n_reactions, seed, thr):
    from ember_gb300.source import GpuMechanism
    from ember_gb300.transport import GpuTransport
    m = synthetic_mechanism(n_species=n_species, n_reactions=n_reactions, seed=seed)
    td = synthetic_transport(m, seed=2)
    T, Y = _states(m, 37, seed=9)
    g = GpuTransport(GpuMechanism(m), td)
    a = g.eval(T, Y, 101325.0, thr)
    b = chem.transport_eval(chem.OracleMech(m), td, T, Y, 101325.0, thr)
    for k in KEYS:
        assert np.array_equal(a[k], b[k], equal_nan=True), (k, np.nanmax(np.abs(a[k] - b[k])))


@pytest.mark.gpu
def test_gpu_transport_device_memory_and_gas_eval_agree(gpu_lib, mech, tdata):
    import torch
    from ember_gb300.source import GpuMechanism
    from ember_gb300.transport import GpuTransport
    gm = GpuMechanism(mech)
    g = GpuTransport(gm, tdata)
    T, Y = _states(mech, 20, seed=4)
    host = g.eval(T, Y)
    dev = g.eval(torch.as_tensor(T, device="cuda"), torch.as_tensor(Y, device="cuda"))
    for k in KEYS:
        assert np.array_equal(dev[k].cpu().numpy(), host[k], equal_nan=True), k
    # density, cp and h_k are the values the source term sees (ember_gas_eval)
    ge = gm.gas_eval(T, Y)
    np.testing.assert_array_equal(host["density"], ge["density"])
    np.testing.assert_array_equal(host["cp_mass"], ge["cp_mass"])
    np.testing.assert_array_equal(host["h_species"], ge["hk"])
    assert g.eval(T[:0], Y[:0])["density"].shape == (0,)


def test_oracle_threads_give_the_same_bits(mech, tdata):
    T, Y = _states(mech, 23, seed=8)
    om = chem.OracleMech(mech)
    one = chem.transport_eval(om, tdata, T, Y, 101325.0, 1e-5, n_threads=1)
    many = chem.transport_eval(om, tdata, T, Y, 101325.0, 1e-5, n_threads=5)
    for k in KEYS:
        assert np.array_equal(one[k], many[k], equal_nan=True), k
