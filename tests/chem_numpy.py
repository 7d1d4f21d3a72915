"""Independent numpy restatement of the published gas-kinetics formulas, used
only by the tests to cross-check the C oracle: ideal-gas state (Cantera's
setState_TPY normalisation), NASA7 thermo, modified Arrhenius, third-body
efficiencies, Lindemann/Troe falloff (Gilbert-Luther-Troe form), reverse
rates from Kc = exp(-dG0/RT) (p0/RT)^dn, and creation / destruction / net
production rates. Vectorised and written without regard to operation order,
so it agrees with the oracle to rounding (~1e-12 relative), not bitwise."""
import numpy as np

R_GAS = 6.02214076e26 * 1.380649e-23
P_REF = 101325.0


def thermo(mech, T):
    a = np.where((T <= mech.nasa_tmid)[:, None], mech.nasa_coeffs[:, :7], mech.nasa_coeffs[:, 7:])
    cp = a[:, 0] + T * (a[:, 1] + T * (a[:, 2] + T * (a[:, 3] + T * a[:, 4])))
    h = a[:, 0] + T * (a[:, 1] / 2 + T * (a[:, 2] / 3 + T * (a[:, 3] / 4 + T * a[:, 4] / 5))) + a[:, 5] / T
    s = a[:, 0] * np.log(T) + T * (a[:, 1] + T * (a[:, 2] / 2 + T * (a[:, 3] / 3 + T * a[:, 4] / 4))) + a[:, 6]
    return cp, h, s


def rates(mech, T, Y, p=101325.0, normalize=True):
    W = mech.mol_weight
    Y = np.asarray(Y, dtype=float)
    if normalize:
        Y = np.maximum(Y, 0.0)
        Y = Y / Y.sum()
    ym = Y / W
    mmw = 1.0 / ym.sum()
    rho = p * mmw / (R_GAS * T)
    c = ym * rho
    ctot = rho / mmw
    cp_R, h_RT, s_R = thermo(mech, T)
    g = h_RT - s_R
    nu_r, nu_p = mech.stoich_matrices()
    dn = nu_p.sum(0) - nu_r.sum(0)
    arr = lambda P: P[:, 0] * np.exp(P[:, 1] * np.log(T) - P[:, 2] / T)
    kf = arr(mech.arrhenius)
    R = mech.n_reactions
    concm = np.zeros(R)
    for i in range(R):
        if mech.rxn_type[i] != 0:
            de = mech.default_efficiency[i]
            cm = de * ctot
            for e in range(mech.efficiency_offsets[i], mech.efficiency_offsets[i + 1]):
                cm += (mech.efficiency_values[e] - de) * c[mech.efficiency_species[e]]
            concm[i] = cm
    fall = (mech.rxn_type == 2) | (mech.rxn_type == 3)
    k0 = arr(mech.arrhenius_low)
    pr = concm * k0 / (kf + 1e-300)
    F = np.ones(R)
    tro = mech.rxn_type == 3
    a, T3, T1, T2 = mech.troe.T
    with np.errstate(divide="ignore", over="ignore", invalid="ignore"):
        fc = (1 - a) * np.exp(-T / T3) + a * np.exp(-T / T1) + np.where(T2 != 0, np.exp(-T2 / T), 0.0)
        lfc = np.log10(np.maximum(fc, 1e-300))
        lpr = np.log10(np.maximum(pr, 1e-300))
        x = lpr - 0.4 - 0.67 * lfc
        f1 = x / (0.75 - 1.27 * lfc - 0.14 * x)
        F = np.where(tro, 10 ** (lfc / (1 + f1 * f1)), F)
    kf = np.where(fall, kf * pr / (1 + pr) * F, kf)
    kf = kf * np.where(mech.rxn_type == 1, concm, 1.0)
    rkc = np.where(mech.reversible != 0,
                   np.minimum(np.exp(g @ (nu_p - nu_r) + dn * np.log(R_GAS * T / P_REF)), 1e300), 0.0)
    logc = np.log(np.maximum(c, 1e-300))
    ropf = kf * np.exp(logc @ nu_r)
    ropr = kf * rkc * np.exp(logc @ nu_p)
    creation = nu_p @ ropf + nu_r @ ropr
    destruction = nu_r @ ropf + nu_p @ ropr
    net = (nu_p - nu_r) @ (ropf - ropr)
    X = ym * mmw
    cp_mass = R_GAS * (X @ cp_R) / mmw
    return {"creation": creation, "destruction": destruction, "net": net, "hk": h_RT * R_GAS * T,
            "cp_mass": cp_mass, "density": rho, "ropf": ropf, "ropr": ropr}
