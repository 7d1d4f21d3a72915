"""Gas-phase mechanism data in the structure-of-arrays form of the C ABI
(``ember_mech_desc`` in include/ember_gpu.h), and a seeded synthetic
mechanism generator.

Units are Cantera's internal SI-kmol units: A in (m^3/kmol)^(n-1)/s, Ea as
Ea/R in K, molecular weights in kg/kmol, NASA7 polynomials in the standard
form (cp/R, h/RT, s/R).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
import itertools

import numpy as np

GAS_CONSTANT = 6.02214076e26 * 1.380649e-23   # J/kmol/K (exact SI definition)
ONE_ATM = 101325.0
KCAL_PER_MOL_TO_K = 4184.0 * 1000.0 / GAS_CONSTANT   # Ea[kcal/mol] -> Ea/R [K]
MAX_STOICH = 4
T_REF = 1000.0   # K, reference temperature of the synthetic rate draws

RXN_ELEMENTARY, RXN_THREE_BODY, RXN_LINDEMANN, RXN_TROE = 0, 1, 2, 3

# IUPAC standard atomic weights (abridged), kg/kmol.
ATOMIC_WEIGHT = {"H": 1.008, "C": 12.011, "N": 14.007, "O": 15.999, "Ar": 39.95}


class MechDesc(C.Structure):
    _fields_ = [
        ("n_species", C.c_int), ("n_reactions", C.c_int),
        ("mol_weight", C.c_void_p), ("nasa_tmid", C.c_void_p), ("nasa_coeffs", C.c_void_p),
        ("rxn_type", C.c_void_p), ("reversible", C.c_void_p), ("reactants", C.c_void_p),
        ("products", C.c_void_p), ("arrhenius", C.c_void_p), ("arrhenius_low", C.c_void_p),
        ("troe", C.c_void_p), ("default_efficiency", C.c_void_p), ("efficiency_offsets", C.c_void_p),
        ("efficiency_species", C.c_void_p), ("efficiency_values", C.c_void_p),
    ]


@dataclass
class Mechanism:
    species: list
    composition: list            # dict element -> count per species
    mol_weight: np.ndarray       # [S]
    nasa_tmid: np.ndarray        # [S]
    nasa_coeffs: np.ndarray      # [S, 14]
    rxn_type: np.ndarray         # [R] int32
    reversible: np.ndarray       # [R] int32
    reactants: np.ndarray        # [R, 4] int32 (-1 unused)
    products: np.ndarray         # [R, 4] int32
    arrhenius: np.ndarray        # [R, 3]
    arrhenius_low: np.ndarray    # [R, 3]
    troe: np.ndarray             # [R, 4]
    default_efficiency: np.ndarray   # [R]
    efficiency_offsets: np.ndarray   # [R+1] int64
    efficiency_species: np.ndarray   # int32
    efficiency_values: np.ndarray    # float64
    name: str = "mechanism"
    _keep: list = field(default_factory=list, repr=False)

    @property
    def n_species(self) -> int:
        return len(self.species)

    @property
    def n_reactions(self) -> int:
        return int(self.rxn_type.size)

    @property
    def n_vars(self) -> int:
        return self.n_species + 2

    def species_index(self, name: str) -> int:
        return self.species.index(name)

    def validate(self) -> None:
        S, R = self.n_species, self.n_reactions
        assert self.mol_weight.shape == (S,) and self.nasa_coeffs.shape == (S, 14)
        assert self.reactants.shape == (R, MAX_STOICH) and self.products.shape == (R, MAX_STOICH)
        for side in (self.reactants, self.products):
            assert ((side >= -1) & (side < S)).all()
            assert (side[:, 0] >= 0).all(), "every reaction side needs a species"
        assert self.efficiency_offsets.shape == (R + 1,) and self.efficiency_offsets[0] == 0

    def desc(self) -> MechDesc:
        """ctypes ember_mech_desc pointing at this object's arrays."""
        arrs = {
            "mol_weight": np.ascontiguousarray(self.mol_weight, dtype=np.float64),
            "nasa_tmid": np.ascontiguousarray(self.nasa_tmid, dtype=np.float64),
            "nasa_coeffs": np.ascontiguousarray(self.nasa_coeffs, dtype=np.float64),
            "rxn_type": np.ascontiguousarray(self.rxn_type, dtype=np.int32),
            "reversible": np.ascontiguousarray(self.reversible, dtype=np.int32),
            "reactants": np.ascontiguousarray(self.reactants, dtype=np.int32),
            "products": np.ascontiguousarray(self.products, dtype=np.int32),
            "arrhenius": np.ascontiguousarray(self.arrhenius, dtype=np.float64),
            "arrhenius_low": np.ascontiguousarray(self.arrhenius_low, dtype=np.float64),
            "troe": np.ascontiguousarray(self.troe, dtype=np.float64),
            "default_efficiency": np.ascontiguousarray(self.default_efficiency, dtype=np.float64),
            "efficiency_offsets": np.ascontiguousarray(self.efficiency_offsets, dtype=np.int64),
            "efficiency_species": np.ascontiguousarray(self.efficiency_species, dtype=np.int32),
            "efficiency_values": np.ascontiguousarray(self.efficiency_values, dtype=np.float64),
        }
        self._keep = list(arrs.values())
        d = MechDesc()
        d.n_species = self.n_species
        d.n_reactions = self.n_reactions
        for k, v in arrs.items():
            setattr(d, k, v.ctypes.data if v.size else None)
        return d

    def stoich_matrices(self):
        """Dense reactant / product stoichiometric coefficients [S, R]."""
        S, R = self.n_species, self.n_reactions
        nu_r = np.zeros((S, R))
        nu_p = np.zeros((S, R))
        for i in range(R):
            for k in self.reactants[i]:
                if k >= 0:
                    nu_r[k, i] += 1
            for k in self.products[i]:
                if k >= 0:
                    nu_p[k, i] += 1
        return nu_r, nu_p

    def element_matrix(self):
        elems = sorted({e for comp in self.composition for e in comp})
        return elems, np.array([[comp.get(e, 0) for comp in self.composition] for e in elems], dtype=float)


# ---------------------------------------------------------------------------
# NASA7 helpers (standard polynomial forms)

def nasa_cp_R(a, T):
    return a[0] + T * (a[1] + T * (a[2] + T * (a[3] + T * a[4])))


def nasa_h_RT(a, T):
    return a[0] + T * (a[1] / 2 + T * (a[2] / 3 + T * (a[3] / 4 + T * a[4] / 5))) + a[5] / T


def nasa_s_R(a, T):
    return a[0] * np.log(T) + T * (a[1] + T * (a[2] / 2 + T * (a[3] / 3 + T * a[4] / 4))) + a[6]


def _fit_nasa(cp_R_fn, h298_R, s298_R, tlow=300.0, tmid=1000.0, thigh=3500.0):
    """Two-range NASA7 fit of a smooth cp/R(T) with cp continuous at tmid, and
    a5/a6 set so that h(298.15) and s(298.15) match and h, s are continuous."""
    Tl = np.linspace(tlow, tmid, 60)
    Th = np.linspace(tmid, thigh, 120)
    V = lambda T: np.vander(T, 5, increasing=True)
    # least squares on both ranges with the constraint cp_low(tmid) = cp_high(tmid)
    A = np.zeros((len(Tl) + len(Th), 10))
    A[:len(Tl), :5] = V(Tl)
    A[len(Tl):, 5:] = V(Th)
    rhs = np.concatenate([cp_R_fn(Tl), cp_R_fn(Th)])
    cons = np.zeros(10)
    cons[:5] = V(np.array([tmid]))[0]
    cons[5:] = -V(np.array([tmid]))[0]
    K = np.zeros((11, 11))
    K[:10, :10] = A.T @ A
    K[:10, 10] = cons
    K[10, :10] = cons
    sol = np.linalg.solve(K, np.concatenate([A.T @ rhs, [0.0]]))
    lo = np.zeros(7)
    hi = np.zeros(7)
    lo[:5], hi[:5] = sol[:5], sol[5:10]
    T0 = 298.15
    lo[5] = (h298_R / T0 - nasa_h_RT(np.concatenate([lo[:5], [0, 0]]), T0)) * T0
    lo[6] = s298_R - nasa_s_R(np.concatenate([lo[:5], [0, 0]]), T0)
    hi[5] = (nasa_h_RT(lo, tmid) - nasa_h_RT(np.concatenate([hi[:5], [0, 0]]), tmid)) * tmid
    hi[6] = nasa_s_R(lo, tmid) - nasa_s_R(np.concatenate([hi[:5], [0, 0]]), tmid)
    return np.concatenate([lo, hi])


def _formula(comp):
    out = ""
    for e in ("C", "H", "O", "N", "Ar"):
        n = comp.get(e, 0)
        if n:
            out += e + (str(n) if n > 1 else "")
    return out


def synthetic_mechanism(n_species: int = 150, n_reactions: int = 1000, seed: int = 150_1000,
                        frac_three_body: float = 0.10, frac_troe: float = 0.05,
                        a_range=(1e8, 1e16), b_range=(-2.0, 3.0), ea_kcal=(0.0, 60.0)) -> Mechanism:
    """Seeded synthetic C/H/O/N mechanism.

    Species: the small molecules needed for a CH4/air blend (CH4, O2, N2,
    CO2, H2O and a few radicals, named by formula) plus random C/H/O/N
    compositions. Thermo: a rigid-rotor / harmonic-oscillator cp/R(T) with
    seeded vibrational temperatures, fitted to two-range NASA7 polynomials;
    seeded formation enthalpies and entropies. Reactions: element-balanced,
    all reversible; exchanges A + B <=> C + D, plus recombinations
    A + B (+M) <=> AB (+M) as three-body (frac_three_body) and Troe falloff
    (frac_troe) reactions, each written in its exothermic direction
    (standard enthalpy change at 298 K <= 0), so that reverse rates follow
    from the equilibrium constant without exceeding the forward ones. Rate
    parameters per reaction: A log-uniform in a_range (cm, mol, s units) as
    the rate at T_REF = 1000 K (Cantera's factor is A T_REF^-b), b uniform in
    b_range, Ea uniform in ea_kcal (kcal/mol).
    """
    rng = np.random.default_rng(seed)
    base = [{"C": 1, "H": 4}, {"O": 2}, {"N": 2}, {"C": 1, "O": 2}, {"H": 2, "O": 1}, {"C": 1, "O": 1},
            {"H": 2}, {"H": 1}, {"O": 1}, {"O": 1, "H": 1}, {"H": 1, "O": 2}, {"H": 2, "O": 2},
            {"C": 1, "H": 3}, {"C": 1, "H": 2, "O": 1}, {"C": 1, "H": 1, "O": 1}, {"N": 1}, {"N": 1, "O": 1}]
    comps = [dict(c) for c in base]
    seen = {tuple(sorted(c.items())) for c in comps}
    # Random small molecules, then closure so recombinations exist.
    while len(comps) < n_species:
        c = {"C": int(rng.integers(0, 4)), "H": int(rng.integers(0, 9)), "O": int(rng.integers(0, 4)),
             "N": int(rng.integers(0, 3)) if rng.random() < 0.3 else 0}
        c = {e: n for e, n in c.items() if n}
        if not c or sum(c.values()) > 10:
            continue
        key = tuple(sorted(c.items()))
        if key in seen:
            continue
        seen.add(key)
        comps.append(c)
    comps = comps[:n_species]
    names = [_formula(c) for c in comps]
    W = np.array([sum(ATOMIC_WEIGHT[e] * n for e, n in c.items()) for c in comps])

    # Thermo
    coeffs = np.zeros((n_species, 14))
    for k, c in enumerate(comps):
        na = sum(c.values())
        if na == 1:
            rot, modes = 0.0, np.zeros(0)
        elif na == 2:
            rot, modes = 1.0, np.exp(rng.uniform(np.log(800), np.log(4500), 1))
        else:
            rot, modes = 1.5, np.exp(rng.uniform(np.log(300), np.log(4500), 3 * na - 6))

        def cp_R(T, modes=modes, rot=rot):
            T = np.asarray(T, dtype=float)
            x = modes[None, :] / T[:, None] if modes.size else np.zeros((T.size, 0))
            ein = (x * x * np.exp(x) / np.expm1(x) ** 2).sum(axis=1) if modes.size else np.zeros(T.size)
            return 2.5 + rot + ein

        h298_R = (-na * rng.uniform(0.0, 120.0) + rng.uniform(-50.0, 150.0)) * 1e6 / GAS_CONSTANT
        s298_R = 15.0 + 2.5 * np.log(W[k]) + 2.0 * na ** 0.8 + rng.uniform(-2, 2)
        coeffs[k] = _fit_nasa(cp_R, h298_R, s298_R)
    tmid = np.full(n_species, 1000.0)

    # Reactions
    index = {tuple(sorted(c.items())): k for k, c in enumerate(comps)}
    add = lambda a, b: tuple(sorted({e: a.get(e, 0) + b.get(e, 0) for e in set(a) | set(b)}.items()))
    pair_sum = {}
    for i, j in itertools.combinations_with_replacement(range(n_species), 2):
        pair_sum.setdefault(add(comps[i], comps[j]), []).append((i, j))
    recomb = [(i, j, index[s]) for s, pairs in pair_sum.items() if s in index for (i, j) in pairs
              if index[s] not in (i, j)]
    exchange_keys = [s for s, pairs in pair_sum.items() if len(pairs) >= 2]
    n_tb = int(round(frac_three_body * n_reactions))
    n_troe = int(round(frac_troe * n_reactions))
    n_el = n_reactions - n_tb - n_troe
    seen_r = set()
    rxns = []

    h298 = np.array([nasa_h_RT(coeffs[k, :7], 298.15) for k in range(n_species)])  # h/RT at 298.15 K

    def exothermic(reac, prod):
        """Orient a reaction so that its standard enthalpy change at 298 K is <= 0."""
        dh = sum(h298[k] for k in prod) - sum(h298[k] for k in reac)
        return (reac, prod) if dh <= 0 else (prod, reac)

    def draw_arr(order):
        # A is drawn as the rate constant at T_REF (cm, mol, s units); Cantera's
        # pre-exponential factor of k = A T^b exp(-Ea/RT) is then A T_REF^-b.
        A = np.exp(rng.uniform(np.log(a_range[0]), np.log(a_range[1])))
        b = rng.uniform(*b_range)
        A *= (1e-3) ** (order - 1) * T_REF ** (-b)  # (cm^3/mol)^(order-1)/s -> (m^3/kmol)^(order-1)/s
        return [A, b, rng.uniform(*ea_kcal) * KCAL_PER_MOL_TO_K]

    rec_order = rng.permutation(len(recomb))
    ri = 0
    for kind, count in ((RXN_THREE_BODY, n_tb), (RXN_TROE, n_troe)):
        made = 0
        while made < count and ri < len(rec_order):
            i, j, p = recomb[rec_order[ri]]
            ri += 1
            key = (tuple(sorted((i, j))), (p,))
            if key in seen_r:
                continue
            seen_r.add(key)
            made += 1
            reac, prod = exothermic([i, j], [p])
            r = {"type": kind, "reac": reac, "prod": prod}
            if kind == RXN_THREE_BODY:
                r["arr"] = draw_arr(len(reac) + 1)
                r["low"] = [0.0, 0.0, 0.0]
                r["troe"] = [0.0, 0.0, 0.0, 0.0]
            else:
                r["arr"] = draw_arr(len(reac))
                r["low"] = draw_arr(len(reac) + 1)
                r["troe"] = [rng.uniform(0.4, 0.8), np.exp(rng.uniform(np.log(50), np.log(500))),
                             np.exp(rng.uniform(np.log(500), np.log(5000))),
                             np.exp(rng.uniform(np.log(2000), np.log(8000))) if rng.random() < 0.5 else 0.0]
            nov = rng.choice(n_species, size=int(rng.integers(2, 6)), replace=False)
            r["eff"] = [(int(k), float(rng.uniform(0.3, 6.0))) for k in nov]
            rxns.append(r)
    tries = 0
    while len(rxns) < n_reactions and tries < 100 * n_reactions:
        tries += 1
        s_key = exchange_keys[int(rng.integers(len(exchange_keys)))]
        pairs = pair_sum[s_key]
        a, b = rng.choice(len(pairs), size=2, replace=False)
        (i, j), (k, l) = pairs[a], pairs[b]
        key = tuple(sorted([tuple(sorted((i, j))), tuple(sorted((k, l)))]))
        if key in seen_r:
            continue
        seen_r.add(key)
        reac, prod = exothermic([i, j], [k, l])
        rxns.append({"type": RXN_ELEMENTARY, "reac": reac, "prod": prod, "arr": draw_arr(2),
                     "low": [0.0, 0.0, 0.0], "troe": [0.0, 0.0, 0.0, 0.0], "eff": []})
    rxns = rxns[:n_reactions]
    order = rng.permutation(len(rxns))
    rxns = [rxns[i] for i in order]
    R = len(rxns)
    reac = -np.ones((R, MAX_STOICH), dtype=np.int32)
    prod = -np.ones((R, MAX_STOICH), dtype=np.int32)
    for i, r in enumerate(rxns):
        reac[i, :len(r["reac"])] = r["reac"]
        prod[i, :len(r["prod"])] = r["prod"]
    eff_off = np.zeros(R + 1, dtype=np.int64)
    eff_sp, eff_val = [], []
    for i, r in enumerate(rxns):
        for k, v in r["eff"]:
            eff_sp.append(k)
            eff_val.append(v)
        eff_off[i + 1] = len(eff_sp)
    mech = Mechanism(
        species=names, composition=comps, mol_weight=W, nasa_tmid=tmid, nasa_coeffs=coeffs,
        rxn_type=np.array([r["type"] for r in rxns], dtype=np.int32),
        reversible=np.ones(R, dtype=np.int32), reactants=reac, products=prod,
        arrhenius=np.array([r["arr"] for r in rxns]), arrhenius_low=np.array([r["low"] for r in rxns]),
        troe=np.array([r["troe"] for r in rxns]),
        default_efficiency=np.array([1.0 if r["type"] != RXN_ELEMENTARY else 0.0 for r in rxns]),
        efficiency_offsets=eff_off, efficiency_species=np.array(eff_sp, dtype=np.int32),
        efficiency_values=np.array(eff_val, dtype=np.float64),
        name=f"synthetic-{n_species}sp-{R}rxn-seed{seed}")
    mech.validate()
    return mech


# ---------------------------------------------------------------------------
# Seeded reactor states (constant-pressure source-term inputs)

def stoichiometric_ch4_air(mech: Mechanism):
    """Mass fractions of stoichiometric CH4/air (O2 + 3.76 N2) and of its
    complete-combustion products (CO2 + 2 H2O + 7.52 N2)."""
    X = np.zeros(mech.n_species)
    X[mech.species_index("CH4")] = 1.0
    X[mech.species_index("O2")] = 2.0
    X[mech.species_index("N2")] = 7.52
    P = np.zeros(mech.n_species)
    P[mech.species_index("CO2")] = 1.0
    P[mech.species_index("H2O")] = 2.0
    P[mech.species_index("N2")] = 7.52
    to_y = lambda x: x * mech.mol_weight / np.sum(x * mech.mol_weight)
    return to_y(X), to_y(P)


def reactor_states(mech: Mechanism, n_points: int, seed: int = 4096, T_range=(800.0, 2400.0),
                   dt_range=(1e-6, 1e-4)):
    """Seeded constant-pressure states: T uniform in T_range, composition a
    mixture-fraction blend Z~U(0,1) of stoichiometric CH4/air and its
    complete-combustion products, renormalised in FP64; dt log-uniform in
    dt_range. Returns (state [n, S+2] as U, T, Y...; dt [n])."""
    rng = np.random.default_rng(seed)
    y_r, y_p = stoichiometric_ch4_air(mech)
    Z = rng.uniform(0.0, 1.0, n_points)
    T = rng.uniform(*T_range, n_points)
    dt = np.exp(rng.uniform(np.log(dt_range[0]), np.log(dt_range[1]), n_points))
    Y = (1.0 - Z)[:, None] * y_r[None, :] + Z[:, None] * y_p[None, :]
    Y /= Y.sum(axis=1, keepdims=True)
    state = np.zeros((n_points, mech.n_vars))
    state[:, 1] = T
    state[:, 2:] = Y
    return state, dt
