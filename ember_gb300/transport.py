"""Mixture-averaged transport properties on the GPU (``ember_transport_*``):
FlameSolver::updateChemicalProperties (src/flameSolver.cpp:652-699) with the
"Approx" model (src/chemistry0d.cpp:12-269), and a seeded generator of the
species fits for synthetic mechanisms.

The fits follow Cantera's non-CK form, quartics in ln T of
sqrt(mu_k)/T^(1/4), lambda_k/T^(1/2) and p D_jk/T^(3/2). Mechanism files with
real transport data (gri30.yaml) are not available here; synthetic_transport
fits curves from kinetic theory with seeded Lennard-Jones parameters instead.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from .mechanism import GAS_CONSTANT, Mechanism, nasa_cp_R

APPROX_THRESHOLD = 1e-5   # Chemistry.threshold default (python/ember/input.py:373-375)


class TransportDesc(C.Structure):
    _fields_ = [("n_species", C.c_int), ("visc_fit", C.c_void_p), ("cond_fit", C.c_void_p),
                ("diff_fit", C.c_void_p)]


class Properties(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in ("density", "mean_mol_weight", "cp_mass", "cp_species", "h_species",
                                          "conductivity", "viscosity", "rho_d")]


@dataclass
class TransportData:
    visc_fit: np.ndarray   # [S, 5]
    cond_fit: np.ndarray   # [S, 5]
    diff_fit: np.ndarray   # [S(S+1)/2, 5], pair (j <= k) at j S - j(j-1)/2 + k - j
    sigma: np.ndarray      # [S] Lennard-Jones diameters (Angstrom) the fits came from
    eps_k: np.ndarray      # [S] well depths / k_B (K)

    def desc(self, S: int):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (self.visc_fit, self.cond_fit, self.diff_fit)]
        self._keep = arrs
        d = TransportDesc()
        d.n_species = S
        d.visc_fit, d.cond_fit, d.diff_fit = (a.ctypes.data for a in arrs)
        return d


def pair_index(S: int, lo: int, hi: int) -> int:
    return lo * S - lo * (lo - 1) // 2 + (hi - lo)


def _omega22(ts):
    """Reduced collision integral Omega(2,2)* of the Lennard-Jones potential,
    Neufeld, Janzen and Aziz (1972) correlation."""
    return 1.16145 * ts ** -0.14874 + 0.52487 * np.exp(-0.77320 * ts) + 2.16178 * np.exp(-2.43787 * ts)


def _omega11(ts):
    """Omega(1,1)*, same correlation family."""
    return (1.06036 * ts ** -0.15610 + 0.19300 * np.exp(-0.47635 * ts) + 1.03587 * np.exp(-1.52996 * ts)
            + 1.76474 * np.exp(-3.89411 * ts))


def kinetic_theory(mech: Mechanism, sigma, eps_k, T):
    """Chapman-Enskog species viscosities [Pa s], modified-Eucken
    conductivities [W/m/K] and binary diffusion coefficients at unit pressure
    (p D_jk [Pa m^2/s]) on the temperatures T."""
    T = np.asarray(T, dtype=float)
    W = mech.mol_weight
    S = mech.n_species
    mu = 2.6693e-6 * np.sqrt(W[:, None] * T[None, :]) / (sigma[:, None] ** 2 * _omega22(T[None, :] / eps_k[:, None]))
    cp_R = np.array([np.where(T <= mech.nasa_tmid[k], nasa_cp_R(mech.nasa_coeffs[k, :7], T),
                              nasa_cp_R(mech.nasa_coeffs[k, 7:], T)) for k in range(S)])
    lam = mu * (GAS_CONSTANT / W[:, None]) * (cp_R + 1.25)
    lo, hi = np.triu_indices(S)
    s_jk = 0.5 * (sigma[lo] + sigma[hi])
    e_jk = np.sqrt(eps_k[lo] * eps_k[hi])
    red = np.sqrt(1.0 / W[lo] + 1.0 / W[hi])
    pD = 1.8583e-7 * 101325.0 * np.sqrt(T[None, :] ** 3) * red[:, None] / (
        s_jk[:, None] ** 2 * _omega11(T[None, :] / e_jk[:, None]))
    return mu, lam, pD


def synthetic_transport(mech: Mechanism, seed: int = 7, t_fit=(300.0, 3500.0)) -> TransportData:
    """Seeded transport fits for a (synthetic) mechanism: Lennard-Jones
    diameters 2.5-4.5 A growing with the number of atoms and well depths
    80-500 K, the kinetic-theory curves of kinetic_theory on 60 points of
    [300, 3500] K, and least-squares quartics in ln T of the fitted forms."""
    rng = np.random.default_rng(seed)
    S = mech.n_species
    atoms = np.array([sum(c.values()) for c in mech.composition], dtype=float)
    sigma = np.clip(2.4 + 0.45 * atoms ** 0.6 + rng.uniform(-0.2, 0.2, S), 2.5, 4.5)
    eps_k = np.clip(60.0 * atoms ** 0.7 + rng.uniform(20.0, 120.0, S), 80.0, 500.0)
    T = np.geomspace(t_fit[0], t_fit[1], 60)
    mu, lam, pD = kinetic_theory(mech, sigma, eps_k, T)
    lnT = np.log(T)
    A = np.vander(lnT, 5, increasing=True)
    fit = lambda Y: np.linalg.lstsq(A, Y.T, rcond=None)[0].T
    visc = fit(np.sqrt(mu) / T[None, :] ** 0.25)
    cond = fit(lam / np.sqrt(T)[None, :])
    diff = fit(pD / T[None, :] ** 1.5)
    return TransportData(visc_fit=visc, cond_fit=cond, diff_fit=diff, sigma=sigma, eps_k=eps_k)


class GpuTransport:
    """Transport fits uploaded next to a GpuMechanism (ember_transport handle)."""

    def __init__(self, gmech, data: TransportData):
        self.gmech = gmech
        self.data = data
        self.S = gmech.mech.n_species
        desc = data.desc(self.S)
        h = C.c_void_p()
        L.check(L.lib().ember_transport_create(gmech.handle, C.byref(desc), C.byref(h)), "ember_transport_create")
        self.handle = h

    def __del__(self):
        try:
            if self.handle:
                L.lib().ember_transport_destroy(self.handle)
        except Exception:
            pass

    def eval(self, T, Y, pressure: float = 101325.0, threshold: float = APPROX_THRESHOLD, stream=None, out=None):
        """Properties of the states (T [n], Y [n, S]; numpy arrays or torch CUDA
        tensors). Returns a dict of arrays shaped like the inputs; ``out``: such
        a dict to fill instead (e.g. page-locked host arrays)."""
        mem = L.mem_of(T)
        n = int(T.shape[0])
        S = self.S
        shapes = {"density": (n,), "mean_mol_weight": (n,), "cp_mass": (n,), "cp_species": (n, S),
                  "h_species": (n, S), "conductivity": (n,), "viscosity": (n,), "rho_d": (n, S)}
        if out is not None:
            assert set(out) == set(shapes) and all(tuple(out[k].shape) == s for k, s in shapes.items())
            if mem == L.MEM_HOST:
                T = np.ascontiguousarray(T, dtype=np.float64)
                Y = np.ascontiguousarray(Y, dtype=np.float64)
        elif mem == L.MEM_HOST:
            T = np.ascontiguousarray(T, dtype=np.float64)
            Y = np.ascontiguousarray(Y, dtype=np.float64)
            out = {k: np.empty(s) for k, s in shapes.items()}
        else:
            import torch
            out = {k: torch.empty(s, dtype=torch.float64, device=T.device) for k, s in shapes.items()}
        props = Properties(**{k: L.ptr(v) for k, v in out.items()})
        L.check(L.lib().ember_transport_eval(self.handle, n, float(pressure), float(threshold), L.ptr(T), L.ptr(Y),
                                             C.byref(props), mem, L.stream_ptr(stream)), "ember_transport_eval")
        return out
