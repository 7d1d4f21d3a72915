// Device thermo / kinetics of the source term, evaluated by one warp per
// grid point (lanes split species and reactions). Restates what the
// reference obtains from Cantera in SourceSystemQSS::odefun and
// SourceSystemCVODE::f (src/sourceSystem.cpp:128-164, 445-499) and the
// 'interp' model of InterpKinetics / MultiArrheniusInterp
// (src/chemistry0d.cpp:271-436):
//   NASA7 cp/R, h/RT, s/R; modified Arrhenius rates; third-body
//   concentrations from efficiencies; Lindemann / Troe falloff; reverse rates
//   through 1/Kc = exp(dG0/RT) (RT/p0)^dn capped at 1e300; creation,
//   destruction and net production rates.
// Every sum over species is a warp reduction in one fixed order (element k
// in lane k mod 32, lanes combined by an xor butterfly). The translation unit
// is compiled without automatic FMA contraction; the multiply-adds that are
// fused are written as fma(), in the same places as in the CPU oracle.
#pragma once

#include <cstdint>

#include "emath.cuh"

namespace ember {

constexpr double kGasConstant = 6.02214076e26 * 1.380649e-23;  // J/kmol/K
constexpr double kOneAtm = 101325.0;
constexpr double kBigNumber = 1e300;
constexpr double kSmallNumber = 1e-300;
constexpr int kMaxStoich = 4;

enum : int { RXN_ELEMENTARY = 0, RXN_THREE_BODY = 1, RXN_LINDEMANN = 2, RXN_TROE = 3 };
enum : int { KIN_STANDARD = 0, KIN_INTERP = 1 };
enum : int { STATE_NORMALIZED = 0, STATE_NO_NORM = 1 };

// Device tables of one mechanism (all arrays in global memory).
struct MechView {
    int S, R, nT;
    double Tmin, Tmax;
    const double* W;      // [S]
    const double* rW;     // [S] 1/W
    const double* tmid;   // [S]
    const double* nasa;   // [S][14]
    const double* hc;     // [S][10] h/RT polynomial coefficients a0, a1/2, a2/3, a3/4, a4/5 per range
    const double* sc;     // [S][8]  s/R polynomial coefficients a1, a2/2, a3/3, a4/4 per range
    const int* type;      // [R]
    const int* rev;       // [R]
    const int* reac;      // [R][4]
    const int* prod;      // [R][4]
    const double* arr;    // [R][3]
    const double* arr_low;// [R][3]
    const double* troe;   // [R][4]
    const double* def_eff;// [R]
    const int* eff_off;   // [R+1]
    const int* eff_sp;
    const double* eff_val;
    const double* mult;   // [R]
    const double* dn;     // [R]
    const int* sp_off;    // [S+1] reactions in which species k occurs
    const int* sp_ent;    // packed: reaction | n_product_occurrences << 24 | n_reactant_occurrences << 28
    const double2* kf_tab;// [nT][R] (value, slope)
    const double2* kc_tab;// [nT][R]
};

// Per-warp shared-memory work area of the kinetics.
struct ChemSmem {
    double* c;     // [S] concentrations
    double* ym;    // [S]
    double* cpR;   // [S]
    double* hRT;   // [S]
    double* gRT;   // [S]
    double* kf;    // [R] forward rate constants at the cached T (falloff rows: unused)
    double* rkc;   // [R] 1/Kc at the cached T
    double* ropf;  // [R]
    double* ropr;  // [R]
    double* wq;    // [S] creation
    double* wd;    // [S] destruction
    double* wn;    // [S] net
    double* hk;    // [S] partial molar enthalpies [J/kmol]

    static __host__ __device__ size_t doubles(int S, int R) { return size_t(9) * S + size_t(4) * R; }

    __device__ void carve(double* base, int S, int R) {
        c = base;
        ym = c + S;
        cpR = ym + S;
        hRT = cpR + S;
        gRT = hRT + S;
        wq = gRT + S;
        wd = wq + S;
        wn = wd + S;
        hk = wn + S;
        kf = hk + S;
        rkc = kf + R;
        ropf = rkc + R;
        ropr = ropf + R;
    }
};

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

__device__ __forceinline__ double warp_sum_partial(double p) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) p = p + __shfl_xor_sync(0xffffffffu, p, off);
    return p;
}

// Sum of x[0..n) in the fixed warp order (x in shared memory).
__device__ __forceinline__ double warp_sum(const double* x, int n) {
    double p = 0.0;
    for (int k = lane_id(); k < n; k += 32) p = p + x[k];
    return warp_sum_partial(p);
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        double o = __shfl_xor_sync(0xffffffffu, v, off);
        v = (v < o) ? o : v;
    }
    return v;
}

__device__ __forceinline__ double dmaxr(double a, double b) { return (a < b) ? b : a; }  // std::max
__device__ __forceinline__ double dminr(double a, double b) { return (b < a) ? b : a; }  // std::min

__device__ __forceinline__ double arrhenius(const double* p, double lnT, double rT) {
    return p[0] * em_exp(fma(p[1], lnT, -(p[2] * rT)));
}

// NASA7 thermo of every species at T into cpR, hRT, gRT (lanes over species).
__device__ __forceinline__ void chem_thermo(const MechView& m, ChemSmem& w, double T, double lnT, double rT) {
    for (int k = lane_id(); k < m.S; k += 32) {
        const int r = (T <= m.tmid[k]) ? 0 : 1;
        const double* a = m.nasa + 14 * k + 7 * r;
        const double* h = m.hc + 10 * k + 5 * r;
        const double* s = m.sc + 8 * k + 4 * r;
        double cp = fma(fma(fma(fma(a[4], T, a[3]), T, a[2]), T, a[1]), T, a[0]);
        double hr = fma(fma(fma(fma(h[4], T, h[3]), T, h[2]), T, h[1]), T, h[0]) + a[5] * rT;
        double sp = fma(fma(fma(s[3], T, s[2]), T, s[1]), T, s[0]);
        double sr = fma(a[0], lnT, fma(sp, T, a[6]));
        w.cpR[k] = cp;
        w.hRT[k] = hr;
        w.gRT[k] = hr - sr;
    }
    __syncwarp();
}

// Temperature-only part: thermo, forward rate constants of non-falloff
// reactions and 1/Kc, standard formulas or interpolation tables.
__device__ __forceinline__ void chem_rate_constants(const MechView& m, ChemSmem& w, double T, int use_tables) {
    const double lnT = em_log(T), rT = 1.0 / T;
    chem_thermo(m, w, T, lnT, rT);
    const double lnRTp = em_log((kGasConstant * T) / kOneAtm);
    const bool in_table = use_tables && T >= m.Tmin && T <= m.Tmax;
    int n = 0;
    double dT = 0.0;
    if (in_table) {
        double fn = floor((T - m.Tmin) / (m.Tmax - m.Tmin) * (m.nT - 1));
        n = static_cast<int>(fn);
        if (n > m.nT - 1) n = m.nT - 1;
        dT = T - static_cast<double>(n) * (m.Tmax - m.Tmin) / (m.nT - 1) - m.Tmin;
    }
    for (int i = lane_id(); i < m.R; i += 32) {
        const int ty = m.type[i];
        double kf = 0.0;
        if (ty == RXN_ELEMENTARY || ty == RXN_THREE_BODY) {
            if (in_table) {
                double2 e = m.kf_tab[size_t(n) * m.R + i];
                kf = e.x + e.y * dT;
            } else {
                kf = arrhenius(m.arr + 3 * i, lnT, rT);
            }
        }
        double rkc = 0.0;
        if (m.rev[i]) {
            if (in_table) {
                double2 e = m.kc_tab[size_t(n) * m.R + i];
                rkc = e.x + e.y * dT;
            } else {
                double dg = 0.0;
                const int* pr = m.prod + kMaxStoich * i;
                const int* rc = m.reac + kMaxStoich * i;
#pragma unroll
                for (int o = 0; o < kMaxStoich; ++o)
                    if (pr[o] >= 0) dg = dg + w.gRT[pr[o]];
#pragma unroll
                for (int o = 0; o < kMaxStoich; ++o)
                    if (rc[o] >= 0) dg = dg - w.gRT[rc[o]];
                rkc = dminr(em_exp(fma(m.dn[i], lnRTp, dg)), kBigNumber);
            }
        }
        w.kf[i] = kf;
        w.rkc[i] = rkc;
    }
    __syncwarp();
}

// Composition part of the state setter (setState_TPY or NoNorm), rates of
// progress, production rates and thermo outputs at (T, Y). Rate constants
// must be current for T (chem_rate_constants). Y is in shared memory.
// Returns rho and cp_mass on every lane.
__device__ __forceinline__ void chem_rates(const MechView& m, ChemSmem& w, double p, int mode, double T,
                                           const double* Y, double& rho_out, double& cp_out, bool want_net) {
    const int S = m.S;
    const int lane = lane_id();
    if (mode == STATE_NORMALIZED) {
        double part = 0.0;
        for (int k = lane; k < S; k += 32) part = part + dmaxr(Y[k], 0.0);
        const double rnorm = 1.0 / warp_sum_partial(part);
        for (int k = lane; k < S; k += 32) w.ym[k] = (dmaxr(Y[k], 0.0) * rnorm) * m.rW[k];
    } else {
        for (int k = lane; k < S; k += 32) w.ym[k] = Y[k] * m.rW[k];
    }
    double part = 0.0;
    for (int k = lane; k < S; k += 32) part = part + w.ym[k];
    const double mmw = 1.0 / warp_sum_partial(part);
    const double rho = (p * mmw) / (kGasConstant * T);
    for (int k = lane; k < S; k += 32) w.c[k] = w.ym[k] * rho;
    __syncwarp();
    const double ctot = rho / mmw;
    const double lnT = em_log(T), rT = 1.0 / T;
    for (int i = lane; i < m.R; i += 32) {
        const int ty = m.type[i];
        double kf = w.kf[i];
        double concm = 0.0;
        if (ty != RXN_ELEMENTARY) {
            const double de = m.def_eff[i];
            concm = de * ctot;
            for (int e = m.eff_off[i]; e < m.eff_off[i + 1]; ++e)
                concm = fma(m.eff_val[e] - de, w.c[m.eff_sp[e]], concm);
        }
        if (ty == RXN_LINDEMANN || ty == RXN_TROE) {
            const double kinf = arrhenius(m.arr + 3 * i, lnT, rT);
            const double k0 = arrhenius(m.arr_low + 3 * i, lnT, rT);
            const double pr = (concm * k0) / (kinf + kSmallNumber);
            double F = 1.0;
            if (ty == RXN_TROE) {
                const double* tp = m.troe + 4 * i;
                double fc = (1.0 - tp[0]) * em_exp(-T / tp[1]) + tp[0] * em_exp(-T / tp[2]);
                if (tp[3] != 0.0) fc = fc + em_exp(-tp[3] * rT);
                const double lfc = em_log10(dmaxr(fc, kSmallNumber));
                const double lpr = em_log10(dmaxr(pr, kSmallNumber));
                const double cc = -0.4 - 0.67 * lfc;
                const double nn = 0.75 - 1.27 * lfc;
                const double x = lpr + cc;
                const double f1 = x / (nn - 0.14 * x);
                F = em_exp10(lfc / (1.0 + f1 * f1));
            }
            kf = (pr * (F / (1.0 + pr))) * kinf;
        }
        double rf = kf * m.mult[i];
        if (ty == RXN_THREE_BODY) rf = rf * concm;
        double ropf = rf, ropr = 0.0;
        const int* rc = m.reac + kMaxStoich * i;
        const int* pd = m.prod + kMaxStoich * i;
#pragma unroll
        for (int o = 0; o < kMaxStoich; ++o)
            if (rc[o] >= 0) ropf = ropf * w.c[rc[o]];
        if (m.rev[i]) {
            ropr = rf * w.rkc[i];
#pragma unroll
            for (int o = 0; o < kMaxStoich; ++o)
                if (pd[o] >= 0) ropr = ropr * w.c[pd[o]];
        }
        w.ropf[i] = ropf;
        w.ropr[i] = ropr;
    }
    __syncwarp();
    const double RT = kGasConstant * T;
    double cpart = 0.0;
    for (int k = lane; k < S; k += 32) {
        double q = 0.0, d = 0.0, nt = 0.0;
        for (int e = m.sp_off[k]; e < m.sp_off[k + 1]; ++e) {
            const int ent = m.sp_ent[e];
            const int i = ent & 0xffffff;
            const int np = (ent >> 24) & 0xf;
            const int nr = (ent >> 28) & 0xf;
            const double f = w.ropf[i], r = w.ropr[i];
            for (int o = 0; o < np; ++o) q = q + f;
            for (int o = 0; o < nr; ++o) q = q + r;
            for (int o = 0; o < nr; ++o) d = d + f;
            for (int o = 0; o < np; ++o) d = d + r;
            if (want_net) {
                const double net = f - r;
                for (int o = 0; o < np; ++o) nt = nt + net;
                for (int o = 0; o < nr; ++o) nt = nt - net;
            }
        }
        w.wq[k] = q;
        w.wd[k] = d;
        w.wn[k] = nt;
        w.hk[k] = w.hRT[k] * RT;  // updateThermo: h_k [J/kmol]
        cpart = cpart + (w.ym[k] * mmw) * w.cpR[k];
    }
    cp_out = (kGasConstant * warp_sum_partial(cpart)) / mmw;
    rho_out = rho;
    __syncwarp();
}

}  // namespace ember
