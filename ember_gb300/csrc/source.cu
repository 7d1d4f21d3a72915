// Production (chemistry source term) stage on the GPU: mechanism upload,
// thermo/rate evaluation and the QSS source-term integrator.
//
// One CTA of kChemThreads threads integrates one grid point; the CTAs of a
// persistent grid take points from an atomic work counter, so that points
// needing many sub-steps do not hold up the others (the reference runs the same per-point integrations
// from a TBB parallel_for over points, src/flameSolver.cpp:754-836).
//
// Compiled with --fmad=false: only the fma() calls written in chem.cuh,
// emath.cuh and here are fused, in the same places as in the CPU oracle.
#include "common.cuh"
#include "chem.cuh"
#include "qss.cuh"
#include "source.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

namespace ember {

// ------------------------------------------------------- table building --

// Rate constants and 1/Kc at the table nodes (one CTA per node), from the
// same device functions as the standard model: InterpKinetics::updateROP /
// MultiArrheniusInterp::rebuildInterpData (src/chemistry0d.cpp:278-326, 401-436).
template <int NT>
__global__ void __launch_bounds__(NT) k_build_tables(MechView m, double* work) {
    const int node = blockIdx.x;
    const size_t sd = ChemSmem::doubles(m.S, m.R, m.n_tb, m.n_fo, false);
    double* base = work + size_t(node) * (sd + ChemSmem::global_doubles(m));
    ChemSmem w;
    w.carve(base, base + sd, m, false);
    const double T = m.Tmin + ((double)node) / (m.nT - 1) * (m.Tmax - m.Tmin);
    chem_rate_constants<NT>(m, w, T, 0);
    double2* kf = const_cast<double2*>(m.kf_tab) + size_t(node) * m.R;
    double2* kc = const_cast<double2*>(m.kc_tab) + size_t(node) * m.R;
    for (int i = threadIdx.x; i < m.R; i += NT) {
        const int ty = rinfo_type(m.rinfo[i]);
        // w.kfm holds kf * multiplier; the multipliers are 1 while tables are built
        kf[i].x = (ty == RXN_ELEMENTARY || ty == RXN_THREE_BODY) ? w.kfm[i] : 0.0;
        kc[i].x = w.rkc[i];
    }
}

__global__ void k_table_slopes(MechView m) {
    const double dT = (m.Tmax - m.Tmin) / (m.nT - 1);
    const size_t total = size_t(m.nT) * m.R;
    for (size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x; e < total; e += size_t(gridDim.x) * blockDim.x) {
        const int n = static_cast<int>(e / m.R);
        double2* kf = const_cast<double2*>(m.kf_tab);
        double2* kc = const_cast<double2*>(m.kc_tab);
        if (n < m.nT - 1) {
            kf[e].y = (kf[e + m.R].x - kf[e].x) / dT;
            kc[e].y = (kc[e + m.R].x - kc[e].x) / dT;
        } else {
            kf[e].y = 0.0;
            kc[e].y = 0.0;
        }
    }
}

// ------------------------------------------------------------- gas eval --

template <int NT>
__global__ void __launch_bounds__(NT) k_gas_eval(MechView m, int n, double p, int model, int mode,
                                                const double* __restrict__ T, const double* __restrict__ Y,
                                                double* kcache, double* creation, double* destruction, double* net,
                                                double* hk, double* cp_mass, double* density) {
    extern __shared__ double smem[];
    ChemSmem w;
    w.carve(smem, kcache + size_t(blockIdx.x) * ChemSmem::global_doubles(m), m, true);
    double* y = smem + ChemSmem::doubles(m.S, m.R, m.n_tb, m.n_fo, true);
    for (int j = blockIdx.x; j < n; j += gridDim.x) {
        for (int k = threadIdx.x; k < m.S; k += NT) y[k] = Y[size_t(j) * m.S + k];
        const double Tj = T[j];
        chem_rate_constants<NT>(m, w, Tj, model == KIN_INTERP);
        double rho, cp;
        chem_rates<NT>(m, w, p, mode, Tj, y, rho, cp, true);
        for (int k = threadIdx.x; k < m.S; k += NT) {
            const size_t o = size_t(j) * m.S + k;
            if (creation) creation[o] = w.wq[k];
            if (destruction) destruction[o] = w.wd[k];
            if (net) net[o] = w.wn[k];
            if (hk) hk[o] = w.hk[k];
        }
        if (threadIdx.x == 0) {
            if (cp_mass) cp_mass[j] = cp;
            if (density) density[j] = rho;
        }
        __syncthreads();
    }
}

// ------------------------------------------------------ QSS source term --

// SourceSystemQSS::odefun (src/sourceSystem.cpp:445-499): q/d of
// [U, T, Y]; T and the thermo (h_k, rho, cp) are refreshed only on
// predictor calls (src/sourceSystem.cpp:461-463, 501-515). With T frozen in
// the corrector, h_k (a function of T only) is the predictor's.
template <int NT>
struct SourceQssOde {
    MechView m;
    ChemSmem w;
    const SourceArgs* a;
    const double* split;  // this point's split constants (global) or null
    double x;
    double T;
    double rrho, rrc;     // 1/rho and 1/(rho cp) of the last predictor call
    double cachedT;

    __device__ void eval(double t, const double* y, double* q, double* d, bool corrector) {
        const int S = m.S;
        const int tid = threadIdx.x;
        if (!corrector) T = y[1];
        if (!(cachedT == T)) {
            chem_rate_constants<NT>(m, w, T, a->kinetics_model == KIN_INTERP);
            cachedT = T;
        }
        double rho_c, cp_c;
        chem_rates<NT>(m, w, a->pressure, STATE_NORMALIZED, T, y + 2, rho_c, cp_c, false);
        if (!corrector) {
            rrho = 1.0 / rho_c;
            rrc = 1.0 / (rho_c * cp_c);
        }
        const double *wq = w.wq, *wd = w.wd, *hk = w.hk;
        const double qdot =
            -block_sum<NT>(w.red, S, [&](int k, double p) { return fma(wq[k] - wd[k], hk[k], p); }) + igniter(*a, t, x);
        for (int i = tid; i < S + 2; i += NT) {
            const double sc = split ? split[i] : 0.0;
            if (i == 0) {
                q[0] = sc;
                d[0] = 0.0;
            } else if (i == 1) {
                q[1] = fma(qdot, rrc, sc);
                d[1] = 0.0 * rrc;
            } else {
                const int k = i - 2;
                q[i] = fma(w.wq[k] * m.W[k], rrho, sc);
                d[i] = (w.wd[k] * m.W[k]) * rrho;
            }
        }
        __syncthreads();
    }
};

struct EnforceNotMomentum {
    __device__ bool operator()(int i) const { return i != 0; }
};

struct SourceYmin {
    double minval;
    __device__ double operator()(int i) const { return i == 0 ? -1e4 : minval; }
};

// ---- longest-first work order ----------------------------------------------
// A point's cost grows with its interval (at least dt/dtmax steps), so the
// work queue hands out points by decreasing dt, bucketed by the binary
// exponent of dt (bucket 0: dt >= 32 s; each bucket spans a factor 2). The
// results do not depend on the order: every point is integrated on its own.

__device__ __forceinline__ int dt_bucket(double dt) {
    if (!(dt > 0.0)) return 63;
    const int e = static_cast<int>((__double_as_longlong(dt) >> 52) & 0x7ff);
    const int b = 1023 + 5 - e;
    return b < 0 ? 0 : (b > 63 ? 63 : b);
}

__global__ void k_order_hist(const double* __restrict__ dt, int n, int* counts) {
    __shared__ int local[64];
    if (threadIdx.x < 64) local[threadIdx.x] = 0;
    __syncthreads();
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
        atomicAdd(&local[dt_bucket(dt[j])], 1);
    __syncthreads();
    if (threadIdx.x < 64 && local[threadIdx.x]) atomicAdd(&counts[threadIdx.x], local[threadIdx.x]);
}

__global__ void k_order_scan(int* counts) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        int acc = 0;
        for (int b = 0; b < 64; ++b) {
            const int c = counts[b];
            counts[b] = acc;  // becomes the bucket's cursor
            acc += c;
        }
    }
}

__global__ void k_order_scatter(const double* __restrict__ dt, int n, int* cursor, int* order) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
        order[atomicAdd(&cursor[dt_bucket(dt[j])], 1)] = j;
}

// Resident CTAs per SM the register budget is sized for (none of the widths
// spills): 16 for NT = 32 (one warp per point, for small mechanisms whose
// passes are too short to hide barrier and shared-memory latency with a few
// points per SM), 6 for NT <= 96 (the shared-memory limit of the
// 150-species mechanism, 35 KB per point), 5 for 128, 4 for 160, 3 for 192,
// 2 for 256.
constexpr int qss_min_blocks(int nt) { return nt <= 32 ? 16 : (nt <= 96 ? 6 : (nt <= 128 ? 5 : (nt <= 160 ? 4 : (nt <= 192 ? 3 : 2)))); }

template <int NT>
__global__ void __launch_bounds__(NT, qss_min_blocks(NT)) k_source_qss(MechView m, SourceArgs a, int* counter,
                                                                      const int* order, double* kcache) {
    extern __shared__ double smem[];
    __shared__ int next_point;
    const int n = m.S + 2;
    const bool stab = a.qss_stability_check != 0;
    const size_t cd = ChemSmem::doubles(m.S, m.R, m.n_tb, m.n_fo, false);
    SourceQssOde<NT> ode;
    ode.m = m;
    ode.w.carve(smem, kcache + size_t(blockIdx.x) * ChemSmem::global_doubles(m), m, false);
    QssSmem v;
    v.carve(smem + cd, n, stab);
    ode.a = &a;
    ode.cachedT = __longlong_as_double(0x7ff8000000000000LL);  // NaN: nothing cached
    QssParams P;
    P.epsmin = a.qss_epsmin;
    P.epsmax = a.qss_epsmax;
    P.dtmin = a.qss_dtmin;
    P.dtmax = a.qss_dtmax;
    P.abstol = a.qss_abstol;
    P.itermax = a.qss_itermax;
    P.stability_check = a.qss_stability_check;
    P.max_steps = a.max_steps;
    const int tid = threadIdx.x;
    // the points of this launch: the work order, or the suspended points being resumed
    // Queue granularity: a CTA claims `chunk` consecutive slots of the order per atomic.
    const int n_work = a.resuming ? *a.susp_n : a.n;
    const int chunk = a.queue_chunk > 1 ? a.queue_chunk : 1;
    int slot = 0, left = 0;  // thread 0's current claim
    for (;;) {
        if (tid == 0) {
            if (left == 0) {
                slot = atomicAdd(counter, chunk);
                left = chunk;
            }
            next_point = slot < n_work ? (a.resuming ? a.susp_list[slot] : order[slot]) : a.n;
            ++slot;
            --left;
        }
        __syncthreads();
        const int j = next_point;
        __syncthreads();
        if (j >= a.n) break;
        const double* yin = (a.resuming ? a.state_out : a.state_in) + size_t(j) * n;
        for (int i = tid; i < n; i += NT) v.y[i] = yin[i];
        ode.split = a.split ? a.split + size_t(j) * n : nullptr;
        ode.x = a.x ? a.x[j] : 0.0;
        ode.T = yin[1];
        ode.rrho = 1.0;
        ode.rrc = 1.0;
        QssStats st;
        QssResume rs{};
        if (a.resuming) rs = a.resume[j];
        double* tape = a.tape ? a.tape + size_t(j) * a.tape_stride : nullptr;
        int ret = qss_integrate_block<NT>(ode, v, n, P, EnforceNotMomentum(), SourceYmin{a.qss_minval}, a.dt[j],
                                          a.t_start_dev ? *a.t_start_dev : a.t_start, ode.w.red, st, a.step_cap,
                                          a.resume ? &rs : nullptr, tape ? tape + kQssTapeHeader : nullptr,
                                          a.tape_cap);
        int nonfinite = 0;
        double* yout = a.state_out + size_t(j) * n;
        for (int i = tid; i < n; i += NT) {
            const double yi = v.y[i];
            nonfinite |= !isfinite(yi);
            yout[i] = yi;
        }
        nonfinite = __syncthreads_or(nonfinite);
        if (ret == 0 && nonfinite) ret = -21;
        if (tid == 0) {
            if (ret == kQssSuspended) {
                a.resume[j] = rs;
                a.susp_list[atomicAdd(a.susp_n, 1)] = j;
            } else if (tape) {
                tape[0] = st.steps;
                tape[1] = st.steps > a.tape_cap ? 1.0 : 0.0;
            }
            a.status[j] = ret;
            if (a.stats) {
                a.stats[4 * size_t(j) + 0] = st.steps;
                a.stats[4 * size_t(j) + 1] = st.gcount;
                a.stats[4 * size_t(j) + 2] = st.rcount;
                a.stats[4 * size_t(j) + 3] = 0;
            }
        }
    }
}

}  // namespace ember

// ================================================================ C ABI ==

using namespace ember;

extern "C" int ember_mech_create(const ember_mech_desc* d, ember_mech* out) {
    EMBER_CHECK_ARG(out != nullptr && d != nullptr, "null argument");
    *out = nullptr;
    const int S = d->n_species, R = d->n_reactions;
    EMBER_CHECK_ARG(S >= 1 && S < 0xffff && R >= 0 && R < (1 << 22), "bad mechanism size (S=%d, R=%d)", S, R);
    EMBER_CHECK_ARG(d->mol_weight && d->nasa_tmid && d->nasa_coeffs, "null species arrays");
    EMBER_CHECK_ARG(R == 0 || (d->rxn_type && d->reversible && d->reactants && d->products && d->arrhenius &&
                               d->arrhenius_low && d->troe && d->default_efficiency && d->efficiency_offsets),
                    "null reaction arrays");
    for (int k = 0; k < S; ++k) EMBER_CHECK_ARG(d->mol_weight[k] > 0, "species %d: molecular weight must be > 0", k);
    const int64_t ne = R ? d->efficiency_offsets[R] : 0;
    EMBER_CHECK_ARG(R == 0 || d->efficiency_offsets[0] == 0, "efficiency_offsets[0] must be 0");
    EMBER_CHECK_ARG(ne < (int64_t(1) << 31), "too many efficiency entries");
    for (int i = 0; i < R; ++i) {
        EMBER_CHECK_ARG(d->rxn_type[i] >= 0 && d->rxn_type[i] <= 3, "reaction %d: bad type %d", i, d->rxn_type[i]);
        EMBER_CHECK_ARG(d->efficiency_offsets[i + 1] >= d->efficiency_offsets[i], "reaction %d: bad efficiency offsets", i);
        int nr = 0, np = 0;
        for (int o = 0; o < EMBER_MAX_STOICH; ++o) {
            int r = d->reactants[i * EMBER_MAX_STOICH + o], p = d->products[i * EMBER_MAX_STOICH + o];
            EMBER_CHECK_ARG(r >= -1 && r < S && p >= -1 && p < S, "reaction %d: species index out of range", i);
            nr += r >= 0;
            np += p >= 0;
        }
        EMBER_CHECK_ARG(nr >= 1 && np >= 1, "reaction %d: needs at least one reactant and one product", i);
    }
    EMBER_CHECK_ARG(ne == 0 || (d->efficiency_species && d->efficiency_values), "null efficiency arrays");
    for (int64_t e = 0; e < ne; ++e)
        EMBER_CHECK_ARG(d->efficiency_species[e] >= 0 && d->efficiency_species[e] < S,
                        "efficiency entry %lld: bad species", (long long)e);
    EMBER_TRY(ensure_device());

    // ---- host-side derived tables ----
    std::vector<double> rW(S), hc(size_t(S) * 10), sc(size_t(S) * 8);
    for (int k = 0; k < S; ++k) {
        rW[k] = 1.0 / d->mol_weight[k];
        for (int r = 0; r < 2; ++r) {
            const double* a = d->nasa_coeffs + 14 * k + 7 * r;
            double* h = hc.data() + 10 * k + 5 * r;
            double* s = sc.data() + 8 * k + 4 * r;
            h[0] = a[0];
            h[1] = a[1] / 2.0;
            h[2] = a[2] / 3.0;
            h[3] = a[3] / 4.0;
            h[4] = a[4] / 5.0;
            s[0] = a[1];
            s[1] = a[2] / 2.0;
            s[2] = a[3] / 3.0;
            s[3] = a[4] / 4.0;
        }
    }
    const size_t Rs = std::max(R, 1);
    std::vector<int4> stoich(Rs, make_int4(-1, -1, -1, -1));
    std::vector<int> rinfo(Rs, 0), tb_rxn, tb_off(1, 0), tb_sp, fo_rxn, fo_tb, tb_fo;
    std::vector<double> dn(Rs, 0.0), mult(Rs, 1.0), tb_eff, tb_def, fo_arr, fo_troe;
    std::vector<std::vector<int>> lists(S);
    for (int i = 0; i < R; ++i) {
        // occurrences, compacted in order (unused slots: 0xffff)
        int rc[4] = {0xffff, 0xffff, 0xffff, 0xffff}, pr[4] = {0xffff, 0xffff, 0xffff, 0xffff};
        int nr = 0, np = 0;
        for (int o = 0; o < EMBER_MAX_STOICH; ++o) {
            int r = d->reactants[i * EMBER_MAX_STOICH + o], p = d->products[i * EMBER_MAX_STOICH + o];
            if (r >= 0) rc[nr++] = r;
            if (p >= 0) pr[np++] = p;
        }
        stoich[i] = make_int4(rc[0] | (rc[1] << 16), rc[2] | (rc[3] << 16), pr[0] | (pr[1] << 16), pr[2] | (pr[3] << 16));
        dn[i] = static_cast<double>(np - nr);
        const int ty = d->rxn_type[i];
        int slot = 0x3fffff;
        if (ty != EMBER_RXN_ELEMENTARY) {
            slot = static_cast<int>(tb_rxn.size());
            tb_rxn.push_back(i);
            const double de = d->default_efficiency[i];
            tb_def.push_back(de);
            for (int64_t e = d->efficiency_offsets[i]; e < d->efficiency_offsets[i + 1]; ++e) {
                tb_sp.push_back(d->efficiency_species[e]);
                tb_eff.push_back(d->efficiency_values[e] - de);
            }
            tb_off.push_back(static_cast<int>(tb_sp.size()));
            tb_fo.push_back(ty == EMBER_RXN_LINDEMANN || ty == EMBER_RXN_TROE ? static_cast<int>(fo_rxn.size()) : -1);
        }
        if (ty == EMBER_RXN_LINDEMANN || ty == EMBER_RXN_TROE) {
            fo_rxn.push_back(i);
            fo_tb.push_back(slot);
            for (int q = 0; q < 3; ++q) fo_arr.push_back(d->arrhenius_low[3 * i + q]);
            // a, 1/T3, 1/T1, T2 (reciprocals as Cantera's Troe rate keeps them)
            fo_troe.push_back(d->troe[4 * i + 0]);
            fo_troe.push_back(1.0 / d->troe[4 * i + 1]);
            fo_troe.push_back(1.0 / d->troe[4 * i + 2]);
            fo_troe.push_back(d->troe[4 * i + 3]);
        }
        rinfo[i] = ty | ((d->reversible[i] ? 1 : 0) << 2) | (nr << 3) | (np << 6) | (slot << 9);
        // per-species participation: (product count, reactant count)
        std::vector<std::pair<int, int>> cnt;
        auto bump = [&](int k, int add) {
            for (auto& c : cnt)
                if (c.first == k) {
                    c.second += add;
                    return;
                }
            cnt.push_back({k, add});
        };
        for (int o = 0; o < np; ++o) bump(pr[o], 1);
        for (int o = 0; o < nr; ++o) bump(rc[o], 16);
        for (auto& c : cnt) lists[c.first].push_back(i | ((c.second & 15) << 24) | ((c.second >> 4) << 28));
    }
    std::vector<int> sp_off(S + 1, 0), sp_ent;
    for (int k = 0; k < S; ++k) {
        sp_off[k + 1] = sp_off[k] + static_cast<int>(lists[k].size());
        sp_ent.insert(sp_ent.end(), lists[k].begin(), lists[k].end());
    }
    // Species by descending number of reactions, the thread order of the
    // per-species loops: the lanes of a warp then walk lists of similar length.
    std::vector<int> sp_order(S);
    for (int k = 0; k < S; ++k) sp_order[k] = k;
    std::stable_sort(sp_order.begin(), sp_order.end(),
                     [&](int a, int b) { return lists[a].size() > lists[b].size(); });
    const int n_tb = static_cast<int>(tb_rxn.size()), n_fo = static_cast<int>(fo_rxn.size());
    const int nT = 200;

    // ---- one device allocation for every table ----
    struct Piece {
        void** dst;
        const void* src;
        size_t bytes;
    };
    MechView v{};
    v.S = S;
    v.R = R;
    v.nT = nT;
    v.n_tb = n_tb;
    v.n_fo = n_fo;
    v.Tmin = 273.0;
    v.Tmax = 3500.0;
    std::vector<Piece> pieces = {
        {(void**)&v.W, d->mol_weight, sizeof(double) * S},
        {(void**)&v.rW, rW.data(), sizeof(double) * S},
        {(void**)&v.tmid, d->nasa_tmid, sizeof(double) * S},
        {(void**)&v.nasa, d->nasa_coeffs, sizeof(double) * S * 14},
        {(void**)&v.hc, hc.data(), sizeof(double) * S * 10},
        {(void**)&v.sc, sc.data(), sizeof(double) * S * 8},
        {(void**)&v.stoich, stoich.data(), sizeof(int4) * Rs},
        {(void**)&v.rinfo, rinfo.data(), sizeof(int) * Rs},
        {(void**)&v.arr, R ? d->arrhenius : nullptr, sizeof(double) * 3 * Rs},
        {(void**)&v.mult, mult.data(), sizeof(double) * Rs},
        {(void**)&v.dn, dn.data(), sizeof(double) * Rs},
        {(void**)&v.tb_rxn, tb_rxn.data(), sizeof(int) * std::max(n_tb, 1)},
        {(void**)&v.tb_off, tb_off.data(), sizeof(int) * (n_tb + 1)},
        {(void**)&v.tb_sp, tb_sp.data(), sizeof(int) * std::max<size_t>(tb_sp.size(), 1)},
        {(void**)&v.tb_eff, tb_eff.data(), sizeof(double) * std::max<size_t>(tb_eff.size(), 1)},
        {(void**)&v.tb_def, tb_def.data(), sizeof(double) * std::max(n_tb, 1)},
        {(void**)&v.fo_rxn, fo_rxn.data(), sizeof(int) * std::max(n_fo, 1)},
        {(void**)&v.fo_tb, fo_tb.data(), sizeof(int) * std::max(n_fo, 1)},
        {(void**)&v.fo_arr, fo_arr.data(), sizeof(double) * 3 * std::max(n_fo, 1)},
        {(void**)&v.fo_troe, fo_troe.data(), sizeof(double) * 4 * std::max(n_fo, 1)},
        {(void**)&v.tb_fo, tb_fo.data(), sizeof(int) * std::max(n_tb, 1)},
        {(void**)&v.sp_off, sp_off.data(), sizeof(int) * (S + 1)},
        {(void**)&v.sp_ent, sp_ent.data(), sizeof(int) * std::max<size_t>(sp_ent.size(), 1)},
        {(void**)&v.sp_order, sp_order.data(), sizeof(int) * S},
        {(void**)&v.kf_tab, nullptr, sizeof(double2) * size_t(nT) * Rs},
        {(void**)&v.kc_tab, nullptr, sizeof(double2) * size_t(nT) * Rs},
    };
    size_t bytes = 0;
    for (auto& pc : pieces) bytes += ((pc.bytes + 255) / 256) * 256;
    auto* mh = new ember_mech_s;
    mh->S = S;
    mh->R = R;
    cudaError_t e = cudaMalloc(&mh->blob, bytes);
    if (e != cudaSuccess) {
        delete mh;
        set_error("ember_mech_create: cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
        return EMBER_ENOMEM;
    }
    char* p = static_cast<char*>(mh->blob);
    for (auto& pc : pieces) {
        *pc.dst = p;
        if (e == cudaSuccess && pc.src && pc.bytes) {
            // sources shorter than the padded count (empty lists) copy what exists
            size_t nbytes = pc.bytes;
            if (pc.src == tb_rxn.data()) nbytes = sizeof(int) * n_tb;
            else if (pc.src == tb_sp.data()) nbytes = sizeof(int) * tb_sp.size();
            else if (pc.src == tb_eff.data()) nbytes = sizeof(double) * tb_eff.size();
            else if (pc.src == tb_def.data()) nbytes = sizeof(double) * n_tb;
            else if (pc.src == fo_rxn.data()) nbytes = sizeof(int) * n_fo;
            else if (pc.src == fo_tb.data()) nbytes = sizeof(int) * n_fo;
            else if (pc.src == fo_arr.data()) nbytes = sizeof(double) * fo_arr.size();
            else if (pc.src == fo_troe.data()) nbytes = sizeof(double) * fo_troe.size();
            else if (pc.src == tb_fo.data()) nbytes = sizeof(int) * tb_fo.size();
            else if (pc.src == sp_ent.data()) nbytes = sizeof(int) * sp_ent.size();
            else if (pc.src == d->arrhenius) nbytes = sizeof(double) * 3 * R;
            if (nbytes) e = cudaMemcpy(p, pc.src, nbytes, cudaMemcpyHostToDevice);
        }
        p += ((pc.bytes + 255) / 256) * 256;
    }
    if (e == cudaSuccess && R) {
        double* work = nullptr;
        e = cudaMalloc(&work, sizeof(double) * (ChemSmem::doubles(S, R, n_tb, n_fo, false) +
                                                 ChemSmem::global_doubles(R, n_fo)) * nT);
        if (e == cudaSuccess) {
            switch (chem_threads_for(S)) {
                case 64: k_build_tables<64><<<nT, 64>>>(v, work); break;
                case 128: k_build_tables<128><<<nT, 128>>>(v, work); break;
                case 160: k_build_tables<160><<<nT, 160>>>(v, work); break;
                default: k_build_tables<256><<<nT, 256>>>(v, work); break;
            }
            k_table_slopes<<<std::min<int64_t>((int64_t(nT) * R + 255) / 256, 4096), 256>>>(v);
            e = cudaDeviceSynchronize();
            cudaFree(work);
        }
    }
    if (e != cudaSuccess) {
        set_error("ember_mech_create: %s", cudaGetErrorString(e));
        cudaFree(mh->blob);
        delete mh;
        return EMBER_ECUDA;
    }
    mh->view = v;
    *out = mh;
    return EMBER_OK;
}

extern "C" int ember_mech_destroy(ember_mech m) {
    if (!m) return EMBER_OK;
    cudaFree(m->blob);
    delete m;
    return EMBER_OK;
}

extern "C" int ember_mech_set_multipliers(ember_mech m, const double* mult, int mem, void* stream) {
    EMBER_CHECK_ARG(m != nullptr, "null mechanism");
    EMBER_CHECK_ARG(mem == EMBER_MEM_HOST || mem == EMBER_MEM_DEVICE, "bad mem flag %d", mem);
    if (m->R == 0) return EMBER_OK;
    cudaStream_t st = as_stream(stream);
    double* dst = const_cast<double*>(m->view.mult);
    if (mult == nullptr) {
        std::vector<double> ones(m->R, 1.0);
        EMBER_CUDA_TRY(cudaMemcpyAsync(dst, ones.data(), sizeof(double) * m->R, cudaMemcpyHostToDevice, st));
        EMBER_CUDA_TRY(cudaStreamSynchronize(st));
        return EMBER_OK;
    }
    EMBER_CUDA_TRY(cudaMemcpyAsync(dst, mult, sizeof(double) * m->R,
                                   mem == EMBER_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, st));
    return finish_call(mem, st);
}

namespace ember {
const MechView* mech_view(ember_mech m) { return m ? &m->view : nullptr; }
}  // namespace ember

extern "C" int ember_gas_eval(ember_mech m, int n, double pressure, int model, int mode, const double* T,
                              const double* Y, double* creation, double* destruction, double* net, double* hk,
                              double* cp_mass, double* density, int mem, void* stream) {
    EMBER_CHECK_ARG(m != nullptr, "null mechanism");
    EMBER_CHECK_ARG(n >= 0 && T && Y, "bad points / null T or Y");
    EMBER_CHECK_ARG(model == EMBER_KINETICS_STANDARD || model == EMBER_KINETICS_INTERP, "bad kinetics model");
    EMBER_CHECK_ARG(mode == EMBER_STATE_NORMALIZED || mode == EMBER_STATE_NO_NORM, "bad state mode");
    EMBER_CHECK_ARG(mem == EMBER_MEM_HOST || mem == EMBER_MEM_DEVICE, "bad mem flag %d", mem);
    EMBER_CHECK_ARG(pressure > 0, "pressure must be positive");
    if (n == 0) return EMBER_OK;
    cudaStream_t st = as_stream(stream);
    Scratch sc(st);
    const int S = m->S;
    const double *dT, *dY;
    EMBER_TRY(stage_in(sc, T, n, mem, st, &dT));
    EMBER_TRY(stage_in(sc, Y, size_t(n) * S, mem, st, &dY));
    double *c1, *c2, *c3, *c4, *c5, *c6;
    EMBER_TRY(stage_buffer(sc, creation, size_t(n) * S, mem, &c1));
    EMBER_TRY(stage_buffer(sc, destruction, size_t(n) * S, mem, &c2));
    EMBER_TRY(stage_buffer(sc, net, size_t(n) * S, mem, &c3));
    EMBER_TRY(stage_buffer(sc, hk, size_t(n) * S, mem, &c4));
    EMBER_TRY(stage_buffer(sc, cp_mass, n, mem, &c5));
    EMBER_TRY(stage_buffer(sc, density, n, mem, &c6));
    const MechView& v = m->view;
    const int NTh = chem_threads_for(S);
    const size_t per = (ChemSmem::doubles(S, m->R, v.n_tb, v.n_fo, true) + S) * sizeof(double);
    EMBER_CHECK_ARG(per <= 227 * 1024, "mechanism too large for the shared-memory work area (%zu B)", per);
    int dev = 0, sms = 0;
    EMBER_CUDA_TRY(cudaGetDevice(&dev));
    EMBER_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = std::min(n, sms * 4);
    double* kcache = nullptr;
    EMBER_TRY(sc.alloc(&kcache, size_t(blocks) * ChemSmem::global_doubles(m->view)));
#define EMBER_GAS_EVAL(NTV)                                                                                  \
    EMBER_TRY(raise_dynamic_smem(reinterpret_cast<const void*>(k_gas_eval<NTV>), per)); \
    k_gas_eval<NTV><<<blocks, NTV, per, st>>>(v, n, pressure, model, mode, dT, dY, kcache, c1, c2, c3, c4, c5, c6)
    switch (NTh) {
        case 64: EMBER_GAS_EVAL(64); break;
        case 128: EMBER_GAS_EVAL(128); break;
        case 160: EMBER_GAS_EVAL(160); break;
        default: EMBER_GAS_EVAL(256); break;
    }
#undef EMBER_GAS_EVAL
    EMBER_TRY(stage_out(creation, c1, size_t(n) * S, mem, st));
    EMBER_TRY(stage_out(destruction, c2, size_t(n) * S, mem, st));
    EMBER_TRY(stage_out(net, c3, size_t(n) * S, mem, st));
    EMBER_TRY(stage_out(hk, c4, size_t(n) * S, mem, st));
    EMBER_TRY(stage_out(cp_mass, c5, n, mem, st));
    EMBER_TRY(stage_out(density, c6, n, mem, st));
    sc.release();
    return finish_call(mem, st);
}

namespace ember {

// CTAs of the capturable gas evaluation (one rate-constant cache slot each):
// the same count when the cache is sized and when the kernel is launched.
static int gas_eval_blocks(int n) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                   cudaSuccess)
        sms = 152;
    return std::max(1, std::min(n, sms * 4));
}

// Thermo and rates of n contiguous states (T [n], Y [n][S] on the device)
// into caller-provided buffers, with a caller-provided rate-constant cache of
// gas_eval_cache_doubles(m, n) doubles: no allocation, so it can be captured
// into a graph.
size_t gas_eval_cache_doubles(const MechView& v, int n) {
    return size_t(gas_eval_blocks(n)) * ChemSmem::global_doubles(v);
}

int launch_gas_eval(const MechView& v, int n, double pressure, int model, int mode, const double* T, const double* Y,
                    double* kcache, double* net, double* hk, double* cp_mass, cudaStream_t st) {
    if (n <= 0) return EMBER_OK;
    const int S = v.S;
    const int NTh = chem_threads_for(S);
    const size_t per = (ChemSmem::doubles(S, v.R, v.n_tb, v.n_fo, true) + S) * sizeof(double);
    EMBER_CHECK_ARG(per <= 227 * 1024, "mechanism too large for the shared-memory work area (%zu B)", per);
    const int blocks = gas_eval_blocks(n);
#define EMBER_GAS_EVAL(NTV)                                                                 \
    EMBER_TRY(raise_dynamic_smem(reinterpret_cast<const void*>(k_gas_eval<NTV>), per)); \
    k_gas_eval<NTV><<<blocks, NTV, per, st>>>(v, n, pressure, model, mode, T, Y, kcache, nullptr, nullptr, net, hk, \
                                              cp_mass, nullptr)
    switch (NTh) {
        case 64: EMBER_GAS_EVAL(64); break;
        case 128: EMBER_GAS_EVAL(128); break;
        case 160: EMBER_GAS_EVAL(160); break;
        default: EMBER_GAS_EVAL(256); break;
    }
#undef EMBER_GAS_EVAL
    EMBER_CUDA_TRY(cudaGetLastError());
    return EMBER_OK;
}

}  // namespace ember

extern "C" int ember_source_options_default(ember_source_options* o) {
    EMBER_CHECK_ARG(o != nullptr, "null options");
    *o = ember_source_options{};
    o->pressure = 101325.0;
    o->kinetics_model = EMBER_KINETICS_INTERP;
    o->max_steps = 1000000;
    o->qss_epsmin = 2e-2;
    o->qss_epsmax = 10.0;
    o->qss_dtmin = 1e-16;
    o->qss_dtmax = 1e-6;
    o->qss_abstol = 1e-11;
    o->qss_minval = 1e-60;
    o->qss_iteration_count = 1;
    o->qss_stability_check = 0;
    o->bdf_reltol = 1e-6;
    o->bdf_abstol_momentum = 1e-7;
    o->bdf_abstol_energy = 1e-8;
    o->bdf_abstol_species = 1e-13;
    o->bdf_min_step = 1e-18;
    o->bdf_max_num_steps = 1000000;
    o->ignition_duration = 1e-3;
    o->ignition_stddev = 1e-4;
    return EMBER_OK;
}

namespace ember {

int source_check_options(const ember_source_options* o) {
    EMBER_CHECK_ARG(o != nullptr, "null options");
    EMBER_CHECK_ARG(o->pressure > 0, "pressure must be positive");
    EMBER_CHECK_ARG(o->kinetics_model == EMBER_KINETICS_STANDARD || o->kinetics_model == EMBER_KINETICS_INTERP,
                    "bad kinetics model %d", o->kinetics_model);
    EMBER_CHECK_ARG(o->max_steps > 0, "max_steps must be positive");
    EMBER_CHECK_ARG(o->qss_epsmin > 0 && o->qss_epsmax > 0 && o->qss_dtmax > 0 && o->qss_iteration_count >= 0,
                    "bad QSS tolerances");
    EMBER_CHECK_ARG(o->bdf_reltol > 0 && o->bdf_abstol_momentum > 0 && o->bdf_abstol_energy > 0 &&
                        o->bdf_abstol_species > 0 && o->bdf_max_num_steps > 0,
                    "bad BDF tolerances");
    bool width_ok = o->threads_per_point == 0, tail_ok = o->qss_tail_threads == 0;
    for (int c : kQssThreadChoices) {
        width_ok = width_ok || o->threads_per_point == c;
        tail_ok = tail_ok || o->qss_tail_threads == c;
    }
    EMBER_CHECK_ARG(width_ok, "threads_per_point must be 0 or one of 32, 64, 96, 128, 160, 192, 256 (got %d)",
                    o->threads_per_point);
    EMBER_CHECK_ARG(tail_ok && o->qss_tail_steps >= -1, "bad QSS two-pass schedule (%d steps, %d threads)",
                    o->qss_tail_steps, o->qss_tail_threads);
    EMBER_CHECK_ARG(o->bdf_layout >= 0 && o->bdf_layout <= 4, "bdf_layout must be 0..4 (got %d)", o->bdf_layout);
    EMBER_CHECK_ARG(o->qss_tail_steps <= 0 || o->qss_stability_check == 0,
                    "the QSS two-pass schedule cannot be combined with the stability check");
    return EMBER_OK;
}

SourceArgs make_source_args(const ember_source_options* o, int n, const double* state_in, const double* split,
                            const double* dt, double t_start, const double* x, double* state_out, int* status,
                            int* stats) {
    SourceArgs a{};
    a.n = n;
    a.threads = o->threads_per_point;
    a.state_in = state_in;
    a.split = split;
    a.dt = dt;
    a.t_start = t_start;
    a.x = x;
    a.state_out = state_out;
    a.status = status;
    a.stats = stats;
    a.pressure = o->pressure;
    a.kinetics_model = o->kinetics_model;
    a.max_steps = o->max_steps;
    a.qss_epsmin = o->qss_epsmin;
    a.qss_epsmax = o->qss_epsmax;
    a.qss_dtmin = o->qss_dtmin;
    a.qss_dtmax = o->qss_dtmax;
    a.qss_abstol = o->qss_abstol;
    a.qss_minval = o->qss_minval;
    a.qss_itermax = o->qss_iteration_count;
    a.qss_stability_check = o->qss_stability_check;
    a.bdf_reltol = o->bdf_reltol;
    a.bdf_atol_u = o->bdf_abstol_momentum;
    a.bdf_atol_t = o->bdf_abstol_energy;
    a.bdf_atol_y = o->bdf_abstol_species;
    a.bdf_min_step = o->bdf_min_step;
    a.bdf_max_steps = o->bdf_max_num_steps;
    a.ign_tstart = o->ignition_tstart;
    a.ign_duration = o->ignition_duration;
    a.ign_energy = o->ignition_energy;
    a.ign_center = o->ignition_center;
    a.ign_stddev = o->ignition_stddev;
    a.tail_steps = o->qss_tail_steps;
    a.tail_threads = o->qss_tail_threads;
    // public placement code -> 1 + BdfLayout mode (bdf.cu)
    a.bdf_layout = o->bdf_layout == 1 ? 2 : o->bdf_layout == 2 ? 3 : o->bdf_layout == 3 ? 1 : o->bdf_layout == 4 ? 4 : 0;
    a.queue_chunk = 0;  // the mechanism's tuned granularity
    return a;
}

// Longest-first processing order of the points (see k_order_hist).
int make_work_order(const SourceArgs& a, Scratch& sc, cudaStream_t st, int** order_out) {
    int *counts = nullptr, *order = nullptr;
    EMBER_TRY(sc.alloc(&counts, 64));
    EMBER_TRY(sc.alloc(&order, a.n));
    EMBER_CUDA_TRY(cudaMemsetAsync(counts, 0, sizeof(int) * 64, st));
    const int blocks = std::min(blocks_for(a.n, 256), 1024);
    k_order_hist<<<blocks, 256, 0, st>>>(a.dt, a.n, counts);
    k_order_scan<<<1, 32, 0, st>>>(counts);
    k_order_scatter<<<blocks, 256, 0, st>>>(a.dt, a.n, counts, order);
    *order_out = order;
    return EMBER_OK;
}

// Dynamic shared memory and persistent grid size of the QSS kernel.
template <int NT>
static int qss_config(const MechView& m, const SourceArgs& a, size_t* per_out, int* blocks_out) {
    const size_t per = qss_smem_doubles(m, a.qss_stability_check != 0) * sizeof(double);
    EMBER_CHECK_ARG(per <= 227 * 1024, "mechanism too large for the QSS shared-memory work area (%zu B)", per);
    EMBER_TRY(raise_dynamic_smem(reinterpret_cast<const void*>(k_source_qss<NT>), per));
    EMBER_CUDA_TRY(cudaFuncSetAttribute(k_source_qss<NT>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                        int(cudaSharedmemCarveoutMaxShared)));
    int dev = 0, sms = 0, per_sm = 0;
    EMBER_CUDA_TRY(cudaGetDevice(&dev));
    EMBER_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    EMBER_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_source_qss<NT>, NT, per));
    per_sm = std::max(per_sm, 1);
    *per_out = per;
    *blocks_out = std::max(1, std::min(a.n, sms * per_sm));
    return EMBER_OK;
}

template <int NT>
static int qss_scratch_nt(const MechView& m, const SourceArgs& a, size_t* bytes) {
    size_t per = 0;
    int blocks = 0;
    EMBER_TRY(qss_config<NT>(m, a, &per, &blocks));
    *bytes = Scratch::rounded(sizeof(double) * size_t(blocks) * ChemSmem::global_doubles(m)) +
             Scratch::rounded(sizeof(int) * 64) + Scratch::rounded(sizeof(int) * size_t(a.n));
    return EMBER_OK;
}

// The two-pass schedule of a launch: the requested one (tail_steps < 0: one
// pass), else the mechanism's.
static void qss_tail_config(const MechView& m, const SourceArgs& a, int* steps, int* threads) {
    *steps = a.tail_steps ? a.tail_steps : m.qss_tail_steps;
    *threads = a.tail_steps ? a.tail_threads : m.qss_tail_threads;
    if (*threads == 0) *threads = 256;
    if (*steps < 0 || a.qss_stability_check) *steps = 0;
}

void source_qss_tail(const MechView& m, const SourceArgs& a, int* steps, int* threads) {
    qss_tail_config(m, a, steps, threads);
}

int source_qss_threads(const MechView& m, const SourceArgs& a) {
    if (a.threads) return a.threads;
    if (m.qss_threads) return m.qss_threads;
    return chem_threads_for(m.S);
}

static int qss_scratch_width(const MechView& m, const SourceArgs& a, int width, size_t* bytes) {
    switch (width) {
        case 32: return qss_scratch_nt<32>(m, a, bytes);
        case 64: return qss_scratch_nt<64>(m, a, bytes);
        case 96: return qss_scratch_nt<96>(m, a, bytes);
        case 128: return qss_scratch_nt<128>(m, a, bytes);
        case 160: return qss_scratch_nt<160>(m, a, bytes);
        case 192: return qss_scratch_nt<192>(m, a, bytes);
        default: return qss_scratch_nt<256>(m, a, bytes);
    }
}

int source_qss_scratch_bytes(const MechView& m, const SourceArgs& a, size_t* bytes) {
    EMBER_TRY(qss_scratch_width(m, a, source_qss_threads(m, a), bytes));
    int tail_steps = 0, tail_threads = 0;
    qss_tail_config(m, a, &tail_steps, &tail_threads);
    if (tail_steps) {
        size_t second = 0;
        EMBER_TRY(qss_scratch_width(m, a, tail_threads, &second));
        *bytes += second + Scratch::rounded(sizeof(QssResume) * size_t(a.n)) +
                  Scratch::rounded(sizeof(int) * size_t(a.n)) + Scratch::rounded(sizeof(int));
    }
    return EMBER_OK;
}

template <int NT>
static int launch_qss_nt(const MechView& m, const SourceArgs& a_in, int* counter, Scratch& sc, cudaStream_t st) {
    SourceArgs a = a_in;
    if (a.queue_chunk == 0) a.queue_chunk = m.qss_chunk > 0 ? m.qss_chunk : 1;
    size_t per = 0;
    int blocks = 0;
    EMBER_TRY(qss_config<NT>(m, a, &per, &blocks));
    double* kcache = nullptr;
    EMBER_TRY(sc.alloc(&kcache, size_t(blocks) * ChemSmem::global_doubles(m)));
    int* order = nullptr;
    EMBER_TRY(make_work_order(a, sc, st, &order));
    k_source_qss<NT><<<blocks, NT, per, st>>>(m, a, counter, order, kcache);
    EMBER_CUDA_TRY(cudaGetLastError());
    return EMBER_OK;
}

static int launch_qss_width(const MechView& m, const SourceArgs& a, int width, int* counter, Scratch& sc,
                            cudaStream_t st) {
    switch (width) {
        case 32: return launch_qss_nt<32>(m, a, counter, sc, st);
        case 64: return launch_qss_nt<64>(m, a, counter, sc, st);
        case 96: return launch_qss_nt<96>(m, a, counter, sc, st);
        case 128: return launch_qss_nt<128>(m, a, counter, sc, st);
        case 160: return launch_qss_nt<160>(m, a, counter, sc, st);
        case 192: return launch_qss_nt<192>(m, a, counter, sc, st);
        default: return launch_qss_nt<256>(m, a, counter, sc, st);
    }
}

static int cuda_check(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return EMBER_OK;
    set_error("%s failed: %s", what, cudaGetErrorString(e));
    return EMBER_ECUDA;
}

// One launch over all points, or the two-pass schedule: every point runs at
// the chosen width for at most tail_steps steps; the points still running are
// suspended (their state in state_out and a QssResume each) and continued,
// after the others, by a second launch at tail_threads threads per point. A
// point's steps and arithmetic are the same either way; only where and when
// they run changes. The suspended-point count stays on the device, so both
// passes can be captured in a graph.
int launch_source_qss(const MechView& m, const SourceArgs& a, int* counter, Scratch& sc, cudaStream_t st) {
    int tail_steps = 0, tail_threads = 0;
    qss_tail_config(m, a, &tail_steps, &tail_threads);
    if (tail_steps == 0) return launch_qss_width(m, a, source_qss_threads(m, a), counter, sc, st);
    SourceArgs a1 = a;
    a1.step_cap = tail_steps;
    EMBER_TRY(sc.alloc(&a1.resume, size_t(a.n)));
    EMBER_TRY(sc.alloc(&a1.susp_list, size_t(a.n)));
    EMBER_TRY(sc.alloc(&a1.susp_n, 1));
    EMBER_CUDA_TRY(cudaMemsetAsync(a1.susp_n, 0, sizeof(int), st));
    EMBER_TRY(launch_qss_width(m, a1, source_qss_threads(m, a), counter, sc, st));
    SourceArgs a2 = a1;
    a2.step_cap = 0;
    a2.resuming = 1;
    EMBER_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(int), st));
    return launch_qss_width(m, a2, tail_threads, counter, sc, st);
}

}  // namespace ember

extern "C" int ember_source_integrate(ember_mech m, int method, int n, const double* state_in,
                                      const double* split_const, const double* dt, double t_start, const double* x,
                                      const ember_source_options* opts, double* state_out, int* status, int* stats,
                                      int mem, void* stream) {
    EMBER_CHECK_ARG(m != nullptr, "null mechanism");
    EMBER_CHECK_ARG(method == EMBER_SOURCE_QSS || method == EMBER_SOURCE_BDF, "bad method %d", method);
    EMBER_CHECK_ARG(n >= 0, "n_points must be >= 0");
    EMBER_CHECK_ARG(n == 0 || (state_in && dt && state_out && status), "null state_in/dt/state_out/status");
    EMBER_CHECK_ARG(mem == EMBER_MEM_HOST || mem == EMBER_MEM_DEVICE, "bad mem flag %d", mem);
    EMBER_TRY(source_check_options(opts));
    if (n == 0) return EMBER_OK;
    EMBER_TRY(ensure_device());
    cudaStream_t st = as_stream(stream);
    Scratch sc(st);
    const int nv = m->S + 2;
    const double *d_in, *d_split, *d_dt, *d_x;
    EMBER_TRY(stage_in(sc, state_in, size_t(n) * nv, mem, st, &d_in));
    EMBER_TRY(stage_in(sc, split_const, size_t(n) * nv, mem, st, &d_split));
    EMBER_TRY(stage_in(sc, dt, n, mem, st, &d_dt));
    EMBER_TRY(stage_in(sc, x, n, mem, st, &d_x));
    double* d_out;
    int *d_status, *d_stats;
    EMBER_TRY(stage_buffer(sc, state_out, size_t(n) * nv, mem, &d_out));
    EMBER_TRY(stage_buffer(sc, status, n, mem, &d_status));
    EMBER_TRY(stage_buffer(sc, stats, size_t(n) * EMBER_STATS_WIDTH, mem, &d_stats));
    int* counter = nullptr;
    EMBER_TRY(sc.alloc(&counter, 1));
    EMBER_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(int), st));
    SourceArgs a = make_source_args(opts, n, d_in, d_split, d_dt, t_start, d_x, d_out, d_status, d_stats);
    if (method == EMBER_SOURCE_QSS) {
        EMBER_TRY(launch_source_qss(m->view, a, counter, sc, st));
    } else {
        EMBER_TRY(launch_source_bdf(m->view, a, counter, sc, st));
    }
    EMBER_TRY(stage_out(state_out, d_out, size_t(n) * nv, mem, st));
    EMBER_TRY(stage_out(status, d_status, n, mem, st));
    EMBER_TRY(stage_out(stats, d_stats, size_t(n) * EMBER_STATS_WIDTH, mem, st));
    sc.release();
    EMBER_TRY(finish_call(mem, st));
    if (mem == EMBER_MEM_HOST) {
        int bad = 0;
        for (int j = 0; j < n; ++j) bad += status[j] != 0;
        if (bad) {
            set_error("%d of %d points failed (see status)", bad, n);
            return EMBER_EFAIL;
        }
    }
    return EMBER_OK;
}

extern "C" int ember_source_autotune(ember_mech m, int method, int n, const double* state_in,
                                     const double* split_const, const double* dt, double t_start, const double* x,
                                     const ember_source_options* opts, int* threads_out, double* ms_out, int mem,
                                     void* stream) {
    EMBER_CHECK_ARG(m != nullptr, "null mechanism");
    EMBER_CHECK_ARG(method == EMBER_SOURCE_QSS || method == EMBER_SOURCE_BDF, "bad method %d", method);
    EMBER_CHECK_ARG(n > 0, "autotuning needs at least one point");
    EMBER_CHECK_ARG(state_in && dt && threads_out, "null state_in/dt/threads_out");
    EMBER_CHECK_ARG(mem == EMBER_MEM_HOST || mem == EMBER_MEM_DEVICE, "bad mem flag %d", mem);
    EMBER_TRY(source_check_options(opts));
    constexpr int kChoices = sizeof(kQssThreadChoices) / sizeof(kQssThreadChoices[0]);
    static_assert(kChoices == EMBER_SOURCE_N_THREAD_CHOICES, "thread choices out of step with the header");
    if (ms_out)
        for (int i = 0; i < kChoices; ++i) ms_out[i] = 0.0;
    EMBER_TRY(ensure_device());
    cudaStream_t st = as_stream(stream);
    Scratch sc(st);
    const int nv = m->S + 2;
    const double *d_in, *d_split, *d_dt, *d_x;
    EMBER_TRY(stage_in(sc, state_in, size_t(n) * nv, mem, st, &d_in));
    EMBER_TRY(stage_in(sc, split_const, size_t(n) * nv, mem, st, &d_split));
    EMBER_TRY(stage_in(sc, dt, n, mem, st, &d_dt));
    EMBER_TRY(stage_in(sc, x, n, mem, st, &d_x));
    double* d_out = nullptr;
    int *d_status = nullptr, *counter = nullptr;
    EMBER_TRY(sc.alloc(&d_out, size_t(n) * nv));
    EMBER_TRY(sc.alloc(&d_status, n));
    EMBER_TRY(sc.alloc(&counter, 1));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    EMBER_CUDA_TRY(cudaEventCreate(&e0));
    int rc = cuda_check(cudaEventCreate(&e1), "cudaEventCreate");
    int best = 0, best_layout = 0;
    float best_ms = 0.0f;
    // QSS: every width; BDF: every width of kBdfThreadChoices x every matrix layout that fits
    const bool bdf = method == EMBER_SOURCE_BDF;
    for (int i = 0; i < kChoices && rc == EMBER_OK; ++i) {
        const int width = kQssThreadChoices[i];
        bool valid = !bdf;
        for (int c : kBdfThreadChoices) valid = valid || width == c;
        if (!valid) continue;
        for (int layout = bdf ? 1 : 0; layout <= (bdf ? 4 : 0) && rc == EMBER_OK; ++layout) {
            if (bdf && !source_bdf_layout_fits(m->view, layout)) continue;
            ember_source_options o = *opts;
            o.threads_per_point = width;
            o.qss_tail_steps = -1;  // one pass while the widths are compared
            SourceArgs a = make_source_args(&o, n, d_in, d_split, d_dt, t_start, d_x, d_out, d_status, nullptr);
            a.bdf_layout = layout;
            float ms = 0.0f;
            for (int rep = 0; rep < 2 && rc == EMBER_OK; ++rep) {  // the first run is untimed
                Scratch work(st);  // the launch's work areas, freed after it on the stream
                rc = cuda_check(cudaMemsetAsync(counter, 0, sizeof(int), st), "cudaMemsetAsync");
                if (rc == EMBER_OK) rc = cuda_check(cudaEventRecord(e0, st), "cudaEventRecord");
                if (rc == EMBER_OK)
                    rc = bdf ? launch_source_bdf(m->view, a, counter, work, st)
                             : launch_source_qss(m->view, a, counter, work, st);
                if (rc == EMBER_OK) rc = cuda_check(cudaEventRecord(e1, st), "cudaEventRecord");
                if (rc == EMBER_OK) rc = cuda_check(cudaEventSynchronize(e1), "cudaEventSynchronize");
                if (rc == EMBER_OK) rc = cuda_check(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
            }
            if (rc != EMBER_OK) break;
            if (ms_out && (ms_out[i] == 0.0 || ms < ms_out[i])) ms_out[i] = ms;
            if (best == 0 || ms < best_ms) {
                best = width;
                best_layout = layout;
                best_ms = ms;
            }
        }
    }
    // QSS: two-pass schedules around the best width, the cap at the 50th / 75th /
    // 90th percentile of the points' step counts, the tail on 128 or 256 threads
    int best_tail = 0, best_tail_threads = 0;
    if (!bdf && rc == EMBER_OK && !opts->qss_stability_check) {
        int* d_stats = nullptr;
        rc = sc.alloc(&d_stats, size_t(n) * EMBER_STATS_WIDTH);
        ember_source_options o = *opts;
        o.threads_per_point = best;
        o.qss_tail_steps = -1;
        SourceArgs a = make_source_args(&o, n, d_in, d_split, d_dt, t_start, d_x, d_out, d_status, d_stats);
        if (rc == EMBER_OK) {
            Scratch work(st);
            rc = cuda_check(cudaMemsetAsync(counter, 0, sizeof(int), st), "cudaMemsetAsync");
            if (rc == EMBER_OK) rc = launch_source_qss(m->view, a, counter, work, st);
        }
        std::vector<int> stats(size_t(n) * EMBER_STATS_WIDTH);
        if (rc == EMBER_OK)
            rc = cuda_check(cudaMemcpyAsync(stats.data(), d_stats, sizeof(int) * stats.size(), cudaMemcpyDeviceToHost, st),
                            "cudaMemcpyAsync");
        if (rc == EMBER_OK) rc = cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
        std::vector<int> steps(n);
        for (int j = 0; j < n; ++j) steps[j] = stats[size_t(j) * EMBER_STATS_WIDTH];
        std::sort(steps.begin(), steps.end());
        for (double pct : {0.5, 0.75, 0.9}) {
            const int cap = std::max(1, steps[std::min(n - 1, int(pct * n))]);
            for (int tw : {128, 256}) {
                if (rc != EMBER_OK) break;
                ember_source_options ot = o;
                ot.qss_tail_steps = cap;
                ot.qss_tail_threads = tw;
                SourceArgs at = make_source_args(&ot, n, d_in, d_split, d_dt, t_start, d_x, d_out, d_status, nullptr);
                float ms = 0.0f;
                for (int rep = 0; rep < 2 && rc == EMBER_OK; ++rep) {
                    Scratch work(st);
                    rc = cuda_check(cudaMemsetAsync(counter, 0, sizeof(int), st), "cudaMemsetAsync");
                    if (rc == EMBER_OK) rc = cuda_check(cudaEventRecord(e0, st), "cudaEventRecord");
                    if (rc == EMBER_OK) rc = launch_source_qss(m->view, at, counter, work, st);
                    if (rc == EMBER_OK) rc = cuda_check(cudaEventRecord(e1, st), "cudaEventRecord");
                    if (rc == EMBER_OK) rc = cuda_check(cudaEventSynchronize(e1), "cudaEventSynchronize");
                    if (rc == EMBER_OK) rc = cuda_check(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
                }
                if (rc == EMBER_OK && ms < best_ms) {
                    best_ms = ms;
                    best_tail = cap;
                    best_tail_threads = tw;
                }
            }
        }
    }
    // QSS: queue granularity (slots claimed per atomic) with the best width and schedule
    int best_chunk = 1;
    for (int chunk : {2, 4}) {
        if (bdf || rc != EMBER_OK) break;
        ember_source_options o = *opts;
        o.threads_per_point = best;
        o.qss_tail_steps = best_tail ? best_tail : -1;
        o.qss_tail_threads = best_tail_threads;
        SourceArgs a = make_source_args(&o, n, d_in, d_split, d_dt, t_start, d_x, d_out, d_status, nullptr);
        a.queue_chunk = chunk;
        float ms = 0.0f;
        for (int rep = 0; rep < 2 && rc == EMBER_OK; ++rep) {
            Scratch work(st);
            rc = cuda_check(cudaMemsetAsync(counter, 0, sizeof(int), st), "cudaMemsetAsync");
            if (rc == EMBER_OK) rc = cuda_check(cudaEventRecord(e0, st), "cudaEventRecord");
            if (rc == EMBER_OK) rc = launch_source_qss(m->view, a, counter, work, st);
            if (rc == EMBER_OK) rc = cuda_check(cudaEventRecord(e1, st), "cudaEventRecord");
            if (rc == EMBER_OK) rc = cuda_check(cudaEventSynchronize(e1), "cudaEventSynchronize");
            if (rc == EMBER_OK) rc = cuda_check(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
        }
        if (rc == EMBER_OK && ms < best_ms) {
            best_ms = ms;
            best_chunk = chunk;
        }
    }
    cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    sc.release();
    EMBER_TRY(rc);
    EMBER_TRY(finish_call(EMBER_MEM_DEVICE, st));
    if (!bdf) {
        m->view.qss_tail_steps = best_tail;
        m->view.qss_tail_threads = best_tail_threads;
        m->view.qss_chunk = best_chunk;
    }
    if (bdf) {
        m->view.bdf_threads = best;
        m->view.bdf_layout = best_layout;
    } else {
        m->view.qss_threads = best;
    }
    *threads_out = best;
    return EMBER_OK;
}

extern "C" int ember_mech_get_tuning(ember_mech m, int* qss_threads, int* qss_tail_steps, int* qss_tail_threads,
                                     int* qss_chunk, int* bdf_threads, int* bdf_layout) {
    EMBER_CHECK_ARG(m != nullptr, "null mechanism");
    if (qss_threads) *qss_threads = m->view.qss_threads;
    if (qss_tail_steps) *qss_tail_steps = m->view.qss_tail_steps;
    if (qss_tail_threads) *qss_tail_threads = m->view.qss_tail_threads;
    if (qss_chunk) *qss_chunk = m->view.qss_chunk;
    if (bdf_threads) *bdf_threads = m->view.bdf_threads;
    if (bdf_layout) {
        // BdfLayout modes (bdf.cu): 0 global, 1 both in shared memory, 2 LU only, 3 LU and rates of
        // progress -> 3, 1, 2, 4
        const int l = m->view.bdf_layout;
        *bdf_layout = l == 0 ? 0 : (l == 1 ? 3 : (l == 2 ? 1 : (l == 3 ? 2 : 4)));
    }
    return EMBER_OK;
}

// ------------------------------------------- QSS known-answer self-test --

namespace ember {

// The CHEMEQ2 cesium relaxation problem of the reference's legacy QSS test
// (test/old/test_qssintegrator.cpp:11-83) as a q/d right-hand side.
struct CesiumOde {
    __device__ void eval(double, const double* y, double* q, double* d, bool) {
        if (threadIdx.x == 0) {
            const double o2m = y[0], csp = y[1], cs = y[2], cso2 = y[3], o2 = y[4], n2 = y[5];
            const double ne = (csp - o2m > 0.0) ? csp - o2m : 0.0;
            const double cr1 = 5.00e-08 * o2m * csp;
            const double cr2 = 1.00e-12 * csp * ne;
            const double cr3 = 3.24e-03 * cs;
            const double cr4 = 4.00e-01 * o2m;
            const double cr5 = 1.00e-31 * o2 * cs * (cs + cso2 + n2 + o2);
            const double cr6 = 1.24e-30 * o2 * o2 * ne;
            const double cr7 = 1.00e-31 * o2 * n2 * ne;
            for (int i = 0; i < 7; ++i) q[i] = d[i] = 0.0;
            q[0] = cr6 + cr7;
            d[0] = cr1 + cr4;
            q[1] = cr3;
            d[1] = cr1 + cr2;
            q[2] = cr1 + cr2;
            d[2] = cr3 + cr5;
            q[3] = cr5;
            q[4] = cr1 + cr4;
            d[4] = cr5 + cr6 + cr7;
        }
        __syncthreads();
    }
};

struct EnforceAll {
    __device__ bool operator()(int) const { return true; }
};

struct CesiumYmin {
    __device__ double operator()(int) const { return 1e-20; }
};

__global__ void __launch_bounds__(64) k_qss_cesium(QssParams P, double* y7, double tf, int* stats, int* ret) {
    __shared__ double buf[11 * 7];
    __shared__ double red[kMaxChemThreads + 2];
    QssSmem v;
    v.carve(buf, 7, P.stability_check != 0);
    for (int i = threadIdx.x; i < 7; i += 64) v.y[i] = y7[i];
    __syncthreads();
    CesiumOde ode;
    QssStats st;
    int r = qss_integrate_block<64>(ode, v, 7, P, EnforceAll(), CesiumYmin(), tf, 0.0, red, st);
    if (threadIdx.x == 0) {
        for (int i = 0; i < 7; ++i) y7[i] = v.y[i];
        y7[6] = y7[1] - y7[0];
        stats[0] = st.steps;
        stats[1] = st.gcount;
        stats[2] = st.rcount;
        stats[3] = 0;
        *ret = r;
    }
}

}  // namespace ember

extern "C" int ember_selftest_qss_cesium(double epsmin, double epsmax, double dtmin, double dtmax, double abstol,
                                         int itermax, int stability_check, double tf, int max_steps, double* y7,
                                         int* stats) {
    EMBER_CHECK_ARG(y7 != nullptr && stats != nullptr, "null argument");
    EMBER_CHECK_ARG(max_steps > 0 && itermax >= 0 && epsmin > 0, "bad parameters");
    EMBER_TRY(ensure_device());
    QssParams P{epsmin, epsmax, dtmin, dtmax, abstol, itermax, stability_check, max_steps};
    double* dy = nullptr;
    int* di = nullptr;
    EMBER_CUDA_TRY(cudaMalloc(&dy, sizeof(double) * 7));
    cudaError_t e = cudaMalloc(&di, sizeof(int) * 5);
    if (e == cudaSuccess) e = cudaMemcpy(dy, y7, sizeof(double) * 7, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_qss_cesium<<<1, 64>>>(P, dy, tf, di, di + 4);
        e = cudaGetLastError();
    }
    int ret = 0;
    if (e == cudaSuccess) e = cudaMemcpy(y7, dy, sizeof(double) * 7, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(stats, di, sizeof(int) * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&ret, di + 4, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(dy);
    cudaFree(di);
    if (e != cudaSuccess) {
        set_error("ember_selftest_qss_cesium: %s", cudaGetErrorString(e));
        return EMBER_ECUDA;
    }
    return ret;
}
