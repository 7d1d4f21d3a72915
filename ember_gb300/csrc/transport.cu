// Thermo and mixture-averaged transport properties of a batch of flame
// states: FlameSolver::updateChemicalProperties (src/flameSolver.cpp:652-699)
// with the "Approx" transport model (ApproxMixTransport,
// src/chemistry0d.cpp:12-269) and CanteraGas::getWeightedDiffusionCoefficientsMass
// (src/chemistry0d.cpp:583-591).
//
// One CTA per grid point (persistent grid). Per point:
//   thermo      NASA7 cp/R and h/RT per species (the expressions of the
//               kinetics' temperature pass), the setState_TPY normalisation,
//               density and cp_mass (the expressions of chem_rates, so the
//               values equal ember_gas_eval's bit for bit);
//   species     sqrt(mu_k) = T^(1/4) P, lambda_k = T^(1/2) P,
//               p D_jk = T^(3/2) P with P a quartic in ln T summed in the
//               order c0 + c1 x + c2 x^2 + c3 x^3 + c4 x^4 (Cantera's dot5);
//   mixture     X_k floored at 1e-20 (Cantera's MixTransport);
//               lambda = (sum X lambda + 1 / sum X / lambda) / 2;
//               mu = sum_k X_k mu_k / sum_j X_j phi_kj over the major species
//               (X >= threshold), phi from Wilke's rule with the reference's
//               triangle identity (updateViscosity_T, 181-205);
//               rho D_k = rho / (p sum_i X_i / D_ki + p X_k / (Wmx - W_k X_k)
//               sum_i X_i W_i / D_ki), the sums over every species i != k for
//               a major k, over the major ones otherwise (getMixDiffCoeffsMass,
//               98-139).
// Sums over species, and a major species' diffusion sums over its S - 1
// partners (one warp per species), run in the fixed 32-lane order of
// block_sum: term m on lane m mod 32, sequential per lane, then an xor
// butterfly; the other per-species sums run sequentially in species order.
// No automatic FMA contraction (--fmad=false): the CPU oracle repeats every
// operation.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "source.cuh"
#include "transport.cuh"

namespace ember {

__device__ __forceinline__ double fit5(const double* c, double x1, double x2, double x3, double x4) {
    double r = c[0];
    r = r + x1 * c[1];
    r = r + x2 * c[2];
    r = r + x3 * c[3];
    r = r + x4 * c[4];
    return r;
}

}  // namespace ember

namespace ember {
namespace {

// Wilke's phi_rc. The reference fills the lower triangle (r >= c) from the
// formula and the upper one from phi_rc = phi_cr mu_r W_c / (mu_c W_r).
__device__ __forceinline__ double wilke_phi(const TransportView& tv, const double* sq, const double* mu,
                                            const double* W, int r, int c) {
    if (r >= c) {
        const int64_t q = pair_index(tv.S, c, r);
        const double f1 = 1.0 + (sq[r] / sq[c]) * tv.w4[q];
        return (f1 * f1) / tv.s8w1[q];
    }
    const int64_t q = pair_index(tv.S, r, c);
    const double f1 = 1.0 + (sq[c] / sq[r]) * tv.w4[q];
    const double phi_cr = (f1 * f1) / tv.s8w1[q];
    return phi_cr / ((mu[c] / mu[r]) * (W[r] / W[c]));
}

template <int NT>
__global__ void __launch_bounds__(NT) k_transport(MechView m, TransportView tv, int n, double p, double thr,
                                                 const double* __restrict__ Tin, int64_t tstride,
                                                 const double* __restrict__ Yin, int64_t ystride,
                                                 ember_properties out) {
    extern __shared__ double sm[];
    const int S = m.S;
    const int t = threadIdx.x;
    double* y = sm;
    double* ym = y + S;
    double* cpR = ym + S;
    double* x = cpR + S;
    double* sq = x + S;
    double* mu = sq + S;
    double* lam = mu + S;
    double* sk = lam + S;
    double* red = sk + S;
    int* rows = reinterpret_cast<int*>(red + kRedDoubles);  // [S]: major species, then the others (ascending)
    __shared__ int s_nmaj;
    for (int j = blockIdx.x; j < n; j += gridDim.x) {
        const double T = Tin[j * tstride];
        for (int k = t; k < S; k += NT) y[k] = Yin[j * ystride + k];
        const double lnT = em_log(T), rT = 1.0 / T;
        const double RT = kGasConstant * T;
        const double sqT = sqrt(T), t14 = sqrt(sqT), t15 = T * sqT;
        const double l2 = lnT * lnT, l3 = l2 * lnT, l4 = l3 * lnT;
        for (int k = t; k < S; k += NT) {
            const int r = (T <= m.tmid[k]) ? 0 : 1;
            const double* a = m.nasa + 14 * k + 7 * r;
            const double* h = m.hc + 10 * k + 5 * r;
            const double cp = fma(fma(fma(fma(a[4], T, a[3]), T, a[2]), T, a[1]), T, a[0]);
            const double hr = fma(fma(fma(fma(h[4], T, h[3]), T, h[2]), T, h[1]), T, h[0]) + a[5] * rT;
            cpR[k] = cp;
            if (out.cp_species) out.cp_species[size_t(j) * S + k] = cp * kGasConstant;
            if (out.h_species) out.h_species[size_t(j) * S + k] = hr * RT;
            const double s = t14 * fit5(tv.visc + 5 * k, lnT, l2, l3, l4);
            sq[k] = s;
            mu[k] = s * s;
            lam[k] = sqT * fit5(tv.cond + 5 * k, lnT, l2, l3, l4);
        }
        // setState_TPY: clip and normalise (as chem_rates, STATE_NORMALIZED)
        const double rnorm = 1.0 / block_sum<NT>(red, S, [&](int k, double q) { return q + dmaxr(y[k], 0.0); });
        for (int k = t; k < S; k += NT) ym[k] = (dmaxr(y[k], 0.0) * rnorm) * m.rW[k];
        const double mmw = 1.0 / block_sum<NT>(red, S, [&](int k, double q) { return q + ym[k]; });
        const double rho = (p * mmw) / (kGasConstant * T);
        const double cpsum = block_sum<NT>(red, S, [&](int k, double q) { return fma(ym[k] * mmw, cpR[k], q); });
        for (int k = t; k < S; k += NT) x[k] = dmaxr(ym[k] * mmw, kMoleFractionFloor);
        const double s1 = block_sum<NT>(red, S, [&](int k, double q) { return q + x[k] * lam[k]; });
        const double s2 = block_sum<NT>(red, S, [&](int k, double q) { return q + x[k] / lam[k]; });
        // Lists of the major species and of the others, each in species order
        // (warp 0, ballot compaction), so that threads take rows of equal
        // cost: a major row has S - 1 partners, any other row the K majors.
        __syncthreads();
        if (t < 32) {
            const unsigned below = (1u << t) - 1u;
            int nm = 0;
            for (int b = 0; b < S; b += 32) {
                const bool f = b + t < S && x[b + t] >= thr;
                const unsigned bal = __ballot_sync(0xffffffffu, f);
                if (f) rows[nm + __popc(bal & below)] = b + t;
                nm += __popc(bal);
            }
            int no = nm;
            for (int b = 0; b < S; b += 32) {
                const bool f = b + t < S && !(x[b + t] >= thr);
                const unsigned bal = __ballot_sync(0xffffffffu, f);
                if (f) rows[no + __popc(bal & below)] = b + t;
                no += __popc(bal);
            }
            if (t == 0) s_nmaj = nm;
        }
        __syncthreads();
        const int K = s_nmaj;
        // Wilke denominators of the major species, one thread per species
        // (partners: the K majors, sequentially in species order)
        for (int r = t; r < K; r += NT) {
            const int k = rows[r];
            double s = 0.0;
            for (int ci = 0; ci < K; ++ci) {
                const int c = rows[ci];
                s = s + x[c] * wilke_phi(tv, sq, mu, m.W, k, c);
            }
            sk[k] = s;
        }
        const double vis = block_sum<NT>(red, S, [&](int k, double q) {
            return x[k] >= thr ? q + (x[k] * mu[k]) / sk[k] : q;
        });
        // rho D_k. A minor species sums over the K majors: one thread per
        // species, sequentially in species order. A major species sums over
        // all S - 1 others: one warp per species, partner m (in species
        // order) on lane m mod 32, the 32 partials combined by an xor
        // butterfly (the order of block_sum).
        if (out.rho_d) {
            auto finish = [&](int k, double a1, double a2) {
                a1 = a1 * p;
                a2 = a2 * ((p * x[k]) / (mmw - m.W[k] * x[k]));
                out.rho_d[size_t(j) * S + k] = (1.0 / (a1 + a2)) * rho;
            };
            auto pair_terms = [&](int k, int i, double& a1, double& a2) {
                const int64_t q = i < k ? pair_index(S, i, k) : pair_index(S, k, i);
                const double bd = t15 * fit5(tv.diff + 5 * q, lnT, l2, l3, l4);
                a1 = a1 + x[i] / bd;
                a2 = a2 + (x[i] * m.W[i]) / bd;
            };
            if (S == 1) {
                if (t == 0) out.rho_d[size_t(j)] = ((t15 * fit5(tv.diff, lnT, l2, l3, l4)) / p) * rho;
            } else {
                for (int r = K + t; r < S; r += NT) {
                    const int k = rows[r];
                    double a1 = 0.0, a2 = 0.0;
                    for (int ii = 0; ii < K; ++ii) pair_terms(k, rows[ii], a1, a2);
                    finish(k, a1, a2);
                }
                const int warp = t >> 5, lane = t & 31;
                for (int r = warp; r < K; r += NT / 32) {
                    const int k = rows[r];
                    double a1 = 0.0, a2 = 0.0;
                    for (int mi = lane; mi < S - 1; mi += 32) pair_terms(k, mi < k ? mi : mi + 1, a1, a2);
#pragma unroll
                    for (int off = 16; off >= 1; off >>= 1) {
                        a1 = a1 + __shfl_xor_sync(0xffffffffu, a1, off);
                        a2 = a2 + __shfl_xor_sync(0xffffffffu, a2, off);
                    }
                    if (lane == 0) finish(k, a1, a2);
                }
            }
        }
        if (t == 0) {
            if (out.density) out.density[j] = rho;
            if (out.mean_mol_weight) out.mean_mol_weight[j] = mmw;
            if (out.cp_mass) out.cp_mass[j] = (kGasConstant * cpsum) / mmw;
            if (out.conductivity) out.conductivity[j] = 0.5 * (s1 + 1.0 / s2);
            if (out.viscosity) out.viscosity[j] = vis;
        }
        __syncthreads();
    }
}

template <int NT>
int launch_transport_nt(const MechView& m, const TransportView& tv, int n, double p, double thr, const double* T,
                        int64_t tstride, const double* Y, int64_t ystride, const ember_properties& out,
                        cudaStream_t st) {
    const size_t smem = (size_t(8) * m.S + kRedDoubles) * sizeof(double) + sizeof(int) * m.S;
    EMBER_CHECK_ARG(smem <= 227 * 1024, "too many species for the transport work area");
    EMBER_TRY(raise_dynamic_smem(reinterpret_cast<const void*>(k_transport<NT>), smem));
    int dev = 0, sms = 0, per_sm = 0;
    EMBER_CUDA_TRY(cudaGetDevice(&dev));
    EMBER_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    EMBER_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_transport<NT>, NT, smem));
    const int blocks = std::max(1, std::min(n, sms * std::max(per_sm, 1)));
    k_transport<NT><<<blocks, NT, smem, st>>>(m, tv, n, p, thr, T, tstride, Y, ystride, out);
    EMBER_CUDA_TRY(cudaGetLastError());
    return EMBER_OK;
}

}  // namespace

int launch_transport(const MechView& m, const TransportView& tv, int n, double p, double thr, const double* T,
                     int64_t tstride, const double* Y, int64_t ystride, const ember_properties& out, cudaStream_t st) {
    switch (chem_threads_for(m.S)) {
        case 64: return launch_transport_nt<64>(m, tv, n, p, thr, T, tstride, Y, ystride, out, st);
        case 128: return launch_transport_nt<128>(m, tv, n, p, thr, T, tstride, Y, ystride, out, st);
        case 160: return launch_transport_nt<160>(m, tv, n, p, thr, T, tstride, Y, ystride, out, st);
        default: return launch_transport_nt<256>(m, tv, n, p, thr, T, tstride, Y, ystride, out, st);
    }
}

}  // namespace ember

using namespace ember;

extern "C" int ember_transport_create(ember_mech mech, const ember_transport_desc* d, ember_transport* out) {
    EMBER_CHECK_ARG(mech != nullptr && d != nullptr && out != nullptr, "null argument");
    EMBER_CHECK_ARG(d->n_species == mech->S, "n_species %d does not match the mechanism's %d", d->n_species, mech->S);
    EMBER_CHECK_ARG(d->visc_fit && d->cond_fit && d->diff_fit, "null fit array");
    const int S = mech->S;
    const int64_t P = int64_t(S) * (S + 1) / 2;
    std::vector<double> W(S);
    EMBER_TRY(ensure_device());
    EMBER_CUDA_TRY(cudaMemcpy(W.data(), mech->view.W, sizeof(double) * S, cudaMemcpyDeviceToHost));
    std::vector<double> w4(P), s8w1(P);
    for (int lo = 0; lo < S; ++lo)
        for (int hi = lo; hi < S; ++hi) {
            const int64_t q = pair_index(S, lo, hi);
            w4[q] = std::sqrt(std::sqrt(W[lo] / W[hi]));
            s8w1[q] = std::sqrt(8.0) * std::sqrt(1.0 + W[hi] / W[lo]);
        }
    const size_t b_fit = sizeof(double) * 5 * S, b_diff = sizeof(double) * 5 * P, b_pair = sizeof(double) * P;
    auto pad = [](size_t b) { return ((b + 255) / 256) * 256; };
    const size_t bytes = 2 * pad(b_fit) + pad(b_diff) + 2 * pad(b_pair);
    auto* h = new ember_transport_s;
    h->mech = mech;
    if (cudaMalloc(&h->blob, bytes) != cudaSuccess) {
        delete h;
        set_error("ember_transport_create: cudaMalloc(%zu) failed", bytes);
        return EMBER_ENOMEM;
    }
    char* p = static_cast<char*>(h->blob);
    struct Piece {
        const double** dst;
        const void* src;
        size_t bytes;
    } pieces[] = {{&h->view.visc, d->visc_fit, b_fit},  {&h->view.cond, d->cond_fit, b_fit},
                  {&h->view.diff, d->diff_fit, b_diff}, {&h->view.w4, w4.data(), b_pair},
                  {&h->view.s8w1, s8w1.data(), b_pair}};
    cudaError_t e = cudaSuccess;
    for (auto& pc : pieces) {
        *pc.dst = reinterpret_cast<const double*>(p);
        if (e == cudaSuccess) e = cudaMemcpy(p, pc.src, pc.bytes, cudaMemcpyHostToDevice);
        p += pad(pc.bytes);
    }
    if (e != cudaSuccess) {
        cudaFree(h->blob);
        delete h;
        set_error("ember_transport_create: upload failed: %s", cudaGetErrorString(e));
        return EMBER_ECUDA;
    }
    h->view.S = S;
    *out = h;
    return EMBER_OK;
}

extern "C" int ember_transport_destroy(ember_transport tr) {
    if (!tr) return EMBER_OK;
    cudaFree(tr->blob);
    delete tr;
    return EMBER_OK;
}

extern "C" int ember_transport_eval(ember_transport tr, int n, double pressure, double threshold, const double* T,
                                    const double* Y, const ember_properties* out, int mem, void* stream) {
    EMBER_CHECK_ARG(tr != nullptr && out != nullptr, "null transport or output");
    EMBER_CHECK_ARG(n >= 0, "n_points must be >= 0");
    EMBER_CHECK_ARG(n == 0 || (T && Y), "null T/Y");
    EMBER_CHECK_ARG(pressure > 0, "pressure must be positive");
    EMBER_CHECK_ARG(threshold >= 0 && threshold < 1, "threshold must be in [0, 1)");
    EMBER_CHECK_ARG(mem == EMBER_MEM_HOST || mem == EMBER_MEM_DEVICE, "bad mem flag %d", mem);
    if (n == 0) return EMBER_OK;
    EMBER_TRY(ensure_device());
    cudaStream_t st = as_stream(stream);
    Scratch sc(st);
    const int S = tr->view.S;
    const double *dT, *dY;
    EMBER_TRY(stage_in(sc, T, n, mem, st, &dT));
    EMBER_TRY(stage_in(sc, Y, size_t(n) * S, mem, st, &dY));
    ember_properties d{};
    EMBER_TRY(stage_buffer(sc, out->density, n, mem, &d.density));
    EMBER_TRY(stage_buffer(sc, out->mean_mol_weight, n, mem, &d.mean_mol_weight));
    EMBER_TRY(stage_buffer(sc, out->cp_mass, n, mem, &d.cp_mass));
    EMBER_TRY(stage_buffer(sc, out->cp_species, size_t(n) * S, mem, &d.cp_species));
    EMBER_TRY(stage_buffer(sc, out->h_species, size_t(n) * S, mem, &d.h_species));
    EMBER_TRY(stage_buffer(sc, out->conductivity, n, mem, &d.conductivity));
    EMBER_TRY(stage_buffer(sc, out->viscosity, n, mem, &d.viscosity));
    EMBER_TRY(stage_buffer(sc, out->rho_d, size_t(n) * S, mem, &d.rho_d));
    EMBER_TRY(launch_transport(tr->mech->view, tr->view, n, pressure, threshold, dT, 1, dY, S, d, st));
    EMBER_TRY(stage_out(out->density, d.density, n, mem, st));
    EMBER_TRY(stage_out(out->mean_mol_weight, d.mean_mol_weight, n, mem, st));
    EMBER_TRY(stage_out(out->cp_mass, d.cp_mass, n, mem, st));
    EMBER_TRY(stage_out(out->cp_species, d.cp_species, size_t(n) * S, mem, st));
    EMBER_TRY(stage_out(out->h_species, d.h_species, size_t(n) * S, mem, st));
    EMBER_TRY(stage_out(out->conductivity, d.conductivity, n, mem, st));
    EMBER_TRY(stage_out(out->viscosity, d.viscosity, n, mem, st));
    EMBER_TRY(stage_out(out->rho_d, d.rho_d, size_t(n) * S, mem, st));
    sc.release();
    return finish_call(mem, st);
}
