// Convection stage of the split step for a batch of flames:
// ConvectionSystemSplit::integrateToTime (src/convectionSystem.cpp:588-627).
//
//   k_conv_prepare   one CTA per flame: grid metrics, the initial mean
//                    molecular weight W from the mass fractions and the W
//                    split constant (src/convectionSystem.cpp:485-511, 572-586)
//   k_conv_utw       one CTA per flame: the UTW system
//                    (ConvectionSystemUTW::f, src/convectionSystem.cpp:14-130)
//                    integrated to the stage end with a stop time, V / rho
//                    recorded after every step (src/convectionSystem.cpp:592-611)
//   k_conv_species   one CTA per (flame, species): ConvectionSystemY::f
//                    (src/convectionSystem.cpp:307-359) with v(t) interpolated
//                    from that record (ConvectionSystemY::update_v, 372-398),
//                    integrated past the stage end and interpolated back
//
// Both integrations use the Adams method (variable order 1..12, Nordsieck
// form) with a diagonal difference-quotient Jacobian: the reference runs
// CVODE's Adams method with a zero-bandwidth banded Jacobian
// (src/convectionSystem.cpp:467-478, 663-676). A CTA owns one system (256
// threads for a UTW system, one warp for a species system, whose integrator
// control is scalar work every warp of a CTA would repeat); thread t of NT
// owns elements t, t + NT, ..., and every operation on the Nordsieck columns
// of an element is one pass; weighted norms are summed in NT slots (term i in
// slot i mod NT) folded in slot order. The continuity
// integral runs on one thread in point order over increments computed in
// parallel. The Nordsieck arrays and the per-system vectors live in a global
// work slice per system (40 vectors). Compiled with --fmad=false, the results
// are bitwise those of the CPU restatement.
#include <cstdint>
#include <type_traits>

#include "common.cuh"
#include "convection.cuh"
#include "emath.cuh"

namespace ember {
namespace {

constexpr int QA = 12;
constexpr int kWorkVectors = 2 * (QA + 2) + 12;
constexpr double kGasConstant = 6.02214076e26 * 1.380649e-23;

__device__ __forceinline__ double dmaxc(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ double dminc(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double cpow_(double x, double e) { return em_exp(e * em_log(x)); }

// Threads of a UTW system's CTA and of a species system's CTA: the control
// of an integrator is scalar work every warp of a CTA repeats, and a species
// system is short (its points), so it gets one warp.
constexpr int kNT = 256;
constexpr int kNTSpecies = 32;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v = v + __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// Norms are summed in NT slots, one per thread of the CTA: element i goes to
// slot i mod NT (each slot in increasing i), the slots are folded into 32 in
// slot order, then an xor butterfly. The CPU restatement sums in the same
// order with the same slot count.
constexpr int kRed = 2 * 256 + 2;  // shared doubles of the reductions (NT <= 256)

// Apply f(i, acc0, acc1) to every element of this thread and return both sums
// to every thread; red: kRed doubles of shared memory.
template <int NT, class F>
__device__ void slot_pass(int n, double* red, F&& f, double& s0, double& s1) {
    const int t = threadIdx.x;
    double a0 = 0.0, a1 = 0.0;
    for (int i = t; i < n; i += NT) f(i, a0, a1);
    __syncthreads();
    red[t] = a0;
    red[NT + t] = a1;
    __syncthreads();
    if (t < 32) {
        double v0 = red[t], v1 = red[NT + t];
        for (int w = 1; w < NT / 32; ++w) {
            v0 = v0 + red[t + 32 * w];
            v1 = v1 + red[NT + t + 32 * w];
        }
        v0 = warp_sum(v0);
        v1 = warp_sum(v1);
        if (t == 0) {
            red[2 * NT] = v0;
            red[2 * NT + 1] = v1;
        }
    }
    __syncthreads();
    s0 = red[2 * NT];
    s1 = red[2 * NT + 1];
}

template <int NT>
__device__ double block_max(double v, double* red) {
    const int t = threadIdx.x;
    __syncthreads();
    red[t] = v;
    __syncthreads();
    if (t < 32) {
        double m = red[t];
        for (int w = 1; w < NT / 32; ++w) m = dmaxc(m, red[t + 32 * w]);
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) m = dmaxc(m, __shfl_xor_sync(0xffffffffu, m, off));
        if (t == 0) red[2 * NT] = m;
    }
    __syncthreads();
    return red[2 * NT];
}

struct AdamsConst {
    double g[QA + 2];
    __device__ AdamsConst() {
        g[0] = 1.0;
        for (int j = 1; j <= QA + 1; ++j) {
            double s = 0.0;
            for (int i = 0; i < j; ++i) s = s + g[i] / (double)(j + 1 - i);
            g[j] = 1.0 - s;
        }
    }
};

__device__ void adams_l(int q, double* l) {
    double p[QA + 2];
    for (int j = 0; j <= QA + 1; ++j) {
        p[j] = 0.0;
        l[j] = 0.0;
    }
    p[0] = 1.0;
    for (int i = 1; i <= q - 1; ++i) {
        for (int j = i; j >= 1; --j) p[j] = p[j - 1] + (double)i * p[j];
        p[0] = (double)i * p[0];
    }
    double q0 = 0.0;
    for (int j = 0; j < q; ++j) {
        const double tj = p[j] / (double)(j + 1);
        q0 = (j % 2 == 0) ? q0 + tj : q0 - tj;
    }
    l[0] = 1.0;
    for (int j = 0; j < q; ++j) l[j + 1] = (p[j] / (double)(j + 1)) / q0;
}

// Block-uniform coefficients, in shared memory: the Adams constants g, the
// corrector's l for every order (row q) with its error constant, and the
// column factors scj of the last rescaling.
struct AdamsShared {
    double g[QA + 2], scj[QA + 2];
    double ltab[QA + 1][QA + 2], cqtab[QA + 1];
};

// scj[j] = eta^j as the running product eta, eta*eta, ... (scj[0] = 1);
// thread 0 writes once every thread is done with the previous factors,
// everyone reads after the second barrier
__device__ __forceinline__ void powers(double eta, int q, double* scj) {
    __syncthreads();
    if (threadIdx.x == 0) {
        scj[0] = 1.0;
        double sc = eta;
        for (int j = 1; j <= q; ++j) {
            scj[j] = sc;
            sc *= eta;
        }
    }
    __syncthreads();
}

// Call f with std::integral_constant<int, q> (1 <= q <= QA): the per-element
// loops over the Nordsieck columns are unrolled for the current order.
template <class F>
__device__ __forceinline__ void with_q(int q, F&& f) {
    switch (q) {
        case 1: f(std::integral_constant<int, 1>{}); break;
        case 2: f(std::integral_constant<int, 2>{}); break;
        case 3: f(std::integral_constant<int, 3>{}); break;
        case 4: f(std::integral_constant<int, 4>{}); break;
        case 5: f(std::integral_constant<int, 5>{}); break;
        case 6: f(std::integral_constant<int, 6>{}); break;
        case 7: f(std::integral_constant<int, 7>{}); break;
        case 8: f(std::integral_constant<int, 8>{}); break;
        case 9: f(std::integral_constant<int, 9>{}); break;
        case 10: f(std::integral_constant<int, 10>{}); break;
        case 11: f(std::integral_constant<int, 11>{}); break;
        default: f(std::integral_constant<int, 12>{}); break;
    }
}

// One CTA of NT threads integrates y' = f(t, y) from t0 to tf (tstop: the
// last step ends on tf; else past tf, then interpolated). `wk` holds
// kWorkVectors * n doubles. Per element, the same operations in the same
// order as the CPU restatement; the Nordsieck columns of an element are
// handled together in one pass.
template <int NT, class Sys>
__device__ int adams_block(Sys& s, double* wk, double* yio, double rtol, double t0, double tf, int tstop,
                           double hmin, int max_steps, int* stats, double* red, AdamsShared& sh) {
    const int n = s.n, tid = threadIdx.x;
    auto Z = [&](int j) { return wk + size_t(j) * n; };
    auto ZS = [&](int j) { return wk + size_t(QA + 2 + j) * n; };
    double* b0 = wk + size_t(2 * (QA + 2)) * n;
    double *acor = b0, *acorp = b0 + n, *ewt = b0 + 2 * size_t(n), *y = b0 + 3 * size_t(n);
    double *ft = b0 + 4 * size_t(n), *bb = b0 + 5 * size_t(n);
    double *f0 = b0 + 7 * size_t(n), *ycopy = b0 + 8 * size_t(n), *f1 = b0 + 9 * size_t(n);
    double *jd = b0 + 10 * size_t(n), *md = b0 + 11 * size_t(n);
    const double uround = 2.220446049250313e-16;
    if (tid == 0) {
        const AdamsConst C;
        for (int j = 0; j <= QA + 1; ++j) sh.g[j] = C.g[j];
        for (int q = 1; q <= QA; ++q) {
            adams_l(q, sh.ltab[q]);
            sh.cqtab[q] = fabs(C.g[q] - C.g[q - 1]) / C.g[q - 1];
        }
    }
    __syncthreads();
    const double* g = sh.g;
    double* scj = sh.scj;
    const double* l = sh.ltab[1];
    int nst = 0, nfe = 0, nje = 0, nfail = 0, status = 0;
#define VLOOP for (int i = tid; i < n; i += NT)
    // restore from the saved columns (restore != 0), rescale column j by
    // scj[j] (rescale != 0), save into the saved columns (save != 0)
    auto cols = [&](int q, bool restore, bool rescale, bool save) {
        with_q(q, [&](auto qc) {
            constexpr int Q = decltype(qc)::value;
            VLOOP {
#pragma unroll
                for (int j = 0; j <= Q; ++j) {
                    double v = restore ? ZS(j)[i] : Z(j)[i];
                    if (rescale && j >= 1) v *= scj[j];
                    if (restore || rescale) Z(j)[i] = v;
                    if (save) ZS(j)[i] = v;
                }
            }
        });
    };
    double sa, sb;

    VLOOP Z(0)[i] = yio[i];
    s.f(t0, Z(0), f0);
    nfe++;
    double rmax = 0.0;
    VLOOP {
        ewt[i] = 1.0 / (rtol * fabs(Z(0)[i]) + s.atol(i));
        rmax = dmaxc(rmax, fabs(f0[i]) / (0.1 * fabs(Z(0)[i]) + s.atol(i)));
    }
    rmax = block_max<NT>(rmax, red);
    double t = t0;
    const double tdist = tf - t0;
    double hub = 0.1 * tdist;
    if (rmax * hub > 1.0) hub = 1.0 / rmax;
    const double hlb = 100.0 * uround * dmaxc(fabs(t0), fabs(tf));
    double hg = sqrt(hlb * hub);
    double h;
    if (hub > hlb) {
        for (int it = 0; it < 4; ++it) {
            VLOOP ycopy[i] = fma(hg, f0[i], Z(0)[i]);
            s.f(t0 + hg, ycopy, f1);
            nfe++;
            slot_pass<NT>(n, red, [&](int i, double& p, double&) {
                const double tv = ((f1[i] - f0[i]) / hg) * ewt[i];
                p = fma(tv, tv, p);
            }, sa, sb);
            const double ydd = sqrt(sa / n);
            const double hnew = (ydd * hub * hub > 2.0) ? sqrt(2.0 / ydd) : sqrt(hg * hub);
            const double ratio = hnew / hg;
            hg = hnew;
            if (ratio > 0.5 && ratio < 2.0) break;
        }
        h = dminc(dmaxc(0.5 * hg, hlb), hub);
    } else {
        h = hlb;
    }
    if (h < hmin) h = hmin;
    VLOOP Z(1)[i] = h * f0[i];

    int q = 1, qwait = 2, nstlp = 0, nstlj = 0, have_m = 0, have_acorp = 0, qsave = 0;
    double gammap = 0.0, crate = 1.0, etamax = 10000.0, acnrm = 0.0, hsave = 0.0;

    while (t < tf) {
        if (nst >= max_steps) {
            status = -11;
            break;
        }
        if (tstop && t + h > tf) {
            powers((tf - t) / h, q, scj);
            cols(q, false, true, true);
            h = tf - t;
        } else {
            cols(q, false, false, true);
        }
        int ncf = 0, nef = 0, convfail_bad_j = 0, force_setup = !have_m;
        double dsm = 0.0;
        for (;;) {
            // predict (Pascal triangle on each element's columns)
            with_q(q, [&](auto qc) {
                constexpr int Q = decltype(qc)::value;
                VLOOP {
                    double v[Q + 1];
#pragma unroll
                    for (int j = 0; j <= Q; ++j) v[j] = Z(j)[i];
#pragma unroll
                    for (int k = 1; k <= Q; ++k)
#pragma unroll
                        for (int j = Q; j >= k; --j) v[j - 1] += v[j];
#pragma unroll
                    for (int j = 0; j <= Q; ++j) Z(j)[i] = v[j];
                }
            });
            const double tn = t + h;
            l = sh.ltab[q];
            const double cq = sh.cqtab[q];
            const double gamma = h / l[1];
            const double tq4 = 0.1 / cq;
            int jcur = 0;
            const double gamrat0 = have_m ? gamma / gammap : 1.0;
            bool fail_conv = false;
            if (force_setup || nst >= nstlp + 20 || fabs(gamrat0 - 1.0) > 0.3) {
                const int jbad = (nst == 0) || (nst >= nstlj + 51) || convfail_bad_j || !have_m;
                int sing = 0;
                if (jbad) {
                    s.f(tn, Z(0), ft);
                    nfe++;
                    slot_pass<NT>(n, red, [&](int i, double& p, double&) {
                        const double tv = ft[i] * ewt[i];
                        p = fma(tv, tv, p);
                    }, sa, sb);
                    const double fnorm = sqrt(sa / n);
                    const double srur = sqrt(uround);
                    const double min_inc = (fnorm != 0.0) ? (1000.0 * fabs(h) * uround * n * fnorm) : 1.0;
                    VLOOP {
                        const double inc = dmaxc(srur * fabs(Z(0)[i]), min_inc / ewt[i]);
                        bb[i] = inc;
                        ycopy[i] = Z(0)[i] + inc;
                    }
                    s.f(tn, ycopy, f1);
                    nfe++;
                    VLOOP {
                        jd[i] = (f1[i] - ft[i]) / bb[i];
                        md[i] = 1.0 - gamma * jd[i];
                        if (md[i] == 0.0) sing = 1;
                    }
                    nje++;
                    nstlj = nst;
                    jcur = 1;
                } else {
                    VLOOP {
                        md[i] = 1.0 - gamma * jd[i];
                        if (md[i] == 0.0) sing = 1;
                    }
                }
                sing = __syncthreads_or(sing);
                gammap = gamma;
                nstlp = nst;
                crate = 1.0;
                have_m = !sing;
                force_setup = 0;
                convfail_bad_j = 0;
                if (sing) fail_conv = true;
            }
            if (!fail_conv) {
                const double gamrat = gamma / gammap;
                VLOOP {
                    acor[i] = 0.0;
                    y[i] = Z(0)[i];
                }
                double delp = 0.0, del = 0.0;
                int converged = 0;
                const double rl1 = 1.0 / l[1];
                const double scg = 2.0 / (1.0 + gamrat);
                for (int mit = 0; mit < 3; ++mit) {
                    s.f(tn, y, ft);
                    nfe++;
                    slot_pass<NT>(n, red, [&](int i, double& p0, double& p1) {
                        double b = (gamma * ft[i] - fma(rl1, Z(1)[i], acor[i])) / md[i];
                        if (gamrat != 1.0) b *= scg;
                        const double tv = b * ewt[i];
                        p0 = fma(tv, tv, p0);
                        const double a = acor[i] + b;
                        acor[i] = a;
                        y[i] = Z(0)[i] + a;
                        const double ta = a * ewt[i];
                        p1 = fma(ta, ta, p1);
                    }, sa, sb);
                    del = sqrt(sa / n);
                    if (mit > 0) crate = dmaxc(0.3 * crate, del / delp);
                    const double dcon = del * dminc(1.0, crate) / tq4;
                    if (dcon <= 1.0) {
                        acnrm = (mit == 0) ? del : sqrt(sb / n);
                        converged = 1;
                        break;
                    }
                    if (mit >= 1 && del > 2.0 * delp) break;
                    delp = del;
                }
                if (!converged) fail_conv = true;
            }
            if (!fail_conv) {
                dsm = acnrm * cq;
                if (dsm <= 1.0) break;
                nef++;
                nfail++;
                if (nef >= 7 || h <= hmin * 1.0000000000000002) {
                    cols(q, true, false, false);
                    status = -13;
                    goto done;
                }
                if (nef <= 3) {
                    double eta = 1.0 / (cpow_(6.0 * dsm, 1.0 / (q + 1)) + 1e-6);
                    eta = dmaxc(0.1, dmaxc(eta, hmin / h));
                    if (nef >= 2) eta = dminc(eta, 0.2);
                    powers(eta, q, scj);
                    cols(q, true, true, true);
                    h *= eta;
                } else {
                    cols(q, true, false, false);
                    const double eta = dmaxc(0.1, hmin / h);
                    h *= eta;
                    q = 1;
                    s.f(t, Z(0), ft);
                    nfe++;
                    VLOOP Z(1)[i] = h * ft[i];
                    cols(q, false, false, true);
                }
                qwait = q + 1;
                have_acorp = 0;
                etamax = 1.0;
                continue;
            }
            // convergence failure
            nfail++;
            if (!jcur && have_m) {
                cols(q, true, false, false);
                force_setup = 1;
                convfail_bad_j = 1;
                continue;
            }
            ncf++;
            if (ncf >= 10 || h <= hmin * 1.0000000000000002) {
                cols(q, true, false, false);
                status = -14;
                goto done;
            }
            {
                const double eta = dmaxc(0.25, hmin / h);
                powers(eta, q, scj);
                cols(q, true, true, true);
                h *= eta;
                qwait = q + 1;
                have_acorp = 0;
                etamax = 1.0;
                force_setup = 1;
            }
        }
        // accepted step: Nordsieck update, weights, the correction saved for the order test
        nst++;
        {
            const double tnew = t + h;
            t = (tstop && (tnew >= tf || tf - tnew <= 100.0 * uround * (fabs(tnew) + fabs(h)))) ? tf : tnew;
        }
        const bool save_acorp = (qwait - 1 == 1) && q < QA;
        with_q(q, [&](auto qc) {
            constexpr int Q = decltype(qc)::value;
            double lr[Q + 1];
#pragma unroll
            for (int j = 0; j <= Q; ++j) lr[j] = l[j];
            VLOOP {
                const double a = acor[i];
#pragma unroll
                for (int j = 0; j <= Q; ++j) Z(j)[i] = fma(lr[j], a, Z(j)[i]);
                ewt[i] = 1.0 / (rtol * fabs(Z(0)[i]) + s.atol(i));
                if (save_acorp) acorp[i] = a;
            }
        });
        s.on_step(t);
        {
            const double etaq = 1.0 / (cpow_(6.0 * dsm, 1.0 / (q + 1)) + 1e-6);
            double eta = etaq;
            int qnew = q;
            qwait--;
            if (qwait == 0) {
                double etaqm1 = 0.0, etaqp1 = 0.0;
                const bool lower = q > 1, upper = q < QA && have_acorp && qsave == q;
                const double cc = upper ? cpow_(h / hsave, (double)(q + 1)) : 0.0;
                if (lower || upper) {
                    const double* zq = Z(q);
                    slot_pass<NT>(n, red, [&](int i, double& p0, double& p1) {
                        const double e = ewt[i];
                        if (lower) {
                            const double tv = zq[i] * e;
                            p0 = fma(tv, tv, p0);
                        }
                        if (upper) {
                            const double tv = fma(-cc, acorp[i], acor[i]) * e;
                            p1 = fma(tv, tv, p1);
                        }
                    }, sa, sb);
                }
                if (lower) {
                    double fact = 1.0;
                    for (int i = 2; i <= q; ++i) fact *= i;
                    const double ddn = sqrt(sa / n) * (fabs(g[q - 1] - g[q - 2]) * fact);
                    etaqm1 = 1.0 / (cpow_(6.0 * ddn, 1.0 / q) + 1e-6);
                }
                if (upper) {
                    const double dup = sqrt(sb / n) * (fabs(g[q + 1] - g[q]) / g[q - 1]);
                    etaqp1 = 1.0 / (cpow_(10.0 * dup, 1.0 / (q + 2)) + 1e-6);
                }
                if (etaq >= etaqm1 && etaq >= etaqp1) {
                    eta = etaq;
                } else if (etaqm1 >= etaqp1) {
                    eta = etaqm1;
                    qnew = q - 1;
                } else {
                    eta = etaqp1;
                    qnew = q + 1;
                }
                qwait = 2;
            } else if (qwait == 1 && q < QA) {
                hsave = h;
                qsave = q;
                have_acorp = 1;
            }
            if (etamax <= 1.0) {
                eta = 1.0;
                qnew = q;
            } else if (eta < 1.5 && qnew == q) {
                eta = 1.0;
            } else {
                eta = dminc(eta, etamax);
                if (h * eta < hmin) eta = hmin / h;
            }
            const bool grow = qnew > q;
            double cnew = 0.0;
            if (grow) {
                double fact = 1.0;
                for (int i = 2; i <= q + 1; ++i) fact *= i;
                cnew = -1.0 / (g[q - 1] * fact);
            }
            const int qold = q;
            if (qnew != q) {
                q = qnew;
                qwait = q + 1;
                have_acorp = 0;
            }
            if (grow || eta != 1.0) {
                powers(eta, q, scj);
                const bool resc = eta != 1.0;
                if (grow) {
                    double* zn = Z(qold + 1);
                    VLOOP zn[i] = acor[i] * cnew;
                }
                if (resc) {
                    with_q(q, [&](auto qc) {
                        constexpr int Q = decltype(qc)::value;
                        double sr[Q + 1];
#pragma unroll
                        for (int j = 1; j <= Q; ++j) sr[j] = scj[j];
                        VLOOP {
#pragma unroll
                            for (int j = 1; j <= Q; ++j) Z(j)[i] *= sr[j];
                        }
                    });
                }
                if (resc) h *= eta;
            }
            etamax = 10.0;
        }
    }
    {
        const double sv = (tf - t) / h;
        VLOOP {
            double v = Z(q)[i];
            for (int j = q - 1; j >= 0; --j) v = fma(v, sv, Z(j)[i]);
            yio[i] = v;
        }
    }
done:
    if (status != 0) {
        VLOOP yio[i] = Z(0)[i];
    }
    __syncthreads();
    if (stats) {
        stats[0] = nst;
        stats[1] = nfe;
        stats[2] = nfail;
        stats[3] = nje;
    }
    return status;
#undef VLOOP
}

constexpr int kStatusBadSlice = -30;

__device__ __forceinline__ void stage_times(const ConvArgs& a, double& t0, double& tf) {
    if (a.t_dev) {
        const double t = *a.t_dev;
        t0 = (a.f0 == 0.0) ? t : t + a.f0 * a.dt;
        tf = t + a.f1 * a.dt;
    } else {
        t0 = a.t0;
        tf = a.tf;
    }
}  // a work slice outside its allocation: nothing was touched

__device__ __forceinline__ double center_volume(const double* x, int alpha) {
    return alpha == 0 ? x[1] : (x[1] * x[1]) / 2.0;
}

// per-flame scratch inside the UTW slice, after the work vectors
struct UtwView {
    double *y3, *hh, *rph, *Wm, *sW, *rho, *rV, *V;
};
constexpr int kUtwScratch = 10;  // doubles per point after the work vectors

__device__ UtwView utw_view(const ConvArgs& a, const ConvFlame& F) {
    const int N = F.f.n_points;
    double* base = a.wk_utw + F.utw_wk + size_t(kWorkVectors) * 3 * N;
    UtwView v;
    v.y3 = base;
    v.hh = base + 3 * size_t(N);
    v.rph = v.hh + N;
    v.Wm = v.rph + N;
    v.sW = v.Wm + N;
    v.rho = v.sW + N;
    v.rV = v.rho + N;
    v.V = v.rV + N;
    return v;
}

__device__ __forceinline__ bool utw_slice_ok(const ConvArgs& a, const ConvFlame& F) {
    const int64_t N = F.f.n_points;
    return F.utw_wk >= 0 && F.utw_wk + (int64_t(kWorkVectors) * 3 + kUtwScratch) * N <= a.wk_utw_n &&
           F.hist >= 0 && F.hist + a.max_history <= a.hist_n && F.histv >= 0 &&
           F.histv + int64_t(a.max_history) * N <= a.histv_n;
}

__global__ void k_conv_prepare(const __grid_constant__ ConvArgs a) {
    const ConvFlame& F = a.flames[blockIdx.x];
    const int N = F.f.n_points, S = a.S;
    if (!utw_slice_ok(a, F)) return;
    const double* x = a.x + F.p0;
    const double* st = a.state + F.v0;
    const double* sc = a.split + F.v0;
    UtwView u = utw_view(a, F);
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
        // rph[N-1]: the radius factor at the last point, for the continuity
        // conditions that read one half point past the grid
        if (j < N - 1) {
            u.hh[j] = x[j + 1] - x[j];
            const double xm = 0.5 * (x[j] + x[j + 1]);
            u.rph[j] = F.f.alpha == 0 ? 1.0 : xm;
        } else {
            u.hh[j] = 0.0;
            u.rph[j] = F.f.alpha == 0 ? 1.0 : x[j];
        }
        double ysum = 0.0;
        for (int k = 0; k < S; ++k) ysum = ysum + dmaxc(st[size_t(2 + k) * N + j], 0.0);
        const double rnorm = 1.0 / ysum;
        double acc = 0.0;
        for (int k = 0; k < S; ++k) acc = acc + (dmaxc(st[size_t(2 + k) * N + j], 0.0) * rnorm) / a.W[k];
        const double wm = 1.0 / acc;
        u.Wm[j] = wm;
        double sw = 0.0;
        for (int k = 0; k < S; ++k) sw = sw + sc[size_t(2 + k) * N + j] / a.W[k];
        u.sW[j] = sw;
        u.y3[3 * j + 0] = st[j];
        u.y3[3 * j + 1] = st[size_t(N) + j];
        u.y3[3 * j + 2] = wm;
    }
}


// a(t) and da/dt of a flame's strain function: LinearFunction
// (src/scalarFunction.cpp:12-22) or ChebyshevFunction (:31-87), with the
// reference's padding (fewer than two coefficients count as zeros) and its
// derivative recurrence, which weights coefficient i by i U_i(x) (the loop
// advances the U recurrence before using it; T'_i = i U_{i-1}).
__device__ __forceinline__ void conv_strain(const ember_convection_flame& fl, double t, double& a, double& dadt) {
    if (fl.strain_type == EMBER_STRAIN_CHEBYSHEV) {
        const int n = fl.n_cheb < 2 ? 2 : fl.n_cheb;
        auto c = [&](int i) { return i < fl.n_cheb ? fl.cheb[i] : 0.0; };
        const double x = (2 * (t - fl.cheb_t0)) / (fl.cheb_t1 - fl.cheb_t0) - 1;
        double cm = 1, cn = x;
        double y = c(0) + x * c(1);
        for (int i = 2; i < n; ++i) {
            const double cp = (2 * x) * cn - cm;
            y += cp * c(i);
            cm = cn;
            cn = cp;
        }
        a = y;
        cm = 1;
        cn = 2 * x;
        double dydx = c(1);
        for (int i = 2; i < n; ++i) {
            const double cp = (2 * x) * cn - cm;
            dydx += (static_cast<double>(i) * cp) * c(i);
            cm = cn;
            cn = cp;
        }
        dadt = dydx * (2.0 / (fl.cheb_t1 - fl.cheb_t0));
        return;
    }
    const double a0 = fl.strain_initial, a1 = fl.strain_final, T0 = fl.strain_t0, Dt = fl.strain_dt;
    a = (t <= T0) ? a0 : (t >= T0 + Dt) ? a1 : a0 + ((a1 - a0) * (t - T0)) / Dt;
    dadt = (t >= T0 && t < T0 + Dt) ? (a1 - a0) / Dt : 0.0;
}

struct UtwSys {
    int n;
    const ConvArgs* a;
    const ember_convection_flame* fl;
    const double *x, *drhodt, *sU, *sT;
    UtwView u;
    double *sm_m, *sm_mb, *sm_rV;  // shared memory, N each: the increments and rV
    double* ht;
    double* hv;
    int n_history, overflow, max_history;

    __device__ double atol(int i) const {
        const int c = i % 3;
        return c == 0 ? a->abstol_u : (c == 1 ? a->abstol_t : 20.0 * a->abstol_y);
    }

    // ConvectionSystemUTW::f: the per-point increments of the continuity
    // integral in parallel, the integral itself on thread 0 in point order,
    // then V and the derivatives in parallel.
    __device__ void f(double t, const double* y, double* ydot) {
        const int N = fl->n_points, jj = N - 1, jc = fl->j_cont, tid = threadIdx.x;
        const double beta = fl->beta;
        const double *hh = u.hh, *rph = u.rph, *sW = u.sW;
        double *rho = u.rho, *V = u.V, *m = sm_m, *mb = sm_mb, *rV = sm_rV;
        const bool backward_own = fl->continuity_bc == EMBER_CONTINUITY_RIGHT ||
                                  fl->continuity_bc == EMBER_CONTINUITY_QDOT ||
                                  fl->continuity_bc == EMBER_CONTINUITY_TEMP;
        __syncthreads();
        for (int j = tid; j < N; j += kNT) {
            const double r = (fl->pressure * y[3 * j + 2]) / (kGasConstant * y[3 * j + 1]);
            rho[j] = r;
            const double flux = drhodt[j] + (r * beta) * y[3 * j + 0];
            if (j < N - 1) m[j] = (hh[j] * rph[j]) * flux;
            if (backward_own && j >= 1) mb[j] = (hh[j - 1] * rph[j]) * flux;
        }
        __syncthreads();
        if (tid == 0) {
            if (fl->continuity_bc == EMBER_CONTINUITY_LEFT) {
                double r = fl->rv_zero;
                rV[0] = r;
#pragma unroll 8
                for (int j = 0; j < N - 1; ++j) {
                    r = r - m[j];
                    rV[j + 1] = r;
                }
            } else if (fl->continuity_bc == EMBER_CONTINUITY_ZERO) {
                int j = jc;
                double dVdx0 = -rph[j] * (drhodt[j] - (rho[j] * beta) * y[3 * j + 0]);
                if (jc != 0)
                    dVdx0 = 0.5 * dVdx0 -
                            (0.5 * rph[j - 1]) * (drhodt[j - 1] + (rho[j - 1] * beta) * y[3 * (j - 1) + 0]);
                double r = (x[j] - fl->x_vzero) * dVdx0;
                rV[j] = r;
                for (j = jc; j < jj; ++j) {
                    r = r - m[j];
                    rV[j + 1] = r;
                }
                if (jc != 0) {
                    j = jc - 1;
                    r = (x[j] - fl->x_vzero) * dVdx0;
                    rV[j] = r;
                    for (j = jc - 1; j > 0; --j) {
                        r = r + m[j - 1];
                        rV[j - 1] = r;
                    }
                }
            } else {
                double r;
                if (fl->continuity_bc == EMBER_CONTINUITY_TEMP) {
                    // at the last point (where the per-step update can put the
                    // temperature crossing) only the backward difference exists
                    const int j = jc;
                    const double Tj = y[3 * j + 1];
                    if (j == 0 || (j < jj && sT[j] / (y[3 * (j + 1) + 1] - Tj) < 0))
                        r = (((rph[j] * rho[j]) * sT[j]) * hh[j]) / (y[3 * (j + 1) + 1] - Tj);
                    else
                        r = (((rph[j - 1] * rho[j]) * sT[j]) * hh[j - 1]) / (Tj - y[3 * (j - 1) + 1]);
                } else {
                    r = fl->rv_cont;
                }
                rV[jc] = r;
                const double r0 = r;
                for (int j = jc; j < N - 1; ++j) {
                    r = r - m[j];
                    rV[j + 1] = r;
                }
                r = r0;
                for (int j = jc; j > 0; --j) {
                    r = r + mb[j];
                    rV[j - 1] = r;
                }
            }
        }
        __syncthreads();
        double aa, dadt;
        conv_strain(*fl, t, aa, dadt);
        const double K = dadt / beta + (aa * aa) / (beta * beta);
        const bool cv = fl->left_bc == EMBER_BC_CONTROL_VOLUME || fl->left_bc == EMBER_BC_WALL_FLUX;
        const double rVjj = rV[jj];
        const bool right_fixed = rVjj < 0 || fl->right_bc == EMBER_BC_FIXED_VALUE;
        for (int j = tid; j < N; j += kNT) {
            const double Vj = (j == 0 || fl->alpha == 0) ? rV[j] : rV[j] / x[j];
            V[j] = Vj;
            const double Uj = y[3 * j + 0], Tj = y[3 * j + 1], Wj = y[3 * j + 2];
            const double rj = rho[j];
            const double strain_term = (fl->rhou / rj) * K;
            if (j == 0) {
                ydot[0] = (sU[0] - Uj * Uj) + strain_term;
                if (cv) {
                    const double cvol = center_volume(x, fl->alpha);
                    const double rvm = dmaxc(rV[0], 0.0);
                    ydot[1] = (-rvm * (Tj - fl->t_left)) / (rj * cvol) + sT[0];
                    ydot[2] = (-rvm * (Wj - fl->w_left)) / (rj * cvol) - (Wj * Wj) * sW[0];
                } else {
                    ydot[1] = sT[0];
                    ydot[2] = -((Wj * Wj) * sW[0]);
                }
            } else if (j < jj) {
                double dT, dU, dW;
                if (rV[j] < 0) {
                    dT = (y[3 * (j + 1) + 1] - Tj) / hh[j];
                    dU = (y[3 * (j + 1) + 0] - Uj) / hh[j];
                    dW = (y[3 * (j + 1) + 2] - Wj) / hh[j];
                } else {
                    dT = (Tj - y[3 * (j - 1) + 1]) / hh[j - 1];
                    dU = (Uj - y[3 * (j - 1) + 0]) / hh[j - 1];
                    dW = (Wj - y[3 * (j - 1) + 2]) / hh[j - 1];
                }
                ydot[3 * j + 0] = (((-Vj * dU) / rj - Uj * Uj) + strain_term) + sU[j];
                ydot[3 * j + 1] = (-Vj * dT) / rj + sT[j];
                ydot[3 * j + 2] = (-Vj * dW) / rj - (Wj * Wj) * sW[j];
            } else if (right_fixed) {
                ydot[3 * jj + 0] = (sU[jj] - Uj * Uj) + strain_term;
                ydot[3 * jj + 1] = sT[jj];
                ydot[3 * jj + 2] = -((Wj * Wj) * sW[jj]);
            } else {
                const double hl = hh[jj - 1];
                ydot[3 * jj + 0] =
                    ((sU[jj] - ((Vj * (Uj - y[3 * (jj - 1) + 0])) / hl) / rj) - Uj * Uj) + strain_term;
                ydot[3 * jj + 1] = sT[jj] - ((Vj * (Tj - y[3 * (jj - 1) + 1])) / hl) / rj;
                ydot[3 * jj + 2] = -((Wj * Wj) * sW[jj]) - ((Vj * (Wj - y[3 * (jj - 1) + 2])) / hl) / rj;
            }
        }
        __syncthreads();
    }

    // V / rho of the last right-hand side, recorded with the time
    __device__ void record(double t) {
        if (n_history >= max_history) {
            overflow = 1;
            return;
        }
        const int N = fl->n_points;
        if (threadIdx.x == 0) ht[n_history] = t;
        double* v = hv + size_t(n_history) * N;
        for (int j = threadIdx.x; j < N; j += kNT) v[j] = u.V[j] / u.rho[j];
        n_history++;
    }
    __device__ void on_step(double t) { record(t); }
};

__global__ void __launch_bounds__(kNT, 2) k_conv_utw(const __grid_constant__ ConvArgs a) {
    __shared__ double red[kRed];
    __shared__ AdamsShared sh;
    extern __shared__ double dyn[];  // 3 * max n_points
    const int fi = blockIdx.x;
    const ConvFlame& F = a.flames[fi];
    const int N = F.f.n_points;
    if (!utw_slice_ok(a, F) || 3 * int64_t(N) > a.dyn_n) {
        if (threadIdx.x == 0) {
            a.status[size_t(fi) * (1 + a.S)] = kStatusBadSlice;
            a.n_hist[fi] = 0;
        }
        return;
    }
    UtwSys s;
    s.n = 3 * N;
    s.a = &a;
    s.fl = &F.f;
    s.x = a.x + F.p0;
    s.drhodt = a.drhodt + F.p0;
    s.sU = a.split + F.v0;
    s.sT = a.split + F.v0 + N;
    s.u = utw_view(a, F);
    s.sm_m = dyn;
    s.sm_mb = dyn + N;
    s.sm_rV = dyn + 2 * N;
    s.ht = a.hist_t + F.hist;
    s.hv = a.hist_v + F.histv;
    s.n_history = 0;
    s.overflow = 0;
    s.max_history = a.max_history;
    double* wk = a.wk_utw + F.utw_wk;
    double t0, tf;
    stage_times(a, t0, tf);
    // the record starts with V / rho of the initial state
    s.f(t0, s.u.y3, wk);
    s.record(t0);
    int st[4];
    int rc = adams_block<kNT>(s, wk, s.u.y3, a.reltol, t0, tf, 1, a.min_step, a.max_steps, st, red, sh);
    if (s.overflow) rc = -20;
    // rV of the last right-hand side (V is already in the slice): the next
    // step's continuity point reads both, as the reference reads its members
    __syncthreads();
    for (int j = threadIdx.x; j < N; j += kNT) s.u.rV[j] = s.sm_rV[j];
    double* state = a.state + F.v0;
    for (int j = threadIdx.x; j < N; j += kNT) {
        state[j] = s.u.y3[3 * j + 0];
        state[size_t(N) + j] = s.u.y3[3 * j + 1];
    }
    if (threadIdx.x == 0) {
        a.status[size_t(fi) * (1 + a.S)] = rc;
        a.n_hist[fi] = s.n_history;
        if (a.stats) {
            a.stats[4 * fi + 0] = st[0];
            a.stats[4 * fi + 1] = st[1];
        }
    }
}

template <int NT>
struct SpecSys {
    int n;
    const ConvArgs* a;
    const ember_convection_flame* fl;
    const double *x, *hh, *split;
    double y_left;
    int H;
    const double *ht, *hv;  // ht: the record's times, in shared memory when they fit

    __device__ double atol(int) const { return a->abstol_y; }

    // ConvectionSystemY::f with v(t) from ConvectionSystemY::update_v: the
    // interval [lower_bound(t), next], moved back by one at the end of the record
    __device__ void f(double t, const double* y, double* ydot) {
        const int N = n, jj = N - 1;
        __syncthreads();
        int iL = -1;
        double s = 0.0;
        if (H > 1) {
            int lo = 0, hi = H;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (ht[mid] < t)
                    lo = mid + 1;
                else
                    hi = mid;
            }
            iL = lo;
            if (iL == H) iL--;
            if (iL + 1 == H) iL--;
            s = (t - ht[iL]) / (ht[iL + 1] - ht[iL]);
        }
        const double* vL = hv + size_t(iL < 0 ? 0 : iL) * N;
        const double* vR = iL < 0 ? vL : vL + N;
        const bool cv = fl->left_bc == EMBER_BC_CONTROL_VOLUME || fl->left_bc == EMBER_BC_WALL_FLUX;
        for (int j = threadIdx.x; j < N; j += NT) {
            const double v = iL < 0 ? vL[j] : vL[j] * (1 - s) + vR[j] * s;
            if (j == 0) {
                if (cv) {
                    const double cvol = center_volume(x, fl->alpha);
                    const double rvm = dmaxc(v, 0.0);
                    ydot[0] = (-rvm * (y[0] - y_left)) / cvol + split[0];
                } else {
                    ydot[0] = split[0];
                }
            } else if (j < jj) {
                const double dYdx = (v < 0) ? (y[j + 1] - y[j]) / hh[j] : (y[j] - y[j - 1]) / hh[j - 1];
                ydot[j] = -v * dYdx + split[j];
            } else if (v < 0 || fl->right_bc == EMBER_BC_FIXED_VALUE) {
                ydot[jj] = split[jj];
            } else {
                ydot[jj] = split[jj] - (v * (y[jj] - y[jj - 1])) / hh[jj - 1];
            }
        }
        __syncthreads();
    }
    __device__ void on_step(double) {}
};

constexpr int kHistShared = 512;

template <int NT>
__global__ void __launch_bounds__(NT, 12) k_conv_species(const __grid_constant__ ConvArgs a) {
    __shared__ double red[kRed];
    __shared__ AdamsShared sh;
    __shared__ double ht_s[kHistShared];
    const int sys = blockIdx.x;
    const int fi = sys / a.S, k = sys % a.S;
    const ConvFlame& F = a.flames[fi];
    const int N = F.f.n_points;
    int* status = a.status + size_t(fi) * (1 + a.S);
    const int utw_rc = status[0];
    if (utw_rc != 0) {
        if (threadIdx.x == 0) status[1 + k] = utw_rc;
        return;
    }
    const int H = a.n_hist[fi];
    if (a.spec_off[sys] < 0 || a.spec_off[sys] + int64_t(kWorkVectors) * N > a.wk_spec_n || H < 1 ||
        H > a.max_history) {
        if (threadIdx.x == 0) status[1 + k] = kStatusBadSlice;
        return;
    }
    SpecSys<NT> s;
    s.n = N;
    s.a = &a;
    s.fl = &F.f;
    s.x = a.x + F.p0;
    s.hh = utw_view(a, F).hh;
    s.split = a.split + F.v0 + size_t(2 + k) * N;
    s.y_left = a.y_left[size_t(fi) * a.S + k];
    s.H = H;
    s.ht = a.hist_t + F.hist;
    if (s.H <= kHistShared) {
        for (int i = threadIdx.x; i < s.H; i += NT) ht_s[i] = s.ht[i];
        __syncthreads();
        s.ht = ht_s;
    }
    s.hv = a.hist_v + F.histv;
    int st[4];
    double* y = a.state + F.v0 + size_t(2 + k) * N;
    double t0, tf;
    stage_times(a, t0, tf);
    const int rc = adams_block<NT>(s, a.wk_spec + a.spec_off[sys], y, a.reltol, t0, tf, 0, a.min_step,
                                   a.max_steps, st, red, sh);
    if (threadIdx.x == 0) {
        status[1 + k] = rc;
        if (a.stats) {
            atomicAdd(&a.stats[4 * fi + 2], st[0]);
            atomicAdd(&a.stats[4 * fi + 3], st[1]);
        }
    }
}

}  // namespace
}  // namespace ember

using namespace ember;

namespace ember {

int conv_plan_layout(ConvPlan& p, int n_flames, const ember_convection_flame* flames, int S,
                     const ember_convection_options* opts) {
    EMBER_CHECK_ARG(opts->reltol > 0 && opts->abstol_u > 0 && opts->abstol_t > 0 && opts->abstol_y > 0,
                    "tolerances must be positive");
    EMBER_CHECK_ARG(opts->max_steps > 0 && opts->max_history >= 2, "max_steps > 0 and max_history >= 2 required");
    EMBER_CHECK_ARG(opts->min_step >= 0, "min_step must be >= 0");
    EMBER_CHECK_ARG(opts->species_threads == 0 || opts->species_threads == kNTSpecies,
                    "species_threads must be 0 or 32");
    const int nv = S + 2;
    p = ConvPlan{};
    p.n_flames = n_flames;
    p.S = S;
    p.hf.resize(n_flames);
    p.spec_off.resize(size_t(n_flames) * S);
    for (int f = 0; f < n_flames; ++f) {
        const ember_convection_flame& g = flames[f];
        const int N = g.n_points;
        EMBER_CHECK_ARG(N >= 3 && N <= EMBER_CONVECTION_MAX_POINTS, "flame %d: n_points must be in [3, %d]", f,
                        EMBER_CONVECTION_MAX_POINTS);
        p.max_points = N > p.max_points ? N : p.max_points;
        EMBER_CHECK_ARG(g.alpha == 0 || g.alpha == 1, "flame %d: alpha must be 0 or 1", f);
        EMBER_CHECK_ARG(g.left_bc >= EMBER_BC_FIXED_VALUE && g.left_bc <= EMBER_BC_WALL_FLUX,
                        "flame %d: bad left boundary condition %d", f, g.left_bc);
        EMBER_CHECK_ARG(g.continuity_bc >= EMBER_CONTINUITY_LEFT && g.continuity_bc <= EMBER_CONTINUITY_TEMP,
                        "flame %d: bad continuity boundary condition %d", f, g.continuity_bc);
        EMBER_CHECK_ARG(g.continuity_bc == EMBER_CONTINUITY_LEFT || (g.j_cont >= 0 && g.j_cont < N),
                        "flame %d: j_cont out of range", f);
        EMBER_CHECK_ARG(g.beta > 0 && g.pressure > 0, "flame %d: beta and pressure must be positive", f);
        EMBER_CHECK_ARG(g.strain_dt >= 0, "flame %d: strain_dt must be >= 0", f);
        EMBER_CHECK_ARG(g.strain_type == EMBER_STRAIN_LINEAR || g.strain_type == EMBER_STRAIN_CHEBYSHEV,
                        "flame %d: bad strain function type %d", f, g.strain_type);
        EMBER_CHECK_ARG(g.strain_type != EMBER_STRAIN_CHEBYSHEV ||
                            (g.n_cheb >= 0 && g.n_cheb <= EMBER_CHEBYSHEV_MAX && g.cheb_t1 != g.cheb_t0),
                        "flame %d: Chebyshev strain needs 0..%d coefficients and cheb_t1 != cheb_t0", f,
                        EMBER_CHEBYSHEV_MAX);
        ConvFlame& c = p.hf[f];
        c.f = g;
        c.p0 = p.P;
        c.v0 = p.V;
        c.utw_wk = p.WU;
        c.hist = p.HS;
        c.histv = p.HV;
        for (int k = 0; k < S; ++k) {
            p.spec_off[size_t(f) * S + k] = p.WS;
            p.WS += int64_t(kWorkVectors) * N;
        }
        p.P += N;
        p.V += int64_t(nv) * N;
        p.WU += int64_t(kWorkVectors) * 3 * N + int64_t(kUtwScratch) * N;
        p.HS += int64_t(opts->max_history);
        p.HV += int64_t(opts->max_history) * N;
    }
    ConvArgs& a = p.a;
    a.n_flames = n_flames;
    a.S = S;
    a.t0 = opts->t_start;
    a.tf = opts->t_end;
    a.reltol = opts->reltol;
    a.abstol_u = opts->abstol_u;
    a.abstol_t = opts->abstol_t;
    a.abstol_y = opts->abstol_y;
    a.min_step = opts->min_step;
    a.max_steps = opts->max_steps;
    a.max_history = opts->max_history;
    a.wk_utw_n = p.WU;
    a.wk_spec_n = p.WS;
    a.hist_n = p.HS;
    a.histv_n = p.HV;
    a.dyn_n = 3 * int64_t(p.max_points);
    return EMBER_OK;
}

size_t conv_plan_bytes(const ConvPlan& p, bool with_stats) {
    const size_t nf = size_t(p.n_flames);
    size_t b = Scratch::rounded(nf * (1 + p.S) * sizeof(int));
    if (with_stats) b += Scratch::rounded(nf * 4 * sizeof(int));
    b += Scratch::rounded(nf * sizeof(ConvFlame)) + Scratch::rounded(p.spec_off.size() * sizeof(int64_t));
    b += Scratch::rounded(size_t(p.WU) * sizeof(double)) + Scratch::rounded(size_t(p.WS) * sizeof(double));
    b += Scratch::rounded(size_t(p.HS) * sizeof(double)) + Scratch::rounded(size_t(p.HV) * sizeof(double));
    b += Scratch::rounded(nf * sizeof(int));
    return b;
}

int conv_plan_alloc(ConvPlan& p, Scratch& sc, bool with_stats, cudaStream_t st) {
    ConvArgs& a = p.a;
    const size_t nf = size_t(p.n_flames);
    int* status = nullptr;
    int* stats = nullptr;
    ConvFlame* dflames = nullptr;
    int64_t* dspec = nullptr;
    double *wku = nullptr, *wks = nullptr, *ht = nullptr, *hv = nullptr;
    int* nh = nullptr;
    EMBER_TRY(sc.alloc(&status, nf * (1 + p.S)));
    if (with_stats) EMBER_TRY(sc.alloc(&stats, nf * 4));
    EMBER_TRY(sc.alloc(&dflames, nf));
    EMBER_TRY(sc.alloc(&dspec, p.spec_off.size()));
    EMBER_TRY(sc.alloc(&wku, size_t(p.WU)));
    EMBER_TRY(sc.alloc(&wks, size_t(p.WS)));
    EMBER_TRY(sc.alloc(&ht, size_t(p.HS)));
    EMBER_TRY(sc.alloc(&hv, size_t(p.HV)));
    EMBER_TRY(sc.alloc(&nh, nf));
    EMBER_CUDA_TRY(cudaMemcpyAsync(dflames, p.hf.data(), nf * sizeof(ConvFlame), cudaMemcpyHostToDevice, st));
    EMBER_CUDA_TRY(
        cudaMemcpyAsync(dspec, p.spec_off.data(), p.spec_off.size() * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    a.status = status;
    a.stats = stats;
    a.flames = dflames;
    a.spec_off = dspec;
    a.wk_utw = wku;
    a.wk_spec = wks;
    a.hist_t = ht;
    a.hist_v = hv;
    a.n_hist = nh;
    const size_t utw_smem = size_t(3) * p.max_points * sizeof(double);
    EMBER_TRY(raise_dynamic_smem(reinterpret_cast<const void*>(k_conv_utw), utw_smem));
    return EMBER_OK;
}

// ConvectionSystemUTW::updateContinuityBoundaryCondition
// (src/convectionSystem.cpp:196-277), run at the start of every split step
// but the first after the stage is attached or the state set (*ready == 0:
// the caller's values stand, as the reference's first update reads its
// initial V): the continuity point from the step-start temperature (state,
// point-major), the heat release rate (qdot, fixedQdot only) and V of the
// UTW system's last right-hand side; x_vzero for the stagnation-point
// condition; rv_cont = rV[j_cont] of that evaluation for fixedRight and
// fixedQdot, whose right-hand side never writes that entry. One thread per
// flame (sequential searches as the reference's).
__global__ void k_conv_continuity(const __grid_constant__ ConvArgs a, ConvFlame* flames, const int* ready,
                                  const double* __restrict__ state, int n_vars, const double* __restrict__ qdot) {
    const int fi = blockIdx.x * blockDim.x + threadIdx.x;
    if (fi >= a.n_flames || *ready == 0) return;
    ConvFlame& F = flames[fi];
    if (!utw_slice_ok(a, F)) return;
    ember_convection_flame& fl = F.f;
    const int N = fl.n_points, jj = N - 1;
    const double* x = a.x + F.p0;
    const UtwView u = utw_view(a, F);
    const double* V = u.V;
    auto T = [&](int j) { return state[(F.p0 + j) * n_vars + 1]; };
    auto sgn = [](double v) { return v > 0 ? 1 : (v < 0 ? -1 : 0); };
    int jc = fl.j_cont;
    switch (fl.continuity_bc) {
        case EMBER_CONTINUITY_LEFT: jc = 0; break;
        case EMBER_CONTINUITY_RIGHT: jc = jj; break;
        case EMBER_CONTINUITY_QDOT: {
            jc = 0;
            double qmax = 0.0;
            for (int j = 0; j < N; ++j) {
                const double q = qdot[F.p0 + j];
                if (q > qmax) {
                    qmax = q;
                    jc = j;
                }
            }
            break;
        }
        case EMBER_CONTINUITY_ZERO: {
            int js = jj;
            if (x[jj] > fl.x_vzero)
                for (int j = 0; j < N; ++j)
                    if (x[j] > fl.x_vzero) {
                        js = j;
                        break;
                    }
            jc = js;
            for (int i = 1; js + i <= jj || js >= i; ++i) {
                if (js + i <= jj && sgn(V[js + i]) != sgn(V[js])) {
                    jc = js + i;
                    break;
                }
                if (js >= i && sgn(V[js - i]) != sgn(V[js])) {
                    jc = js - i + 1;
                    break;
                }
            }
            if (jc == 0) fl.x_vzero = x[0] - V[0] * (x[1] - x[0]) / (V[1] - V[0]);
            else if (jc == jj) fl.x_vzero = x[jj] - V[jj] * (x[jj] - x[jj - 1]) / (V[jj] - V[jj - 1]);
            else fl.x_vzero = x[jc] - V[jc] * (x[jc] - x[jc - 1]) / (V[jc] - V[jc - 1]);
            break;
        }
        default: {  // fixedTemperature: the first crossing of the mid temperature
            double tmax = T(0), tmin = T(0);
            for (int j = 1; j < N; ++j) {
                tmax = fmax(tmax, T(j));
                tmin = fmin(tmin, T(j));
            }
            const double tmid = 0.5 * (tmax + tmin);
            jc = 0;
            for (int j = 1; j < N; ++j)
                if ((T(j) - tmid) * (T(j - 1) - tmid) <= 0) {
                    jc = j;
                    break;
                }
            break;
        }
    }
    fl.j_cont = jc;
    if (fl.continuity_bc == EMBER_CONTINUITY_RIGHT || fl.continuity_bc == EMBER_CONTINUITY_QDOT) fl.rv_cont = u.rV[jc];
}

__global__ void k_conv_ready(int* ready) { *ready = 1; }

// V of every flame's UTW system at its last right-hand side evaluation into
// out (point-major across flames), one CTA per flame.
__global__ void k_conv_velocity(const __grid_constant__ ConvArgs a, double* out) {
    const int fi = blockIdx.x;
    if (fi >= a.n_flames) return;
    const ConvFlame& F = a.flames[fi];
    if (!utw_slice_ok(a, F)) return;
    const UtwView u = utw_view(a, F);
    for (int j = threadIdx.x; j < F.f.n_points; j += blockDim.x) out[F.p0 + j] = u.V[j];
}

int conv_velocity_launch(const ConvPlan& p, const ConvArgs& a, double* out, cudaStream_t st) {
    k_conv_velocity<<<p.n_flames, 128, 0, st>>>(a, out);
    EMBER_CUDA_TRY(cudaGetLastError());
    return EMBER_OK;
}

int conv_continuity_launch(const ConvPlan& p, const ConvArgs& a, const int* ready, const double* state, int n_vars,
                           const double* qdot, cudaStream_t st) {
    k_conv_continuity<<<blocks_for(p.n_flames, 32), 32, 0, st>>>(a, const_cast<ConvFlame*>(a.flames), ready, state,
                                                                 n_vars, qdot);
    EMBER_CUDA_TRY(cudaGetLastError());
    k_conv_ready<<<1, 1, 0, st>>>(const_cast<int*>(ready));
    EMBER_CUDA_TRY(cudaGetLastError());
    return EMBER_OK;
}

int conv_launch(const ConvPlan& p, const ConvArgs& a, cudaStream_t st) {
    if (a.stats) EMBER_CUDA_TRY(cudaMemsetAsync(a.stats, 0, size_t(p.n_flames) * 4 * sizeof(int), st));
    k_conv_prepare<<<p.n_flames, 128, 0, st>>>(a);
    EMBER_CUDA_TRY(cudaGetLastError());
    const size_t utw_smem = size_t(3) * p.max_points * sizeof(double);
    k_conv_utw<<<p.n_flames, kNT, utw_smem, st>>>(a);
    EMBER_CUDA_TRY(cudaGetLastError());
    k_conv_species<kNTSpecies><<<p.n_flames * p.S, kNTSpecies, 0, st>>>(a);
    EMBER_CUDA_TRY(cudaGetLastError());
    return EMBER_OK;
}

}  // namespace ember

extern "C" int ember_convection_integrate(int n_flames, const ember_convection_flame* flames, int n_species,
                                          const double* mol_weight, const double* x, const double* y_left,
                                          const double* drhodt, const double* split_const, double* state,
                                          const ember_convection_options* opts, int* status, int* stats, int mem,
                                          void* stream) {
    EMBER_CHECK_ARG(n_flames >= 0, "n_flames must be >= 0");
    EMBER_CHECK_ARG(n_flames == 0 || (flames && mol_weight && x && y_left && drhodt && split_const && state && opts),
                    "null argument");
    EMBER_CHECK_ARG(n_species >= 1, "n_species must be >= 1");
    EMBER_CHECK_ARG(mem == EMBER_MEM_HOST || mem == EMBER_MEM_DEVICE, "bad mem flag %d", mem);
    if (n_flames == 0) return EMBER_OK;
    EMBER_CHECK_ARG(opts->t_end > opts->t_start, "t_end must be > t_start");
    const int S = n_species;
    ConvPlan p;
    EMBER_TRY(conv_plan_layout(p, n_flames, flames, S, opts));
    EMBER_TRY(ensure_device());
    cudaStream_t st = as_stream(stream);
    Scratch sc(st);
    ConvArgs& a = p.a;
    EMBER_TRY(stage_in(sc, mol_weight, size_t(S), mem, st, &a.W));
    EMBER_TRY(stage_in(sc, x, size_t(p.P), mem, st, &a.x));
    EMBER_TRY(stage_in(sc, y_left, size_t(n_flames) * S, mem, st, &a.y_left));
    EMBER_TRY(stage_in(sc, drhodt, size_t(p.P), mem, st, &a.drhodt));
    EMBER_TRY(stage_in(sc, split_const, size_t(p.V), mem, st, &a.split));
    EMBER_TRY(stage_buffer(sc, state, size_t(p.V), mem, &a.state));
    if (mem == EMBER_MEM_HOST)
        EMBER_CUDA_TRY(cudaMemcpyAsync(a.state, state, size_t(p.V) * sizeof(double), cudaMemcpyHostToDevice, st));
    EMBER_TRY(conv_plan_alloc(p, sc, stats != nullptr, st));
    EMBER_TRY(conv_launch(p, a, st));
    EMBER_TRY(stage_out(state, a.state, size_t(p.V), mem, st));
    const cudaMemcpyKind kind = mem == EMBER_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    if (status)
        EMBER_CUDA_TRY(cudaMemcpyAsync(status, a.status, size_t(n_flames) * (1 + S) * sizeof(int), kind, st));
    if (stats) EMBER_CUDA_TRY(cudaMemcpyAsync(stats, a.stats, size_t(n_flames) * 4 * sizeof(int), kind, st));
    const int rc = finish_call(mem, st);
    sc.release();
    return rc;
}
