// Variable-order BDF source-term integrator on the GPU (the CVODE path of the
// reference: SourceSystemCVODE::f, src/sourceSystem.cpp:128-164, integrated
// by CVODE in BDF mode with a dense direct solver, src/sundialsUtils.cpp:
// 33-172, integrateToTime with CV_NORMAL).
//
// Method (identical, operation for operation, to the CPU oracle): BDF of
// orders 1-5 in Nordsieck form, rescaled on step changes (LSODE/EPISODE
// form); CVODE's documented Newton iteration (modified Newton on
// M = I - gamma J, convergence-rate estimate, divergence test, 3 iterations,
// constant 0.1), WRMS error weights 1/(rtol|y| + atol), local error test,
// order selection from the q-1 / q / q+1 estimates, failure handling and
// Jacobian / iteration-matrix reuse (M every 20 steps or on a 30% change of
// gamma; J every 51 steps or after a failure with a stale J). The Jacobian is
// analytic in the species with a forward-difference temperature column.
//
// One CTA of NT threads per grid point, persistent grid with the
// longest-first work queue of the QSS path. Vectors live in shared memory;
// the Jacobian and the LU factors (column-major, partial pivoting) live in a
// per-CTA slice of global memory.
//
// Compiled with --fmad=false: only explicit fma() calls are fused.
#include "common.cuh"
#include "source.cuh"

#include <algorithm>

namespace ember {

constexpr int kQmax = 5;

// Shared-memory vectors of the BDF integrator (n entries each).
struct BdfSmem {
    double* z[kQmax + 2];   // Nordsieck array z_0..z_{q+1}
    double* zs[kQmax + 1];  // saved array for step retries
    double *acor, *acorp, *ewt, *y, *ft, *bb, *f0, *ycopy, *f1;
    int* piv;
    static __host__ __device__ size_t doubles(int n) { return size_t(2 * kQmax + 3 + 9) * n + (n + 1) / 2; }
    __device__ void carve(double* base, int n) {
        double* p = base;
        for (int j = 0; j <= kQmax + 1; ++j, p += n) z[j] = p;
        for (int j = 0; j <= kQmax; ++j, p += n) zs[j] = p;
        acor = p; p += n;
        acorp = p; p += n;
        ewt = p; p += n;
        y = p; p += n;
        ft = p; p += n;
        bb = p; p += n;
        f0 = p; p += n;
        ycopy = p; p += n;
        f1 = p; p += n;
        piv = reinterpret_cast<int*>(p);
    }
};

template <int NT>
struct BdfPoint {
    MechView m;
    ChemSmem w;
    BdfSmem v;
    const SourceArgs* a;
    const double* split;
    double x;
    double* J;       // global, column-major n x n
    double* M;       // global, column-major n x n (LU factors)
    int n, S;
    double rho, cp, qdot;
    double cachedT;
    int nfe;

    __device__ double atol(int i) const { return i == 0 ? a->bdf_atol_u : (i == 1 ? a->bdf_atol_t : a->bdf_atol_y); }

    // SourceSystemCVODE::f: ydot of [U, T, Y] (NoNorm state). Ends with a barrier.
    __device__ void f(double t, const double* y, double* ydot) {
        const int tid = threadIdx.x;
        const double T = y[1];
        if (!(cachedT == T)) {
            chem_rate_constants<NT>(m, w, T, a->kinetics_model == KIN_INTERP);
            cachedT = T;
        }
        double rho_c, cp_c;
        chem_rates<NT>(m, w, a->pressure, STATE_NO_NORM, T, y + 2, rho_c, cp_c, true);
        double part = 0.0;
        for (int k = tid; k < S; k += NT) part = fma(w.wn[k], w.hk[k], part);
        double qd = -block_sum<NT>(w.red, part);
        qd = qd + igniter(*a, t, x);
        const double rrho = 1.0 / rho_c;
        const double rrc = 1.0 / (rho_c * cp_c);
        for (int i = tid; i < n; i += NT) {
            const double sc = split ? split[i] : 0.0;
            double r;
            if (i == 0) r = sc;
            else if (i == 1) r = fma(qd, rrc, sc);
            else r = fma(w.wn[i - 2] * m.W[i - 2], rrho, sc);
            ydot[i] = r;
        }
        rho = rho_c;
        cp = cp_c;
        qdot = qd;
        ++nfe;
        __syncthreads();
    }

    __device__ double wrms(const double* vec) {
        double part = 0.0;
        for (int i = threadIdx.x; i < n; i += NT) {
            const double xv = vec[i] * v.ewt[i];
            part = fma(xv, xv, part);
        }
        return sqrt(block_sum<NT>(w.red, part) / n);
    }

    __device__ double jc(int r, int c) const { return J[size_t(c) * n + r]; }

    // Analytic Jacobian at y = z0 (rates of the preceding f(y) call in w),
    // f0: f(y). Column-major into J.
    __device__ void jacobian(double t, const double* yv, const double* f0v) {
        const int tid = threadIdx.x;
        const double T = yv[1];
        const double A = 1.0 / w.mmw;
        double bpart = 0.0;
        for (int k = tid; k < S; k += NT) bpart = fma(yv[2 + k] * m.rW[k], w.cpR[k], bpart);
        const double B = block_sum<NT>(w.red, bpart);
        const double rhoj = rho, rc = rho * cp;
        for (size_t e = tid; e < size_t(n) * n; e += NT) J[e] = 0.0;
        __syncthreads();
        // rows of d wdot / dc: one thread per species row, reactions in order
        for (int k = tid; k < S; k += NT) {
            double* colk = J + (size_t(2) * n + 2 + k);  // element (2+k, 2+j) at colk[j*n]
            double dense = 0.0;
            const int e1 = m.sp_off[k + 1];
            for (int e = m.sp_off[k]; e < e1; ++e) {
                const int ent = m.sp_ent[e];
                const int i = ent & 0xffffff;
                const int npk = (ent >> 24) & 0xf;
                const int nrk = (ent >> 28) & 0xf;
                const int info = m.rinfo[i];
                const int ty = rinfo_type(info);
                const bool rev = rinfo_rev(info);
                const int4 st = m.stoich[i];
                const int rc4[4] = {unpack_lo(st.x), unpack_hi(st.x), unpack_lo(st.y), unpack_hi(st.y)};
                const int pd4[4] = {unpack_lo(st.z), unpack_hi(st.z), unpack_lo(st.w), unpack_hi(st.w)};
                double rf = w.kfm[i];
                double pf = 1.0, pp = 1.0;
#pragma unroll
                for (int o = 0; o < 4; ++o)
                    if (rc4[o] != 0xffff) pf = pf * w.c[rc4[o]];
                if (rev) {
#pragma unroll
                    for (int o = 0; o < 4; ++o)
                        if (pd4[o] != 0xffff) pp = pp * w.c[pd4[o]];
                }
                const double kr = rev ? w.rkc[i] : 0.0;
                double dropdm = 0.0;
                int slot = -1;
                if (ty != RXN_ELEMENTARY) slot = rinfo_tbslot(info);
                if (ty == RXN_THREE_BODY) {
                    dropdm = rf * (pf - kr * pp);
                    rf = rf * w.concm[slot];
                } else if (ty == RXN_LINDEMANN || ty == RXN_TROE) {
                    const int fs = m.tb_fo[slot];
                    const double pr1 = 1.0 + w.fo_pr[fs];
                    dropdm = ((w.fo_F[fs] * (w.fo_k0[fs] * m.mult[i])) / (pr1 * pr1)) * (pf - kr * pp);
                }
                double dv[8];
                int dj[8];
                int nd = 0;
#pragma unroll
                for (int o = 0; o < 4; ++o) {
                    if (rc4[o] == 0xffff) continue;
                    double d = rf;
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        if (q != o && rc4[q] != 0xffff) d = d * w.c[rc4[q]];
                    dj[nd] = rc4[o];
                    dv[nd++] = d;
                }
                if (rev) {
#pragma unroll
                    for (int o = 0; o < 4; ++o) {
                        if (pd4[o] == 0xffff) continue;
                        double d = rf * kr;
#pragma unroll
                        for (int q = 0; q < 4; ++q)
                            if (q != o && pd4[q] != 0xffff) d = d * w.c[pd4[q]];
                        dj[nd] = pd4[o];
                        dv[nd++] = -d;
                    }
                }
                for (int side = 0; side < 2; ++side) {
                    const int cnt = side == 0 ? npk : nrk;
                    const double sgn = side == 0 ? 1.0 : -1.0;
                    for (int c = 0; c < cnt; ++c) {
                        for (int q = 0; q < nd; ++q) {
                            double* pj = colk + size_t(dj[q]) * n;
                            *pj = fma(sgn, dv[q], *pj);
                        }
                        if (ty != RXN_ELEMENTARY) {
                            const double de = m.tb_def[slot];
                            dense = fma(sgn * dropdm, de, dense);
                            const int g1 = m.tb_off[slot + 1];
                            for (int g = m.tb_off[slot]; g < g1; ++g) {
                                double* pj = colk + size_t(m.tb_sp[g]) * n;
                                *pj = fma(sgn * dropdm, m.tb_eff[g], *pj);
                            }
                        }
                    }
                }
            }
            // dense [M] part, then d wdot_k / dY_m in place
            double s_k = 0.0;
            for (int j = 0; j < S; ++j) {
                double* pj = colk + size_t(j) * n;
                const double vj = *pj + dense;
                *pj = vj;
                s_k = fma(vj, w.c[j], s_k);
            }
            const double sA = s_k / A;
            for (int j = 0; j < S; ++j) {
                double* pj = colk + size_t(j) * n;
                *pj = (rhoj * *pj - sA) * m.rW[j];
            }
        }
        __syncthreads();
        // energy row (one thread per column)
        const double rrc = 1.0 / rc, qrc2 = qdot / (rc * rc), pT = a->pressure / T;
        for (int mm = tid; mm < S; mm += NT) {
            const double* col = J + size_t(2 + mm) * n + 2;
            double hsum = 0.0;
            for (int k = 0; k < S; ++k) hsum = fma(col[k], w.hk[k], hsum);
            const double drc = pT * ((w.cpR[mm] * m.rW[mm]) / A - (B * m.rW[mm]) / (A * A));
            J[size_t(2 + mm) * n + 1] = -hsum * rrc - qrc2 * drc;
        }
        __syncthreads();
        // species rows
        const double wr = 1.0 / rhoj, rtp = (kGasConstant * T) / a->pressure;
        for (int k = tid; k < S; k += NT) {
            double* colk = J + (size_t(2) * n + 2 + k);
            const double aa = m.W[k] * wr, bk = (w.wn[k] * m.W[k]) * rtp;
            for (int j = 0; j < S; ++j) {
                double* pj = colk + size_t(j) * n;
                *pj = fma(aa, *pj, bk * m.rW[j]);
            }
        }
        // temperature column by forward difference
        const double dT = fabs(T) * 1.4901161193847656e-08;
        for (int i = tid; i < n; i += NT) v.ycopy[i] = i == 1 ? T + dT : yv[i];
        __syncthreads();
        const double saved_rho = rho, saved_cp = cp, saved_qdot = qdot;
        f(t, v.ycopy, v.f1);
        rho = saved_rho;
        cp = saved_cp;
        qdot = saved_qdot;
        const double rdT = 1.0 / ((T + dT) - T);
        for (int i = tid; i < n; i += NT) J[size_t(1) * n + i] = (v.f1[i] - f0v[i]) * rdT;
        __syncthreads();
    }

    // LU with partial pivoting of column-major M (first maximum as pivot;
    // multipliers a_ik * (1/a_kk)). Returns 0, or k+1 when column k has no
    // usable pivot: all zeros, or a NaN anywhere in it (then no row index is
    // chosen at all, so nothing is swapped or read out of range).
    __device__ int lu_factor() {
        const int tid = threadIdx.x;
        __shared__ double sbest[32];
        __shared__ int sidx[32];
        __shared__ int s_p;
        __shared__ double s_best;
        for (int k = 0; k < n; ++k) {
            double* colk = M + size_t(k) * n;
            double best = -1.0;
            int bi = n;
            int has_nan = 0;
            for (int i = k + tid; i < n; i += NT) {
                const double vv = fabs(colk[i]);
                if (vv != vv) has_nan = 1;
                if (vv > best) {
                    best = vv;
                    bi = i;
                }
            }
#pragma unroll
            for (int off = 16; off >= 1; off >>= 1) {
                const double ob = __shfl_xor_sync(0xffffffffu, best, off);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
                if (ob > best || (ob == best && oi < bi)) {
                    best = ob;
                    bi = oi;
                }
            }
            if (lane_id() == 0) {
                sbest[tid >> 5] = best;
                sidx[tid >> 5] = bi;
            }
            const int col_nan = __syncthreads_or(has_nan);
            if (col_nan) return k + 1;
            if (tid == 0) {
                double b = sbest[0];
                int p = sidx[0];
                for (int q = 1; q < NT / 32; ++q)
                    if (sbest[q] > b || (sbest[q] == b && sidx[q] < p)) {
                        b = sbest[q];
                        p = sidx[q];
                    }
                s_p = p;
                s_best = b;
                v.piv[k] = p;
            }
            __syncthreads();
            const int p = s_p;
            if (s_best == 0.0) return k + 1;
            if (p != k)
                for (int j = tid; j < n; j += NT) {
                    double* a1 = M + size_t(j) * n + k;
                    double* a2 = M + size_t(j) * n + p;
                    const double tt = *a1;
                    *a1 = *a2;
                    *a2 = tt;
                }
            __syncthreads();
            const double r = 1.0 / colk[k];
            for (int i = k + 1 + tid; i < n; i += NT) colk[i] = colk[i] * r;
            __syncthreads();
            // trailing update: one thread per row, columns in order
            for (int i = k + 1 + tid; i < n; i += NT) {
                const double l = colk[i];
                for (int j = k + 1; j < n; ++j) {
                    double* aij = M + size_t(j) * n + i;
                    *aij = fma(-l, M[size_t(j) * n + k], *aij);
                }
            }
            __syncthreads();
        }
        return 0;
    }

    __device__ void lu_solve(double* b) {
        const int tid = threadIdx.x;
        if (tid == 0)
            for (int k = 0; k < n; ++k) {
                const int p = v.piv[k];
                if (p != k) {
                    const double tt = b[k];
                    b[k] = b[p];
                    b[p] = tt;
                }
            }
        __syncthreads();
        for (int k = 0; k < n; ++k) {
            const double bk = b[k];
            const double* colk = M + size_t(k) * n;
            for (int i = k + 1 + tid; i < n; i += NT) b[i] = fma(-colk[i], bk, b[i]);
            __syncthreads();
        }
        for (int k = n - 1; k >= 0; --k) {
            const double* colk = M + size_t(k) * n;
            const double bk = b[k] / colk[k];
            __syncthreads();
            if (tid == 0) b[k] = bk;
            for (int i = tid; i < k; i += NT) b[i] = fma(-colk[i], bk, b[i]);
            __syncthreads();
        }
    }
};

__device__ __forceinline__ void bdf_l(int q, double* l) {
    for (int j = 0; j <= kQmax + 1; ++j) l[j] = 0.0;
    l[0] = 1.0;
    for (int i = 1; i <= q; ++i) {
        const double ri = 1.0 / i;
        for (int j = i; j >= 1; --j) l[j] = fma(l[j - 1], ri, l[j]);
    }
}

__device__ __forceinline__ double bdf_pow(double x, double e) { return em_exp(e * em_log(x)); }

template <int NT>
__device__ int bdf_integrate(BdfPoint<NT>& P, double tf, double t_start, int* stats) {
    const int tid = threadIdx.x;
    const int n = P.n;
    BdfSmem& v = P.v;
    const SourceArgs& a = *P.a;
    const double rtol = a.bdf_reltol, hmin = a.bdf_min_step;
    const double uround = 2.220446049250313e-16;
    int nst = 0, nje = 0, nef_total = 0, ncf_total = 0;
    int status = 0;
    P.nfe = 0;

    auto set_ewt = [&](const double* vec) {
        for (int i = tid; i < n; i += NT) v.ewt[i] = 1.0 / (rtol * fabs(vec[i]) + P.atol(i));
    };
    auto copy_z = [&](double* const* dst, double* const* src, int q) {
        for (int j = 0; j <= q; ++j)
            for (int i = tid; i < n; i += NT) dst[j][i] = src[j][i];
    };
    auto scale_z = [&](int q, double eta) {
        double s = eta;
        for (int j = 1; j <= q; ++j) {
            for (int i = tid; i < n; i += NT) v.z[j][i] *= s;
            s *= eta;
        }
    };

    // initial state and derivative
    P.f(t_start, v.z[0], v.f0);
    set_ewt(v.z[0]);
    double t = 0.0;
    double hub = 0.1 * tf;
    {
        double loc = 0.0;
        for (int i = tid; i < n; i += NT) {
            const double den = 0.1 * fabs(v.z[0][i]) + P.atol(i);
            loc = dmaxr(loc, fabs(v.f0[i]) / den);
        }
        const double rmax = block_max<NT>(P.w.red, loc);
        if (rmax * hub > 1.0) hub = 1.0 / rmax;
    }
    const double hlb = 100.0 * uround * tf;
    double hg = sqrt(hlb * hub);
    double h = hg;
    __syncthreads();
    if (hub > hlb) {
        for (int it = 0; it < 4; ++it) {
            for (int i = tid; i < n; i += NT) v.ycopy[i] = fma(hg, v.f0[i], v.z[0][i]);
            __syncthreads();
            P.f(t_start + hg, v.ycopy, v.f1);
            for (int i = tid; i < n; i += NT) v.bb[i] = (v.f1[i] - v.f0[i]) / hg;
            const double ydd = P.wrms(v.bb);
            const double hnew = (ydd * hub * hub > 2.0) ? sqrt(2.0 / ydd) : sqrt(hg * hub);
            const double ratio = hnew / hg;
            hg = hnew;
            if (ratio > 0.5 && ratio < 2.0) break;
        }
        h = dminr(dmaxr(0.5 * hg, hlb), hub);
    } else {
        h = hlb;
    }
    if (h < hmin) h = hmin;
    for (int i = tid; i < n; i += NT) v.z[1][i] = h * v.f0[i];
    __syncthreads();

    int q = 1, qwait = 2, nstlp = 0, nstlj = 0, qsave = 0;
    bool have_m = false, have_acorp = false;
    double gammap = 0.0, crate = 1.0, etamax = 10000.0, acnrm = 0.0, hsave = 0.0;
    double l[kQmax + 2];

    while (t < tf) {
        if (nst >= a.bdf_max_steps) {
            status = -11;
            break;
        }
        copy_z(v.zs, v.z, q);
        int ncf = 0, nef = 0;
        bool convfail_bad_j = false, force_setup = !have_m;
        double dsm = 0.0;
        bool accepted = false;
        while (!accepted) {
            // predict
            for (int k = 1; k <= q; ++k)
                for (int j = q; j >= k; --j)
                    for (int i = tid; i < n; i += NT) v.z[j - 1][i] += v.z[j][i];
            __syncthreads();
            const double tn = t + h;
            bdf_l(q, l);
            const double cq = 1.0 / ((q + 1) * l[1]);
            const double gamma = h / l[1];
            const double tq4 = 0.1 / cq;
            bool jcur = false;
            bool failed_conv = false;
            const double gamrat0 = have_m ? gamma / gammap : 1.0;
            if (force_setup || nst >= nstlp + 20 || fabs(gamrat0 - 1.0) > 0.3) {
                const bool jbad = (nst == 0) || (nst >= nstlj + 51) || convfail_bad_j || !have_m;
                if (jbad) {
                    P.f(t_start + tn, v.z[0], v.ft);
                    P.jacobian(t_start + tn, v.z[0], v.ft);
                    ++nje;
                    nstlj = nst;
                    jcur = true;
                }
                for (size_t e = tid; e < size_t(n) * n; e += NT) {
                    const int c = static_cast<int>(e / n), r = static_cast<int>(e - size_t(c) * n);
                    P.M[e] = (r == c ? 1.0 : 0.0) - gamma * P.J[e];
                }
                __syncthreads();
                const int sing = P.lu_factor();
                gammap = gamma;
                nstlp = nst;
                crate = 1.0;
                have_m = (sing == 0);
                force_setup = false;
                convfail_bad_j = false;
                if (sing) failed_conv = true;
            }
            if (!failed_conv) {
                const double gamrat = gamma / gammap;
                for (int i = tid; i < n; i += NT) {
                    v.acor[i] = 0.0;
                    v.y[i] = v.z[0][i];
                }
                __syncthreads();
                double delp = 0.0, del = 0.0;
                bool converged = false;
                const double rl1 = 1.0 / l[1];
                for (int mit = 0; mit < 3; ++mit) {
                    P.f(t_start + tn, v.y, v.ft);
                    for (int i = tid; i < n; i += NT) v.bb[i] = gamma * v.ft[i] - fma(rl1, v.z[1][i], v.acor[i]);
                    __syncthreads();
                    P.lu_solve(v.bb);
                    if (gamrat != 1.0) {
                        const double sc = 2.0 / (1.0 + gamrat);
                        for (int i = tid; i < n; i += NT) v.bb[i] *= sc;
                    }
                    del = P.wrms(v.bb);
                    for (int i = tid; i < n; i += NT) {
                        v.acor[i] += v.bb[i];
                        v.y[i] = v.z[0][i] + v.acor[i];
                    }
                    __syncthreads();
                    if (mit > 0) crate = dmaxr(0.3 * crate, del / delp);
                    const double dcon = del * dminr(1.0, crate) / tq4;
                    if (dcon <= 1.0) {
                        acnrm = (mit == 0) ? del : P.wrms(v.acor);
                        converged = true;
                        break;
                    }
                    if (mit >= 1 && del > 2.0 * delp) break;
                    delp = del;
                }
                if (!converged) failed_conv = true;
            }
            if (!failed_conv) {
                dsm = acnrm * cq;
                if (dsm <= 1.0) {
                    accepted = true;
                    break;
                }
                // error-test failure
                ++nef;
                ++nef_total;
                copy_z(v.z, v.zs, q);
                __syncthreads();
                if (nef >= 7 || h <= hmin * 1.0000000000000002) {
                    status = -13;
                    break;
                }
                if (nef <= 3) {
                    double eta = 1.0 / (bdf_pow(6.0 * dsm, 1.0 / (q + 1)) + 1e-6);
                    eta = dmaxr(0.1, dmaxr(eta, hmin / h));
                    if (nef >= 2) eta = dminr(eta, 0.2);
                    scale_z(q, eta);
                    h *= eta;
                } else {
                    const double eta = dmaxr(0.1, hmin / h);
                    h *= eta;
                    q = 1;
                    P.f(t_start + t, v.z[0], v.ft);
                    for (int i = tid; i < n; i += NT) v.z[1][i] = h * v.ft[i];
                }
                qwait = q + 1;
                have_acorp = false;
                etamax = 1.0;
                __syncthreads();
                copy_z(v.zs, v.z, q);
                __syncthreads();
                continue;
            }
            // convergence failure
            copy_z(v.z, v.zs, q);
            __syncthreads();
            ++ncf_total;
            if (!jcur && have_m) {
                force_setup = true;
                convfail_bad_j = true;
                continue;
            }
            ++ncf;
            if (ncf >= 10 || h <= hmin * 1.0000000000000002) {
                status = -14;
                break;
            }
            {
                const double eta = dmaxr(0.25, hmin / h);
                scale_z(q, eta);
                h *= eta;
                qwait = q + 1;
                have_acorp = false;
                etamax = 1.0;
                force_setup = true;
                __syncthreads();
                copy_z(v.zs, v.z, q);
                __syncthreads();
            }
        }
        if (status != 0) break;
        // ---- accepted step ----
        ++nst;
        t += h;
        for (int j = 0; j <= q; ++j)
            for (int i = tid; i < n; i += NT) v.z[j][i] = fma(l[j], v.acor[i], v.z[j][i]);
        set_ewt(v.z[0]);
        __syncthreads();
        const double etaq = 1.0 / (bdf_pow(6.0 * dsm, 1.0 / (q + 1)) + 1e-6);
        double eta = etaq;
        int qnew = q;
        --qwait;
        if (qwait == 0) {
            double etaqm1 = 0.0, etaqp1 = 0.0;
            if (q > 1) {
                double lm[kQmax + 2];
                bdf_l(q - 1, lm);
                double fact = 1.0;
                for (int i = 2; i <= q; ++i) fact *= i;
                const double ddn = P.wrms(v.z[q]) * (fact / (q * lm[1]));
                etaqm1 = 1.0 / (bdf_pow(6.0 * ddn, 1.0 / q) + 1e-6);
            }
            if (q < kQmax && have_acorp && qsave == q) {
                double lp[kQmax + 2];
                bdf_l(q + 1, lp);
                const double cqq = bdf_pow(h / hsave, (double)(q + 1));
                for (int i = tid; i < n; i += NT) v.bb[i] = fma(-cqq, v.acorp[i], v.acor[i]);
                const double dup = P.wrms(v.bb) / ((q + 2) * lp[1]);
                etaqp1 = 1.0 / (bdf_pow(10.0 * dup, 1.0 / (q + 2)) + 1e-6);
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
        } else if (qwait == 1 && q < kQmax) {
            for (int i = tid; i < n; i += NT) v.acorp[i] = v.acor[i];
            hsave = h;
            qsave = q;
            have_acorp = true;
        }
        if (etamax <= 1.0) {
            eta = 1.0;
            qnew = q;
        } else if (eta < 1.5 && qnew == q) {
            eta = 1.0;
        } else {
            eta = dminr(eta, etamax);
            if (h * eta < hmin) eta = hmin / h;
        }
        if (qnew > q) {
            const double c = l[q] / (q + 1);
            for (int i = tid; i < n; i += NT) v.z[q + 1][i] = v.acor[i] * c;
        }
        if (qnew != q) {
            q = qnew;
            qwait = q + 1;
            have_acorp = false;
        }
        if (eta != 1.0) {
            scale_z(q, eta);
            h *= eta;
        }
        etamax = 10.0;
        __syncthreads();
    }
    // interpolate at tf (CV_NORMAL) or return the last state
    if (status == 0) {
        const double s = (tf - t) / h;
        for (int i = tid; i < n; i += NT) {
            double val = v.z[q][i];
            for (int j = q - 1; j >= 0; --j) val = fma(val, s, v.z[j][i]);
            v.y[i] = val;
        }
    } else {
        for (int i = tid; i < n; i += NT) v.y[i] = v.z[0][i];
    }
    __syncthreads();
    stats[0] = nst;
    stats[1] = P.nfe;
    stats[2] = nef_total + ncf_total;
    stats[3] = nje;
    return status;
}

template <int NT>
__global__ void __launch_bounds__(NT) k_source_bdf(MechView m, SourceArgs a, int* counter, const int* order,
                                                  double* kcache, double* jm) {
    extern __shared__ double smem[];
    __shared__ int next_point;
    const int n = m.S + 2;
    const size_t cd = ChemSmem::doubles(m.S, m.R, m.n_tb, m.n_fo, true);
    BdfPoint<NT> P;
    P.m = m;
    P.w.carve(smem, kcache + size_t(blockIdx.x) * ChemSmem::global_doubles(m.R), m, true);
    P.w.fo_F = smem + cd;
    P.w.fo_pr = P.w.fo_F + m.n_fo;
    P.v.carve(P.w.fo_pr + m.n_fo, n);
    P.a = &a;
    P.n = n;
    P.S = m.S;
    P.J = jm + size_t(blockIdx.x) * 2 * size_t(n) * n;
    P.M = P.J + size_t(n) * n;
    P.cachedT = __longlong_as_double(0x7ff8000000000000LL);
    const int tid = threadIdx.x;
    for (;;) {
        if (tid == 0) {
            const int slot = atomicAdd(counter, 1);
            next_point = slot < a.n ? order[slot] : a.n;
        }
        __syncthreads();
        const int j = next_point;
        __syncthreads();
        if (j >= a.n) break;
        const double* yin = a.state_in + size_t(j) * n;
        for (int i = tid; i < n; i += NT) P.v.z[0][i] = yin[i];
        P.split = a.split ? a.split + size_t(j) * n : nullptr;
        P.x = a.x ? a.x[j] : 0.0;
        __syncthreads();
        int st4[4];
        int ret = bdf_integrate<NT>(P, a.dt[j], a.t_start_dev ? *a.t_start_dev : a.t_start, st4);
        int nonfinite = 0;
        double* yout = a.state_out + size_t(j) * n;
        for (int i = tid; i < n; i += NT) {
            const double yi = P.v.y[i];
            nonfinite |= !isfinite(yi);
            yout[i] = yi;
        }
        nonfinite = __syncthreads_or(nonfinite);
        if (ret == 0 && nonfinite) ret = -21;
        if (tid == 0) {
            a.status[j] = ret;
            if (a.stats)
                for (int q = 0; q < 4; ++q) a.stats[4 * size_t(j) + q] = st4[q];
        }
    }
}

// Dynamic shared memory and persistent grid size of the BDF kernel.
template <int NT>
static int bdf_config(const MechView& m, const SourceArgs& a, size_t* per_out, int* blocks_out) {
    const int n = m.S + 2;
    const size_t per = (ChemSmem::doubles(m.S, m.R, m.n_tb, m.n_fo, true) + size_t(2) * m.n_fo +
                        BdfSmem::doubles(n)) * sizeof(double);
    EMBER_CHECK_ARG(per <= 227 * 1024, "mechanism too large for the BDF shared-memory work area (%zu B)", per);
    EMBER_CUDA_TRY(cudaFuncSetAttribute(k_source_bdf<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(per)));
    int dev = 0, sms = 0, per_sm = 0;
    EMBER_CUDA_TRY(cudaGetDevice(&dev));
    EMBER_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    EMBER_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_source_bdf<NT>, NT, per));
    per_sm = std::max(per_sm, 1);
    *per_out = per;
    *blocks_out = std::max(1, std::min(a.n, sms * per_sm));
    return EMBER_OK;
}

template <int NT>
static int bdf_scratch_nt(const MechView& m, const SourceArgs& a, size_t* bytes) {
    size_t per = 0;
    int blocks = 0;
    EMBER_TRY(bdf_config<NT>(m, a, &per, &blocks));
    const size_t n = size_t(m.S) + 2;
    *bytes = Scratch::rounded(sizeof(double) * size_t(blocks) * ChemSmem::global_doubles(m.R)) +
             Scratch::rounded(sizeof(double) * size_t(blocks) * 2 * n * n) + Scratch::rounded(sizeof(int) * 64) +
             Scratch::rounded(sizeof(int) * size_t(a.n));
    return EMBER_OK;
}

int source_bdf_scratch_bytes(const MechView& m, const SourceArgs& a, size_t* bytes) {
    switch (chem_threads_for(m.S)) {
        case 64: return bdf_scratch_nt<64>(m, a, bytes);
        case 128: return bdf_scratch_nt<128>(m, a, bytes);
        case 160: return bdf_scratch_nt<160>(m, a, bytes);
        default: return bdf_scratch_nt<256>(m, a, bytes);
    }
}

template <int NT>
static int launch_bdf_nt(const MechView& m, const SourceArgs& a, int* counter, Scratch& sc, cudaStream_t st) {
    const int n = m.S + 2;
    size_t per = 0;
    int blocks = 0;
    EMBER_TRY(bdf_config<NT>(m, a, &per, &blocks));
    double *kcache = nullptr, *jm = nullptr;
    EMBER_TRY(sc.alloc(&kcache, size_t(blocks) * ChemSmem::global_doubles(m.R)));
    EMBER_TRY(sc.alloc(&jm, size_t(blocks) * 2 * size_t(n) * n));
    int* order = nullptr;
    EMBER_TRY(make_work_order(a, sc, st, &order));
    k_source_bdf<NT><<<blocks, NT, per, st>>>(m, a, counter, order, kcache, jm);
    EMBER_CUDA_TRY(cudaGetLastError());
    return EMBER_OK;
}

int launch_source_bdf(const MechView& m, const SourceArgs& a, int* counter, Scratch& sc, cudaStream_t st) {
    switch (chem_threads_for(m.S)) {
        case 64: return launch_bdf_nt<64>(m, a, counter, sc, st);
        case 128: return launch_bdf_nt<128>(m, a, counter, sc, st);
        case 160: return launch_bdf_nt<160>(m, a, counter, sc, st);
        default: return launch_bdf_nt<256>(m, a, counter, sc, st);
    }
}

}  // namespace ember
