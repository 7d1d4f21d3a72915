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

// Rows of a Nordsieck-type array stored contiguously: a[j] is row j (n
// values). Row addresses are computed, so no pointer table sits on the stack.
struct ZArr {
    double* base = nullptr;
    int n = 0;
    __device__ double* operator[](int j) const { return base + size_t(j) * n; }
};

// Shared-memory vectors of the BDF integrator (n entries each).
struct BdfSmem {
    ZArr z;   // Nordsieck array z_0..z_{q+1}
    ZArr zs;  // saved array for step retries
    double *acor, *acorp, *ewt, *y, *ft, *bb, *f0, *ycopy, *f1;
    double* rdiag;  // 1 / pivot of each column of the LU factors
    int* piv;
    int* perm;      // the row interchanges composed: after them, row i holds original row perm[i]
    // shared-memory doubles (zs_smem: the saved array in shared memory)
    static __host__ __device__ size_t doubles(int n, bool zs_smem = true) {
        return size_t(zs_smem ? 2 * kQmax + 3 + 10 : kQmax + 2 + 10) * n + 2 * ((n + 1) / 2);
    }
    // zs_global: (kQmax + 1) n doubles of global memory for zs, or null
    __device__ void carve(double* base, int n, double* zs_global = nullptr) {
        double* p = base;
        z = ZArr{p, n};
        p += size_t(kQmax + 2) * n;
        if (zs_global) {
            zs = ZArr{zs_global, n};
        } else {
            zs = ZArr{p, n};
            p += size_t(kQmax + 1) * n;
        }
        acor = p; p += n;
        acorp = p; p += n;
        ewt = p; p += n;
        y = p; p += n;
        ft = p; p += n;
        bb = p; p += n;
        f0 = p; p += n;
        ycopy = p; p += n;
        f1 = p; p += n;
        rdiag = p; p += n;
        piv = reinterpret_cast<int*>(p);
        perm = piv + 2 * ((n + 1) / 2);
    }
};

template <int NT>
struct BdfPoint {
    // the kernel's __grid_constant__ parameter: read in place, never copied to the stack
    const MechView& m;
    __device__ explicit BdfPoint(const MechView& mv) : m(mv) {}
    ChemSmem w;
    BdfSmem v;
    const SourceArgs* a = nullptr;
    const double* split = nullptr;
    double x = 0.0;
    double* J = nullptr;  // global, column-major n x n
    double* M = nullptr;  // global, column-major n x n (LU factors)
    int n = 0, S = 0;
    double rho = 0.0, cp = 0.0, qdot = 0.0;
    double cachedT = 0.0;
    int nfe = 0;
    double* tape = nullptr;  // this point's tape, or null

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
        chem_rates<NT>(m, w, a->pressure, STATE_NO_NORM, T, y + 2, rho_c, cp_c, true, false);
        const double *wn = w.wn, *hk = w.hk;
        double qd = -block_sum<NT>(w.red, S, [&](int k, double p) { return fma(wn[k], hk[k], p); });
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
        const double* ewt = v.ewt;
        return sqrt(block_sum<NT>(w.red, n, [&](int i, double p) {
                        const double xv = vec[i] * ewt[i];
                        return fma(xv, xv, p);
                    }) /
                    n);
    }

    __device__ double jc(int r, int c) const { return J[size_t(c) * n + r]; }

    // Analytic Jacobian at y = z0 (rates of the preceding f(y) call in w),
    // f0: f(y). Column-major into J.
    __device__ void jacobian(double t, const double* yv, const double* f0v) {
        const int tid = threadIdx.x;
        const double T = yv[1];
        const double A = 1.0 / w.mmw;
        const double *rW = m.rW, *cpR = w.cpR;
        const double B = block_sum<NT>(w.red, S, [&](int k, double p) { return fma(yv[2 + k] * rW[k], cpR[k], p); });
        const double rhoj = rho, rc = rho * cp;
        for (size_t e = tid; e < size_t(n) * n; e += NT) J[e] = 0.0;
        __syncthreads();
        // rows of d wdot / dc: one thread per species row, reactions in order
        for (int kk = tid; kk < S; kk += NT) {
            const int k = m.sp_order[kk];
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
                    // d/d[M] of kinf mult Pr/(1+Pr) F(Pr), Pr = k0 [M] / kinf
                    const int fs = m.tb_fo[slot];
                    const double pr1 = 1.0 + w.fo_pr[fs];
                    const double k0m = w.fo_k0[fs] * m.mult[i];
                    dropdm = ((w.fo_F[fs] * k0m) / (pr1 * pr1) + (k0m * (w.fo_pr[fs] / pr1)) * w.fo_dF[fs]) *
                             (pf - kr * pp);
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

    // In-place LU with partial pivoting (CVODE's dense getrf, first maximum
    // of |a_ik| as pivot, multipliers a_ik * (1/a_kk)): M = P^-1 L U, in
    // panels of kLuPanel columns with one panel of lookahead. While warp 0
    // brings the next panel up to date and factors it (its row interchanges
    // applied to its own columns only), the other warps, and warp 0 when it is
    // done, apply the current panel's steps to the rest of the trailing matrix;
    // then every thread applies the next panel's interchanges to the columns
    // outside it. Each element still receives the one-column algorithm's
    // operations in its order (an interchange only relabels rows, and the
    // columns a panel's interchanges reach later have by then received exactly
    // the updates that preceded the interchange), so the factors are the same
    // bits. Pivot searches compare |a_ik| through the bit pattern (integer
    // order = numeric order for doubles with the sign cleared, a NaN above
    // +inf), which keeps them off the FP64 pipe. Returns 0, or k + 1 when
    // column k has no usable pivot (all zeros, or a NaN anywhere in it).
    static constexpr int kLuPanel = 8;
    static constexpr int kLuGroup = 16;  // trailing columns per task of a warp

    // Panel [k0, k1) by the calling warp alone.
    __device__ int lu_panel_warp(int k0, int k1) {
        const int lane = threadIdx.x & 31;
        const long long kInf = 0x7ff0000000000000LL;
        for (int c = k0; c < k1; ++c) {
            double* colc = M + size_t(c) * n;
            for (int t = k0; t < c; ++t) {
                const double atc = colc[t];
                const double* colt = M + size_t(t) * n;
                for (int i = t + 1 + lane; i < n; i += 32) colc[i] = fma(-colt[i], atc, colc[i]);
                __syncwarp();
            }
            long long best = -1;
            int bi = n;
            int has_nan = 0;
            for (int i = c + lane; i < n; i += 32) {
                const long long vv = __double_as_longlong(colc[i]) & 0x7fffffffffffffffLL;
                if (vv > kInf) has_nan = 1;
                if (vv > best) {
                    best = vv;
                    bi = i;
                }
            }
#pragma unroll
            for (int off = 16; off >= 1; off >>= 1) {
                const long long ob = __shfl_xor_sync(0xffffffffu, best, off);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
                if (ob > best || (ob == best && oi < bi)) {
                    best = ob;
                    bi = oi;
                }
            }
            if (__any_sync(0xffffffffu, has_nan)) return c + 1;
            if (best == 0) return c + 1;
            if (lane == 0) v.piv[c] = bi;
            if (bi != c && lane < k1 - k0) {
                double* colj = M + size_t(k0 + lane) * n;
                const double tt = colj[c];
                colj[c] = colj[bi];
                colj[bi] = tt;
            }
            __syncwarp();
            const double r = 1.0 / colc[c];
            if (lane == 0) v.rdiag[c] = r;
            for (int i = c + 1 + lane; i < n; i += 32) colc[i] = colc[i] * r;
            __syncwarp();
        }
        return 0;
    }

    // Panel [k, kend)'s steps on columns [j0, j1) (j1 - j0 <= 32) by the
    // calling warp: the pivot rows k+1..kend-1 (a lane per column, the earlier
    // panel steps in order), then every other row (lanes over rows, all the
    // panel's steps in order).
    __device__ void lu_panel_update(int k, int kend, int j0, int j1) {
        const int lane = threadIdx.x & 31;
        if (j0 + lane < j1) {
            double* colj = M + size_t(j0 + lane) * n;
            for (int r = k + 1; r < kend; ++r) {
                double a = colj[r];
                for (int t = k; t < r; ++t) a = fma(-M[size_t(t) * n + r], colj[t], a);
                colj[r] = a;
            }
        }
        __syncwarp();
        if (n - kend <= 64) {
            // few rows: columns outer, the column's u in registers
            for (int j = j0; j < j1; ++j) {
                double* colj = M + size_t(j) * n;
                double u[kLuPanel];
#pragma unroll
                for (int t = 0; t < kLuPanel; ++t) u[t] = (k + t < kend) ? colj[k + t] : 0.0;
                for (int i = kend + lane; i < n; i += 32) {
                    double a = colj[i];
#pragma unroll
                    for (int t = 0; t < kLuPanel; ++t)
                        if (k + t < kend) a = fma(-M[size_t(k + t) * n + i], u[t], a);
                    colj[i] = a;
                }
            }
            __syncwarp();
            return;
        }
        // many rows: rows outer, columns inner, so that a lane loads its row's
        // panel multipliers once for the whole column group (u is the same for
        // every lane); each element takes the same steps in the same order
        for (int i0 = kend; i0 < n; i0 += 32) {
            const int i = i0 + lane;
            const bool in = i < n;
            double l[kLuPanel];
#pragma unroll
            for (int t = 0; t < kLuPanel; ++t) l[t] = (in && k + t < kend) ? M[size_t(k + t) * n + i] : 0.0;
            if (in) {
                for (int j = j0; j < j1; ++j) {
                    double* colj = M + size_t(j) * n;
                    double a = colj[i];
#pragma unroll
                    for (int t = 0; t < kLuPanel; ++t)
                        if (k + t < kend) a = fma(-l[t], colj[k + t], a);
                    colj[i] = a;
                }
            }
        }
        __syncwarp();
    }

    // The row interchanges of panel [k0, k1), in pivot order, on columns
    // [j0, j1) (j1 - j0 <= 32), a lane per column, by the calling warp.
    __device__ void lu_swaps_warp(int k0, int k1, int j0, int j1) {
        const int lane = threadIdx.x & 31;
        if (j0 + lane < j1) {
            double* colj = M + size_t(j0 + lane) * n;
            for (int c = k0; c < k1; ++c) {
                const int p = v.piv[c];
                if (p != c) {
                    const double tt = colj[c];
                    colj[c] = colj[p];
                    colj[p] = tt;
                }
            }
        }
        __syncwarp();
    }

    // A panel's row interchanges reach the columns to its right just before
    // they take the panel's steps (the warp that updates a column group swaps
    // it first), and the columns to its left (the L factors, which no later
    // step reads) at the end. Every column still receives every interchange
    // in pivot order before any step that reads it, so the factors are those
    // of applying each interchange to whole rows at once. One barrier per
    // panel; the work counters alternate so that the next panel's is reset
    // while this one's is in use.
    __device__ int lu_factor() {
        const int tid = threadIdx.x;
        const int warp = tid >> 5, lane = tid & 31;
        __shared__ int s_sing, s_next[2];
        const int k1 = min(kLuPanel, n);
        if (warp == 0) {
            const int sg = lu_panel_warp(0, k1);
            if (lane == 0) s_sing = sg;
        }
        if (tid == 0) {
            s_next[0] = 0;
            s_next[1] = 0;
        }
        __syncthreads();
        if (s_sing) return s_sing;
        int it = 0;
        for (int k = 0; k + kLuPanel < n; k += kLuPanel, ++it) {
            const int kend = k + kLuPanel;
            const int k2e = min(kend + kLuPanel, n);
            int* counter = &s_next[it & 1];
            if (warp == 0) {
                lu_swaps_warp(k, kend, kend, k2e);
                lu_panel_update(k, kend, kend, k2e);
                const int sg = lu_panel_warp(kend, k2e);
                if (lane == 0) s_sing = sg;
            }
            for (;;) {
                int g = 0;
                if (lane == 0) g = atomicAdd(counter, 1);
                g = __shfl_sync(0xffffffffu, g, 0);
                const int j0 = k2e + g * kLuGroup;
                if (j0 >= n) break;
                const int j1 = min(j0 + kLuGroup, n);
                lu_swaps_warp(k, kend, j0, j1);
                lu_panel_update(k, kend, j0, j1);
            }
            if (tid == 0) s_next[(it + 1) & 1] = 0;
            __syncthreads();
            if (s_sing) return s_sing;
        }
        // the L factors: the interchanges of every panel after the column's own
        for (int j = tid; j < n; j += NT) {
            double* colj = M + size_t(j) * n;
            for (int c = (j / kLuPanel + 1) * kLuPanel; c < n; ++c) {
                const int p = v.piv[c];
                if (p != c) {
                    const double tt = colj[c];
                    colj[c] = colj[p];
                    colj[p] = tt;
                }
            }
        }
        lu_compose_interchanges();
        return 0;
    }

    // v.perm from v.piv (the interchanges applied in order to the identity),
    // so that a solve gathers its right-hand side in one pass.
    __device__ void lu_compose_interchanges() {
        if (threadIdx.x == 0) {
            int* pm = v.perm;
            for (int i = 0; i < n; ++i) pm[i] = i;
            for (int k = 0; k < n; ++k) {
                const int p = v.piv[k];
                const int t = pm[k];
                pm[k] = pm[p];
                pm[p] = t;
            }
        }
        __syncthreads();
    }

    // Solve M^T w = b in place with the factors and pivots of lu_factor
    // (P M = L U, so M^T = U^T L^T P): U^T forward, L^T backward, then the
    // row interchanges undone in reverse order.
    __device__ void lu_solve_transpose(double* b) {
        __syncthreads();
        if (threadIdx.x < 32) {
            const int lane = threadIdx.x;
            for (int k = 0; k < n; ++k) {
                const double zk = b[k] * v.rdiag[k];
                __syncwarp();
                if (lane == 0) b[k] = zk;
                for (int j = k + 1 + lane; j < n; j += 32) b[j] = fma(-M[size_t(j) * n + k], zk, b[j]);
                __syncwarp();
            }
            for (int k = n - 1; k >= 1; --k) {
                const double uk = b[k];
                for (int i = lane; i < k; i += 32) b[i] = fma(-M[size_t(i) * n + k], uk, b[i]);
                __syncwarp();
            }
            if (lane == 0)
                for (int k = n - 1; k >= 0; --k) {
                    const int p = v.piv[k];
                    if (p != k) {
                        const double tt = b[k];
                        b[k] = b[p];
                        b[p] = tt;
                    }
                }
        }
        __syncthreads();
    }

    // out = J^T vec (J column-major: column c holds d f_r / d y_c).
    __device__ void jacobian_transpose_times(const double* vec, double* out, bool accumulate) {
        for (int c = threadIdx.x; c < n; c += NT) {
            const double* col = J + size_t(c) * n;
            double acc = 0.0;
            for (int r = 0; r < n; ++r) acc = fma(col[r], vec[r], acc);
            out[c] = accumulate ? out[c] + acc : acc;
        }
        __syncthreads();
    }

    // pbar_i += vec . d f / d ln(multiplier_i) at the state of the last f()
    // call: reaction i's net rate of progress r_i enters dY_k/dt as
    // nu_ki r_i W_k / rho and dT/dt as -(sum_k nu_ki h_k) r_i / (rho cp).
    __device__ void multiplier_vjp(const double* vec, double* pbar) {
        const double rrho = 1.0 / rho, rrc = 1.0 / (rho * cp);
        for (int i = threadIdx.x; i < m.R; i += NT) {
            const double r = w.ropf[i] - w.ropr[i];
            const int4 st = m.stoich[i];
            const int sp[8] = {unpack_lo(st.x), unpack_hi(st.x), unpack_lo(st.y), unpack_hi(st.y),
                               unpack_lo(st.z), unpack_hi(st.z), unpack_lo(st.w), unpack_hi(st.w)};
            double ey = 0.0, eh = 0.0;
#pragma unroll
            for (int o = 0; o < 8; ++o) {
                const int k = sp[o];
                if (k == 0xffff) continue;
                const double sg = o < 4 ? -1.0 : 1.0;
                ey = fma(sg * m.W[k], vec[2 + k], ey);
                eh = fma(sg, w.hk[k], eh);
            }
            pbar[i] += r * (ey * rrho - eh * (vec[1] * rrc));
        }
    }

    // Forward and back substitution with the factors, by the first warp, with
    // the right-hand side in its registers (lane l holds rows l, l + 32, ...):
    // the row interchanges as one gather through v.perm, then per column a
    // shuffle broadcast and one fma per row held (L unit lower), and per
    // column the product with the pivot reciprocal then the updates above
    // (U). Each element receives the same operations in the same order as
    // SUNDIALS' dense getrs with fused multiply-adds.
    static constexpr int kSolveRegRows = 8;  // n <= 256
    __device__ void lu_solve(double* b) {
        __syncthreads();
        if (n > 32 * kSolveRegRows) {
            lu_solve_smem(b);
            return;
        }
        if (threadIdx.x < 32) {
            const int lane = threadIdx.x;
            double r[kSolveRegRows];
#pragma unroll
            for (int j = 0; j < kSolveRegRows; ++j) {
                const int i = 32 * j + lane;
                r[j] = i < n ? b[v.perm[i]] : 0.0;
            }
#pragma unroll
            for (int j = 0; j < kSolveRegRows; ++j) {
                if (32 * j < n) {
                    const int kend = min(32, n - 32 * j);
                    for (int kk = 0; kk < kend; ++kk) {
                        const int k = 32 * j + kk;
                        const double bk = __shfl_sync(0xffffffffu, r[j], kk);
                        const double* colk = M + size_t(k) * n;
#pragma unroll
                        for (int jj = j; jj < kSolveRegRows; ++jj) {
                            if (32 * jj >= n) break;  // uniform: no issue slots for rows beyond n
                            const int i = 32 * jj + lane;
                            if (i > k && i < n) r[jj] = fma(-colk[i], bk, r[jj]);
                        }
                    }
                }
            }
#pragma unroll
            for (int j = kSolveRegRows - 1; j >= 0; --j) {
                if (32 * j < n) {
                    const int kend = min(32, n - 32 * j);
                    for (int kk = kend - 1; kk >= 0; --kk) {
                        const int k = 32 * j + kk;
                        const double bk = __shfl_sync(0xffffffffu, r[j], kk) * v.rdiag[k];
                        if (lane == kk) r[j] = bk;
                        const double* colk = M + size_t(k) * n;
#pragma unroll
                        for (int jj = 0; jj <= j; ++jj) {
                            const int i = 32 * jj + lane;
                            if (i < k) r[jj] = fma(-colk[i], bk, r[jj]);
                        }
                    }
                }
            }
#pragma unroll
            for (int j = 0; j < kSolveRegRows; ++j) {
                const int i = 32 * j + lane;
                if (i < n) b[i] = r[j];
            }
        }
        __syncthreads();
    }

    // The same in shared memory, for n > 256.
    __device__ void lu_solve_smem(double* b) {
        if (threadIdx.x < 32) {
            const int lane = threadIdx.x;
            if (lane == 0)
                for (int k = 0; k < n; ++k) {
                    const int p = v.piv[k];
                    if (p != k) {
                        const double tt = b[k];
                        b[k] = b[p];
                        b[p] = tt;
                    }
                }
            __syncwarp();
            for (int k = 0; k < n; ++k) {
                const double bk = b[k];
                const double* colk = M + size_t(k) * n;
                for (int i = k + 1 + lane; i < n; i += 32) b[i] = fma(-colk[i], bk, b[i]);
                __syncwarp();
            }
            for (int k = n - 1; k >= 0; --k) {
                const double* colk = M + size_t(k) * n;
                const double bk = b[k] * v.rdiag[k];
                __syncwarp();
                if (lane == 0) b[k] = bk;
                for (int i = lane; i < k; i += 32) b[i] = fma(-colk[i], bk, b[i]);
                __syncwarp();
            }
        }
        __syncthreads();
    }
};

// Where a point's Jacobian J and LU factors M (n^2 doubles each) live:
//   BDF_JM_SMEM   both in shared memory, next to the kinetics and BDF vectors;
//   BDF_M_SMEM    M in shared memory, J in a per-CTA slice of global memory
//                 (M is read by every Newton solve, J once per matrix update);
//                 to make room, the rates of progress and the saved Nordsieck
//                 array move to that slice as well;
//   BDF_JM_GLOBAL both in the global slice;
//   BDF_M_ROP_SMEM M and the rates of progress in shared memory, J and the
//                 saved Nordsieck array in the global slice (more points per
//                 SM than BDF_JM_SMEM, the species sums still on chip).
enum : int { BDF_JM_GLOBAL = 0, BDF_JM_SMEM = 1, BDF_M_SMEM = 2, BDF_M_ROP_SMEM = 3 };

struct BdfLayout {
    int mode;
    size_t smem_bytes;      // dynamic shared memory per CTA
    size_t global_doubles;  // global slice per CTA
};

constexpr size_t kBdfSmemBudget = 225 * 1024;  // leaves room for the static shared arrays

// The layout of a mode, or mode -1 for the default: the first of
// BDF_JM_SMEM, BDF_M_SMEM, BDF_JM_GLOBAL that fits. smem_bytes is 0 when the
// requested mode does not fit.
inline BdfLayout bdf_layout_of(const MechView& m, int mode) {
    const size_t n = size_t(m.S) + 2, nn = n * n;
    const size_t full = ChemSmem::doubles(m.S, m.R, m.n_tb, m.n_fo, true) + size_t(3) * m.n_fo + BdfSmem::doubles(int(n));
    const size_t lean = ChemSmem::doubles(m.S, m.R, m.n_tb, m.n_fo, true, false) + size_t(3) * m.n_fo +
                        BdfSmem::doubles(int(n), false);
    const size_t mrop_smem = ChemSmem::doubles(m.S, m.R, m.n_tb, m.n_fo, true) + size_t(3) * m.n_fo +
                             BdfSmem::doubles(int(n), false) + nn;
    const BdfLayout both{BDF_JM_SMEM, (full + 2 * nn) * sizeof(double), 0};
    const BdfLayout lu{BDF_M_SMEM, (lean + nn) * sizeof(double), nn + size_t(kQmax + 1) * n + size_t(2) * m.R};
    const BdfLayout none{BDF_JM_GLOBAL, full * sizeof(double), 2 * nn};
    const BdfLayout mrop{BDF_M_ROP_SMEM, mrop_smem * sizeof(double), nn + size_t(kQmax + 1) * n};
    const BdfLayout opts[4] = {both, lu, none, mrop};
    for (const BdfLayout& l : opts) {
        const bool fits = l.smem_bytes <= kBdfSmemBudget;
        if (mode < 0 && fits) return l;
        if (l.mode == mode) return fits ? l : BdfLayout{mode, 0, 0};
    }
    return none;
}

// The layout a launch uses: the one requested by the arguments or tuned for
// the mechanism (1 + mode; when it fits), else the default.
inline BdfLayout bdf_layout(const MechView& m, const SourceArgs& a) {
    const int req = a.bdf_layout ? a.bdf_layout - 1 : (m.bdf_layout ? m.bdf_layout - 1 : -1);
    if (req >= 0) {
        const BdfLayout l = bdf_layout_of(m, req);
        if (l.smem_bytes) return l;
    }
    return bdf_layout_of(m, -1);
}

// Carves one CTA's work areas: smem (dynamic shared memory), kc (its slice of
// the rate-constant cache), g (its global slice of bdf_layout().global_doubles).
template <int NT>
__device__ __forceinline__ void bdf_carve(BdfPoint<NT>& P, double* smem, double* kc, double* g, int mode) {
    const MechView& m = P.m;
    const int n = m.S + 2;
    const size_t nn = size_t(n) * n;
    const bool lean = mode == BDF_M_SMEM;            // rates of progress and saved Nordsieck array global
    const bool zs_global = lean || mode == BDF_M_ROP_SMEM;
    P.w.carve(smem, kc, m, true, lean ? g + nn + size_t(kQmax + 1) * n : nullptr);
    P.w.fo_F = smem + ChemSmem::doubles(m.S, m.R, m.n_tb, m.n_fo, true, !lean);
    P.w.fo_pr = P.w.fo_F + m.n_fo;
    P.w.fo_dF = P.w.fo_pr + m.n_fo;
    P.v.carve(P.w.fo_dF + m.n_fo, n, zs_global ? g + nn : nullptr);
    double* after = P.w.fo_dF + m.n_fo + BdfSmem::doubles(n, !zs_global);
    if (mode == BDF_JM_SMEM) {
        P.J = after;
        P.M = after + nn;
    } else if (zs_global) {
        P.J = g;
        P.M = after;
    } else {
        P.J = g;
        P.M = g + nn;
    }
    P.n = n;
    P.S = m.S;
}

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
    auto copy_z = [&](const ZArr& dst, const ZArr& src, int q) {
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
    bool restart_pending = false;  // for the tape: a q = 1 restart since the last accepted step
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
                {
                    // M = I - gamma J, column-major; (row, column) of element e advanced without a division
                    int c = tid / n, r = tid - c * n;
                    for (size_t e = tid; e < size_t(n) * n; e += NT) {
                        P.M[e] = (r == c ? 1.0 : 0.0) - gamma * P.J[e];
                        r += NT;
                        while (r >= n) {
                            r -= n;
                            ++c;
                        }
                    }
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
                    restart_pending = true;
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
        if (P.tape && nst <= a.tape_cap) {
            double* rec = P.tape + kTapeHeader + int64_t(nst - 1) * (n + 4);
            if (tid == 0) {
                rec[0] = t;
                rec[1] = h;
                rec[2] = q;
                rec[3] = restart_pending ? 1.0 : 0.0;
            }
            for (int i = tid; i < n; i += NT) rec[4 + i] = v.z[0][i];
        }
        restart_pending = false;
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
    if (P.tape && tid == 0) {
        P.tape[0] = nst < a.tape_cap ? nst : a.tape_cap;
        P.tape[1] = q;
        P.tape[2] = t;
        P.tape[3] = nst > a.tape_cap ? 1.0 : 0.0;
        P.tape[4] = status;
        P.tape[5] = tf;
    }
    stats[0] = nst;
    stats[1] = P.nfe;
    stats[2] = nef_total + ncf_total;
    stats[3] = nje;
    return status;
}

template <int NT>
__global__ void __maxnreg__(168) k_source_bdf(const __grid_constant__ MechView m,
                                                  const __grid_constant__ SourceArgs a, int* counter, const int* order,
                                                  double* kcache, double* jm, size_t jm_stride, int jm_mode) {
    extern __shared__ double smem[];
    __shared__ int next_point;
    const int n = m.S + 2;
    BdfPoint<NT> P(m);
    bdf_carve(P, smem, kcache + size_t(blockIdx.x) * ChemSmem::global_doubles(m), jm + size_t(blockIdx.x) * jm_stride,
              jm_mode);
    P.a = &a;
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
        P.tape = a.tape ? a.tape + size_t(j) * a.tape_stride : nullptr;
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
    const size_t per = bdf_layout(m, a).smem_bytes;
    EMBER_CHECK_ARG(per <= 227 * 1024, "mechanism too large for the BDF shared-memory work area (%zu B)", per);
    EMBER_TRY(raise_dynamic_smem(reinterpret_cast<const void*>(k_source_bdf<NT>), per));
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
    *bytes = Scratch::rounded(sizeof(double) * size_t(blocks) * ChemSmem::global_doubles(m)) +
             Scratch::rounded(sizeof(double) * size_t(blocks) * bdf_layout(m, a).global_doubles) +
             Scratch::rounded(sizeof(int) * 64) + Scratch::rounded(sizeof(int) * size_t(a.n));
    return EMBER_OK;
}

int source_bdf_threads(const MechView& m, const SourceArgs& a) {
    for (int c : kBdfThreadChoices)
        if (a.threads == c) return c;
    if (m.bdf_threads) return m.bdf_threads;
    return chem_threads_for(m.S);
}

int source_bdf_layout(const MechView& m, const SourceArgs& a) { return 1 + bdf_layout(m, a).mode; }

bool source_bdf_layout_fits(const MechView& m, int layout) {
    return layout >= 1 && layout <= 4 && bdf_layout_of(m, layout - 1).smem_bytes != 0;
}

int source_bdf_scratch_bytes(const MechView& m, const SourceArgs& a, size_t* bytes) {
    switch (source_bdf_threads(m, a)) {
        case 32: return bdf_scratch_nt<32>(m, a, bytes);
        case 64: return bdf_scratch_nt<64>(m, a, bytes);
        case 128: return bdf_scratch_nt<128>(m, a, bytes);
        case 160: return bdf_scratch_nt<160>(m, a, bytes);
        default: return bdf_scratch_nt<256>(m, a, bytes);
    }
}

template <int NT>
static int launch_bdf_nt(const MechView& m, const SourceArgs& a, int* counter, Scratch& sc, cudaStream_t st) {
    size_t per = 0;
    int blocks = 0;
    EMBER_TRY(bdf_config<NT>(m, a, &per, &blocks));
    double *kcache = nullptr, *jm = nullptr;
    EMBER_TRY(sc.alloc(&kcache, size_t(blocks) * ChemSmem::global_doubles(m)));
    const BdfLayout lay = bdf_layout(m, a);
    EMBER_TRY(sc.alloc(&jm, size_t(blocks) * lay.global_doubles));
    int* order = nullptr;
    EMBER_TRY(make_work_order(a, sc, st, &order));
    k_source_bdf<NT><<<blocks, NT, per, st>>>(m, a, counter, order, kcache, jm, lay.global_doubles, lay.mode);
    EMBER_CUDA_TRY(cudaGetLastError());
    return EMBER_OK;
}

// ------------------------------------------------------------------ adjoint --
//
// Discrete adjoint of the BDF integration of one point, replayed backwards
// over the tape of its accepted steps. Each step is linearised with the step
// sizes, orders and the converged corrector held fixed:
//   predictor   z_p = Pascal(z)                         (transpose: reversed sums)
//   corrector   acor = gamma f(z_p0 + acor) - z_p1 / l1, so
//               (I - gamma J) d acor = gamma J d z_p0 - d z_p1 / l1 + gamma f_p d p
//   update      z_j = z_pj + l_j acor,  order increase  z_{q+1} = l_q/(q+1) acor
//   rescaling   z_j *= (h_next/h)^j, or a q = 1 restart z = [z0, h f(z0)]
//   start       z = [y0, h0 f(y0)],  end  y(tf) = sum_j z_j s^j.
// J is the analytic Jacobian (exact falloff derivative, forward-difference
// temperature column) at the step's end state, recomputed from the tape; the
// transposed solve reuses the LU of I - gamma J. The gradient with respect to
// ln(multiplier_i) of every reaction is accumulated per point.
template <int NT>
__global__ void __maxnreg__(168) k_source_bdf_adjoint(const __grid_constant__ MechView m,
                                                          const __grid_constant__ SourceArgs a, int* counter,
                                                          double* kcache,
                                                          double* jm, size_t jm_stride, int jm_mode,
                                                          const double* __restrict__ ybar_out,
                                                          double* __restrict__ ybar_in, double* __restrict__ pbar,
                                                          int* __restrict__ adj_status) {
    extern __shared__ double smem[];
    __shared__ int next_point;
    const int n = m.S + 2;
    BdfPoint<NT> P(m);
    bdf_carve(P, smem, kcache + size_t(blockIdx.x) * ChemSmem::global_doubles(m), jm + size_t(blockIdx.x) * jm_stride,
              jm_mode);
    P.a = &a;
    P.cachedT = __longlong_as_double(0x7ff8000000000000LL);
    P.tape = nullptr;
    BdfSmem& v = P.v;
    const ZArr zb = v.z;  // adjoint of the Nordsieck array
    const int tid = threadIdx.x;
    const double t_start = a.t_start_dev ? *a.t_start_dev : a.t_start;
    for (;;) {
        if (tid == 0) {
            const int slot = atomicAdd(counter, 1);
            next_point = slot < a.n ? slot : a.n;
        }
        __syncthreads();
        const int j = next_point;
        __syncthreads();
        if (j >= a.n) break;
        const double* tape = a.tape + size_t(j) * a.tape_stride;
        P.split = a.split ? a.split + size_t(j) * n : nullptr;
        P.x = a.x ? a.x[j] : 0.0;
        double* pb = pbar + size_t(j) * m.R;
        for (int i = tid; i < m.R; i += NT) pb[i] = 0.0;
        const int N = static_cast<int>(tape[0]);
        const int fstat = static_cast<int>(tape[4]);
        int status = 0;
        if (tape[3] != 0.0) status = -30;  // tape overflow
        if (fstat != 0) status = fstat;
        if (N < 1 && status == 0) status = -31;
        if (status != 0) {
            for (int i = tid; i < n; i += NT) ybar_in[size_t(j) * n + i] = 0.0;
            if (tid == 0) adj_status[j] = status;
            __syncthreads();
            continue;
        }
        const int rec_len = n + 4;
        const double tf = tape[5];
        const double* last = tape + kTapeHeader + int64_t(N - 1) * rec_len;
        const int q_final = static_cast<int>(tape[1]);
        {
            const double s = (tf - tape[2]) / last[1];
            for (int jj = 0; jj <= kQmax + 1; ++jj)
                for (int i = tid; i < n; i += NT) zb[jj][i] = 0.0;
            __syncthreads();
            double sp = 1.0;
            for (int jj = 0; jj <= q_final; ++jj, sp *= s)
                for (int i = tid; i < n; i += NT) zb[jj][i] = sp * ybar_out[size_t(j) * n + i];
        }
        int q_next = q_final;
        double h_next = last[1];
        bool restart_next = false;
        double l[kQmax + 2];
        for (int r = N - 1; r >= 0 && status == 0; --r) {
            const double* rec = tape + kTapeHeader + int64_t(r) * rec_len;
            const double t_r = rec[0], h_r = rec[1];
            const int q_r = static_cast<int>(rec[2]);
            const bool flag_r = rec[3] != 0.0;
            for (int i = tid; i < n; i += NT) v.y[i] = rec[4 + i];
            __syncthreads();
            P.f(t_start + t_r, v.y, v.ft);
            P.jacobian(t_start + t_r, v.y, v.ft);
            // v.acorp: the vector whose J^T and f_p^T products this step adds to zb0 and pbar
            if (restart_next) {
                for (int i = tid; i < n; i += NT) {
                    v.acorp[i] = h_next * zb[1][i];
                    for (int jj = 1; jj <= kQmax + 1; ++jj) zb[jj][i] = 0.0;
                }
            } else {
                const double ratio = h_next / h_r;
                double sc = ratio;
                for (int jj = 1; jj <= q_next; ++jj, sc *= ratio)
                    for (int i = tid; i < n; i += NT) zb[jj][i] *= sc;
                for (int i = tid; i < n; i += NT) v.acorp[i] = 0.0;
            }
            __syncthreads();
            bdf_l(q_r, l);
            for (int i = tid; i < n; i += NT) {
                double ab = 0.0;
                if (!restart_next && q_next == q_r + 1) {
                    ab = (l[q_r] / (q_r + 1)) * zb[q_r + 1][i];
                    zb[q_r + 1][i] = 0.0;
                }
                for (int jj = 0; jj <= q_r; ++jj) ab = fma(l[jj], zb[jj][i], ab);
                v.bb[i] = ab;
            }
            const double gamma = h_r / l[1];
            const double rl1 = 1.0 / l[1];
            for (size_t e = tid; e < size_t(n) * n; e += NT) {
                const int c = static_cast<int>(e / n), rr = static_cast<int>(e - size_t(c) * n);
                P.M[e] = (rr == c ? 1.0 : 0.0) - gamma * P.J[e];
            }
            __syncthreads();
            if (P.lu_factor() != 0) {
                status = -32;  // singular iteration matrix
                break;
            }
            P.lu_solve_transpose(v.bb);  // w
            for (int i = tid; i < n; i += NT) {
                v.acorp[i] = fma(gamma, v.bb[i], v.acorp[i]);
                zb[1][i] = fma(-rl1, v.bb[i], zb[1][i]);
            }
            __syncthreads();
            P.jacobian_transpose_times(v.acorp, zb[0], true);
            P.f(t_start + t_r, v.y, v.ft);  // rates at the step's end state again (the FD column moved them)
            P.multiplier_vjp(v.acorp, pb);
            __syncthreads();
            // predictor transpose: the forward ran z[j-1] += z[j] for k = 1..q, j = q..k
            for (int k = q_r; k >= 1; --k)
                for (int jj = k; jj <= q_r; ++jj)
                    for (int i = tid; i < n; i += NT) zb[jj][i] += zb[jj - 1][i];
            __syncthreads();
            q_next = q_r;
            h_next = h_r;
            restart_next = flag_r;
        }
        if (status == 0) {
            // z at the start of the first step: [y0, h0 f(y0)]
            const double* y0 = a.state_in + size_t(j) * n;
            for (int i = tid; i < n; i += NT) {
                v.y[i] = y0[i];
                v.acorp[i] = h_next * zb[1][i];
            }
            __syncthreads();
            P.f(t_start, v.y, v.ft);
            P.jacobian(t_start, v.y, v.ft);
            P.jacobian_transpose_times(v.acorp, zb[0], true);
            P.f(t_start, v.y, v.ft);
            P.multiplier_vjp(v.acorp, pb);
            for (int i = tid; i < n; i += NT) ybar_in[size_t(j) * n + i] = zb[0][i];
        } else {
            for (int i = tid; i < n; i += NT) ybar_in[size_t(j) * n + i] = 0.0;
        }
        if (tid == 0) adj_status[j] = status;
        __syncthreads();
    }
}

template <int NT>
static int launch_bdf_adjoint_nt(const MechView& m, const SourceArgs& a, int* counter, const double* ybar_out,
                                 double* ybar_in, double* pbar, int* adj_status, Scratch& sc, cudaStream_t st) {
    size_t per = 0;
    int blocks = 0;
    EMBER_TRY(bdf_config<NT>(m, a, &per, &blocks));
    EMBER_TRY(raise_dynamic_smem(reinterpret_cast<const void*>(k_source_bdf_adjoint<NT>), per));
    double *kcache = nullptr, *jm = nullptr;
    EMBER_TRY(sc.alloc(&kcache, size_t(blocks) * ChemSmem::global_doubles(m)));
    const BdfLayout lay = bdf_layout(m, a);
    EMBER_TRY(sc.alloc(&jm, size_t(blocks) * lay.global_doubles));
    k_source_bdf_adjoint<NT><<<blocks, NT, per, st>>>(m, a, counter, kcache, jm, lay.global_doubles, lay.mode,
                                                      ybar_out, ybar_in, pbar, adj_status);
    EMBER_CUDA_TRY(cudaGetLastError());
    return EMBER_OK;
}

// Gradient, at each point's state y = [U, T, Y] (Y >= 0), of
//   psi = gq * qdot + gcp * cp + gT * T,
// qdot = -sum_k wdot_k h_k and cp the mass heat capacity of the normalised
// state (FlameSolver::calculateQdot, setState_TPY). The NoNorm derivatives
// come from the analytic Jacobian of the source right-hand side with the
// split constant and igniter off: d qdot = rho cp d(dT/dt) + dT/dt d(rho cp);
// rho cp = (p/T) B/A and cp = R B with A = sum_k Y_k/W_k, B = sum_k
// Y_k cp_k/(R W_k); then the normalisation Y/sum(Y) is projected out. Also
// d psi / d ln(multiplier_i) = gq * (-sum_k nu_ki h_k) r_i, per point.
template <int NT>
__global__ void __maxnreg__(168) k_objective_vjp(const __grid_constant__ MechView m,
                                                     const __grid_constant__ SourceArgs a, int n_pts,
                                                     const double* __restrict__ state, const double* __restrict__ gq,
                                                     const double* __restrict__ gcp, const double* __restrict__ gT,
                                                     int* counter, double* kcache, double* jm, size_t jm_stride, int jm_mode,
                                                     double* __restrict__ ybar, double* __restrict__ pbar) {
    extern __shared__ double smem[];
    __shared__ int next_point;
    const int n = m.S + 2;
    BdfPoint<NT> P(m);
    bdf_carve(P, smem, kcache + size_t(blockIdx.x) * ChemSmem::global_doubles(m), jm + size_t(blockIdx.x) * jm_stride,
              jm_mode);
    P.a = &a;
    P.cachedT = __longlong_as_double(0x7ff8000000000000LL);
    P.tape = nullptr;
    P.split = nullptr;
    P.x = 0.0;
    BdfSmem& v = P.v;
    const int tid = threadIdx.x;
    const int S = m.S;
    for (;;) {
        if (tid == 0) {
            const int slot = atomicAdd(counter, 1);
            next_point = slot < n_pts ? slot : n_pts;
        }
        __syncthreads();
        const int j = next_point;
        __syncthreads();
        if (j >= n_pts) break;
        for (int i = tid; i < n; i += NT) v.y[i] = state[size_t(j) * n + i];
        __syncthreads();
        P.f(0.0, v.y, v.ft);
        P.jacobian(0.0, v.y, v.ft);
        const double T = v.y[1];
        const double rho = P.rho, cp = P.cp, rc = rho * cp;
        const double A = 1.0 / P.w.mmw;
        const double *yv = v.y, *cpR = P.w.cpR;
        const double B = block_sum<NT>(P.w.red, S, [&](int k, double q) { return fma(yv[2 + k] * m.rW[k], cpR[k], q); });
        const double dB = block_sum<NT>(P.w.red, S, [&](int k, double q) {
            const int r = (T <= m.tmid[k]) ? 0 : 1;
            const double* c = m.nasa + 14 * k + 7 * r;
            const double dcp = fma(fma(fma(4.0 * c[4], T, 3.0 * c[3]), T, 2.0 * c[2]), T, c[1]);
            return fma(yv[2 + k] * m.rW[k], dcp, q);
        });
        const double ysum = block_sum<NT>(P.w.red, S, [&](int k, double q) { return q + yv[2 + k]; });
        const double p = a.pressure, dTdt = v.ft[1];
        const double g_q = gq[j], g_cp = gcp ? gcp[j] : 0.0, g_T = gT ? gT[j] : 0.0;
        // d psi / d y_c (NoNorm) into v.bb
        for (int c = tid; c < n; c += NT) {
            double drc, dcpc;
            if (c == 0) {
                drc = 0.0;
                dcpc = 0.0;
            } else if (c == 1) {
                drc = -rc / T + (p / (T * A)) * dB;
                dcpc = kGasConstant * dB;
            } else {
                const int mm = c - 2;
                drc = (p / T) * ((P.w.cpR[mm] * m.rW[mm]) / A - (B * m.rW[mm]) / (A * A));
                dcpc = kGasConstant * (P.w.cpR[mm] * m.rW[mm]);
            }
            const double dq = fma(rc, P.J[size_t(c) * n + 1], dTdt * drc);
            v.bb[c] = g_q * dq + g_cp * dcpc + (c == 1 ? g_T : 0.0);
        }
        __syncthreads();
        // project out the normalisation of Y
        const double* bb = v.bb;
        const double pr = block_sum<NT>(P.w.red, S, [&](int k, double q) { return fma(yv[2 + k], bb[2 + k], q); });
        for (int c = tid; c < n; c += NT) {
            double g = v.bb[c];
            if (c >= 2) g = (g - pr / ysum) / ysum;
            ybar[size_t(j) * n + c] = g;
        }
        // rate multipliers (the FD column of the Jacobian moved the rates: evaluate again)
        P.f(0.0, v.y, v.ft);
        double* pb = pbar + size_t(j) * m.R;
        for (int i = tid; i < m.R; i += NT) {
            const double r = P.w.ropf[i] - P.w.ropr[i];
            const int4 st = m.stoich[i];
            const int sp[8] = {unpack_lo(st.x), unpack_hi(st.x), unpack_lo(st.y), unpack_hi(st.y),
                               unpack_lo(st.z), unpack_hi(st.z), unpack_lo(st.w), unpack_hi(st.w)};
            double eh = 0.0;
#pragma unroll
            for (int o = 0; o < 8; ++o) {
                if (sp[o] == 0xffff) continue;
                eh = fma(o < 4 ? -1.0 : 1.0, P.w.hk[sp[o]], eh);
            }
            pb[i] = g_q * (-eh * r);
        }
        __syncthreads();
    }
}

template <int NT>
static int launch_objective_vjp_nt(const MechView& m, const SourceArgs& a, int n_pts, const double* state,
                                   const double* gq, const double* gcp, const double* gT, double* ybar, double* pbar,
                                   Scratch& sc, cudaStream_t st) {
    size_t per = 0;
    int blocks = 0;
    SourceArgs b = a;
    b.n = n_pts;
    EMBER_TRY(bdf_config<NT>(m, b, &per, &blocks));
    EMBER_TRY(raise_dynamic_smem(reinterpret_cast<const void*>(k_objective_vjp<NT>), per));
    double *kcache = nullptr, *jm = nullptr;
    int* counter = nullptr;
    EMBER_TRY(sc.alloc(&kcache, size_t(blocks) * ChemSmem::global_doubles(m)));
    const BdfLayout lay = bdf_layout(m, a);
    EMBER_TRY(sc.alloc(&jm, size_t(blocks) * lay.global_doubles));
    EMBER_TRY(sc.alloc(&counter, 1));
    EMBER_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(int), st));
    k_objective_vjp<NT><<<blocks, NT, per, st>>>(m, b, n_pts, state, gq, gcp, gT, counter, kcache, jm,
                                                 lay.global_doubles, lay.mode, ybar, pbar);
    EMBER_CUDA_TRY(cudaGetLastError());
    return EMBER_OK;
}

int launch_objective_vjp(const MechView& m, const SourceArgs& a, int n_pts, const double* state, const double* gq,
                         const double* gcp, const double* gT, double* ybar, double* pbar, Scratch& sc,
                         cudaStream_t st) {
    switch (source_bdf_threads(m, a)) {
        case 32: return launch_objective_vjp_nt<32>(m, a, n_pts, state, gq, gcp, gT, ybar, pbar, sc, st);
        case 64: return launch_objective_vjp_nt<64>(m, a, n_pts, state, gq, gcp, gT, ybar, pbar, sc, st);
        case 128: return launch_objective_vjp_nt<128>(m, a, n_pts, state, gq, gcp, gT, ybar, pbar, sc, st);
        case 160: return launch_objective_vjp_nt<160>(m, a, n_pts, state, gq, gcp, gT, ybar, pbar, sc, st);
        default: return launch_objective_vjp_nt<256>(m, a, n_pts, state, gq, gcp, gT, ybar, pbar, sc, st);
    }
}

int launch_source_bdf_adjoint(const MechView& m, const SourceArgs& a, int* counter, const double* ybar_out,
                              double* ybar_in, double* pbar, int* adj_status, Scratch& sc, cudaStream_t st) {
    switch (source_bdf_threads(m, a)) {
        case 32: return launch_bdf_adjoint_nt<32>(m, a, counter, ybar_out, ybar_in, pbar, adj_status, sc, st);
        case 64: return launch_bdf_adjoint_nt<64>(m, a, counter, ybar_out, ybar_in, pbar, adj_status, sc, st);
        case 128: return launch_bdf_adjoint_nt<128>(m, a, counter, ybar_out, ybar_in, pbar, adj_status, sc, st);
        case 160: return launch_bdf_adjoint_nt<160>(m, a, counter, ybar_out, ybar_in, pbar, adj_status, sc, st);
        default: return launch_bdf_adjoint_nt<256>(m, a, counter, ybar_out, ybar_in, pbar, adj_status, sc, st);
    }
}

int launch_source_bdf(const MechView& m, const SourceArgs& a, int* counter, Scratch& sc, cudaStream_t st) {
    switch (source_bdf_threads(m, a)) {
        case 32: return launch_bdf_nt<32>(m, a, counter, sc, st);
        case 64: return launch_bdf_nt<64>(m, a, counter, sc, st);
        case 128: return launch_bdf_nt<128>(m, a, counter, sc, st);
        case 160: return launch_bdf_nt<160>(m, a, counter, sc, st);
        default: return launch_bdf_nt<256>(m, a, counter, sc, st);
    }
}

}  // namespace ember

namespace ember {
namespace {

// Sum of the per-point gradients [n][R] over points, in point order.
__global__ void k_sum_points(int n, int R, const double* __restrict__ rows, double* __restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < R; i += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int j = 0; j < n; ++j) s += rows[size_t(j) * R + i];
        out[i] = s;
    }
}

}  // namespace

int source_bdf_adjoint_run(const MechView& m, SourceArgs a, int tape_cap, const double* ybar_out, double* ybar_in,
                           double* lnk_bar, double* lnk_bar_points, int* adj_status, Scratch& sc, cudaStream_t st) {
    const int n = m.S + 2;
    a.tape_cap = tape_cap;
    a.tape_stride = bdf_tape_doubles(n, tape_cap);
    EMBER_TRY(sc.alloc(&a.tape, size_t(a.n) * a.tape_stride));
    int* counter = nullptr;
    EMBER_TRY(sc.alloc(&counter, 2));
    EMBER_CUDA_TRY(cudaMemsetAsync(counter, 0, 2 * sizeof(int), st));
    EMBER_TRY(launch_source_bdf(m, a, counter, sc, st));
    double* rows = lnk_bar_points;
    if (!rows) EMBER_TRY(sc.alloc(&rows, size_t(a.n) * std::max(m.R, 1)));
    EMBER_TRY(launch_source_bdf_adjoint(m, a, counter + 1, ybar_out, ybar_in, rows, adj_status, sc, st));
    if (lnk_bar && m.R > 0)
        k_sum_points<<<blocks_for(m.R, 128), 128, 0, st>>>(a.n, m.R, rows, lnk_bar);
    EMBER_CUDA_TRY(cudaGetLastError());
    return EMBER_OK;
}

}  // namespace ember

using namespace ember;

extern "C" int ember_source_adjoint(ember_mech m, int n, const double* state_in, const double* split_const,
                                    const double* dt, double t_start, const double* x,
                                    const ember_source_options* opts, const double* state_bar, int tape_cap,
                                    double* state_out, int* status, double* state_in_bar, double* lnk_bar, int mem,
                                    void* stream) {
    EMBER_CHECK_ARG(m != nullptr, "null mechanism");
    EMBER_CHECK_ARG(n > 0 && state_in && dt && state_bar && state_out && status && state_in_bar,
                    "need points, state_in, dt, state_bar, state_out, status and state_in_bar");
    EMBER_CHECK_ARG(mem == EMBER_MEM_HOST || mem == EMBER_MEM_DEVICE, "bad mem flag %d", mem);
    EMBER_CHECK_ARG(tape_cap >= 0 && tape_cap <= (1 << 20), "bad tape_cap %d", tape_cap);
    EMBER_TRY(source_check_options(opts));
    EMBER_TRY(ensure_device());
    if (tape_cap == 0) tape_cap = 1024;
    cudaStream_t st = as_stream(stream);
    Scratch sc(st);
    const int nv = m->S + 2;
    const double *d_in, *d_split, *d_dt, *d_x, *d_bar;
    EMBER_TRY(stage_in(sc, state_in, size_t(n) * nv, mem, st, &d_in));
    EMBER_TRY(stage_in(sc, split_const, size_t(n) * nv, mem, st, &d_split));
    EMBER_TRY(stage_in(sc, dt, n, mem, st, &d_dt));
    EMBER_TRY(stage_in(sc, x, n, mem, st, &d_x));
    EMBER_TRY(stage_in(sc, state_bar, size_t(n) * nv, mem, st, &d_bar));
    double *d_out, *d_inbar, *d_lnk = nullptr;
    int *d_status, *d_adj;
    EMBER_TRY(stage_buffer(sc, state_out, size_t(n) * nv, mem, &d_out));
    EMBER_TRY(stage_buffer(sc, status, n, mem, &d_status));
    EMBER_TRY(stage_buffer(sc, state_in_bar, size_t(n) * nv, mem, &d_inbar));
    EMBER_TRY(stage_buffer(sc, lnk_bar, size_t(std::max(m->R, 1)), mem, &d_lnk));
    EMBER_TRY(sc.alloc(&d_adj, n));
    SourceArgs a = make_source_args(opts, n, d_in, d_split, d_dt, t_start, d_x, d_out, d_status, nullptr);
    EMBER_TRY(source_bdf_adjoint_run(m->view, a, tape_cap, d_bar, d_inbar, d_lnk, nullptr, d_adj, sc, st));
    // status: the forward's, or the adjoint's when the forward succeeded
    EMBER_CUDA_TRY(cudaMemcpyAsync(d_status, d_adj, sizeof(int) * n, cudaMemcpyDeviceToDevice, st));
    EMBER_TRY(stage_out(state_out, d_out, size_t(n) * nv, mem, st));
    EMBER_TRY(stage_out(status, d_status, n, mem, st));
    EMBER_TRY(stage_out(state_in_bar, d_inbar, size_t(n) * nv, mem, st));
    if (lnk_bar) EMBER_TRY(stage_out(lnk_bar, d_lnk, size_t(m->R), mem, st));
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
