// Warp-parallel diffusion stage: one warp per (flame, variable) system.
//
// The stage is the one of tridiag.cu -- DiffusionSystem rows
// (src/diffusionSystem.cpp:10-76), the step size of
// FlameSolver::setDiffusionSolverState (src/flameSolver.cpp:702-718) and
// TridiagonalIntegrator's 8 x BDF1 first step and BDF2 later steps
// (src/integrator.cpp:37-47, 133-204) -- with the sequential Thomas algorithm
// split into 32 chunks, one per lane, joined by exact prefix scans:
//
//  * factorisation: the pivots den_i = b'_i - a_i lu_c_{i-1} (b' = b - shift)
//    follow a Moebius recurrence. It is carried in the variable u = 1 + lu_c,
//    in which a diffusion row (b = -(a + c) - x_i, x_i >= 0 the row's excess
//    over a conservative row, zero except at a wall-flux boundary) gives
//        u_i = (sigma_i + a_i u_{i-1}) / (c_i + sigma_i + a_i u_{i-1}),
//        den_i = -(c_i + sigma_i + a_i u_{i-1}),  sigma_i = shift + x_i,
//    a map with a positive matrix [[a, sigma], [a, c + sigma]]. Each lane
//    multiplies the matrices of its chunk, a warp scan of the 2x2 products
//    gives every lane the u entering its chunk, and the lane runs the
//    recurrence. Every term is positive, so nothing cancels: the shift is
//    never added to a diagonal that can be 1e17 times larger (where the
//    reference's b - shift loses it), and products of many nearly-parabolic
//    maps (a ~ c >> shift, lu_c -> -1) stay accurate. Against the same
//    recurrences in extended precision this factorisation is accurate to
//    ~1e-14 of max|y| even on grids whose spacing varies by 1e4 or more,
//    where the reference's own rounding error reaches 1e-11.
//  * forward sweep d_i = rho_i - alpha_i d_{i-1} and back substitution
//    y_i = d_i - c'_i y_{i+1} are affine in the value entering the chunk: a
//    lane sweeps its chunk from zero, a scan of the affine maps gives the
//    entering values, and the next pass adds G_i * carry (forward) or
//    H_i * carry (backward), G and H being the chunk's running products of
//    -alpha and -c'. That correction rides along with the following sweep, so
//    a sub-step is two passes over the chunk and five FP64 operations a point.
//
// FP64 throughput bounds this kernel on GB300: each SM sub-partition issues
// one FP64 warp instruction per 64 cycles whatever the number of active lanes
// (about 1.7 FP64 lanes per clock per SM), so the work per point is kept
// small: the geometric factors of the rows (0.5 / (dlj r^alpha) and
// r_{j+1/2}^alpha / hh) are computed once per grid point and shared by the
// variables of a flame; 1/den is computed once per factorisation and folded
// into alpha = a/den, c' = c/den, e = -s/den and kappa = -k/den; a sub-step
// then costs one fma for the right-hand side, one per sweep and one per carry
// correction.
//
// Lane groups: a system of N points is split over G = 1, 2, 4 or 8 warps (the
// fewest that give each lane at most kPointsPerLane points), so that a lane's
// chunk, its sequential chain and the scan overhead per point stay about the
// same for every N. The warps of a group combine their scans through shared
// memory and a named barrier (bar.sync 1+group, 32 G threads). A CTA of eight
// warps takes one task at a time from an atomic counter: one system of eight
// warps, or two of four, four of two, eight of one, largest systems first.
// With short chunks the live workspace of the resident warps (about
// kPointsPerLane x 64 bytes per lane) stays inside L2, which the 16 passes
// over it per stage need: with one warp per system the chunks of the largest
// systems were 125 points long and the live workspace spilled to DRAM.
//
// Workspace: per system, m = ceil(N / 32G) rows of 8 slots x 32G lanes
// (alpha, c', e, kappa, G, H, state, y_prev), point j of a lane at row j, so
// that the 32 lanes of a warp touch one contiguous 256-byte segment per slot.
#include "common.cuh"
#include "tridiag.cuh"

#include <algorithm>
#include <cstdlib>
#include <numeric>
#include <vector>

namespace ember {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kSlots = 8;
constexpr int kCtaWarps = 8;  // warps per CTA (one task)
constexpr int kTaskInts = 1 + kCtaWarps;
enum : int { S_ALPHA = 0, S_CP = 1, S_E = 2, S_KAPPA = 3, S_G = 4, S_H = 5, S_W = 6, S_YP = 7 };

struct WarpDiffView {
    int n_systems;
    int n_tasks;
    const DiffSysInfo* info;
    const int* tasks;         // [n_tasks][1 + kCtaWarps]: G, then 8/G systems (-1: none), largest first
    const int64_t* ws_off;    // first workspace double of each system
    const double* x;
    const double2* geo;       // per grid point: (0.5 / (dlj r^alpha), r_{j+1/2}^alpha / hh)
    const double* B;
    const double* D;
    const double* split_const;
    const double* h;
    const double* wall_const;
    const double* y_inf;
    double* y;
    double* ws;
    int* status;
    unsigned int* counter;
    StageTime tm;
    double mult, gdt;
};

// Geometric factors of the interior rows, one grid point per thread:
// c1_j = B_j * g1_j and c2_j = (D_j + D_{j+1}) * g2_j for 1 <= j <= N-2.
__global__ void k_diffusion_geometry(const DiffSysInfo* __restrict__ info, int n_flames, int n_vars,
                                     const double* __restrict__ x, double2* __restrict__ geo) {
    for (int f = blockIdx.y; f < n_flames; f += gridDim.y) {
        const DiffSysInfo fi = info[int64_t(f) * n_vars];
        const double* xf = x + fi.grid_off;
        for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < fi.n; j += gridDim.x * blockDim.x) {
            double g1 = 0.0, g2 = 0.0;
            if (j >= 1 && j <= fi.n - 2) {
                const double dlj = 0.5 * (xf[j + 1] - xf[j - 1]);
                g1 = 0.5 / (dlj * grid_pow(xf[j], fi.alpha));
                g2 = grid_pow(0.5 * (xf[j] + xf[j + 1]), fi.alpha) / (xf[j + 1] - xf[j]);
            }
            geo[fi.grid_off + j] = make_double2(g1, g2);
        }
    }
}

__device__ __forceinline__ int exponent_field(double v) { return (__double2hiint(v) >> 20) & 0x7ff; }

// Scale a 2x2 matrix by the power of two that brings its largest entry into
// [1, 2): exact, and the Moebius map it stands for is unchanged.
__device__ __forceinline__ void normalize(double& m11, double& m12, double& m21, double& m22) {
    const int e = max(max(exponent_field(m11), exponent_field(m12)), max(exponent_field(m21), exponent_field(m22)));
    const int f = min(max(2046 - e, 1), 2046);
    const double s = __hiloint2double(f << 20, 0);
    m11 *= s;
    m12 *= s;
    m21 *= s;
    m22 *= s;
}

__device__ __forceinline__ double shfl_up(double v, int o) { return __shfl_up_sync(kFull, v, o); }
__device__ __forceinline__ double shfl_down(double v, int o) { return __shfl_down_sync(kFull, v, o); }

// One system as seen by one lane of its group.
struct LaneChunk {
    int N, i0, cnt;       // global index of the chunk's first point, points in the chunk
    int stride;           // lanes of the group (32 G)
    int64_t base;         // workspace offset of row 0, this lane
    __device__ double& at(double* ws, int j, int slot) const {
        return ws[base + (int64_t(j) * kSlots + slot) * stride];
    }
};

// The warps of one system. Shared memory: 8 doubles per warp of the CTA,
// sh[w * 8 + ...]: [0..3] chunk-matrix totals and reductions, [4] forward
// totals, [5] backward totals, [6] forward slope total, [7] backward slope
// total of warp w.
struct Group {
    int G;       // warps
    int wl;      // this warp's index in the group
    int lane;
    int w0;      // the group's first warp in the CTA
    int bar;     // named barrier id
    double* sh;  // the CTA's shared slots
    __device__ void sync() const {
        if (G > 1) asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(G * 32) : "memory");
        else __syncwarp();
    }
    __device__ double* slot(int j) const { return sh + (w0 + j) * 8; }
    __device__ double* mine() const { return slot(wl); }
};

// Row i of A and k_i as (a_i, c_i, x_i = -(a_i + b_i + c_i), k_i): interior
// rows from the shared geometric factors (x = 0 by construction), the rows
// next to the boundaries from diffusion_row().
struct RowCtx {
    int N, alpha, left_bc, right_bc;
    const double* x;
    const double2* geo;
    const double* B;
    const double* D;
    const double* S;
    double wall_const, y_inf;
};

__device__ __forceinline__ void boundary_row(const RowCtx& r, int i, double& a, double& c, double& xs, double& k) {
    const DiffRow row = diffusion_row(i, r.N, r.x, r.alpha, r.left_bc, r.right_bc, r.B, r.D, r.wall_const);
    a = row.a;
    c = row.c;
    // b = -(a + c) exactly in every boundary row but the wall-flux one, whose
    // excess is c0 * wall_const (and the 3-point ZeroGradient/non-fixed
    // corner row, where the reference's overlapping writes leave a sum).
    xs = -((row.a + row.b) + row.c);
    k = r.S ? r.S[i] : 0.0;
    if (i == 0 && r.left_bc == EMBER_BC_WALL_FLUX) {
        const double c0 = r.B[0] * static_cast<double>(r.alpha + 1) / (r.x[1] - r.x[0]);
        xs = c0 * r.wall_const;
        k += c0 * r.wall_const * r.y_inf;
    }
}

// Pass R: a, c, sigma = shift + x and k of the lane's chunk into the alpha,
// c', e and kappa slots; returns the chunk's matrix in u = 1 + lu_c
// coordinates (normalised).
__device__ void rows_and_moebius(const RowCtx& r, const LaneChunk& ch, double* ws, double shift, double& m11,
                                 double& m12, double& m21, double& m22) {
    m11 = 1.0;
    m12 = 0.0;
    m21 = 0.0;
    m22 = 1.0;
    double c2m = 0.0;  // c2 of the previous point (interior rows)
    for (int j = 0; j < ch.cnt; ++j) {
        const int i = ch.i0 + j;
        double a, c, xs, k;
        if (i >= 2 && i <= r.N - 3) {
            if (j == 0 || i == 2) {
                const double2 gp = r.geo[i - 1];
                c2m = (r.D[i - 1] + r.D[i]) * gp.y;
            }
            const double2 g = r.geo[i];
            const double c1 = r.B[i] * g.x;
            const double c2 = (r.D[i] + r.D[i + 1]) * g.y;
            a = c1 * c2m;
            c = c1 * c2;
            xs = 0.0;
            k = r.S ? r.S[i] : 0.0;
            c2m = c2;
        } else {
            boundary_row(r, i, a, c, xs, k);
        }
        const double sg = shift + xs;
        ch.at(ws, j, S_ALPHA) = a;
        ch.at(ws, j, S_CP) = c;
        ch.at(ws, j, S_E) = sg;
        ch.at(ws, j, S_KAPPA) = k;
        // [[a, sg], [a, c + sg]] * M
        const double p1 = a * m11, p2 = a * m12, cs = c + sg;
        const double n11 = fma(sg, m21, p1), n12 = fma(sg, m22, p2);
        const double n21 = fma(cs, m21, p1), n22 = fma(cs, m22, p2);
        m11 = n11;
        m12 = n12;
        m21 = n21;
        m22 = n22;
        if ((j & 3) == 3) normalize(m11, m12, m21, m22);
    }
    normalize(m11, m12, m21, m22);
}

// The carried scan coefficients of a factorisation: per level the slope
// before it (warp Kogge-Stone), and the lane's inclusive slopes from the
// warp's start (forward) and to the warp's end (backward).
struct ScanCoef {
    double pf[5], pb[5];
    double pin, qin;
};

// Factorisation of (A - shift I) for one group; srhs is the factor of y in the
// right-hand side (-8/h for BDF1 sub-steps, -2/h for BDF2). Leaves alpha, c',
// e, kappa, G, H in the workspace and returns the scan coefficients.
__device__ void factorize(const RowCtx& r, const LaneChunk& ch, double* ws, const Group& gr, double shift,
                          double srhs, ScanCoef& sc) {
    const int lane = gr.lane;
    double m11, m12, m21, m22;
    rows_and_moebius(r, ch, ws, shift, m11, m12, m21, m22);
    // Inclusive scan of the chunk matrices over the warp, later chunks on the left.
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double u11 = shfl_up(m11, o), u12 = shfl_up(m12, o), u21 = shfl_up(m21, o), u22 = shfl_up(m22, o);
        if (lane >= o) {
            const double r11 = fma(m11, u11, m12 * u21), r12 = fma(m11, u12, m12 * u22);
            const double r21 = fma(m21, u11, m22 * u21), r22 = fma(m21, u12, m22 * u22);
            m11 = r11;
            m12 = r12;
            m21 = r21;
            m22 = r22;
            normalize(m11, m12, m21, m22);
        }
    }
    // Product of the earlier warps' totals, E = T_{wl-1} ... T_0.
    double e11 = 1.0, e12 = 0.0, e21 = 0.0, e22 = 1.0;
    if (gr.G > 1) {
        if (lane == 31) {
            double* q = gr.mine();
            q[0] = m11;
            q[1] = m12;
            q[2] = m21;
            q[3] = m22;
        }
        gr.sync();
        for (int j = 0; j < gr.wl; ++j) {
            const double* q = gr.slot(j);
            const double r11 = fma(q[0], e11, q[1] * e21), r12 = fma(q[0], e12, q[1] * e22);
            const double r21 = fma(q[2], e11, q[3] * e21), r22 = fma(q[2], e12, q[3] * e22);
            e11 = r11;
            e12 = r12;
            e21 = r21;
            e22 = r22;
            normalize(e11, e12, e21, e22);
        }
    }
    // u entering the chunk: the exclusive prefix (the previous lane's
    // inclusive product times E; E alone for lane 0) applied to u = 1.
    double x11 = shfl_up(m11, 1), x12 = shfl_up(m12, 1);
    double x21 = shfl_up(m21, 1), x22 = shfl_up(m22, 1);
    double p11, p12, p21, p22;
    if (lane == 0) {
        p11 = e11;
        p12 = e12;
        p21 = e21;
        p22 = e22;
    } else if (gr.wl == 0) {
        p11 = x11;
        p12 = x12;
        p21 = x21;
        p22 = x22;
    } else {
        p11 = fma(x11, e11, x12 * e21);
        p12 = fma(x11, e12, x12 * e22);
        p21 = fma(x21, e11, x22 * e21);
        p22 = fma(x21, e12, x22 * e22);
    }
    double u = (lane == 0 && gr.wl == 0) ? 1.0 : (p11 + p12) / (p21 + p22);

    // Pass F: the recurrence itself, with the per-point coefficients.
    double G = 1.0;
    for (int j = 0; j < ch.cnt; ++j) {
        const int i = ch.i0 + j;
        const double a = ch.at(ws, j, S_ALPHA), c = ch.at(ws, j, S_CP);
        const double sg = ch.at(ws, j, S_E), k = ch.at(ws, j, S_KAPPA);
        const double t = fma(a, u, sg);
        const double rd = 1.0 / (t + c);  // -1/den
        const double ar = a * rd;         // -alpha
        G *= ar;
        u = t * rd;
        ch.at(ws, j, S_ALPHA) = -ar;
        ch.at(ws, j, S_CP) = i == r.N - 1 ? 0.0 : -c * rd;
        ch.at(ws, j, S_E) = -srhs * rd;
        ch.at(ws, j, S_KAPPA) = k * rd;
        ch.at(ws, j, S_G) = G;
    }
    // Pass H: running products of -c' from the chunk's end.
    double H = 1.0;
    for (int j = ch.cnt - 1; j >= 0; --j) {
        H *= -ch.at(ws, j, S_CP);
        ch.at(ws, j, S_H) = H;
    }
    // Scan coefficients (Kogge-Stone): the map's slope before each level.
    double P = G, Q = H;
#pragma unroll
    for (int lev = 0, o = 1; lev < 5; ++lev, o <<= 1) {
        sc.pf[lev] = P;
        sc.pb[lev] = Q;
        const double tp = shfl_up(P, o), tq = shfl_down(Q, o);
        if (lane >= o) P *= tp;
        if (lane + o < 32) Q *= tq;
    }
    sc.pin = P;
    sc.qin = Q;
    if (gr.G > 1) {
        // the warp's slope totals for the other warps' carries (read after
        // the next sub-step's barrier)
        const double pt = __shfl_sync(kFull, P, 31), qt = __shfl_sync(kFull, Q, 0);
        if (lane == 0) {
            gr.mine()[6] = pt;
            gr.mine()[7] = qt;
        }
    }
}

// One sub-step: solve (A - shift I) y_new = rhs(y). On entry the state slot
// holds the back substitution of the previous sub-step without its carry,
// i.e. y_j = state_j + H_j * cb; on exit likewise with the new cb.
template <bool kBdf2>
__device__ __forceinline__ void substep(const LaneChunk& ch, double* ws, const Group& gr, const ScanCoef& sc,
                                        double& cb) {
    const int lane = gr.lane;
    double d = 0.0;
#pragma unroll 4
    for (int j = 0; j < ch.cnt; ++j) {
        double yv = fma(ch.at(ws, j, S_H), cb, ch.at(ws, j, S_W));
        if (kBdf2) {
            const double yp = ch.at(ws, j, S_YP);
            ch.at(ws, j, S_YP) = yv;
            yv = fma(-0.25, yp, yv);
        }
        const double rho = fma(ch.at(ws, j, S_E), yv, ch.at(ws, j, S_KAPPA));
        d = fma(-ch.at(ws, j, S_ALPHA), d, rho);
        ch.at(ws, j, S_W) = d;
    }
#pragma unroll
    for (int lev = 0, o = 1; lev < 5; ++lev, o <<= 1) {
        const double t = shfl_up(d, o);
        if (lane >= o) d = fma(sc.pf[lev], t, d);
    }
    double cw = 0.0;  // value entering the warp
    if (gr.G > 1) {
        if (lane == 31) gr.mine()[4] = d;
        gr.sync();
        for (int j = 0; j < gr.wl; ++j) cw = fma(gr.slot(j)[6], cw, gr.slot(j)[4]);
        d = fma(sc.pin, cw, d);
    }
    double cf = shfl_up(d, 1);
    if (lane == 0) cf = cw;
    double yv = 0.0;
#pragma unroll 4
    for (int j = ch.cnt - 1; j >= 0; --j) {
        const double dd = fma(ch.at(ws, j, S_G), cf, ch.at(ws, j, S_W));
        yv = fma(-ch.at(ws, j, S_CP), yv, dd);
        ch.at(ws, j, S_W) = yv;
    }
#pragma unroll
    for (int lev = 0, o = 1; lev < 5; ++lev, o <<= 1) {
        const double t = shfl_down(yv, o);
        if (lane + o < 32) yv = fma(sc.pb[lev], t, yv);
    }
    double cr = 0.0;  // value entering the warp from the right
    if (gr.G > 1) {
        if (lane == 0) gr.mine()[5] = yv;
        gr.sync();
        for (int j = gr.G - 1; j > gr.wl; --j) cr = fma(gr.slot(j)[7], cr, gr.slot(j)[5]);
        yv = fma(sc.qin, cr, yv);
    }
    cb = shfl_down(yv, 1);
    if (lane == 31) cb = cr;
}

__device__ __forceinline__ void apply_carry(const LaneChunk& ch, double* ws, double& cb) {
    for (int j = 0; j < ch.cnt; ++j) ch.at(ws, j, S_W) = fma(ch.at(ws, j, S_H), cb, ch.at(ws, j, S_W));
    cb = 0.0;
}

// One system by one group of warps.
__device__ void run_system(const WarpDiffView& v, int s, const Group& gr) {
    const int lane = gr.lane;
    const DiffSysInfo info = v.info[s];
    const int N = info.n;
    const int L = 32 * gr.G;
    const int gl = gr.wl * 32 + lane;
    const int m = (N + L - 1) / L;
    LaneChunk ch;
    ch.N = N;
    ch.i0 = min(gl * m, N);
    ch.cnt = min(N - ch.i0, m);
    ch.stride = L;
    ch.base = v.ws_off[s] + gl;

    RowCtx r;
    r.N = N;
    r.alpha = info.alpha;
    r.left_bc = info.left_bc;
    r.right_bc = info.right_bc;
    r.x = v.x + info.grid_off;
    r.geo = v.geo + info.grid_off;
    r.B = v.B + info.off;
    r.D = v.D + info.off;
    r.S = v.split_const ? v.split_const + info.off : nullptr;
    r.wall_const = v.wall_const ? v.wall_const[s] : 0.0;
    r.y_inf = v.y_inf ? v.y_inf[s] : 0.0;

    // Step size: explicit, or min(mult * min_j dlj^2 / (B_j D_j), gdt)
    // with the reference's rounding (a minimum does not depend on order).
    double h;
    if (v.h) {
        h = v.h[s];
    } else {
        double mn = 0.0;
        bool have = false;
        for (int j = 0; j < ch.cnt; ++j) {
            const int i = ch.i0 + j;
            if (i < 1 || i > N - 2) continue;
            const double dlj = __dmul_rn(0.5, __dsub_rn(r.x[i + 1], r.x[i - 1]));
            const double q = __ddiv_rn(__dmul_rn(dlj, dlj), __dmul_rn(r.B[i], r.D[i]));
            if (!have || q < mn) mn = q;
            have = true;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double t = __shfl_xor_sync(kFull, mn, o);
            const bool th = __shfl_xor_sync(kFull, have, o);
            if (th && (!have || t < mn)) mn = t;
            have = have || th;
        }
        if (gr.G > 1) {
            if (lane == 0) {
                gr.mine()[0] = mn;
                gr.mine()[1] = have ? 1.0 : 0.0;
            }
            gr.sync();
            for (int j = 0; j < gr.G; ++j) {
                const double t = gr.slot(j)[0];
                const bool th = gr.slot(j)[1] != 0.0;
                if (th && (!have || t < mn)) mn = t;
                have = have || th;
            }
            gr.sync();  // the slots are reused by the factorisation
        }
        const double hm = __dmul_rn(v.mult, mn);
        h = v.gdt < hm ? v.gdt : hm;
    }
    // Integrator::integrateToTime step rounding.
    double t0, t1;
    v.tm.get(t0, t1);
    const double q = __dadd_rn(__ddiv_rn(__dsub_rn(t1, t0), h), 1e-5);
    if (!(h > 0.0) || !(q < 2147483647.0)) {
        if (gl == 0 && v.status) v.status[s] = TRI_BAD_STEP;
        return;
    }
    const int n_steps = q >= 1.0 ? static_cast<int>(q) : 1;
    h = __ddiv_rn(__dsub_rn(t1, t0), static_cast<double>(n_steps));

    double* y = v.y + info.off;
    for (int j = 0; j < ch.cnt; ++j) {
        const double y0 = y[ch.i0 + j];
        ch.at(v.ws, j, S_W) = y0;
        if (n_steps > 1) ch.at(v.ws, j, S_YP) = y0;
    }
    ScanCoef sc;
    double cb = 0.0;
    // First step: 8 BDF1 sub-steps of h/8 with one factorisation.
    factorize(r, ch, v.ws, gr, 8.0 / h, -8.0 / h, sc);
    for (int sub = 0; sub < 8; ++sub) substep<false>(ch, v.ws, gr, sc, cb);
    // Later steps: BDF2 with (A - 3/(2h) I).
    if (n_steps > 1) {
        apply_carry(ch, v.ws, cb);
        factorize(r, ch, v.ws, gr, 1.5 / h, -2.0 / h, sc);
        for (int step = 1; step < n_steps; ++step) substep<true>(ch, v.ws, gr, sc, cb);
    }
    bool finite = true;
    for (int j = 0; j < ch.cnt; ++j) {
        const double yv = fma(ch.at(v.ws, j, S_H), cb, ch.at(v.ws, j, S_W));
        y[ch.i0 + j] = yv;
        finite = finite && isfinite(yv);
    }
    bool all_finite = __all_sync(kFull, finite);
    if (gr.G > 1) {
        if (lane == 0) gr.mine()[4] = all_finite ? 1.0 : 0.0;
        gr.sync();
        for (int j = 0; j < gr.G; ++j) all_finite = all_finite && gr.slot(j)[4] != 0.0;
    }
    if (gl == 0 && v.status) v.status[s] = all_finite ? TRI_OK : TRI_NONFINITE;
}

__global__ void __launch_bounds__(32 * kCtaWarps, 2) k_diffusion_warp(const __grid_constant__ WarpDiffView v) {
    __shared__ double sh[kCtaWarps * 8];
    __shared__ int s_task;
    const int warp = threadIdx.x >> 5;
    for (;;) {
        if (threadIdx.x == 0) s_task = static_cast<int>(atomicAdd(v.counter, 1u));
        __syncthreads();
        const int task = s_task;
        if (task >= v.n_tasks) return;
        const int* t = v.tasks + int64_t(task) * kTaskInts;
        const int G = t[0];
        const int g = warp / G;
        const int s = t[1 + g];
        if (s >= 0) {
            Group gr;
            gr.G = G;
            gr.wl = warp - g * G;
            gr.lane = threadIdx.x & 31;
            gr.w0 = g * G;
            gr.bar = 1 + g;
            gr.sh = sh;
            run_system(v, s, gr);
        }
        __syncthreads();  // every group done with the shared slots and s_task
    }
}

// Tuning knobs (environment, read once): EMBER_DIFFUSION_POINTS_PER_LANE
// (chunk length that sets the group size; default 24) and
// EMBER_DIFFUSION_CTAS_PER_SM (resident CTAs of eight warps; default 2).
int env_int(const char* name, int lo, int hi, int dflt) {
    const char* e = std::getenv(name);
    const int v = e ? std::atoi(e) : 0;
    return (v >= lo && v <= hi) ? v : dflt;
}
int points_per_lane() {
    static int p = env_int("EMBER_DIFFUSION_POINTS_PER_LANE", 1, 4096, 24);
    return p;
}
int ctas_per_sm() {
    static int c = env_int("EMBER_DIFFUSION_CTAS_PER_SM", 1, 8, 2);
    return c;
}

// Warps of the group of a system of n points.
int group_warps(int n) {
    const int per_warp = 32 * points_per_lane();
    const int need = (n + per_warp - 1) / per_warp;
    return need <= 1 ? 1 : need <= 2 ? 2 : need <= 4 ? 4 : kCtaWarps;
}

int64_t system_doubles(int n) {
    const int L = 32 * group_warps(n);
    return int64_t(kSlots) * L * ((n + L - 1) / L);
}

// Tasks, largest systems first: per group size, systems by descending n,
// 8/G to a task.
std::vector<int> make_tasks(const std::vector<DiffSysInfo>& info) {
    const int n_sys = static_cast<int>(info.size());
    std::vector<int> order(n_sys);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return info[a].n > info[b].n; });
    std::vector<int> tasks;
    int cur_g = 0, filled = 0;
    for (int s : order) {
        const int G = group_warps(info[s].n);
        if (G != cur_g || filled == kCtaWarps / G) {
            tasks.push_back(G);
            for (int k = 0; k < kCtaWarps; ++k) tasks.push_back(-1);
            cur_g = G;
            filled = 0;
        }
        tasks[tasks.size() - kCtaWarps + filled] = s;
        ++filled;
    }
    return tasks;
}

}  // namespace

size_t diffusion_warp_plan_bytes(const std::vector<DiffSysInfo>& info, int64_t n_pts) {
    int64_t total = 0;
    for (const DiffSysInfo& d : info) total += system_doubles(d.n);
    const size_t n_sys = info.size();
    const size_t n_task_ints = make_tasks(info).size();
    return Scratch::rounded(sizeof(double) * size_t(total)) + Scratch::rounded(sizeof(double2) * size_t(n_pts)) +
           Scratch::rounded(sizeof(int64_t) * n_sys) + Scratch::rounded(sizeof(int) * n_task_ints) +
           Scratch::rounded(sizeof(unsigned int));
}

int diffusion_warp_plan_init(DiffusionWarpPlan* p, const std::vector<DiffSysInfo>& info, int n_flames, int n_vars,
                             int64_t n_pts, Scratch& sc, cudaStream_t st) {
    const int n_sys = static_cast<int>(info.size());
    std::vector<int64_t> off(n_sys);
    int64_t total = 0;
    int nmax = 0;
    for (int s = 0; s < n_sys; ++s) {
        off[s] = total;
        total += system_doubles(info[s].n);
        nmax = std::max(nmax, info[s].n);
    }
    const std::vector<int> tasks = make_tasks(info);

    p->n_sys = n_sys;
    p->n_flames = n_flames;
    p->n_vars = n_vars;
    p->n_pts = n_pts;
    p->nmax = nmax;
    p->n_tasks = static_cast<int>(tasks.size() / kTaskInts);
    EMBER_TRY(sc.alloc(&p->ws, size_t(total)));
    EMBER_TRY(sc.alloc(&p->geo, size_t(n_pts)));
    EMBER_TRY(sc.alloc(&p->ws_off, size_t(n_sys)));
    EMBER_TRY(sc.alloc(&p->tasks, tasks.size()));
    EMBER_TRY(sc.alloc(&p->counter, 1));
    EMBER_CUDA_TRY(cudaMemcpyAsync(p->ws_off, off.data(), sizeof(int64_t) * n_sys, cudaMemcpyHostToDevice, st));
    EMBER_CUDA_TRY(cudaMemcpyAsync(p->tasks, tasks.data(), sizeof(int) * tasks.size(), cudaMemcpyHostToDevice, st));

    int dev = 0, sms = 0;
    EMBER_CUDA_TRY(cudaGetDevice(&dev));
    EMBER_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    p->blocks = static_cast<int>(std::min<int64_t>(p->n_tasks, int64_t(sms) * ctas_per_sm()));
    return EMBER_OK;
}

int diffusion_warp_geometry(const DiffusionWarpPlan& p, const DiffSysInfo* d_info, const double* x, cudaStream_t st) {
    dim3 ggeo(std::min(blocks_for(p.nmax, 256), 16), std::min(p.n_flames, 65535));
    k_diffusion_geometry<<<ggeo, 256, 0, st>>>(d_info, p.n_flames, p.n_vars, x, p.geo);
    EMBER_CUDA_TRY(cudaGetLastError());
    return EMBER_OK;
}

int diffusion_warp_run(const DiffusionWarpPlan& p, const DiffusionView& dv, double* y, const StageTime& tm,
                       double mult, double gdt, cudaStream_t st) {
    if (p.n_tasks == 0) return EMBER_OK;
    EMBER_CUDA_TRY(cudaMemsetAsync(p.counter, 0, sizeof(unsigned int), st));
    WarpDiffView v;
    v.n_systems = p.n_sys;
    v.n_tasks = p.n_tasks;
    v.info = dv.info;
    v.tasks = p.tasks;
    v.ws_off = p.ws_off;
    v.x = dv.x;
    v.geo = p.geo;
    v.B = dv.B;
    v.D = dv.D;
    v.split_const = dv.split_const;
    v.h = dv.h;
    v.wall_const = dv.wall_const;
    v.y_inf = dv.y_inf;
    v.y = y;
    v.ws = p.ws;
    v.status = dv.status;
    v.counter = p.counter;
    v.tm = tm;
    v.mult = mult;
    v.gdt = gdt;
    k_diffusion_warp<<<p.blocks, 32 * kCtaWarps, 0, st>>>(v);
    EMBER_CUDA_TRY(cudaGetLastError());
    return EMBER_OK;
}

}  // namespace ember
