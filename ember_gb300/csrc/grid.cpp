// Adaptive flame grid on the host: the regrid block of FlameSolver::finishStep
// (src/flameSolver.cpp:279-352) with the rules of OneDimGrid (src/grid.cpp):
//
//   boundary regrid   strained flames: addRight / addLeft, else removeRight /
//                     removeLeft until a boundary is no longer flat
//                     (regrid, src/grid.cpp:721-783); unstrained flames: the
//                     right end from the heat-release profile
//                     (regridUnstrained, 785-838);
//   damping values    interpolated onto the new grid, clipped at the ends
//                     (mathUtils::interp1 without extrapolation);
//   interior adapt    point insertion where a variable or its first
//                     derivative changes by more than vtol / dvtol of its
//                     range, where the spacing exceeds the damping length,
//                     gridMax or the uniformity ratio; then removal where all
//                     criteria hold with rmTol of margin (adapt, 77-359).
//
// Inserted points sit midway between their neighbours and take the value of
// the natural cubic spline through each row (mathUtils::splines,
// src/mathUtils.cpp:233-254 with computeSplines, src/mathUtils.h:186-247);
// points added at a boundary repeat the boundary value. Every criterion is
// evaluated with the reference's expressions and operation order. The
// derivative used by the criteria is the centred three-point difference of
// OneDimGrid::updateValues; its end entries are zero.
//
// Plain host code: no CUDA call, usable without a device.
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/ember_gpu.h"

namespace ember {
void set_error(const char* fmt, ...);
}

namespace {

using Row = std::vector<double>;

// Natural cubic spline through (x, y) evaluated at xo (computeSplines +
// splines: the interval is the one whose right end is the first node >= xo).
double spline_at(const Row& x, const Row& y, double xo) {
    const int n = static_cast<int>(x.size());
    Row h(n - 1), b(n - 1), u(n - 1, 0.0), v(n - 1, 0.0), z(n, 0.0);
    for (int i = 0; i < n - 1; ++i) {
        h[i] = x[i + 1] - x[i];
        b[i] = (y[i + 1] - y[i]) / h[i];
    }
    if (n > 2) {
        u[1] = 2 * (h[0] + h[1]);
        v[1] = 6 * (b[1] - b[0]);
        for (int i = 2; i < n - 1; ++i) {
            u[i] = 2 * (h[i - 1] + h[i]) - h[i - 1] * h[i - 1] / u[i - 1];
            v[i] = 6 * (b[i] - b[i - 1]) - h[i - 1] * v[i - 1] / u[i - 1];
        }
        for (int i = n - 2; i > 0; --i) z[i] = (v[i] - h[i] * z[i + 1]) / u[i];
    }
    int j = -1;
    for (int i = 0; i < n; ++i)
        if (x[i] >= xo) {
            j = i;
            break;
        }
    if (j < 0) j = n - 2;  // past the last node: the last interval
    else if (j > 0) j -= 1;
    const double c0 = y[j];
    const double c1 = -h[j] / 6 * z[j + 1] - h[j] / 3 * z[j] + (y[j + 1] - y[j]) / h[j];
    const double c2 = 0.5 * z[j];
    const double c3 = (z[j + 1] - z[j]) / (6 * h[j]);
    const double dx = xo - x[j];
    return c0 + dx * (c1 + dx * (c2 + dx * c3));
}

// Linear interpolation of (xi, yi) at xo, the end values outside.
double interp_clipped(const Row& xi, const Row& yi, double xo) {
    const int n = static_cast<int>(xi.size());
    int j = -1;
    for (int i = 0; i < n; ++i)
        if (xi[i] >= xo) {
            j = i;
            break;
        }
    if (j == 0) return yi[0];
    if (j < 0) return yi[n - 1];
    j -= 1;
    return yi[j] + (yi[j + 1] - yi[j]) / (xi[j + 1] - xi[j]) * (xo - xi[j]);
}

double max_of(const Row& v) {
    double m = v[0];
    for (double a : v) m = a > m ? a : m;
    return m;
}

double range_of(const Row& v, int i0, int i1) {
    double lo = v[i0], hi = v[i0];
    for (int i = i0; i <= i1; ++i) {
        lo = v[i] < lo ? v[i] : lo;
        hi = v[i] > hi ? v[i] : hi;
    }
    return hi - lo;
}

constexpr int kMomentum = 0;  // U is the first state variable

}  // namespace

struct ember_grid_s {
    ember_grid_options o;
    Row x, damp;
    std::vector<Row> y;  // rows: the first n_adapt drive the criteria
    int n_adapt = 0;
    int ju = 0, jb = 0;
    bool updated = false;
    Row hh, cfm, cf, cfp;

    int jj() const { return static_cast<int>(x.size()) - 1; }

    void boundary_indices() {
        if (o.unburned_left) {
            ju = 0;
            jb = jj();
        } else {
            jb = 0;
            ju = jj();
        }
    }

    // OneDimGrid::updateValues: spacings and centred-difference weights.
    void metrics() {
        const int J = jj();
        hh.assign(J, 0.0);
        cfm.assign(J, 0.0);
        cf.assign(J, 0.0);
        cfp.assign(J, 0.0);
        for (int j = 0; j < J; ++j) hh[j] = x[j + 1] - x[j];
        for (int j = 1; j < J; ++j) {
            cfp[j] = hh[j - 1] / (hh[j] * (hh[j] + hh[j - 1]));
            cf[j] = (hh[j] - hh[j - 1]) / (hh[j] * hh[j - 1]);
            cfm[j] = -hh[j] / (hh[j - 1] * (hh[j] + hh[j - 1]));
        }
    }

    // Per adapted row: the derivative (zero at both ends), the row's range
    // and the derivative's range over the interior.
    void derivatives(std::vector<Row>& dv, Row& vr, Row& dvr) const {
        const int J = jj();
        dv.assign(n_adapt, Row(J + 1, 0.0));
        vr.assign(n_adapt, 0.0);
        dvr.assign(n_adapt, 0.0);
        for (int k = 0; k < n_adapt; ++k) {
            const Row& v = y[k];
            for (int i = 1; i < J; ++i) dv[k][i] = cfp[i] * v[i + 1] + cf[i] * v[i] + cfm[i] * v[i - 1];
            vr[k] = range_of(v, 0, J);
            dvr[k] = range_of(dv[k], 1, J - 1);
        }
    }

    bool pinned_left() const {
        return o.left_bc == EMBER_BC_CONTROL_VOLUME || o.left_bc == EMBER_BC_WALL_FLUX;
    }

    void insert_after(int j) {
        const double xi = 0.5 * (x[j + 1] + x[j]);
        damp.insert(damp.begin() + j + 1, spline_at(x, damp, xi));
        for (Row& r : y) r.insert(r.begin() + j + 1, spline_at(x, r, xi));
        x.insert(x.begin() + j + 1, xi);
    }

    void erase_at(int j) {
        x.erase(x.begin() + j);
        damp.erase(damp.begin() + j);
        for (Row& r : y) r.erase(r.begin() + j);
    }

    // OneDimGrid::adapt: insertion sweep, then removal sweep.
    void adapt() {
        std::vector<Row> dv;
        Row vr, dvr;
        metrics();
        derivatives(dv, vr, dvr);
        int j = 0;
        while (j < jj()) {
            const int J = jj();
            bool insert = false;
            for (int k = 0; k < n_adapt; ++k) {
                if (vr[k] < o.absvtol) continue;
                const Row& v = y[k];
                if (std::fabs(v[j + 1] - v[j]) > o.vtol * vr[k]) insert = true;
                if (j != 0 && j != J - 1 && std::fabs(dv[k][j + 1] - dv[k][j]) > o.dvtol * dvr[k]) insert = true;
            }
            if (hh[j] > o.damp_const * damp[j]) insert = true;
            if (hh[j] > o.grid_max) insert = true;
            if (j != 0 && hh[j] / hh[j - 1] > o.uniformity_tol) insert = true;
            if (j != J - 1 && hh[j] / hh[j + 1] > o.uniformity_tol) insert = true;
            if (j == 0 && pinned_left()) {
                const double xmin = std::fmin(o.center_grid_min, 0.02 * x[J]);
                if (hh[j] < 2 * xmin) insert = false;
            }
            if (insert && hh[j] < 2 * o.grid_min) insert = false;
            if (insert) {
                insert_after(j);
                updated = true;
                metrics();
                derivatives(dv, vr, dvr);
                j += 2;
            } else {
                ++j;
            }
        }
        j = 1;
        while (j < jj()) {
            const int J = jj();
            bool remove = true;
            for (int k = 0; k < n_adapt; ++k) {
                if (vr[k] < o.absvtol) continue;
                const Row& v = y[k];
                if (std::fabs(v[j + 1] - v[j - 1]) > o.rm_tol * o.vtol * vr[k]) remove = false;
                // (the reference skips j == 2 here, not j == 1, whose test reads the zero end entry)
                if (j != 2 && j != J - 1 && std::fabs(dv[k][j + 1] - dv[k][j - 1]) > o.rm_tol * o.dvtol * dvr[k])
                    remove = false;
            }
            if (hh[j] + hh[j - 1] >= o.rm_tol * o.damp_const * damp[j]) remove = false;
            if (hh[j] + hh[j - 1] > o.grid_max) remove = false;
            if (j >= 2 && hh[j] + hh[j - 1] > o.uniformity_tol * hh[j - 2]) remove = false;
            if (j <= J - 2 && hh[j] + hh[j - 1] > o.uniformity_tol * hh[j + 1]) remove = false;
            if (j == 1 && pinned_left()) remove = false;
            if (remove) {
                erase_at(j);
                updated = true;
                metrics();
                derivatives(dv, vr, dvr);
            } else {
                ++j;
            }
        }
        if (updated) boundary_indices();
    }

    // Flatness of row k at a boundary: |y[k][a] - y[k][b]| / max(y[k]) above tol.
    bool steep(int k, int a, int b, double tol) const {
        const double ymax = max_of(y[k]);
        return std::fabs(y[k][a] - y[k][b]) / ymax > tol && ymax > o.absvtol;
    }

    void append_right(Row* qdot) {
        const double ratio = std::pow(o.uniformity_tol, 1.0 / (1 + o.add_point_count));
        for (int i = 0; i < o.add_point_count; ++i) {
            const int J = jj();
            x.push_back(x[J] + ratio * (x[J] - x[J - 1]));
            damp.push_back(damp[J]);
            if (qdot) qdot->push_back((*qdot)[J]);
            for (Row& r : y) r.push_back(r[J]);
        }
        boundary_indices();
    }

    bool add_right() {
        const int J = jj();
        const int dj_other = (jb == J && !o.fixed_burned_val) ? 2 : 1;
        bool add = false;
        for (int k = 0; k < n_adapt && !add; ++k)
            add = steep(k, J, J - (k == kMomentum ? 1 : dj_other), o.boundary_tol);
        if (add) append_right(nullptr);
        return add;
    }

    bool add_left() {
        const int dj_other = (jb == 1 && !o.fixed_burned_val) ? 2 : 1;
        bool add = false;
        if (!o.fixed_left_loc)
            for (int k = 0; k < n_adapt && !add; ++k)
                add = steep(k, k == kMomentum ? 1 : dj_other, 0, o.boundary_tol);
        if (o.fixed_left_loc && !pinned_left() && x[0] > 0.0) add = true;
        if (!add) return false;
        for (int i = 0; i < o.add_point_count; ++i) {
            double xl = x[0] - std::sqrt(o.uniformity_tol) * (x[1] - x[0]);
            if (o.twin_flame || o.cylindrical_flame) {
                if (x[0] == 0) break;
                const double xmin = std::fmin(o.center_grid_min, 0.005 * x[jj()]);
                if (xl < 0.0) xl = 0.0;
                else if (xl < xmin) xl = xmin;
            }
            x.insert(x.begin(), xl);
            damp.insert(damp.begin(), damp[0]);
            for (Row& r : y) r.insert(r.begin(), r[0]);
        }
        boundary_indices();
        return true;
    }

    bool remove_right() {
        const int J = jj();
        const int dj_other = (jb == J && !o.fixed_burned_val) ? 3 : 2;
        bool rm = true;
        for (int k = 0; k < n_adapt && rm; ++k)
            if (steep(k, J, J - (k == kMomentum ? 2 : dj_other), o.boundary_tol_rm)) rm = false;
        if (J < 3) rm = false;
        if (rm) {
            erase_at(J);
            boundary_indices();
        }
        return rm;
    }

    bool remove_left() {
        const int dj_other = (jb == 1 && !o.fixed_burned_val) ? 3 : 2;
        bool rm = !o.fixed_left_loc;
        for (int k = 0; k < n_adapt; ++k)
            if (steep(k, k == kMomentum ? 2 : dj_other, 0, o.boundary_tol_rm)) rm = false;
        if (jj() < 3) rm = false;
        if (rm) {
            erase_at(0);
            boundary_indices();
        }
        return rm;
    }

    // The reaction zone of an unstrained flame: the points nearest the heat
    // release peak where |qdot| falls below 1 % of the peak.
    void reaction_zone(const Row& q, int& jq, double& width) const {
        const int J = jj();
        jq = 0;
        for (int j = 1; j <= J; ++j)
            if (q[j] > q[jq]) jq = j;
        const double qmax = q[jq];
        int jl = 0, jr = J;
        for (int j = jq; j >= 1; --j)
            if (std::fabs(q[j]) < 0.01 * qmax) {
                jl = j;
                break;
            }
        for (int j = jq; j <= J; ++j)
            if (std::fabs(q[j]) < 0.01 * qmax) {
                jr = j;
                break;
            }
        width = x[jr] - x[jl];
    }

    bool add_right_unstrained(Row& q) {
        int jq;
        double w;
        reaction_zone(q, jq, w);
        const bool add = x[jq] + o.unstrained_downstream_width * w > x[jj()];
        if (add) append_right(&q);
        return add;
    }

    bool remove_right_unstrained(Row& q) {
        int jq;
        double w;
        reaction_zone(q, jq, w);
        bool rm = x[jj()] > x[jq] + 1.25 * o.unstrained_downstream_width * w;
        if (jj() < 3) rm = false;
        if (rm) {
            erase_at(jj());
            q.pop_back();
            boundary_indices();
        }
        return rm;
    }

    void regrid_boundaries(Row* qdot) {
        bool changed = false;
        if (qdot) {
            const bool right = add_right_unstrained(*qdot);
            if (!right)
                while (remove_right_unstrained(*qdot)) changed = true;
            const bool left = add_left();
            if (!left)
                while (remove_left()) changed = true;
            changed = changed || right || left;
        } else {
            const bool right = add_right();
            const bool left = add_left();
            if (!right)
                while (remove_right()) changed = true;
            if (!left)
                while (remove_left()) changed = true;
            changed = changed || right || left;
        }
        updated = updated || changed;
        if (updated) boundary_indices();
    }
};

extern "C" int ember_grid_options_default(ember_grid_options* o) {
    if (!o) {
        ember::set_error("null options");
        return EMBER_EINVAL;
    }
    std::memset(o, 0, sizeof(*o));
    o->vtol = 0.12;
    o->dvtol = 0.2;
    o->absvtol = 1e-8;
    o->rm_tol = 0.6;
    o->uniformity_tol = 2.5;
    o->grid_min = 5e-7;
    o->grid_max = 2e-4;
    o->damp_const = 7.0;
    o->center_grid_min = 1e-4;
    o->boundary_tol = 5e-5;
    o->boundary_tol_rm = 1e-5;
    o->unstrained_downstream_width = 5.0;
    o->add_point_count = 3;
    o->fixed_burned_val = 1;
    o->unburned_left = 1;
    o->fixed_left_loc = 0;
    o->twin_flame = 0;
    o->cylindrical_flame = 0;
    o->left_bc = EMBER_BC_FIXED_VALUE;
    o->right_bc = EMBER_BC_FIXED_VALUE;
    return EMBER_OK;
}

extern "C" int ember_grid_create(const ember_grid_options* opts, int n_points, const double* x, ember_grid* out) {
    if (!opts || !x || !out || n_points < 3) {
        ember::set_error("ember_grid_create: need options, x and at least 3 points");
        return EMBER_EINVAL;
    }
    for (int j = 0; j + 1 < n_points; ++j)
        if (!(x[j + 1] > x[j])) {
            ember::set_error("ember_grid_create: x must increase strictly (x[%d] = %g, x[%d] = %g)", j, x[j], j + 1,
                             x[j + 1]);
            return EMBER_EINVAL;
        }
    if (opts->add_point_count < 0 || !(opts->uniformity_tol > 1.0)) {
        ember::set_error("ember_grid_create: add_point_count must be >= 0 and uniformity_tol > 1");
        return EMBER_EINVAL;
    }
    ember_grid g = new (std::nothrow) ember_grid_s;
    if (!g) {
        ember::set_error("ember_grid_create: out of host memory");
        return EMBER_ENOMEM;
    }
    g->o = *opts;
    g->x.assign(x, x + n_points);
    g->boundary_indices();
    *out = g;
    return EMBER_OK;
}

extern "C" int ember_grid_destroy(ember_grid g) {
    delete g;
    return EMBER_OK;
}

extern "C" int ember_grid_regrid(ember_grid g, int n_rows, int n_adapt, const double* rows, const double* damp_val,
                                 const double* qdot, double strain_rate, int boundaries, int* n_points_out,
                                 int* updated) {
    if (!g || !rows || !damp_val || n_rows < 1 || n_adapt < 0 || n_adapt > n_rows) {
        ember::set_error("ember_grid_regrid: bad arguments (n_rows %d, n_adapt %d)", n_rows, n_adapt);
        return EMBER_EINVAL;
    }
    const int N = static_cast<int>(g->x.size());
    for (int j = 0; j < N; ++j)
        if (!(damp_val[j] > 0)) {
            ember::set_error("ember_grid_regrid: damp_val[%d] = %g must be positive", j, damp_val[j]);
            return EMBER_EINVAL;
        }
    if (boundaries && strain_rate == 0.0 && !qdot) {
        ember::set_error("ember_grid_regrid: an unstrained flame needs qdot for the boundary regrid");
        return EMBER_EINVAL;
    }
    g->n_adapt = n_adapt;
    g->y.assign(n_rows, Row());
    for (int k = 0; k < n_rows; ++k) g->y[k].assign(rows + size_t(k) * N, rows + size_t(k + 1) * N);
    g->damp.assign(damp_val, damp_val + N);
    g->updated = false;
    const Row x_prev = g->x, damp_prev = g->damp;
    if (boundaries) {
        if (strain_rate == 0.0) {
            Row q(qdot, qdot + N);
            g->regrid_boundaries(&q);
        } else {
            g->regrid_boundaries(nullptr);
        }
    }
    // damping values interpolated onto the (possibly extended) grid, clipped
    // at the ends, as the reference does whether or not the ends moved
    Row d(g->x.size());
    for (size_t j = 0; j < g->x.size(); ++j) d[j] = interp_clipped(x_prev, damp_prev, g->x[j]);
    g->damp = d;
    g->adapt();
    if (n_points_out) *n_points_out = static_cast<int>(g->x.size());
    if (updated) *updated = g->updated ? 1 : 0;
    return EMBER_OK;
}

extern "C" int ember_grid_get(ember_grid g, double* x, double* rows, int* ju, int* jb) {
    if (!g) {
        ember::set_error("null ember_grid handle");
        return EMBER_EINVAL;
    }
    const size_t N = g->x.size();
    if (x) std::memcpy(x, g->x.data(), N * sizeof(double));
    if (rows)
        for (size_t k = 0; k < g->y.size(); ++k) std::memcpy(rows + k * N, g->y[k].data(), N * sizeof(double));
    if (ju) *ju = g->ju;
    if (jb) *jb = g->jb;
    return EMBER_OK;
}

extern "C" int ember_grid_damping(int n_points, int n_species, const double* mu, const double* conductivity,
                                  const double* cp, const double* rho_d, const double* rho, double strain_rate,
                                  double* damp_val) {
    if (n_points < 1 || n_species < 0 || !mu || !conductivity || !cp || !rho || !damp_val ||
        (n_species > 0 && !rho_d)) {
        ember::set_error("ember_grid_damping: bad arguments");
        return EMBER_EINVAL;
    }
    for (int j = 0; j < n_points; ++j) {
        double num = std::fmin(mu[j], conductivity[j] / cp[j]);
        for (int k = 0; k < n_species; ++k) {
            const double d = rho_d[size_t(j) * n_species + k];
            if (d > 0) num = std::fmin(num, d);
        }
        const double den = std::fmax(std::fabs(rho[j] * strain_rate), 1e-100);
        damp_val[j] = std::sqrt(num / den);
    }
    return EMBER_OK;
}
