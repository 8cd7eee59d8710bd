/*
 * pto.cpp -- CPU oracle of the PENTrack tracking hot path (TEST INFRASTRUCTURE,
 * see pto.h).  Plain FP64, compiled with -ffp-contract=off.  Every function
 * cites the reference code it restates.
 */
#include "pto.h"

/* spin steps of one trajectory step before the particle stops with ID_ODEINT_ERROR */
#define PTO_MAX_SPIN_STEPS (1 << 22)
#include "../include/pt_constants.h"
#include "../include/pt_detmath.h"
#include "harmonic_terms.h"
#include "../include/pt_solenoid.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstring>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace {

thread_local std::string g_err;

/* ------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).  The reference draws
 * from one std::mt19937_64 per process (src/main.cpp:127-134); the engine
 * instead keys a counter-based stream by (seed, particle id), so draws do not
 * depend on particle order or partitioning.  Counter = (draw lo, draw hi,
 * id lo, id hi), key = (seed lo, seed hi); one draw = one block, the first
 * two words give a 53-bit uniform in [0,1).                              */
/* ------------------------------------------------------------------ */
inline void philox(const uint32_t c[4], const uint32_t k[2], uint32_t o[4]) {
    uint32_t x0 = c[0], x1 = c[1], x2 = c[2], x3 = c[3], k0 = k[0], k1 = k[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * x0, p1 = (uint64_t)0xCD9E8D57u * x2;
        uint32_t y0 = (uint32_t)(p1 >> 32) ^ x1 ^ k0, y1 = (uint32_t)p1;
        uint32_t y2 = (uint32_t)(p0 >> 32) ^ x3 ^ k1, y3 = (uint32_t)p0;
        x0 = y0; x1 = y1; x2 = y2; x3 = y3;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    o[0] = x0; o[1] = x1; o[2] = x2; o[3] = x3;
}

inline double uniform_draw(uint64_t seed, int64_t id, uint64_t draw) {
    uint32_t c[4] = {(uint32_t)draw, (uint32_t)(draw >> 32), (uint32_t)(uint64_t)id, (uint32_t)((uint64_t)id >> 32)};
    uint32_t k[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t o[4];
    philox(c, k, o);
    uint64_t v = ((uint64_t)o[0] << 32) | o[1];
    return (double)(v >> 11) * 0x1.0p-53;
}

struct Rng {
    uint64_t seed; int64_t id; uint64_t n;
    double u() { return uniform_draw(seed, id, n++); }
};

/* ------------------------------------------------------------------ */
/* ALGLIB spline1dgriddiffcubic with default (parabolically terminated)
 * boundaries: alglib-3.15.0/cpp/src/interpolation.cpp:3078-3105 (wrapper),
 * 22519-22610 (driver), 26709-26880 (internal), 26970-27005 (tridiagonal).  */
/* ------------------------------------------------------------------ */
void spline_derivs(int n, const double *x, const double *y, double *d) {
    if (n == 2) {
        d[0] = (y[1] - y[0]) / (x[1] - x[0]);
        d[1] = d[0];
        return;
    }
    std::vector<double> a1(n), a2(n), a3(n), b(n);
    a1[0] = 0; a2[0] = 1; a3[0] = 1;
    b[0] = 2 * (y[1] - y[0]) / (x[1] - x[0]);
    for (int i = 1; i <= n - 2; ++i) {
        a1[i] = x[i + 1] - x[i];
        a2[i] = 2 * (x[i + 1] - x[i - 1]);
        a3[i] = x[i] - x[i - 1];
        b[i] = 3 * (y[i] - y[i - 1]) / (x[i] - x[i - 1]) * (x[i + 1] - x[i]) +
               3 * (y[i + 1] - y[i]) / (x[i + 1] - x[i]) * (x[i] - x[i - 1]);
    }
    a1[n - 1] = 1; a2[n - 1] = 1; a3[n - 1] = 0;
    b[n - 1] = 2 * (y[n - 1] - y[n - 2]) / (x[n - 1] - x[n - 2]);
    /* Thomas algorithm, same operation order as spline1d_solvetridiagonal */
    for (int k = 1; k <= n - 1; ++k) {
        double t = a1[k] / a2[k - 1];
        a2[k] = a2[k] - t * a3[k - 1];
        b[k] = b[k] - t * b[k - 1];
    }
    d[n - 1] = b[n - 1] / a2[n - 1];
    for (int k = n - 2; k >= 0; --k) d[k] = (b[k] - a3[k] * d[k + 1]) / a2[k];
}

/* ------------------------------------------------------------------ */
/* libtricubic tricubic_get_coeff (libtricubic.cpp:24-48): a = A x with the
 * 64x64 integer matrix of the Lekien-Marsden scheme.  The matrix is not
 * copied: it is the tensor product of the 1D cubic-Hermite-to-monomial map
 * M (rows: power 0..3; columns: f(0), f(1), f'(0), f'(1)), laid out on the
 * stacked input [f, fx, fy, fz, fxy, fxz, fyz, fxyz] x corner(cx+2cy+4cz).
 * The sum runs over j = 0..63 in order, as tricubic_get_coeff_stacked does. */
/* ------------------------------------------------------------------ */
struct LMMatrix {
    int A[64][64];
    LMMatrix() {
        static const int M[4][4] = {{1, 0, 0, 0}, {0, 0, 1, 0}, {-3, 3, -2, -1}, {2, -2, 1, 1}};
        static const int der[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j)
                for (int k = 0; k < 4; ++k)
                    for (int dt = 0; dt < 8; ++dt)
                        for (int c = 0; c < 8; ++c) {
                            int cx = c & 1, cy = (c >> 1) & 1, cz = (c >> 2) & 1;
                            A[i + 4 * j + 16 * k][8 * dt + c] = M[i][cx + 2 * der[dt][0]] * M[j][cy + 2 * der[dt][1]] *
                                                                M[k][cz + 2 * der[dt][2]];
                        }
    }
};
const LMMatrix &lm_matrix() { static LMMatrix m; return m; }

void tricubic_coeff(const double *x, double *a) {
    const LMMatrix &L = lm_matrix();
    for (int i = 0; i < 64; ++i) {
        a[i] = 0.0;
        for (int j = 0; j < 64; ++j) a[i] += (double)L.A[i][j] * x[j];
    }
}

/* tricubic_eval_fast, value (src/field_3d.cpp:36-64) */
inline double tricubic_value(const double *a, double x, double y, double z) {
    double rx = 0.;
    for (int i = 3; i >= 0; --i) {
        double ry = 0.;
        for (int j = 3; j >= 0; --j) {
            double rz = 0.;
            for (int k = 3; k >= 0; --k) {
                rz += a[i + 4 * j + 16 * k];
                if (k > 0) rz *= z;
            }
            ry += rz;
            if (j > 0) ry *= y;
        }
        rx += ry;
        if (i > 0) rx *= x;
    }
    return rx;
}

/* tricubic_eval_fast with derivative orders (src/field_3d.cpp:82-121) */
inline double tricubic_deriv(const double *a, double x, double y, double z, int derx, int dery, int derz) {
    static const double fact[4][4] = {{1.0, 0.0, 0.0, 0.0}, {1.0, 1.0, 0.0, 0.0}, {1.0, 2.0, 2.0, 0.0}, {1.0, 3.0, 6.0, 6.0}};
    double rx = 0.;
    for (int i = 3; i >= derx; --i) {
        double ry = 0.;
        for (int j = 3; j >= dery; --j) {
            double rz = 0.;
            for (int k = 3; k >= derz; --k) {
                rz += fact[k][derz] * a[i + 4 * j + 16 * k];
                if (k > derz) rz *= z;
            }
            ry += fact[j][dery] * rz;
            if (j > dery) ry *= y;
        }
        rx += fact[i][derx] * ry;
        if (i > derx) rx *= x;
    }
    return rx;
}

/* ------------------------------------------------------------------ */
/* Fields                                                              */
/* ------------------------------------------------------------------ */
struct Tab3 {
    std::vector<double> ax[3];
    std::vector<double> coeff[4]; /* Bx, By, Bz, V: per cell 64 doubles; empty if absent */

    /* TabField3::CalcDerivs (src/field_3d.cpp:336-364) on a [ix][iy][iz] table */
    void calc_derivs(const std::vector<double> &tab, int dim, std::vector<double> &out) const {
        size_t n[3] = {ax[0].size(), ax[1].size(), ax[2].size()};
        out.assign(tab.size(), 0.0);
        int d1 = (dim + 1) % 3, d2 = (dim + 2) % 3;
        size_t len = n[dim];
        std::vector<double> y(len), d(len);
        size_t idx[3];
        for (idx[d1] = 0; idx[d1] < n[d1]; ++idx[d1])
            for (idx[d2] = 0; idx[d2] < n[d2]; ++idx[d2]) {
                for (idx[dim] = 0; idx[dim] < len; ++idx[dim]) y[idx[dim]] = tab[(idx[0] * n[1] + idx[1]) * n[2] + idx[2]];
                spline_derivs((int)len, ax[dim].data(), y.data(), d.data());
                for (idx[dim] = 0; idx[dim] < len; ++idx[dim]) out[(idx[0] * n[1] + idx[1]) * n[2] + idx[2]] = d[idx[dim]];
            }
    }

    /* TabField3::PreInterpol (src/field_3d.cpp:367-414) */
    void preinterpol(const std::vector<double> &tab, std::vector<double> &coeffs) const {
        size_t n[3] = {ax[0].size(), ax[1].size(), ax[2].size()};
        std::vector<double> dx, dy, dz, dxy, dxz, dyz, dxyz;
        calc_derivs(tab, 0, dx);
        calc_derivs(tab, 1, dy);
        calc_derivs(tab, 2, dz);
        calc_derivs(dx, 1, dxy);
        calc_derivs(dx, 2, dxz);
        calc_derivs(dy, 2, dyz);
        calc_derivs(dxy, 2, dxyz);
        size_t len[3] = {n[0] - 1, n[1] - 1, n[2] - 1};
        coeffs.assign(len[0] * len[1] * len[2] * 64, 0.0);
        for (size_t ix = 0; ix < len[0]; ++ix)
            for (size_t iy = 0; iy < len[1]; ++iy)
                for (size_t iz = 0; iz < len[2]; ++iz) {
                    double cellx = ax[0][ix + 1] - ax[0][ix];
                    double celly = ax[1][iy + 1] - ax[1][iy];
                    double cellz = ax[2][iz + 1] - ax[2][iz];
                    double x64[64];
                    for (int c = 0; c < 8; ++c) {
                        size_t i = ix + (c & 1), j = iy + ((c >> 1) & 1), k = iz + ((c >> 2) & 1);
                        size_t id = (i * n[1] + j) * n[2] + k;
                        x64[0 + c] = tab[id];
                        x64[8 + c] = dx[id] * cellx;
                        x64[16 + c] = dy[id] * celly;
                        x64[24 + c] = dz[id] * cellz;
                        x64[32 + c] = dxy[id] * cellx * celly;
                        x64[40 + c] = dxz[id] * cellx * cellz;
                        x64[48 + c] = dyz[id] * celly * cellz;
                        x64[56 + c] = dxyz[id] * cellx * celly * cellz;
                    }
                    tricubic_coeff(x64, &coeffs[((ix * len[1] + iy) * len[2] + iz) * 64]);
                }
    }

    void build(const pt_field &f) {
        ax[0].assign(f.x, f.x + f.nx);
        ax[1].assign(f.y, f.y + f.ny);
        ax[2].assign(f.z, f.z + f.nz);
        const double *src[4] = {f.bx, f.by, f.bz, f.v};
        size_t tot = (size_t)f.nx * f.ny * f.nz;
        for (int c = 0; c < 4; ++c)
            if (src[c]) preinterpol(std::vector<double>(src[c], src[c] + tot), coeff[c]);
    }

    /* TabField3::Interpolate (src/field_3d.cpp:487-513): outside the grid the
     * outputs are left untouched. */
    void interpolate(double x, double y, double z, const std::vector<double> &cf, double &F, double *dF) const {
        double r[3] = {x, y, z}, dist[3];
        size_t index[3];
        for (int i = 0; i < 3; ++i) {
            auto it = std::upper_bound(ax[i].begin(), ax[i].end(), r[i]);
            if (it == ax[i].end() || it == ax[i].begin()) return;
            auto low = it - 1;
            index[i] = (size_t)(low - ax[i].begin());
            dist[i] = *it - *low;
            r[i] = (r[i] - *low) / dist[i];
        }
        if (!cf.empty()) {
            size_t l1 = ax[1].size() - 1, l2 = ax[2].size() - 1;
            const double *a = &cf[((index[0] * l1 + index[1]) * l2 + index[2]) * 64];
            F = tricubic_value(a, r[0], r[1], r[2]);
            if (dF) {
                dF[0] = tricubic_deriv(a, r[0], r[1], r[2], 1, 0, 0) / dist[0];
                dF[1] = tricubic_deriv(a, r[0], r[1], r[2], 0, 1, 0) / dist[1];
                dF[2] = tricubic_deriv(a, r[0], r[1], r[2], 0, 0, 1) / dist[2];
            }
        }
    }
};

/* ------------------------------------------------------------------ */
/* ALGLIB spline1dbuildcubic (parabolically terminated ends) and spline1dcalc
 * (alglib-3.15.0/cpp/src/interpolation.cpp: spline1dbuildhermite
 * 23642-23710, spline1dcalc 23850-23912), as IntegrateSpin interpolates the
 * precession axis (src/tracking.cpp:404-421) and SpinDerivs reads it
 * (src/particle.cpp:180-184).                                             */
/* ------------------------------------------------------------------ */
struct Spline1 {
    std::vector<double> x, c; /* nodes; per interval c0, c1, c2, c3 */
    void build(int n, const double *xs, const double *ys) {
        x.assign(xs, xs + n);
        std::vector<double> d(n);
        spline_derivs(n, xs, ys, d.data());
        c.assign((size_t)4 * (n - 1), 0.0);
        for (int i = 0; i + 1 < n; ++i) {
            const double delta = xs[i + 1] - xs[i], delta2 = delta * delta, delta3 = delta * delta2;
            c[4 * i + 0] = ys[i];
            c[4 * i + 1] = d[i];
            c[4 * i + 2] = (3 * (ys[i + 1] - ys[i]) - 2 * d[i] * delta - d[i + 1] * delta) / delta2;
            c[4 * i + 3] = (2 * (ys[i] - ys[i + 1]) + d[i] * delta + d[i + 1] * delta) / delta3;
        }
    }
    double calc(double t) const {
        int l = 0, r = (int)x.size() - 1;
        while (l != r - 1) {
            const int m = (l + r) / 2;
            if (x[m] >= t) r = m;
            else l = m;
        }
        const double u = t - x[l];
        const double *k = &c[4 * l];
        return k[0] + u * (k[1] + u * (k[2] + u * k[3]));
    }
};

/* ------------------------------------------------------------------ */
/* TabField (src/field_2d.cpp:232-399): ALGLIB bicubic spline2d in (r, z),
 * restated from alglib-3.15.0/cpp/src/interpolation.cpp:
 *   spline2dbuildbicubicv / spline2d_bicubiccalcderivatives (44925-45080,
 *   46791-46880): d/dr along every z row, d/dz along every r column, d2/drdz
 *   along the rows of d/dz, each from spline1dbuildcubic with parabolically
 *   terminated ends (the derivatives of spline_derivs) read back with
 *   spline1ddiff at the nodes (spline1dbuildhermite 23642-23710, spline1ddiff
 *   23914-23975: every node but the first takes the left piece's derivative
 *   at its right end);
 *   spline2dcalc (43381-43537) and spline2ddiff (43538-43700): the cell
 *   l with x[l] < v <= x[l+1] by bisection, the Hermite basis scaled by the
 *   cell widths, the 16 products summed in the library's order.            */
/* ------------------------------------------------------------------ */
struct Tab2 {
    std::vector<double> r, z;            /* axes (ALGLIB's x and y) */
    std::vector<double> t[7];            /* Br, Bphi, Bz, V, Er, Ephi, Ez: 4 tables f, fx, fy, fxy of nr*nz each, [iz][ir] */
    double r_lo = 0, r_hi = 0, z_lo = 0, z_hi = 0;

    /* spline1ddiff of spline1dbuildcubic(x, y) at every node */
    static void node_slopes(int n, const double *x, const double *y, double *ds) {
        std::vector<double> d(n);
        spline_derivs(n, x, y, d.data());
        ds[0] = d[0];
        for (int j = 1; j < n; ++j) {
            const double delta = x[j] - x[j - 1], delta2 = delta * delta, delta3 = delta * delta2;
            const double c1 = d[j - 1];
            const double c2 = (3 * (y[j] - y[j - 1]) - 2 * d[j - 1] * delta - d[j] * delta) / delta2;
            const double c3 = (2 * (y[j - 1] - y[j]) + d[j - 1] * delta + d[j] * delta) / delta3;
            const double u = x[j] - x[j - 1];
            ds[j] = c1 + 2 * u * c2 + 3 * (u * u) * c3;
        }
    }

    void build_one(const double *src /* [ir][iz] */, std::vector<double> &out) const {
        const int m = (int)r.size(), n = (int)z.size();
        out.assign((size_t)4 * m * n, 0.0);
        double *F = out.data(), *DX = F + (size_t)m * n, *DY = DX + (size_t)m * n, *DXY = DY + (size_t)m * n;
        for (int ir = 0; ir < m; ++ir)
            for (int iz = 0; iz < n; ++iz) F[(size_t)iz * m + ir] = src[(size_t)ir * n + iz];
        std::vector<double> row(std::max(m, n)), ds(std::max(m, n));
        for (int iz = 0; iz < n; ++iz) { /* dF/dr */
            for (int ir = 0; ir < m; ++ir) row[ir] = F[(size_t)iz * m + ir];
            node_slopes(m, r.data(), row.data(), ds.data());
            for (int ir = 0; ir < m; ++ir) DX[(size_t)iz * m + ir] = ds[ir];
        }
        for (int ir = 0; ir < m; ++ir) { /* dF/dz */
            for (int iz = 0; iz < n; ++iz) row[iz] = F[(size_t)iz * m + ir];
            node_slopes(n, z.data(), row.data(), ds.data());
            for (int iz = 0; iz < n; ++iz) DY[(size_t)iz * m + ir] = ds[iz];
        }
        for (int iz = 0; iz < n; ++iz) { /* d2F/drdz */
            for (int ir = 0; ir < m; ++ir) row[ir] = DY[(size_t)iz * m + ir];
            node_slopes(m, r.data(), row.data(), ds.data());
            for (int ir = 0; ir < m; ++ir) DXY[(size_t)iz * m + ir] = ds[ir];
        }
    }

    void build(const pt_field &f) {
        r.assign(f.x, f.x + f.nx);
        z.assign(f.z, f.z + f.nz);
        const double *src[7] = {f.bx, f.by, f.bz, f.v, f.er, f.ephi, f.ez};
        const bool etab = f.er || f.ephi || f.ez; /* an E map replaces the potential (src/field_2d.cpp:262-283) */
        for (int c = 0; c < 7; ++c)
            if (src[c] && !(c == 3 && etab)) build_one(src[c], t[c]);
        /* TabField::CheckTab (src/field_2d.cpp:193-200) and the range of BField/EField */
        const double rdist = r[1] - r[0], zdist = z[1] - z[0];
        r_lo = r[0];
        z_lo = z[0];
        r_hi = r_lo + rdist * (double)(f.nx - 1);
        z_hi = z_lo + zdist * (double)(f.nz - 1);
    }
    bool in_range(double rr, double zz) const { return rr >= r_lo && rr < r_hi && zz >= z_lo && zz < z_hi; }
    bool has(int c) const { return !t[c].empty(); }

    static int cell(const std::vector<double> &ax, double v) {
        int l = 0, h = (int)ax.size() - 1;
        while (l != h - 1) {
            const int k = (l + h) / 2;
            if (ax[k] >= v) h = k;
            else l = k;
        }
        return l;
    }

    /* spline2dcalc */
    double calc(int c, double x, double y) const {
        const int m = (int)r.size(), n = (int)z.size();
        const int ix = cell(r, x), iy = cell(z, y);
        const double dt = 1.0 / (r[ix + 1] - r[ix]), t_ = (x - r[ix]) * dt;
        const double du = 1.0 / (z[iy + 1] - z[iy]), u = (y - z[iy]) * du;
        const double *F = t[c].data();
        const size_t sfx = (size_t)m * n, sfy = 2 * sfx, sfxy = 3 * sfx;
        const size_t s1 = (size_t)m * iy + ix, s2 = s1 + 1, s3 = (size_t)m * (iy + 1) + ix, s4 = s3 + 1;
        const double t2 = t_ * t_, t3 = t_ * t2, u2 = u * u, u3 = u * u2;
        double ht00 = 2 * t3 - 3 * t2 + 1, ht10 = t3 - 2 * t2 + t_, ht01 = -2 * t3 + 3 * t2, ht11 = t3 - t2;
        double hu00 = 2 * u3 - 3 * u2 + 1, hu10 = u3 - 2 * u2 + u, hu01 = -2 * u3 + 3 * u2, hu11 = u3 - u2;
        ht10 = ht10 / dt; ht11 = ht11 / dt; hu10 = hu10 / du; hu11 = hu11 / du;
        double v = 0;
        v = v + F[s1] * ht00 * hu00 + F[s2] * ht01 * hu00 + F[s3] * ht00 * hu01 + F[s4] * ht01 * hu01;
        v = v + F[sfx + s1] * ht10 * hu00 + F[sfx + s2] * ht11 * hu00 + F[sfx + s3] * ht10 * hu01 + F[sfx + s4] * ht11 * hu01;
        v = v + F[sfy + s1] * ht00 * hu10 + F[sfy + s2] * ht01 * hu10 + F[sfy + s3] * ht00 * hu11 + F[sfy + s4] * ht01 * hu11;
        v = v + F[sfxy + s1] * ht10 * hu10 + F[sfxy + s2] * ht11 * hu10 + F[sfxy + s3] * ht10 * hu11 + F[sfxy + s4] * ht11 * hu11;
        return v;
    }

    /* spline2ddiff: value, d/dr, d/dz (d2/drdz is not used by TabField) */
    void diff(int c, double x, double y, double &f, double &fx, double &fy) const {
        const int m = (int)r.size(), n = (int)z.size();
        const int ix = cell(r, x), iy = cell(z, y);
        const double t_ = (x - r[ix]) / (r[ix + 1] - r[ix]), dt = 1.0 / (r[ix + 1] - r[ix]);
        const double u = (y - z[iy]) / (z[iy + 1] - z[iy]), du = 1.0 / (z[iy + 1] - z[iy]);
        const double *F = t[c].data();
        const size_t sfx = (size_t)m * n, sfy = 2 * sfx, sfxy = 3 * sfx;
        const size_t s1 = (size_t)m * iy + ix, s2 = s1 + 1, s3 = (size_t)m * (iy + 1) + ix, s4 = s3 + 1;
        const double t2 = t_ * t_, t3 = t_ * t2, u2 = u * u, u3 = u * u2;
        double ht00 = 2 * t3 - 3 * t2 + 1, ht10 = t3 - 2 * t2 + t_, ht01 = -2 * t3 + 3 * t2, ht11 = t3 - t2;
        double hu00 = 2 * u3 - 3 * u2 + 1, hu10 = u3 - 2 * u2 + u, hu01 = -2 * u3 + 3 * u2, hu11 = u3 - u2;
        ht10 = ht10 / dt; ht11 = ht11 / dt; hu10 = hu10 / du; hu11 = hu11 / du;
        double dht00 = 6 * t2 - 6 * t_, dht10 = 3 * t2 - 4 * t_ + 1, dht01 = -6 * t2 + 6 * t_, dht11 = 3 * t2 - 2 * t_;
        double dhu00 = 6 * u2 - 6 * u, dhu10 = 3 * u2 - 4 * u + 1, dhu01 = -6 * u2 + 6 * u, dhu11 = 3 * u2 - 2 * u;
        dht00 = dht00 * dt; dht01 = dht01 * dt; dhu00 = dhu00 * du; dhu01 = dhu01 * du;
        f = fx = fy = 0;
        const size_t blk[4] = {0, sfx, sfy, sfxy};
        for (int b = 0; b < 4; ++b) {
            const double v0 = F[blk[b] + s1], v1 = F[blk[b] + s2], v2 = F[blk[b] + s3], v3 = F[blk[b] + s4];
            const double p0 = (b & 1) ? ht10 : ht00, p1 = (b & 1) ? ht11 : ht01;    /* x data: value or slope */
            const double q0 = (b & 2) ? hu10 : hu00, q1 = (b & 2) ? hu11 : hu01;
            const double dp0 = (b & 1) ? dht10 : dht00, dp1 = (b & 1) ? dht11 : dht01;
            const double dq0 = (b & 2) ? dhu10 : dhu00, dq1 = (b & 2) ? dhu11 : dhu01;
            f = f + v0 * p0 * q0 + v1 * p1 * q0 + v2 * p0 * q1 + v3 * p1 * q1;
            fx = fx + v0 * dp0 * q0 + v1 * dp1 * q0 + v2 * dp0 * q1 + v3 * dp1 * q1;
            fy = fy + v0 * p0 * dq0 + v1 * p1 * dq0 + v2 * p0 * dq1 + v3 * p1 * dq1;
        }
    }

    /* cos(phi), sin(phi) of phi = atan2(y, x), formed as x/r and y/r (equal up to
     * rounding, (1, 0) on the axis where atan2(0, 0) = 0) */
    static void axis_angle(double x, double y, double rr, double &cp, double &sp) {
        if (rr > 0) { cp = x / rr; sp = y / rr; }
        else { cp = 1.0; sp = 0.0; }
    }

    /* TabField::BField (src/field_2d.cpp:289-335) */
    void bfield(double x, double y, double zz, double B[3], double dB[3][3]) const {
        const double rr = sqrt(x * x + y * y);
        if (!in_range(rr, zz)) return;
        double cp, sp;
        axis_angle(x, y, rr, cp, sp);
        double Br = 0, Bphi = 0, Bz = 0;
        if (dB) {
            double dBrdr = 0, dBrdz = 0, dBphidr = 0, dBphidz = 0, dBzdr = 0, dBzdz = 0;
            if (has(0)) diff(0, rr, zz, Br, dBrdr, dBrdz);
            if (has(1)) diff(1, rr, zz, Bphi, dBphidr, dBphidz);
            if (rr > 0) {
                dB[0][0] = dBrdr * cp * cp - dBphidr * cp * sp + (Br * sp * sp + Bphi * cp * sp) / rr;
                dB[0][1] = dBrdr * cp * sp - dBphidr * sp * sp - (Br * cp * sp + Bphi * cp * cp) / rr;
                dB[1][0] = dBrdr * cp * sp + dBphidr * cp * cp - (Br * cp * sp - Bphi * sp * sp) / rr;
                dB[1][1] = dBrdr * sp * sp + dBphidr * cp * sp + (Br * cp * cp - Bphi * cp * sp) / rr;
            }
            dB[0][2] = dBrdz * cp - dBphidz * sp;
            dB[1][2] = dBrdz * sp + dBphidz * cp;
            if (has(2)) {
                diff(2, rr, zz, Bz, dBzdr, dBzdz);
                dB[2][0] = dBzdr * cp;
                dB[2][1] = dBzdr * sp;
                dB[2][2] = dBzdz;
            }
        } else {
            if (has(0)) Br = calc(0, rr, zz);
            if (has(1)) Bphi = calc(1, rr, zz);
            if (has(2)) Bz = calc(2, rr, zz);
        }
        B[0] = Br * cp - Bphi * sp;
        B[1] = Br * sp + Bphi * cp;
        B[2] = Bz;
    }

    /* TabField::EField (src/field_2d.cpp:337-399) */
    void efield(double x, double y, double zz, double &V, double E[3]) const {
        const double rr = sqrt(x * x + y * y);
        if (!in_range(rr, zz)) return;
        double cp, sp;
        axis_angle(x, y, rr, cp, sp);
        if (has(4) || has(5) || has(6)) {
            const double Er = has(4) ? calc(4, rr, zz) : 0.0, Ephi = has(5) ? calc(5, rr, zz) : 0.0;
            E[0] = Er * cp - Ephi * sp;
            E[1] = Er * sp + Ephi * cp;
            E[2] = has(6) ? calc(6, rr, zz) : 0.0;
        } else if (has(3)) {
            double dVdr, dVdz;
            diff(3, rr, zz, V, dVdr, dVdz);
            E[0] = -dVdr * cp;
            E[1] = -dVdr * sp;
            E[2] = -dVdz;
        }
    }
};

struct Field {
    int type = 0;
    double bscale = 1, escale = 1;
    double xmax = 0, xmin = 0, ymax = 0, ymin = 0, zmax = 0, zmin = 0, bw = 0;
    Tab3 tab;
    Tab2 tab2;
    double e[3] = {0, 0, 0};
    /* HarmonicExpandedBField (src/harmonicfields.cpp:50-829): (l, m, G) terms and offset */
    std::vector<int> hl, hm;
    std::vector<double> hg;
    double offset[3] = {0, 0, 0};
    double sol_a = 0, sol_b = 0, sol_B0 = 0; /* finite solenoid (include/pt_solenoid.h) */

    /* TFieldBoundaryBox (src/field.cpp:48-125) */
    bool has_bounds() const { return xmin < xmax && ymin < ymax && zmin < zmax; }
    bool in_bounds(double x, double y, double z) const {
        if (!has_bounds()) return true;
        return x >= xmin && x < xmax && y >= ymin && y < ymax && z >= zmin && z < zmax;
    }
    static double smthr(double x) { return ((6 * x - 15) * x + 10) * x * x * x; }
    static double smthr_der(double x) { return ((30 * x - 60) * x + 30) * x * x; }
    void scale_at_bounds(double x, double y, double z, double &F, double *dF) const {
        if (!has_bounds() || (F == 0 && dF == nullptr) || (F == 0 && dF[0] == 0 && dF[1] == 0 && dF[2] == 0)) return;
        if (!in_bounds(x, y, z)) {
            F = 0.;
            if (dF) dF[0] = dF[1] = dF[2] = 0.;
        } else if (bw > 0) {
            double Fscale = 1.;
            double dFadd[3] = {0., 0., 0.};
            double lo[3] = {(x - xmin) / bw, (y - ymin) / bw, (z - zmin) / bw};
            double hi[3] = {(xmax - x) / bw, (ymax - y) / bw, (zmax - z) / bw};
            for (int i = 0; i < 3; ++i) {
                if (0 <= lo[i] && lo[i] <= 1) {
                    Fscale *= smthr(lo[i]);
                    if (dF) dFadd[i] += F * smthr_der(lo[i]) / bw / smthr(lo[i]);
                } else if (0 <= hi[i] && hi[i] <= 1) {
                    Fscale *= smthr(hi[i]);
                    if (dF) dFadd[i] += -F * smthr_der(hi[i]) / bw / smthr(hi[i]);
                }
            }
            if (Fscale != 1.) {
                F *= Fscale;
                if (dF)
                    for (int i = 0; i < 3; i++) dF[i] = dF[i] * Fscale + dFadd[i] * Fscale;
            }
        }
    }

    /* TFieldContainer::BField (src/field.cpp:139-155) */
    void bfield(double x, double y, double z, double B[3], double dB[3][3]) const {
        for (int i = 0; i < 3; ++i) {
            B[i] = 0;
            if (dB) for (int j = 0; j < 3; ++j) dB[i][j] = 0;
        }
        if (!in_bounds(x, y, z) || bscale == 0.) return;
        if (type == PT_FIELD_TAB3D) {
            for (int i = 0; i < 3; ++i) tab.interpolate(x, y, z, tab.coeff[i], B[i], dB ? dB[i] : nullptr);
        } else if (type == PT_FIELD_TAB2D) {
            tab2.bfield(x, y, z, B, dB);
        } else if (type == PT_FIELD_SOLENOID) {
            pts_solenoid_field(sol_a, sol_b, sol_B0, x - offset[0], y - offset[1], z - offset[2], B, dB);
        } else if (type == PT_FIELD_HARMONIC) {
            const double xo = x + offset[0], yo = y + offset[1], zo = z + offset[2];
            for (size_t k = 0; k < hg.size(); ++k)
                if (hg[k] != 0.) harmonic_term(hl[k], hm[k], hg[k], xo, yo, zo, B, dB);
        } else {
            return; /* the uniform E field has no B */
        }
        for (int i = 0; i < 3; ++i) { /* TFieldScaler::scaleVectorField (src/field.cpp:12-32) */
            B[i] *= bscale;
            if (dB) for (int j = 0; j < 3; ++j) dB[i][j] *= bscale;
        }
        for (int i = 0; i < 3; ++i) scale_at_bounds(x, y, z, B[i], dB ? dB[i] : nullptr);
    }

    /* TFieldContainer::EField (src/field.cpp:157-169) */
    void efield(double x, double y, double z, double &V, double E[3]) const {
        V = 0; E[0] = E[1] = E[2] = 0;
        if (!in_bounds(x, y, z) || escale == 0.) return;
        if (type == PT_FIELD_UNIFORM_E) {
            /* TEDMStaticEField::EField (src/edmfields.cpp:181-187) */
            E[0] = e[0]; E[1] = e[1]; E[2] = e[2];
            V = E[2] * z;
        } else if (type == PT_FIELD_TAB3D) {
            if (tab.coeff[3].empty()) return; /* no potential column: zero field */
            double dV[3] = {0, 0, 0};
            tab.interpolate(x, y, z, tab.coeff[3], V, dV);
            for (int i = 0; i < 3; ++i) E[i] = -dV[i];
        } else if (type == PT_FIELD_TAB2D) {
            tab2.efield(x, y, z, V, E);
        } else {
            return;
        }
        V *= escale;
        for (int i = 0; i < 3; ++i) E[i] *= escale;
        scale_at_bounds(x, y, z, V, E);
    }
};

/* ------------------------------------------------------------------ */
/* Geometry                                                            */
/* ------------------------------------------------------------------ */
struct Tri { double a[3], b[3], c[3], n[3]; double lo[3], hi[3]; int solid; };

struct Coll { double s; double normal[3]; int solid; uint32_t id; double distnormal; bool ignored; };

inline double orient3d(const double *a, const double *b, const double *c, const double *d) {
    double adx = a[0] - d[0], bdx = b[0] - d[0], cdx = c[0] - d[0];
    double ady = a[1] - d[1], bdy = b[1] - d[1], cdy = c[1] - d[1];
    double adz = a[2] - d[2], bdz = b[2] - d[2], cdz = c[2] - d[2];
    return adx * (bdy * cdz - bdz * cdy) + bdx * (cdy * adz - cdz * ady) + cdx * (ady * bdz - adz * bdy);
}
inline bool lex_less(const double *u, const double *v) {
    if (u[0] != v[0]) return u[0] < v[0];
    if (u[1] != v[1]) return u[1] < v[1];
    return u[2] < v[2];
}
/* orientation of segment (p,q) against edge (u,v), computed in a canonical
 * vertex order so neighbouring triangles see exactly opposite signs */
inline double edge_orient(const double *p, const double *q, const double *u, const double *v) {
    if (lex_less(v, u)) return -orient3d(p, q, v, u);
    return orient3d(p, q, u, v);
}

/* closed segment vs closed triangle (CGAL do_intersect/intersection semantics
 * for Segment_3 x Triangle_3).  Returns 1 with parameter s on a point hit,
 * 0 on no hit, -1 when the segment lies in the triangle's plane. */
inline int seg_tri(const double *p, const double *q, const Tri &t, double &s) {
    double dp = orient3d(t.a, t.b, t.c, p), dq = orient3d(t.a, t.b, t.c, q);
    if ((dp > 0 && dq > 0) || (dp < 0 && dq < 0)) return 0;
    if (dp == 0 && dq == 0) return -1;
    double e1 = edge_orient(p, q, t.a, t.b), e2 = edge_orient(p, q, t.b, t.c), e3 = edge_orient(p, q, t.c, t.a);
    bool neg = (e1 < 0) || (e2 < 0) || (e3 < 0), pos = (e1 > 0) || (e2 > 0) || (e3 > 0);
    if (neg && pos) return 0;
    s = dp / (dp - dq);
    return 1;
}

struct Solid { uint32_t id; int mat; std::vector<double> ign;
    /* solid::is_ignored (include/geometry.h:61-66) */
    bool ignored(double t) const {
        for (size_t i = 0; i + 1 < ign.size(); i += 2) if (t >= ign[i] && t < ign[i + 1]) return true;
        return false;
    }
};

struct BVHNode { double lo[3], hi[3]; int left, right, first, count; };

struct Mesh {
    std::vector<Tri> tris;
    std::vector<BVHNode> nodes;
    std::vector<int> order;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    std::vector<double> slo, shi; /* per-solid boxes (one AABB tree per STL in the reference) */

    int build(int first, int count) {
        BVHNode nd;
        for (int k = 0; k < 3; ++k) { nd.lo[k] = 1e300; nd.hi[k] = -1e300; }
        for (int i = first; i < first + count; ++i)
            for (int k = 0; k < 3; ++k) {
                nd.lo[k] = std::min(nd.lo[k], tris[order[i]].lo[k]);
                nd.hi[k] = std::max(nd.hi[k], tris[order[i]].hi[k]);
            }
        int idx = (int)nodes.size();
        nodes.push_back(nd);
        if (count <= 4) {
            nodes[idx].left = nodes[idx].right = -1;
            nodes[idx].first = first; nodes[idx].count = count;
            return idx;
        }
        int axis = 0;
        double ext = -1;
        for (int k = 0; k < 3; ++k) if (nd.hi[k] - nd.lo[k] > ext) { ext = nd.hi[k] - nd.lo[k]; axis = k; }
        int mid = first + count / 2;
        std::nth_element(order.begin() + first, order.begin() + mid, order.begin() + first + count, [&](int u, int v) {
            return tris[u].lo[axis] + tris[u].hi[axis] < tris[v].lo[axis] + tris[v].hi[axis];
        });
        int l = build(first, mid - first);
        int r = build(mid, first + count - mid);
        nodes[idx].left = l; nodes[idx].right = r; nodes[idx].first = 0; nodes[idx].count = 0;
        return idx;
    }

    template <class F> void visit(const double *blo, const double *bhi, F f) const {
        if (nodes.empty()) return;
        int stack[128]; int sp = 0; stack[sp++] = 0;
        while (sp) {
            const BVHNode &nd = nodes[stack[--sp]];
            if (nd.lo[0] > bhi[0] || nd.hi[0] < blo[0] || nd.lo[1] > bhi[1] || nd.hi[1] < blo[1] || nd.lo[2] > bhi[2] || nd.hi[2] < blo[2]) continue;
            if (nd.left < 0) { for (int i = 0; i < nd.count; ++i) f(tris[order[nd.first + i]]); }
            else { stack[sp++] = nd.left; stack[sp++] = nd.right; }
        }
    }
};

struct Scene {
    Mesh mesh;
    std::vector<Solid> solids;
    std::vector<pt_material> mats;
    std::vector<Field> fields;

    /* TTriangleMesh::InBoundingBox + TGeometry::CheckSegment (include/trianglemesh.h:197-199,
     * include/geometry.h:104-106): the segment touches the box of any solid's mesh */
    bool check_segment(const double *p, const double *q) const {
        for (size_t s = 1; s < solids.size(); ++s) {
            const double *lo = &mesh.slo[3 * s], *hi = &mesh.shi[3 * s];
            if (lo[0] > hi[0]) continue;
            if (seg_box(p, q, lo, hi)) return true;
        }
        return false;
    }
    static bool seg_box(const double *p, const double *q, const double *lo, const double *hi) {
        double t0 = 0, t1 = 1;
        for (int k = 0; k < 3; ++k) {
            double d = q[k] - p[k];
            if (d == 0) { if (p[k] < lo[k] || p[k] > hi[k]) return false; continue; }
            double ta = (lo[k] - p[k]) / d, tb = (hi[k] - p[k]) / d;
            if (ta > tb) std::swap(ta, tb);
            t0 = std::max(t0, ta); t1 = std::min(t1, tb);
            if (t0 > t1) return false;
        }
        return true;
    }

    /* TTriangleMesh::Collision + TGeometry::GetCollisions (src/trianglemesh.cpp:134-164,
     * src/geometry.cpp:139-148).  Returns false on a coplanar segment (CGAL error). */
    bool collisions(double x1, const double *p, double x2, const double *q, std::vector<Coll> &out) const {
        out.clear();
        double blo[3], bhi[3];
        for (int k = 0; k < 3; ++k) { blo[k] = std::min(p[k], q[k]); bhi[k] = std::max(p[k], q[k]); }
        bool ok = true;
        mesh.visit(blo, bhi, [&](const Tri &t) {
            if (t.lo[0] > bhi[0] || t.hi[0] < blo[0] || t.lo[1] > bhi[1] || t.hi[1] < blo[1] || t.lo[2] > bhi[2] || t.hi[2] < blo[2]) return;
            double s;
            int r = seg_tri(p, q, t, s);
            if (r < 0) { ok = false; return; }
            if (r == 0) return;
            Coll c;
            c.s = s;
            for (int k = 0; k < 3; ++k) c.normal[k] = t.n[k];
            c.solid = t.solid;
            c.id = solids[t.solid].id;
            c.distnormal = (q[0] - p[0]) * t.n[0] + (q[1] - p[1]) * t.n[1] + (q[2] - p[2]) * t.n[2];
            c.ignored = solids[t.solid].ignored(x1 + (x2 - x1) * s);
            out.push_back(c);
        });
        std::sort(out.begin(), out.end(), [](const Coll &a, const Coll &b) {
            if (a.s == b.s) return a.id > b.id;
            return a.s < b.s;
        });
        return ok;
    }

    /* TTriangleMesh::GetSolids (include/trianglemesh.h:181-188): odd number of
     * triangles of a solid hit by the +z ray from p */
    uint64_t point_solids(const double *p) const {
        double q[3] = {p[0], p[1], std::max(mesh.hi[2], p[2]) + 1.0};
        double blo[3] = {p[0], p[1], p[2]}, bhi[3] = {p[0], p[1], q[2]};
        uint64_t mask = 0;
        mesh.visit(blo, bhi, [&](const Tri &t) {
            double s;
            if (seg_tri(p, q, t, s) == 1) mask ^= (1ull << t.solid);
        });
        return mask;
    }
};

} // namespace

/* the event logs of the last pto_track call (TLogger::PrintHit /
 * PrintSnapshot records, the library's record layout) */
struct pto_ctx {
    Scene sc;
    std::vector<double> hits, snaps, tracks, spins;
};

/* ------------------------------------------------------------------ */
/* Particle tracking                                                   */
/* ------------------------------------------------------------------ */
namespace {

typedef double state9[9];

struct Species { double q, m, mu, gamma, mkg, inv_mkg, fgrav, mu_over_e, q_over_e, mc2, mg; int kind; };
Species species_of(int s) {
    if (s == PT_PROTON) return {PT_PROTON_Q, PT_PROTON_M, PT_PROTON_MU, PT_PROTON_GAMMA, PT_PROTON_MKG, PT_PROTON_INV_MKG, PT_PROTON_FGRAV, PT_PROTON_MU_OVER_E, PT_PROTON_Q_OVER_E, PT_PROTON_MC2, PT_PROTON_MG, s};
    if (s == PT_ELECTRON) return {PT_ELECTRON_Q, PT_ELECTRON_M, PT_ELECTRON_MU, PT_ELECTRON_GAMMA, PT_ELECTRON_MKG, PT_ELECTRON_INV_MKG, PT_ELECTRON_FGRAV, PT_ELECTRON_MU_OVER_E, PT_ELECTRON_Q_OVER_E, PT_ELECTRON_MC2, PT_ELECTRON_MG, s};
    return {PT_NEUTRON_Q, PT_NEUTRON_M, PT_NEUTRON_MU, PT_NEUTRON_GAMMA, PT_NEUTRON_MKG, PT_NEUTRON_INV_MKG, PT_NEUTRON_FGRAV, PT_NEUTRON_MU_OVER_E, PT_NEUTRON_Q_OVER_E, PT_NEUTRON_MC2, PT_NEUTRON_MG, PT_NEUTRON};
}

struct OdeintError {};

/* err^p of the step adjuster through the deterministic pow of pt_detmath.h
 * (an infinite error gives 0, as the library pow does for negative p) */
inline double det_pow(double m, double p) { return (m < 1e300) ? ptdm_pow(m, p) : 0.0; }

/* Boost.odeint dense_output_runge_kutta<controlled_runge_kutta<runge_kutta_dopri5>>
 * made by make_dense_output(eps_abs, eps_rel, stepper) (src/tracking.cpp:63).
 * Restated from the published Dormand-Prince 5(4) tableau (FSAL), odeint's
 * default_error_checker (max norm of |err_i|/(eps_abs + eps_rel*(|x_i| + |dt|*|dxdt_i|))),
 * default_step_adjuster (reject: dt *= max(0.9*err^(-1/3), 0.2); accept and
 * err<0.5: dt *= 0.9*max(err, 5^-5)^(-1/5)), the failed-step checker (500
 * tries) and odeint's dopri5 continuous extension. */
template <int N> struct Dense5 {
    double x[N], dxdt[N], xo[N], dxdto[N], k2[N], k3[N], k4[N], k5[N], k6[N];
    double t = 0, to = 0, dt = 0, eps_abs, eps_rel;
    bool deriv_init = false;
    Dense5(double ea, double er) : eps_abs(ea), eps_rel(er) {}
    void initialize(const double *x0, double t0, double dt0) {
        for (int i = 0; i < N; ++i) x[i] = x0[i];
        t = t0; dt = dt0; deriv_init = false;
    }
    template <class Sys> void do_step(Sys &sys, int64_t &n_rej) {
        if (!deriv_init) { sys(x, dxdt, t); deriv_init = true; }
        const double a2 = 1.0 / 5, a3 = 3.0 / 10, a4 = 4.0 / 5, a5 = 8.0 / 9;
        const double b21 = 1.0 / 5;
        const double b31 = 3.0 / 40, b32 = 9.0 / 40;
        const double b41 = 44.0 / 45, b42 = -56.0 / 15, b43 = 32.0 / 9;
        const double b51 = 19372.0 / 6561, b52 = -25360.0 / 2187, b53 = 64448.0 / 6561, b54 = -212.0 / 729;
        const double b61 = 9017.0 / 3168, b62 = -355.0 / 33, b63 = 46732.0 / 5247, b64 = 49.0 / 176, b65 = -5103.0 / 18656;
        const double c1 = 35.0 / 384, c3 = 500.0 / 1113, c4 = 125.0 / 192, c5 = -2187.0 / 6784, c6 = 11.0 / 84;
        const double dc1 = c1 - 5179.0 / 57600, dc3 = c3 - 7571.0 / 16695, dc4 = c4 - 393.0 / 640,
                     dc5 = c5 - (-92097.0) / 339200, dc6 = c6 - 187.0 / 2100, dc7 = -1.0 / 40;
        to = t;
        int tries = 0;
        double xt[N], out[N], dout[N], err[N];
        while (true) {
            ++tries;
            if (tries > 500) throw OdeintError();
            /* stage combinations as explicit fused multiply-add chains, term by
             * term in tableau order (the kernels evaluate the same chains) */
            for (int i = 0; i < N; ++i) xt[i] = std::fma(dt * b21, dxdt[i], x[i]);
            sys(xt, k2, t + dt * a2);
            for (int i = 0; i < N; ++i) xt[i] = std::fma(dt * b32, k2[i], std::fma(dt * b31, dxdt[i], x[i]));
            sys(xt, k3, t + dt * a3);
            for (int i = 0; i < N; ++i)
                xt[i] = std::fma(dt * b43, k3[i], std::fma(dt * b42, k2[i], std::fma(dt * b41, dxdt[i], x[i])));
            sys(xt, k4, t + dt * a4);
            for (int i = 0; i < N; ++i)
                xt[i] = std::fma(dt * b54, k4[i], std::fma(dt * b53, k3[i], std::fma(dt * b52, k2[i], std::fma(dt * b51, dxdt[i], x[i]))));
            sys(xt, k5, t + dt * a5);
            for (int i = 0; i < N; ++i)
                xt[i] = std::fma(dt * b65, k5[i], std::fma(dt * b64, k4[i], std::fma(dt * b63, k3[i],
                        std::fma(dt * b62, k2[i], std::fma(dt * b61, dxdt[i], x[i])))));
            sys(xt, k6, t + dt);
            for (int i = 0; i < N; ++i)
                out[i] = std::fma(dt * c6, k6[i], std::fma(dt * c5, k5[i], std::fma(dt * c4, k4[i],
                         std::fma(dt * c3, k3[i], std::fma(dt * c1, dxdt[i], x[i])))));
            sys(out, dout, t + dt);
            for (int i = 0; i < N; ++i)
                err[i] = std::fma(dt * dc7, dout[i], std::fma(dt * dc6, k6[i], std::fma(dt * dc5, k5[i],
                         std::fma(dt * dc4, k4[i], std::fma(dt * dc3, k3[i], (dt * dc1) * dxdt[i])))));
            double adt = std::fabs(dt), m = 0;
            for (int i = 0; i < N; ++i) {
                double e = std::fabs(err[i]) / (eps_abs + eps_rel * (1.0 * std::fabs(x[i]) + adt * std::fabs(dxdt[i])));
                m = (m < e || e != e) ? e : m; /* a NaN estimate sticks and rejects the step */
            }
            if (!(m <= 1.0)) {
                dt *= std::fmax(0.9 * (m < 1e300 ? det_pow(m, -1.0 / 3.0) : 0.0), 0.2);
                ++n_rej;
                continue;
            }
            t += dt;
            if (m < 0.5) {
                m = std::max(0.00032, m); /* 5^-5 */
                dt *= 0.9 * det_pow(m, -1.0 / 5.0);
            }
            for (int i = 0; i < N; ++i) { xo[i] = x[i]; dxdto[i] = dxdt[i]; x[i] = out[i]; dxdt[i] = dout[i]; }
            return;
        }
    }
    /* runge_kutta_dopri5::calc_state: odeint's continuous extension between the
     * last two accepted points.  Its weights b_i(theta) (odeint's
     * A b_i -/+ C X_i (+D) form with X_i linear in theta) are expanded here
     * into monomials theta..theta^5 and evaluated by Horner's rule, with one
     * division for theta; the engine evaluates the same expression. */
    void calc_state(double tt, double *y) const {
        static const double W[6][5] = {
            {1.0, -2.8605386690370884, 3.099577878709121, -1.1618105836403092, 0.013917207301610328},
            {0.0, 4.047141499642786, -6.345354046938926, 2.795465086414005, -0.04801624082496286},
            {0.0, -3.941160071112659, 10.904003027940295, -6.729317509209278, 0.4175162190483098},
            {0.0, 2.8419447015870345, -7.547675862959386, 4.957636724931253, -0.5742817428041846},
            {0.0, -1.6109886359167997, 4.218915839039518, -2.950103865566732, 0.47312904339639456},
            {0.0, 1.523601174836727, -4.329466835790622, 3.0881301470710616, -0.2822644861171672}};
        const double h = t - to;
        const double th = (tt - to) / h;
        double hb[6];
        for (int k = 0; k < 6; ++k) {
            double p = W[k][4];
            p = std::fma(p, th, W[k][3]);
            p = std::fma(p, th, W[k][2]);
            p = std::fma(p, th, W[k][1]);
            p = std::fma(p, th, W[k][0]);
            hb[k] = h * (p * th);
        }
        for (int i = 0; i < N; ++i)
            y[i] = std::fma(hb[5], dxdt[i], std::fma(hb[4], k6[i], std::fma(hb[3], k5[i], std::fma(hb[2], k4[i],
                   std::fma(hb[1], k3[i], std::fma(hb[0], dxdto[i], xo[i]))))));
    }
};

/* principal complex square root of (a + ib), branch cut on the negative real
 * axis with the sign of b selecting the side (as std::sqrt(std::complex)). */
inline void csqrt(double a, double b, double &re, double &im) {
    double m = std::sqrt(a * a + b * b);
    if (a >= 0) {
        double t = std::sqrt((a + m) * 0.5);
        re = t;
        im = (t == 0) ? b : b / (2 * t);
    } else {
        double t = std::sqrt((m - a) * 0.5);
        re = std::fabs(b) / (2 * t);
        im = std::copysign(t, b);
    }
}

/* RotateVector (src/globals.cpp:40-64): rotate v into the frame whose z axis
 * is n and whose x axis is the projection of x onto the plane normal to n
 * (CGAL Plane_3::base1() when x is absent or parallel to n). */
void rotate_vector(double v[3], const double n[3], const double *x) {
    double nn = n[0] * n[0] + n[1] * n[1] + n[2] * n[2];
    double xv[3];
    auto base1 = [&](double *b) {
        double a = std::fabs(n[0]), bb = std::fabs(n[1]), c = std::fabs(n[2]);
        if (n[0] == 0) { b[0] = 1; b[1] = 0; b[2] = 0; }
        else if (n[1] == 0) { b[0] = 0; b[1] = 1; b[2] = 0; }
        else if (n[2] == 0) { b[0] = 0; b[1] = 0; b[2] = 1; }
        else if (a <= bb && a <= c) { b[0] = 0; b[1] = -n[2]; b[2] = n[1]; }
        else if (bb <= a && bb <= c) { b[0] = -n[2]; b[1] = 0; b[2] = n[0]; }
        else { b[0] = -n[1]; b[1] = n[0]; b[2] = 0; }
    };
    if (x == nullptr) base1(xv);
    else {
        double lam = (n[0] * x[0] + n[1] * x[1] + n[2] * x[2]) / nn;
        for (int k = 0; k < 3; ++k) xv[k] = x[k] - lam * n[k];
        if (xv[0] * xv[0] + xv[1] * xv[1] + xv[2] * xv[2] < 1e-30) base1(xv);
    }
    double xl = std::sqrt(xv[0] * xv[0] + xv[1] * xv[1] + xv[2] * xv[2]);
    double zl = std::sqrt(nn);
    double xu[3] = {xv[0] / xl, xv[1] / xl, xv[2] / xl}, zu[3] = {n[0] / zl, n[1] / zl, n[2] / zl};
    double yu[3] = {zu[1] * xu[2] - zu[2] * xu[1], zu[2] * xu[0] - zu[0] * xu[2], zu[0] * xu[1] - zu[1] * xu[0]};
    double r[3];
    for (int k = 0; k < 3; ++k) r[k] = xu[k] * v[0] + yu[k] * v[1] + zu[k] * v[2];
    v[0] = r[0]; v[1] = r[1]; v[2] = r[2];
}

struct SolidRef { int idx; bool ignored; };

/* ------------------------------------------------------------------ */
/* MicroRoughness (src/microroughness.cpp:15-134), restated with the
 * reference's complex amplitudes and the library Bessel function.
 * MRProb integrates like Boost.odeint's integrate() (Dormand-Prince 5(4)
 * dense output, tolerances 1e-6, first step 0.01, last step shortened to
 * the end); MRDistMax takes the maximum from a grid and golden-section
 * refinement where the reference runs ALGLIB's conjugate-gradient
 * minimiser from pi/4 (a local search that can stop below the maximum).  */
/* ------------------------------------------------------------------ */
namespace mr {

/* MR::MRValid (src/microroughness.cpp:15-33) */
bool valid(const double v[3], double Estep, double b, double w) {
    if (b == 0 || w == 0) return false;
    double v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    double E = 0.5 * PT_M_N * v2;
    double ki = std::sqrt(2 * PT_M_N * E) * PT_ELE_E / PT_HBAR;
    if (Estep >= 0) {
        double kc = std::sqrt(2 * PT_M_N * Estep) * PT_ELE_E / PT_HBAR;
        return 2 * b * ki < 2 && 2 * b * kc < 2;
    }
    double kt = std::sqrt(2 * PT_M_N * (E - Estep)) * PT_ELE_E / PT_HBAR;
    return 2 * b * ki < 2 && 2 * b * kt < 2;
}

/* MR::MRDist (src/microroughness.cpp:35-85) */
double dist(bool transmit, bool integral, const double v[3], const double normal[3], double Estep, double b, double w,
            double theta, double phi) {
    if (theta < 0 || theta > PT_PI / 2) return 0;
    double v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    double vnormal = v[0] * normal[0] + v[1] * normal[1] + v[2] * normal[2];
    double E = 0.5 * PT_M_N * v2;
    if (transmit && E <= Estep) return 0;
    double ki = std::sqrt(2 * PT_M_N * E) * PT_ELE_E / PT_HBAR;
    std::complex<double> kc = std::sqrt(2 * PT_M_N * std::complex<double>(Estep, 0.)) * PT_ELE_E / PT_HBAR;
    double kt = 0;
    double costheta_i = std::fabs(vnormal / std::sqrt(v2));
    std::complex<double> Si = 2 * costheta_i / (costheta_i + std::sqrt(costheta_i * costheta_i - kc * kc / ki / ki));
    std::complex<double> So;
    double ct = std::cos(theta), st = std::sin(theta);
    if (transmit) {
        kt = std::sqrt(2 * PT_M_N * (E - Estep)) * PT_ELE_E / PT_HBAR;
        if (-std::real(kc * kc) / kt / kt > ct * ct) return 0;
        So = 2 * ct / (ct + std::sqrt(ct * ct + kc * kc / kt / kt));
    } else {
        So = 2 * ct / (ct + std::sqrt(ct * ct - kc * kc / ki / ki));
    }
    double theta_i = std::acos(costheta_i), sti = std::sin(theta_i);
    double Fmu;
    if (!integral && !transmit)
        Fmu = std::exp(-w * w / 2 * ki * ki * (sti * sti + st * st - 2 * sti * st * std::cos(phi)));
    else if (!integral && transmit)
        Fmu = std::exp(-w * w / 2 * (ki * ki * sti * sti + kt * kt * st * st - 2 * ki * kt * sti * st * std::cos(phi)));
    else if (!transmit)
        Fmu = std::exp(-w * w / 2 * ki * ki * (sti * sti + st * st)) * 2 * PT_PI * std::cyl_bessel_i(0.0, w * w * ki * ki * sti * st);
    else
        Fmu = std::exp(-w * w / 2 * (ki * ki * sti * sti + kt * kt * st * st)) * 2 * PT_PI *
              std::cyl_bessel_i(0.0, w * w * ki * kt * sti * st);
    double factor = std::real(kc * kc * kc * kc) * b * b * w * w / 8 / PT_PI / costheta_i;
    if (transmit) factor *= kt / ki;
    if (integral) factor *= st;
    return factor * std::norm(Si) * std::norm(So) * Fmu;
}

/* MR::MRProb (src/microroughness.cpp:101-107); ok = false when a step
 * fails 500 times (odeint throws) */
double prob(bool transmit, const double v[3], const double normal[3], double Estep, double b, double w, bool &ok) {
    auto f = [&](double th) { return dist(transmit, true, v, normal, Estep, b, w, th, 0); };
    const double T = PT_PI / 2, eps = std::numeric_limits<double>::epsilon();
    static const double c3 = 3.0 / 10, c4 = 4.0 / 5, c5 = 8.0 / 9;
    static const double b1 = 35.0 / 384, b3 = 500.0 / 1113, b4 = 125.0 / 192, b5 = -2187.0 / 6784, b6 = 11.0 / 84;
    static const double e1 = 35.0 / 384 - 5179.0 / 57600, e3 = 500.0 / 1113 - 7571.0 / 16695, e4 = 125.0 / 192 - 393.0 / 640,
                        e5 = -2187.0 / 6784 + 92097.0 / 339200, e6 = 11.0 / 84 - 187.0 / 2100, e7 = -1.0 / 40;
    double t = 0, x = 0, dt = 0.01, d0 = f(0.0);
    long steps = 0;
    while (T - t > eps) {
        while (t + dt - T <= eps) {
            for (int tries = 0;; ++tries) {
                if (tries >= 500) { ok = false; return x; }
                double k3 = f(t + dt * c3), k4 = f(t + dt * c4), k5 = f(t + dt * c5), k6 = f(t + dt);
                double xn = x + dt * (b1 * d0 + b3 * k3 + b4 * k4 + b5 * k5 + b6 * k6);
                double xe = dt * (e1 * d0 + e3 * k3 + e4 * k4 + e5 * k5 + e6 * k6 + e7 * k6);
                double err = std::fabs(xe) / (1e-6 + 1e-6 * (std::fabs(x) + std::fabs(dt) * std::fabs(d0)));
                if (!(err <= 1.0)) {
                    if (err != err) err = 1e300;
                    dt *= std::max(0.9 * std::pow(err, -1.0 / 3.0), 0.2);
                    continue;
                }
                t += dt;
                x = xn;
                d0 = k6;
                if (err < 0.5) dt *= 0.9 * std::pow(std::max(3.2e-4, err), -1.0 / 5.0);
                break;
            }
            if (++steps > 100000) { ok = false; return x; }
        }
        if (T - t > eps) {
            dt = T - t;
            d0 = f(t);
        }
    }
    return x;
}

/* MR::MRDistMax (src/microroughness.cpp:123-132): the largest of 65 grid
 * values over [0, pi/2], refined by 60 golden-section steps between the
 * best point's neighbours, and of the values beside the amplitude's cusp */
double distmax(bool transmit, const double v[3], const double normal[3], double Estep, double b, double w) {
    auto f = [&](double th) { return dist(transmit, false, v, normal, Estep, b, w, th, 0); };
    const double h = PT_PI / 2 / 64;
    int best = 0;
    double fbest = f(0.0);
    for (int k = 1; k <= 64; ++k) {
        double fk = f(k * h);
        if (fk > fbest) { fbest = fk; best = k; }
    }
    const double g = 0.6180339887498949;
    double lo = std::max(best - 1, 0) * h, hi = std::min(best + 1, 64) * h;
    double c = hi - g * (hi - lo), d = lo + g * (hi - lo), fc = f(c), fd = f(d);
    for (int i = 0; i < 60; ++i) {
        if (fc >= fd) { hi = d; d = c; fd = fc; c = hi - g * (hi - lo); fc = f(c); }
        else { lo = c; c = d; fc = fd; d = lo + g * (hi - lo); fd = f(d); }
    }
    double m = std::max(fbest, f(0.5 * (lo + hi)));
    /* the cusp where the outgoing amplitude's square root turns complex
     * (reflection: cos theta = kc / ki above the step; transmission below a
     * negative step: the cut-off cos^2 theta = -kc^2 / kt^2, approached from
     * inside) is a local maximum narrower than the grid */
    double v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2], E = 0.5 * PT_M_N * v2;
    double kc2 = 2 * PT_M_N * Estep * (PT_ELE_E / PT_HBAR) * (PT_ELE_E / PT_HBAR);
    double ki2 = 2 * PT_M_N * E * (PT_ELE_E / PT_HBAR) * (PT_ELE_E / PT_HBAR);
    double kt2 = 2 * PT_M_N * (E - Estep) * (PT_ELE_E / PT_HBAR) * (PT_ELE_E / PT_HBAR);
    double c2 = -1;
    if (!transmit && kc2 > 0 && kc2 < ki2) c2 = kc2 / ki2;
    if (transmit && E > Estep && kc2 < 0 && -kc2 < kt2) c2 = -kc2 / kt2;
    if (c2 > 0) {
        double th = std::acos(std::sqrt(c2));
        for (double fac : {1 - 1e-12, 1 - 1e-9, 1 + 1e-12, 1 + 1e-9}) m = std::max(m, f(th * fac));
    }
    return m;
}

} // namespace mr

struct Tracker {
    const Scene &sc;
    const pt_run_params &P;
    Species sp;
    Rng rng;
    Dense5<9> st;
    std::vector<SolidRef> cur; /* TTracker::currentsolids */
    int stopID = PT_ID_UNKNOWN;
    int Nhit = 0, Nstep = 0, Nspinflip = 0;
    double Hmax = 0, noflip = 1;
    int64_t nacc = 0, nrej = 0;
    pt_stats *stats;
    std::vector<Coll> cbuf;
    int64_t pid = 0;                        /* the particle being tracked */
    std::vector<double> hitlog, snaplog, tracklog, spinlog; /* records of this thread's particles */

    /* TLogger::PrintSpin (src/logger.cpp:237-284) */
    void log_spin(double x1, double x, const double *S) {
        const double iv = P.spinloginterval;
        if (!P.spinlog || !(iv > 0)) return;
        if (x > x1 && (int)(x1 / iv) == (int)(x / iv)) return;
        double y[9], dydt[9], B[3], dB[3][3], V, E[3], W[3];
        st.calc_state(x, y);
        bfield(y[0], y[1], y[2], x, B, dB);
        efield(y[0], y[1], y[2], x, V, E);
        eom(y, dydt, B, dB, E);
        spin_axis(B, E, dydt, W);
        const double r[PT_SPIN_RECORD] = {(double)pid, x, y[0], y[1], y[2], S[0], S[1], S[2], W[0], W[1], W[2], B[0], B[1], B[2]};
        spinlog.insert(spinlog.end(), r, r + PT_SPIN_RECORD);
    }

    /* TLogger::PrintTrack (src/logger.cpp:143-200): at zero path length and
     * when a step from path length l1 to y[8] crossed a multiple of the
     * interval */
    void log_track(double l1, double x, const double *y) {
        const double iv = P.trackloginterval;
        if (!P.tracklog || !(iv > 0)) return;
        if (y[8] > 0 && (int)(l1 / iv) == (int)(y[8] / iv)) return;
        const double r[PT_TRACK_RECORD] = {(double)pid, x, y[0], y[1], y[2], y[3], y[4], y[5], y[7],
                                            (double)sc.solids[current_solid(cur)].id};
        tracklog.insert(tracklog.end(), r, r + PT_TRACK_RECORD);
    }

    Tracker(const Scene &s, const pt_run_params &p, pt_stats *stt) : sc(s), P(p), sp(species_of(p.species)), st(1e-9, 1e-9), stats(stt) {}

    /* TFieldManager::BField / EField (src/fields.cpp:139-182) */
    void bfield(double x, double y, double z, double t, double B[3], double dB[3][3]) const {
        for (int i = 0; i < 3; ++i) { B[i] = 0; if (dB) for (int j = 0; j < 3; ++j) dB[i][j] = 0; }
        for (const Field &f : sc.fields) {
            double Bt[3] = {0, 0, 0}, dBt[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            f.bfield(x, y, z, Bt, dB ? dBt : nullptr);
            for (int i = 0; i < 3; ++i) {
                B[i] += Bt[i];
                if (dB) for (int j = 0; j < 3; ++j) dB[i][j] += dBt[i][j];
            }
        }
        (void)t;
    }
    void efield(double x, double y, double z, double t, double &V, double E[3]) const {
        V = 0; E[0] = E[1] = E[2] = 0;
        for (const Field &f : sc.fields) {
            double Vt = 0, Et[3] = {0, 0, 0};
            f.efield(x, y, z, Vt, Et);
            V += Vt;
            for (int i = 0; i < 3; ++i) E[i] += Et[i];
        }
        (void)t;
    }

    /* TParticle::SpinPrecessionAxis (src/particle.cpp:148-175): BMT precession
     * in the relativistically distorted field plus Thomas precession; 1/c^2
     * as the reciprocal constant, as in the equation of motion */
    void spin_axis(const double B[3], const double E[3], const double *dydt, double W[3]) const {
        const double v2 = dydt[0] * dydt[0] + dydt[1] * dydt[1] + dydt[2] * dydt[2];
        const double gr = 1. / std::sqrt(1. - v2 * PT_INV_C0_SQ);
        const double Bdotv = B[0] * dydt[0] + B[1] * dydt[1] + B[2] * dydt[2];
        double Bpar[3], vxE[3], axv[3];
        for (int j = 0; j < 3; ++j) Bpar[j] = Bdotv * dydt[j] / v2;
        vxE[0] = dydt[1] * E[2] - dydt[2] * E[1];
        vxE[1] = dydt[2] * E[0] - dydt[0] * E[2];
        vxE[2] = dydt[0] * E[1] - dydt[1] * E[0];
        axv[0] = dydt[4] * dydt[2] - dydt[5] * dydt[1];
        axv[1] = dydt[5] * dydt[0] - dydt[3] * dydt[2];
        axv[2] = dydt[3] * dydt[1] - dydt[4] * dydt[0];
        const double cb = -sp.gamma / gr, ct = gr * gr / (gr + 1) * PT_INV_C0_SQ;
        for (int j = 0; j < 3; ++j)
            W[j] = cb * ((1 - gr) * Bpar[j] + gr * B[j] - gr * vxE[j] * PT_INV_C0_SQ) + ct * axv[j];
    }
    /* TParticle::SpinDerivs (src/particle.cpp:178-193) along the trajectory's
     * dense output: dS/dt = Omega x S, integrated time, integrated phase */
    void spin_axis_at(double t, double W[3]) {
        double y[9], dydt[9], B[3], dB[3][3], V, E[3];
        st.calc_state(t, y);
        bfield(y[0], y[1], y[2], t, B, dB);
        efield(y[0], y[1], y[2], t, V, E);
        eom(y, dydt, B, dB, E);
        spin_axis(B, E, dydt, W);
    }
    const Spline1 *omega = nullptr; /* interpolatefields: the axis splines of the current step */
    void spin_derivs(const double *S, double *dS, double t) {
        double W[3];
        if (omega)
            for (int k = 0; k < 3; ++k) W[k] = omega[k].calc(t);
        else
            spin_axis_at(t, W);
        dS[0] = W[1] * S[2] - W[2] * S[1];
        dS[1] = W[2] * S[0] - W[0] * S[2];
        dS[2] = W[0] * S[1] - W[1] * S[0];
        dS[3] = 1.;
        dS[4] = std::sqrt(W[0] * W[0] + W[1] * W[1] + W[2] * W[2]);
    }

    /* TParticle::derivs + EquationOfMotion (src/particle.cpp:96-135) */
    void derivs(const double *y, double *dydx, double x) {
        double B[3] = {0, 0, 0}, dB[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, E[3] = {0, 0, 0}, V = 0;
        if (sp.q != 0 || (sp.mu != 0 && y[7] != 0)) bfield(y[0], y[1], y[2], x, B, (sp.mu != 0 && y[7] != 0) ? dB : nullptr);
        if (sp.q != 0) efield(y[0], y[1], y[2], x, V, E);
        if (stats) stats->rhs_evals++;
        eom(y, dydx, B, dB, E);
    }
    void eom(const double *y, double *dydx, const double B[3], const double dB[3][3], const double E[3]) const {
        dydx[0] = y[3]; dydx[1] = y[4]; dydx[2] = y[5];
        double F[3] = {0, 0, 0};
        F[2] += sp.fgrav;
        if (sp.q != 0) {
            F[0] += sp.q * (E[0] + y[4] * B[2] - y[5] * B[1]);
            F[1] += sp.q * (E[1] + y[5] * B[0] - y[3] * B[2]);
            F[2] += sp.q * (E[2] + y[3] * B[1] - y[4] * B[0]);
        }
        if (sp.mu != 0 && y[7] != 0 && (B[0] != 0 || B[1] != 0 || B[2] != 0)) {
            /* grad|B| = (B . dB/dx_i)/|B| with one reciprocal */
            double inv = 1.0 / std::sqrt(B[0] * B[0] + B[1] * B[1] + B[2] * B[2]);
            double dBdxi[3] = {(B[0] * dB[0][0] + B[1] * dB[1][0] + B[2] * dB[2][0]) * inv,
                               (B[0] * dB[0][1] + B[1] * dB[1][1] + B[2] * dB[2][1]) * inv,
                               (B[0] * dB[0][2] + B[1] * dB[1][2] + B[2] * dB[2][2]) * inv};
            F[0] += y[7] * sp.mu * dBdxi[0];
            F[1] += y[7] * sp.mu * dBdxi[1];
            F[2] += y[7] * sp.mu * dBdxi[2];
        }
        double v2 = y[3] * y[3] + y[4] * y[4] + y[5] * y[5];
        double ig = std::sqrt(1 - v2 * PT_INV_C0_SQ);
        double vF = (y[3] * F[0] + y[4] * F[1] + y[5] * F[2]) * PT_INV_C0_SQ;
        double s = ig * sp.inv_mkg;
        dydx[3] = s * (F[0] - y[3] * vF);
        dydx[4] = s * (F[1] - y[4] * vF);
        dydx[5] = s * (F[2] - y[5] * vF);
        dydx[6] = ig;
        dydx[7] = 0;
        dydx[8] = std::sqrt(v2);
    }

    /* TParticle::GetKineticEnergy (src/particle.cpp:237-251) */
    double ekin(const double *v) const {
        double beta2 = (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) / PT_C0_SQ;
        double gm1;
        double b4 = beta2 * beta2;
        if (b4 * b4 * beta2 < std::numeric_limits<double>::epsilon())
            gm1 = (0.5 + (3.0 / 8.0 + (5.0 / 16.0 + 35.0 / 128.0 * beta2) * beta2) * beta2) * beta2;
        else
            gm1 = 1.0 / std::sqrt(1.0 - beta2) - 1.0;
        return sp.mc2 * gm1;
    }
    /* MaterialPotential (include/neutron.h:53-55) */
    double mat_pot(const pt_material &m, double pol) const {
        return m.fermi_real * 1e-9 - m.internal_bfield * sp.mu_over_e * pol;
    }
    /* TParticle::GetPotentialEnergy (src/particle.cpp:254-269) + TNeutron's material term (src/neutron.cpp:378-380) */
    double epot(double t, const double *y, int solid) const {
        double r = 0;
        if (sp.q != 0 || sp.mu != 0) {
            if (sp.mu != 0) {
                double B[3];
                bfield(y[0], y[1], y[2], t, B, nullptr);
                r += -y[7] * sp.mu_over_e * std::sqrt(B[0] * B[0] + B[1] * B[1] + B[2] * B[2]);
            }
            if (sp.q != 0) {
                double V, E[3];
                efield(y[0], y[1], y[2], t, V, E);
                r += sp.q_over_e * V;
            }
        }
        r += sp.mg * y[2];
        if (sp.kind == PT_NEUTRON) r += mat_pot(sc.mats[sc.solids[solid].mat], y[7]);
        return r;
    }

    /* TTracker::GetCurrentsolid (src/tracking.cpp:367-370) */
    int current_solid(const std::vector<SolidRef> &v) const {
        int best = 0;
        for (size_t i = 1; i < v.size(); ++i) {
            const SolidRef &a = v[best], &b = v[i];
            bool less = a.ignored || (!b.ignored && sc.solids[a.idx].id < sc.solids[b.idx].id);
            if (less) best = (int)i;
        }
        return v[best].idx;
    }
    /* TGeometry::GetSolids (src/geometry.cpp:151-158) */
    std::vector<SolidRef> get_solids(double t, const double *p) const {
        std::vector<SolidRef> v{{0, false}};
        uint64_t m = sc.point_solids(p);
        for (size_t s = 1; s < sc.solids.size(); ++s)
            if (m & (1ull << s)) v.push_back({(int)s, sc.solids[s].ignored(t)});
        return v;
    }

    bool get_collisions(double x1, const double *p, double x2, const double *q, std::vector<Coll> &c) {
        if (stats) stats->bvh_nodes++;
        if (!sc.collisions(x1, p, x2, q, c)) throw std::runtime_error("coplanar");
        return !c.empty();
    }

    /* ---------------- particle-specific physics ---------------- */
    /* TNeutron::Reflect (src/neutron.cpp:99-115) */
    void reflect(double x1, const double *y1, double &x2, double *y2, const double *n) const {
        double vn = y1[3] * n[0] + y1[4] * n[1] + y1[5] * n[2];
        x2 = x1;
        y2[0] = y1[0]; y2[1] = y1[1]; y2[2] = y1[2];
        y2[3] -= 2 * vn * n[0]; y2[4] -= 2 * vn * n[1]; y2[5] -= 2 * vn * n[2];
        y2[6] = y1[6]; y2[8] = y1[8];
    }
    /* sincos_distribution(0, pi/2) (include/mc.h:159-175) */
    double sincos_draw() {
        double u = rng.u();
        double ca = std::cos(0.0), cb = std::cos(PT_PI / 2.);
        return std::acos(std::sqrt(u * (cb * cb - ca * ca) + ca * ca));
    }
    /* TNeutron::ReflectLambert (src/neutron.cpp:151-184) */
    void reflect_lambert(double x1, const double *y1, double &x2, double *y2, const double *normal, const pt_material &mat) {
        double vn = y1[3] * normal[0] + y1[4] * normal[1] + y1[5] * normal[2];
        double n[3] = {normal[0], normal[1], normal[2]};
        if (vn > 0) { vn *= -1; n[0] *= -1; n[1] *= -1; n[2] *= -1; }
        x2 = x1;
        y2[0] = y1[0]; y2[1] = y1[1]; y2[2] = y1[2];
        double vabs = std::sqrt(y1[3] * y1[3] + y1[4] * y1[4] + y1[5] * y1[5]);
        for (int it = 0;; ++it) {
            double phi = 2. * PT_PI * rng.u();
            double th = sincos_draw();
            y2[3] = vabs * std::cos(phi) * std::sin(th);
            y2[4] = vabs * std::sin(phi) * std::sin(th);
            y2[5] = vabs * std::cos(th);
            if (mat.diff_prob > 0) rotate_vector(&y2[3], n, &y1[3]);
            else {
                double spec[3] = {y1[3] - 2 * vn * n[0], y1[4] - 2 * vn * n[1], y1[5] - 2 * vn * n[2]};
                rotate_vector(&y2[3], spec, &y1[3]);
            }
            if (y2[3] * n[0] + y2[4] * n[1] + y2[5] * n[2] > 0) break;
            if (it > 10000) { stopID = PT_ID_GEOMETRY_ERROR; break; }
        }
        y2[6] = y1[6]; y2[8] = y1[8];
    }
    /* TNeutron::Transmit (src/neutron.cpp:25-35) */
    void transmit(const double *y1, double *y2, const double *n, double Estep) const {
        double vn = y1[3] * n[0] + y1[4] * n[1] + y1[5] * n[2];
        double En = 0.5 * sp.m * vn * vn;
        double k1 = std::sqrt(En), k2 = std::sqrt(En - Estep);
        for (int i = 0; i < 3; i++) y2[i + 3] += (k2 / k1 - 1) * (n[i] * vn);
    }
    /* TNeutron::TransmitLambert (src/neutron.cpp:65-96) */
    void transmit_lambert(const double *y1, double *y2, const double *normal, double Estep, const pt_material &mat) {
        double vn = y1[3] * normal[0] + y1[4] * normal[1] + y1[5] * normal[2];
        double n[3] = {normal[0], normal[1], normal[2]};
        if (vn < 0) { vn *= -1; n[0] *= -1; n[1] *= -1; n[2] *= -1; }
        double En = 0.5 * sp.m * vn * vn;
        double k1 = std::sqrt(En), k2 = std::sqrt(En - Estep);
        double spec[3] = {y2[3], y2[4], y2[5]};
        for (int i = 0; i < 3; ++i) spec[i] += (k2 / k1 - 1) * n[i] * vn;
        double vabs = std::sqrt(spec[0] * spec[0] + spec[1] * spec[1] + spec[2] * spec[2]);
        for (int it = 0;; ++it) {
            double phi = 2. * PT_PI * rng.u();
            double th = sincos_draw();
            y2[3] = vabs * std::cos(phi) * std::sin(th);
            y2[4] = vabs * std::sin(phi) * std::sin(th);
            y2[5] = vabs * std::cos(th);
            if (mat.diff_prob > 0) rotate_vector(&y2[3], n, &y1[3]);
            else rotate_vector(&y2[3], spec, &y1[3]);
            if (y2[3] * n[0] + y2[4] * n[1] + y2[5] * n[2] > 0) break;
            if (it > 10000) { stopID = PT_ID_GEOMETRY_ERROR; break; }
        }
    }
    /* the MicroRoughness direction (TNeutron::ReflectMR / TransmitMR,
     * src/neutron.cpp:38-62, 118-148): rejection under 1.5 times the
     * transmission distribution's maximum, phi uniform, theta
     * sin-distributed on [0, pi/2] */
    void mr_direction(bool transmit, const double *v, const double *normal, double Estep, const pt_material &mat,
                      double &theta, double &phi) {
        double env = 1.5 * mr::distmax(true, v, normal, Estep, mat.rms_roughness, mat.correl_length);
        for (int it = 0;; ++it) {
            phi = 2. * PT_PI * rng.u();
            theta = std::acos(std::cos(0.0) - rng.u() * (std::cos(0.0) - std::cos(PT_PI / 2.)));
            if (!(rng.u() * env > mr::dist(transmit, false, v, normal, Estep, mat.rms_roughness, mat.correl_length, theta, phi)))
                break;
            if (it > 10000) { stopID = PT_ID_GEOMETRY_ERROR; break; }
        }
    }
    void reflect_mr(double x1, const double *y1, double &x2, double *y2, const double *normal, double Estep, const pt_material &mat) {
        double th, ph;
        mr_direction(false, &y1[3], normal, Estep, mat, th, ph);
        double vn = y1[3] * normal[0] + y1[4] * normal[1] + y1[5] * normal[2];
        if (vn > 0) th = PT_PI - th;
        x2 = x1;
        y2[0] = y1[0]; y2[1] = y1[1]; y2[2] = y1[2];
        double vabs = std::sqrt(y1[3] * y1[3] + y1[4] * y1[4] + y1[5] * y1[5]);
        y2[3] = vabs * std::cos(ph) * std::sin(th);
        y2[4] = vabs * std::sin(ph) * std::sin(th);
        y2[5] = vabs * std::cos(th);
        rotate_vector(&y2[3], normal, &y1[3]);
        y2[6] = y1[6]; y2[8] = y1[8];
    }
    void transmit_mr(const double *y1, double *y2, const double *normal, double Estep, const pt_material &mat) {
        double th, ph;
        mr_direction(true, &y1[3], normal, Estep, mat, th, ph);
        double vabs = std::sqrt(y1[3] * y1[3] + y1[4] * y1[4] + y1[5] * y1[5] - 2 * Estep / PT_M_N);
        double vn = y1[3] * normal[0] + y1[4] * normal[1] + y1[5] * normal[2];
        if (vn < 0) th = PT_PI - th;
        y2[3] = vabs * std::cos(ph) * std::sin(th);
        y2[4] = vabs * std::sin(ph) * std::sin(th);
        y2[5] = vabs * std::cos(th);
        rotate_vector(&y2[3], normal, &y1[3]);
    }
    /* TNeutron::OnHit (src/neutron.cpp:187-264) */
    void on_hit(double x1, const double *y1, double &x2, double *y2, const double *normal, int leaving, int entering) {
        if (sp.kind != PT_NEUTRON) return; /* TProton/TElectron::OnHit are empty */
        const pt_material &ml = sc.mats[sc.solids[leaving].mat], &me = sc.mats[sc.solids[entering].mat];
        double vn = y1[3] * normal[0] + y1[4] * normal[1] + y1[5] * normal[2];
        double En = 0.5 * sp.m * vn * vn;
        const pt_material &mat = vn < 0 ? me : ml;
        if (rng.u() < mat.spinflip_prob) y2[7] *= -1;
        double Estep = mat_pot(me, y2[7]) - mat_pot(ml, y2[7]);
        bool use_mr = mr::valid(&y1[3], Estep, mat.rms_roughness, mat.correl_length);
        double mrr = 0, mrt = 0;
        if (use_mr) {
            bool ok = true;
            mrr = mr::prob(false, &y1[3], normal, Estep, mat.rms_roughness, mat.correl_length, ok);
            if (ekin(&y1[3]) > Estep) mrt = mr::prob(true, &y1[3], normal, Estep, mat.rms_roughness, mat.correl_length, ok);
            if (!ok) { stopID = PT_ID_ODEINT_ERROR; return; }
        }
        double prob = rng.u();
        if (use_mr && prob < mrr) { reflect_mr(x1, y1, x2, y2, normal, Estep, mat); return; }
        if (use_mr && prob < mrr + mrt) { transmit_mr(y1, y2, normal, Estep, mat); return; }
        double k1r, k1i, k2r, k2i;
        csqrt(En, -ml.fermi_imag * 1e-9, k1r, k1i);
        csqrt(En - Estep, -me.fermi_imag * 1e-9, k2r, k2i);
        /* norm((k1-k2)/(k1+k2)) */
        double nr = k1r - k2r, ni = k1i - k2i, dr = k1r + k2r, di = k1i + k2i;
        double reflprob = (nr * nr + ni * ni) / (dr * dr + di * di);
        if (En > Estep) {
            if (prob < mrr + mrt + reflprob * (1 - mrr - mrt)) {
                if (!use_mr && rng.u() < mat.diff_prob + mat.modified_lambert_prob) reflect_lambert(x1, y1, x2, y2, normal, mat);
                else reflect(x1, y1, x2, y2, normal);
            } else {
                if (!use_mr && rng.u() < mat.diff_prob + mat.modified_lambert_prob) transmit_lambert(y1, y2, normal, Estep, mat);
                else transmit(y1, y2, normal, Estep);
            }
        } else {
            double absprob = 1 - reflprob + mat.loss_per_bounce;
            if (use_mr) {
                double kc = std::sqrt(2 * PT_M_N * Estep) * PT_ELE_E / PT_HBAR;
                double addtrans = 2 * std::pow(me.rms_roughness, 2) * kc * kc /
                                  (1 + 0.85 * kc * me.correl_length + 2 * kc * kc * std::pow(me.correl_length, 2));
                absprob *= std::sqrt(1 + addtrans); /* second-order correction for rough surfaces */
            }
            if (prob < mrr + mrt + absprob * (1 - mrr - mrt)) stopID = PT_ID_ABSORBED_ON_SURFACE;
            else {
                if (!use_mr && rng.u() < mat.diff_prob + mat.modified_lambert_prob) reflect_lambert(x1, y1, x2, y2, normal, mat);
                else reflect(x1, y1, x2, y2, normal);
            }
        }
    }
    /* TNeutron::OnStep (src/neutron.cpp:267-282), TProton/TElectron::OnStep */
    void on_step(double x1, const double *y1, double &x2, double *y2, int solid) {
        if (sp.kind == PT_NEUTRON) {
            const pt_material &m = sc.mats[sc.solids[solid].mat];
            if (m.fermi_imag > 0) {
                double Er = 0.5 * sp.m * (y1[3] * y1[3] + y1[4] * y1[4] + y1[5] * y1[5]), Ei = m.fermi_imag * 1e-9;
                double kr, ki;
                csqrt(2 * sp.m * Er, 2 * sp.m * Ei, kr, ki); /* k = sqrt(2 m E) e / hbar */
                ki = ki * PT_ELE_E / PT_HBAR;
                double dx = y2[0] - y1[0], dy = y2[1] - y1[1], dz = y2[2] - y1[2];
                double l = std::sqrt(dx * dx + dy * dy + dz * dz);
                double abspath = -std::log(1 - rng.u()) / (2 * ki);
                if (abspath < l) {
                    x2 = x1 + abspath / l * (x2 - x1);
                    st.calc_state(x2, y2);
                    stopID = PT_ID_ABSORBED_IN_MATERIAL;
                }
            }
        } else {
            if (sc.solids[solid].id > 1) {
                x2 = x1;
                for (int i = 0; i < 9; ++i) y2[i] = y1[i];
                stopID = PT_ID_ABSORBED_IN_MATERIAL;
            }
        }
    }

    /* TTracker::DoStep + TParticle::DoStep (src/tracking.cpp:268-278, src/particle.cpp:196-206) */
    bool do_step(double x1, const double *y1, double &x2, double *y2, int solid) {
        double x2t = x2, y2t[9];
        std::copy(y2, y2 + 9, y2t);
        on_step(x1, y1, x2, y2, solid);
        Hmax = std::max(ekin(&y2[3]) + epot(x2, y2, solid), Hmax);
        if (y2t[7] != y2[7]) Nspinflip++;
        Nstep++;
        if (stats) stats->subsegments++;
        return !(x2t == x2 && std::equal(y2, y2 + 9, y2t));
    }

    /* TTracker::iterate_collision (src/tracking.cpp:228-265) */
    bool iterate_collision(double &x1, double *y1, double &x2, double *y2, unsigned iteration) {
        if (std::pow(y2[0] - y1[0], 2) + std::pow(y2[1] - y1[1], 2) + std::pow(y2[2] - y1[2], 2) < PT_REFLECT_TOLERANCE * PT_REFLECT_TOLERANCE)
            return true;
        if (x2 - x1 < 4 * (x1 + x2) * std::numeric_limits<double>::epsilon()) return true;
        if (iteration >= 100) return true;
        if (stats) stats->bisection_levels++;
        double xc = x1 + (x2 - x1) * 0.5;
        double yc[9];
        st.calc_state(xc, yc);
        std::vector<Coll> c;
        if (get_collisions(x1, y1, xc, yc, c)) {
            if (iterate_collision(x1, y1, xc, yc, iteration + 1)) {
                x2 = xc; std::copy(yc, yc + 9, y2);
                return true;
            }
        }
        if (get_collisions(xc, yc, x2, y2, c)) {
            if (iterate_collision(xc, yc, x2, y2, iteration + 1)) {
                x1 = xc; std::copy(yc, yc + 9, y1);
                return true;
            }
        }
        if (stats) stats->bisect_dead++;
        return false;
    }

    /* TTracker::DoHit (src/tracking.cpp:280-365) */
    bool do_hit(double x1, const double *y1, double &x2, double *y2) {
        bool altered = false, traversed = true;
        std::vector<Coll> colls;
        if (!get_collisions(x1, y1, x2, y2, colls)) throw std::runtime_error("DoHit without collision");
        std::vector<SolidRef> ns = cur;
        for (const Coll &c : colls) {
            auto found = std::find_if(ns.begin(), ns.end(), [&](const SolidRef &r) { return sc.solids[r.idx].id == c.id; });
            if (c.distnormal < 0) {
                if (found != ns.end()) {
                    if (c.s > 0) ns.push_back({c.solid, found->ignored});
                } else ns.push_back({c.solid, c.ignored});
            } else if (c.distnormal > 0) {
                if (found == ns.end()) {
                    if (c.s > 0) { stopID = PT_ID_GEOMETRY_ERROR; return true; }
                } else ns.erase(found);
            } else {
                stopID = PT_ID_GEOMETRY_ERROR;
                return true;
            }
        }
        int leaving = current_solid(cur);
        int entering = 0;
        for (const SolidRef &r : ns)
            if (!r.ignored && sc.solids[r.idx].id > sc.solids[entering].id) entering = r.idx;
        if (sc.solids[leaving].id != sc.solids[entering].id) {
            auto c = std::find_if(colls.begin(), colls.end(), [&](const Coll &k) {
                return k.id == sc.solids[leaving].id || (k.id == sc.solids[entering].id && !k.ignored);
            });
            if (c == colls.end()) { stopID = PT_ID_GEOMETRY_ERROR; return true; }
            double x2t = x2, y2t[9];
            std::copy(y2, y2 + 9, y2t);
            /* TParticle::DoHit (src/particle.cpp:208-217) */
            on_hit(x1, y1, x2, y2, c->normal, leaving, entering);
            if (y2t[7] != y2[7]) Nspinflip++;
            Nhit++;
            if (stats) stats->hits++;
            if (x2t == x2 && std::equal(y2, y2 + 9, y2t)) { altered = false; traversed = true; }
            else {
                altered = true;
                if (x2 == x2t && y2[0] == y2t[0] && y2[1] == y2t[1] && y2[2] == y2t[2]) traversed = true;
                else if (x2 == x1 && y2[0] == y1[0] && y2[1] == y1[1] && y2[2] == y1[2]) traversed = false;
                else { stopID = PT_ID_GEOMETRY_ERROR; return true; }
            }
            if (P.hitlog) { /* TLogger::PrintHit (src/logger.cpp:202-235) */
                const double r[PT_HIT_RECORD] = {(double)pid, x1, y1[0], y1[1], y1[2], y1[3], y1[4], y1[5], y1[7], y2[3], y2[4], y2[5],
                                                  y2[7], c->normal[0], c->normal[1], c->normal[2], (double)sc.solids[leaving].id,
                                                  (double)sc.solids[entering].id};
                hitlog.insert(hitlog.end(), r, r + PT_HIT_RECORD);
            }
        }
        if (traversed) cur = ns;
        return altered || stopID != PT_ID_UNKNOWN;
    }

    /* TTracker::CheckHit (src/tracking.cpp:176-226) */
    bool check_hit(double x1, const double *y1, double &x2, double *y2) {
        if (!sc.check_segment(y1, y2)) { stopID = PT_ID_HIT_BOUNDARIES; return true; }
        if (x2 == x1) return false;
        int currentsolid = current_solid(cur);
        std::vector<Coll> colls;
        bool found;
        try { found = get_collisions(x1, y1, x2, y2, colls); }
        catch (...) { stopID = PT_ID_CGAL_ERROR; return true; }
        if (found) {
            double xc1 = x1, xc2 = x2, yc1[9], yc2[9];
            std::copy(y1, y1 + 9, yc1);
            std::copy(y2, y2 + 9, yc2);
            if (iterate_collision(xc1, yc1, xc2, yc2, 0)) {
                if (xc1 > x1 && do_step(x1, y1, xc1, yc1, currentsolid)) {
                    x2 = xc1; std::copy(yc1, yc1 + 9, y2);
                    return true;
                }
                if (do_hit(xc1, yc1, xc2, yc2)) {
                    x2 = xc2; std::copy(yc2, yc2 + 9, y2);
                    return true;
                }
                if (!(xc2 > x1)) { stopID = PT_ID_CGAL_ERROR; return true; }
                if (check_hit(xc2, yc2, x2, y2)) return true;
            }
        } else {
            return do_step(x1, y1, x2, y2, currentsolid);
        }
        return false;
    }

    /* TTracker::IntegrateSpin decision logic (src/tracking.cpp:373-483); the
     * Bloch integration (LOOP D) is bloch() below. */
    double integrate_spin(double *spin, double x2, const double *y2) {
        double x1 = st.to;
        const double *y1 = st.xo;
        double B1[3], B2[3];
        bfield(y1[0], y1[1], y1[2], x1, B1, nullptr);
        bfield(y2[0], y2[1], y2[2], x2, B2, nullptr);
        double Babs1 = std::sqrt(B1[0] * B1[0] + B1[1] * B1[1] + B1[2] * B1[2]);
        double Babs2 = std::sqrt(B2[0] * B2[0] + B2[1] * B2[1] + B2[2] * B2[2]);
        if (sp.gamma == 0 || Babs2 == 0) {
            std::fill(spin, spin + 5, 0.0);
            return y1[7];
        } else if (Babs1 == 0 && Babs2 > 0) {
            double sp_ = (rng.u() < 0.5 ? 0 : 1) * 2 - 1;
            std::fill(spin, spin + 5, 0.0);
            return sp_;
        } else if (x2 > x1 && (Babs1 < P.bmax || Babs2 < P.bmax)) {
            bool i1 = false, i2 = false;
            for (int i = 0; i + 1 < P.n_spintimes; i += 2) {
                i1 |= (x1 >= P.spintimes[i] && x1 < P.spintimes[i + 1]);
                i2 |= (x2 >= P.spintimes[i] && x2 < P.spintimes[i + 1]);
            }
            if (i1 || i2) {
                /* LOOP D: a fresh dopri5 dense-output stepper (abs = rel = 1e-12)
                 * started with half a Larmor turn as its step */
                Spline1 om[3];
                if (P.interpolatefields) { /* the axis at 11 times of the step, one cubic spline per component */
                    const int int_points = 10;
                    double ts[int_points + 1], w[3][int_points + 1];
                    for (int i = 0; i <= int_points; ++i) {
                        const double t = x1 + i * (x2 - x1) / int_points;
                        ts[i] = t;
                        double W[3];
                        spin_axis_at(t, W);
                        for (int k = 0; k < 3; ++k) w[k][i] = W[k];
                    }
                    for (int k = 0; k < 3; ++k) om[k].build(int_points + 1, ts, w[k]);
                }
                struct OmegaScope {
                    const Spline1 *&slot;
                    OmegaScope(const Spline1 *&s_, const Spline1 *v) : slot(s_) { slot = v; }
                    ~OmegaScope() { slot = nullptr; }
                } scope(omega, P.interpolatefields ? om : nullptr);
                if (spin[0] == 0 && spin[1] == 0 && spin[2] == 0)
                    for (int k = 0; k < 3; ++k) spin[k] = B1[k] * y1[7] / Babs1;
                Dense5<5> ss(1e-12, 1e-12);
                ss.initialize(spin, x1, std::fabs(PT_PI / sp.gamma / Babs1));
                log_spin(x1, x1, spin);
                auto sys = [this](const double *S, double *dS, double t) { spin_derivs(S, dS, t); };
                int64_t rej = 0;
                for (int64_t steps = 0;; ++steps) {
                    if (steps >= PTO_MAX_SPIN_STEPS) throw OdeintError();
                    ss.do_step(sys, rej);
                    double t = ss.t;
                    if (t > x2) {
                        t = x2;
                        ss.calc_state(t, spin);
                    } else {
                        std::copy(ss.x, ss.x + 5, spin);
                    }
                    if (stats) stats->spin_steps++;
                    log_spin(ss.to, t, spin);
                    if (t >= x2) break;
                }
            } else if (spin[0] != 0 || spin[1] != 0 || spin[2] != 0) {
                double proj = (spin[0] * B1[0] + spin[1] * B1[1] + spin[2] * B1[2]) / Babs1 /
                              std::sqrt(spin[0] * spin[0] + spin[1] * spin[1] + spin[2] * spin[2]);
                if (proj * proj >= 1) { spin[0] = 0; spin[1] = 0; }
                else {
                    double az = 2. * PT_PI * rng.u();
                    spin[0] = std::sqrt(1 - proj * proj) * std::sin(az);
                    spin[1] = std::sqrt(1 - proj * proj) * std::cos(az);
                }
                spin[2] = proj;
                rotate_vector(spin, B2, nullptr);
            }
        }
        if (Babs2 > P.bmax && (spin[0] != 0 || spin[1] != 0 || spin[2] != 0)) {
            double proj = (spin[0] * B2[0] + spin[1] * B2[1] + spin[2] * B2[2]) / Babs2 /
                          std::sqrt(spin[0] * spin[0] + spin[1] * spin[1] + spin[2] * spin[2]);
            std::fill(spin, spin + 5, 0.0);
            return proj;
        }
        return y1[7];
    }

    /* TTracker::IntegrateParticle (src/tracking.cpp:17-173) */
    void integrate(int64_t id, double t0, const double *ystart, const double *spinstart, pt_particles *out, int64_t i) {
        rng = Rng{P.seed, id, 0};
        pid = id;
        stopID = PT_ID_UNKNOWN; Nhit = Nstep = Nspinflip = 0; noflip = 1; nacc = nrej = 0;
        double tau = 0;
        if (P.tau > 0) tau = -std::log(1 - rng.u()) * P.tau; /* exponential_distribution(1/tau) */
        else tau = P.tmax;
        const double tmax = P.simtime, maxtraj = P.lmax;
        double x = t0, y[9], spin[5];
        std::copy(ystart, ystart + 9, y);
        std::copy(spinstart, spinstart + 5, spin);
        double hstart = 0;
        cur = get_solids(x, y);
        {   /* TParticle ctor: Hmax = initial total energy (src/particle.cpp:88-89) */
            hstart = ekin(&y[3]) + epot(x, y, current_solid(cur));
            Hmax = hstart;
        }
        bool reset = false;
        log_track(y[8], x, y); /* the track log's first point (src/tracking.cpp:43) */
        if (x > tmax) stopID = PT_ID_NOT_FINISH;
        st.initialize(y, x, 10. * PT_MAX_TRACK_DEVIATION / std::sqrt(y[3] * y[3] + y[4] * y[4] + y[5] * y[5]));
        while (stopID == PT_ID_UNKNOWN) {
            if (reset) st.initialize(y, x, st.dt);
            double x1 = x, y1[9];
            std::copy(y, y + 9, y1);
            try {
                int64_t before = nrej;
                st.do_step(*this, nrej);
                (void)before;
                nacc++;
                bool finite = std::isfinite(st.t);
                for (int i = 0; i < 9; ++i) finite = finite && std::isfinite(st.x[i]);
                if (!finite) throw OdeintError(); /* a non-finite state would never stop */
                x = st.t;
                std::copy(st.x, st.x + 9, y);
            } catch (OdeintError &) {
                stopID = PT_ID_ODEINT_ERROR;
                break;
            }
            if (tau > 0 && y[6] > tau) {
                x = x1 + (x - x1) * (tau - y1[6]) / (y[6] - y1[6]);
                st.calc_state(x, y);
            }
            if (x > tmax) { x = tmax; st.calc_state(x, y); }
            try {
                int nsub = 0;
                while (x1 < x) {
                    if (++nsub > (1 << 20)) { stopID = PT_ID_ODEINT_ERROR; break; }
                    double l2 = std::pow(y[8] - y1[8], 2);
                    double d2 = std::pow(y[0] - y1[0], 2) + std::pow(y[1] - y1[1], 2) + std::pow(y[2] - y1[2], 2);
                    double dev2 = 0.25 * (l2 - d2);
                    double x2 = x, y2[9];
                    std::copy(y, y + 9, y2);
                    if (dev2 > PT_MAX_TRACK_DEVIATION * PT_MAX_TRACK_DEVIATION) {
                        x2 = x1 + (x - x1) / std::ceil(std::sqrt(dev2) / PT_MAX_TRACK_DEVIATION);
                        if (!(x2 > x1)) { stopID = PT_ID_ODEINT_ERROR; break; }
                        st.calc_state(x2, y2);
                    }
                    reset = check_hit(x1, y1, x2, y2);
                    if (reset) { x = x2; std::copy(y2, y2 + 9, y); }
                    x1 = x2;
                    std::copy(y2, y2 + 9, y1);
                }
            } catch (...) {
                stopID = PT_ID_CGAL_ERROR;
            }
            if (P.snapshotlog) /* TLogger::PrintSnapshot (src/logger.cpp:128-141) */
                for (int k = 0; k < P.n_snapshots; ++k) {
                    const double ts = P.snapshots[k];
                    if (!(st.to <= ts && ts < x)) continue;
                    double ys[9];
                    st.calc_state(ts, ys);
                    double r[PT_SNAPSHOT_RECORD] = {(double)pid, ts};
                    for (int c = 0; c < 9; ++c) r[2 + c] = ys[c];
                    for (int c = 0; c < 5; ++c) r[11 + c] = spin[c];
                    r[16] = stopID; r[17] = Nspinflip; r[18] = noflip; r[19] = Nhit; r[20] = Nstep; r[21] = Hmax;
                    snaplog.insert(snaplog.end(), r, r + PT_SNAPSHOT_RECORD);
                    break;
                }
            {
                double sproj = st.xo[7];
                try {
                    sproj = integrate_spin(spin, x, y);
                } catch (OdeintError &) {
                    stopID = PT_ID_ODEINT_ERROR;
                }
                bool flipped = st.xo[7] != y[7];
                if (sproj != st.xo[7]) {
                    /* TParticle::DoPolarize (src/particle.cpp:225-234) */
                    double flipprob = 0.5 * (1 - y[7] * sproj);
                    noflip *= 1. - flipprob;
                    if (P.flipspin) {
                        double prev = y[7];
                        y[7] = rng.u() < 0.5 * (sproj + 1) ? 1 : -1;
                        if (y[7] != prev) ++Nspinflip;
                    }
                    if (P.flipspin && flipped) y[7] *= -1;
                } else if (flipped) {
                    std::fill(spin, spin + 5, 0.0);
                }
            }
            log_track(st.xo[8], x, y); /* src/tracking.cpp:140 */
            if (stopID == PT_ID_UNKNOWN && y[6] >= tau) stopID = PT_ID_DECAYED;
            else if (stopID == PT_ID_UNKNOWN && (x >= tmax || y[8] >= maxtraj)) stopID = PT_ID_NOT_FINISH;
        }
        /* TNeutron::Decay creates secondaries only; they are not tracked here. */
        int64_t n = out->n;
        if (out->t) out->t[i] = x;
        if (out->y) for (int c = 0; c < 9; ++c) out->y[c * n + i] = y[c];
        if (out->spin) for (int c = 0; c < 5; ++c) out->spin[c * n + i] = spin[c];
        if (out->stop_id) out->stop_id[i] = stopID;
        if (out->solid) out->solid[i] = (int32_t)sc.solids[current_solid(cur)].id;
        if (out->n_hit) out->n_hit[i] = Nhit;
        if (out->n_step) out->n_step[i] = Nstep;
        if (out->n_spinflip) out->n_spinflip[i] = Nspinflip;
        if (out->h_max) out->h_max[i] = Hmax;
        if (out->noflip_prob) out->noflip_prob[i] = noflip;
        if (out->tau) out->tau[i] = tau;
        if (out->h_start) out->h_start[i] = hstart;
        if (out->n_accepted) out->n_accepted[i] = nacc;
        if (out->n_rejected) out->n_rejected[i] = nrej;
        if (stats) { stats->rk_accepted += nacc; stats->rk_rejected += nrej; stats->particle_seconds += x - t0; }
    }

    void operator()(const double *y, double *dydx, double t) { derivs(y, dydx, t); }
};

} // namespace

/* ------------------------------------------------------------------ */
/* C entry points                                                      */
/* ------------------------------------------------------------------ */
extern "C" {

const char *pto_last_error(void) { return g_err.c_str(); }

int pto_create(const pt_scene_desc *d, pto_ctx **out) {
    try {
        auto ctx = std::make_unique<pto_ctx>();
        Scene &sc = ctx->sc;
        if (d->n_solids < 1 || d->solids[0].id != 1) throw std::runtime_error("solids[0] must be the default solid (ID 1)");
        if (d->n_solids > 64) throw std::runtime_error("at most 64 solids");
        for (int i = 0; i < d->n_materials; ++i) {
            const pt_material &m = d->materials[i];
            if (m.rms_roughness < 0 || m.correl_length < 0) throw std::runtime_error("negative roughness or correlation length");
            sc.mats.push_back(m);
        }
        for (int i = 0; i < d->n_solids; ++i) {
            Solid s;
            s.id = d->solids[i].id;
            s.mat = d->solids[i].material;
            if (s.mat < 0 || s.mat >= d->n_materials) throw std::runtime_error("bad material index");
            s.ign.assign(d->solids[i].ignore_times, d->solids[i].ignore_times + 2 * d->solids[i].n_ignore);
            sc.solids.push_back(s);
        }
        sc.mesh.slo.assign(3 * sc.solids.size(), 1e300);
        sc.mesh.shi.assign(3 * sc.solids.size(), -1e300);
        for (int64_t t = 0; t < d->n_triangles; ++t) {
            Tri tr;
            const double *v = d->triangles + 9 * t;
            for (int k = 0; k < 3; ++k) { tr.a[k] = v[k]; tr.b[k] = v[3 + k]; tr.c[k] = v[6 + k]; }
            double e1[3] = {tr.b[0] - tr.a[0], tr.b[1] - tr.a[1], tr.b[2] - tr.a[2]};
            double e2[3] = {tr.c[0] - tr.a[0], tr.c[1] - tr.a[1], tr.c[2] - tr.a[2]};
            double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
            double nl = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
            for (int k = 0; k < 3; ++k) {
                tr.n[k] = n[k] / nl;
                tr.lo[k] = std::min(tr.a[k], std::min(tr.b[k], tr.c[k]));
                tr.hi[k] = std::max(tr.a[k], std::max(tr.b[k], tr.c[k]));
            }
            tr.solid = d->triangle_solid[t];
            if (tr.solid <= 0 || tr.solid >= d->n_solids) throw std::runtime_error("bad triangle solid index");
            for (int k = 0; k < 3; ++k) {
                sc.mesh.lo[k] = std::min(sc.mesh.lo[k], tr.lo[k]);
                sc.mesh.hi[k] = std::max(sc.mesh.hi[k], tr.hi[k]);
                sc.mesh.slo[3 * tr.solid + k] = std::min(sc.mesh.slo[3 * tr.solid + k], tr.lo[k]);
                sc.mesh.shi[3 * tr.solid + k] = std::max(sc.mesh.shi[3 * tr.solid + k], tr.hi[k]);
            }
            sc.mesh.tris.push_back(tr);
        }
        sc.mesh.order.resize(sc.mesh.tris.size());
        for (size_t i = 0; i < sc.mesh.order.size(); ++i) sc.mesh.order[i] = (int)i;
        if (!sc.mesh.tris.empty()) sc.mesh.build(0, (int)sc.mesh.tris.size());
        for (int i = 0; i < d->n_fields; ++i) {
            const pt_field &f = d->fields[i];
            Field F;
            F.type = f.type; F.bscale = f.b_scale; F.escale = f.e_scale;
            F.xmax = f.xmax; F.xmin = f.xmin; F.ymax = f.ymax; F.ymin = f.ymin; F.zmax = f.zmax; F.zmin = f.zmin;
            F.bw = f.boundary_width;
            if (f.type == PT_FIELD_TAB3D) F.tab.build(f);
            else if (f.type == PT_FIELD_TAB2D) {
                if (f.nx < 2 || f.nz < 2 || !f.x || !f.z) throw std::runtime_error("2D table needs at least 2 points per axis");
                F.tab2.build(f);
            }
            else if (f.type == PT_FIELD_UNIFORM_E) { F.e[0] = f.e[0]; F.e[1] = f.e[1]; F.e[2] = f.e[2]; }
            else if (f.type == PT_FIELD_HARMONIC) {
                for (int k = 0; k < f.n_coeff; ++k) {
                    if (f.l[k] < 0 || f.l[k] > 5 || f.m[k] < -f.l[k] - 1 || f.m[k] > f.l[k] + 1)
                        throw std::runtime_error("harmonic term out of range");
                    F.hl.push_back(f.l[k]); F.hm.push_back(f.m[k]); F.hg.push_back(f.g[k]);
                }
                for (int k = 0; k < 3; ++k) F.offset[k] = f.offset[k];
            }
            else if (f.type == PT_FIELD_SOLENOID) {
                F.sol_a = f.sol_radius;
                F.sol_b = f.sol_half_length;
                F.sol_B0 = f.sol_bcenter * std::sqrt(f.sol_radius * f.sol_radius + f.sol_half_length * f.sol_half_length) /
                           (PT_PI * f.sol_half_length);
                for (int k = 0; k < 3; ++k) F.offset[k] = f.offset[k];
            }
            else throw std::runtime_error("field type not supported by the oracle");
            sc.fields.push_back(std::move(F));
        }
        *out = ctx.release();
        return 0;
    } catch (std::exception &e) {
        g_err = e.what();
        return PT_ERR_INVALID;
    }
}

void pto_destroy(pto_ctx *ctx) { delete ctx; }

/* the records of the last pto_track call's log `kind` (PT_LOG_HIT,
 * PT_LOG_SNAPSHOT): their number, and up to cap of them into rec */
int64_t pto_log_read(pto_ctx *ctx, int32_t kind, int64_t cap, double *rec) {
    const std::vector<double> &v =
        kind == PT_LOG_HIT ? ctx->hits : kind == PT_LOG_SNAPSHOT ? ctx->snaps : kind == PT_LOG_TRACK ? ctx->tracks : ctx->spins;
    const int w = kind == PT_LOG_HIT ? PT_HIT_RECORD : kind == PT_LOG_SNAPSHOT ? PT_SNAPSHOT_RECORD : kind == PT_LOG_TRACK ? PT_TRACK_RECORD : PT_SPIN_RECORD;
    const int64_t n = (int64_t)v.size() / w;
    if (rec) std::copy(v.begin(), v.begin() + std::min(n, cap) * w, rec);
    return n;
}

int pto_track(pto_ctx *ctx, const pt_run_params *params, const pt_particles *in, pt_particles *out, int nthreads,
              pt_stats *stats) {
    if (!ctx || !params || !in || !out) return PT_ERR_INVALID;
    if (nthreads < 1) nthreads = 1;
    int64_t n = in->n;
    auto t0 = std::chrono::steady_clock::now();
    std::vector<pt_stats> st(nthreads);
    std::memset(st.data(), 0, sizeof(pt_stats) * nthreads);
    std::atomic<int64_t> next{0};
    std::vector<std::vector<double>> hits(nthreads), snaps(nthreads), tracks(nthreads), spins(nthreads);
    auto work = [&](int w) {
        Tracker tr(ctx->sc, *params, &st[w]);
        double ys[9], ss[5];
        while (true) {
            int64_t i = next.fetch_add(1);
            if (i >= n) break;
            for (int c = 0; c < 9; ++c) ys[c] = in->y[c * n + i];
            for (int c = 0; c < 5; ++c) ss[c] = in->spin ? in->spin[c * n + i] : 0.0;
            tr.integrate(in->id[i], in->t[i], ys, ss, out, i);
        }
        hits[w].swap(tr.hitlog);
        snaps[w].swap(tr.snaplog);
        tracks[w].swap(tr.tracklog);
        spins[w].swap(tr.spinlog);
    };
    std::vector<std::thread> th;
    for (int w = 1; w < nthreads; ++w) th.emplace_back(work, w);
    work(0);
    for (auto &t : th) t.join();
    ctx->hits.clear();
    ctx->snaps.clear();
    ctx->tracks.clear();
    ctx->spins.clear();
    for (int w = 0; w < nthreads; ++w) {
        ctx->hits.insert(ctx->hits.end(), hits[w].begin(), hits[w].end());
        ctx->snaps.insert(ctx->snaps.end(), snaps[w].begin(), snaps[w].end());
        ctx->tracks.insert(ctx->tracks.end(), tracks[w].begin(), tracks[w].end());
        ctx->spins.insert(ctx->spins.end(), spins[w].begin(), spins[w].end());
    }
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        for (auto &s : st) {
            stats->rk_accepted += s.rk_accepted; stats->rk_rejected += s.rk_rejected; stats->rhs_evals += s.rhs_evals;
            stats->hits += s.hits; stats->bisection_levels += s.bisection_levels; stats->bisect_dead += s.bisect_dead; stats->spin_steps += s.spin_steps; stats->subsegments += s.subsegments;
            stats->bvh_nodes += s.bvh_nodes; stats->particle_seconds += s.particle_seconds;
        }
        stats->wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    return 0;
}

int pto_field(pto_ctx *ctx, int64_t n, const double *xyzt, double *B, double *dB, double *V, double *E) {
    pt_run_params p;
    std::memset(&p, 0, sizeof(p));
    Tracker tr(ctx->sc, p, nullptr);
    for (int64_t i = 0; i < n; ++i) {
        const double *q = xyzt + 4 * i;
        double b[3], db[3][3], v, e[3];
        tr.bfield(q[0], q[1], q[2], q[3], b, dB ? db : nullptr);
        tr.efield(q[0], q[1], q[2], q[3], v, e);
        if (B) for (int k = 0; k < 3; ++k) B[3 * i + k] = b[k];
        if (dB) for (int k = 0; k < 9; ++k) dB[9 * i + k] = db[k / 3][k % 3];
        if (V) V[i] = v;
        if (E) for (int k = 0; k < 3; ++k) E[3 * i + k] = e[k];
    }
    return 0;
}

int pto_segment_collisions(pto_ctx *ctx, int64_t n, const double *seg, int32_t max_hits, int32_t *count, double *s,
                           double *normal, int32_t *solid_id, double *distnormal) {
    std::vector<Coll> c;
    for (int64_t i = 0; i < n; ++i) {
        const double *p = seg + 6 * i, *q = p + 3;
        if (!ctx->sc.collisions(0.0, p, 1.0, q, c)) { count[i] = -1; continue; }
        int k = (int)std::min<size_t>(c.size(), (size_t)max_hits);
        count[i] = (int32_t)c.size();
        for (int j = 0; j < k; ++j) {
            int64_t o = i * max_hits + j;
            s[o] = c[j].s;
            for (int a = 0; a < 3; ++a) normal[3 * o + a] = c[j].normal[a];
            solid_id[o] = (int32_t)c[j].id;
            distnormal[o] = c[j].distnormal;
        }
    }
    return 0;
}

int pto_point_solids(pto_ctx *ctx, int64_t n, const double *p, uint64_t *mask) {
    for (int64_t i = 0; i < n; ++i) mask[i] = ctx->sc.point_solids(p + 3 * i);
    return 0;
}

/* Spline1 (the interpolatefields axis spline) at np points */
int pto_spline1d_calc(int32_t n, const double *x, const double *y, int32_t np, const double *pts, double *out) {
    if (n < 2) return PT_ERR_INVALID;
    Spline1 s;
    s.build(n, x, y);
    for (int32_t k = 0; k < np; ++k) out[k] = s.calc(pts[k]);
    return 0;
}

/* MicroRoughness building blocks; what: 0 MRDist, 1 MRProb (NaN when the
 * integration fails), 2 MRDistMax */
double pto_mr(int32_t what, int32_t transmit, int32_t integral, const double *v, const double *normal, double Estep, double b,
              double w, double theta, double phi) {
    if (what == 0) return mr::dist(transmit != 0, integral != 0, v, normal, Estep, b, w, theta, phi);
    if (what == 1) {
        bool ok = true;
        double p = mr::prob(transmit != 0, v, normal, Estep, b, w, ok);
        return ok ? p : std::numeric_limits<double>::quiet_NaN();
    }
    return mr::distmax(transmit != 0, v, normal, Estep, b, w);
}

int pto_spline_derivs(int32_t n, const double *x, const double *y, double *d) {
    if (n < 2) return PT_ERR_INVALID;
    spline_derivs(n, x, y, d);
    return 0;
}

void pto_tricubic_coeff(const double *x, double *a) { tricubic_coeff(x, a); }

void pto_tricubic_eval(const double *a, double x, double y, double z, int derx, int dery, int derz, double *out) {
    if (derx == 0 && dery == 0 && derz == 0) *out = tricubic_value(a, x, y, z);
    else *out = tricubic_deriv(a, x, y, z, derx, dery, derz);
}

void pto_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) { philox(ctr, key, out); }

double pto_uniform(uint64_t seed, int64_t id, uint64_t draw) { return uniform_draw(seed, id, draw); }

double pto_detpow(double x, double p) { return ptdm_pow(x, p); }

int pto_dopri5_selftest(double t0, const double *y0, double dt0, int nsteps, double *t_out, double *y_out) {
    struct Osc {
        void operator()(const double *y, double *d, double t) { d[0] = y[1]; d[1] = -y[0] - 0.1 * y[1] + 0.5 * std::cos(3 * t); }
    } sys;
    Dense5<2> st(1e-9, 1e-9);
    st.initialize(y0, t0, dt0);
    int64_t rej = 0;
    for (int i = 0; i < nsteps; ++i) {
        st.do_step(sys, rej);
        t_out[2 * i] = st.to; t_out[2 * i + 1] = st.t;
        double mid = 0.5 * (st.to + st.t), ym[2];
        st.calc_state(mid, ym);
        y_out[4 * i + 0] = st.x[0]; y_out[4 * i + 1] = st.x[1];
        y_out[4 * i + 2] = ym[0]; y_out[4 * i + 3] = ym[1];
    }
    return (int)rej;
}

} // extern "C"
