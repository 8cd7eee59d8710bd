/*
 * pt_scene.cpp -- host-side preparation of the device scene (see pt_scene.hpp).
 * Compiled with -ffp-contract=off so triangle normals and derivative tables
 * round exactly like the oracle's.
 */
#include "pt_scene.hpp"

#include <algorithm>
#include <cmath>
#include <functional>
#include <map>

namespace pth {

/* ---------------------------------------------------------------- BVH */
namespace {
inline float down(double v) {
    float f = (float)v;
    if ((double)f > v) f = std::nextafter(f, -INFINITY);
    return f;
}
inline float up(double v) {
    float f = (float)v;
    if ((double)f < v) f = std::nextafter(f, INFINITY);
    return f;
}
struct Build {
    std::vector<HostTri> &tris;
    std::vector<int> idx;
    std::vector<double> lo, hi, cen;
    std::vector<HostNode> nodes;
    std::vector<HostTri> out;

    explicit Build(std::vector<HostTri> &t) : tris(t) {
        size_t n = t.size();
        idx.resize(n);
        lo.resize(3 * n); hi.resize(3 * n); cen.resize(3 * n);
        for (size_t i = 0; i < n; ++i) {
            idx[i] = (int)i;
            for (int k = 0; k < 3; ++k) {
                lo[3 * i + k] = std::min(t[i].a[k], std::min(t[i].b[k], t[i].c[k]));
                hi[3 * i + k] = std::max(t[i].a[k], std::max(t[i].b[k], t[i].c[k]));
                cen[3 * i + k] = 0.5 * (lo[3 * i + k] + hi[3 * i + k]);
            }
        }
    }
    static double area(const double *l, const double *h) {
        double dx = h[0] - l[0], dy = h[1] - l[1], dz = h[2] - l[2];
        return dx * dy + dy * dz + dz * dx;
    }
    /* binned surface-area heuristic, 12 bins on the widest centroid axis */
    int rec(int first, int count) {
        double bl[3] = {1e300, 1e300, 1e300}, bh[3] = {-1e300, -1e300, -1e300};
        double cl[3] = {1e300, 1e300, 1e300}, ch[3] = {-1e300, -1e300, -1e300};
        for (int i = first; i < first + count; ++i) {
            int t = idx[i];
            for (int k = 0; k < 3; ++k) {
                bl[k] = std::min(bl[k], lo[3 * t + k]); bh[k] = std::max(bh[k], hi[3 * t + k]);
                cl[k] = std::min(cl[k], cen[3 * t + k]); ch[k] = std::max(ch[k], cen[3 * t + k]);
            }
        }
        int me = (int)nodes.size();
        HostNode nd;
        for (int k = 0; k < 3; ++k) { nd.lo[k] = down(bl[k]); nd.hi[k] = up(bh[k]); }
        nd.skip = -1;
        nd.leaf = -1;
        nodes.push_back(nd);
        auto make_leaf = [&]() {
            int f = (int)out.size();
            for (int i = first; i < first + count; ++i) out.push_back(tris[idx[i]]);
            nodes[me].leaf = f * 8 + count;
            nodes[me].skip = (int)nodes.size();
            return me;
        };
        if (count <= 4) return make_leaf();
        int axis = 0;
        double ext = -1;
        for (int k = 0; k < 3; ++k) if (ch[k] - cl[k] > ext) { ext = ch[k] - cl[k]; axis = k; }
        int mid = first + count / 2;
        if (ext > 0) {
            const int NB = 12;
            int bc[NB] = {0};
            double bbl[NB][3], bbh[NB][3];
            for (int b = 0; b < NB; ++b) for (int k = 0; k < 3; ++k) { bbl[b][k] = 1e300; bbh[b][k] = -1e300; }
            auto bin = [&](int t) {
                int b = (int)((cen[3 * t + axis] - cl[axis]) / ext * NB);
                return std::min(std::max(b, 0), NB - 1);
            };
            for (int i = first; i < first + count; ++i) {
                int t = idx[i], b = bin(t);
                ++bc[b];
                for (int k = 0; k < 3; ++k) { bbl[b][k] = std::min(bbl[b][k], lo[3 * t + k]); bbh[b][k] = std::max(bbh[b][k], hi[3 * t + k]); }
            }
            double best = 1e300;
            int bsplit = -1;
            for (int s = 1; s < NB; ++s) {
                double l1[3] = {1e300, 1e300, 1e300}, h1[3] = {-1e300, -1e300, -1e300}, l2[3] = {1e300, 1e300, 1e300}, h2[3] = {-1e300, -1e300, -1e300};
                int c1 = 0, c2 = 0;
                for (int b = 0; b < s; ++b) { c1 += bc[b]; for (int k = 0; k < 3; ++k) { l1[k] = std::min(l1[k], bbl[b][k]); h1[k] = std::max(h1[k], bbh[b][k]); } }
                for (int b = s; b < NB; ++b) { c2 += bc[b]; for (int k = 0; k < 3; ++k) { l2[k] = std::min(l2[k], bbl[b][k]); h2[k] = std::max(h2[k], bbh[b][k]); } }
                if (c1 == 0 || c2 == 0) continue;
                double cost = c1 * area(l1, h1) + c2 * area(l2, h2);
                if (cost < best) { best = cost; bsplit = s; }
            }
            if (bsplit > 0) {
                auto it = std::partition(idx.begin() + first, idx.begin() + first + count, [&](int t) { return bin(t) < bsplit; });
                mid = (int)(it - idx.begin());
                if (mid == first || mid == first + count) mid = first + count / 2;
            }
        }
        if (mid == first + count / 2)
            std::nth_element(idx.begin() + first, idx.begin() + mid, idx.begin() + first + count,
                             [&](int u, int v) { return cen[3 * u + axis] < cen[3 * v + axis]; });
        rec(first, mid - first);
        rec(mid, first + count - mid);
        nodes[me].skip = (int)nodes.size();
        return me;
    }
};
} // namespace

void build_bvh(std::vector<HostTri> &tris, std::vector<HostNode> &nodes) {
    nodes.clear();
    if (tris.empty()) return;
    Build b(tris);
    b.rec(0, (int)tris.size());
    nodes = std::move(b.nodes);
    tris = std::move(b.out);
}

/* ---------------------------------------------------------------- splines */
void spline_derivs(int n, const double *x, const double *y, double *d) {
    if (n == 2) {
        d[0] = (y[1] - y[0]) / (x[1] - x[0]);
        d[1] = d[0];
        return;
    }
    std::vector<double> lower(n), diag(n), upper(n), rhs(n);
    lower[0] = 0; diag[0] = 1; upper[0] = 1;
    rhs[0] = 2 * (y[1] - y[0]) / (x[1] - x[0]);
    for (int i = 1; i < n - 1; ++i) {
        double hl = x[i] - x[i - 1], hr = x[i + 1] - x[i];
        lower[i] = hr;
        diag[i] = 2 * (x[i + 1] - x[i - 1]);
        upper[i] = hl;
        rhs[i] = 3 * (y[i] - y[i - 1]) / hl * hr + 3 * (y[i + 1] - y[i]) / hr * hl;
    }
    lower[n - 1] = 1; diag[n - 1] = 1; upper[n - 1] = 0;
    rhs[n - 1] = 2 * (y[n - 1] - y[n - 2]) / (x[n - 1] - x[n - 2]);
    for (int k = 1; k < n; ++k) {
        double f = lower[k] / diag[k - 1];
        diag[k] = diag[k] - f * upper[k - 1];
        rhs[k] = rhs[k] - f * rhs[k - 1];
    }
    d[n - 1] = rhs[n - 1] / diag[n - 1];
    for (int k = n - 2; k >= 0; --k) d[k] = (rhs[k] - upper[k] * d[k + 1]) / diag[k];
}

namespace {
void derivs_along(const std::vector<double> ax[3], const std::vector<double> &tab, int dim, std::vector<double> &out) {
    size_t n[3] = {ax[0].size(), ax[1].size(), ax[2].size()};
    out.assign(tab.size(), 0.0);
    size_t len = n[dim];
    std::vector<double> yv(len), dv(len);
    size_t st[3] = {n[1] * n[2], n[2], 1};
    int d1 = (dim + 1) % 3, d2 = (dim + 2) % 3;
    for (size_t a = 0; a < n[d1]; ++a)
        for (size_t b = 0; b < n[d2]; ++b) {
            size_t base = a * st[d1] + b * st[d2];
            for (size_t k = 0; k < len; ++k) yv[k] = tab[base + k * st[dim]];
            spline_derivs((int)len, ax[dim].data(), yv.data(), dv.data());
            for (size_t k = 0; k < len; ++k) out[base + k * st[dim]] = dv[k];
        }
}
} // namespace

void hermite_nodes(const std::vector<double> ax[3], const double *tabp, int comp, int stride, std::vector<double> &out) {
    size_t tot = ax[0].size() * ax[1].size() * ax[2].size();
    std::vector<double> tab(tabp, tabp + tot), dx, dy, dz, dxy, dxz, dyz, dxyz;
    derivs_along(ax, tab, 0, dx);
    derivs_along(ax, tab, 1, dy);
    derivs_along(ax, tab, 2, dz);
    derivs_along(ax, dx, 1, dxy);
    derivs_along(ax, dx, 2, dxz);
    derivs_along(ax, dy, 2, dyz);
    derivs_along(ax, dxy, 2, dxyz);
    const std::vector<double> *src[8] = {&tab, &dx, &dy, &dz, &dxy, &dxz, &dyz, &dxyz};
    for (size_t i = 0; i < tot; ++i)
        for (int k = 0; k < 8; ++k) out[i * stride + comp * 8 + k] = (*src[k])[i];
}

/* spline1ddiff of spline1dbuildcubic(x, y) (parabolically terminated) at
 * every node: the first node's slope is the spline derivative itself, every
 * other node's is the derivative of the piece on its left at its right end,
 * from the Hermite coefficients as spline1dbuildhermite forms them */
static void node_slopes(int n, const double *x, const double *y, double *ds) {
    std::vector<double> d(n);
    spline_derivs(n, x, y, d.data());
    ds[0] = d[0];
    for (int j = 1; j < n; ++j) {
        const double w = x[j] - x[j - 1], w2 = w * w, w3 = w * w2;
        const double c2 = (3 * (y[j] - y[j - 1]) - 2 * d[j - 1] * w - d[j] * w) / w2;
        const double c3 = (2 * (y[j - 1] - y[j]) + d[j - 1] * w + d[j] * w) / w3;
        const double u = x[j] - x[j - 1];
        ds[j] = d[j - 1] + 2 * u * c2 + 3 * (u * u) * c3;
    }
}

void bicubic_nodes(const std::vector<double> &r, const std::vector<double> &z, const double *tab, int comp, int stride,
                   std::vector<double> &out) {
    const int m = (int)r.size(), n = (int)z.size();
    std::vector<double> dz((size_t)m * n), line(std::max(m, n)), ds(std::max(m, n));
    auto at = [&](int ir, int iz) -> double * { return &out[((size_t)ir * n + iz) * stride + comp * 4]; };
    for (int ir = 0; ir < m; ++ir)
        for (int iz = 0; iz < n; ++iz) at(ir, iz)[0] = tab[(size_t)ir * n + iz];
    for (int iz = 0; iz < n; ++iz) { /* d/dr along each z row */
        for (int ir = 0; ir < m; ++ir) line[ir] = tab[(size_t)ir * n + iz];
        node_slopes(m, r.data(), line.data(), ds.data());
        for (int ir = 0; ir < m; ++ir) at(ir, iz)[1] = ds[ir];
    }
    for (int ir = 0; ir < m; ++ir) { /* d/dz along each r column */
        node_slopes(n, z.data(), tab + (size_t)ir * n, ds.data());
        for (int iz = 0; iz < n; ++iz) { at(ir, iz)[2] = ds[iz]; dz[(size_t)ir * n + iz] = ds[iz]; }
    }
    for (int iz = 0; iz < n; ++iz) { /* d2/drdz: d/dr of d/dz along each z row */
        for (int ir = 0; ir < m; ++ir) line[ir] = dz[(size_t)ir * n + iz];
        node_slopes(m, r.data(), line.data(), ds.data());
        for (int ir = 0; ir < m; ++ir) at(ir, iz)[3] = ds[ir];
    }
}

int node_table32(const std::vector<double> &nodes, int ncomp, std::vector<float> &out) {
    const int stride = (ncomp * 9 + 3) / 4 * 4;
    const size_t nn = nodes.size() / (size_t)(ncomp * 8);
    out.assign(nn * stride, 0.0f);
    for (size_t i = 0; i < nn; ++i)
        for (int c = 0; c < ncomp; ++c) {
            const double *src = &nodes[(i * ncomp + c) * 8];
            float *dst = &out[i * stride + c * 9];
            const float hi = (float)src[0];
            dst[0] = hi;
            dst[1] = (float)(src[0] - (double)hi);
            for (int k = 1; k < 8; ++k) dst[k + 1] = (float)src[k];
        }
    return stride;
}

/* ---------------------------------------------------------------- harmonic */
namespace {
typedef std::map<int, double> Poly; /* packed exponent -> coefficient */
inline int pk(int i, int j, int k) { return i | (j << 4) | (k << 8); }
Poly mul(const Poly &a, const Poly &b) {
    Poly r;
    for (auto &x : a)
        for (auto &y : b) {
            int i = (x.first & 15) + (y.first & 15), j = ((x.first >> 4) & 15) + ((y.first >> 4) & 15),
                k = ((x.first >> 8) & 15) + ((y.first >> 8) & 15);
            r[pk(i, j, k)] += x.second * y.second;
        }
    return r;
}
double fact(int n) { double f = 1; for (int i = 2; i <= n; ++i) f *= i; return f; }
double binom(int n, int k) { return fact(n) / (fact(k) * fact(n - k)); }
} // namespace

bool harmonic_polynomial(int n, const int32_t *l, const int32_t *m, const double *g, std::vector<double> &coef,
                         std::vector<int> &expo, std::string &err) {
    Poly total;
    for (int c = 0; c < n; ++c) {
        int L = l[c], M = m[c];
        if (L < 0 || L > 5 || std::abs(M) > L + 1) {
            err = "invalid HarmonicExpansionBField coefficient (l,m)";
            return false;
        }
        if (g[c] == 0) continue;
        int N = L + 1, A = std::abs(M);
        /* Legendre P_N(u) = 2^-N sum_k (-1)^k C(N,k) C(2N-2k,N) u^(N-2k), then the A-th derivative */
        std::vector<double> pu(N + 1, 0.0);
        for (int k = 0; 2 * k <= N; ++k) pu[N - 2 * k] = std::pow(-1.0, k) * binom(N, k) * binom(2 * N - 2 * k, N) / std::pow(2.0, N);
        std::vector<double> du(N + 1, 0.0);
        for (int p = A; p <= N; ++p) du[p - A] = pu[p] * fact(p) / fact(p - A);
        /* r^(N-A) P_N^(A)(z/r) = sum_p du[p] z^p (x^2+y^2+z^2)^((N-A-p)/2) */
        Poly zr;
        for (int p = 0; p <= N - A; ++p) {
            if (du[p] == 0) continue;
            int q = (N - A - p) / 2;
            Poly r2{{pk(0, 0, 0), 1.0}};
            Poly rr{{pk(2, 0, 0), 1.0}, {pk(0, 2, 0), 1.0}, {pk(0, 0, 2), 1.0}};
            for (int s = 0; s < q; ++s) r2 = mul(r2, rr);
            for (auto &t : r2) {
                int e = t.first + pk(0, 0, p);
                zr[e] += du[p] * t.second;
            }
        }
        /* (x + i y)^A: real part for m >= 0, imaginary part for m < 0 */
        Poly trig;
        for (int j = 0; j <= A; ++j) {
            double b = binom(A, j);
            if (M >= 0 && j % 2 == 0) trig[pk(A - j, j, 0)] += b * ((j / 2) % 2 ? -1.0 : 1.0);
            if (M < 0 && j % 2 == 1) trig[pk(A - j, j, 0)] += b * (((j - 1) / 2) % 2 ? -1.0 : 1.0);
        }
        double C = fact(N - 1) * std::pow(2.0, A) / fact(N + A);
        Poly term = mul(zr, trig);
        for (auto &t : term) total[t.first] += g[c] * C * t.second;
    }
    coef.clear();
    expo.clear();
    for (auto &t : total)
        if (t.second != 0) { expo.push_back(t.first); coef.push_back(t.second); }
    return true;
}

} // namespace pth
