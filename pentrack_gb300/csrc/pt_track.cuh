/*
 * pt_track.cuh -- per-lane tracking physics (device functions).
 *
 * Restates, for one particle per lane, the reference's hot loop
 *   TTracker::IntegrateParticle   src/tracking.cpp:17-173
 *   TTracker::CheckHit            src/tracking.cpp:176-226   (tail recursion -> loop)
 *   TTracker::iterate_collision   src/tracking.cpp:228-265   (recursion -> path-bit DFS)
 *   TTracker::DoStep / DoHit      src/tracking.cpp:268-365
 *   TTracker::IntegrateSpin       src/tracking.cpp:373-483   (decision logic; LOOP D not on device)
 *   TParticle::derivs / EquationOfMotion / energies  src/particle.cpp:96-135, 196-269
 *   TNeutron::OnHit / OnStep / Reflect* / Transmit*  src/neutron.cpp:25-282
 *   TProton / TElectron ::OnStep  src/proton.cpp:25-33, src/electron.cpp:25-32
 *   TFieldManager / TFieldContainer / TabField3     src/fields.cpp:139-182, src/field.cpp:48-169,
 *                                                   src/field_3d.cpp:487-529
 *   TGeometry::GetCollisions / GetSolids, TTriangleMesh::Collision
 *                                 src/geometry.cpp:139-175, src/trianglemesh.cpp:134-171
 * and Boost.odeint's dense-output Dormand-Prince 5(4) stepper with its
 * default error checker and step adjuster (abs = rel = 1e-9, src/tracking.cpp:63).
 */
#pragma once
#include "pt_device.cuh"
#include "../../include/pt_solenoid.h"

namespace ptd {
/* internal linkage: every kernel translation unit has its own copy */
namespace {

/* ---------------------------------------------------------------- */
/* Philox4x32-10 stream keyed by (seed, particle id)                 */
/* ---------------------------------------------------------------- */
__device__ __forceinline__ double uniform(uint64_t seed, int64_t id, uint64_t draw) {
    uint32_t x0 = (uint32_t)draw, x1 = (uint32_t)(draw >> 32), x2 = (uint32_t)(uint64_t)id, x3 = (uint32_t)((uint64_t)id >> 32);
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(0xD2511F53u, x0), lo0 = 0xD2511F53u * x0;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, x2), lo1 = 0xCD9E8D57u * x2;
        uint32_t y0 = hi1 ^ x1 ^ k0, y2 = hi0 ^ x3 ^ k1;
        x0 = y0; x1 = lo1; x2 = y2; x3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    uint64_t v = ((uint64_t)x0 << 32) | x1;
    return (double)(v >> 11) * 0x1.0p-53;
}

/* ---------------------------------------------------------------- */
/* exact-rounding geometric predicates (no FMA contraction, so the   */
/* signs equal the oracle's FP64 evaluation bit for bit)             */
/* ---------------------------------------------------------------- */
__device__ __forceinline__ double orient3d(const double *a, const double *b, const double *c, const double *d) {
    double adx = __dsub_rn(a[0], d[0]), bdx = __dsub_rn(b[0], d[0]), cdx = __dsub_rn(c[0], d[0]);
    double ady = __dsub_rn(a[1], d[1]), bdy = __dsub_rn(b[1], d[1]), cdy = __dsub_rn(c[1], d[1]);
    double adz = __dsub_rn(a[2], d[2]), bdz = __dsub_rn(b[2], d[2]), cdz = __dsub_rn(c[2], d[2]);
    double t1 = __dmul_rn(adx, __dsub_rn(__dmul_rn(bdy, cdz), __dmul_rn(bdz, cdy)));
    double t2 = __dmul_rn(bdx, __dsub_rn(__dmul_rn(cdy, adz), __dmul_rn(cdz, ady)));
    double t3 = __dmul_rn(cdx, __dsub_rn(__dmul_rn(ady, bdz), __dmul_rn(adz, bdy)));
    return __dadd_rn(__dadd_rn(t1, t2), t3);
}
__device__ __forceinline__ bool lex_less(const double *u, const double *v) {
    if (u[0] != v[0]) return u[0] < v[0];
    if (u[1] != v[1]) return u[1] < v[1];
    return u[2] < v[2];
}
__device__ __forceinline__ double edge_orient(const double *p, const double *q, const double *u, const double *v) {
    if (lex_less(v, u)) return -orient3d(p, q, v, u);
    return orient3d(p, q, u, v);
}
/* ---------------------------------------------------------------- */
/* Certified FP32 segment-triangle decisions.  The FP64 test seg_tri  */
/* decides from signs of orient3d determinants.  Each sign is first  */
/* computed in FP32 from inputs rounded to FP32, with a bound on its  */
/* error: moving each point by at most d = 2^-23 M per coordinate     */
/* (M = max |coordinate|) changes 6x the tetrahedron volume by at     */
/* most 2 d (sum of products of its edge lengths); the FP32           */
/* arithmetic adds at most 16 eps32 x the permanent; the FP64         */
/* rounding of seg_tri's own determinant is far below both.  A sign   */
/* whose magnitude exceeds twice that bound equals the exact sign and */
/* hence seg_tri's FP64 sign, so decided cases need no FP64 work.     */
/* ---------------------------------------------------------------- */
struct Seg32 {
    float p[3], q[3];
    float m; /* max |coordinate| of p, q (FP64 values), rounded up */
};
__device__ __forceinline__ void seg32_make(const double *p, const double *q, Seg32 &s) {
    double m = 0;
    for (int k = 0; k < 3; ++k) {
        s.p[k] = (float)p[k];
        s.q[k] = (float)q[k];
        m = fmax(m, fmax(fabs(p[k]), fabs(q[k])));
    }
    s.m = __double2float_ru(m);
}
/* orient3d(a, b, c, d) in FP32 with its certification bound; returns the
 * sign (+1/-1) when certain, 0 otherwise */
__device__ __forceinline__ int orient_sign32(const float *a, const float *b, const float *c, const float *d, float M) {
    const float adx = a[0] - d[0], bdx = b[0] - d[0], cdx = c[0] - d[0];
    const float ady = a[1] - d[1], bdy = b[1] - d[1], cdy = c[1] - d[1];
    const float adz = a[2] - d[2], bdz = b[2] - d[2], cdz = c[2] - d[2];
    const float bc = bdy * cdz - bdz * cdy, ca = cdy * adz - cdz * ady, ab = ady * bdz - adz * bdy;
    const float det = adx * bc + bdx * ca + cdx * ab;
    const float perm = fabsf(adx) * (fabsf(bdy * cdz) + fabsf(bdz * cdy)) + fabsf(bdx) * (fabsf(cdy * adz) + fabsf(cdz * ady)) +
                       fabsf(cdx) * (fabsf(ady * bdz) + fabsf(adz * bdy));
    const float la = fabsf(adx) + fabsf(ady) + fabsf(adz), lb = fabsf(bdx) + fabsf(bdy) + fabsf(bdz),
                lc = fabsf(cdx) + fabsf(cdy) + fabsf(cdz);
    const float lab = fabsf(bdx - adx) + fabsf(bdy - ady) + fabsf(bdz - adz);
    const float lac = fabsf(cdx - adx) + fabsf(cdy - ady) + fabsf(cdz - adz);
    const float d_in = 2.4e-7f * M; /* 2 x 2^-23 M: rounding of the inputs, with slack */
    const float s2 = lb * lc + la * lc + la * lb + lab * lac;
    const float bound = 2.0f * (2.0f * d_in * s2 + 2.0e-6f * perm) + 1e-30f;
    if (det > bound) return 1;
    if (det < -bound) return -1;
    return 0;
}
/* 1: certainly a point hit, 0: certainly no hit, -1: undecided (use seg_tri) */
__device__ __forceinline__ int seg_tri32(const Seg32 &s, const DTri32 &t) {
    const float M = fmaxf(s.m, t.m);
    const int sp = orient_sign32(t.a, t.b, t.c, s.p, M), sq = orient_sign32(t.a, t.b, t.c, s.q, M);
    if (sp != 0 && sp == sq) return 0;         /* both ends strictly on one side */
    if (sp == 0 || sq == 0) return -1;
    /* the segment crosses the plane: the edge signs decide (canonical edge order as in edge_orient) */
    const float *v[3] = {t.a, t.b, t.c};
    int e[3];
    for (int k = 0; k < 3; ++k) {
        const float *u = v[k], *w = v[(k + 1) % 3];
        bool swap = (w[0] < u[0]) || (w[0] == u[0] && (w[1] < u[1] || (w[1] == u[1] && w[2] < u[2])));
        int sg = swap ? -orient_sign32(s.p, s.q, w, u, M) : orient_sign32(s.p, s.q, u, w, M);
        e[k] = sg;
    }
    bool neg = (e[0] < 0) || (e[1] < 0) || (e[2] < 0), pos = (e[0] > 0) || (e[1] > 0) || (e[2] > 0);
    if (neg && pos) return 0;                  /* certainly outside */
    if (e[0] != 0 && e[1] != 0 && e[2] != 0) return 1; /* certainly inside */
    return -1;
}

/* Certified decision from FP64 differences, the second tier after
 * seg_tri32.  The plane sides are n . (x - a) with the FP64 normal n =
 * (b - a) x (c - a) (orient3d(a, b, c, x) = -n_exact . (x - a)); the edge
 * signs are orient3d(p, q, u, v) = (p - v) . ((q - p) x (u - v)) evaluated in
 * FP32 from FP64 differences, whose relative rounding does not depend on the
 * distance from the origin.  Each value is compared against its own error
 * bound plus the error bound of seg_tri's FP64 orient3d, (7 + 56 eps) eps x
 * permanent (Shewchuk, "Adaptive precision floating-point arithmetic and
 * fast robust geometric predicates", 1997), with the permanent bounded by
 * 6 x the product of the three difference norms; a value that clears both
 * has the sign of the exact determinant and of seg_tri's FP64 one.
 * 1: hit, 0: no hit, -1: undecided. */
__device__ __forceinline__ int seg_tri64c(const double *p, const double *q, const Seg32 &s, const DTri &t, const DTri32 &t32,
                                          const DTriC &c) {
    const float u32 = 5.9604645e-8f;  /* 2^-24 */
    const float e64 = 1.1102231e-16f; /* 2^-53, rounded up */
    const float din = 2.4e-7f * fmaxf(s.m, t32.m); /* rounding of both FP32 copies of a coordinate difference */
    float Rp = 0, Rq = 0;
    for (int k = 0; k < 3; ++k) {
        Rp = fmaxf(Rp, fabsf(s.p[k] - t32.a[k]));
        Rq = fmaxf(Rq, fabsf(s.q[k] - t32.a[k]));
    }
    Rp = (Rp + din) * 1.0001f; /* >= |p - a|_inf */
    Rq = (Rq + din) * 1.0001f;
    double da[3], qa[3];
    for (int k = 0; k < 3; ++k) { da[k] = p[k] - t.a[k]; qa[k] = q[k] - t.a[k]; }
    const double sp = fma(c.n[0], da[0], fma(c.n[1], da[1], c.n[2] * da[2]));
    const double sq = fma(c.n[0], qa[0], fma(c.n[1], qa[1], c.n[2] * qa[2]));
    /* |sp - n_exact . (p - a)| <= 3 dn R + 4 eps |n|_1 R; seg_tri's orient3d(a, b, c, p) is within
     * 7.01 eps x 6 R (ea + R)^2 of the exact determinant */
    const float bp = 1.01f * ((3.0f * c.dn + 5.0f * e64 * c.n1) * Rp + 42.1f * e64 * Rp * (c.ea + Rp) * (c.ea + Rp));
    const float bq = 1.01f * ((3.0f * c.dn + 5.0f * e64 * c.n1) * Rq + 42.1f * e64 * Rq * (c.ea + Rq) * (c.ea + Rq));
    const float fp = __double2float_rz(sp), fq = __double2float_rz(sq);
    const int gp = fp > bp ? 1 : (fp < -bp ? -1 : 0), gq = fq > bq ? 1 : (fq < -bq ? -1 : 0);
    if (gp == 0 || gq == 0) return -1;
    if (gp == gq) return 0; /* both ends strictly on one side */
    /* the segment crosses the plane: edge signs (canonical order as in edge_orient) */
    float D[3], Dn = 0;
    for (int k = 0; k < 3; ++k) {
        D[k] = (float)(q[k] - p[k]);
        Dn = fmaxf(Dn, fabsf(D[k]));
    }
    Dn *= 1.0001f;
    bool neg = false, pos = false, unsure = false;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int vi = (c.edges >> (2 * k)) & 3;
        const double *v = vi == 0 ? t.a : (vi == 1 ? t.b : t.c);
        float r[3], Rn = 0;
        for (int i = 0; i < 3; ++i) {
            r[i] = (float)(p[i] - v[i]);
            Rn = fmaxf(Rn, fabsf(r[i]));
        }
        Rn *= 1.0001f;
        const float *E = c.e[k];
        const float c0 = D[1] * E[2] - D[2] * E[1], c1 = D[2] * E[0] - D[0] * E[2], c2 = D[0] * E[1] - D[1] * E[0];
        const float val = r[0] * c0 + r[1] * c1 + r[2] * c2;
        const float P = fabsf(r[0]) * (fabsf(D[1] * E[2]) + fabsf(D[2] * E[1])) + fabsf(r[1]) * (fabsf(D[2] * E[0]) + fabsf(D[0] * E[2])) +
                        fabsf(r[2]) * (fabsf(D[0] * E[1]) + fabsf(D[1] * E[0]));
        const float b = 1.01f * (16.0f * u32 * P + 42.1f * e64 * Rn * (Rn + Dn) * c.en[k]);
        int g = val > b ? 1 : (val < -b ? -1 : 0);
        if ((c.edges >> (6 + k)) & 1) g = -g;
        neg = neg || g < 0;
        pos = pos || g > 0;
        unsure = unsure || g == 0;
    }
    if (neg && pos) return 0; /* certainly outside */
    return unsure ? -1 : 1;
}

/* closed segment x closed triangle: 1 hit (parameter s), 0 none, -1 coplanar */
__device__ __forceinline__ int seg_tri(const double *p, const double *q, const DTri &t, double &s) {
    double dp = orient3d(t.a, t.b, t.c, p), dq = orient3d(t.a, t.b, t.c, q);
    if ((dp > 0 && dq > 0) || (dp < 0 && dq < 0)) return 0;
    if (dp == 0 && dq == 0) return -1;
    double e1 = edge_orient(p, q, t.a, t.b), e2 = edge_orient(p, q, t.b, t.c), e3 = edge_orient(p, q, t.c, t.a);
    bool neg = (e1 < 0) || (e2 < 0) || (e3 < 0), pos = (e1 > 0) || (e2 > 0) || (e3 > 0);
    if (neg && pos) return 0;
    s = __ddiv_rn(dp, __dsub_rn(dp, dq));
    return 1;
}

/* principal complex square root (same formula as the oracle) */
__device__ __forceinline__ void csqrt(double a, double b, double &re, double &im) {
    double m = sqrt(a * a + b * b);
    if (a >= 0) {
        double t = sqrt((a + m) * 0.5);
        re = t;
        im = (t == 0) ? b : b / (2 * t);
    } else {
        double t = sqrt((m - a) * 0.5);
        re = fabs(b) / (2 * t);
        im = copysign(t, b);
    }
}

/* ---------------------------------------------------------------- */
/* fields                                                            */
/* ---------------------------------------------------------------- */
__device__ __forceinline__ bool fbox_has(const DField &f) { return f.xmin < f.xmax && f.ymin < f.ymax && f.zmin < f.zmax; }
__device__ __forceinline__ bool fbox_in(const DField &f, double x, double y, double z) {
    if (!fbox_has(f)) return true;
    return x >= f.xmin && x < f.xmax && y >= f.ymin && y < f.ymax && z >= f.zmin && z < f.zmax;
}
__device__ __forceinline__ double smthr(double x) { return ((6 * x - 15) * x + 10) * x * x * x; }
__device__ __forceinline__ double smthr_der(double x) { return ((30 * x - 60) * x + 30) * x * x; }

/* TFieldBoundaryBox::scaleScalarFieldAtBounds (src/field.cpp:71-112) */
__device__ void scale_at_bounds(const DField &f, double x, double y, double z, double &F, double *dF) {
    if (!fbox_has(f) || (F == 0 && dF == nullptr) || (F == 0 && dF[0] == 0 && dF[1] == 0 && dF[2] == 0)) return;
    if (!fbox_in(f, x, y, z)) {
        F = 0.;
        if (dF) dF[0] = dF[1] = dF[2] = 0.;
    } else if (f.bw > 0) {
        double Fscale = 1.;
        double dFadd[3] = {0., 0., 0.};
        double lo[3] = {(x - f.xmin) / f.bw, (y - f.ymin) / f.bw, (z - f.zmin) / f.bw};
        double hi[3] = {(f.xmax - x) / f.bw, (f.ymax - y) / f.bw, (f.zmax - z) / f.bw};
        for (int i = 0; i < 3; ++i) {
            if (0 <= lo[i] && lo[i] <= 1) {
                Fscale *= smthr(lo[i]);
                if (dF) dFadd[i] += F * smthr_der(lo[i]) / f.bw / smthr(lo[i]);
            } else if (0 <= hi[i] && hi[i] <= 1) {
                Fscale *= smthr(hi[i]);
                if (dF) dFadd[i] += -F * smthr_der(hi[i]) / f.bw / smthr(hi[i]);
            }
        }
        if (Fscale != 1.) {
            F *= Fscale;
            if (dF)
                for (int i = 0; i < 3; i++) dF[i] = dF[i] * Fscale + dFadd[i] * Fscale;
        }
    }
}

/* upper_bound cell search of TabField3::Interpolate (src/field_3d.cpp:492-501):
 * first grid coordinate > r; outside when none or the first one. */
__device__ __forceinline__ bool locate(const DField &f, int a, double r, int &idx, double &u, double &h) {
    const double *ax = f.ax[a];
    int n = f.n[a];
    double g = (r - f.a0[a]) * f.inv_h[a];
    int k;
    if (!(g > -1.0)) k = 0;
    else if (!(g < (double)n)) k = n;
    else k = (int)floor(g) + 1;
    while (k < n && ax[k] <= r) ++k;
    while (k > 0 && ax[k - 1] > r) --k;
    if (k >= n || k == 0) return false;
    idx = k - 1;
    h = ax[k] - ax[k - 1];
    u = (r - ax[k - 1]) / h;
    return true;
}

template <class T> struct Herm {
    T w[4], dw[4];
    /* cubic Hermite weights of (f(0), f(1), h f'(0), h f'(1)) and their
     * derivatives with respect to the physical coordinate */
    __device__ __forceinline__ void set(T t, T h, T invh) {
        T t2 = t * t, t3 = t2 * t;
        w[0] = (T)2 * t3 - (T)3 * t2 + (T)1;
        w[1] = (T)3 * t2 - (T)2 * t3;
        w[2] = h * (t3 - (T)2 * t2 + t);
        w[3] = h * (t3 - t2);
        dw[0] = ((T)6 * t2 - (T)6 * t) * invh;
        dw[1] = ((T)6 * t - (T)6 * t2) * invh;
        dw[2] = (T)3 * t2 - (T)4 * t + (T)1;
        dw[3] = (T)3 * t2 - (T)2 * t;
    }
};

/* Tricubic value (+ gradient) of `nc` components starting at `c0` in one cell
 * from the per-node Hermite data (f, fx, fy, fz, fxy, fxz, fyz, fxyz).  The
 * tensor-product cubic Hermite interpolant equals the reference's
 * Lekien-Marsden polynomial (src/field_3d.cpp:367-414 + tricubic_get_coeff):
 * both are the unique tricubic matching those 64 corner data. */
template <class T, bool GRAD, bool SKIPF = false>
__device__ void hermite_cell(const T *__restrict__ nodes, int ncomp, int c0, int nc, const int *n, int ix, int iy, int iz,
                             const Herm<T> &U, const Herm<T> &V, const Herm<T> &W, double *F, double (*dF)[3]) {
    const int dtab[2][2][2] = {{{0, 3}, {2, 6}}, {{1, 5}, {4, 7}}};
    const int64_t sz = n[2], sy = (int64_t)n[1] * n[2];
    const int64_t base = ((int64_t)ix * n[1] + iy) * n[2] + iz;
    const int stride = ncomp * 8;
    for (int c = c0; c < c0 + nc; ++c) {
        T f = 0, fx = 0, fy = 0, fz = 0;
#pragma unroll
        for (int cx = 0; cx < 2; ++cx)
#pragma unroll
            for (int ax = 0; ax < 2; ++ax) {
                const int p = cx + 2 * ax;
                T tp = 0, typ = 0, tzp = 0;
#pragma unroll
                for (int cy = 0; cy < 2; ++cy) {
                    const T *n0 = nodes + (base + cx * sy + cy * sz) * stride + c * 8;
                    const T *n1 = n0 + stride;
#pragma unroll
                    for (int ay = 0; ay < 2; ++ay) {
                        const int q = cy + 2 * ay;
                        const int d0 = dtab[ax][ay][0], d1 = dtab[ax][ay][1];
                        T v0 = n0[d0], v1 = n1[d0], v2 = n0[d1], v3 = n1[d1];
                        if (SKIPF && ax == 0 && ay == 0) { v0 = 0; v1 = 0; } /* value data handled in FP64 */
                        T s = v0 * W.w[0] + v1 * W.w[1] + v2 * W.w[2] + v3 * W.w[3];
                        tp += s * V.w[q];
                        if (GRAD) {
                            T sp = v0 * W.dw[0] + v1 * W.dw[1] + v2 * W.dw[2] + v3 * W.dw[3];
                            typ += s * V.dw[q];
                            tzp += sp * V.w[q];
                        }
                    }
                }
                f += tp * U.w[p];
                if (GRAD) {
                    fx += tp * U.dw[p];
                    fy += typ * U.w[p];
                    fz += tzp * U.w[p];
                }
            }
        F[c - c0] = (double)f;
        if (GRAD) {
            dF[c - c0][0] = (double)fx;
            dF[c - c0][1] = (double)fy;
            dF[c - c0][2] = (double)fz;
        }
    }
}

/* Cell lookup on one axis of the FP32 node table: the cell index and the
 * local coordinate, false outside the grid. */
__device__ __forceinline__ bool locate32(const DField &f, int a, float r, int &idx, float &loc) {
    const float *ax = f.ax32[a];
    const int n = f.n[a];
    const float g = (r - f.a0f[a]) * f.inv_hf[a];
    int k;
    if (!(g > -1.0f)) k = 0;
    else if (!(g < (float)n)) k = n;
    else k = (int)floorf(g) + 1;
    while (k < n && ax[k] <= r) ++k;
    while (k > 0 && ax[k - 1] > r) --k;
    if (k >= n || k == 0) return false;
    idx = k - 1;
    loc = (r - ax[k - 1]) * f.inv_w32[a][k - 1];
    return true;
}

/* FP32 field mode: tricubic value (+ gradient) of components C0 .. C0+NC-1
 * from the FP32 node table.  The component range is a template constant so
 * that the outputs stay in registers. */
template <bool GRAD, int C0, int NC>
__device__ void tab3_f32(const DField &f, float x, float y, float z, float *F, float (*dF)[3]) {
    int ix, iy, iz;
    float u, v, w;
    if (!locate32(f, 0, x, ix, u) || !locate32(f, 1, y, iy, v) || !locate32(f, 2, z, iz, w)) return;
    Herm<float> U, V, W;
    U.set(u, f.ax32[0][ix + 1] - f.ax32[0][ix], f.inv_w32[0][ix]);
    V.set(v, f.ax32[1][iy + 1] - f.ax32[1][iy], f.inv_w32[1][iy]);
    W.set(w, f.ax32[2][iz + 1] - f.ax32[2][iz], f.inv_w32[2][iz]);
    /* Node records of the cell's corners.  The tricubic is evaluated as the
     * linear function L = f0 + g0 . (r - r0) of corner (0, 0, 0) (value f0 from
     * its FP32 high/low parts, gradient g0 from its derivative data) plus the
     * interpolant of f - L, which cubic Hermite interpolation reproduces
     * exactly.  The data of f - L are curvature-sized, so FP32 accumulation
     * keeps B and grad B to ~1e-7 relative instead of cancelling. */
    const int S = f.node32_stride;
    const int64_t nz = f.n[2], nyz = (int64_t)f.n[1] * nz;
    const float *T0 = f.node32 + (((int64_t)ix * f.n[1] + iy) * nz + iz) * S;
    const float hx = f.ax32[0][ix + 1] - f.ax32[0][ix], hy = f.ax32[1][iy + 1] - f.ax32[1][iy],
                hz = f.ax32[2][iz + 1] - f.ax32[2][iz];
    const float rx = x - f.ax32[0][ix], ry = y - f.ax32[1][iy], rz = z - f.ax32[2][iz];
    const int dtab[2][2][2] = {{{0, 3}, {2, 6}}, {{1, 5}, {4, 7}}};
#pragma unroll
    for (int c = C0; c < C0 + NC; ++c) {
        const float h0 = T0[c * 9], l0 = T0[c * 9 + 1];
        const float g[3] = {T0[c * 9 + 2], T0[c * 9 + 3], T0[c * 9 + 4]};
        float fr = 0, fx = 0, fy = 0, fz = 0;
#pragma unroll
        for (int cx = 0; cx < 2; ++cx)
#pragma unroll
            for (int ax_ = 0; ax_ < 2; ++ax_) {
                const int p = cx + 2 * ax_;
                float tp = 0, typ = 0, tzp = 0;
#pragma unroll
                for (int cy = 0; cy < 2; ++cy) {
                    const float *n0 = T0 + (cx * nyz + cy * nz) * S + c * 9; /* corner (cx, cy, 0) */
                    const float *n1 = n0 + S;                               /* corner (cx, cy, 1) */
                    const float lxy = fmaf(g[1], cy ? hy : 0.0f, g[0] * (cx ? hx : 0.0f)); /* L - f0 at (cx, cy, 0) */
#pragma unroll
                    for (int ay = 0; ay < 2; ++ay) {
                        const int q = cy + 2 * ay;
                        const int d0 = dtab[ax_][ay][0], d1 = dtab[ax_][ay][1];
                        float v0, v1, v2, v3;
                        if (d0 == 0) {
                            v0 = ((n0[0] - h0) + (n0[1] - l0)) - lxy;
                            v1 = ((n1[0] - h0) + (n1[1] - l0)) - fmaf(g[2], hz, lxy);
                        } else if (d0 <= 3) {
                            v0 = n0[d0 + 1] - g[d0 - 1];
                            v1 = n1[d0 + 1] - g[d0 - 1];
                        } else {
                            v0 = n0[d0 + 1];
                            v1 = n1[d0 + 1];
                        }
                        if (d1 <= 3) {
                            v2 = n0[d1 + 1] - g[d1 - 1];
                            v3 = n1[d1 + 1] - g[d1 - 1];
                        } else {
                            v2 = n0[d1 + 1];
                            v3 = n1[d1 + 1];
                        }
                        const float sv = fmaf(v3, W.w[3], fmaf(v2, W.w[2], fmaf(v1, W.w[1], v0 * W.w[0])));
                        tp = fmaf(sv, V.w[q], tp);
                        if (GRAD) {
                            const float sp = fmaf(v3, W.dw[3], fmaf(v2, W.dw[2], fmaf(v1, W.dw[1], v0 * W.dw[0])));
                            typ = fmaf(sv, V.dw[q], typ);
                            tzp = fmaf(sp, V.w[q], tzp);
                        }
                    }
                }
                fr = fmaf(tp, U.w[p], fr);
                if (GRAD) {
                    fx = fmaf(tp, U.dw[p], fx);
                    fy = fmaf(typ, U.w[p], fy);
                    fz = fmaf(tzp, U.w[p], fz);
                }
            }
        F[c - C0] = h0 + (l0 + (fmaf(g[2], rz, fmaf(g[1], ry, g[0] * rx)) + fr));
        if (GRAD) {
            dF[c - C0][0] = g[0] + fx;
            dF[c - C0][1] = g[1] + fy;
            dF[c - C0][2] = g[2] + fz;
        }
    }
}

/* TabField3 B (and gradient) of one field; outputs untouched outside the grid */
template <bool GRAD>
__device__ void tab3_b(const DField &f, double x, double y, double z, double B[3], double (*dB)[3]) {
    int ix, iy, iz;
    double u, v, w, hx, hy, hz;
    if (!locate(f, 0, x, ix, u, hx) || !locate(f, 1, y, iy, v, hy) || !locate(f, 2, z, iz, w, hz)) return;
    {
        Herm<double> U, V, W;
        U.set(u, hx, 1.0 / hx);
        V.set(v, hy, 1.0 / hy);
        W.set(w, hz, 1.0 / hz);
        hermite_cell<double, GRAD>(f.node64, f.ncomp, 0, 3, f.n, ix, iy, iz, U, V, W, B, dB);
    }
}

/* TabField3 potential V and E = -grad V */
__device__ void tab3_v(const DField &f, int prec, double x, double y, double z, double &Vv, double E[3]) {
    double F[1] = {Vv}, dF[1][3] = {{0, 0, 0}};
    if (prec == PT_PREC_FP32 && f.node32) {
        float F32[1] = {(float)Vv}, dF32[1][3] = {{0, 0, 0}};
        tab3_f32<true, 3, 1>(f, (float)x, (float)y, (float)z, F32, dF32);
        F[0] = F32[0];
        for (int k = 0; k < 3; ++k) dF[0][k] = dF32[0][k];
    } else {
        int ix, iy, iz;
        double u, v, w, hx, hy, hz;
        if (!locate(f, 0, x, ix, u, hx) || !locate(f, 1, y, iy, v, hy) || !locate(f, 2, z, iz, w, hz)) return;
        Herm<double> U, V, W;
        U.set(u, hx, 1.0 / hx);
        V.set(v, hy, 1.0 / hy);
        W.set(w, hz, 1.0 / hz);
        hermite_cell<double, true>(f.node64, f.ncomp, 3, 1, f.n, ix, iy, iz, U, V, W, F, dF);
    }
    Vv = F[0];
    E[0] = -dF[0][0];
    E[1] = -dF[0][1];
    E[2] = -dF[0][2];
}

/* ---- TabField: ALGLIB's bicubic spline2d in (r, z) (src/field_2d.cpp:232-399) ---- */

/* the cell of spline2dcalc / spline2ddiff's bisection: l in [0, n-2] with
 * ax[l] < v <= ax[l+1] (l = 0 at the first node), found from the
 * uniform-grid guess and walked to the same answer */
__device__ __forceinline__ int cell2(const DField &f, int a, double v) {
    const double *ax = f.ax[a];
    const int n = f.n[a];
    const double g = (v - f.a0[a]) * f.inv_h[a];
    int l = 0;
    if (g > 0.0) l = g < (double)(n - 2) ? (int)g : n - 2;
    while (l > 0 && ax[l] >= v) --l;
    while (l < n - 2 && ax[l + 1] < v) ++l;
    return l;
}

/* Hermite basis of one cell in the library's form and operation order:
 * ht/hu weigh the value and (scaled by the cell width) slope data, dht/dhu
 * are their derivatives.  DIFF: spline2ddiff (t = (v - x_l) / w), else
 * spline2dcalc (t = (v - x_l) * (1 / w)). */
struct Bic2 {
    double ht[4], hu[4];   /* h00, h01, h10, h11 */
    double dht[4], dhu[4];
    int64_t s1, s2, s3, s4; /* nodes (l_r, l_z), (l_r + 1, l_z), (l_r, l_z + 1), (l_r + 1, l_z + 1) */
};

template <bool DIFF>
__device__ __forceinline__ void bic2_basis(double t, double dt, double *h, double *dh) {
    const double t2 = t * t, t3 = t * t2;
    h[0] = 2 * t3 - 3 * t2 + 1;
    h[1] = -2 * t3 + 3 * t2;
    h[2] = (t3 - 2 * t2 + t) / dt;
    h[3] = (t3 - t2) / dt;
    if (DIFF) {
        dh[0] = (6 * t2 - 6 * t) * dt;
        dh[1] = (-6 * t2 + 6 * t) * dt;
        dh[2] = 3 * t2 - 4 * t + 1;
        dh[3] = 3 * t2 - 2 * t;
    }
}

template <bool DIFF>
__device__ __forceinline__ void bic2_setup(const DField &f, double r, double z, Bic2 &b) {
    const int lr = cell2(f, 0, r), lz = cell2(f, 2, z);
    const double *ar = f.ax[0], *az = f.ax[2];
    double t, dt, u, du;
    if (DIFF) {
        t = (r - ar[lr]) / (ar[lr + 1] - ar[lr]);
        dt = 1.0 / (ar[lr + 1] - ar[lr]);
        u = (z - az[lz]) / (az[lz + 1] - az[lz]);
        du = 1.0 / (az[lz + 1] - az[lz]);
    } else {
        dt = 1.0 / (ar[lr + 1] - ar[lr]);
        t = (r - ar[lr]) * dt;
        du = 1.0 / (az[lz + 1] - az[lz]);
        u = (z - az[lz]) * du;
    }
    bic2_basis<DIFF>(t, dt, b.ht, b.dht);
    bic2_basis<DIFF>(u, du, b.hu, b.dhu);
    const int64_t nz = f.n[2];
    b.s1 = (int64_t)lr * nz + lz;
    b.s2 = b.s1 + nz;
    b.s3 = b.s1 + 1;
    b.s4 = b.s2 + 1;
}

/* one component: the 16 products in spline2ddiff's order (value, d/dr
 * data, d/dz data, d2/drdz data); DIFF adds the r and z derivatives */
template <bool DIFF>
__device__ __forceinline__ void bic2_eval(const DField &f, const Bic2 &b, int c, double &F, double &Fr, double &Fz) {
    const double *n1 = f.node64 + b.s1 * (PT_T2_NCOMP * 4) + c * 4, *n2 = f.node64 + b.s2 * (PT_T2_NCOMP * 4) + c * 4,
                 *n3 = f.node64 + b.s3 * (PT_T2_NCOMP * 4) + c * 4, *n4 = f.node64 + b.s4 * (PT_T2_NCOMP * 4) + c * 4;
    double v = 0, vr = 0, vz = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        /* data k: 0 value, 1 d/dr, 2 d/dz, 3 d2/drdz; it pairs with the r
         * basis of slope (k & 1) and the z basis of slope (k >> 1) */
        const double v0 = n1[k], v1 = n2[k], v2 = n3[k], v3 = n4[k];
        const int pr = (k & 1) ? 2 : 0, pz = (k & 2) ? 2 : 0;
        const double p0 = b.ht[pr], p1 = b.ht[pr + 1], q0 = b.hu[pz], q1 = b.hu[pz + 1];
        v = v + v0 * p0 * q0 + v1 * p1 * q0 + v2 * p0 * q1 + v3 * p1 * q1;
        if (DIFF) {
            const double dp0 = b.dht[pr], dp1 = b.dht[pr + 1], dq0 = b.dhu[pz], dq1 = b.dhu[pz + 1];
            vr = vr + v0 * dp0 * q0 + v1 * dp1 * q0 + v2 * dp0 * q1 + v3 * dp1 * q1;
            vz = vz + v0 * p0 * dq0 + v1 * p1 * dq0 + v2 * p0 * dq1 + v3 * p1 * dq1;
        }
    }
    F = v;
    if (DIFF) { Fr = vr; Fz = vz; }
}

__device__ __forceinline__ bool tab2_in(const DField &f, double r, double z) {
    return r >= f.t2_lim[0] && r < f.t2_lim[1] && z >= f.t2_lim[2] && z < f.t2_lim[3];
}

/* cos(phi), sin(phi) of phi = atan2(y, x) as x / r, y / r ((1, 0) on the axis) */
__device__ __forceinline__ void tab2_angle(double x, double y, double r, double &cp, double &sp) {
    if (r > 0) { cp = x / r; sp = y / r; }
    else { cp = 1.0; sp = 0.0; }
}

/* TabField::BField (src/field_2d.cpp:289-335); outputs untouched outside the range */
template <bool GRAD>
__device__ __noinline__ void tab2_b(const DField &f, double x, double y, double z, double B[3], double (*dB)[3]) {
    const double r = sqrt(x * x + y * y);
    if (!tab2_in(f, r, z)) return;
    double cp, sp;
    tab2_angle(x, y, r, cp, sp);
    Bic2 b;
    bic2_setup<GRAD>(f, r, z, b);
    double Br = 0, Bphi = 0, Bz = 0, dBrdr = 0, dBrdz = 0, dBphidr = 0, dBphidz = 0, dBzdr = 0, dBzdz = 0;
    if (f.t2_mask & 1) bic2_eval<GRAD>(f, b, 0, Br, dBrdr, dBrdz);
    if (f.t2_mask & 2) bic2_eval<GRAD>(f, b, 1, Bphi, dBphidr, dBphidz);
    if (f.t2_mask & 4) bic2_eval<GRAD>(f, b, 2, Bz, dBzdr, dBzdz);
    if (GRAD) {
        if (r > 0) {
            dB[0][0] = dBrdr * cp * cp - dBphidr * cp * sp + (Br * sp * sp + Bphi * cp * sp) / r;
            dB[0][1] = dBrdr * cp * sp - dBphidr * sp * sp - (Br * cp * sp + Bphi * cp * cp) / r;
            dB[1][0] = dBrdr * cp * sp + dBphidr * cp * cp - (Br * cp * sp - Bphi * sp * sp) / r;
            dB[1][1] = dBrdr * sp * sp + dBphidr * cp * sp + (Br * cp * cp - Bphi * cp * sp) / r;
        }
        dB[0][2] = dBrdz * cp - dBphidz * sp;
        dB[1][2] = dBrdz * sp + dBphidz * cp;
        if (f.t2_mask & 4) {
            dB[2][0] = dBzdr * cp;
            dB[2][1] = dBzdr * sp;
            dB[2][2] = dBzdz;
        }
    }
    B[0] = Br * cp - Bphi * sp;
    B[1] = Br * sp + Bphi * cp;
    B[2] = Bz;
}

/* TabField::EField (src/field_2d.cpp:337-399): an E map (values) takes
 * precedence over the potential (value and gradient) */
__device__ __noinline__ void tab2_e(const DField &f, double x, double y, double z, double &V, double E[3]) {
    const double r = sqrt(x * x + y * y);
    if (!tab2_in(f, r, z)) return;
    double cp, sp;
    tab2_angle(x, y, r, cp, sp);
    double d0, d1;
    if (f.t2_mask & 0x70) {
        Bic2 b;
        bic2_setup<false>(f, r, z, b);
        double Er = 0, Ephi = 0, Ez = 0;
        if (f.t2_mask & 16) bic2_eval<false>(f, b, 4, Er, d0, d1);
        if (f.t2_mask & 32) bic2_eval<false>(f, b, 5, Ephi, d0, d1);
        if (f.t2_mask & 64) bic2_eval<false>(f, b, 6, Ez, d0, d1);
        E[0] = Er * cp - Ephi * sp;
        E[1] = Er * sp + Ephi * cp;
        E[2] = Ez;
    } else if (f.t2_mask & 8) {
        Bic2 b;
        bic2_setup<true>(f, r, z, b);
        double dVdr, dVdz;
        bic2_eval<true>(f, b, 3, V, dVdr, dVdz);
        E[0] = -dVdr * cp;
        E[1] = -dVdr * sp;
        E[2] = -dVdz;
    }
}

/* finite solenoid (include/pt_solenoid.h); one out-of-line copy: its
 * elliptic-integral loops would otherwise be inlined at every field call */
__device__ __noinline__ void solenoid_b(const DField &f, double x, double y, double z, double B[3], double (*dB)[3]) {
    pts_solenoid_field(f.sol_a, f.sol_b, f.sol_B0, x - f.offset[0], y - f.offset[1], z - f.offset[2], B, dB);
}

/* harmonic expansion: B = grad Phi of a polynomial Phi (offset applied),
 * evaluated from the precomputed polynomials of B and of its Jacobian over
 * one set of monomials (each monomial value formed once, then one FMA per
 * output) */
template <bool GRAD>
__device__ void harmonic_b(const DField &f, double x, double y, double z, double B[3], double (*dB)[3]) {
    x += f.offset[0];
    y += f.offset[1];
    z += f.offset[2];
    double px[7], py[7], pz[7];
    px[0] = py[0] = pz[0] = 1.0;
    for (int i = 1; i <= f.hp_deg; ++i) { px[i] = px[i - 1] * x; py[i] = py[i - 1] * y; pz[i] = pz[i - 1] * z; }
    const int n = f.hp_n, n1 = f.hp_n1;
    const double *c = f.hp_c;
    double b0 = 0, b1 = 0, b2 = 0, d00 = 0, d01 = 0, d02 = 0, d11 = 0, d12 = 0, d22 = 0;
    for (int m = 0; m < n; ++m) {
        const int e = f.hp_e[m];
        const double v = px[e & 15] * py[(e >> 4) & 15] * pz[(e >> 8) & 15];
        b0 = fma(c[m], v, b0);
        b1 = fma(c[n + m], v, b1);
        b2 = fma(c[2 * n + m], v, b2);
        if (GRAD && m < n1) {
            d00 = fma(c[3 * n + m], v, d00);
            d01 = fma(c[4 * n + m], v, d01);
            d02 = fma(c[5 * n + m], v, d02);
            d11 = fma(c[6 * n + m], v, d11);
            d12 = fma(c[7 * n + m], v, d12);
            d22 = fma(c[8 * n + m], v, d22);
        }
    }
    B[0] += b0;
    B[1] += b1;
    B[2] += b2;
    if (GRAD) {
        dB[0][0] += d00; dB[0][1] += d01; dB[0][2] += d02;
        dB[1][0] += d01; dB[1][1] += d11; dB[1][2] += d12;
        dB[2][0] += d02; dB[2][1] += d12; dB[2][2] += d22;
    }
}

/* TFieldManager::BField (src/fields.cpp:139-164) over TFieldContainer::BField
 * (src/field.cpp:139-155) in FP64 */
template <bool GRAD>
__device__ void bfield64(const DScene &S, double x, double y, double z, double B[3], double (*dB)[3]) {
    B[0] = B[1] = B[2] = 0;
    if (GRAD)
        for (int i = 0; i < 3; ++i) dB[i][0] = dB[i][1] = dB[i][2] = 0;
    for (int fi = 0; fi < S.n_fields; ++fi) {
        const DField &f = S.fields[fi];
        if (!f.has_b) continue;
        if (!fbox_in(f, x, y, z) || f.bscale == 0.) continue;
        double Bt[3] = {0, 0, 0}, dBt[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        if (f.type == PT_FIELD_TAB3D) tab3_b<GRAD>(f, x, y, z, Bt, dBt);
        else if (f.type == PT_FIELD_HARMONIC) harmonic_b<GRAD>(f, x, y, z, Bt, dBt);
        else if (f.type == PT_FIELD_SOLENOID) solenoid_b(f, x, y, z, Bt, GRAD ? dBt : nullptr);
        else if (f.type == PT_FIELD_TAB2D) tab2_b<GRAD>(f, x, y, z, Bt, dBt);
        for (int i = 0; i < 3; ++i) {
            Bt[i] *= f.bscale;
            if (GRAD) for (int j = 0; j < 3; ++j) dBt[i][j] *= f.bscale;
        }
        for (int i = 0; i < 3; ++i) scale_at_bounds(f, x, y, z, Bt[i], GRAD ? dBt[i] : nullptr);
        for (int i = 0; i < 3; ++i) {
            B[i] += Bt[i];
            if (GRAD) for (int j = 0; j < 3; ++j) dB[i][j] += dBt[i][j];
        }
    }
}

/* One field of a type without an FP32 table, evaluated in FP64 and rounded */
template <bool GRAD>
__device__ __forceinline__ void bfield_other32(const DField &f, double x, double y, double z, float Bt[3], float (*dBt)[3]) {
    double Bd[3] = {0, 0, 0}, dBd[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    if (f.type == PT_FIELD_TAB3D) tab3_b<GRAD>(f, x, y, z, Bd, dBd);
    else if (f.type == PT_FIELD_HARMONIC) harmonic_b<GRAD>(f, x, y, z, Bd, dBd);
    else if (f.type == PT_FIELD_SOLENOID) solenoid_b(f, x, y, z, Bd, GRAD ? dBd : nullptr);
    else if (f.type == PT_FIELD_TAB2D) tab2_b<GRAD>(f, x, y, z, Bd, dBd);
    for (int i = 0; i < 3; ++i) {
        Bd[i] *= f.bscale;
        if (GRAD) for (int j = 0; j < 3; ++j) dBd[i][j] *= f.bscale;
    }
    for (int i = 0; i < 3; ++i) scale_at_bounds(f, x, y, z, Bd[i], GRAD ? dBd[i] : nullptr);
    for (int i = 0; i < 3; ++i) {
        Bt[i] = (float)Bd[i];
        if (GRAD) for (int j = 0; j < 3; ++j) dBt[i][j] = (float)dBd[i][j];
    }
}

/* The same superposition in the FP32 field mode: tables without a smoothing
 * band are evaluated in FP32 from the cell's FP32 linear base plus the FP32
 * Hermite remainder (relative error ~1e-7 in B and grad B, no cancellation
 * since the base gradient is stored); every other field is evaluated in FP64
 * and rounded.  TAB_ONLY: the scene's magnetic fields are all such tables
 * (checked on the host), so the other field types are compiled out. */
template <bool GRAD, bool TAB_ONLY = false>
__device__ void bfield32(const DScene &S, double x, double y, double z, float B[3], float (*dB)[3]) {
    B[0] = B[1] = B[2] = 0;
    if (GRAD)
        for (int i = 0; i < 3; ++i) dB[i][0] = dB[i][1] = dB[i][2] = 0;
    for (int fi = 0; fi < S.n_fields; ++fi) {
        const DField &f = S.fields[fi];
        if (!f.has_b) continue;
        if (!fbox_in(f, x, y, z) || f.bscale == 0.) continue;
        float Bt[3] = {0, 0, 0}, dBt[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        if (f.type == PT_FIELD_TAB3D && f.node32 && !(f.bw > 0 && fbox_has(f))) {
            tab3_f32<GRAD, 0, 3>(f, (float)x, (float)y, (float)z, Bt, dBt);
            if (f.bscale != 1.0) {
                const float sc = (float)f.bscale;
                for (int i = 0; i < 3; ++i) {
                    Bt[i] *= sc;
                    if (GRAD) for (int j = 0; j < 3; ++j) dBt[i][j] *= sc;
                }
            }
        } else if (!TAB_ONLY) {
            bfield_other32<GRAD>(f, x, y, z, Bt, dBt);
        }
        for (int i = 0; i < 3; ++i) {
            B[i] += Bt[i];
            if (GRAD) for (int j = 0; j < 3; ++j) dB[i][j] += dBt[i][j];
        }
    }
}

/* B (and grad B) in the requested field precision */
template <bool GRAD>
__device__ void bfield(const DScene &S, int prec, double x, double y, double z, double B[3], double (*dB)[3]) {
    if (prec == PT_PREC_FP32) {
        float Bf[3], dBf[3][3];
        bfield32<GRAD>(S, x, y, z, Bf, dBf);
        for (int i = 0; i < 3; ++i) {
            B[i] = Bf[i];
            if (GRAD) for (int j = 0; j < 3; ++j) dB[i][j] = dBf[i][j];
        }
        return;
    }
    bfield64<GRAD>(S, x, y, z, B, dB);
}

/* TFieldManager::EField (src/fields.cpp:167-182) */
__device__ void efield(const DScene &S, int prec, double x, double y, double z, double &V, double E[3]) {
    V = 0;
    E[0] = E[1] = E[2] = 0;
    for (int fi = 0; fi < S.n_fields; ++fi) {
        const DField &f = S.fields[fi];
        if (!f.has_v) continue;
        if (!fbox_in(f, x, y, z) || f.escale == 0.) continue;
        double Vt = 0, Et[3] = {0, 0, 0};
        if (f.type == PT_FIELD_UNIFORM_E) {
            Et[0] = f.e[0]; Et[1] = f.e[1]; Et[2] = f.e[2];
            Vt = Et[2] * z;
        } else if (f.type == PT_FIELD_TAB3D) {
            tab3_v(f, prec, x, y, z, Vt, Et);
        } else if (f.type == PT_FIELD_TAB2D) {
            tab2_e(f, x, y, z, Vt, Et);
        }
        Vt *= f.escale;
        for (int i = 0; i < 3; ++i) Et[i] *= f.escale;
        scale_at_bounds(f, x, y, z, Vt, Et);
        V += Vt;
        for (int i = 0; i < 3; ++i) E[i] += Et[i];
    }
}

/* ---------------------------------------------------------------- */
/* geometry queries                                                  */
/* ---------------------------------------------------------------- */
struct Coll {
    double s, n[3], dn;
    int solid;
    uint32_t id;
    bool ign;
};

__device__ __forceinline__ bool solid_ignored(const DSolid &s, double t) {
    for (int i = 0; i < s.n_ign; ++i)
        if (t >= s.ign[2 * i] && t < s.ign[2 * i + 1]) return true;
    return false;
}

__device__ __forceinline__ bool seg_box(const double *p, const double *q, const double *lo, const double *hi) {
    double t0 = 0, t1 = 1;
    for (int k = 0; k < 3; ++k) {
        double d = q[k] - p[k];
        if (d == 0) {
            if (p[k] < lo[k] || p[k] > hi[k]) return false;
            continue;
        }
        double ta = __ddiv_rn(__dsub_rn(lo[k], p[k]), d), tb = __ddiv_rn(__dsub_rn(hi[k], p[k]), d);
        if (ta > tb) { double tt = ta; ta = tb; tb = tt; }
        t0 = fmax(t0, ta);
        t1 = fmin(t1, tb);
        if (t0 > t1) return false;
    }
    return true;
}

/* TGeometry::CheckSegment (include/geometry.h:104-106) */
__device__ bool check_segment(const DScene &S, const double *p, const double *q) {
    for (int s = 1; s < S.n_solids; ++s) {
        const DSolid &so = S.solids[s];
        if (so.lo[0] > so.hi[0]) continue;
        if (seg_box(p, q, so.lo, so.hi)) return true;
    }
    return false;
}

struct QueryStats { unsigned nodes, tris; };

/* the triangle's own box touches the box of segment p-q (exact FP64 compares,
 * the pre-test the oracle applies before every segment-triangle test) */
__device__ __forceinline__ bool tri_box_touch(const DTri &t, const double *p, const double *q) {
    for (int k = 0; k < 3; ++k) {
        double tlo = fmin(t.a[k], fmin(t.b[k], t.c[k])), thi = fmax(t.a[k], fmax(t.b[k], t.c[k]));
        double slo = fmin(p[k], q[k]), shi = fmax(p[k], q[k]);
        if (tlo > shi || thi < slo) return false;
    }
    return true;
}

/* Separating-axis overlap test of a triangle and an axis-aligned box given by
 * centre c and half sizes e (Akenine-Moeller, "Fast 3D triangle-box overlap
 * testing", 2001): box axes, triangle normal, and the nine edge x axis
 * cross products, in FP32 on the triangle's FP32 copy.  Every axis the test
 * uses is the FP32 vector it computes, taken as exact; the vertices' FP32
 * rounding (<= 2^-24 of the coordinate each for the vertex and the centre)
 * and the arithmetic of a projection (<= 3 x 2^-24 of its terms) move a
 * projection by at most |axis|_1 x 10 x 2^-24 x M, M the largest coordinate
 * magnitude involved; the caller widens e by that much per unit axis, so
 * separation is only reported where it exactly holds.  A candidate set built
 * with it can only be too large, never miss a triangle. */
__device__ bool tri_box_overlap32(const DTri32 &t, const float *c, const float *e) {
    float v0[3], v1[3], v2[3];
    for (int k = 0; k < 3; ++k) { v0[k] = t.a[k] - c[k]; v1[k] = t.b[k] - c[k]; v2[k] = t.c[k] - c[k]; }
    for (int k = 0; k < 3; ++k) {
        const float mn = fminf(v0[k], fminf(v1[k], v2[k])), mx = fmaxf(v0[k], fmaxf(v1[k], v2[k]));
        if (mn > e[k] || mx < -e[k]) return false;
    }
    float f[3][3];
    for (int k = 0; k < 3; ++k) { f[0][k] = v1[k] - v0[k]; f[1][k] = v2[k] - v1[k]; f[2][k] = v0[k] - v2[k]; }
    const float *vv[3] = {v0, v1, v2};
#pragma unroll
    for (int i = 0; i < 3; ++i)       /* edge i */
#pragma unroll
        for (int a = 0; a < 3; ++a) { /* box axis a: axis = e_a x f_i */
            const int a1 = (a + 1) % 3, a2 = (a + 2) % 3;
            const float x1 = -f[i][a2], x2 = f[i][a1];
            float pmin = 3e38f, pmax = -3e38f;
            for (int v = 0; v < 3; ++v) {
                const float pr = x1 * vv[v][a1] + x2 * vv[v][a2];
                pmin = fminf(pmin, pr);
                pmax = fmaxf(pmax, pr);
            }
            const float r = (e[a1] * fabsf(x1) + e[a2] * fabsf(x2)) * 1.0000005f;
            if (pmin > r || pmax < -r) return false;
        }
    /* plane of the triangle */
    const float d = t.n[0] * v0[0] + t.n[1] * v0[1] + t.n[2] * v0[2];
    const float r = (e[0] * fabsf(t.n[0]) + e[1] * fabsf(t.n[1]) + e[2] * fabsf(t.n[2])) * 1.0000005f;
    if (d > r || d < -r) return false;
    return true;
}

/* indices of the triangles that may touch the box [lo, hi]; -1 if more than maxc */
__device__ int collect_candidates(const DScene &S, const double *lo, const double *hi, int *cand, int maxc, QueryStats &qs) {
    float flo[3], fhi[3], c[3], e[3];
    double m = 0;
    for (int k = 0; k < 3; ++k) {
        flo[k] = __double2float_rd(lo[k]);
        fhi[k] = __double2float_ru(hi[k]);
        c[k] = (float)(0.5 * (lo[k] + hi[k]));
        m = fmax(m, fmax(fabs(lo[k]), fabs(hi[k])));
    }
    const float M = __double2float_ru(m);
    for (int k = 0; k < 3; ++k) e[k] = __double2float_ru(0.5 * (hi[k] - lo[k]));
    int nc = 0;
    int i = 0;
    while (i < S.n_nodes) {
        const DNode nd = S.nodes[i];
        ++qs.nodes;
        bool ov = !(nd.lo[0] > fhi[0] || nd.hi[0] < flo[0] || nd.lo[1] > fhi[1] || nd.hi[1] < flo[1] || nd.lo[2] > fhi[2] ||
                    nd.hi[2] < flo[2]);
        if (!ov) { i = nd.skip; continue; }
        if (nd.leaf < 0) { ++i; continue; }
        int first = nd.leaf >> 3, cnt = nd.leaf & 7;
        for (int j = first; j < first + cnt; ++j) {
            const DTri32 &t = S.tri32[j];
            /* widen the box by the FP32 error bound of the test (per unit axis) */
            const float w = 1.3e-6f * fmaxf(M, t.m) + 1e-30f;
            const float ew[3] = {e[0] + w, e[1] + w, e[2] + w};
            if (!tri_box_overlap32(t, c, ew)) continue;
            if (nc >= maxc) return -1;
            cand[nc++] = j;
        }
        i = nd.skip;
    }
    return nc;
}

/* Stackless traversal of the depth-first BVH with FP32 boxes rounded outward;
 * the segment box is rounded outward too, so no triangle the FP64 test would
 * hit is ever skipped.  mode 0: stop at the first hit; mode 1: collect all
 * (sorted by s, then solid ID descending); mode 2: ray parity mask. */
template <int MODE>
__device__ int mesh_query(const DScene &S, const double *p, const double *q, double x1, double x2, Coll *out, int maxc,
                          uint64_t *mask, QueryStats &qs, bool &coplanar) {
    float lo[3], hi[3];
    for (int k = 0; k < 3; ++k) {
        double a = fmin(p[k], q[k]), b = fmax(p[k], q[k]);
        lo[k] = __double2float_rd(a);
        hi[k] = __double2float_ru(b);
    }
    int nh = 0;
    coplanar = false;
    int i = 0;
    const int nn = S.n_nodes;
    Seg32 s32;
    seg32_make(p, q, s32);
    /* Slab test of the segment against a node's box, for segments whose box is
     * loose (long diagonal chords).  The FP32 segment o + t d, t in [0, 1], is
     * within eps of the FP64 one everywhere, so boxes are widened by eps with
     * outward rounding; the t interval is computed as in Ize, "Robust BVH Ray
     * Traversal" (JCGT 2, 2013), and a node is skipped only when the interval
     * is empty by more than 1e-6, above the FP32 error of t near [0, 1]. */
    float so[3], sinv[3];
    double sm = 0, sd = 0;
    for (int k = 0; k < 3; ++k) {
        const double dk = q[k] - p[k];
        so[k] = (float)p[k];
        const float d32 = (float)dk;
        sinv[k] = d32 != 0.0f ? 1.0f / d32 : 0.0f;
        sm = fmax(sm, fabs(p[k]));
        sd = fmax(sd, fabs(dk));
    }
    const float seps = __double2float_ru(1.2e-7 * (sm + sd) + 1e-30);
    const bool slab = (MODE != 2) && sd > 2e-3;
    while (i < nn) {
        const DNode nd = S.nodes[i];
        ++qs.nodes;
        bool ov = !(nd.lo[0] > hi[0] || nd.hi[0] < lo[0] || nd.lo[1] > hi[1] || nd.hi[1] < lo[1] || nd.lo[2] > hi[2] ||
                    nd.hi[2] < lo[2]);
        if (ov && slab) {
            float t0 = 0.0f, t1 = 1.0f;
            for (int k = 0; k < 3; ++k) {
                if (sinv[k] == 0.0f) continue; /* parallel to this slab: the box test above decides */
                const float a = (__fsub_rd(nd.lo[k], seps) - so[k]) * sinv[k], b = (__fadd_ru(nd.hi[k], seps) - so[k]) * sinv[k];
                t0 = fmaxf(t0, fminf(a, b));
                t1 = fminf(t1, fmaxf(a, b));
            }
            ov = !(t0 > t1 + 1e-6f); /* both ends lie in [0, 1] when close: an absolute slack above 2 gamma_3 */
        }
        if (!ov) { i = nd.skip; continue; }
        if (nd.leaf < 0) { ++i; continue; }
        int first = nd.leaf >> 3, cnt = nd.leaf & 7;
        for (int j = first; j < first + cnt; ++j) {
            const int r32 = seg_tri32(s32, S.tri32[j]);
            if (r32 == 0) continue;
            if (MODE == 0 && r32 == 1) return 1; /* a certain hit ends an any-hit query */
            const DTri &t = S.tris[j];
            if (r32 < 0) {
                const int r64 = seg_tri64c(p, q, s32, t, S.tri32[j], S.tric[j]);
                if (r64 == 0) continue;
                if (MODE == 0 && r64 == 1) return 1;
            }
            if (MODE != 2 && !tri_box_touch(t, p, q)) continue;
            ++qs.tris;
            double s;
            int r = seg_tri(p, q, t, s);
            if (r < 0) {
                if (MODE != 2) coplanar = true;
                continue;
            }
            if (r == 0) continue;
            if (MODE == 0) return 1;
            if (MODE == 2) { *mask ^= (1ull << t.solid); continue; }
            Coll c;
            c.s = s;
            c.n[0] = t.n[0]; c.n[1] = t.n[1]; c.n[2] = t.n[2];
            c.solid = t.solid;
            c.id = S.solids[t.solid].id;
            c.dn = (q[0] - p[0]) * t.n[0] + (q[1] - p[1]) * t.n[1] + (q[2] - p[2]) * t.n[2];
            c.ign = solid_ignored(S.solids[t.solid], x1 + (x2 - x1) * s);
            if (nh < maxc) {
                /* insertion sort: ascending s, descending ID on ties (src/trianglemesh.cpp:151-161) */
                int k = nh;
                while (k > 0 && (out[k - 1].s > c.s || (out[k - 1].s == c.s && out[k - 1].id < c.id))) {
                    out[k] = out[k - 1];
                    --k;
                }
                out[k] = c;
            }
            ++nh;
        }
        i = nd.skip;
    }
    return nh;
}

/* TTriangleMesh::GetSolids (include/trianglemesh.h:181-188): +z ray parity */
__device__ uint64_t point_solids(const DScene &S, const double *p, QueryStats &qs) {
    double q[3] = {p[0], p[1], fmax(S.mesh_zmax, p[2]) + 1.0};
    uint64_t mask = 0;
    bool cp;
    mesh_query<2>(S, p, q, 0, 0, nullptr, 0, &mask, qs, cp);
    return mask;
}

} // namespace
} // namespace ptd
