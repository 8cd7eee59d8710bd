/*
 * pt_adjoint.cuh -- data layout and device helpers of the adjoint pass
 * (pt_adjoint): the recording tapes of a lane and the field derivatives the
 * reverse sweep needs.
 *
 * The adjoint differentiates the discrete forward map pathwise: with every
 * accepted step size (trajectory and Bloch), every bisection bracket and the
 * sequence of specular hits frozen, the end spin of a particle is a smooth
 * function of the coefficients G of one harmonic field.  The forward pass
 * (TTracker::IntegrateParticle with IntegrateSpin, src/tracking.cpp:17-173,
 * 373-483) records one segment per accepted trajectory step (its Dormand-
 * Prince data, how it ended) and a Bloch checkpoint every K accepted spin
 * steps; the reverse sweep walks the segments backwards, recomputes each
 * K-step chunk of the Bloch integration from its checkpoint with the stage
 * precession axes recorded, and runs the adjoint of the Bloch steps, of the
 * dense output and of the trajectory's Dormand-Prince step.
 */
#pragma once
#include "pt_lane.cuh"

namespace ptd {

#define PT_ADJ_MAX_COEF 16

/* segment record (doubles) */
enum {
    SEG_TO = 0, SEG_TN = 1, SEG_XEND = 2, SEG_DT0 = 3, SEG_NSPIN = 4, SEG_CK = 5, SEG_FLAGS = 6,
    SEG_XA = 7, SEG_XB = 8, SEG_N = 9,                           /* reflection: bracket [xa, xb], normal */
    SEG_XO = 12, SEG_DXO = 21, SEG_K2 = 30, SEG_K3 = 39, SEG_K4 = 48, SEG_K5 = 57, SEG_K6 = 66,
    SEG_YN = 75, SEG_DYN = 84, SEG_YL = 93, SEG_SPIN = 102,
    SEG_FIRST = 107,                                             /* particle-wide index of its first Bloch step */
    SEG_DOUBLES = 108
};
enum { SEGF_BLOCH = 1, SEGF_REFLECT = 2, SEGF_RESET = 4, SEGF_OTHER = 8 };
/* Bloch checkpoint at particle-wide Bloch step c K: segment index, ts, dt,
 * x[5], dxdt[5], the segment's Bloch steps before it */
enum { CK_SEG = 0, CK_TS = 1, CK_DT = 2, CK_X = 3, CK_DXDT = 8, CK_STEPS = 13, CK_DOUBLES = 14 };
/* chunk record: step start, step size, start spin (3), precession axis at
 * the 7 stages, segment index */
enum { STEP_SEG = 26, STEP_DOUBLES = 27 };

/* per-lane status bits of the adjoint kernels */
enum { ADJ_OVF_SEG = 1, ADJ_OVF_CK = 2, ADJ_OVF_TAPE = 4, ADJ_UNSUPPORTED = 8, ADJ_MISMATCH = 16, ADJ_FAILED = 32, ADJ_CANCELLED = 64 };

/* The forward pass's recording hooks: a segment record per accepted
 * trajectory try, a Bloch checkpoint at the top of every K-th Bloch step of
 * the particle (counted across segments). */
struct FwdTape {
    static constexpr bool kSpinStages = false;
    double *seg = nullptr, *ck = nullptr;
    int cap_seg = 0, cap_ck = 0, K = 1;
    int nseg = 0, nck = 0, status = 0;
    long nspin = 0;                    /* accepted spin steps of the current segment */
    long nspin_tot = 0;                /* accepted spin steps of the particle */
    double k2[9];
    double rx[2] = {0, 0}, rn[3] = {0, 0, 0}; /* reflection of the current step: bracket and normal */
    int reflected = 0, other = 0;
    template <class L> __device__ void on_accept(L &, const double *k2src) {
        for (int c = 0; c < 9; ++c) k2[c] = k2src[c];
    }
    template <class L> __device__ void on_reflect(L &, double xa, double xb, const double *n) {
        rx[0] = xa; rx[1] = xb;
        rn[0] = n[0]; rn[1] = n[1]; rn[2] = n[2];
        ++reflected;
    }
    template <class L> __device__ void on_other(L &) { ++other; }
    template <class L> __device__ void on_segment(L &l, double x, const double *yl, bool reset) {
        if (nseg >= cap_seg) { status |= ADJ_OVF_SEG; reflected = other = 0; return; }
        double *r = seg + (size_t)nseg * SEG_DOUBLES;
        r[SEG_TO] = l.to; r[SEG_TN] = l.tn; r[SEG_XEND] = x; r[SEG_DT0] = 0; r[SEG_NSPIN] = 0; r[SEG_CK] = nck;
        const int f = (reset ? SEGF_RESET : 0) | (reflected == 1 ? SEGF_REFLECT : 0) | ((other || reflected > 1) ? SEGF_OTHER : 0);
        r[SEG_FLAGS] = f;
        r[SEG_XA] = rx[0]; r[SEG_XB] = rx[1];
        for (int k = 0; k < 3; ++k) r[SEG_N + k] = rn[k];
        for (int c = 0; c < 9; ++c) {
            r[SEG_XO + c] = l.xo[c]; r[SEG_DXO + c] = l.dxo[c]; r[SEG_K2 + c] = k2[c];
            r[SEG_K3 + c] = l.k3[c]; r[SEG_K4 + c] = l.k4[c]; r[SEG_K5 + c] = l.k5[c]; r[SEG_K6 + c] = l.k6[c];
            r[SEG_YN + c] = l.yn[c]; r[SEG_DYN + c] = l.dyn[c]; r[SEG_YL + c] = yl[c];
        }
        for (int c = 0; c < 5; ++c) r[SEG_SPIN + c] = l.spin[c];
        r[SEG_FIRST] = (double)nspin_tot;
        ++nseg;
        nspin = 0;
        reflected = other = 0;
    }
    template <class L> __device__ void on_bloch_start(L &, double, double, double dt0) {
        if (nseg == 0 || (status & ADJ_OVF_SEG)) return;
        double *r = seg + (size_t)(nseg - 1) * SEG_DOUBLES;
        r[SEG_DT0] = dt0;
        r[SEG_FLAGS] = (double)((int)r[SEG_FLAGS] | SEGF_BLOCH);
    }
    template <class L> __device__ bool on_step_top(L &, const BlochState &bs) {
        if (nspin_tot % K == 0) {
            if (nck >= cap_ck) { status |= ADJ_OVF_CK; return true; }
            double *c = ck + (size_t)nck * CK_DOUBLES;
            c[CK_SEG] = nseg - 1; c[CK_TS] = bs.ts; c[CK_DT] = bs.dt;
            for (int i = 0; i < 5; ++i) { c[CK_X + i] = bs.x[i]; c[CK_DXDT + i] = bs.dxdt[i]; }
            c[CK_STEPS] = (double)bs.steps;
            ++nck;
        }
        return true;
    }
    template <class L> __device__ bool on_spin_step(L &, double, double, const double *, const double (*)[3]) {
        ++nspin;
        ++nspin_tot;
        if (nseg > 0 && !(status & ADJ_OVF_SEG)) seg[(size_t)(nseg - 1) * SEG_DOUBLES + SEG_NSPIN] = (double)nspin;
        return true;
    }
};

/* The reverse sweep's recording hooks: the accepted steps of one Bloch
 * chunk with the precession axis at every stage. */
struct RecTape {
    static constexpr bool kSpinStages = true;
    double *tape = nullptr;
    int cap = 0, n = 0, overflow = 0;
    int seg_idx = 0; /* segment of the steps being recorded */
    template <class L> __device__ __forceinline__ void on_accept(L &, const double *) {}
    template <class L> __device__ __forceinline__ void on_reflect(L &, double, double, const double *) {}
    template <class L> __device__ __forceinline__ void on_other(L &) {}
    template <class L> __device__ __forceinline__ void on_segment(L &, double, const double *, bool) {}
    template <class L> __device__ __forceinline__ void on_bloch_start(L &, double, double, double) {}
    template <class L> __device__ __forceinline__ bool on_step_top(L &, const BlochState &) { return true; }
    template <class L> __device__ bool on_spin_step(L &, double tso, double h, const double *x, const double (*w)[3]) {
        if (n >= cap) { overflow = 1; return false; }
        double *r = tape + (size_t)n * STEP_DOUBLES;
        r[0] = tso; r[1] = h; r[2] = x[0]; r[3] = x[1]; r[4] = x[2];
        for (int s = 0; s < 7; ++s)
            for (int k = 0; k < 3; ++k) r[5 + 3 * s + k] = w[s][k];
        r[STEP_SEG] = seg_idx;
        ++n;
        return true;
    }
};

/* Gradient, Hessian (H != nullptr) and third derivatives (T != nullptr) of
 * the scalar potential Phi = sum c x^i y^j z^k of a harmonic field at
 * (x, y, z) (offset applied by the caller), added to g, H, T: B = grad Phi,
 * dB/dx = Hessian, the second derivatives of B = third derivatives. */
__device__ __forceinline__ double ffact(int a, int p) { /* a (a-1) ... (a-p+1) */
    double r = 1;
    for (int q = 0; q < p; ++q) r *= (double)(a - q);
    return r;
}
__device__ void phi_derivs(const double *c, const int *e, int n, double x, double y, double z, double g[3], double (*H)[3],
                           double (*T)[3][3]) {
    double px[8], py[8], pz[8];
    px[0] = py[0] = pz[0] = 1.0;
    for (int i = 1; i < 8; ++i) { px[i] = px[i - 1] * x; py[i] = py[i - 1] * y; pz[i] = pz[i - 1] * z; }
    for (int m = 0; m < n; ++m) {
        const int ex[3] = {e[m] & 15, (e[m] >> 4) & 15, (e[m] >> 8) & 15};
        const double cm = c[m];
        auto term = [&](int dx, int dy, int dz) -> double {
            if (dx > ex[0] || dy > ex[1] || dz > ex[2]) return 0.0;
            return cm * ffact(ex[0], dx) * ffact(ex[1], dy) * ffact(ex[2], dz) * px[ex[0] - dx] * py[ex[1] - dy] * pz[ex[2] - dz];
        };
        for (int a = 0; a < 3; ++a) {
            int d1[3] = {0, 0, 0};
            ++d1[a];
            g[a] += term(d1[0], d1[1], d1[2]);
            if (!H) continue;
            for (int b = 0; b < 3; ++b) {
                int d2[3] = {d1[0], d1[1], d1[2]};
                ++d2[b];
                H[a][b] += term(d2[0], d2[1], d2[2]);
                if (T)
                    for (int k = 0; k < 3; ++k) {
                        int d3[3] = {d2[0], d2[1], d2[2]};
                        ++d3[k];
                        T[a][b][k] += term(d3[0], d3[1], d3[2]);
                    }
            }
        }
    }
}

/* B, dB/dx (dB[i][j] = dB_i/dx_j) and, when d2B != nullptr, the second
 * derivatives d2B[i][j][k] of the scene's magnetic field in FP64 -- the
 * field types the adjoint supports (harmonic expansions without a box;
 * checked on the host) */
__device__ void adj_bfield(const DScene &S, double x, double y, double z, double B[3], double dB[3][3], double (*d2B)[3][3]) {
    for (int i = 0; i < 3; ++i) {
        B[i] = 0;
        for (int j = 0; j < 3; ++j) {
            dB[i][j] = 0;
            if (d2B) for (int k = 0; k < 3; ++k) d2B[i][j][k] = 0;
        }
    }
    for (int fi = 0; fi < S.n_fields; ++fi) {
        const DField &f = S.fields[fi];
        if (!f.has_b || f.type != PT_FIELD_HARMONIC || f.bscale == 0.) continue;
        double g[3] = {0, 0, 0}, H[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, T[3][3][3] = {};
        phi_derivs(f.mono_c, f.mono_e, f.n_mono, x + f.offset[0], y + f.offset[1], z + f.offset[2], g, H, d2B ? T : nullptr);
        for (int i = 0; i < 3; ++i) {
            B[i] += f.bscale * g[i];
            for (int j = 0; j < 3; ++j) {
                dB[i][j] += f.bscale * H[i][j];
                if (d2B) for (int k = 0; k < 3; ++k) d2B[i][j][k] += f.bscale * T[i][j][k];
            }
        }
    }
}

/* every basis field b_k = dB/dG_k (k < nc) of harmonic field f at a point,
 * from the basis polynomials over the field's monomials (each monomial
 * value formed once) */
__device__ void adj_basis_all(const DField &f, int nc, double x, double y, double z, double (*b)[3]) {
    x += f.offset[0];
    y += f.offset[1];
    z += f.offset[2];
    double px[7], py[7], pz[7];
    px[0] = py[0] = pz[0] = 1.0;
    for (int i = 1; i <= f.hp_deg; ++i) { px[i] = px[i - 1] * x; py[i] = py[i - 1] * y; pz[i] = pz[i - 1] * z; }
    const int n = f.hp_n;
    for (int k = 0; k < nc; ++k) b[k][0] = b[k][1] = b[k][2] = 0;
    for (int m = 0; m < n; ++m) {
        const int e = f.hp_e[m];
        const double v = px[e & 15] * py[(e >> 4) & 15] * pz[(e >> 8) & 15];
        for (int k = 0; k < nc; ++k) {
            const double *c = f.basis_hp + (size_t)k * 3 * n + m;
            b[k][0] = fma(c[0], v, b[k][0]);
            b[k][1] = fma(c[n], v, b[k][1]);
            b[k][2] = fma(c[2 * n], v, b[k][2]);
        }
    }
    for (int k = 0; k < nc; ++k)
        for (int i = 0; i < 3; ++i) b[k][i] *= f.bscale;
}

/* basis field b_k = dB/dG_k of coefficient k of harmonic field f and, when
 * db != nullptr, its Jacobian */
__device__ void adj_basis(const DField &f, int k, double x, double y, double z, double b[3], double (*db)[3]) {
    for (int i = 0; i < 3; ++i) {
        b[i] = 0;
        if (db) for (int j = 0; j < 3; ++j) db[i][j] = 0;
    }
    const int a = f.term_start[k], n = f.term_start[k + 1] - a;
    phi_derivs(f.basis_c + a, f.basis_e + a, n, x + f.offset[0], y + f.offset[1], z + f.offset[2], b, db, nullptr);
    for (int i = 0; i < 3; ++i) {
        b[i] *= f.bscale;
        if (db) for (int j = 0; j < 3; ++j) db[i][j] *= f.bscale;
    }
}

} // namespace ptd
