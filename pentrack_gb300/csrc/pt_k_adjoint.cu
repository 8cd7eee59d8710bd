/*
 * pt_k_adjoint.cu -- the adjoint pass: gradients of the end spin (Bloch
 * integration, TTracker::IntegrateSpin src/tracking.cpp:373-483, with
 * TParticle::SpinDerivs / SpinPrecessionAxis src/particle.cpp:141-193) and
 * of the end trajectory state with respect to the coefficients of one
 * harmonic field (HarmonicExpandedBField, src/harmonicfields.cpp:50-829),
 * taken pathwise along the particle's fixed sequence of specular hits
 * (TNeutron::Reflect, src/neutron.cpp:99-115).
 *
 * Discretise-then-differentiate: the derivative is that of the forward
 * kernels' own arithmetic with every accepted step size, every bisection
 * bracket and every hit frozen (a hit's time is a bracket end, a fixed
 * fraction of its step, so the discrete map has no hit-time saltation term).
 * Terms of the exact derivative below 1e-15 relative for UCN are left out
 * and named where they are (the v-dependence of the Lorentz factors, the
 * Thomas term, v (v.F)/c^2 in the equation of motion).
 */
#include "pt_kcommon.cuh"
#include "pt_adjoint.cuh"
#include "pt_kernels.cuh"

namespace ptk {

/* ---------------- forward pass with recording ---------------- */

/* One lane per particle, warp-synchronous like k_plain_spin: a lane whose
 * step reaches its Bloch integration runs one try of its Bloch step per loop
 * iteration, every lane stays in the loop and the warp is re-synchronised at
 * its top; the FwdTape hooks record the segments and the checkpoints. */
__global__ void __launch_bounds__(128) k_adj_forward(const __grid_constant__ DScene S, const __grid_constant__ DRun R,
                                                     const __grid_constant__ DBatch b, DCounters *C, const __grid_constant__ DAdj A) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool have = i < b.n;
    LaneT<FwdTape> L(S, R);
    double t0 = 0;
    bool done = !have, inbloch = false;
    if (have) {
        L.tp.seg = A.seg + (size_t)i * A.cap_seg * SEG_DOUBLES;
        L.tp.cap_seg = A.cap_seg;
        L.tp.ck = A.ck + (size_t)i * A.cap_ck * CK_DOUBLES;
        L.tp.cap_ck = A.cap_ck;
        L.tp.K = A.K;
        L.load(b, i);
        t0 = L.t;
        done = L.stop != PT_ID_UNKNOWN;
    }
    int fin = 0, waited = 0;
    /* a trajectory step ended (or the tape ran out): whether the lane stops */
    auto step_end = [&]() {
        if (L.tp.status || L.stop != PT_ID_UNKNOWN) done = true;
        else if (*R.cancel) { L.tp.status |= ADJ_CANCELLED; done = true; }
        return done;
    };
    for (;;) { /* the passes of k_plain_spin, trajectory work batched the same way */
        __syncwarp();
        if (__all_sync(0xffffffffu, done)) break;
        const bool traj = !done && !inbloch;
        const int ntraj = __popc(__ballot_sync(0xffffffffu, traj));
        const bool go = ntraj >= TRAJ_BATCH || !__any_sync(0xffffffffu, !done && inbloch) ||
                        __any_sync(0xffffffffu, traj && waited >= TRAJ_WAIT);
        if (done) continue;
        if (inbloch) {
            const int r = L.bloch_try(L.bst, L.bx2);
            if (r != 0 && r != 2) {
                fin = r;
                inbloch = false;
                waited = 0;
            }
            if (L.tp.status) done = true;
            continue;
        }
        if (!go) {
            ++waited;
            continue;
        }
        waited = 0;
        if (fin) {
            L.bloch_finish(fin);
            fin = 0;
            if (step_end()) continue;
        }
        int r;
        do { r = L.rk_try(); } while (r == 0);
        if (r < 0) {
            L.stop = PT_ID_ODEINT_ERROR;
            step_end();
            continue;
        }
        L.ps.stage = PS_BEGIN;
        int q;
        while ((q = L.post_resume<true>()) == 1)
            L.ps.bres = L.bisect(L.ps.cx1, L.ps.cya, L.ps.x2, L.ps.y2, L.ps.bxa, L.ps.bao, L.ps.bxb, L.ps.bbo);
        if (q == 2) {
            inbloch = true;
            if (L.tp.status) done = true;
        } else {
            step_end();
        }
    }
    if (have) {
        L.store(b, i);
        A.nseg[i] = L.tp.nseg;
        A.nck[i] = L.tp.nck;
        A.status[i] = L.tp.status;
        flush_counters(C, L.lc, L.t - t0, false);
    }
}

/* ---------------- reverse sweep ---------------- */

using RLane = LaneT<RecTape>;

/* cotangents of one trajectory segment's dense-output data: xo (lxo) and
 * the stage vectors K1 = dxo, K2, K3 .. K6, K7 = dyn (lK[0..6]); position and
 * velocity components */
struct SegAdj {
    double lxo[6], lK[7][6];
};

/* adjoint of calc_state at time t: lam (position, velocity) into the dense
 * data's cotangents */
static __device__ void dense_adj(const RLane &L, double t, const double *lam, SegAdj &a) {
    double hb[6];
    L.dense_coef(t, hb);
    const int kidx[6] = {0, 2, 3, 4, 5, 6};
    for (int c = 0; c < 6; ++c) {
        a.lxo[c] += lam[c];
        for (int k = 0; k < 6; ++k) a.lK[kidx[k]][c] += hb[k] * lam[c];
    }
}

/* adjoint of the neutral equation of motion dx/dt = v, dv/dt = s (F_grav +
 * pol mu grad|B|) at y (position, velocity): out = J^T lam, lG += (df/dG)^T
 * lam.  J's position block is s pol mu times the Hessian of |B|; the
 * dependence of s (the Lorentz factor) on v and the v (v.F)/c^2 term are
 * relative 1e-16 for UCN and left out. */
static __device__ void eom_adj(const DScene &S, const DRun &R, const DField &F, int nc, double pol, const double *y, const double *lam,
                               double *out, double *lG) {
    out[3] = lam[0]; out[4] = lam[1]; out[5] = lam[2];
    out[0] = out[1] = out[2] = 0;
    const DSpecies &sp = R.sp;
    if (sp.mu == 0 || pol == 0) return;
    double B[3], dB[3][3], d2B[3][3][3];
    adj_bfield(S, y[0], y[1], y[2], B, dB, d2B);
    const double Bn = sqrt(B[0] * B[0] + B[1] * B[1] + B[2] * B[2]);
    if (Bn == 0) return;
    const double Bh[3] = {B[0] / Bn, B[1] / Bn, B[2] / Bn};
    const double v2 = y[3] * y[3] + y[4] * y[4] + y[5] * y[5];
    const double sc = sqrt(1 - v2 * PT_INV_C0_SQ) * sp.inv_mkg * pol * sp.mu;
    double gB[3]; /* (dB)^T Bh = grad|B| */
    for (int j = 0; j < 3; ++j) gB[j] = Bh[0] * dB[0][j] + Bh[1] * dB[1][j] + Bh[2] * dB[2][j];
    /* Hessian of |B|: sum_i Bh_i d2B_i + (dB^T dB - grad|B| grad|B|^T) / |B| */
    for (int j = 0; j < 3; ++j) {
        double o = 0;
        for (int k = 0; k < 3; ++k) {
            double h = Bh[0] * d2B[0][j][k] + Bh[1] * d2B[1][j][k] + Bh[2] * d2B[2][j][k];
            h += (dB[0][j] * dB[0][k] + dB[1][j] * dB[1][k] + dB[2][j] * dB[2][k] - gB[j] * gB[k]) / Bn;
            o += h * lam[3 + k];
        }
        out[j] = sc * o;
    }
    /* d(grad|B|)/dG_k = db_k^T Bh + dB^T (b_k - Bh (Bh.b_k)) / |B| */
    for (int k = 0; k < nc; ++k) {
        double bk[3], dbk[3][3];
        adj_basis(F, k, y[0], y[1], y[2], bk, dbk);
        const double bb = Bh[0] * bk[0] + Bh[1] * bk[1] + Bh[2] * bk[2];
        double s = 0;
        for (int j = 0; j < 3; ++j) {
            double g = Bh[0] * dbk[0][j] + Bh[1] * dbk[1][j] + Bh[2] * dbk[2][j];
            g += (dB[0][j] * (bk[0] - Bh[0] * bb) + dB[1][j] * (bk[1] - Bh[1] * bb) + dB[2][j] * (bk[2] - Bh[2] * bb)) / Bn;
            s += g * lam[3 + j];
        }
        lG[k] += sc * s;
    }
}

/* adjoint of one spin right-hand side dS = (W x S, 1, |W|) at time t with
 * stage spin Ss and precession axis W: lSs = d/dS, and the cotangents of W
 * pushed to the coefficients (W is linear in B: W = M B + (terms without
 * B), M = cb ((1 - gr) v v^T / v^2 + gr I)) and to the trajectory's dense
 * output (position through B, velocity through the v x E term; the
 * v-dependence of gr, cb and of the parallel part, and the Thomas term, are
 * below 1e-15 relative for UCN and left out) */
static __device__ void rhs_adj(RLane &L, const DField &F, int nc, double t, const double *Ss, const double *W, const double *lk,
                               double *lSs, double *lG, SegAdj &a) {
    lSs[0] = lk[1] * W[2] - lk[2] * W[1];
    lSs[1] = lk[2] * W[0] - lk[0] * W[2];
    lSs[2] = lk[0] * W[1] - lk[1] * W[0];
    const double Wn = sqrt(W[0] * W[0] + W[1] * W[1] + W[2] * W[2]);
    const double q = Wn > 0 ? lk[4] / Wn : 0.0;
    const double lW[3] = {Ss[1] * lk[2] - Ss[2] * lk[1] + q * W[0], Ss[2] * lk[0] - Ss[0] * lk[2] + q * W[1],
                          Ss[0] * lk[1] - Ss[1] * lk[0] + q * W[2]};
    double yt[9];
    L.calc_spin_state(t, yt); /* position and velocity as the forward's spin_derivs had them */
    const double *v = yt + 3;
    const double v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    const double gr = 1. / sqrt(1. - v2 * PT_INV_C0_SQ);
    const double cb = -L.R.sp.gamma / gr;
    const double vl = v2 > 0 ? (v[0] * lW[0] + v[1] * lW[1] + v[2] * lW[2]) / v2 : 0.0;
    double lB[3];
    for (int k = 0; k < 3; ++k) lB[k] = cb * ((1 - gr) * vl * v[k] + gr * lW[k]);
    double B[3], dB[3][3];
    bfield64<true>(L.S, yt[0], yt[1], yt[2], B, dB); /* the forward's B polynomials */
    double V, E[3];
    efield(L.S, L.R.prec, yt[0], yt[1], yt[2], V, E);
    const double ce = cb * gr * PT_INV_C0_SQ;
    double lam[6];
    for (int j = 0; j < 3; ++j) lam[j] = dB[0][j] * lB[0] + dB[1][j] * lB[1] + dB[2][j] * lB[2];
    lam[3] = ce * (lW[1] * E[2] - lW[2] * E[1]);
    lam[4] = ce * (lW[2] * E[0] - lW[0] * E[2]);
    lam[5] = ce * (lW[0] * E[1] - lW[1] * E[0]);
    double bk[PT_ADJ_MAX_COEF][3];
    adj_basis_all(F, nc, yt[0], yt[1], yt[2], bk);
    for (int k = 0; k < nc; ++k) lG[k] += lB[0] * bk[k][0] + lB[1] * bk[k][1] + lB[2] * bk[k][2];
    dense_adj(L, t, lam, a);
}

/* Adjoint of one accepted Bloch step from the chunk tape: the stage spins
 * are recomputed from the step's start spin and the recorded precession
 * axes with the forward's arithmetic.  lS: cotangent of the state after the
 * step (in) and before it (out); lK1n: cotangent of this step's FSAL
 * derivative from the next step of the segment (in), replaced by that of
 * this step's first stage (out); last: the segment's final step, whose result
 * is the dense output at x2 when the step overshot it; first: the segment's
 * first step, whose first stage the stepper start evaluated. */
static __device__ void spin_step_adj(RLane &L, const DField &F, int nc, const double *rec, bool last, bool first, double x2, double *lS,
                                     double *lK1n, double *lG, SegAdj &a) {
    const double a2 = 1.0 / 5, a3 = 3.0 / 10, a4 = 4.0 / 5, a5 = 8.0 / 9;
    const double b21 = 1.0 / 5;
    const double b31 = 3.0 / 40, b32 = 9.0 / 40;
    const double b41 = 44.0 / 45, b42 = -56.0 / 15, b43 = 32.0 / 9;
    const double b51 = 19372.0 / 6561, b52 = -25360.0 / 2187, b53 = 64448.0 / 6561, b54 = -212.0 / 729;
    const double b61 = 9017.0 / 3168, b62 = -355.0 / 33, b63 = 46732.0 / 5247, b64 = 49.0 / 176, b65 = -5103.0 / 18656;
    const double c1 = 35.0 / 384, c3 = 500.0 / 1113, c4 = 125.0 / 192, c5 = -2187.0 / 6784, c6 = 11.0 / 84;
    const double tso = rec[0], h = rec[1];
    const double *W[7];
    for (int s = 0; s < 7; ++s) W[s] = rec + 5 + 3 * s;
    double St[7][3], kk[7][5];
    for (int i = 0; i < 3; ++i) St[0][i] = rec[2 + i];
    for (int s = 0; s < 7; ++s) {
        if (s == 1) for (int i = 0; i < 3; ++i) St[1][i] = fma(h * b21, kk[0][i], St[0][i]);
        if (s == 2) for (int i = 0; i < 3; ++i) St[2][i] = fma(h * b32, kk[1][i], fma(h * b31, kk[0][i], St[0][i]));
        if (s == 3) for (int i = 0; i < 3; ++i) St[3][i] = fma(h * b43, kk[2][i], fma(h * b42, kk[1][i], fma(h * b41, kk[0][i], St[0][i])));
        if (s == 4)
            for (int i = 0; i < 3; ++i)
                St[4][i] = fma(h * b54, kk[3][i], fma(h * b53, kk[2][i], fma(h * b52, kk[1][i], fma(h * b51, kk[0][i], St[0][i]))));
        if (s == 5)
            for (int i = 0; i < 3; ++i)
                St[5][i] = fma(h * b65, kk[4][i], fma(h * b64, kk[3][i], fma(h * b63, kk[2][i], fma(h * b62, kk[1][i], fma(h * b61, kk[0][i], St[0][i])))));
        if (s == 6)
            for (int i = 0; i < 3; ++i)
                St[6][i] = fma(h * c6, kk[5][i], fma(h * c5, kk[4][i], fma(h * c4, kk[3][i], fma(h * c3, kk[2][i], fma(h * c1, kk[0][i], St[0][i])))));
        kk[s][0] = W[s][1] * St[s][2] - W[s][2] * St[s][1];
        kk[s][1] = W[s][2] * St[s][0] - W[s][0] * St[s][2];
        kk[s][2] = W[s][0] * St[s][1] - W[s][1] * St[s][0];
        kk[s][3] = 1.;
        kk[s][4] = sqrt(W[s][0] * W[s][0] + W[s][1] * W[s][1] + W[s][2] * W[s][2]);
    }
    const double ts_ = tso + h; /* the forward's ts after the step */
    const double tst[7] = {tso, tso + h * a2, tso + h * a3, tso + h * a4, tso + h * a5, ts_, ts_};
    double lk[7][5] = {};
    double lout[5] = {0, 0, 0, 0, 0};
    double lSn[5] = {0, 0, 0, 0, 0};
    if (last && ts_ > x2) {
        /* the spin at x2 is the continuous extension of this step */
        const double Wd[6][5] = {
            {1.0, -2.8605386690370884, 3.099577878709121, -1.1618105836403092, 0.013917207301610328},
            {0.0, 4.047141499642786, -6.345354046938926, 2.795465086414005, -0.04801624082496286},
            {0.0, -3.941160071112659, 10.904003027940295, -6.729317509209278, 0.4175162190483098},
            {0.0, 2.8419447015870345, -7.547675862959386, 4.957636724931253, -0.5742817428041846},
            {0.0, -1.6109886359167997, 4.218915839039518, -2.950103865566732, 0.47312904339639456},
            {0.0, 1.523601174836727, -4.329466835790622, 3.0881301470710616, -0.2822644861171672}};
        const double hh = ts_ - tso, th = (x2 - tso) / hh;
        double hb[6];
        for (int k = 0; k < 6; ++k) {
            double p = Wd[k][4];
            p = fma(p, th, Wd[k][3]);
            p = fma(p, th, Wd[k][2]);
            p = fma(p, th, Wd[k][1]);
            p = fma(p, th, Wd[k][0]);
            hb[k] = hh * (p * th);
        }
        const int kidx[6] = {0, 2, 3, 4, 5, 6};
        for (int c = 0; c < 5; ++c) {
            lSn[c] += lS[c];
            for (int k = 0; k < 6; ++k) lk[kidx[k]][c] += hb[k] * lS[c];
        }
    } else {
        for (int c = 0; c < 5; ++c) lout[c] = lS[c];
        if (!last)
            for (int c = 0; c < 5; ++c) lk[6][c] += lK1n[c];
    }
    double ls[3];
    /* stage 7 (FSAL point): k7 = f(out) */
    rhs_adj(L, F, nc, tst[6], St[6], W[6], lk[6], ls, lG, a);
    for (int c = 0; c < 3; ++c) lout[c] += ls[c];
    for (int c = 0; c < 5; ++c) {
        lSn[c] += lout[c];
        lk[0][c] += h * c1 * lout[c];
        lk[2][c] += h * c3 * lout[c];
        lk[3][c] += h * c4 * lout[c];
        lk[4][c] += h * c5 * lout[c];
        lk[5][c] += h * c6 * lout[c];
    }
    const double bt[5][5] = {{b21, 0, 0, 0, 0}, {b31, b32, 0, 0, 0}, {b41, b42, b43, 0, 0}, {b51, b52, b53, b54, 0}, {b61, b62, b63, b64, b65}};
    for (int s = 5; s >= 1; --s) { /* stages 6 .. 2 */
        rhs_adj(L, F, nc, tst[s], St[s], W[s], lk[s], ls, lG, a);
        for (int c = 0; c < 3; ++c) {
            lSn[c] += ls[c];
            for (int i = 0; i < s; ++i) lk[i][c] += h * bt[s - 1][i] * ls[c];
        }
    }
    if (first) { /* the segment's first step: k1 = f(S) evaluated at the stepper start */
        rhs_adj(L, F, nc, tst[0], St[0], W[0], lk[0], ls, lG, a);
        for (int c = 0; c < 3; ++c) lSn[c] += ls[c];
        for (int c = 0; c < 5; ++c) lK1n[c] = 0;
    } else {
        for (int c = 0; c < 5; ++c) lK1n[c] = lk[0][c];
    }
    for (int c = 0; c < 5; ++c) lS[c] = lSn[c];
}

/* Adjoint of the segment's accepted trajectory try (Lane::rk_try_with with
 * the FSAL derivative K7 = f(yn)): lyn_in is the cotangent of yn, a holds the
 * dense-output cotangents; returns the cotangent of the segment's start
 * state in lY. */
static __device__ void traj_step_adj(const DScene &S, const DRun &R, const DField &F, int nc, const double *r, const double *lyn_in,
                                     SegAdj &a, double *lY, double *lG) {
    const double b21 = 1.0 / 5;
    const double b31 = 3.0 / 40, b32 = 9.0 / 40;
    const double b41 = 44.0 / 45, b42 = -56.0 / 15, b43 = 32.0 / 9;
    const double b51 = 19372.0 / 6561, b52 = -25360.0 / 2187, b53 = 64448.0 / 6561, b54 = -212.0 / 729;
    const double b61 = 9017.0 / 3168, b62 = -355.0 / 33, b63 = 46732.0 / 5247, b64 = 49.0 / 176, b65 = -5103.0 / 18656;
    const double c1 = 35.0 / 384, c3 = 500.0 / 1113, c4 = 125.0 / 192, c5 = -2187.0 / 6784, c6 = 11.0 / 84;
    const double bt[5][5] = {{b21, 0, 0, 0, 0}, {b31, b32, 0, 0, 0}, {b41, b42, b43, 0, 0}, {b51, b52, b53, b54, 0}, {b61, b62, b63, b64, b65}};
    const double h = r[SEG_TN] - r[SEG_TO];
    const double pol = r[SEG_XO + 7];
    const int kofs[7] = {SEG_DXO, SEG_K2, SEG_K3, SEG_K4, SEG_K5, SEG_K6, SEG_DYN};
    double lyn[6], tmp[6];
    /* K7 = f(yn) */
    eom_adj(S, R, F, nc, pol, r + SEG_YN, a.lK[6], tmp, lG);
    for (int c = 0; c < 6; ++c) lyn[c] = lyn_in[c] + tmp[c];
    double lYn[6];
    for (int c = 0; c < 6; ++c) {
        lYn[c] = lyn[c] + a.lxo[c];
        a.lK[0][c] += h * c1 * lyn[c];
        a.lK[2][c] += h * c3 * lyn[c];
        a.lK[3][c] += h * c4 * lyn[c];
        a.lK[4][c] += h * c5 * lyn[c];
        a.lK[5][c] += h * c6 * lyn[c];
    }
    for (int s = 5; s >= 1; --s) { /* stage s + 1: xt = Y + h sum_{i < s} b K_i, K_{s+1} = f(xt) */
        double xt[6];
        for (int c = 0; c < 6; ++c) {
            double v = r[SEG_XO + c];
            for (int i = 0; i < s; ++i) v = fma(h * bt[s - 1][i], r[kofs[i] + c], v);
            xt[c] = v;
        }
        eom_adj(S, R, F, nc, pol, xt, a.lK[s], tmp, lG);
        for (int c = 0; c < 6; ++c) {
            lYn[c] += tmp[c];
            for (int i = 0; i < s; ++i) a.lK[i][c] += h * bt[s - 1][i] * tmp[c];
        }
    }
    eom_adj(S, R, F, nc, pol, r + SEG_XO, a.lK[0], tmp, lG); /* K1 = f(Y) */
    for (int c = 0; c < 6; ++c) lY[c] = lYn[c] + tmp[c];
}

/* The reverse sweep of one particle per lane over its Bloch steps in chunks
 * of K: chunk c starts at the particle's Bloch step c K (its checkpoint) and
 * holds K steps (the last one the rest), across segment boundaries.  For
 * every chunk, from the last, the warp recomputes the chunk one Bloch step
 * per lane and iteration (recording the stage precession axes), then sweeps
 * it backwards one step per lane and iteration; both phases end together for
 * the whole warp, so the lanes stay converged whatever their segments look
 * like.  Between Bloch steps of different segments the sweep finishes the
 * later segment (the adjoint of its trajectory step) and opens the earlier
 * one (the adjoint of how it ended: next step, reflection or stop). */
struct RevState {
    int j;              /* segment being swept */
    double lS[5], lK1n[5], lY[6], lyn[6];
    SegAdj a;
};

static __device__ void load_seg_dense(RLane &L, const double *r) {
    L.to = r[SEG_TO];
    L.tn = r[SEG_TN];
    for (int c = 0; c < 9; ++c) {
        L.xo[c] = r[SEG_XO + c]; L.dxo[c] = r[SEG_DXO + c];
        L.k3[c] = r[SEG_K3 + c]; L.k4[c] = r[SEG_K4 + c]; L.k5[c] = r[SEG_K5 + c]; L.k6[c] = r[SEG_K6 + c];
        L.yn[c] = r[SEG_YN + c]; L.dyn[c] = r[SEG_DYN + c];
    }
}

/* open segment j for the sweep: its dense data in L, zero cotangents, and
 * the adjoint of how it ended applied to the cotangent lY of what followed */
static __device__ int seg_enter(RLane &L, const double *segb, int j, RevState &v) {
    const double *r = segb + (size_t)j * SEG_DOUBLES;
    load_seg_dense(L, r);
    v.j = j;
    for (int c = 0; c < 6; ++c) {
        v.a.lxo[c] = 0;
        v.lyn[c] = 0;
        for (int k = 0; k < 7; ++k) v.a.lK[k][c] = 0;
    }
    for (int c = 0; c < 5; ++c) v.lK1n[c] = 0;
    const int flags = (int)r[SEG_FLAGS];
    if (flags & SEGF_OTHER) return ADJ_UNSUPPORTED;
    const double xend = r[SEG_XEND];
    if (flags & SEGF_REFLECT) {
        /* TNeutron::Reflect: position at xa, velocity at xb minus 2 (v(xa).n) n */
        const double *nn = r + SEG_N;
        const double ln = nn[0] * v.lY[3] + nn[1] * v.lY[4] + nn[2] * v.lY[5];
        const double la[6] = {v.lY[0], v.lY[1], v.lY[2], -2 * ln * nn[0], -2 * ln * nn[1], -2 * ln * nn[2]};
        const double lb[6] = {0, 0, 0, v.lY[3], v.lY[4], v.lY[5]};
        dense_adj(L, r[SEG_XA], la, v.a);
        dense_adj(L, r[SEG_XB], lb, v.a);
        return 0;
    }
    bool normal = !(flags & SEGF_RESET) && xend == L.tn;
    for (int c = 0; c < 9; ++c) normal = normal && r[SEG_YL + c] == L.yn[c];
    if (normal) { /* the next segment starts from yn */
        for (int c = 0; c < 6; ++c) v.lyn[c] = v.lY[c];
        return 0;
    }
    double yd[9]; /* stopped at a point of the dense output */
    L.calc_state(xend, yd);
    bool same = true;
    for (int c = 0; c < 9; ++c) same = same && yd[c] == r[SEG_YL + c];
    if (!same) return ADJ_UNSUPPORTED;
    dense_adj(L, xend, v.lY, v.a);
    return 0;
}

__global__ void __launch_bounds__(128) k_adj_reverse(const __grid_constant__ DScene S, const __grid_constant__ DRun R,
                                                     const __grid_constant__ DBatch b, DCounters *C, const __grid_constant__ DAdj A) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool have = i < b.n;
    const int64_t n = b.n;
    const DField &F = S.fields[A.field];
    const int nc = A.ncoef;
    const int K = A.K;
    RLane L(S, R);
    RevState v;
    double lG[PT_ADJ_MAX_COEF];
    for (int k = 0; k < PT_ADJ_MAX_COEF; ++k) lG[k] = 0;
    int status = have ? A.status[i] : 0;
    const double *segb = A.seg + (size_t)(have ? i : 0) * A.cap_seg * SEG_DOUBLES;
    const double *ckb = A.ck + (size_t)(have ? i : 0) * A.cap_ck * CK_DOUBLES;
    const int nseg = (have && !status) ? A.nseg[i] : 0;
    int ch = -1;          /* current chunk */
    long total = 0;       /* Bloch steps of the particle */
    if (nseg > 0) {
        for (int c = 0; c < 5; ++c) v.lS[c] = A.dl_dspin ? A.dl_dspin[c * n + i] : 0.0;
        for (int c = 0; c < 6; ++c) v.lY[c] = A.dl_dy ? A.dl_dy[c * n + i] : 0.0;
        const double *rl = segb + (size_t)(nseg - 1) * SEG_DOUBLES;
        total = (long)rl[SEG_FIRST] + (long)rl[SEG_NSPIN];
        ch = (int)((total + K - 1) / K) - 1;
        if (A.nck[i] != ch + 1) status |= ADJ_MISMATCH;
        status |= seg_enter(L, segb, nseg - 1, v);
    }
    L.tp.tape = A.tape + (size_t)(have ? i : 0) * K * STEP_DOUBLES;
    L.tp.cap = K;
    for (;;) { /* one chunk per pass */
        const bool act = !status && ch >= 0;
        if (!__any_sync(0xffffffffu, act)) break;
        const long c0 = (long)ch * K;
        const long len = act ? min((long)K, total - c0) : 0;
        /* recompute phase */
        BlochState bs;
        int jr = 0;
        double x2 = 0;
        long left = len;
        if (act) {
            const double *q = ckb + (size_t)ch * CK_DOUBLES;
            jr = (int)q[CK_SEG];
            const double *r = segb + (size_t)jr * SEG_DOUBLES;
            load_seg_dense(L, r);
            x2 = r[SEG_XEND];
            bs.ts = q[CK_TS];
            bs.dt = q[CK_DT];
            for (int c = 0; c < 5; ++c) { bs.x[c] = q[CK_X + c]; bs.dxdt[c] = q[CK_DXDT + c]; }
            bs.steps = (long)q[CK_STEPS];
            bs.tries = 0;
            double tmp[5];
            L.spin_derivs(bs.x, tmp, bs.ts, bs.w);
            L.tp.n = 0;
            L.tp.seg_idx = jr;
        }
        for (;;) {
            __syncwarp();
            const bool busy = act && left > 0 && !status;
            if (!__any_sync(0xffffffffu, busy)) break;
            if (!busy) continue;
            const int rr = L.bloch_try(bs, x2);
            if (rr == 2) continue; /* rejected: the step is retried in the next pass */
            --left;
            if (rr < 0 || L.tp.overflow) { status |= ADJ_MISMATCH; continue; }
            if (rr == 1 && left > 0) { /* this segment's Bloch integration ended: the next one with Bloch steps */
                int jn = jr + 1;
                while (jn < nseg && !(((int)segb[(size_t)jn * SEG_DOUBLES + SEG_FLAGS] & SEGF_BLOCH) &&
                                      segb[(size_t)jn * SEG_DOUBLES + SEG_NSPIN] > 0))
                    ++jn;
                if (jn >= nseg) { status |= ADJ_MISMATCH; continue; }
                jr = jn;
                const double *r = segb + (size_t)jr * SEG_DOUBLES;
                load_seg_dense(L, r);
                x2 = r[SEG_XEND];
                for (int c = 0; c < 5; ++c) L.spin[c] = r[SEG_SPIN + c];
                L.bloch_begin(bs, L.to, x2, r[SEG_DT0]);
                L.tp.seg_idx = jr;
            }
        }
        if (act && !status && L.tp.n != len) status |= ADJ_MISMATCH;
        /* sweep phase */
        if (act && !status) load_seg_dense(L, segb + (size_t)v.j * SEG_DOUBLES);
        long t = len - 1;
        for (;;) {
            __syncwarp();
            const bool busy = act && t >= 0 && !status;
            if (!__any_sync(0xffffffffu, busy)) break;
            if (!busy) continue;
            const double *rec = L.tp.tape + (size_t)t * STEP_DOUBLES;
            const int js = (int)rec[STEP_SEG];
            while (v.j > js && !status) { /* finish the later segment, open the earlier one */
                traj_step_adj(S, R, F, nc, segb + (size_t)v.j * SEG_DOUBLES, v.lyn, v.a, v.lY, lG);
                status |= seg_enter(L, segb, v.j - 1, v);
            }
            if (status) continue;
            const double *r = segb + (size_t)js * SEG_DOUBLES;
            const long gi = c0 + t, first = (long)r[SEG_FIRST], last = first + (long)r[SEG_NSPIN] - 1;
            spin_step_adj(L, F, nc, rec, gi == last, gi == first, r[SEG_XEND], v.lS, v.lK1n, lG, v.a);
            --t;
        }
        --ch;
    }
    /* the segments before the first Bloch step and the trajectory steps of the rest */
    if (nseg > 0 && !status) {
        for (;;) {
            traj_step_adj(S, R, F, nc, segb + (size_t)v.j * SEG_DOUBLES, v.lyn, v.a, v.lY, lG);
            if (v.j == 0) break;
            status |= seg_enter(L, segb, v.j - 1, v);
            if (status) break;
        }
    }
    if (have) {
        for (int k = 0; k < nc; ++k) A.dl_dg[(size_t)k * n + i] = lG[k];
        A.status[i] = status;
        flush_counters(C, L.lc, 0.0, false);
    }
}

} // namespace ptk
