/*
 * pt_lane.cuh -- one particle's integration loop on one lane.
 *
 * Lane holds the particle state of one TTracker::IntegrateParticle call
 * (src/tracking.cpp:17-173) between kernel launches plus the dense-output
 * data of its last accepted Dormand-Prince step.  step() performs exactly one
 * iteration of the reference's LOOP A.
 */
#pragma once
#include "pt_track.cuh"
#include "pt_mr.cuh"
#include "../../include/pt_detmath.h"

namespace ptd {

struct LaneCounters {
    unsigned rk_acc, rk_rej, rhs, fields, hits, bisect, subseg, dense;
    unsigned nodes, tris, bisect_max;
    unsigned cand_calls, cand_overflow, cand_sum, tri32, dead, spin;
};

/* Resumable state of one post-step (the remainder of LOOP A after an accepted
 * try) while a bisection runs: the chord-piece loop (x1, x, x2 and states),
 * the CheckHit loop position (cx1, cya, cs, pass) and the bisection request
 * and result. */
struct PostState {
    double x1, x, x2, cx1;
    double y1[9], yl[9], y2[9], cya[9];
    double bxa, bxb;
    int stage, cs, nsub, pass, bres;
    bool reset, bao, bbo;
};
enum { PS_BEGIN = 0, PS_OUTER = 1, PS_CHECK = 2, PS_AFTER_BISECT = 3, PS_CHECK_DONE = 4 };

/* State of one bisection between its steps: the current interval [A, B] with
 * its end positions and origin flags, the midpoint, the stack of interval
 * ends per level, the choice and tried bits per level, the query count and
 * the phase of the current level (ENTER: first half next, SECOND: second
 * half next, RESUME: back at a stacked level after a dead end). */
struct BisectState {
    enum { ENTER, SECOND, RESUME };
    double stA[PT_MAX_BISECT_LEVELS + 1], stB[PT_MAX_BISECT_LEVELS + 1];
    uint64_t ch0, ch1, tr0, tr1;
    double A, B, pA[3], pB[3], p2[3], xc, pc[3];
    int level, work, phase;
    bool Ao, Bo;
};
enum { BISECT_RUNNING = 2 };

/* Entries of a packed current-solids list (one byte each: solid index in
 * bits 0-5, ignored flag in bit 7). */
static __device__ __forceinline__ int stk_idx(uint64_t s, int k) { return (int)((s >> (8 * k)) & 63); }
static __device__ __forceinline__ bool stk_ign(uint64_t s, int k) { return (s >> (8 * k + 7)) & 1; }
static __device__ __forceinline__ uint64_t stk_put(uint64_t s, int k, int idx, bool ign) {
    const int sh = 8 * k;
    return (s & ~(0xFFull << sh)) | ((uint64_t)(idx | (ign ? 128 : 0)) << sh);
}
/* remove entry k of the n entries: entries k+1 .. n-1 move down one place,
 * entry n-1 keeps its old value (as the element-wise shift leaves it) */
static __device__ __forceinline__ uint64_t stk_erase(uint64_t s, int k, int n) {
    for (int i = k; i + 1 < n; ++i) s = stk_put(s, i, stk_idx(s, i + 1), stk_ign(s, i + 1));
    return s;
}

/* TParticle::EquationOfMotion (src/particle.cpp:105-135) with given fields */
static __device__ __forceinline__ void eom(const DSpecies &sp, const double *yy, const double B[3], const double (*dB)[3],
                                           const double E[3], double *d) {
    d[0] = yy[3]; d[1] = yy[4]; d[2] = yy[5];
    double F0 = 0, F1 = 0, F2 = sp.fgrav;
    if (sp.q != 0) {
        F0 += sp.q * (E[0] + yy[4] * B[2] - yy[5] * B[1]);
        F1 += sp.q * (E[1] + yy[5] * B[0] - yy[3] * B[2]);
        F2 += sp.q * (E[2] + yy[3] * B[1] - yy[4] * B[0]);
    }
    if (sp.mu != 0 && yy[7] != 0 && (B[0] != 0 || B[1] != 0 || B[2] != 0)) {
        double inv = 1.0 / sqrt(B[0] * B[0] + B[1] * B[1] + B[2] * B[2]);
        double g0 = (B[0] * dB[0][0] + B[1] * dB[1][0] + B[2] * dB[2][0]) * inv;
        double g1 = (B[0] * dB[0][1] + B[1] * dB[1][1] + B[2] * dB[2][1]) * inv;
        double g2 = (B[0] * dB[0][2] + B[1] * dB[1][2] + B[2] * dB[2][2]) * inv;
        F0 += yy[7] * sp.mu * g0;
        F1 += yy[7] * sp.mu * g1;
        F2 += yy[7] * sp.mu * g2;
    }
    double v2 = yy[3] * yy[3] + yy[4] * yy[4] + yy[5] * yy[5];
    double ig = sqrt(1 - v2 * PT_INV_C0_SQ);
    double vF = (yy[3] * F0 + yy[4] * F1 + yy[5] * F2) * PT_INV_C0_SQ;
    double s = ig * sp.inv_mkg;
    d[3] = s * (F0 - yy[3] * vF);
    d[4] = s * (F1 - yy[4] * vF);
    d[5] = s * (F2 - yy[5] * vF);
    d[6] = ig;
    d[7] = 0;
    d[8] = sqrt(v2);
}

/* TParticle::derivs (src/particle.cpp:105-135) for every species and field
 * mode but the FP32 neutral one: B (with its Jacobian when the
 * magnetic-moment force needs it), E, then the equation of motion.  Returns
 * whether B was evaluated (its value in B). */
static __device__ __forceinline__ bool rhs_general(const DScene &S, const DRun &R, const double *yy, double *d, double B[3]) {
    const DSpecies &sp = R.sp;
    double dB[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, E[3] = {0, 0, 0}, V = 0;
    B[0] = B[1] = B[2] = 0;
    bool have = false;
    if (sp.q != 0 || (sp.mu != 0 && yy[7] != 0)) {
        /* the Jacobian only feeds the magnetic-moment force */
        if (sp.mu != 0 && yy[7] != 0) bfield<true>(S, R.prec, yy[0], yy[1], yy[2], B, dB);
        else bfield<false>(S, R.prec, yy[0], yy[1], yy[2], B, nullptr);
        have = true;
    }
    if (sp.q != 0) efield(S, R.prec, yy[0], yy[1], yy[2], V, E);
    eom(sp, yy, B, dB, E, d);
    return have;
}

/* State of a Bloch (LOOP D) integration between its steps: time, step
 * size, spin state, its FSAL derivative and the precession axis at it, and
 * the accepted steps so far. */
#define PT_OM_POINTS 10 /* intervals of the precession-axis spline (src/tracking.cpp:409) */

struct BlochState {
    double ts, dt, x[5], dxdt[5], w[3];
    long steps;
    int tries; /* tries of the current step so far (0: at a step's top) */
};

/* Recording hooks of a lane.  The production kernels use NoTape, whose
 * hooks are empty and compile away; the adjoint's taped forward and its
 * chunk recomputation (pt_k_adjoint.cu) record the trajectory segments and
 * the accepted Bloch steps through them, so both run exactly the
 * arithmetic of the production lane. */
struct NoTape {
    static constexpr bool kSpinStages = false; /* whether bloch collects the precession axis of every stage */
    template <class L> __device__ __forceinline__ void on_accept(L &, const double *) {}
    template <class L> __device__ __forceinline__ void on_segment(L &, double, const double *, bool) {}
    template <class L> __device__ __forceinline__ void on_bloch_start(L &, double, double, double) {}
    template <class L> __device__ __forceinline__ bool on_spin_step(L &, double, double, const double *, const double (*)[3]) { return true; }
    template <class L> __device__ __forceinline__ bool on_step_top(L &, const BlochState &) { return true; }
    template <class L> __device__ __forceinline__ void on_reflect(L &, double, double, const double *) {}
    template <class L> __device__ __forceinline__ void on_other(L &) {} /* a diffuse reflection or a transmission */
};

template <class Tape> struct LaneT {
    const DScene &S;
    const DRun &R;
    Tape tp;
    /* persistent state */
    int64_t id;
    double t, y[9], dydt[9], dt;
    uint32_t flags;
    double spin[5];
    double tau, hmax, noflip;
    int stop, nhit, nstep, nspinflip, nsol;
    /* current-solids list packed one byte per entry (solid index | ignored
     * << 7), entry k in bits 8k .. 8k+7: bit operations keep it in a register
     * where indexed arrays would put the whole lane in local memory */
    uint64_t stk;
    uint64_t rn;
    int64_t nacc, nrej;
    int ntry;           /* consecutive rejected tries of the current step */
    /* dense output of the last accepted try: [to, tn], start state xo/dxo,
     * stages k3..k6, end state yn with derivative dyn (FSAL) */
    double to, tn, xo[9], dxo[9], k3[9], k4[9], k5[9], k6[9], yn[9], dyn[9];
    /* two-slot cache of B-only field values keyed by (x, y, z, t) */
    double bc_p[2][4], bc_B[2][3];
    bool bc_ok[2];
    int bc_next;
    /* triangles that can touch the dense-output curve of the current chord piece
     * (ncand < 0: not available, use the full BVH query) */
    int cand[PT_MAX_CAND];
    int ncand;
    /* the candidates serve chords whose end times lie in [cand_ta, cand_tb];
     * cand_span is the length of the last interval a set was built for */
    double cand_ta, cand_tb, cand_span;
    PostState ps;
    LaneCounters lc;
    /* a pending Bloch integration (spin_begin / finish_begin): its stepper,
     * end time, B at the step's end point and the finish_step arguments */
    BlochState bst;
    double bx2, sBabs2, sB2[3], fx;
    double *fyl;
    bool freset;

    __device__ LaneT(const DScene &s, const DRun &r) : S(s), R(r) {
        om_on = false;
        bc_ok[0] = bc_ok[1] = false;
        bc_next = 0;
        ntry = 0;
        ncand = -1;
        cand_ta = cand_tb = 0;
        cand_span = INFINITY;
        lc = LaneCounters{};
    }

    __device__ double u01() { return uniform(R.seed, id, rn++); }

    /* ---------------- persistence ---------------- */
    __device__ void load(const DBatch &b, int64_t i) {
        const int64_t n = b.n;
        id = __ldcs(&b.id[i]);
        t = __ldcs(&b.t[i]);
        for (int c = 0; c < 9; ++c) { y[c] = __ldcs(&b.y[c * n + i]); dydt[c] = __ldcs(&b.dydt[c * n + i]); }
        dt = __ldcs(&b.dt[i]);
        flags = __ldcs(&b.flags[i]);
        for (int c = 0; c < 5; ++c) spin[c] = __ldcs(&b.spin[c * n + i]);
        tau = __ldcs(&b.tau[i]); hmax = __ldcs(&b.hmax[i]); noflip = __ldcs(&b.noflip[i]);
        stop = __ldcs(&b.stop_id[i]); nhit = __ldcs(&b.nhit[i]); nstep = __ldcs(&b.nstep[i]); nspinflip = __ldcs(&b.nspinflip[i]); nsol = __ldcs(&b.nsol[i]);
        stk = __ldcs(&b.stack[i]) & 0xBFBFBFBFBFBFBFBFull;
        rn = __ldcs(&b.rng_n[i]);
        nacc = __ldcs(&b.nacc[i]); nrej = __ldcs(&b.nrej[i]);
        ntry = __ldcs(&b.ntry[i]);
    }
    /* the committed step state only (what one RK try needs) */
    __device__ void load_try_input(const DBatch &b, int64_t i) {
        const int64_t n = b.n;
        t = __ldcs(&b.t[i]);
        for (int c = 0; c < 9; ++c) { y[c] = __ldcs(&b.y[c * n + i]); dydt[c] = __ldcs(&b.dydt[c * n + i]); }
        dt = __ldcs(&b.dt[i]);
        ntry = __ldcs(&b.ntry[i]);
        nacc = __ldcs(&b.nacc[i]); nrej = __ldcs(&b.nrej[i]);
    }
    /* the same with y and dydt into ks's state slots */
    template <class K> __device__ void load_try_input(const DBatch &b, int64_t i, const K &ks) {
        const int64_t n = b.n;
        t = __ldcs(&b.t[i]);
        for (int c = 0; c < 9; ++c) { ks.y(c) = __ldcs(&b.y[c * n + i]); ks.dy(c) = __ldcs(&b.dydt[c * n + i]); }
        dt = __ldcs(&b.dt[i]);
        ntry = __ldcs(&b.ntry[i]);
        nacc = __ldcs(&b.nacc[i]); nrej = __ldcs(&b.nrej[i]);
    }
    /* the try's outputs; stage vectors k3 .. k6 from ks(1 .. 4, c) */
    template <class K> __device__ void store_try_output(const DBatch &b, int64_t i, bool accepted, const K &ks) const {
        const int64_t n = b.n;
        __stcs(&b.dt[i], dt);
        __stcs(&b.ntry[i], ntry);
        __stcs(&b.nacc[i], nacc); __stcs(&b.nrej[i], nrej);
        if (accepted) {
            for (int c = 0; c < 9; ++c) { __stcs(&b.yn[c * n + i], yn[c]); __stcs(&b.dyn[c * n + i], dyn[c]); }
            for (int c = 0; c < 9; ++c) {
                __stcs(&b.kst[(0 * 9 + c) * n + i], ks(1, c));
                __stcs(&b.kst[(1 * 9 + c) * n + i], ks(2, c));
                __stcs(&b.kst[(2 * 9 + c) * n + i], ks(3, c));
                __stcs(&b.kst[(3 * 9 + c) * n + i], ks(4, c));
            }
            __stcs(&b.tn[i], tn);
        }
    }
    /* dense data of the accepted try (start = committed state) */
    __device__ void load_dense(const DBatch &b, int64_t i) {
        const int64_t n = b.n;
        to = t;
        for (int c = 0; c < 9; ++c) { xo[c] = y[c]; dxo[c] = dydt[c]; yn[c] = __ldcs(&b.yn[c * n + i]); dyn[c] = __ldcs(&b.dyn[c * n + i]); }
        for (int c = 0; c < 9; ++c) {
            k3[c] = __ldcs(&b.kst[(0 * 9 + c) * n + i]);
            k4[c] = __ldcs(&b.kst[(1 * 9 + c) * n + i]);
            k5[c] = __ldcs(&b.kst[(2 * 9 + c) * n + i]);
            k6[c] = __ldcs(&b.kst[(3 * 9 + c) * n + i]);
        }
        tn = __ldcs(&b.tn[i]);
    }
    /* what the fast completion reads of the accepted try: its end point and
     * end derivative (no stage vectors: it never evaluates the dense output) */
    __device__ void load_try_end(const DBatch &b, int64_t i) {
        const int64_t n = b.n;
        to = t;
        for (int c = 0; c < 9; ++c) { xo[c] = y[c]; dxo[c] = dydt[c]; yn[c] = __ldcs(&b.yn[c * n + i]); dyn[c] = __ldcs(&b.dyn[c * n + i]); }
        tn = __ldcs(&b.tn[i]);
    }
    /* global B caches: slot 0 holds B at the committed point (t, y), slot 1 B
     * at the end point of the last accepted try (tn, yn) */
    __device__ void load_bc(const DBatch &b, int64_t i) {
        const int64_t n = b.n;
        bc_ok[0] = (flags & PT_F_BC0) != 0;
        bc_ok[1] = (flags & PT_F_BC1) != 0;
        for (int k = 0; k < 2; ++k) {
            for (int c = 0; c < 4; ++c) bc_p[k][c] = __ldcs(&b.bc[(k * 7 + c) * n + i]);
            for (int c = 0; c < 3; ++c) bc_B[k][c] = __ldcs(&b.bc[(k * 7 + 4 + c) * n + i]);
        }
        bc_next = 0;
    }
    __device__ int bc_find(double x, double yy, double z, double tt) const {
        for (int k = 0; k < 2; ++k)
            if (bc_ok[k] && bc_p[k][0] == x && bc_p[k][1] == yy && bc_p[k][2] == z && bc_p[k][3] == tt) return k;
        return -1;
    }
    template <int K> __device__ void bc_write_from(const DBatch &b, int64_t i, int slot) const {
        const int64_t n = b.n;
        for (int c = 0; c < 4; ++c) __stcs(&b.bc[(slot * 7 + c) * n + i], bc_p[K][c]);
        for (int c = 0; c < 3; ++c) __stcs(&b.bc[(slot * 7 + 4 + c) * n + i], bc_B[K][c]);
    }
    __device__ void bc_write(const DBatch &b, int64_t i, int slot, int k) const {
        if (k == 0) bc_write_from<0>(b, i, slot);
        else bc_write_from<1>(b, i, slot);
    }
    /* after a commit: keep B at the new committed point (flags stored by store()) */
    __device__ void store_bc_commit(const DBatch &b, int64_t i) {
        int k = bc_find(y[0], y[1], y[2], t);
        flags &= ~(PT_F_BC0 | PT_F_BC1);
        if (k >= 0) {
            bc_write(b, i, 0, k);
            flags |= PT_F_BC0;
        }
    }
    /* hand-off of an accepted try to the full post-step (persistent form):
     * slot 0 keeps B at the committed point, slot 1 B at the try's end
     * point, whichever the lane's cache holds (flags stored by store()) */
    __device__ void store_bc_handoff(const DBatch &b, int64_t i) {
        const int k0 = bc_find(y[0], y[1], y[2], t), k1 = bc_find(yn[0], yn[1], yn[2], tn);
        flags &= ~(PT_F_BC0 | PT_F_BC1);
        if (k0 >= 0) {
            bc_write(b, i, 0, k0);
            flags |= PT_F_BC0;
        }
        if (k1 >= 0) {
            bc_write(b, i, 1, k1);
            flags |= PT_F_BC1;
        }
    }
    /* after an accepted try: keep B at its end point (flags stored separately) */
    __device__ void store_bc_try(const DBatch &b, int64_t i) {
        int k = bc_find(yn[0], yn[1], yn[2], tn);
        flags &= ~PT_F_BC1;
        if (k >= 0) {
            bc_write(b, i, 1, k);
            flags |= PT_F_BC1;
        }
    }
    /* suspended post-step (batched form) */
    __device__ void load_post(const DBatch &b, int64_t i) {
        const int64_t n = b.n;
        const double *d = b.ps_d;
        ps.x1 = d[0 * n + i]; ps.x = d[1 * n + i]; ps.x2 = d[2 * n + i]; ps.cx1 = d[3 * n + i];
        ps.bxa = d[4 * n + i]; ps.bxb = d[5 * n + i];
        for (int c = 0; c < 9; ++c) {
            ps.y1[c] = d[(6 + c) * n + i];
            ps.yl[c] = d[(15 + c) * n + i];
            ps.y2[c] = d[(24 + c) * n + i];
            ps.cya[c] = d[(33 + c) * n + i];
        }
        const int32_t *q = b.ps_i;
        ps.stage = q[0 * n + i]; ps.cs = q[1 * n + i]; ps.nsub = q[2 * n + i]; ps.pass = q[3 * n + i]; ps.bres = q[4 * n + i];
        const int fl = q[5 * n + i];
        ps.reset = fl & 1; ps.bao = (fl >> 1) & 1; ps.bbo = (fl >> 2) & 1;
        ncand = q[6 * n + i];
        for (int k = 0; k < ncand; ++k) cand[k] = q[(7 + k) * n + i]; /* entries past ncand are never read */
        cand_ta = d[42 * n + i]; cand_tb = d[43 * n + i]; cand_span = d[44 * n + i];
    }
    __device__ void store_post(const DBatch &b, int64_t i) const {
        const int64_t n = b.n;
        double *d = b.ps_d;
        d[0 * n + i] = ps.x1; d[1 * n + i] = ps.x; d[2 * n + i] = ps.x2; d[3 * n + i] = ps.cx1;
        d[4 * n + i] = ps.bxa; d[5 * n + i] = ps.bxb;
        for (int c = 0; c < 9; ++c) {
            d[(6 + c) * n + i] = ps.y1[c];
            d[(15 + c) * n + i] = ps.yl[c];
            d[(24 + c) * n + i] = ps.y2[c];
            d[(33 + c) * n + i] = ps.cya[c];
        }
        int32_t *q = b.ps_i;
        q[0 * n + i] = ps.stage; q[1 * n + i] = ps.cs; q[2 * n + i] = ps.nsub; q[3 * n + i] = ps.pass; q[4 * n + i] = ps.bres;
        q[5 * n + i] = (ps.reset ? 1 : 0) | (ps.bao ? 2 : 0) | (ps.bbo ? 4 : 0);
        q[6 * n + i] = ncand;
        for (int k = 0; k < ncand; ++k) q[(7 + k) * n + i] = cand[k];
        d[42 * n + i] = cand_ta; d[43 * n + i] = cand_tb; d[44 * n + i] = cand_span;
    }
    /* what a bisection of a suspended post-step reads: the dense data of the
     * accepted try and the interval (cx1, cya) -> (x2, y2) (positions only)
     * with its candidate triangles */
    __device__ void load_bisect_request(const DBatch &b, int64_t i) {
        const int64_t n = b.n;
        to = b.t[i];
        tn = b.tn[i];
        for (int c = 0; c < 3; ++c) { /* calc_pos reads the position components only */
            xo[c] = b.y[c * n + i];
            dxo[c] = b.dydt[c * n + i];
            k3[c] = b.kst[(0 * 9 + c) * n + i];
            k4[c] = b.kst[(1 * 9 + c) * n + i];
            k5[c] = b.kst[(2 * 9 + c) * n + i];
            k6[c] = b.kst[(3 * 9 + c) * n + i];
            dyn[c] = b.dyn[c * n + i];
        }
        const double *d = b.ps_d;
        ps.x2 = d[2 * n + i];
        ps.cx1 = d[3 * n + i];
        for (int c = 0; c < 3; ++c) {
            ps.y2[c] = d[(24 + c) * n + i];
            ps.cya[c] = d[(33 + c) * n + i];
        }
        const int32_t *q = b.ps_i;
        ncand = q[6 * n + i];
        for (int k = 0; k < ncand; ++k) cand[k] = q[(7 + k) * n + i]; /* entries past ncand are never read */
        cand_ta = d[42 * n + i]; cand_tb = d[43 * n + i]; cand_span = d[44 * n + i];
    }
    __device__ void store_bisect_result(const DBatch &b, int64_t i) const {
        const int64_t n = b.n;
        b.ps_d[4 * n + i] = ps.bxa;
        b.ps_d[5 * n + i] = ps.bxb;
        int32_t *q = b.ps_i;
        q[4 * n + i] = ps.bres;
        q[5 * n + i] = (q[5 * n + i] & 1) | (ps.bao ? 2 : 0) | (ps.bbo ? 4 : 0);
        q[0 * n + i] = PS_AFTER_BISECT;
        /* the bisection may have narrowed the candidate set */
        q[6 * n + i] = ncand;
        for (int k = 0; k < ncand; ++k) q[(7 + k) * n + i] = cand[k];
        b.ps_d[42 * n + i] = cand_ta; b.ps_d[43 * n + i] = cand_tb; b.ps_d[44 * n + i] = cand_span;
    }
    __device__ void store(const DBatch &b, int64_t i) const {
        const int64_t n = b.n;
        __stcs(&b.t[i], t);
        for (int c = 0; c < 9; ++c) { __stcs(&b.y[c * n + i], y[c]); __stcs(&b.dydt[c * n + i], dydt[c]); }
        __stcs(&b.dt[i], dt);
        __stcs(&b.flags[i], flags);
        for (int c = 0; c < 5; ++c) __stcs(&b.spin[c * n + i], spin[c]);
        __stcs(&b.tau[i], tau); __stcs(&b.hmax[i], hmax); __stcs(&b.noflip[i], noflip);
        __stcs(&b.stop_id[i], stop); __stcs(&b.nhit[i], nhit); __stcs(&b.nstep[i], nstep); __stcs(&b.nspinflip[i], nspinflip); __stcs(&b.nsol[i], nsol);
        __stcs(&b.stack[i], stk);
        __stcs(&b.rng_n[i], rn);
        __stcs(&b.nacc[i], nacc); __stcs(&b.nrej[i], nrej);
        __stcs(&b.ntry[i], ntry);
    }

    /* ---------------- fields and equation of motion ---------------- */
    /* the slot index is a template constant so that the caches stay in registers */
    template <int K> __device__ void bc_set(double x, double yy, double z, double tt, const double B[3]) {
        bc_p[K][0] = x; bc_p[K][1] = yy; bc_p[K][2] = z; bc_p[K][3] = tt;
        bc_B[K][0] = B[0]; bc_B[K][1] = B[1]; bc_B[K][2] = B[2];
        bc_ok[K] = true;
    }
    __device__ void bc_put(double x, double yy, double z, double tt, const double B[3]) {
        if (bc_next == 0) bc_set<0>(x, yy, z, tt, B);
        else bc_set<1>(x, yy, z, tt, B);
        bc_next ^= 1;
    }
    __device__ void bonly(double x, double yy, double z, double tt, double B[3]) {
        for (int k = 0; k < 2; ++k)
            if (bc_ok[k] && bc_p[k][0] == x && bc_p[k][1] == yy && bc_p[k][2] == z && bc_p[k][3] == tt) {
                B[0] = bc_B[k][0]; B[1] = bc_B[k][1]; B[2] = bc_B[k][2];
                return;
            }
        bfield<false>(S, R.prec, x, yy, z, B, nullptr);
        ++lc.fields;
        bc_put(x, yy, z, tt, B);
    }

    /* TParticle::derivs + EquationOfMotion (src/particle.cpp:96-135) */
    /* TAB_ONLY: a neutral species in the FP32 field mode whose magnetic
     * fields are all FP32 tables (the host selects it), the other paths
     * compiled out */
    template <bool TAB_ONLY = false> __device__ void derivs(const double *yy, double tt, double *d, bool keepB = false) {
        if (TAB_ONLY || (R.sp.q == 0 && R.prec == PT_PREC_FP32)) {
            derivs_neutral32<TAB_ONLY>(yy, tt, d, keepB);
            return;
        }
        double B[3];
        if (rhs_general(S, R, yy, d, B)) {
            ++lc.fields;
            /* the value part of the gradient evaluation is bit-identical to a
             * B-only evaluation, so it can serve later B-only queries */
            if (keepB) bc_put(yy[0], yy[1], yy[2], tt, B);
        }
        ++lc.rhs;
    }

    /* TParticle::EquationOfMotion (src/particle.cpp:105-135) with given fields */
    __device__ __forceinline__ void eom_fields(const double *yy, const double B[3], const double (*dB)[3], const double E[3], double *d) const {
        eom(R.sp, yy, B, dB, E, d);
    }
    /* TParticle::SpinPrecessionAxis (src/particle.cpp:148-175).  Three of
     * its six divisions are folded (B.v / v^2 once for the three components
     * of the parallel field, -gamma / gr as -gamma sqrt(1 - v^2/c^2)): on
     * GB300 an FP64 division is a sequence of a dozen FP64-pipe
     * instructions, and the axis is evaluated six times per Bloch step.
     * The result differs from the unfolded expression by rounding only. */
    __device__ void spin_axis(const double B[3], const double E[3], const double *dydt, double W[3]) const {
        const double v2 = dydt[0] * dydt[0] + dydt[1] * dydt[1] + dydt[2] * dydt[2];
        const double sq = sqrt(1. - v2 * PT_INV_C0_SQ);
        const double gr = 1. / sq;
        const double Bdotv = B[0] * dydt[0] + B[1] * dydt[1] + B[2] * dydt[2];
        const double bv = Bdotv / v2;
        double Bpar[3], vxE[3], axv[3];
        for (int j = 0; j < 3; ++j) Bpar[j] = bv * dydt[j];
        vxE[0] = dydt[1] * E[2] - dydt[2] * E[1];
        vxE[1] = dydt[2] * E[0] - dydt[0] * E[2];
        vxE[2] = dydt[0] * E[1] - dydt[1] * E[0];
        axv[0] = dydt[4] * dydt[2] - dydt[5] * dydt[1];
        axv[1] = dydt[5] * dydt[0] - dydt[3] * dydt[2];
        axv[2] = dydt[3] * dydt[1] - dydt[4] * dydt[0];
        const double cb = -R.sp.gamma * sq, ct = gr * gr / (gr + 1) * PT_INV_C0_SQ;
        for (int j = 0; j < 3; ++j) W[j] = cb * ((1 - gr) * Bpar[j] + gr * B[j] - gr * vxE[j] * PT_INV_C0_SQ) + ct * axv[j];
    }
    /* the precession axis at tt from the trajectory's dense output */
    __device__ void spin_axis_at(double tt, double W[3]) {
        double yy[9], dydt[9], B[3], dB[3][3], V, E[3];
        calc_spin_state(tt, yy);
        bfield<true>(S, R.prec, yy[0], yy[1], yy[2], B, dB);
        efield(S, R.prec, yy[0], yy[1], yy[2], V, E);
        ++lc.fields;
        eom_fields(yy, B, dB, E, dydt);
        spin_axis(B, E, dydt, W);
    }
    /* interpolatefields (src/tracking.cpp:404-421): the axis at x1 + i (x2 -
     * x1) / 10, i = 0..10, and per component ALGLIB's spline1dbuildcubic with
     * parabolically terminated ends (the slopes of spline_slopes, the
     * coefficients as spline1dbuildhermite forms them) */
    __device__ __noinline__ void omega_spline(double x1, double x2) {
        const int n = PT_OM_POINTS + 1;
        double w[3][PT_OM_POINTS + 1];
        for (int i = 0; i < n; ++i) {
            const double t = x1 + i * (x2 - x1) / PT_OM_POINTS;
            om_t[i] = t;
            double W[3];
            spin_axis_at(t, W);
            for (int c = 0; c < 3; ++c) w[c][i] = W[c];
        }
        for (int c = 0; c < 3; ++c) {
            double d[PT_OM_POINTS + 1];
            spline_slopes(n, om_t, w[c], d);
            for (int i = 0; i + 1 < n; ++i) {
                const double delta = om_t[i + 1] - om_t[i], delta2 = delta * delta, delta3 = delta * delta2;
                om_c[c][i][0] = w[c][i];
                om_c[c][i][1] = d[i];
                om_c[c][i][2] = (3 * (w[c][i + 1] - w[c][i]) - 2 * d[i] * delta - d[i + 1] * delta) / delta2;
                om_c[c][i][3] = (2 * (w[c][i] - w[c][i + 1]) + d[i] * delta + d[i + 1] * delta) / delta3;
            }
        }
        om_on = true;
    }
    /* ALGLIB spline1dgriddiffcubic's slopes with parabolically terminated
     * ends (tridiagonal system, Thomas algorithm in the library's order) */
    __device__ static void spline_slopes(int n, const double *x, const double *y, double *d) {
        if (n == 2) {
            d[0] = (y[1] - y[0]) / (x[1] - x[0]);
            d[1] = d[0];
            return;
        }
        double a1[PT_OM_POINTS + 1], a2[PT_OM_POINTS + 1], a3[PT_OM_POINTS + 1], b[PT_OM_POINTS + 1];
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
        for (int k = 1; k <= n - 1; ++k) {
            const double t = a1[k] / a2[k - 1];
            a2[k] = a2[k] - t * a3[k - 1];
            b[k] = b[k] - t * b[k - 1];
        }
        d[n - 1] = b[n - 1] / a2[n - 1];
        for (int k = n - 2; k >= 0; --k) d[k] = (b[k] - a3[k] * d[k + 1]) / a2[k];
    }
    /* spline1dcalc of the three axis splines: the interval by the library's
     * bisection (the last one whose start is below tt, the first at or
     * below om_t[0]), then Horner in u = tt - its start */
    __device__ void omega_eval(double tt, double W[3]) const {
        int l = 0, r = PT_OM_POINTS + 1 - 1;
        while (l != r - 1) {
            const int m = (l + r) / 2;
            if (om_t[m] >= tt) r = m;
            else l = m;
        }
        const double u = tt - om_t[l];
        for (int c = 0; c < 3; ++c) {
            const double *k = om_c[c][l];
            W[c] = k[0] + u * (k[1] + u * (k[2] + u * k[3]));
        }
    }
    /* TParticle::SpinDerivs (src/particle.cpp:178-193) along the trajectory's
     * dense output, or from the axis splines (interpolatefields) */
    __device__ __noinline__ void spin_derivs(const double *Sv, double *dS, double tt, double *Wout = nullptr) {
        double W[3];
        if (om_on) omega_eval(tt, W);
        else spin_axis_at(tt, W);
        dS[0] = W[1] * Sv[2] - W[2] * Sv[1];
        dS[1] = W[2] * Sv[0] - W[0] * Sv[2];
        dS[2] = W[0] * Sv[1] - W[1] * Sv[0];
        dS[3] = 1.;
        dS[4] = sqrt(W[0] * W[0] + W[1] * W[1] + W[2] * W[2]);
        if (Wout) { Wout[0] = W[0]; Wout[1] = W[1]; Wout[2] = W[2]; }
    }

    /* LOOP D of TTracker::IntegrateSpin (src/tracking.cpp:423-446): a fresh
     * dopri5 dense-output stepper with abs = rel = 1e-12 from (x1, spin) to
     * x2, the same controller and arithmetic as the trajectory's; false when
     * a step fails (500 tries) or the step count bound is reached */
    __device__ __noinline__ bool bloch(double x1, double x2, double dt0) {
        BlochState bs;
        bloch_begin(bs, x1, x2, dt0);
        return bloch_run(bs, x2, -1) == 1;
    }
    /* the stepper's start: spin state, first step size and FSAL derivative */
    __device__ void bloch_begin(BlochState &bs, double x1, double x2, double dt0) {
        tp.on_bloch_start(*this, x1, x2, dt0);
        for (int i = 0; i < 5; ++i) bs.x[i] = spin[i];
        bs.ts = x1;
        bs.dt = dt0;
        bs.steps = 0;
        bs.tries = 0;
        if (R.log.spin) log_spin(x1, x1, spin);
        spin_derivs(bs.x, bs.dxdt, bs.ts, Tape::kSpinStages ? bs.w : nullptr);
    }
    /* Runs the stepper from `bs` towards x2 for at most max_steps accepted
     * steps (< 0: no limit).  Returns 1 when x2 is reached (the spin at x2 in
     * spin[]), 0 when max_steps steps are done (state in bs, spin[] = the
     * state after the last step), -1 on a failed step or the step bound. */
    __device__ __noinline__ int bloch_run(BlochState &bs, double x2, long max_steps) {
        for (long done = 0;;) {
            if (max_steps >= 0 && done >= max_steps && bs.tries == 0) {
                for (int i = 0; i < 5; ++i) spin[i] = bs.x[i];
                return 0;
            }
            const int r = bloch_try(bs, x2);
            if (r == 2) continue;
            if (r != 0) return r;
            ++done;
        }
    }
    /* One try of the stepper's current step (the unit a warp runs
     * converged: a lane whose try is rejected retries in the next call,
     * together with the other lanes' next tries).  Returns 2 when the try is
     * rejected (step size reduced), 0 when it is accepted and x2 is not yet
     * reached (spin[] = the new state), 1 when x2 is reached (the spin at x2
     * in spin[]), -1 on the step bound or the 500-try limit.  The hooks see
     * the top of every step (before its first try) and every accepted step:
     * its start time, step size, start state and (kSpinStages) the
     * precession axis at each of its seven stages (the last is the FSAL
     * point). */
    __device__ __noinline__ int bloch_try(BlochState &bs, double x2) {
        const double a2 = 1.0 / 5, a3 = 3.0 / 10, a4 = 4.0 / 5, a5 = 8.0 / 9;
        const double b21 = 1.0 / 5;
        const double b31 = 3.0 / 40, b32 = 9.0 / 40;
        const double b41 = 44.0 / 45, b42 = -56.0 / 15, b43 = 32.0 / 9;
        const double b51 = 19372.0 / 6561, b52 = -25360.0 / 2187, b53 = 64448.0 / 6561, b54 = -212.0 / 729;
        const double b61 = 9017.0 / 3168, b62 = -355.0 / 33, b63 = 46732.0 / 5247, b64 = 49.0 / 176, b65 = -5103.0 / 18656;
        const double c1 = 35.0 / 384, c3 = 500.0 / 1113, c4 = 125.0 / 192, c5 = -2187.0 / 6784, c6 = 11.0 / 84;
        const double dc1 = c1 - 5179.0 / 57600, dc3 = c3 - 7571.0 / 16695, dc4 = c4 - 393.0 / 640,
                     dc5 = c5 - (-92097.0) / 339200, dc6 = c6 - 187.0 / 2100, dc7 = -1.0 / 40;
        const double eps = 1e-12;
        double *x = bs.x, *dxdt = bs.dxdt;
        double xo5[5], dxo5[5], k2_[5], k3_[5], k4_[5], k5_[5], k6_[5], xt[5], out[5], dout[5];
        double wst[7][3]; /* precession axis per stage (kSpinStages only) */
        double &ts = bs.ts, &dt_ = bs.dt;
        const double tso = ts;
        if (bs.tries == 0) {
            if (bs.steps >= PT_MAX_SPIN_STEPS) return -1;
            if (!tp.on_step_top(*this, bs)) return -1;
        }
        if (++bs.tries > PT_MAX_TRIES) return -1;
        for (int i = 0; i < 5; ++i) xt[i] = fma(dt_ * b21, dxdt[i], x[i]);
        spin_derivs(xt, k2_, ts + dt_ * a2, Tape::kSpinStages ? wst[1] : nullptr);
        for (int i = 0; i < 5; ++i) xt[i] = fma(dt_ * b32, k2_[i], fma(dt_ * b31, dxdt[i], x[i]));
        spin_derivs(xt, k3_, ts + dt_ * a3, Tape::kSpinStages ? wst[2] : nullptr);
        for (int i = 0; i < 5; ++i) xt[i] = fma(dt_ * b43, k3_[i], fma(dt_ * b42, k2_[i], fma(dt_ * b41, dxdt[i], x[i])));
        spin_derivs(xt, k4_, ts + dt_ * a4, Tape::kSpinStages ? wst[3] : nullptr);
        for (int i = 0; i < 5; ++i)
            xt[i] = fma(dt_ * b54, k4_[i], fma(dt_ * b53, k3_[i], fma(dt_ * b52, k2_[i], fma(dt_ * b51, dxdt[i], x[i]))));
        spin_derivs(xt, k5_, ts + dt_ * a5, Tape::kSpinStages ? wst[4] : nullptr);
        for (int i = 0; i < 5; ++i)
            xt[i] = fma(dt_ * b65, k5_[i], fma(dt_ * b64, k4_[i], fma(dt_ * b63, k3_[i], fma(dt_ * b62, k2_[i], fma(dt_ * b61, dxdt[i], x[i])))));
        spin_derivs(xt, k6_, ts + dt_, Tape::kSpinStages ? wst[5] : nullptr);
        for (int i = 0; i < 5; ++i)
            out[i] = fma(dt_ * c6, k6_[i], fma(dt_ * c5, k5_[i], fma(dt_ * c4, k4_[i], fma(dt_ * c3, k3_[i], fma(dt_ * c1, dxdt[i], x[i])))));
        spin_derivs(out, dout, ts + dt_, Tape::kSpinStages ? wst[6] : nullptr);
        double adt = fabs(dt_), m = 0;
        for (int i = 0; i < 5; ++i) {
            const double er = fma(dt_ * dc7, dout[i], fma(dt_ * dc6, k6_[i], fma(dt_ * dc5, k5_[i], fma(dt_ * dc4, k4_[i],
                              fma(dt_ * dc3, k3_[i], (dt_ * dc1) * dxdt[i])))));
            const double e = fabs(er) / (eps + eps * (1.0 * fabs(x[i]) + adt * fabs(dxdt[i])));
            m = (m < e || e != e) ? e : m;
        }
        if (!(m <= 1.0)) {
            dt_ *= fmax(0.9 * (m < 1e300 ? ptdm_pow(m, -1.0 / 3.0) : 0.0), 0.2);
            return 2;
        }
        if (Tape::kSpinStages) {
            wst[0][0] = bs.w[0]; wst[0][1] = bs.w[1]; wst[0][2] = bs.w[2];
            bs.w[0] = wst[6][0]; bs.w[1] = wst[6][1]; bs.w[2] = wst[6][2];
        }
        if (!tp.on_spin_step(*this, tso, dt_, x, wst)) return -1;
        ts += dt_;
        if (m < 0.5) {
            m = fmax(0.00032, m);
            dt_ *= 0.9 * ptdm_pow(m, -1.0 / 5.0);
        }
        for (int i = 0; i < 5; ++i) { xo5[i] = x[i]; dxo5[i] = dxdt[i]; x[i] = out[i]; dxdt[i] = dout[i]; }
        bs.tries = 0;
        ++lc.spin;
        ++bs.steps;
        if (ts > x2) { /* overshoot: the continuous extension at x2 */
            const double W_[6][5] = {
                {1.0, -2.8605386690370884, 3.099577878709121, -1.1618105836403092, 0.013917207301610328},
                {0.0, 4.047141499642786, -6.345354046938926, 2.795465086414005, -0.04801624082496286},
                {0.0, -3.941160071112659, 10.904003027940295, -6.729317509209278, 0.4175162190483098},
                {0.0, 2.8419447015870345, -7.547675862959386, 4.957636724931253, -0.5742817428041846},
                {0.0, -1.6109886359167997, 4.218915839039518, -2.950103865566732, 0.47312904339639456},
                {0.0, 1.523601174836727, -4.329466835790622, 3.0881301470710616, -0.2822644861171672}};
            const double h = ts - tso, th = (x2 - tso) / h;
            double hb[6];
            for (int k = 0; k < 6; ++k) {
                double p = W_[k][4];
                p = fma(p, th, W_[k][3]);
                p = fma(p, th, W_[k][2]);
                p = fma(p, th, W_[k][1]);
                p = fma(p, th, W_[k][0]);
                hb[k] = h * (p * th);
            }
            for (int i = 0; i < 5; ++i)
                spin[i] = fma(hb[5], dxdt[i], fma(hb[4], k6_[i], fma(hb[3], k5_[i], fma(hb[2], k4_[i], fma(hb[1], k3_[i], fma(hb[0], dxo5[i], xo5[i]))))));
            if (R.log.spin) log_spin(tso, x2, spin);
            return 1;
        }
        for (int i = 0; i < 5; ++i) spin[i] = x[i];
        if (R.log.spin) log_spin(tso, ts, spin);
        return ts >= x2 ? 1 : 0;
    }

    /* The neutral-particle equation of motion in the FP32 field mode: B,
     * grad B and the magnetic gradient force pol mu grad|B| in FP32 (relative
     * error ~1e-7 of a force well below gravity), gravity, the relativistic
     * factors and the state derivative in FP64. */
    template <bool TAB_ONLY = false> __device__ void derivs_neutral32(const double *yy, double tt, double *d, bool keepB) {
        const DSpecies &sp = R.sp;
        double F0 = 0, F1 = 0, F2 = sp.fgrav;
        if (sp.mu != 0 && yy[7] != 0) {
            float B[3], dB[3][3];
            bfield32<true, TAB_ONLY>(S, yy[0], yy[1], yy[2], B, dB);
            ++lc.fields;
            if (keepB) {
                const double Bd[3] = {B[0], B[1], B[2]};
                bc_put(yy[0], yy[1], yy[2], tt, Bd);
            }
            if (B[0] != 0 || B[1] != 0 || B[2] != 0) {
                const float bb = fmaf(B[2], B[2], fmaf(B[1], B[1], B[0] * B[0]));
                const float s = (float)yy[7] * sp.muf / sqrtf(bb);
                const float g0 = fmaf(B[2], dB[2][0], fmaf(B[1], dB[1][0], B[0] * dB[0][0]));
                const float g1 = fmaf(B[2], dB[2][1], fmaf(B[1], dB[1][1], B[0] * dB[0][1]));
                const float g2 = fmaf(B[2], dB[2][2], fmaf(B[1], dB[1][2], B[0] * dB[0][2]));
                F0 += (double)(s * g0);
                F1 += (double)(s * g1);
                F2 += (double)(s * g2);
            }
        }
        ++lc.rhs;
        d[0] = yy[3]; d[1] = yy[4]; d[2] = yy[5];
        double v2 = yy[3] * yy[3] + yy[4] * yy[4] + yy[5] * yy[5];
        double ig = sqrt(1 - v2 * PT_INV_C0_SQ);
        double vF = (yy[3] * F0 + yy[4] * F1 + yy[5] * F2) * PT_INV_C0_SQ;
        double s = ig * sp.inv_mkg;
        d[3] = s * (F0 - yy[3] * vF);
        d[4] = s * (F1 - yy[4] * vF);
        d[5] = s * (F2 - yy[5] * vF);
        d[6] = ig;
        d[7] = 0;
        d[8] = sqrt(v2);
    }

    /* TParticle::GetKineticEnergy (src/particle.cpp:237-251) */
    __device__ double ekin(const double *v) const {
        double beta2 = (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) / PT_C0_SQ;
        double gm1;
        double b4 = beta2 * beta2;
        if (b4 * b4 * beta2 < 2.220446049250313e-16)
            gm1 = (0.5 + (3.0 / 8.0 + (5.0 / 16.0 + 35.0 / 128.0 * beta2) * beta2) * beta2) * beta2;
        else
            gm1 = 1.0 / sqrt(1.0 - beta2) - 1.0;
        return R.sp.mc2 * gm1;
    }
    __device__ double mat_pot(const DMat &m, double pol) const { return m.fermi_real * 1e-9 - m.ibf * R.sp.mu_over_e * pol; }
    /* TParticle::GetPotentialEnergy (src/particle.cpp:254-269) + TNeutron material term */
    __device__ double epot(double tt, const double *yy, int solid) {
        const DSpecies &sp = R.sp;
        double r = 0;
        if (sp.q != 0 || sp.mu != 0) {
            if (sp.mu != 0) {
                double B[3];
                bonly(yy[0], yy[1], yy[2], tt, B);
                r += -yy[7] * sp.mu_over_e * sqrt(B[0] * B[0] + B[1] * B[1] + B[2] * B[2]);
            }
            if (sp.q != 0) {
                double V, E[3];
                efield(S, R.prec, yy[0], yy[1], yy[2], V, E);
                r += sp.q_over_e * V;
            }
        }
        r += sp.mg * yy[2];
        if (sp.kind == PT_NEUTRON) r += mat_pot(S.mats[S.solids[solid].mat], yy[7]);
        return r;
    }

    /* ---------------- solids ---------------- */
    /* TTracker::GetCurrentsolid (src/tracking.cpp:367-370) */
    __device__ int current_solid(int n, uint64_t st) const {
        int best = 0;
        for (int i = 1; i < n; ++i) {
            bool less = stk_ign(st, best) || (!stk_ign(st, i) && S.solids[stk_idx(st, best)].id < S.solids[stk_idx(st, i)].id);
            if (less) best = i;
        }
        return stk_idx(st, best);
    }
    __device__ int cur_solid() const { return current_solid(nsol, stk); }

    /* ---------------- Dormand-Prince 5(4) with odeint's controller ---------------- */
    /* Storage of one try's vectors: ks(s, i) is component i of stage s + 2
     * (k2 .. k6), ks.y(i) / ks.dy(i) of the committed state and its
     * derivative.  KReg keeps the stages in a local array and the state in the
     * lane's members (registers). */
    struct KReg {
        double (*a)[9];
        double *ys, *dys;
        __device__ __forceinline__ double &operator()(int s, int i) const { return a[s][i]; }
        __device__ __forceinline__ double &y(int i) const { return ys[i]; }
        __device__ __forceinline__ double &dy(int i) const { return dys[i]; }
    };

    /* One try of controlled_runge_kutta::try_step on the committed state
     * (t, y, dydt).  Returns 1 when accepted (dense data set, dt grown), 0
     * when rejected (dt shrunk), -1 after 500 consecutive rejections (odeint's
     * failed_step_checker).  The stage sums are explicit fused multiply-add
     * chains in tableau order, the same chains the oracle evaluates; the
     * stage vectors live wherever `ks` puts them, which changes no operation.
     * On acceptance yn and dyn are set; the caller takes k3 .. k6 from ks. */
    template <bool TAB_ONLY = false, class K> __device__ __forceinline__ int rk_try_with(const K &ks) {
        const double a2 = 1.0 / 5, a3 = 3.0 / 10, a4 = 4.0 / 5, a5 = 8.0 / 9;
        const double b21 = 1.0 / 5;
        const double b31 = 3.0 / 40, b32 = 9.0 / 40;
        const double b41 = 44.0 / 45, b42 = -56.0 / 15, b43 = 32.0 / 9;
        const double b51 = 19372.0 / 6561, b52 = -25360.0 / 2187, b53 = 64448.0 / 6561, b54 = -212.0 / 729;
        const double b61 = 9017.0 / 3168, b62 = -355.0 / 33, b63 = 46732.0 / 5247, b64 = 49.0 / 176, b65 = -5103.0 / 18656;
        const double c1 = 35.0 / 384, c3 = 500.0 / 1113, c4 = 125.0 / 192, c5 = -2187.0 / 6784, c6 = 11.0 / 84;
        const double dc1 = c1 - 5179.0 / 57600, dc3 = c3 - 7571.0 / 16695, dc4 = c4 - 393.0 / 640,
                     dc5 = c5 - (-92097.0) / 339200, dc6 = c6 - 187.0 / 2100, dc7 = -1.0 / 40;
        if (ntry >= PT_MAX_TRIES) return -1;
        ++ntry;
        double xt[9], d[9];
        const double h = dt;
        for (int i = 0; i < 9; ++i) xt[i] = fma(h * b21, ks.dy(i), ks.y(i));
        derivs<TAB_ONLY>(xt, t + h * a2, d);
        for (int i = 0; i < 9; ++i) ks(0, i) = d[i];
        for (int i = 0; i < 9; ++i) xt[i] = fma(h * b32, ks(0, i), fma(h * b31, ks.dy(i), ks.y(i)));
        derivs<TAB_ONLY>(xt, t + h * a3, d);
        for (int i = 0; i < 9; ++i) ks(1, i) = d[i];
        for (int i = 0; i < 9; ++i) xt[i] = fma(h * b43, ks(1, i), fma(h * b42, ks(0, i), fma(h * b41, ks.dy(i), ks.y(i))));
        derivs<TAB_ONLY>(xt, t + h * a4, d);
        for (int i = 0; i < 9; ++i) ks(2, i) = d[i];
        for (int i = 0; i < 9; ++i)
            xt[i] = fma(h * b54, ks(2, i), fma(h * b53, ks(1, i), fma(h * b52, ks(0, i), fma(h * b51, ks.dy(i), ks.y(i)))));
        derivs<TAB_ONLY>(xt, t + h * a5, d);
        for (int i = 0; i < 9; ++i) ks(3, i) = d[i];
        for (int i = 0; i < 9; ++i)
            xt[i] = fma(h * b65, ks(3, i), fma(h * b64, ks(2, i), fma(h * b63, ks(1, i), fma(h * b62, ks(0, i), fma(h * b61, ks.dy(i), ks.y(i))))));
        derivs<TAB_ONLY>(xt, t + h, d);
        for (int i = 0; i < 9; ++i) ks(4, i) = d[i];
        for (int i = 0; i < 9; ++i)
            yn[i] = fma(h * c6, ks(4, i), fma(h * c5, ks(3, i), fma(h * c4, ks(2, i), fma(h * c3, ks(1, i), fma(h * c1, ks.dy(i), ks.y(i))))));
        derivs<TAB_ONLY>(yn, t + h, dyn, true);
        const double adt = fabs(h);
        double m = 0;
        for (int i = 0; i < 9; ++i) {
            double e = fma(h * dc7, dyn[i], fma(h * dc6, ks(4, i), fma(h * dc5, ks(3, i), fma(h * dc4, ks(2, i), fma(h * dc3, ks(1, i), (h * dc1) * ks.dy(i))))));
            double r = fabs(e) / (1e-9 + 1e-9 * (fabs(ks.y(i)) + adt * fabs(ks.dy(i))));
            m = (m < r || r != r) ? r : m; /* a NaN estimate sticks and rejects the step */
        }
        if (!(m <= 1.0)) {
            dt *= fmax(0.9 * (m < 1e300 ? ptdm_pow(m, -1.0 / 3.0) : 0.0), 0.2);
            ++nrej;
            ++lc.rk_rej;
            return 0;
        }
        to = t;
        tn = t + h;
        if (m < 0.5) {
            m = fmax(0.00032, m); /* 5^-5 */
            dt *= 0.9 * ptdm_pow(m, -1.0 / 5.0);
        }
        for (int i = 0; i < 9; ++i) { xo[i] = ks.y(i); dxo[i] = ks.dy(i); }
        ntry = 0;
        ++nacc;
        ++lc.rk_acc;
        return 1;
    }
    /* rk_try with the stage vectors in registers; k3 .. k6 kept for the dense output */
    __device__ int rk_try() {
        double ks[5][9];
        const int r = rk_try_with(KReg{ks, y, dydt});
        if (r == 1) {
            for (int i = 0; i < 9; ++i) { k3[i] = ks[1][i]; k4[i] = ks[2][i]; k5[i] = ks[3][i]; k6[i] = ks[4][i]; }
            tp.on_accept(*this, ks[0]);
        }
        return r;
    }

    /* runge_kutta_dopri5::calc_state: continuous extension on [to, tn]; the
     * weights b_i(theta) in monomial form by Horner's rule (the oracle
     * evaluates the same expression) */
    __device__ void dense_coef(double tt, double hb[6]) const {
        const double W[6][5] = {
            {1.0, -2.8605386690370884, 3.099577878709121, -1.1618105836403092, 0.013917207301610328},
            {0.0, 4.047141499642786, -6.345354046938926, 2.795465086414005, -0.04801624082496286},
            {0.0, -3.941160071112659, 10.904003027940295, -6.729317509209278, 0.4175162190483098},
            {0.0, 2.8419447015870345, -7.547675862959386, 4.957636724931253, -0.5742817428041846},
            {0.0, -1.6109886359167997, 4.218915839039518, -2.950103865566732, 0.47312904339639456},
            {0.0, 1.523601174836727, -4.329466835790622, 3.0881301470710616, -0.2822644861171672}};
        const double h = tn - to;
        const double th = (tt - to) / h;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            double p = W[k][4];
            p = fma(p, th, W[k][3]);
            p = fma(p, th, W[k][2]);
            p = fma(p, th, W[k][1]);
            p = fma(p, th, W[k][0]);
            hb[k] = h * (p * th);
        }
    }
    __device__ void calc_state(double tt, double *o) {
        double b[6];
        dense_coef(tt, b);
        for (int i = 0; i < 9; ++i)
            o[i] = fma(b[5], dyn[i], fma(b[4], k6[i], fma(b[3], k5[i], fma(b[2], k4[i], fma(b[1], k3[i], fma(b[0], dxo[i], xo[i]))))));
        ++lc.dense;
    }
    /* the state the precession axis needs: position, velocity and the
     * polarisation (component 7, constant along a step: its derivative is 0,
     * so every stage adds an exact zero and calc_state returns xo[7]); the
     * proper time and the path length are not needed (set to 0) */
    __device__ void calc_spin_state(double tt, double *o) {
        double b[6];
        dense_coef(tt, b);
        for (int i = 0; i < 6; ++i)
            o[i] = fma(b[5], dyn[i], fma(b[4], k6[i], fma(b[3], k5[i], fma(b[2], k4[i], fma(b[1], k3[i], fma(b[0], dxo[i], xo[i]))))));
        o[6] = 0;
        o[7] = xo[7];
        o[8] = 0;
        ++lc.dense;
    }
    __device__ void calc_pos(double tt, double *o) {
        double b[6];
        dense_coef(tt, b);
        for (int i = 0; i < 3; ++i)
            o[i] = fma(b[5], dyn[i], fma(b[4], k6[i], fma(b[3], k5[i], fma(b[2], k4[i], fma(b[1], k3[i], fma(b[0], dxo[i], xo[i]))))));
        ++lc.dense;
    }

    /* ---------------- geometry wrappers ---------------- */
    __device__ bool cand_cover(double ta, double tb) const { return ncand >= 0 && ta >= cand_ta && tb <= cand_tb; }
    /* any collision on segment p->q; returns -1 on a coplanar (CGAL error) case */
    __device__ int any_hit(const double *p, const double *q) { return any_hit(p, q, NAN, NAN); }
    /* the same for a chord between the dense-output points at tp and tq */
    __device__ int any_hit(const double *p, const double *q, double tp, double tq) {
        if (cand_cover(tp, tq)) {
            bool cp = false;
            Seg32 s32;
            seg32_make(p, q, s32);
            for (int j = 0; j < ncand; ++j) {
                ++lc.tri32;
                const int r32 = seg_tri32(s32, S.tri32[cand[j]]);
                if (r32 == 0) continue;
                if (r32 == 1) return 1;
                const DTri &t = S.tris[cand[j]];
                const int r64 = seg_tri64c(p, q, s32, t, S.tri32[cand[j]], S.tric[cand[j]]);
                if (r64 == 0) continue;
                if (r64 == 1) return 1;
                if (!tri_box_touch(t, p, q)) continue;
                ++lc.tris;
                double sv;
                int r = seg_tri(p, q, t, sv);
                if (r > 0) return 1;
                if (r < 0) cp = true;
            }
            return cp ? -1 : 0;
        }
        QueryStats qs{0, 0};
        bool cp;
        Coll dummy;
        int h = mesh_query<0>(S, p, q, 0, 0, &dummy, 0, nullptr, qs, cp);
        lc.nodes += qs.nodes;
        lc.tris += qs.tris;
        if (h) return 1;
        return cp ? -1 : 0;
    }
    __device__ int all_hits(double x1, const double *p, double x2, const double *q, Coll *c) {
        if (cand_cover(x1, x2)) {
            int nh = 0;
            for (int j = 0; j < ncand; ++j) {
                const DTri &t = S.tris[cand[j]];
                if (!tri_box_touch(t, p, q)) continue;
                ++lc.tris;
                double sv;
                int r = seg_tri(p, q, t, sv);
                if (r < 0) return -1;
                if (r == 0) continue;
                Coll cl;
                cl.s = sv;
                cl.n[0] = t.n[0]; cl.n[1] = t.n[1]; cl.n[2] = t.n[2];
                cl.solid = t.solid;
                cl.id = S.solids[t.solid].id;
                cl.dn = (q[0] - p[0]) * t.n[0] + (q[1] - p[1]) * t.n[1] + (q[2] - p[2]) * t.n[2];
                cl.ign = solid_ignored(S.solids[t.solid], x1 + (x2 - x1) * sv);
                if (nh >= PT_MAX_COLLS) return -2;
                int k = nh;
                while (k > 0 && (c[k - 1].s > cl.s || (c[k - 1].s == cl.s && c[k - 1].id < cl.id))) { c[k] = c[k - 1]; --k; }
                c[k] = cl;
                ++nh;
            }
            return nh;
        }
        QueryStats qs{0, 0};
        bool cp;
        int h = mesh_query<1>(S, p, q, x1, x2, c, PT_MAX_COLLS, nullptr, qs, cp);
        lc.nodes += qs.nodes;
        lc.tris += qs.tris;
        if (cp) return -1;
        if (h > PT_MAX_COLLS) return -2;
        return h;
    }

    /* Conservative box of the dense-output positions for t in [ta, tb]: each
     * coordinate is a degree-5 polynomial in theta = (t - to)/(tn - to); its
     * Bernstein coefficients on [theta_a, theta_b] bound it (convex hull
     * property), widened by 1e-9 m + 1e-12 relative to cover rounding.
     * Every chord between two dense-output points of that interval lies in
     * the box, so the triangles touching the box are all the bisection and
     * DoHit can ever hit. */
    __device__ void curve_box(double ta, double tb, double lo[3], double hi[3]) const {
        /* theta^1..theta^5 coefficients of the continuous-extension weights of
         * k1 (dxo), k3, k4, k5, k6, k7 (dyn), from runge_kutta_dopri5::calc_state */
        const double Wc[6][5] = {
            {1.0, -2.8605386690370884, 3.099577878709121, -1.1618105836403092, 0.013917207301610328},
            {0.0, 4.047141499642786, -6.345354046938926, 2.795465086414005, -0.04801624082496286},
            {0.0, -3.941160071112659, 10.904003027940295, -6.729317509209278, 0.4175162190483098},
            {0.0, 2.8419447015870345, -7.547675862959386, 4.957636724931253, -0.5742817428041846},
            {0.0, -1.6109886359167997, 4.218915839039518, -2.950103865566732, 0.47312904339639456},
            {0.0, 1.523601174836727, -4.329466835790622, 3.0881301470710616, -0.2822644861171672}};
        /* C(k,j)/C(5,j) for the monomial-to-Bernstein map */
        const double Bm[6][6] = {{1, 0, 0, 0, 0, 0},
                                 {1, 0.2, 0, 0, 0, 0},
                                 {1, 0.4, 0.1, 0, 0, 0},
                                 {1, 0.6, 0.3, 0.1, 0, 0},
                                 {1, 0.8, 0.6, 0.4, 0.2, 0},
                                 {1, 1, 1, 1, 1, 1}};
        const double h = tn - to;
        double t1 = (ta - to) / h, t2 = (tb - to) / h;
        const double D = t2 - t1;
        for (int k = 0; k < 3; ++k) {
            double c[6];
            c[0] = xo[k];
            for (int j = 1; j <= 5; ++j)
                c[j] = h * (Wc[0][j - 1] * dxo[k] + Wc[1][j - 1] * k3[k] + Wc[2][j - 1] * k4[k] + Wc[3][j - 1] * k5[k] +
                            Wc[4][j - 1] * k6[k] + Wc[5][j - 1] * dyn[k]);
            for (int i = 0; i < 5; ++i) /* Taylor shift to theta_a */
                for (int j = 4; j >= i; --j) c[j] += t1 * c[j + 1];
            double dj = 1;
            for (int j = 1; j <= 5; ++j) { dj *= D; c[j] *= dj; }
            double mn = 1e300, mx = -1e300, mag = 0;
            for (int r = 0; r <= 5; ++r) {
                double beta = 0;
                for (int j = 0; j <= r; ++j) beta += Bm[r][j] * c[j];
                mn = fmin(mn, beta);
                mx = fmax(mx, beta);
                mag = fmax(mag, fabs(beta));
            }
            double margin = 1e-9 + 1e-12 * mag;
            lo[k] = mn - margin;
            hi[k] = mx + margin;
        }
    }
    /* set up the candidate triangles for chord pieces within [ta, tb] */
    __device__ void prepare_candidates(double ta, double tb) {
        cand_span = tb - ta;
        double lo[3], hi[3];
        curve_box(ta, tb, lo, hi);
        bool ok = true;
        for (int k = 0; k < 3; ++k) ok = ok && isfinite(lo[k]) && isfinite(hi[k]);
        if (!ok) { ncand = -1; return; }
        QueryStats qs{0, 0};
        ncand = collect_candidates(S, lo, hi, cand, PT_MAX_CAND, qs);
        lc.nodes += qs.nodes;
        ++lc.cand_calls;
        if (ncand < 0) {
            ++lc.cand_overflow;
        } else {
            lc.cand_sum += ncand;
            cand_ta = ta;
            cand_tb = tb;
        }
    }
    /* candidates for [ta, tb] when the current set does not cover it and the
     * interval is at most a quarter of the last one tried (a set that
     * overflowed is retried once the search has narrowed) */
    __device__ void refresh_candidates(double ta, double tb) {
        if (cand_cover(ta, tb) || !(tb - ta <= 0.25 * cand_span) || ta < to || tb > tn) return;
        prepare_candidates(ta, tb);
    }
    __device__ void reset_candidates() {
        ncand = -1;
        cand_span = INFINITY;
    }

    /* ---------------- event logs ---------------- */
    /* TLogger::PrintHit (src/logger.cpp:202-235): time, state before and
     * after OnHit, the hit surface's normal, the solids left and entered */
    __device__ __noinline__ void log_hit(double x1, const double *y1, const double *y2, const double *nrm, uint32_t leaving, uint32_t entering) const {
        const unsigned long long k = atomicAdd(R.log.hit_n, 1ull);
        if ((long long)k >= R.log.cap) return;
        double *r = R.log.hit + k * PT_HIT_RECORD;
        const double v[PT_HIT_RECORD] = {(double)id, x1, y1[0], y1[1], y1[2], y1[3], y1[4], y1[5], y1[7],
                                         y2[3], y2[4], y2[5], y2[7], nrm[0], nrm[1], nrm[2], (double)leaving, (double)entering};
        for (int j = 0; j < PT_HIT_RECORD; ++j) r[j] = v[j];
    }
    /* TLogger::PrintSnapshot (src/logger.cpp:128-141): at the first
     * snapshot time in [to, x), the dense-output state there with the spin
     * and counters as they stand before the step's spin integration.  The
     * log functions stay out of line: inlined, they enlarge the fast step
     * completion that runs without them. */
    /* TLogger::PrintTrack (src/logger.cpp:143-200): at zero path length (a
     * particle's start) and when the step from path length l1 to y[8] crossed
     * a multiple of the interval, the state with the current solid */
    __device__ __noinline__ void log_track(double l1, double x, const double *y) const {
        const double iv = R.log.track_interval;
        if (!(iv > 0)) return;
        if (y[8] > 0 && (int)(l1 / iv) == (int)(y[8] / iv)) return;
        const unsigned long long k = atomicAdd(R.log.track_n, 1ull);
        if ((long long)k >= R.log.cap) return;
        double *r = R.log.track + k * PT_TRACK_RECORD;
        const double v[PT_TRACK_RECORD] = {(double)id, x, y[0], y[1], y[2], y[3], y[4], y[5], y[7], (double)S.solids[cur_solid()].id};
        for (int j = 0; j < PT_TRACK_RECORD; ++j) r[j] = v[j];
    }
    /* TLogger::PrintSpin (src/logger.cpp:237-284): at the start of a Bloch
     * integration (x == x1) and when a Bloch step from x1 to x crossed a
     * multiple of the interval: position, spin, precession axis and B at x */
    __device__ __noinline__ void log_spin(double x1, double x, const double *Sv) {
        const double iv = R.log.spin_interval;
        if (!(iv > 0)) return;
        if (x > x1 && (int)(x1 / iv) == (int)(x / iv)) return;
        double yy[9], W[3], B[3], dB[3][3];
        calc_spin_state(x, yy);
        spin_axis_at(x, W); /* TLogger::PrintSpin evaluates SpinPrecessionAxis itself */
        bfield<true>(S, R.prec, yy[0], yy[1], yy[2], B, dB);
        const unsigned long long k = atomicAdd(R.log.spin_n, 1ull);
        if ((long long)k >= R.log.cap) return;
        double *r = R.log.spin + k * PT_SPIN_RECORD;
        const double v[PT_SPIN_RECORD] = {(double)id, x, yy[0], yy[1], yy[2], Sv[0], Sv[1], Sv[2], W[0], W[1], W[2], B[0], B[1], B[2]};
        for (int j = 0; j < PT_SPIN_RECORD; ++j) r[j] = v[j];
    }
    __device__ __noinline__ bool snapshot_due(double x) const {
        for (int k = 0; k < R.log.n_snap; ++k)
            if (to <= R.log.snap_t[k] && R.log.snap_t[k] < x) return true;
        return false;
    }
    __device__ __noinline__ void log_snapshot(double x) {
        for (int k = 0; k < R.log.n_snap; ++k) {
            const double ts = R.log.snap_t[k];
            if (!(to <= ts && ts < x)) continue;
            double ys[9];
            calc_state(ts, ys);
            const unsigned long long j = atomicAdd(R.log.snap_n, 1ull);
            if ((long long)j < R.log.cap) {
                double *r = R.log.snap + j * PT_SNAPSHOT_RECORD;
                r[0] = (double)id;
                r[1] = ts;
                for (int c = 0; c < 9; ++c) r[2 + c] = ys[c];
                for (int c = 0; c < 5; ++c) r[11 + c] = spin[c];
                r[16] = (double)stop;
                r[17] = (double)nspinflip;
                r[18] = noflip;
                r[19] = (double)nhit;
                r[20] = (double)nstep;
                r[21] = hmax;
            }
            return;
        }
    }

    /* ---------------- RotateVector (src/globals.cpp:40-64) ---------------- */
    __device__ __forceinline__ static void rotate_vector(double v[3], const double n[3], const double *x) {
        double nn = n[0] * n[0] + n[1] * n[1] + n[2] * n[2];
        double xv[3];
        bool use_base = (x == nullptr);
        if (!use_base) {
            double lam = (n[0] * x[0] + n[1] * x[1] + n[2] * x[2]) / nn;
            for (int k = 0; k < 3; ++k) xv[k] = x[k] - lam * n[k];
            if (xv[0] * xv[0] + xv[1] * xv[1] + xv[2] * xv[2] < 1e-30) use_base = true;
        }
        if (use_base) { /* CGAL Plane_3::base1() */
            double a = fabs(n[0]), bb = fabs(n[1]), c = fabs(n[2]);
            if (n[0] == 0) { xv[0] = 1; xv[1] = 0; xv[2] = 0; }
            else if (n[1] == 0) { xv[0] = 0; xv[1] = 1; xv[2] = 0; }
            else if (n[2] == 0) { xv[0] = 0; xv[1] = 0; xv[2] = 1; }
            else if (a <= bb && a <= c) { xv[0] = 0; xv[1] = -n[2]; xv[2] = n[1]; }
            else if (bb <= a && bb <= c) { xv[0] = -n[2]; xv[1] = 0; xv[2] = n[0]; }
            else { xv[0] = -n[1]; xv[1] = n[0]; xv[2] = 0; }
        }
        double xl = sqrt(xv[0] * xv[0] + xv[1] * xv[1] + xv[2] * xv[2]);
        double zl = sqrt(nn);
        double xu[3] = {xv[0] / xl, xv[1] / xl, xv[2] / xl}, zu[3] = {n[0] / zl, n[1] / zl, n[2] / zl};
        double yu[3] = {zu[1] * xu[2] - zu[2] * xu[1], zu[2] * xu[0] - zu[0] * xu[2], zu[0] * xu[1] - zu[1] * xu[0]};
        double r[3];
        for (int k = 0; k < 3; ++k) r[k] = xu[k] * v[0] + yu[k] * v[1] + zu[k] * v[2];
        v[0] = r[0]; v[1] = r[1]; v[2] = r[2];
    }

    /* ---------------- neutron wall physics (src/neutron.cpp) ---------------- */
    __device__ void reflect(double x1, const double *y1, double &x2, double *y2, const double *n) {
        tp.on_reflect(*this, x1, x2, n);
        double vn = y1[3] * n[0] + y1[4] * n[1] + y1[5] * n[2];
        x2 = x1;
        y2[0] = y1[0]; y2[1] = y1[1]; y2[2] = y1[2];
        y2[3] -= 2 * vn * n[0]; y2[4] -= 2 * vn * n[1]; y2[5] -= 2 * vn * n[2];
        y2[6] = y1[6]; y2[8] = y1[8];
    }
    __device__ double sincos_draw() {
        double u = u01();
        double ca = cos(0.0), cb = cos(PT_PI / 2.);
        return acos(sqrt(u * (cb * cb - ca * ca) + ca * ca));
    }
    __device__ void reflect_lambert(double x1, const double *y1, double &x2, double *y2, const double *normal, const DMat &mat) {
        tp.on_other(*this);
        double vn = y1[3] * normal[0] + y1[4] * normal[1] + y1[5] * normal[2];
        double n[3] = {normal[0], normal[1], normal[2]};
        if (vn > 0) { vn *= -1; n[0] *= -1; n[1] *= -1; n[2] *= -1; }
        x2 = x1;
        y2[0] = y1[0]; y2[1] = y1[1]; y2[2] = y1[2];
        double vabs = sqrt(y1[3] * y1[3] + y1[4] * y1[4] + y1[5] * y1[5]);
        for (int it = 0;; ++it) {
            double phi = 2. * PT_PI * u01();
            double th = sincos_draw();
            y2[3] = vabs * cos(phi) * sin(th);
            y2[4] = vabs * sin(phi) * sin(th);
            y2[5] = vabs * cos(th);
            if (mat.diff > 0) rotate_vector(&y2[3], n, &y1[3]);
            else {
                double spec[3] = {y1[3] - 2 * vn * n[0], y1[4] - 2 * vn * n[1], y1[5] - 2 * vn * n[2]};
                rotate_vector(&y2[3], spec, &y1[3]);
            }
            if (y2[3] * n[0] + y2[4] * n[1] + y2[5] * n[2] > 0) break;
            if (it > PT_MAX_LAMBERT) { stop = PT_ID_GEOMETRY_ERROR; break; }
        }
        y2[6] = y1[6]; y2[8] = y1[8];
    }
    __device__ void transmit(const double *y1, double *y2, const double *n, double Estep) {
        tp.on_other(*this);
        double vn = y1[3] * n[0] + y1[4] * n[1] + y1[5] * n[2];
        double En = 0.5 * R.sp.m * vn * vn;
        double k1 = sqrt(En), k2 = sqrt(En - Estep);
        for (int i = 0; i < 3; i++) y2[i + 3] += (k2 / k1 - 1) * (n[i] * vn);
    }
    __device__ void transmit_lambert(const double *y1, double *y2, const double *normal, double Estep, const DMat &mat) {
        tp.on_other(*this);
        double vn = y1[3] * normal[0] + y1[4] * normal[1] + y1[5] * normal[2];
        double n[3] = {normal[0], normal[1], normal[2]};
        if (vn < 0) { vn *= -1; n[0] *= -1; n[1] *= -1; n[2] *= -1; }
        double En = 0.5 * R.sp.m * vn * vn;
        double k1 = sqrt(En), k2 = sqrt(En - Estep);
        double spec[3] = {y2[3], y2[4], y2[5]};
        for (int i = 0; i < 3; ++i) spec[i] += (k2 / k1 - 1) * n[i] * vn;
        double vabs = sqrt(spec[0] * spec[0] + spec[1] * spec[1] + spec[2] * spec[2]);
        for (int it = 0;; ++it) {
            double phi = 2. * PT_PI * u01();
            double th = sincos_draw();
            y2[3] = vabs * cos(phi) * sin(th);
            y2[4] = vabs * sin(phi) * sin(th);
            y2[5] = vabs * cos(th);
            if (mat.diff > 0) rotate_vector(&y2[3], n, &y1[3]);
            else rotate_vector(&y2[3], spec, &y1[3]);
            if (y2[3] * n[0] + y2[4] * n[1] + y2[5] * n[2] > 0) break;
            if (it > PT_MAX_LAMBERT) { stop = PT_ID_GEOMETRY_ERROR; break; }
        }
    }
    /* direction drawn from MRDist by rejection under 1.5 times the
     * transmission distribution's maximum, as TNeutron::ReflectMR and
     * TransmitMR both take it (src/neutron.cpp:46, 125): phi uniform, theta
     * sin-distributed on [0, pi/2], a uniform test draw; the polar angle is
     * turned to the far side of the surface as the motion requires */
    __device__ __noinline__ void mr_direction(const MRHit &h, bool transmit, double &theta, double &phi) {
        const double env = 1.5 * mr_distmax(h, true);
        for (int it = 0;; ++it) {
            phi = 2. * PT_PI * u01();
            theta = acos(cos(0.0) - u01() * (cos(0.0) - cos(PT_PI / 2.)));
            if (!(u01() * env > mr_dist(h, transmit, false, theta, phi))) break;
            if (it > PT_MAX_LAMBERT) { stop = PT_ID_GEOMETRY_ERROR; break; }
        }
    }
    /* TNeutron::ReflectMR (src/neutron.cpp:118-148) */
    __device__ void reflect_mr(double x1, const double *y1, double &x2, double *y2, const double *normal, const MRHit &h) {
        tp.on_other(*this);
        double th, ph;
        mr_direction(h, false, th, ph);
        double vn = y1[3] * normal[0] + y1[4] * normal[1] + y1[5] * normal[2];
        if (vn > 0) th = PT_PI - th;
        x2 = x1;
        y2[0] = y1[0]; y2[1] = y1[1]; y2[2] = y1[2];
        double vabs = sqrt(y1[3] * y1[3] + y1[4] * y1[4] + y1[5] * y1[5]);
        y2[3] = vabs * cos(ph) * sin(th);
        y2[4] = vabs * sin(ph) * sin(th);
        y2[5] = vabs * cos(th);
        rotate_vector(&y2[3], normal, &y1[3]);
        y2[6] = y1[6]; y2[8] = y1[8];
    }
    /* TNeutron::TransmitMR (src/neutron.cpp:38-62) */
    __device__ void transmit_mr(const double *y1, double *y2, const double *normal, double Estep, const MRHit &h) {
        tp.on_other(*this);
        double th, ph;
        mr_direction(h, true, th, ph);
        double vabs = sqrt(y1[3] * y1[3] + y1[4] * y1[4] + y1[5] * y1[5] - 2 * Estep / PT_M_N);
        double vn = y1[3] * normal[0] + y1[4] * normal[1] + y1[5] * normal[2];
        if (vn < 0) th = PT_PI - th;
        y2[3] = vabs * cos(ph) * sin(th);
        y2[4] = vabs * sin(ph) * sin(th);
        y2[5] = vabs * cos(th);
        rotate_vector(&y2[3], normal, &y1[3]);
    }
    /* TNeutron::OnHit (src/neutron.cpp:187-264); charged species: empty */
    __device__ void on_hit(double x1, const double *y1, double &x2, double *y2, const double *normal, int leaving, int entering) {
        if (R.sp.kind != PT_NEUTRON) return;
        const DMat &ml = S.mats[S.solids[leaving].mat], &me = S.mats[S.solids[entering].mat];
        double vn = y1[3] * normal[0] + y1[4] * normal[1] + y1[5] * normal[2];
        double En = 0.5 * R.sp.m * vn * vn;
        const DMat &mat = vn < 0 ? me : ml;
        if (u01() < mat.spinflip) y2[7] *= -1;
        double Estep = mat_pot(me, y2[7]) - mat_pot(ml, y2[7]);
        /* MicroRoughness reflection and transmission probabilities */
        const bool use_mr = mat.rms != 0 && mat.corr != 0 && mr_valid(&y1[3], Estep, mat.rms, mat.corr);
        double mrr = 0, mrt = 0;
        MRHit h;
        if (use_mr) {
            bool ok = true;
            mr_setup(h, &y1[3], normal, Estep, mat.rms, mat.corr);
            mrr = mr_prob(h, false, ok);
            if (ekin(&y1[3]) > Estep) mrt = mr_prob(h, true, ok);
            if (!ok) { stop = PT_ID_ODEINT_ERROR; return; }
        }
        double prob = u01();
        if (use_mr && prob < mrr) { reflect_mr(x1, y1, x2, y2, normal, h); return; }
        if (use_mr && prob < mrr + mrt) { transmit_mr(y1, y2, normal, Estep, h); return; }
        double k1r, k1i, k2r, k2i;
        csqrt(En, -ml.fermi_imag * 1e-9, k1r, k1i);
        csqrt(En - Estep, -me.fermi_imag * 1e-9, k2r, k2i);
        double nr = k1r - k2r, ni = k1i - k2i, dr = k1r + k2r, di = k1i + k2i;
        double reflprob = (nr * nr + ni * ni) / (dr * dr + di * di);
        if (En > Estep) {
            if (prob < mrr + mrt + reflprob * (1 - mrr - mrt)) {
                if (!use_mr && u01() < mat.diff + mat.modlambert) reflect_lambert(x1, y1, x2, y2, normal, mat);
                else reflect(x1, y1, x2, y2, normal);
            } else {
                if (!use_mr && u01() < mat.diff + mat.modlambert) transmit_lambert(y1, y2, normal, Estep, mat);
                else transmit(y1, y2, normal, Estep);
            }
        } else {
            double absprob = 1 - reflprob + mat.loss;
            if (use_mr) { /* second-order correction for reflection on rough surfaces, with the entered solid's roughness */
                double kc = sqrt(2 * PT_M_N * Estep) * PT_ELE_E / PT_HBAR;
                double addtrans = 2 * (me.rms * me.rms) * kc * kc / (1 + 0.85 * kc * me.corr + 2 * kc * kc * (me.corr * me.corr));
                absprob *= sqrt(1 + addtrans);
            }
            if (prob < mrr + mrt + absprob * (1 - mrr - mrt)) stop = PT_ID_ABSORBED_ON_SURFACE;
            else {
                if (!use_mr && u01() < mat.diff + mat.modlambert) reflect_lambert(x1, y1, x2, y2, normal, mat);
                else reflect(x1, y1, x2, y2, normal);
            }
        }
    }
    /* TNeutron::OnStep (src/neutron.cpp:267-282), TProton/TElectron::OnStep */
    __device__ void on_step(double x1, const double *y1, double &x2, double *y2, int solid) {
        if (R.sp.kind == PT_NEUTRON) {
            const DMat &m = S.mats[S.solids[solid].mat];
            if (m.fermi_imag > 0) {
                double Er = 0.5 * R.sp.m * (y1[3] * y1[3] + y1[4] * y1[4] + y1[5] * y1[5]), Ei = m.fermi_imag * 1e-9;
                double kr, ki;
                csqrt(2 * R.sp.m * Er, 2 * R.sp.m * Ei, kr, ki);
                ki = ki * PT_ELE_E / PT_HBAR;
                double dx = y2[0] - y1[0], dy = y2[1] - y1[1], dz = y2[2] - y1[2];
                double l = sqrt(dx * dx + dy * dy + dz * dz);
                double abspath = -log(1 - u01()) / (2 * ki);
                if (abspath < l) {
                    x2 = x1 + abspath / l * (x2 - x1);
                    calc_state(x2, y2);
                    stop = PT_ID_ABSORBED_IN_MATERIAL;
                }
            }
        } else {
            if (S.solids[solid].id > 1) {
                x2 = x1;
                for (int i = 0; i < 9; ++i) y2[i] = y1[i];
                stop = PT_ID_ABSORBED_IN_MATERIAL;
            }
        }
    }

    /* TTracker::DoStep + TParticle::DoStep (src/tracking.cpp:268-278, src/particle.cpp:196-206) */
    __device__ bool do_step(double x1, const double *y1, double &x2, double *y2, int solid) {
        double x2t = x2, y2t[9];
        for (int i = 0; i < 9; ++i) y2t[i] = y2[i];
        on_step(x1, y1, x2, y2, solid);
        hmax = fmax(ekin(&y2[3]) + epot(x2, y2, solid), hmax);
        if (y2t[7] != y2[7]) nspinflip++;
        nstep++;
        ++lc.subseg;
        bool same = (x2t == x2);
        for (int i = 0; i < 9; ++i) same = same && (y2[i] == y2t[i]);
        return !same;
    }

    /* One bisection as a resumable state machine: bisect_begin sets it up and
     * each bisect_step runs one iteration of the search (at most one chord
     * query), so a kernel can interleave the bisections of several particles
     * on one lane and keep the lanes of a warp on the same iteration. */
    __device__ void bisect_begin(BisectState &bs, double x1, const double *p1, double x2, const double *p2) const {
        bs.ch0 = bs.ch1 = bs.tr0 = bs.tr1 = 0;
        bs.level = 0;
        bs.A = x1;
        bs.B = x2;
        for (int k = 0; k < 3; ++k) {
            bs.pA[k] = p1[k];
            bs.pB[k] = p2[k];
            bs.p2[k] = p2[k];
            bs.pc[k] = 0;
        }
        bs.xc = 0;
        bs.Ao = bs.Bo = true;
        bs.work = 0;
        bs.phase = BisectState::ENTER;
    }
    /* BISECT_RUNNING while the search goes on, else bisect()'s result */
    __device__ int bisect_step(BisectState &bs, double &xa, bool &aorig, double &xb, bool &borig) {
        auto getbit = [](uint64_t a, uint64_t b, int l) -> bool { return l < 64 ? ((a >> l) & 1) : ((b >> (l - 64)) & 1); };
        auto setbit = [](uint64_t &a, uint64_t &b, int l, bool v) {
            if (l < 64) { if (v) a |= (1ull << l); else a &= ~(1ull << l); }
            else { if (v) b |= (1ull << (l - 64)); else b &= ~(1ull << (l - 64)); }
        };
        if (bs.phase == BisectState::ENTER) {
            /* termination tests at the entry of iterate_collision */
            double dx = bs.pB[0] - bs.pA[0], dy = bs.pB[1] - bs.pA[1], dz = bs.pB[2] - bs.pA[2];
            if (dx * dx + dy * dy + dz * dz < PT_REFLECT_TOLERANCE * PT_REFLECT_TOLERANCE ||
                bs.B - bs.A < 4 * (bs.A + bs.B) * 2.220446049250313e-16 || bs.level >= PT_MAX_BISECT_LEVELS) {
                xa = bs.A; aorig = bs.Ao; xb = bs.B; borig = bs.Bo;
                lc.bisect_max = max(lc.bisect_max, (unsigned)bs.work);
                return 1;
            }
            ++lc.bisect;
            bs.stA[bs.level] = bs.A;
            bs.stB[bs.level] = bs.B;
            refresh_candidates(bs.A, bs.B);
            bs.xc = bs.A + (bs.B - bs.A) * 0.5;
            calc_pos(bs.xc, bs.pc);
        } else if (bs.phase == BisectState::RESUME) {
            /* second half of a stacked level: the start is the input start
             * iff every choice above took the first half, the end is the
             * input end iff every choice took the second half */
            bs.A = bs.stA[bs.level];
            bs.B = bs.stB[bs.level];
            bool allsecond = true;
            for (int l = 0; l < bs.level; ++l) allsecond = allsecond && getbit(bs.ch0, bs.ch1, l);
            bs.Bo = allsecond;
            if (bs.Bo) { bs.pB[0] = bs.p2[0]; bs.pB[1] = bs.p2[1]; bs.pB[2] = bs.p2[2]; }
            else calc_pos(bs.B, bs.pB);
            bs.xc = bs.A + (bs.B - bs.A) * 0.5;
            calc_pos(bs.xc, bs.pc);
        }
        /* the one chord query of this iteration: first half (A, xc) on
         * entering a level, else second half (xc, B) */
        const bool first = (bs.phase == BisectState::ENTER);
        double P[3], Q[3];
        for (int k = 0; k < 3; ++k) {
            P[k] = first ? bs.pA[k] : bs.pc[k];
            Q[k] = first ? bs.pc[k] : bs.pB[k];
        }
        if (++bs.work > PT_MAX_BISECT_WORK) { lc.bisect_max = max(lc.bisect_max, (unsigned)bs.work); return -1; }
        const int h = any_hit(P, Q, first ? bs.A : bs.xc, first ? bs.xc : bs.B);
        if (h < 0) { lc.bisect_max = max(lc.bisect_max, (unsigned)bs.work); return -1; }
        if (bs.phase == BisectState::RESUME) setbit(bs.tr0, bs.tr1, bs.level, true);
        if (h) {
            setbit(bs.ch0, bs.ch1, bs.level, !first);
            if (bs.phase == BisectState::ENTER) setbit(bs.tr0, bs.tr1, bs.level, false);
            if (bs.phase == BisectState::SECOND) setbit(bs.tr0, bs.tr1, bs.level, true);
            if (first) { bs.B = bs.xc; bs.pB[0] = bs.pc[0]; bs.pB[1] = bs.pc[1]; bs.pB[2] = bs.pc[2]; bs.Bo = false; }
            else { bs.A = bs.xc; bs.pA[0] = bs.pc[0]; bs.pA[1] = bs.pc[1]; bs.pA[2] = bs.pc[2]; bs.Ao = false; }
            ++bs.level;
            bs.phase = BisectState::ENTER;
            return BISECT_RUNNING;
        }
        if (bs.phase == BisectState::ENTER) { bs.phase = BisectState::SECOND; return BISECT_RUNNING; }
        /* neither half of this level leads to a collision: a dead end;
         * back up to the nearest level whose second half is untried */
        ++lc.dead;
        bool found = false;
        while (bs.level > 0) {
            --bs.level;
            if (getbit(bs.tr0, bs.tr1, bs.level)) { ++lc.dead; continue; } /* both halves of this level done */
            found = true;
            break;
        }
        if (!found) {
            lc.bisect_max = max(lc.bisect_max, (unsigned)bs.work);
            return 0;
        }
        bs.phase = BisectState::RESUME;
        return BISECT_RUNNING;
    }
    /* TTracker::iterate_collision (src/tracking.cpp:228-265) without recursion:
     * a depth-first search over halves with an explicit stack of interval
     * times (positions of stacked interval ends are recomputed from the dense
     * output, which is deterministic).  Every step (bisect_step) makes at most one
     * chord query, from one call site, so lanes of a warp that bisect at the
     * same time stay converged whichever half they are in.  Returns 1 with the
     * final bracket [xa, xb] (aorig/borig: the bracket end is an input end), 0
     * when no sub-chord collides, -1 on a CGAL-error case or when the search
     * exceeds its work bound. */
    __device__ int bisect(double x1, const double *p1, double x2, const double *p2, double &xa, bool &aorig, double &xb,
                          bool &borig) {
        BisectState bs;
        bisect_begin(bs, x1, p1, x2, p2);
        int r;
        while ((r = bisect_step(bs, xa, aorig, xb, borig)) == BISECT_RUNNING) {}
        return r;
    }

    /* TTracker::DoHit (src/tracking.cpp:280-365) */
    __device__ bool do_hit(double x1, const double *y1, double &x2, double *y2) {
        bool altered = false, traversed = true;
        Coll colls[PT_MAX_COLLS];
        int nc = all_hits(x1, y1, x2, y2, colls);
        if (nc <= 0) { stop = PT_ID_CGAL_ERROR; return true; }
        int nn = nsol;
        uint64_t ns = stk; /* the new list, same packing */
        for (int c = 0; c < nc; ++c) {
            const Coll &cl = colls[c];
            int found = -1;
            for (int i = 0; i < nn; ++i) if (S.solids[stk_idx(ns, i)].id == cl.id) { found = i; break; }
            if (cl.dn < 0) {
                if (found >= 0) {
                    if (cl.s > 0) {
                        if (nn >= PT_MAX_STACK) { stop = PT_ID_GEOMETRY_ERROR; return true; }
                        ns = stk_put(ns, nn, cl.solid, stk_ign(ns, found)); ++nn;
                    }
                } else {
                    if (nn >= PT_MAX_STACK) { stop = PT_ID_GEOMETRY_ERROR; return true; }
                    ns = stk_put(ns, nn, cl.solid, cl.ign); ++nn;
                }
            } else if (cl.dn > 0) {
                if (found < 0) {
                    if (cl.s > 0) { stop = PT_ID_GEOMETRY_ERROR; return true; }
                } else {
                    ns = stk_erase(ns, found, nn);
                    --nn;
                }
            } else {
                stop = PT_ID_GEOMETRY_ERROR;
                return true;
            }
        }
        int leaving = cur_solid();
        int entering = 0;
        for (int i = 0; i < nn; ++i)
            if (!stk_ign(ns, i) && S.solids[stk_idx(ns, i)].id > S.solids[entering].id) entering = stk_idx(ns, i);
        if (S.solids[leaving].id != S.solids[entering].id) {
            int ci = -1;
            for (int c = 0; c < nc; ++c)
                if (colls[c].id == S.solids[leaving].id || (colls[c].id == S.solids[entering].id && !colls[c].ign)) { ci = c; break; }
            if (ci < 0) { stop = PT_ID_GEOMETRY_ERROR; return true; }
            double x2t = x2, y2t[9];
            for (int i = 0; i < 9; ++i) y2t[i] = y2[i];
            on_hit(x1, y1, x2, y2, colls[ci].n, leaving, entering);
            if (y2t[7] != y2[7]) nspinflip++;
            nhit++;
            ++lc.hits;
            bool same = (x2t == x2);
            for (int i = 0; i < 9; ++i) same = same && (y2[i] == y2t[i]);
            if (same) { altered = false; traversed = true; }
            else {
                altered = true;
                if (x2 == x2t && y2[0] == y2t[0] && y2[1] == y2t[1] && y2[2] == y2t[2]) traversed = true;
                else if (x2 == x1 && y2[0] == y1[0] && y2[1] == y1[1] && y2[2] == y1[2]) traversed = false;
                else { stop = PT_ID_GEOMETRY_ERROR; return true; }
            }
            if (R.log.hit) log_hit(x1, y1, y2, colls[ci].n, S.solids[leaving].id, S.solids[entering].id);
        }
        if (traversed) {
            nsol = nn;
            stk = ns;
        }
        return altered || stop != PT_ID_UNKNOWN;
    }

    /* TTracker::IntegrateSpin decision logic (src/tracking.cpp:373-483), in
     * two parts around the Bloch integration so that a kernel can run the
     * latter one step at a time: spin_begin returns 1 when the Bloch
     * integration is to run (its stepper set up in bst, towards bx2), 0 when
     * IntegrateSpin is complete (its result in sproj); spin_end(r) finishes
     * it after bloch_run returned r.  BLOCH = false compiles the variant
     * without the Bloch integration, for callers that have checked
     * spin_integrates() first. */
    template <bool BLOCH = true>
    __device__ int spin_begin(double x2, const double *y2, double &sproj) {
        double B1[3], B2[3];
        bonly(xo[0], xo[1], xo[2], to, B1);
        bonly(y2[0], y2[1], y2[2], x2, B2);
        double Babs1 = sqrt(B1[0] * B1[0] + B1[1] * B1[1] + B1[2] * B1[2]);
        double Babs2 = sqrt(B2[0] * B2[0] + B2[1] * B2[1] + B2[2] * B2[2]);
        if (R.sp.gamma == 0 || Babs2 == 0) {
            for (int k = 0; k < 5; ++k) spin[k] = 0;
            sproj = xo[7];
            return 0;
        } else if (Babs1 == 0 && Babs2 > 0) {
            double s = (u01() < 0.5 ? 0 : 1) * 2 - 1;
            for (int k = 0; k < 5; ++k) spin[k] = 0;
            sproj = s;
            return 0;
        } else if (x2 > to && (Babs1 < R.bmax || Babs2 < R.bmax)) {
            bool i1 = false, i2 = false;
            for (int i = 0; i + 1 < R.n_spintimes; i += 2) {
                i1 |= (to >= R.spintimes[i] && to < R.spintimes[i + 1]);
                i2 |= (x2 >= R.spintimes[i] && x2 < R.spintimes[i + 1]);
            }
            if (i1 || i2) {
                if (spin[0] == 0 && spin[1] == 0 && spin[2] == 0)
                    for (int k = 0; k < 3; ++k) spin[k] = B1[k] * xo[7] / Babs1;
                if (!BLOCH) {
                    stop = PT_ID_ODEINT_ERROR;
                    sproj = xo[7];
                    return 0;
                }
                sBabs2 = Babs2;
                for (int k = 0; k < 3; ++k) sB2[k] = B2[k];
                bx2 = x2;
                om_on = false;
                if (R.interp) omega_spline(to, x2);
                bloch_begin(bst, to, x2, fabs(PT_PI / R.sp.gamma / Babs1));
                return 1;
            } else if (spin[0] != 0 || spin[1] != 0 || spin[2] != 0) {
                double proj = (spin[0] * B1[0] + spin[1] * B1[1] + spin[2] * B1[2]) / Babs1 /
                              sqrt(spin[0] * spin[0] + spin[1] * spin[1] + spin[2] * spin[2]);
                if (proj * proj >= 1) { spin[0] = 0; spin[1] = 0; }
                else {
                    double az = 2. * PT_PI * u01();
                    spin[0] = sqrt(1 - proj * proj) * sin(az);
                    spin[1] = sqrt(1 - proj * proj) * cos(az);
                }
                spin[2] = proj;
                rotate_vector(spin, B2, nullptr);
            }
        }
        sproj = spin_tail(Babs2, B2);
        return 0;
    }
    /* the end of IntegrateSpin: projection onto B where |B| exceeds Bmax */
    __device__ double spin_tail(double Babs2, const double *B2) {
        if (Babs2 > R.bmax && (spin[0] != 0 || spin[1] != 0 || spin[2] != 0)) {
            double proj = (spin[0] * B2[0] + spin[1] * B2[1] + spin[2] * B2[2]) / Babs2 /
                          sqrt(spin[0] * spin[0] + spin[1] * spin[1] + spin[2] * spin[2]);
            for (int k = 0; k < 5; ++k) spin[k] = 0;
            return proj;
        }
        return xo[7];
    }
    __device__ double spin_end(int r) {
        if (r != 1) {
            stop = PT_ID_ODEINT_ERROR;
            return xo[7];
        }
        return spin_tail(sBabs2, sB2);
    }
    template <bool BLOCH = true>
    __device__ double integrate_spin(double x2, const double *y2) {
        double sp;
        if (spin_begin<BLOCH>(x2, y2, sp)) return spin_end(bloch_run(bst, bx2, -1));
        return sp;
    }

    /* whether integrate_spin(x2, y2) would run the Bloch integration */
    __device__ bool spin_integrates(double x2, const double *y2) {
        if (R.sp.gamma == 0 || R.n_spintimes < 2 || !(x2 > to)) return false;
        bool i1 = false, i2 = false;
        for (int i = 0; i + 1 < R.n_spintimes; i += 2) {
            i1 |= (to >= R.spintimes[i] && to < R.spintimes[i + 1]);
            i2 |= (x2 >= R.spintimes[i] && x2 < R.spintimes[i + 1]);
        }
        if (!(i1 || i2)) return false;
        double B1[3], B2[3];
        bonly(xo[0], xo[1], xo[2], to, B1);
        bonly(y2[0], y2[1], y2[2], x2, B2);
        const double Babs1 = sqrt(B1[0] * B1[0] + B1[1] * B1[1] + B1[2] * B1[2]);
        const double Babs2 = sqrt(B2[0] * B2[0] + B2[1] * B2[1] + B2[2] * B2[2]);
        if (Babs2 == 0 || Babs1 == 0) return false;
        return Babs1 < R.bmax || Babs2 < R.bmax;
    }

    /* first-call setup: IntegrateParticle's prologue (src/tracking.cpp:19-69)
     * and the TParticle constructor's Hmax (src/particle.cpp:88-89) */
    __device__ void init(QueryStats &qs) {
        rn = 0;
        if (R.tau > 0) tau = -log(1 - u01()) * R.tau;
        else tau = R.tmax;
        nsol = 1;
        stk = 0; /* entry 0: solid 0, not ignored */
        uint64_t m = point_solids(S, y, qs);
        for (int s = 1; s < S.n_solids; ++s)
            if (m & (1ull << s)) {
                if (nsol < PT_MAX_STACK) { stk = stk_put(stk, nsol, s, solid_ignored(S.solids[s], t)); ++nsol; }
                else stop = PT_ID_GEOMETRY_ERROR;
            }
        double h0 = ekin(&y[3]) + epot(t, y, cur_solid());
        hmax = h0;
        noflip = 1;
        nhit = nstep = nspinflip = 0;
        nacc = nrej = 0;
        dt = 10. * PT_MAX_TRACK_DEVIATION / sqrt(y[3] * y[3] + y[4] * y[4] + y[5] * y[5]);
        ntry = 0;
        derivs(y, t, dydt); /* stepper.initialize + first derivative */
        flags = PT_F_INIT | PT_F_DERIV;
        if (stop == PT_ID_UNKNOWN && t > R.simtime) stop = PT_ID_NOT_FINISH;
    }

    /* The remainder of one LOOP-A iteration (src/tracking.cpp:87-147) after an
     * accepted try -- decay/tmax clipping, chord splitting, CheckHit with its
     * bisection, spin and stop checks, commit -- as a resumable state machine.
     * Returns 1 when it needs the bisection of (ps.cx1, ps.cya) -> (ps.x2,
     * ps.y2) (result expected in ps.bres/bxa/bxb/bao/bbo, then call again), 0
     * when the step is finished; with SPLIT, 2 when only its Bloch
     * integration is left (run bloch_run on bst, then bloch_finish).  Call
     * with ps.stage = PS_BEGIN first. */
    template <bool SPLIT = false>
    __device__ int post_resume() {
        PostState &P = ps;
        bool ch = false;
        if (P.stage == PS_BEGIN) {
            P.x1 = to;
            for (int i = 0; i < 9; ++i) P.y1[i] = xo[i];
            P.x = tn;
            for (int i = 0; i < 9; ++i) P.yl[i] = yn[i];
            bool finite = isfinite(tn);
            for (int i = 0; i < 9; ++i) finite = finite && isfinite(yn[i]);
            if (!finite) { /* a non-finite state would never stop: report it as an integrator failure */
                stop = PT_ID_ODEINT_ERROR;
                return 0;
            }
            if (tau > 0 && P.yl[6] > tau) {
                P.x = P.x1 + (P.x - P.x1) * (tau - P.y1[6]) / (P.yl[6] - P.y1[6]);
                calc_state(P.x, P.yl);
            }
            if (P.x > R.simtime) {
                P.x = R.simtime;
                calc_state(P.x, P.yl);
            }
            P.reset = false;
            P.nsub = 0;
            P.stage = PS_OUTER;
        }
        while (true) {
            if (P.stage == PS_OUTER) {
                if (!(P.x1 < P.x)) break;
                if (++P.nsub > PT_MAX_SUBSEGMENTS) { stop = PT_ID_ODEINT_ERROR; break; }
                double l2 = (P.yl[8] - P.y1[8]) * (P.yl[8] - P.y1[8]);
                double d2 = (P.yl[0] - P.y1[0]) * (P.yl[0] - P.y1[0]) + (P.yl[1] - P.y1[1]) * (P.yl[1] - P.y1[1]) +
                            (P.yl[2] - P.y1[2]) * (P.yl[2] - P.y1[2]);
                double dev2 = 0.25 * (l2 - d2);
                P.x2 = P.x;
                for (int i = 0; i < 9; ++i) P.y2[i] = P.yl[i];
                if (dev2 > PT_MAX_TRACK_DEVIATION * PT_MAX_TRACK_DEVIATION) {
                    P.x2 = P.x1 + (P.x - P.x1) / ceil(sqrt(dev2) / PT_MAX_TRACK_DEVIATION);
                    if (!(P.x2 > P.x1)) { stop = PT_ID_ODEINT_ERROR; break; } /* split below time resolution */
                    calc_state(P.x2, P.y2);
                }
                /* TTracker::CheckHit (src/tracking.cpp:176-226) on (x1, y1) -> (x2, y2);
                 * its tail recursion is the PS_CHECK loop */
                reset_candidates();
                P.cx1 = P.x1;
                for (int i = 0; i < 9; ++i) P.cya[i] = P.y1[i];
                P.pass = 0;
                P.stage = PS_CHECK;
            } else if (P.stage == PS_CHECK) {
                if (P.pass++ >= PT_MAX_HITS_PER_SEGMENT) { stop = PT_ID_CGAL_ERROR; ch = true; P.stage = PS_CHECK_DONE; continue; }
                if (!check_segment(S, P.cya, P.y2)) { stop = PT_ID_HIT_BOUNDARIES; ch = true; P.stage = PS_CHECK_DONE; continue; }
                if (P.x2 == P.cx1) { ch = false; P.stage = PS_CHECK_DONE; continue; }
                P.cs = cur_solid();
                /* the candidate triangles of the chord's stretch of curve serve
                 * this query and the bisection that follows a hit */
                refresh_candidates(P.cx1, P.x2);
                int h = any_hit(P.cya, P.y2, P.cx1, P.x2);
                if (h < 0) { stop = PT_ID_CGAL_ERROR; ch = true; P.stage = PS_CHECK_DONE; continue; }
                if (!h) {
                    reset_candidates();
                    ch = do_step(P.cx1, P.cya, P.x2, P.y2, P.cs);
                    P.stage = PS_CHECK_DONE;
                    continue;
                }
                P.stage = PS_AFTER_BISECT;
                return 1; /* TTracker::iterate_collision on (cx1, cya) -> (x2, y2) */
            } else if (P.stage == PS_AFTER_BISECT) {
                if (P.bres < 0) { stop = PT_ID_CGAL_ERROR; ch = true; P.stage = PS_CHECK_DONE; continue; }
                if (P.bres == 0) { ch = false; P.stage = PS_CHECK_DONE; continue; }
                double yc1[9], yc2[9];
                if (P.bao) for (int i = 0; i < 9; ++i) yc1[i] = P.cya[i];
                else calc_state(P.bxa, yc1);
                if (P.bbo) for (int i = 0; i < 9; ++i) yc2[i] = P.y2[i];
                else calc_state(P.bxb, yc2);
                double xc1 = P.bxa, xc2 = P.bxb;
                if (xc1 > P.cx1 && do_step(P.cx1, P.cya, xc1, yc1, P.cs)) {
                    P.x2 = xc1;
                    for (int i = 0; i < 9; ++i) P.y2[i] = yc1[i];
                    ch = true;
                    P.stage = PS_CHECK_DONE;
                    continue;
                }
                if (do_hit(xc1, yc1, xc2, yc2)) {
                    P.x2 = xc2;
                    for (int i = 0; i < 9; ++i) P.y2[i] = yc2[i];
                    ch = true;
                    P.stage = PS_CHECK_DONE;
                    continue;
                }
                if (!(xc2 > P.cx1)) { stop = PT_ID_CGAL_ERROR; ch = true; P.stage = PS_CHECK_DONE; continue; } /* no progress */
                P.cx1 = xc2;
                for (int i = 0; i < 9; ++i) P.cya[i] = yc2[i];
                P.stage = PS_CHECK;
            } else { /* PS_CHECK_DONE: back in the chord-piece loop */
                reset_candidates();
                P.reset = ch;
                if (P.reset) {
                    P.x = P.x2;
                    for (int i = 0; i < 9; ++i) P.yl[i] = P.y2[i];
                }
                P.x1 = P.x2;
                for (int i = 0; i < 9; ++i) P.y1[i] = P.y2[i];
                P.stage = PS_OUTER;
            }
        }
        if (SPLIT) { /* return 2 with the Bloch integration pending (see finish_begin) */
            double sp;
            if (finish_begin<true>(P.x, P.yl, P.reset, sp)) return 2;
            finish_end(P.x, P.yl, P.reset, sp);
            return 0;
        }
        finish_step(P.x, P.yl, P.reset);
        return 0;
    }

    /* the whole post-step with the bisections run inline (plain form) */
    __device__ void post_step() {
        ps.stage = PS_BEGIN;
        while (post_resume() == 1)
            ps.bres = bisect(ps.cx1, ps.cya, ps.x2, ps.y2, ps.bxa, ps.bao, ps.bxb, ps.bbo);
    }

    /* IntegrateSpin + polarisation bookkeeping + stop checks
     * (src/tracking.cpp:128-147), then commit the loop state. */
    template <bool BLOCH = true>
    __device__ void finish_step(double x, double *yl, bool reset) {
        double sp;
        if (finish_begin<BLOCH>(x, yl, reset, sp)) sp = spin_end(bloch_run(bst, bx2, -1));
        finish_end(x, yl, reset, sp);
    }
    /* finish_step up to its Bloch integration: true when that is to run
     * (then bloch_finish(bloch_run's result) completes the step) */
    template <bool BLOCH = true>
    __device__ bool finish_begin(double x, double *yl, bool reset, double &sproj) {
        tp.on_segment(*this, x, yl, reset);
        if (R.log.snap) log_snapshot(x);
        if (spin_begin<BLOCH>(x, yl, sproj)) {
            fx = x;
            fyl = yl;
            freset = reset;
            return true;
        }
        return false;
    }
    __device__ void bloch_finish(int r) { finish_end(fx, fyl, freset, spin_end(r)); }
    __device__ void finish_end(double x, double *yl, bool reset, double sproj) {
        bool flipped = xo[7] != yl[7];
        if (sproj != xo[7]) {
            double flipprob = 0.5 * (1 - yl[7] * sproj);
            noflip *= 1. - flipprob;
            if (R.flipspin) {
                double prev = yl[7];
                yl[7] = u01() < 0.5 * (sproj + 1) ? 1 : -1;
                if (yl[7] != prev) ++nspinflip;
            }
            if (R.flipspin && flipped) yl[7] *= -1;
        } else if (flipped) {
            for (int k = 0; k < 5; ++k) spin[k] = 0;
        }
        if (R.log.track) log_track(xo[8], x, yl);
        if (stop == PT_ID_UNKNOWN && yl[6] >= tau) stop = PT_ID_DECAYED;
        else if (stop == PT_ID_UNKNOWN && (x >= R.simtime || yl[8] >= R.lmax)) stop = PT_ID_NOT_FINISH;
        /* After a reset the stepper restarts from the loop's (x, y) with a fresh
         * derivative (stepper.initialize); otherwise it continues from its own
         * state (so a polarisation change by DoPolarize without a reset does
         * not reach the stepper, as in the reference); a stopped particle
         * reports the loop's (x, y). */
        if (reset || stop != PT_ID_UNKNOWN) {
            t = x;
            for (int i = 0; i < 9; ++i) y[i] = yl[i];
            if (stop == PT_ID_UNKNOWN) derivs(y, t, dydt);
        } else {
            t = tn;
            for (int i = 0; i < 9; ++i) { y[i] = yn[i]; dydt[i] = dyn[i]; }
        }
        flags |= PT_F_DERIV;
    }

    /* The common case of post_step decided up front: no decay/tmax clipping,
     * no chord split, the chord inside the geometry box and no collision on
     * it.  Then CheckHit reduces to DoStep and the sequence below is exactly
     * what post_step would execute.  Returns false (nothing changed) when the
     * step needs the full post_step. */
    __device__ bool fast_post() {
        bool finite = isfinite(tn);
        for (int i = 0; i < 9; ++i) finite = finite && isfinite(yn[i]);
        if (!finite) return false;
        if (tau > 0 && yn[6] > tau) return false;
        if (tn > R.simtime) return false;
        double l2 = (yn[8] - xo[8]) * (yn[8] - xo[8]);
        double d2 = (yn[0] - xo[0]) * (yn[0] - xo[0]) + (yn[1] - xo[1]) * (yn[1] - xo[1]) + (yn[2] - xo[2]) * (yn[2] - xo[2]);
        if (0.25 * (l2 - d2) > PT_MAX_TRACK_DEVIATION * PT_MAX_TRACK_DEVIATION) return false;
        if (!(to < tn)) return false;
        if (!check_segment(S, xo, yn)) return false;
        int cs = cur_solid();
        const DMat &m = S.mats[S.solids[cs].mat];
        if (R.sp.kind == PT_NEUTRON ? (m.fermi_imag > 0) : (S.solids[cs].id > 1)) return false; /* OnStep may act */
        if (any_hit(xo, yn) != 0) return false;
        if (spin_integrates(tn, yn)) return false; /* the Bloch integration runs in the full post-step */
        if (R.log.snap && snapshot_due(tn)) return false; /* a snapshot needs the try's stages, which the full post-step loads */
        double x2 = tn, y2[9];
        for (int i = 0; i < 9; ++i) y2[i] = yn[i];
        do_step(to, xo, x2, y2, cs); /* cannot alter the step here */
        finish_step<false>(tn, y2, false);
        return true;
    }

    /* One iteration of LOOP A (src/tracking.cpp:71-148) for the plain form. */
    __device__ void step() {
        int r;
        do { r = rk_try(); } while (r == 0);
        if (r < 0) { stop = PT_ID_ODEINT_ERROR; return; }
        post_step();
    }

    /* interpolatefields: the precession axis of the pending Bloch
     * integration as cubic splines over its trajectory step (times om_t,
     * per component and interval the coefficients of
     * c0 + u (c1 + u (c2 + u c3)), u = t - om_t[interval]) */
    bool om_on;
    double om_t[PT_OM_POINTS + 1], om_c[3][PT_OM_POINTS][4];
};

using Lane = LaneT<NoTape>;

} // namespace ptd
