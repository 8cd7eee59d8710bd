/*
 * pt_device.cuh -- device-side data layout and per-particle physics of the
 * GB300 tracking engine (sm_103a).
 *
 * One lane tracks one particle.  The per-lane step is the reference's LOOP A
 * body (src/tracking.cpp:71-148): an error-controlled Dormand-Prince 5(4)
 * step, decay/tmax clipping on the dense output, chord splitting to 1 mm,
 * the segment-mesh test with bisection to 1e-8 m, the solid-stack update and
 * the particle's wall/bulk physics.  All state arithmetic, step control and
 * the narrow-phase triangle test are FP64; the broad phase of the mesh query
 * runs on conservatively rounded FP32 boxes; the tricubic field can run in
 * FP64 or FP32 (PT_PREC_*).
 */
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>
#include "../../include/pentrack_gpu.h"
#include "../../include/pt_constants.h"

#define PT_MAX_STACK 8        /* entries of the current-solids list (the reference's vector is unbounded) */
#define PT_MAX_COLLS 8        /* collisions of one segment kept for DoHit */
#define PT_MAX_FIELDS 8
#define PT_T2_NCOMP 7       /* components of a 2D table node: B_r, B_phi, B_z, V, E_r, E_phi, E_z */
#define PT_MAX_SPINTIMES 16
#define PT_MAX_IGNORE 4       /* ignore intervals per solid */
#define PT_MAX_SOLIDS 64
#define PT_MAX_TRIES 500      /* odeint failed_step_checker */
#define PT_MAX_BISECT_WORK 4096 /* collision queries per bisection (the reference recurses without a bound) */
#define PT_MAX_BISECT_LEVELS 100
#define PT_MAX_LAMBERT 10000
#define PT_MAX_SUBSEGMENTS (1 << 20) /* chord pieces of one RK step */
#define PT_MAX_HITS_PER_SEGMENT 64   /* surfaces crossed by one chord piece */
#define PT_MAX_CAND 48               /* candidate triangles kept for a bisection */
#define PT_MAX_SPIN_STEPS (1 << 22)  /* spin (Bloch) steps within one trajectory step */

/* lane flags */
#define PT_F_DERIV 1u   /* FSAL derivative valid */
#define PT_F_RESET 2u   /* re-initialise the stepper before the next step */
#define PT_F_INIT 4u    /* initialised (tau sampled, solids found, Hmax set) */

struct DTri {           /* one triangle, 112 B */
    double a[3], b[3], c[3], n[3];
    int solid;
    int pad;
};

struct DTri32 {         /* FP32 copy of a triangle for certified pre-tests, 64 B */
    float a[3], b[3], c[3]; /* vertices rounded to nearest */
    float n[3];             /* unit normal */
    float m;                /* max |coordinate| of the FP64 vertices, rounded up */
    float pad[3];
};

struct DTriC {          /* data of the certified FP64 pre-test (seg_tri64c), 96 B */
    double n[3];        /* (b - a) x (c - a) evaluated in FP64 */
    float dn;           /* bound on |n - exact| per component */
    float n1;           /* |n|_1, rounded up */
    float ea;           /* max(|b - a|_inf, |c - a|_inf), rounded up */
    int edges;          /* edge k (a-b, b-c, c-a): bits 2k..2k+1 = index of its lexicographically larger vertex v, bit 6+k = swapped */
    float e[3][3];      /* edge k in canonical order: u - v (u lexicographically smaller), rounded to FP32 */
    float en[3];        /* |u - v|_inf, rounded up */
    float pad[2];
};

struct DNode {          /* flattened BVH node in depth-first order, 32 B */
    float lo[3], hi[3];
    int skip;           /* next node when this subtree is skipped */
    int leaf;           /* -1 for inner nodes, else first_triangle*8 + count */
};

struct DSolid {
    uint32_t id;
    int mat;
    int n_ign;
    int pad;
    double ign[2 * PT_MAX_IGNORE];
    double lo[3], hi[3]; /* box of this solid's triangles (lo > hi: none) */
};

struct DMat {
    double fermi_real, fermi_imag, diff, spinflip, ibf, modlambert, loss;
    double rms, corr; /* MicroRoughness: RMS roughness and correlation length [m] */
};

struct DField {
    int type;
    int ncomp;          /* Hermite components per node: 3 (B) or 4 (B and V) */
    int has_b, has_v;
    double bscale, escale;
    double xmax, xmin, ymax, ymin, zmax, zmin, bw;
    int n[3];
    int pad0;
    const double *ax[3];
    double a0[3], inv_h[3];
    const double *node64;  /* [node][comp][8]: f, fx, fy, fz, fxy, fxz, fyz, fxyz */
    /* FP32 node table of the FP32 field mode: per node, for each component,
     * the value split into FP32 high and low parts and the seven derivative
     * values (fx, fy, fz, fxy, fxz, fyz, fxyz); node32_stride floats per node */
    const float *node32;
    int node32_stride;
    int pad2;
    const double *inv_w[3]; /* 1 / cell width per axis interval */
    const float *ax32[3];   /* FP32 copies of the axes and widths for the FP32 field mode */
    const float *inv_w32[3];
    float a0f[3], inv_hf[3];
    double e[3];
    /* harmonic polynomial: Phi = sum c * x^i y^j z^k, B = grad Phi */
    int n_mono;
    int pad1;
    const double *mono_c;  /* coefficient of each monomial */
    const int *mono_e;     /* packed exponents i | j<<4 | k<<8 */
    double offset[3];      /* harmonic: added to the coordinates; solenoid: its centre */
    /* harmonic: B and its Jacobian as polynomials over the monomials
     * x^a y^b z^c of total degree <= hp_deg in graded order (hp_e packed
     * a | b << 4 | c << 8): hp_c holds 9 rows of hp_n coefficients, B_x,
     * B_y, B_z, then dB_xx, dB_xy, dB_xz, dB_yy, dB_yz, dB_zz, which use the
     * first hp_n1 monomials (degree <= hp_deg - 1) */
    int hp_deg, hp_n, hp_n1, pad4;
    const double *hp_c;
    const int *hp_e;
    /* harmonic: the potential of each coefficient with G = 1 (the basis
     * fields dB/dG_k the adjoint uses), terms term_start[k] .. term_start[k+1]-1 */
    int n_terms;
    int pad3;
    const int *term_start;
    const double *basis_c;
    const int *basis_e;
    /* the basis fields themselves as polynomials over the hp monomials:
     * n_terms x 3 rows of hp_n coefficients (b_k,x, b_k,y, b_k,z) */
    const double *basis_hp;
    double sol_a, sol_b, sol_B0; /* solenoid radius, half length, mu0 n I / pi */
    /* 2D table (TabField): r axis in ax[0] / n[0], z axis in ax[2] / n[2];
     * node64 holds [ir][iz][component][4] = f, df/dr, df/dz, d2f/drdz of
     * the components B_r, B_phi, B_z, V, E_r, E_phi, E_z (t2_mask bit c set
     * when component c is tabulated); t2_lim = r_lo, r_hi, z_lo, z_hi of the
     * half-open range test */
    int t2_mask, pad5;
    double t2_lim[4];
};

struct DScene {
    int n_tris, n_nodes, n_solids, n_fields, n_mats;
    int pad;
    const DTri *tris;
    const DTri32 *tri32;
    const DTriC *tric;
    const DNode *nodes;
    const DSolid *solids;
    const DMat *mats;
    DField fields[PT_MAX_FIELDS];
    double mesh_zmax;
};

struct DSpecies {
    int kind;
    int pad;
    double q, m, mu, gamma, inv_mkg, fgrav, mu_over_e, q_over_e, mc2, mg;
    float muf;          /* mu rounded to FP32 (FP32 field mode) */
    float pad2;
};

/* event-log buffers (null when the log is off): records appended at an
 * atomic count; counts past the capacity are kept, records dropped */
struct DLog {
    double *hit, *snap, *track, *spin;
    unsigned long long *hit_n, *snap_n, *track_n, *spin_n;
    long long cap;
    const double *snap_t;
    int n_snap, pad;
    double track_interval, spin_interval;
};

struct DRun {
    DSpecies sp;
    DLog log;
    double simtime, tau, tmax, lmax, bmax;
    double spintimes[PT_MAX_SPINTIMES];
    int n_spintimes, flipspin, prec, steps_per_launch;
    int mode, max_steps;      /* max_steps: accepted RK steps per particle in one advance call (0 = no limit) */
    int interp, pad_i;        /* interpolatefields: spline of the precession axis per trajectory step */
    uint64_t seed;
    double t_pause;
    volatile int *cancel;   /* host-mapped cancel word (the reference's quit flag) */
};

/* particle batch in device memory (structure of arrays, component-major) */
struct DBatch {
    int64_t n;
    int64_t *id;
    double *t, *y, *dydt, *dt, *spin, *tau, *hmax, *noflip, *hstart, *t_last;
    int32_t *stop_id, *nhit, *nstep, *nspinflip, *nsol;
    uint32_t *flags;
    uint64_t *stack;    /* up to 8 entries: byte k = solid index (6 bits) | ignored << 7 */
    uint64_t *rng_n;
    int64_t *nacc, *nrej;
    int32_t *ntry;
    int64_t *nacc0;              /* accepted steps at the start of the current advance call */
    /* phase-split form: result of the last accepted try and B-value caches */
    double *yn, *dyn, *kst, *tn; /* yn, dyn: 9n; kst: k3..k6, 36n; tn: n */
    double *bc;                  /* 2 slots x (x, y, z, t, Bx, By, Bz): 14n */
    /* suspended post-steps: 45 doubles and 7 + PT_MAX_CAND ints per particle */
    double *ps_d;
    int32_t *ps_i;
    /* work lists of particle indices and their counts */
    int32_t *list[5];            /* 0/1: active (ping-pong), 2: post, 3: slow, 4: bisection */
    int32_t *count;              /* counts of the lists */
    struct DSched *sched;        /* scheduler state of the persistent batched form */
};

#define PT_F_BC0 8u   /* cache slot 0 valid */
#define PT_F_BC1 16u  /* cache slot 1 valid */
#define PT_F_PENDING 32u /* an accepted try waits for the full post-step logic */
#define PT_F_SUSPENDED 64u /* that post-step is suspended at a bisection (state in ps_d/ps_i) */

/* Device-side state of the batched form's scheduler (one per batch): loop
 * counts, the period's iteration cap and tail threshold, and the device time
 * of the timed kernels (k_run, k_slow, k_bisect) measured on %globaltimer
 * inside the CUDA graph, where no event can be recorded. */
enum { PT_SPAN_RUN = 0, PT_SPAN_SLOW = 1, PT_SPAN_BISECT = 2, PT_SPAN_TRY = 3, PT_SPAN_POST = 4, PT_SPANS = 5 };
/* Slow rounds of one scheduler iteration before the device loop gives up
 * with an error (every post-step completes after a bounded number of rounds:
 * bisections and chord pieces are bounded, see PT_MAX_*; the cap keeps a
 * logic error from looping on the device). */
#define PT_MAX_SLOW_ROUNDS (1 << 16)
struct DSched {
    int outer_iters, inner_iters, period_start, max_iters;
    int tail, last_going, last_active, inner_this; /* inner_this: slow rounds of the current iteration */
    int error, last_slow;                           /* error: the slow-round cap was reached; post-steps left queued */
    unsigned long long t0[PT_SPANS], t1[PT_SPANS], ns[PT_SPANS], launches[PT_SPANS];
};

/* Device buffers of one pt_adjoint call (per particle i: segment records
 * at seg + i cap_seg SEG_DOUBLES, Bloch checkpoints at ck + i cap_ck
 * CK_DOUBLES, one chunk tape of K steps at tape + i K STEP_DOUBLES) */
struct DAdj {
    double *seg, *ck, *tape;
    int cap_seg, cap_ck, K, field, ncoef, pad;
    int *nseg, *nck, *status;
    const double *dl_dspin, *dl_dy; /* 5n, 9n component-major (dl_dy may be null) */
    double *dl_dg;                  /* ncoef x n */
};

/* a volume source on the device (pt_source_params, checked on the host) */
struct DSourceSpec {
    int shape, solid, phase_space, max_rounds;
    uint64_t seed;
    double lo[3], hi[3];
    double rmin, rmax, phimin, phimax, zmin, zmax;
    double emin, emax, polarization, tmin, tmax;
    double thetamin, thetamax, phimin_v, phimax_v;
    double enormal;
    /* surface sources: the candidate triangles (9 doubles each, the scene's
     * order) and their cumulative areas */
    const double *surf_tri, *surf_cum;
    int n_surf, pad;
    const DScene *region; /* STL surface source: the region's scene (solid index 1), device copy */
};

/* device event counters (one set per launch, summed with atomics per block) */
struct DCounters {
    unsigned long long rk_accepted, rk_rejected, rhs_evals, field_evals, hits, bisection_levels;
    unsigned long long bvh_nodes, tri_tests, subsegments, dense_evals, active, paused;
    double particle_seconds;
    unsigned int bisect_max;
    unsigned long long cand_calls, cand_overflow, cand_sum, tri32, bisect_dead, spin_steps;
};
