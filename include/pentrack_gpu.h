/*
 * pentrack_gpu.h -- C ABI of the GB300 particle-tracking engine.
 *
 * Drop-in for PENTrack's per-particle hot path
 *   TTracker::IntegrateParticle            (include/tracking.h:46-47, src/tracking.cpp:17-173)
 * together with the collaborators it calls on every step
 *   TFieldManager::BField / EField          (include/fields.h:46,61; src/fields.cpp:139-182)
 *   TGeometry::CheckSegment / GetCollisions (include/geometry.h:104-155; src/geometry.cpp:139-175)
 *   TNeutron::OnHit / OnStep, TProton/TElectron::OnStep (src/neutron.cpp:187-282,
 *                                            src/proton.cpp:25-33, src/electron.cpp:25-32)
 *
 * The reference keeps its scene in private members (TGeometry::solids,
 * TTriangleMesh::meshes, TFieldManager::fields), so the engine is built from
 * the same raw inputs those classes read from config.in: triangles of the STL
 * files, the [MATERIALS]/[GEOMETRY] tables and the [FIELDS] lines.  The C++
 * host layer (pentrack_gb300/csrc/pt_host.hpp) fills these structs from a
 * config.in exactly like TGeometry(TConfig&) and TFieldManager(TConfig&).
 *
 * Conventions: only C types cross the boundary; the caller owns every array
 * it passes and no pointer to caller memory is kept after a call returns;
 * a context owns all device memory; calls on one context come from one host
 * thread.  Errors never throw across the ABI: every entry returns pt_status.
 * Per-particle outcomes use the reference's stopID integers.
 */
#ifndef PENTRACK_GPU_H
#define PENTRACK_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the reference throws std::runtime_error instead) ---- */
typedef int32_t pt_status;
enum {
    PT_OK = 0,
    PT_ERR_INVALID = -1,      /* invalid scene / parameters (reference: runtime_error at setup) */
    PT_ERR_UNSUPPORTED = -2,  /* field type or option the device path does not implement */
    PT_ERR_OOM = -3,
    PT_ERR_CUDA = -4,
    PT_ERR_TIMEOUT = -5,
    PT_ERR_CANCELLED = -6,    /* pt_cancel() was called: partial results are valid */
    PT_ERR_IO = -7,
    PT_ERR_NO_DEVICE = -8
};

/* ---- per-particle stop IDs: identical integers to include/globals.h:13-23 ---- */
enum {
    PT_ID_UNKNOWN = 0,
    PT_ID_NOT_FINISH = -1,
    PT_ID_HIT_BOUNDARIES = -2,
    PT_ID_ODEINT_ERROR = -3,
    PT_ID_DECAYED = -4,
    PT_ID_INITIAL_NOT_FOUND = -5,
    PT_ID_CGAL_ERROR = -6,
    PT_ID_GEOMETRY_ERROR = -7,
    PT_ID_ABSORBED_IN_MATERIAL = 1,
    PT_ID_ABSORBED_ON_SURFACE = 2
};

/* particle species (src/neutron.cpp:15, src/proton.cpp, src/electron.cpp) */
enum { PT_NEUTRON = 0, PT_PROTON = 1, PT_ELECTRON = 2 };

/* field kinds the device path implements (src/fields.cpp:31-130) */
enum {
    PT_FIELD_TAB3D = 1,     /* OPERA3D / 3Dtable / COMSOL: TabField3, tricubic  (src/field_3d.cpp:417-529) */
    PT_FIELD_HARMONIC = 2,  /* HarmonicExpansionBField, l <= 5        (src/harmonicfields.cpp:50-829) */
    PT_FIELD_UNIFORM_E = 3, /* EDMStaticEField                        (src/edmfields.cpp:181-187) */
    PT_FIELD_SOLENOID = 4,  /* finite ideal solenoid along z, closed form (no reference counterpart:
                               the reference approximates it with Conductor segments, src/conductor.cpp) */
    PT_FIELD_TAB2D = 5      /* OPERA2D / 2Dtable: TabField, bicubic in (r, z)  (src/field_2d.cpp:232-399) */
};

/* scheduling form of the tracking kernels */
enum {
    PT_MODE_PLAIN = 0,   /* fixed step-batch launches: one lane per particle, K accepted steps per launch */
    PT_MODE_BATCHED = 1, /* the loop is a CUDA graph whose iterations the device schedules; each iteration
                            runs the steps without hits either as a phase split (k_try + k_post over work
                            lists) or in persistent lanes refilled from a device work queue (k_run), hit
                            resolution in work-list launches (k_slow, k_bisect); pt_run_params.scheduler */
    PT_MODE_PHASED = 2   /* host-driven phase split: one RK-try launch and one completion launch per
                            iteration over work lists, the host reading the list counts in between */
};

/* arithmetic of the field evaluation (the state update, step control and
 * narrow-phase intersection are always FP64) */
enum { PT_PREC_FP64 = 0, PT_PREC_FP32 = 1 };

/* material: the nine columns of materials.in, in order (src/geometry.cpp:10-52).
 * Units as in the file: neV, neV, probability, probability, m, m, T, probability, probability. */
typedef struct pt_material {
    double fermi_real;
    double fermi_imag;
    double diff_prob;
    double spinflip_prob;
    double rms_roughness;     /* MicroRoughness (src/microroughness.cpp): RMS roughness; with correl_length > 0 */
    double correl_length;     /* the model applies where MRValid holds (src/neutron.cpp:203) */
    double internal_bfield;
    double modified_lambert_prob;
    double loss_per_bounce;
} pt_material;

/* solid: one [GEOMETRY] line (include/geometry.h:40-68).  solids[0] must be the
 * default solid (ID 1), which owns no triangles. */
typedef struct pt_solid {
    uint32_t id;               /* priority: higher ID wins */
    int32_t material;          /* index into pt_scene_desc.materials */
    int32_t n_ignore;          /* number of [start,end) ignore intervals */
    int32_t reserved;
    const double *ignore_times; /* 2*n_ignore values: start0, end0, start1, end1, ... */
} pt_solid;

/* one [FIELDS] entry wrapped in its TFieldContainer (include/field.h:268-281):
 * constant B/E scale factors, box [min,max) and smooth boundary width. */
typedef struct pt_field {
    int32_t type;
    int32_t reserved0;
    double b_scale;             /* TFieldScaler restricted to a constant; 0 switches B off */
    double e_scale;             /* likewise for E/V */
    double xmax, xmin, ymax, ymin, zmax, zmin; /* box; xmax<=xmin etc. means "no box" */
    double boundary_width;
    /* PT_FIELD_TAB3D: rectilinear grid of raw samples in SI units (m, T, V) */
    int32_t nx, ny, nz, reserved1;
    const double *x, *y, *z;   /* sorted, unique axis coordinates */
    const double *bx, *by, *bz, *v; /* [ix][iy][iz] row-major (iz fastest); NULL = component absent */
    /* PT_FIELD_HARMONIC */
    double offset[3];
    int32_t n_coeff, reserved2;
    const int32_t *l, *m;
    const double *g;
    /* PT_FIELD_UNIFORM_E: E [V/m]; potential V = e[2]*z as in src/edmfields.cpp:186 */
    double e[3];
    /* PT_FIELD_SOLENOID: centre = offset, radius [m], half length [m] and the
     * field at the centre [T] of a sheet current on the cylinder */
    double sol_radius, sol_half_length, sol_bcenter;
    /* PT_FIELD_TAB2D (rotationally symmetric about z): nx radii r >= 0 in x,
     * nz heights in z (ny, y unused), samples [ir][iz] (iz fastest) in bx
     * (B_r), by (B_phi), bz (B_z), v (V) and in er, ephi, ez (E_r, E_phi,
     * E_z, which take precedence over v as in src/field_2d.cpp:262-283);
     * NULL = column absent */
    const double *er, *ephi, *ez;
} pt_field;

typedef struct pt_scene_desc {
    int64_t n_triangles;
    const double *triangles;      /* 9 doubles per triangle: v0, v1, v2 [m] in STL winding (normal = (v1-v0)x(v2-v0)) */
    const int32_t *triangle_solid;/* index into solids[] for every triangle */
    int32_t n_solids;
    int32_t n_materials;
    const pt_solid *solids;
    const pt_material *materials;
    int32_t n_fields;
    int32_t reserved;
    const pt_field *fields;
} pt_scene_desc;

/* run parameters: the [GLOBAL] simtime plus the particle's [PARTICLES]/species
 * options read by TTracker::IntegrateParticle (src/tracking.cpp:19-60). */
typedef struct pt_run_params {
    int32_t species;
    int32_t mode;              /* PT_MODE_* */
    int32_t field_precision;   /* PT_PREC_* */
    int32_t flipspin;          /* particle option flipspin */
    double simtime;            /* lab-time limit: reaching it gives ID_NOT_FINISH */
    double tau;                /* mean lifetime [s]; >0: proper-time limit ~ Exp(1/tau) */
    double tmax;               /* proper-time limit used when tau == 0 (reaching it gives ID_DECAYED) */
    double lmax;               /* trajectory-length limit */
    double bmax;               /* spin option Bmax [T] */
    int32_t n_spintimes;       /* number of doubles in spintimes (pairs of [start,end)) */
    int32_t steps_per_launch;  /* plain form: accepted RK steps per lane per launch (0 = default) */
    const double *spintimes;
    uint64_t seed;             /* Philox4x32-10 key; stream counter keyed by particle id */
    int32_t block_size;        /* 0 = autotuned */
    int32_t max_launches;      /* 0 = unlimited */
    double timeout_s;          /* host wait limit per call (0 = none) */
    int32_t max_run;           /* batched form, persistent scheduler: consecutive steps a lane keeps one particle
                                  (0 = step budget only) */
    int32_t period_iters;      /* batched form: scheduler iterations per graph launch (0 = 64) */
    int32_t scheduler;         /* batched form: PT_SCHED_* (PT_SCHED_AUTO: measured on the batch's first periods) */
    int32_t reserved3;
    /* event logs (TLogger::PrintHit / PrintSnapshot, src/logger.cpp:128-235):
     * hitlog: one record per wall hit that changes the particle's solid (after
     * its OnHit); snapshotlog: at the first of the snapshot times in each
     * trajectory step's [start, end), the dense-output state.  Records are read
     * with pt_log_read after the call (pt_integrate) or the advances
     * (pt_batch_*, collected from pt_batch_create on). */
    int32_t hitlog, snapshotlog;
    const double *snapshots;   /* snapshot times [s] (snapshotlog) */
    int32_t n_snapshots;       /* at most PT_MAX_SNAPSHOTS */
    int32_t reserved4;
    int64_t log_capacity;      /* records kept per log (0: 1,000,000); later events are counted, not kept */
    /* tracklog: a record at the particle's start (zero path length) and after
     * every trajectory step whose path length crosses a multiple of
     * trackloginterval (TLogger::PrintTrack, src/logger.cpp:143-200) */
    int32_t tracklog, reserved5;
    double trackloginterval;   /* [m] */
    /* spinlog: a record at the start of each Bloch integration and after every
     * Bloch step whose time crossed a multiple of spinloginterval
     * (TLogger::PrintSpin, src/logger.cpp:237-284) */
    int32_t spinlog, reserved6;
    double spinloginterval;    /* [s] */
    /* interpolatefields 1 (TTracker::IntegrateSpin, src/tracking.cpp:404-421):
     * the Bloch integration of a trajectory step takes the precession axis
     * from cubic splines through its values at 11 equally spaced times of the
     * step instead of evaluating it at every stage */
    int32_t interpolatefields, reserved7;
} pt_run_params;

enum { PT_LOG_HIT = 0, PT_LOG_SNAPSHOT = 1, PT_LOG_TRACK = 2, PT_LOG_SPIN = 3 };
#define PT_MAX_SNAPSHOTS 1024
/* hit record: particle, t, x, y, z, v1x, v1y, v1z, pol1, v2x, v2y, v2z, pol2,
 * nx, ny, nz, solid1 (leaving), solid2 (entering) -- the reference's hit-log
 * columns after jobnumber */
#define PT_HIT_RECORD 18
/* snapshot record: particle, t, y[9] (x, y, z, vx, vy, vz, proper time,
 * polarisation, path length), spin[5], stopID, Nspinflip, no-flip
 * probability, Nhit, Nstep, Hmax -- what TLogger::Print needs besides the
 * particle's start and the fields */
#define PT_SNAPSHOT_RECORD 22
/* track record: particle, t, x, y, z, vx, vy, vz, polarisation, ID of the
 * current solid (the fields, energies and potential of the track log's
 * columns follow from these) */
#define PT_TRACK_RECORD 10
/* spin record: particle, t, x, y, z, Sx, Sy, Sz, Wx, Wy, Wz, Bx, By, Bz (the
 * reference's spin-log columns after jobnumber) */
#define PT_SPIN_RECORD 14

/* schedulers of the batched form (results are the same bits with each) */
enum { PT_SCHED_AUTO = 0, PT_SCHED_PHASED = 1, PT_SCHED_PERSISTENT = 2, PT_SCHED_PERSISTENT_WIDE = 3, PT_SCHED_PHASED_WIDE = 4 };

/* structure-of-arrays particle batch (host memory).  y and spin are
 * component-major: y[c*n + i] is component c of particle i.
 * y = (x, y, z, vx, vy, vz, proper time, polarisation, path length)  include/particle.h:21
 * spin = (Sx, Sy, Sz, integrated time, integrated phase)               include/particle.h:22 */
typedef struct pt_particles {
    int64_t n;
    int64_t *id;       /* particle number: keys the random stream */
    double *t;
    double *y;         /* 9*n */
    double *spin;      /* 5*n */
    /* written by the engine (may be NULL on input): */
    int32_t *stop_id;
    int32_t *solid;    /* ID of the highest-priority solid the particle is in */
    int32_t *n_hit;
    int32_t *n_step;   /* sub-segments, as TParticle::Nstep (src/particle.cpp:205) */
    int32_t *n_spinflip;
    int32_t *reserved;
    double *h_max;     /* max total energy [eV] (src/particle.cpp:202) */
    double *noflip_prob;
    double *tau;       /* sampled proper-time limit */
    double *h_start;   /* initial total energy [eV] */
    int64_t *n_accepted; /* accepted RK steps */
    int64_t *n_rejected; /* rejected RK tries */
} pt_particles;

/* event counters and timings of one call */
typedef struct pt_stats {
    double kernel_ms;          /* device time of this call's tracking launches (CUDA events on the launch stream) */
    double span_ms;            /* device time from the call's first to its last event on the launch stream */
    double wall_ms;            /* host wall time of the call */
    double particle_seconds;   /* sum over particles of the lab time tracked in this call */
    int64_t launches;
    int64_t active;            /* particles not yet stopped after the call */
    int64_t rk_accepted, rk_rejected, rhs_evals, field_evals, hits, bisection_levels;
    int64_t bvh_nodes, tri_tests, subsegments, dense_evals;
    double dominant_kernel_ms; /* summed device time of the dominant kernel */
    int64_t dominant_launches;
    char dominant_kernel[48];
    double try_ms, post_ms, slow_ms; /* batched forms: device time per phase kernel (try_ms: k_run in the
                                        persistent form, k_try in the phased one) */
    int64_t bisect_max;        /* largest number of collision queries of one bisection */
    int64_t cand_calls, cand_overflow, cand_sum; /* candidate-triangle sets built for bisections */
    int64_t tri32_tests;       /* FP32 certified segment-triangle tests */
    double bisect_ms;          /* batched form: device time of the bisection kernel */
    int64_t bisect_dead;       /* bisection intervals abandoned because neither half collides */
    int64_t spin_steps;        /* accepted steps of the spin (Bloch) integration */
    double tail_ms;            /* batched form: device time of the plain-form tail launches */
    int64_t aux_launches;      /* bookkeeping kernel launches (work-list gathers, list-count resets) */
    int64_t graph_launches;    /* batched form: CUDA graph launches (periods) of the call */
    int64_t sched_outer_iters; /* batched form: scheduler iterations (k_run launches) */
    int64_t sched_inner_iters; /* batched form: slow rounds (k_slow + k_bisect launches) */
    double adj_forward_ms;     /* pt_adjoint: device time of the recording forward pass(es) */
    double adj_reverse_ms;     /* pt_adjoint: device time of the reverse sweep */
    int64_t scheduler;         /* batched form: the scheduler that ran (PT_SCHED_*; 0 while still tuning) */
    double tune_ns_per_try[4]; /* batched form: the autotuner's device ns per RK try of each scheduler, PT_SCHED_* - 1 (0 = untried) */
} pt_stats;

typedef struct pt_ctx pt_ctx;
typedef struct pt_batch pt_batch;

/* Build the device scene (BVH, Hermite field tables, materials) on CUDA device
 * `device`.  Replaces TGeometry(TConfig&) (src/geometry.cpp:93-137) and
 * TFieldManager(TConfig&) (src/fields.cpp:19-136) as far as the hot path needs. */
pt_status pt_create(const pt_scene_desc *scene, int32_t device, pt_ctx **out);
void pt_destroy(pt_ctx *ctx);
/* Text of the last error on this context (or of the last failed pt_create when ctx is NULL). */
const char *pt_last_error(const pt_ctx *ctx);
/* Ask running kernels to stop at the next step boundary (the reference's quit
 * flag, include/globals.h:33, polled at src/tracking.cpp:97). */
pt_status pt_cancel(pt_ctx *ctx);

/* One-shot drop-in for a loop of TTracker::IntegrateParticle calls
 * (src/main.cpp:152-172): host arrays in, host arrays out, all particles
 * tracked to their stop ID. */
pt_status pt_integrate(pt_ctx *ctx, const pt_run_params *params, const pt_particles *in,
                       pt_particles *out, pt_stats *stats);

/* Device-resident batch: upload once, advance in windows, read back. */
pt_status pt_batch_create(pt_ctx *ctx, const pt_run_params *params, const pt_particles *in, pt_batch **out);
/* Advance every live particle until it stops or, at a step boundary, its lab
 * time reaches t_pause (resuming later is bit-identical to never pausing). */
pt_status pt_batch_advance(pt_ctx *ctx, pt_batch *batch, double t_pause, pt_stats *stats);
/* As pt_batch_advance, but each particle also pauses after max_steps accepted
 * RK steps in this call (one fixed step-batch of the plain form; 0 = no limit). */
pt_status pt_batch_advance_steps(pt_ctx *ctx, pt_batch *batch, double t_pause, int32_t max_steps, pt_stats *stats);
pt_status pt_batch_read(pt_ctx *ctx, pt_batch *batch, pt_particles *out);
/* The records of log `kind` (PT_LOG_HIT, PT_LOG_SNAPSHOT, PT_LOG_TRACK, PT_LOG_SPIN) collected by the
 * last pt_integrate call or since the last pt_batch_create: *total receives the
 * number of events, up to `cap` records (of PT_HIT_RECORD / PT_SNAPSHOT_RECORD /
 * PT_TRACK_RECORD / PT_SPIN_RECORD doubles, in no particular order) are copied to `rec` (may be NULL with
 * cap = 0 to ask for the count). */
pt_status pt_log_read(pt_ctx *ctx, int32_t kind, int64_t cap, double *rec, int64_t *total);
void pt_batch_destroy(pt_batch *batch);

/* Field of the whole scene at n points (x,y,z,t interleaved, 4n doubles):
 * TFieldManager::BField and EField.  Any output may be NULL; B is evaluated
 * with its gradient when dB is given and without (the value-only path, e.g.
 * spline2dcalc for 2D tables) when dB is NULL. */
pt_status pt_field_eval(pt_ctx *ctx, int64_t n, const double *xyzt, int32_t precision,
                        double *B, double *dBidxj, double *V, double *E);

/* All segment-mesh collisions of n segments (p1, p2: 6 doubles each), sorted by
 * (s ascending, solid ID descending) as TTriangleMesh::Collision
 * (src/trianglemesh.cpp:134-164).  For segment i, count[i] hits are written to
 * s/normal(3)/solid_id/distnormal at offsets i*max_hits.. ; count[i] = -1 on a
 * coplanar (CGAL error) case. */
pt_status pt_segment_collisions(pt_ctx *ctx, int64_t n, const double *seg, int32_t max_hits,
                                int32_t *count, double *s, double *normal, int32_t *solid_id,
                                double *distnormal);

/* pt_segment_collisions without any device allocation: no counterpart in the
 * reference (an addition for callers that must not allocate device memory
 * per call).  Same arguments, results and
 * errors as pt_segment_collisions; device scratch is a fixed 8 MiB array in
 * the library's module, addressed with cudaGetSymbolAddress (that device
 * current) on the first call after each pt_create on the device, so make that
 * first call before any stream capture.  A cudaDeviceReset invalidates every
 * context on the device (their scene memory) and with them that address:
 * create a new context before calling again.  Scratch needed: 48 n + 4 n + 44 n max_hits bytes plus
 * 256-byte alignment per block; larger requests return PT_ERR_INVALID with the
 * sizes in pt_last_error (n = 16384, max_hits = 8 fits).  Not reentrant: every
 * context on a device shares the one scratch array, so calls on the same
 * device must not overlap. */
pt_status pt_segment_collisions_noalloc(pt_ctx *ctx, int64_t n, const double *seg, int32_t max_hits,
                                        int32_t *count, double *s, double *normal, int32_t *solid_id,
                                        double *distnormal);

/* Gradient of a scalar loss L of the particles' end states with respect to
 * the coefficients G_k of harmonic field `field` of the scene: the adjoint
 * (reverse mode) of the whole tracking path of TTracker::IntegrateParticle
 * with IntegrateSpin (src/tracking.cpp:17-173, 373-483), taken pathwise
 * along each particle's fixed sequence of specular hits (TNeutron::Reflect,
 * src/neutron.cpp:99-115): the Dormand-Prince trajectory steps with their
 * dense output, the reflection map, and the Bloch integration of the spin
 * (SpinDerivs / SpinPrecessionAxis, src/particle.cpp:141-193) in the
 * harmonic field (src/harmonicfields.cpp:50-829), with every accepted step
 * size and bisection bracket frozen (the derivative of the discrete map).
 * The call runs the forward pass (its end states go to `out` when not
 * NULL), recording every trajectory step and a Bloch checkpoint every
 * `checkpoint_interval` accepted spin steps, then the reverse sweep, which
 * recomputes each chunk of checkpoint_interval spin steps from its
 * checkpoint.  dL_dspin (5n, component-major like pt_particles.spin) and
 * dL_dy (9n like pt_particles.y, or NULL) are dL/d(end state) per particle;
 * dL_dG receives the field's n_coeff derivatives summed over particles.
 * Supported: neutrons, FP64 field mode, scenes of harmonic expansions and
 * uniform E fields without boxes, at most 16 coefficients, walls that
 * reflect specularly (a diffuse reflection or transmission on a path gives
 * PT_ERR_UNSUPPORTED).  No counterpart in the reference, which has no
 * derivatives. */
pt_status pt_adjoint(pt_ctx *ctx, const pt_run_params *params, const pt_particles *in, int32_t field, int32_t checkpoint_interval,
                     const double *dL_dspin, const double *dL_dy, double *dL_dG, pt_particles *out, pt_stats *stats);

/* IDs of solids containing each point by +z ray parity (TTriangleMesh::GetSolids,
 * include/trianglemesh.h:181-188) as a bit mask over scene solid indices. */
pt_status pt_point_solids(pt_ctx *ctx, int64_t n, const double *p, uint64_t *mask);

/* ---- volume particle sources on the device ----
 * TVolumeSource::CreateParticle (src/source.cpp:102-194) for the cuboid,
 * cylindrical and STL volumes (TCuboidVolumeSource, TCylindricalVolumeSource,
 * TSTLVolumeSource: include/source.h:186-331), with or without
 * PhaseSpaceWeighting, with a flat energy spectrum, the azimuth uniform and
 * the polar angle sine-distributed, the start time uniform. */
enum { PT_SOURCE_BOX = 0, PT_SOURCE_CYLINDER = 1, PT_SOURCE_SOLID = 2, PT_SOURCE_SURFACE_CYLINDER = 3, PT_SOURCE_SURFACE_STL = 4 };
typedef struct pt_source_params {
    int32_t species;
    int32_t shape;             /* PT_SOURCE_* */
    uint64_t seed;             /* keys every particle's stream with its id */
    double lo[3], hi[3];       /* BOX: the box; SOLID: the box points are proposed in (the STL's bounding box) */
    double rmin, rmax, phimin, phimax, zmin, zmax; /* CYLINDER [m, rad] */
    int32_t solid;             /* SOLID: index (pt_scene_desc order) of the scene solid whose inside is the volume */
    int32_t phase_space;       /* PhaseSpaceWeighting: emin/emax bound the total energy H; a point with potential V
                                  is accepted with probability sqrt(H - V) / sqrt(H - Vmin), kinetic energy H - V */
    double emin, emax;         /* eV: kinetic energy (or total, phase_space) */
    double polarization;       /* probability of +1 is (1 + polarization) / 2 */
    double tmin, tmax;         /* start time, uniform */
    double thetamin, thetamax, phimin_v, phimax_v; /* velocity direction [rad] */
    int64_t n_min_samples;     /* phase_space: points for the minimum potential Vmin (0: 100,000) */
    int32_t max_rounds;        /* proposal rounds per particle (0: 100,000); STL points: 10,000 box proposals each */
    int32_t reserved;
    /* the cylindrical surface source (TSurfaceSource::CreateParticle,
     * src/source.cpp:102-131; TCylindricalSurfaceSource, include/source.h:
     * 255-283): a point on the scene's surfaces inside the cylinder's r, phi, z
     * ranges, moved 1e-8 m off the surface along the face normal, a
     * cos(theta) sin(theta) direction about the normal, the normal energy
     * raised by enormal [eV]. */
    double enormal;
    /* PT_SOURCE_SURFACE_STL (TSTLSurfaceSource, include/source.h:287-298):
     * the same on the scene's surfaces inside an STL that is not part of the
     * geometry, given as a context on the same device whose scene holds that
     * STL as solid index 1 (its triangles' box is the source box) */
    const struct pt_ctx *region;
} pt_source_params;

/* n particles with ids `ids` from the source: out->id, t, y (9n) and spin
 * (5n, zero) are written (host buffers); *vmin (may be NULL) receives the
 * minimum potential of a phase-space weighted source.  PT_ERR_INVALID when
 * the spectrum lies below that minimum or a particle's rounds run out. */
pt_status pt_source_volume(pt_ctx *ctx, const pt_source_params *sp, int64_t n, const int64_t *ids, pt_particles *out,
                           double *vmin);

/* MicroRoughness of n wall contacts with the kernels' own code (MR::MRDist,
 * MRProb, MRDistMax, src/microroughness.cpp:35-132; no entry point of the
 * reference): what 0 = MRDist at (theta[i], phi[i]) (with `integral`: its
 * phi integral times sin theta), 1 = MRProb, 2 = MRDistMax; v and normal
 * 3n, Estep [eV], b and w [m] per contact; out[i] NaN where MRProb's
 * integration failed.  theta and phi may be NULL unless what == 0. */
pt_status pt_mr_eval(pt_ctx *ctx, int32_t what, int32_t transmit, int32_t integral, int64_t n, const double *v,
                     const double *normal, const double *Estep, const double *b, const double *w, const double *theta,
                     const double *phi, double *out);

/* TNeutron::Decay (src/neutron.cpp:285-375) on the device: for n decayed
 * neutrons (ids, decay times t, end states y: 9n SoA, host buffers) the
 * proton and the electron each makes, written to protons / electrons (n
 * entries each, SoA stride n: id, t, y, spin = 0).  Ids: the parent's +
 * 2^40 (proton) and + 2^41 (electron); the draws come from the parent's
 * source stream with `seed`.  PT_ERR_INVALID when a proton's recoil-spectrum
 * sampling did not converge. */
pt_status pt_neutron_decay(pt_ctx *ctx, uint64_t seed, int64_t n, const int64_t *ids, const double *t, const double *y,
                           pt_particles *protons, pt_particles *electrons);

/* The reference's secondaries chain (`secondaries 1`, src/main.cpp:163-172)
 * in one call: the neutrons of `in` tracked with `neutron` into `out`, the
 * proton and electron of every neutron that decayed (pt_neutron_decay with
 * neutron->seed), then the protons tracked with `proton` and the electrons
 * with `electron` (species are per run on the device, so the secondaries
 * run as two batches after the neutrons).  out_p and out_e hold up to their
 * n entries (SoA stride their n; in->n always suffices) and receive the
 * secondaries' end states in the order of their parents; *n_decayed their
 * number; stats (may be NULL) sums the three runs.  PT_ERR_INVALID when
 * out_p or out_e is too small. */
pt_status pt_integrate_secondaries(pt_ctx *ctx, const pt_run_params *neutron, const pt_run_params *proton,
                                   const pt_run_params *electron, const pt_particles *in, pt_particles *out,
                                   pt_particles *out_p, pt_particles *out_e, int64_t *n_decayed, pt_stats *stats);

/* Calibration: FP64 fused-multiply-add throughput of this device measured by
 * a dependent-chain DFMA kernel over all SMs (TFLOP/s, 2 flops per FMA). */
pt_status pt_probe_fp64(pt_ctx *ctx, double *tflops);

/* ---- config.in front end (the reference's host inputs) ----
 * TConfig::ReadFromFile (src/config.cpp:14-53) plus TGeometry(TConfig&)
 * (src/geometry.cpp:93-137) and TFieldManager(TConfig&) (src/fields.cpp:19-136):
 * builds a pt_scene_desc from a config.in with its [GEOMETRY], [MATERIALS] or
 * materials_file, [FIELDS] (OPERA3D, 3Dtable, HarmonicExpansionBField,
 * EDMStaticEField with constant scales) and [FORMULAS] sections; STL and table
 * paths are relative to the config file.  The scene owns every array its
 * descriptor points to until pt_config_free.  Errors: PT_ERR_IO (files),
 * PT_ERR_INVALID (malformed entries), PT_ERR_UNSUPPORTED (field types, scale
 * formulas or options the device path does not implement); message in
 * pt_config_error(). */
typedef struct pt_config_scene pt_config_scene;
pt_status pt_config_load(const char *config_path, pt_config_scene **out);
const pt_scene_desc *pt_config_scene_desc(const pt_config_scene *scene);
void pt_config_free(pt_config_scene *scene);
/* [GLOBAL] simtime and the particle options of [PARTICLES] overridden by the
 * species section (tau, tmax, lmax, Bmax, spintimes, flipspin;
 * src/tracking.cpp:19-60); spintimes are copied into the caller's buffer of
 * max_spintimes doubles, which out->spintimes then points to. */
pt_status pt_config_run_params(const char *config_path, const char *species, pt_run_params *out, double *spintimes,
                               int32_t max_spintimes);
const char *pt_config_error(void);

/* The end log of one species' particles in the reference's text layout
 * (TLogger::Print with suffix "end", src/logger.cpp:42-126, written as
 * TTextLogger::DoLog does, src/logger.cpp:314-334): the file
 * <directory>/<jobnumber, 12 digits><particle>end.out with a header of the
 * variable names and one line per particle, values at 15 significant
 * digits, each followed by a space.  No reference counterpart as a function:
 * the reference writes the line per particle from TTracker.  `start` holds
 * the tracked inputs, `end` pt_integrate's outputs (n = start->n); the caller
 * passes B (3 per particle, row-major) and V at the start and end points and
 * the index into scene->solids of the solid each point is in
 * (pt_field_eval, pt_point_solids).  `logvars` (space-separated names, the
 * config's endlogvars) selects columns, NULL or "" the default 43; formulas
 * are refused with PT_ERR_UNSUPPORTED.  Errors: PT_ERR_INVALID, PT_ERR_IO;
 * message in pt_config_error(). */
/* The solid index each point is in, from its pt_point_solids mask at time t:
 * the default solid plus the masked solids in index order, the highest ID
 * not ignored at t winning (TTracker::GetCurrentsolid, src/tracking.cpp:
 * 367-370, over TGeometry::GetSolids, src/geometry.cpp:151-158).  Host only. */
pt_status pt_current_solid(const pt_scene_desc *scene, int64_t n, const uint64_t *masks, const double *t,
                           int32_t *solid_index);
pt_status pt_endlog_write(const char *directory, int64_t jobnumber, int32_t species, const pt_scene_desc *scene,
                          const pt_particles *start, const pt_particles *end, const double *b_start,
                          const double *v_start, const int32_t *solid_start, const double *b_end, const double *v_end,
                          const int32_t *solid_end, const char *logvars);

/* Library version string. */
const char *pt_version(void);

#ifdef __cplusplus
}
#endif

#endif /* PENTRACK_GPU_H */
