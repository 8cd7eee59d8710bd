/*
 * pto.h -- CPU oracle for the PENTrack tracking hot path (TEST INFRASTRUCTURE).
 *
 * This library is the checker of the GPU engine, never part of it: only the
 * tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
 * It restates in plain FP64 C++17 (no Boost, no CGAL) the reference's
 *   TTracker::IntegrateParticle / CheckHit / iterate_collision / DoStep / DoHit /
 *   IntegrateSpin decision logic           src/tracking.cpp:17-483
 *   TParticle EoM, energies, counters      src/particle.cpp:36-269
 *   TNeutron wall and bulk physics         src/neutron.cpp:25-282, include/neutron.h:53-68
 *   TProton/TElectron::OnStep              src/proton.cpp:25-33, src/electron.cpp:25-32
 *   field container + manager              src/field.cpp:48-169, src/fields.cpp:139-182
 *   TabField3 coefficients and evaluation  src/field_3d.cpp:36-121, 336-529
 *   EDM uniform E field                    src/edmfields.cpp:181-187
 *   geometry and collisions                src/geometry.cpp:139-175, src/trianglemesh.cpp:134-171,
 *                                          include/trianglemesh.h:57-91, 181-199
 *   RotateVector                           src/globals.cpp:40-64
 * and the third-party arithmetic the path depends on:
 *   Boost.odeint runge_kutta_dopri5 + controlled_runge_kutta + dense_output_runge_kutta
 *     (version unpinned by the reference, restated from the published method),
 *   ALGLIB 3.15.0 spline1dgriddiffcubic (alglib-3.15.0/cpp/src/interpolation.cpp:26709-26880),
 *   libtricubic tricubic_get_coeff      (tricubic-1.0/src/libtricubic/libtricubic.cpp:24-48).
 * Parity pins: oracle/_ref builds the reference's own ALGLIB and libtricubic
 * sources; tests/golden holds vectors generated from them (spline derivatives,
 * tricubic coefficients) plus the IntegrationTest known answer.  The odeint
 * step sequence itself is unpinned (Boost is absent from the reference tree).
 */
#ifndef PTO_H
#define PTO_H
#include <stdint.h>
#include "../include/pentrack_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pto_ctx pto_ctx;

int pto_create(const pt_scene_desc *scene, pto_ctx **out);
void pto_destroy(pto_ctx *ctx);
const char *pto_last_error(void);

/* Track every particle of `in` to its stop ID with `nthreads` host threads
 * (disjoint particle ranges, like the reference's job arrays). */
int pto_track(pto_ctx *ctx, const pt_run_params *params, const pt_particles *in, pt_particles *out,
              int nthreads, pt_stats *stats);

int pto_field(pto_ctx *ctx, int64_t n, const double *xyzt, double *B, double *dBidxj, double *V, double *E);
int pto_segment_collisions(pto_ctx *ctx, int64_t n, const double *seg, int32_t max_hits, int32_t *count,
                           double *s, double *normal, int32_t *solid_id, double *distnormal);
int pto_point_solids(pto_ctx *ctx, int64_t n, const double *p, uint64_t *mask);

/* building blocks exposed for the golden-vector tests */
int pto_spline_derivs(int32_t n, const double *x, const double *y, double *d);
int pto_spline1d_calc(int32_t n, const double *x, const double *y, int32_t np, const double *pts, double *out);
double pto_mr(int32_t what, int32_t transmit, int32_t integral, const double *v, const double *normal, double Estep, double b,
              double w, double theta, double phi);
void pto_tricubic_coeff(const double *stacked64, double *a64);
void pto_tricubic_eval(const double *a64, double x, double y, double z, int derx, int dery, int derz, double *out);
void pto_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
double pto_uniform(uint64_t seed, int64_t id, uint64_t draw);
/* the step adjuster's deterministic x^p (include/pt_detmath.h) */
double pto_detpow(double x, double p);
/* dopri5 dense-output evaluation of one accepted step of dy/dt = f on a
 * fixed test system (harmonic oscillator with drag); for unit tests. */
int pto_dopri5_selftest(double t0, const double *y0, double dt0, int nsteps, double *t_out, double *y_out);

#ifdef __cplusplus
}
#endif
#endif
