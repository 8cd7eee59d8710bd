/*
 * pt_kernels.cuh -- the engine's kernels, defined in pt_k_*.cu and launched
 * from the host code in pt_api.cu.
 */
#pragma once
#include "pt_device.cuh"

/* k_try: resident blocks of 128 per SM (register budget 168) */
#define PT_TRY_BLOCKS_PER_SM 3

namespace ptk {

__global__ void k_init(const __grid_constant__ DScene S, const __grid_constant__ DRun R, const __grid_constant__ DBatch b, DCounters *C);
__global__ void k_gather(const __grid_constant__ DBatch b, double t_pause, int32_t *list, int32_t *count);
__global__ void k_regather(const __grid_constant__ DBatch b, double t_pause, int max_steps, int32_t *list, int32_t *count);
__global__ void k_zero_counts(int32_t *count, int a, int b, int c);
__global__ void k_try(const __grid_constant__ DScene S, const __grid_constant__ DRun R, const __grid_constant__ DBatch b, DCounters *C, int in, int out,
                      DSched *sc);
__global__ void k_try_tab32(const __grid_constant__ DScene S, const __grid_constant__ DRun R, const __grid_constant__ DBatch b, DCounters *C, int in,
                            int out, DSched *sc);
__global__ void k_try_w(const __grid_constant__ DScene S, const __grid_constant__ DRun R, const __grid_constant__ DBatch b, DCounters *C, int in, int out,
                        DSched *sc);
__global__ void k_try_tab32_w(const __grid_constant__ DScene S, const __grid_constant__ DRun R, const __grid_constant__ DBatch b, DCounters *C, int in,
                              int out, DSched *sc);
__global__ void k_post(const __grid_constant__ DScene S, const __grid_constant__ DRun R, const __grid_constant__ DBatch b, DCounters *C, int out,
                       DSched *sc);
__global__ void k_sched_after_post(const __grid_constant__ DBatch b, DSched *sc, cudaGraphConditionalHandle slow);
__global__ void k_sched_after_slow_phased(const __grid_constant__ DBatch b, DSched *sc, const __grid_constant__ DRun R,
                                          cudaGraphConditionalHandle slow);
__global__ void k_sched_end_phased(const __grid_constant__ DBatch b, DSched *sc, const __grid_constant__ DRun R,
                                   cudaGraphConditionalHandle outer);
__global__ void k_slow(const __grid_constant__ DScene S, const __grid_constant__ DRun R, const __grid_constant__ DBatch b, DCounters *C, int out,
                       DSched *sc);
__global__ void k_bisect(const __grid_constant__ DScene S, const __grid_constant__ DRun R, const __grid_constant__ DBatch b, DCounters *C,
                         DSched *sc);
__global__ void k_run(const __grid_constant__ DScene S, const __grid_constant__ DRun R, const __grid_constant__ DBatch b, DCounters *C, DSched *sc,
                      int max_run);
__global__ void k_run_tab32(const __grid_constant__ DScene S, const __grid_constant__ DRun R, const __grid_constant__ DBatch b, DCounters *C,
                            DSched *sc, int max_run);
__global__ void k_run2(const __grid_constant__ DScene S, const __grid_constant__ DRun R, const __grid_constant__ DBatch b, DCounters *C, DSched *sc,
                       int max_run);
__global__ void k_run2_tab32(const __grid_constant__ DScene S, const __grid_constant__ DRun R, const __grid_constant__ DBatch b, DCounters *C,
                             DSched *sc, int max_run);
__global__ void k_sched_begin(const __grid_constant__ DBatch b, DSched *sc);
__global__ void k_sched_after_run(const __grid_constant__ DBatch b, DSched *sc, cudaGraphConditionalHandle slow);
__global__ void k_sched_after_slow(const __grid_constant__ DBatch b, DSched *sc, const __grid_constant__ DRun R,
                                   cudaGraphConditionalHandle slow);
__global__ void k_sched_end(const __grid_constant__ DBatch b, DSched *sc, const __grid_constant__ DRun R,
                            cudaGraphConditionalHandle outer);
__global__ void k_sched_period(DSched *sc);
__global__ void k_adj_forward(const __grid_constant__ DScene S, const __grid_constant__ DRun R, const __grid_constant__ DBatch b, DCounters *C,
                              const __grid_constant__ DAdj A);
__global__ void k_adj_reverse(const __grid_constant__ DScene S, const __grid_constant__ DRun R, const __grid_constant__ DBatch b, DCounters *C,
                              const __grid_constant__ DAdj A);
__global__ void k_plain(const __grid_constant__ DScene S, const __grid_constant__ DRun R, const __grid_constant__ DBatch b, DCounters *C, int steps,
                        int budget_from_nacc0);
__global__ void k_plain_spin(const __grid_constant__ DScene S, const __grid_constant__ DRun R, const __grid_constant__ DBatch b, DCounters *C, int steps,
                             int budget_from_nacc0);
__global__ void k_fp64_probe(double *out, int iters, double a, double b);
__global__ void k_mr(int what, int transmit, int integral, int64_t n, const double *v, const double *nrm, const double *Estep,
                     const double *b, const double *w, const double *theta, const double *phi, double *out);
__global__ void k_field(const __grid_constant__ DScene S, int prec, int64_t n, const double *xyzt, double *B, double *dB, double *V, double *E);
__global__ void k_collisions(const __grid_constant__ DScene S, int64_t n, const double *seg, int maxh, int *count, double *s, double *nrm, int *sid,
                             double *dn);
__global__ void k_point_solids(const __grid_constant__ DScene S, int64_t n, const double *p, unsigned long long *mask);
__global__ void k_decay(uint64_t seed, int64_t n, const int64_t *id, const double *t, const double *y, int64_t *pid, double *pt,
                        double *py, int64_t *eid, double *et, double *ey, int *status);
__global__ void k_source_vmin(const __grid_constant__ DScene S, const __grid_constant__ DSourceSpec Q, DSpecies sp, int64_t n, double *v);
__global__ void k_source(const __grid_constant__ DScene S, const __grid_constant__ DSourceSpec Q, DSpecies sp, int64_t n, const int64_t *ids,
                         double vmin, double *t_out, double *y, double *spin, int *status);
__global__ void k_source_surface(const __grid_constant__ DScene S, const __grid_constant__ DSourceSpec Q, DSpecies sp, int64_t n,
                                 const int64_t *ids, double *t_out, double *y, double *spin, int *status);

} // namespace ptk
