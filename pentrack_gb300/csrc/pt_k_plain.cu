/*
 * pt_k_plain.cu -- plain form: whole LOOP-A iterations per lane.
 */
#include "pt_kcommon.cuh"
#include "pt_kernels.cuh"

namespace ptk {

/* Plain form: every lane advances its particle by up to `steps` LOOP-A
 * iterations, then the launch ends and the host relaunches. */
__global__ void __launch_bounds__(128) k_plain(const __grid_constant__ DScene S, const __grid_constant__ DRun R, const __grid_constant__ DBatch b, DCounters *C, int steps,
                                               int budget_from_nacc0) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.n) return;
    if (b.stop_id[i] != PT_ID_UNKNOWN || b.t[i] >= R.t_pause) return;
    /* a step budget counts from the start of the advance call: in the tail of
     * the batched form the particle has already used part of it */
    if (R.max_steps > 0) steps = budget_from_nacc0 ? (int)(R.max_steps - (b.nacc[i] - b.nacc0[i])) : R.max_steps;
    if (steps <= 0) return;
    Lane L(S, R);
    L.load(b, i);
    const double t0 = L.t;
    for (int s = 0; s < steps; ++s) {
        L.step();
        if (L.stop != PT_ID_UNKNOWN || L.t >= R.t_pause) break;
        if (*R.cancel) break;
    }
    L.store(b, i);
    bool active = (L.stop == PT_ID_UNKNOWN && L.t < R.t_pause);
    flush_counters(C, L.lc, L.t - t0, active);
}

} // namespace ptk
