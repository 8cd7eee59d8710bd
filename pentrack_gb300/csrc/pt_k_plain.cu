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

/* The plain form for runs that integrate the spin (IntegrateSpin's Bloch
 * integration, LOOP D): the same LOOP-A iterations as k_plain, but a lane
 * whose step reaches its Bloch integration runs one try of its current
 * Bloch step per loop iteration, and every lane of the warp stays in the
 * loop and is re-synchronised at its top.  The lanes in their Bloch
 * integration -- almost all of them, since it takes hundreds of Bloch steps
 * per trajectory step -- then execute each try as one converged pass: a lane
 * whose try is rejected retries in the next pass with the others' next
 * tries, where retrying at once would leave the rest of the warp idle for a
 * whole try, and calling the integration per lane would let the warp split
 * into groups that run it separately.
 * The launch's quota of `steps` trajectory steps is a per-warp one: a lane
 * that reaches it keeps stepping until every lane of its warp has, then
 * finishes the step it is in (the trajectory steps of a spin run hold
 * hundreds of Bloch steps each, so lanes that stopped at their own quota
 * would leave the warp waiting on its slowest lane for a large part of the
 * launch).  An exact step budget (max_steps) and the pause time stay exact
 * per particle, so the results do not depend on where launches end. */
__global__ void __launch_bounds__(128) k_plain_spin(const __grid_constant__ DScene S, const __grid_constant__ DRun R, const __grid_constant__ DBatch b, DCounters *C,
                                                    int steps, int budget_from_nacc0) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool done = i >= b.n;
    if (!done) {
        if (b.stop_id[i] != PT_ID_UNKNOWN || b.t[i] >= R.t_pause) done = true;
        else if (R.max_steps > 0) steps = budget_from_nacc0 ? (int)(R.max_steps - (b.nacc[i] - b.nacc0[i])) : R.max_steps;
        if (steps <= 0) done = true;
    }
    Lane L(S, R);
    double t0 = 0;
    const bool had = !done;
    if (had) {
        L.load(b, i);
        t0 = L.t;
    }
    int s = 0, fin = 0, waited = 0;
    const bool exact = R.max_steps > 0;
    bool inbloch = false, quota = false, closing = false;
    /* a trajectory step ended: count it; true when the lane stops here */
    auto step_end = [&]() {
        ++s;
        if (L.stop != PT_ID_UNKNOWN || L.t >= R.t_pause || (exact && s >= steps) || *R.cancel) done = true;
        else if (s >= steps) quota = true;
        return done || (quota && closing);
    };
    for (;;) {
        __syncwarp();
        closing = closing || __all_sync(0xffffffffu, done || quota);
        const bool idle = done || (closing && !inbloch && !fin);
        if (__all_sync(0xffffffffu, idle)) break;
        /* The trajectory work (completing a finished Bloch integration and
         * the next trajectory step with its collision checks and
         * bisections) runs for the lanes that need it together: once
         * TRAJ_BATCH of them wait, once one has waited TRAJ_WAIT passes, or
         * when no lane is in its Bloch integration.  Run one lane at a time,
         * it would hold the warp's other lanes for whole bisections. */
        const bool traj = !idle && !inbloch;
        const int ntraj = __popc(__ballot_sync(0xffffffffu, traj));
        const bool go = ntraj >= TRAJ_BATCH || !__any_sync(0xffffffffu, !idle && inbloch) ||
                        __any_sync(0xffffffffu, traj && waited >= TRAJ_WAIT);
        if (idle) continue;
        if (inbloch) {
            const int r = L.bloch_try(L.bst, L.bx2);
            if (r != 0 && r != 2) {
                fin = r;
                inbloch = false;
                waited = 0;
            }
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
        if (q == 2) inbloch = true;
        else step_end();
    }
    if (had) {
        L.store(b, i);
        const bool active = (L.stop == PT_ID_UNKNOWN && L.t < R.t_pause);
        flush_counters(C, L.lc, L.t - t0, active);
    }
}

} // namespace ptk
