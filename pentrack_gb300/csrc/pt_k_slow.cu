/*
 * pt_k_slow.cu -- batched form: the full post-step state machine and the bisections.
 */
#include "pt_kcommon.cuh"
#include "pt_kernels.cuh"

namespace ptk {

/* Batched form, phase 3: the full post-step logic (chord split, CheckHit,
 * hit physics, clipping) for the queued steps, run until the step completes
 * or needs a bisection; those post-steps are suspended and queued for k_bisect. */
__global__ void __launch_bounds__(128) k_slow(const __grid_constant__ DScene S, const __grid_constant__ DRun R, const __grid_constant__ DBatch b, DCounters *C, int out,
                                              DSched *sc) {
    span_begin(sc, PT_SPAN_SLOW);
    const int n = b.count[3];
    const int32_t *ls = b.list[3];
    Lane L(S, R);
    double ps = 0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int i = ls[k];
        L.load(b, i);
        L.load_dense(b, i);
        L.load_bc(b, i);
        if (L.flags & PT_F_SUSPENDED) L.load_post(b, i);
        else L.ps.stage = PS_BEGIN;
        L.flags &= ~(PT_F_PENDING | PT_F_SUSPENDED);
        const double t0 = L.t;
        if (L.post_resume()) {
            L.flags |= PT_F_PENDING | PT_F_SUSPENDED;
            L.store_post(b, i);
            L.store(b, i);
            list_push(b.list[4], &b.count[4], i);
            continue;
        }
        ps += L.t - t0;
        L.store_bc_commit(b, i);
        L.store(b, i);
        if (keeps_going(R, b, L, i)) list_push(b.list[out], &b.count[out], i);
    }
    flush_counters(C, L.lc, ps, false);
    span_end(sc, PT_SPAN_SLOW);
}

/* Batched form, phase 4: the bisections (TTracker::iterate_collision) that
 * suspended post-steps asked for.  Every loop iteration runs one step (one
 * chord query) of the lane's current bisection; a lane whose bisection ends
 * stores the result and takes the next request from the list, so the lanes of
 * a warp stay on the same code while bisections of very different lengths
 * run.  All lanes of a warp stay in the loop until the warp is done and the
 * warp is re-synchronised at the top of each iteration, so the step runs as
 * one converged pass however the lanes' refills interleave.  The post-steps
 * go back to the slow list.  count[5] (zero at launch) is the take cursor of
 * the request list. */
__global__ void __launch_bounds__(128, 4) k_bisect(const __grid_constant__ DScene S, const __grid_constant__ DRun R, const __grid_constant__ DBatch b, DCounters *C,
                                                   DSched *sc) {
    span_begin(sc, PT_SPAN_BISECT);
    const int n = b.count[4];
    const int32_t *lq = b.list[4];
    Lane L(S, R);
    BisectState bs;
    int i = -1;
    bool done = false;
    for (;;) {
        __syncwarp();
        if (!done && i < 0) {
            const int k = atomicAdd(&b.count[5], 1);
            if (k >= n) done = true;
            else {
                i = lq[k];
                L.load_bisect_request(b, i);
                L.bisect_begin(bs, L.ps.cx1, L.ps.cya, L.ps.x2, L.ps.y2);
            }
        }
        if (__all_sync(0xffffffffu, done)) break;
        if (done) continue;
        const int r = L.bisect_step(bs, L.ps.bxa, L.ps.bao, L.ps.bxb, L.ps.bbo);
        if (r != BISECT_RUNNING) {
            L.ps.bres = r;
            L.store_bisect_result(b, i);
            list_push(b.list[3], &b.count[3], i);
            i = -1;
        }
    }
    flush_counters(C, L.lc, 0.0, false);
    span_end(sc, PT_SPAN_BISECT);
}

} // namespace ptk
