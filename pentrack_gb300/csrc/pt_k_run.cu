/*
 * pt_k_run.cu -- batched form: the persistent stepping kernel and the
 * device-side scheduling kernels of its CUDA graph.
 *
 * k_run replaces the reference's serial particle loop (src/main.cpp:153-175
 * over TTracker::IntegrateParticle, src/tracking.cpp:71-148) by lanes that
 * each hold one particle in registers and run whole LOOP-A iterations on it
 * for as long as they complete without the full post-step logic (no decay or
 * tmax clip, no chord split, no collision, no Bloch integration).  A lane
 * whose particle needs that logic, stops, or reaches its step budget hands
 * the particle on and takes the next one from the active list through an
 * atomic cursor, so particles of very different trajectory lengths share
 * one launch.  Steps that need the full logic are queued for k_slow /
 * k_bisect.  Each particle executes exactly its own plain-form operations in
 * its own order, so results are bit-identical to the plain form.
 */
#include "pt_kcommon.cuh"
#include "pt_kernels.cuh"

namespace ptk {

/* The persistent stepping kernel over the active list b.list[0] (count[0]).
 * count[6] is the take cursor; a particle handed back because the list ran
 * dry (drain) or its run reached max_run, and that keeps going, is counted in
 * count[1]; steps that need the full post-step go to list 3.
 * max_run: consecutive steps of one particle before the lane hands it back
 * (0 = no limit besides the step budget).
 * Every lane of a warp stays in the loop until the whole warp is done and
 * the warp is re-synchronised at the top of each iteration, so the RK try --
 * whether a retry after a rejection, the next step or a fresh particle's
 * step -- runs as one converged pass per warp. */
template <bool TAB_ONLY>
static __device__ __forceinline__ void run_phase(const DScene &S, const DRun &R, const DBatch &b, DCounters *C, DSched *sc,
                                                 int max_run) {
    span_begin(sc, PT_SPAN_RUN);
    const int n = b.count[0];
    const int32_t *lst = b.list[0];
    volatile int32_t *cursor = &b.count[6];
    Lane L(S, R);
    double ksr[5][9];
    const Lane::KReg ks{ksr, L.y, L.dydt};
    double ps = 0;
    int i = -1, run = 0;
    bool done = false;
    for (;;) {
        __syncwarp();
        if (!done && i < 0) {
            const int k = atomicAdd(&b.count[6], 1);
            if (k >= n) done = true;
            else {
                i = lst[k];
                L.load(b, i);
                L.load_bc(b, i);
                run = 0;
            }
        }
        if (__all_sync(0xffffffffu, done)) break;
        if (done) continue;
        const int r = L.rk_try_with<TAB_ONLY>(ks);
        if (r == 0) continue; /* rejected: the same lane retries with the shrunk step */
        if (r < 0) {
            L.stop = PT_ID_ODEINT_ERROR;
            L.store(b, i);
            i = -1;
            continue;
        }
        const double t0 = L.t;
        if (L.fast_post()) {
            ps += L.t - t0;
            ++run;
            const bool going = keeps_going(R, b, L, i);
            /* hand the particle back when it is done for this call, when its
             * run reaches max_run, or once the list has run dry (the others
             * then finish their current step and the launch ends) */
            if (!going || (max_run > 0 && run >= max_run) || *cursor >= n) {
                L.store_bc_commit(b, i);
                L.store(b, i);
                if (going) atomicAdd(&b.count[1], 1);
                i = -1;
            }
        } else {
            /* the full post-step runs in k_slow: the committed state, the
             * accepted try and its B values are handed over */
            L.store_try_output(b, i, true, ks);
            L.store_bc_handoff(b, i);
            L.flags |= PT_F_PENDING;
            L.store(b, i);
            list_push(b.list[3], &b.count[3], i);
            i = -1;
        }
    }
    flush_counters(C, L.lc, ps, false);
    span_end(sc, PT_SPAN_RUN);
}

/* instances: general / FP32-table-only right-hand side, at 3 resident
 * blocks of 128 per SM (168 registers) or 2 (255 registers, fewer spills of
 * the lane state the kernel keeps across steps); the host picks one */
__global__ void __launch_bounds__(128, 3) k_run(const __grid_constant__ DScene S, const __grid_constant__ DRun R,
                                               const __grid_constant__ DBatch b, DCounters *C, DSched *sc, int max_run) {
    run_phase<false>(S, R, b, C, sc, max_run);
}
__global__ void __launch_bounds__(128, 3) k_run_tab32(const __grid_constant__ DScene S, const __grid_constant__ DRun R,
                                                     const __grid_constant__ DBatch b, DCounters *C, DSched *sc, int max_run) {
    run_phase<true>(S, R, b, C, sc, max_run);
}
__global__ void __launch_bounds__(128, 2) k_run2(const __grid_constant__ DScene S, const __grid_constant__ DRun R,
                                                const __grid_constant__ DBatch b, DCounters *C, DSched *sc, int max_run) {
    run_phase<false>(S, R, b, C, sc, max_run);
}
__global__ void __launch_bounds__(128, 2) k_run2_tab32(const __grid_constant__ DScene S, const __grid_constant__ DRun R,
                                                      const __grid_constant__ DBatch b, DCounters *C, DSched *sc, int max_run) {
    run_phase<true>(S, R, b, C, sc, max_run);
}

/* ---- scheduling kernels of the batched form's CUDA graph (one thread) ---- */

/* start of a period (one graph launch): its iterations count from here */
__global__ void k_sched_period(DSched *sc) {
    if (threadIdx.x == 0) sc->period_start = sc->outer_iters;
}

/* start of an outer iteration: empty the active list, the continuing count
 * and the cursor */
__global__ void k_sched_begin(const __grid_constant__ DBatch b, DSched *sc) {
    if (threadIdx.x != 0) return;
    b.count[0] = 0;
    b.count[1] = 0;
    b.count[2] = 0;
    b.count[6] = 0;
    sc->outer_iters += 1;
    sc->inner_this = 0;
}

/* after k_run: close its time span; run the slow rounds while list 3 is
 * non-empty */
__global__ void k_sched_after_run(const __grid_constant__ DBatch b, DSched *sc, cudaGraphConditionalHandle slow) {
    if (threadIdx.x != 0) return;
    span_close(sc, PT_SPAN_RUN);
    sc->last_active = b.count[0];
    cudaGraphSetConditional(slow, b.count[3] > 0 ? 1u : 0u);
}

/* end of one slow round (k_slow + k_bisect): another while list 3 holds
 * post-steps, unless the call was cancelled or the round cap is reached */
__global__ void k_sched_after_slow(const __grid_constant__ DBatch b, DSched *sc, const __grid_constant__ DRun R,
                                   cudaGraphConditionalHandle slow) {
    if (threadIdx.x != 0) return;
    span_close(sc, PT_SPAN_SLOW);
    span_close(sc, PT_SPAN_BISECT);
    sc->inner_iters += 1;
    if (++sc->inner_this >= PT_MAX_SLOW_ROUNDS && b.count[3] > 0) sc->error = 1;
    const bool more = b.count[3] > 0 && *R.cancel == 0 && !sc->error;
    cudaGraphSetConditional(slow, more ? 1u : 0u);
}

/* end of an outer iteration: continue while particles keep going, more than
 * the tail threshold of them, within the period's iteration cap and not
 * cancelled; the host finishes the rest */
__global__ void k_sched_end(const __grid_constant__ DBatch b, DSched *sc, const __grid_constant__ DRun R,
                            cudaGraphConditionalHandle outer) {
    if (threadIdx.x != 0) return;
    const int going = b.count[1];
    sc->last_going = going;
    const bool more = going > sc->tail && (sc->outer_iters - sc->period_start) < sc->max_iters && *R.cancel == 0 &&
                      b.count[3] == 0 && !sc->error;
    cudaGraphSetConditional(outer, more ? 1u : 0u);
}

/* ---- the phase-split iteration in the same graph form ----
 * k_regather, k_try (one RK try per active particle), k_post (the common
 * completion), then slow rounds while the slow list fills the GPU: the
 * decisions the host-driven phase split takes between its launches, taken
 * here on the device (count[1]: particles that keep stepping, count[3]:
 * queued post-steps) */
static __device__ __forceinline__ bool slow_rounds_due(const DBatch &b, const DSched *sc) {
    const int active = b.count[1], slow = b.count[3];
    return slow > 0 && (slow >= max(2048, active / 4) || active == 0 || active <= sc->tail);
}

__global__ void k_sched_after_post(const __grid_constant__ DBatch b, DSched *sc, cudaGraphConditionalHandle slow) {
    if (threadIdx.x != 0) return;
    span_close(sc, PT_SPAN_TRY);
    span_close(sc, PT_SPAN_POST);
    sc->last_active = b.count[0];
    cudaGraphSetConditional(slow, slow_rounds_due(b, sc) ? 1u : 0u);
}

__global__ void k_sched_after_slow_phased(const __grid_constant__ DBatch b, DSched *sc, const __grid_constant__ DRun R,
                                          cudaGraphConditionalHandle slow) {
    if (threadIdx.x != 0) return;
    span_close(sc, PT_SPAN_SLOW);
    span_close(sc, PT_SPAN_BISECT);
    sc->inner_iters += 1;
    if (++sc->inner_this >= PT_MAX_SLOW_ROUNDS && b.count[3] > 0) sc->error = 1;
    const bool more = slow_rounds_due(b, sc) && *R.cancel == 0 && !sc->error;
    cudaGraphSetConditional(slow, more ? 1u : 0u);
}

__global__ void k_sched_end_phased(const __grid_constant__ DBatch b, DSched *sc, const __grid_constant__ DRun R,
                                   cudaGraphConditionalHandle outer) {
    if (threadIdx.x != 0) return;
    const int going = b.count[1], slow = b.count[3];
    sc->last_going = going;
    sc->last_slow = slow;
    const bool finished = going == 0 && slow == 0;
    const bool tail = going <= sc->tail && slow == 0;
    const bool more = !finished && !tail && (sc->outer_iters - sc->period_start) < sc->max_iters && *R.cancel == 0 && !sc->error;
    cudaGraphSetConditional(outer, more ? 1u : 0u);
}

} // namespace ptk
