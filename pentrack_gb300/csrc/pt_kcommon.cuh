/*
 * pt_kcommon.cuh -- device helpers shared by the kernel translation units:
 * warp-aggregated counter flushes and work-list appends.
 */
#pragma once
#include "pt_lane.cuh"

namespace ptk {
using namespace ptd;

/* sum of v over the lanes in `mask` (any subset of the warp) */
template <class T> static __device__ __forceinline__ T warp_sum(unsigned mask, T v) {
    T s = 0;
    for (unsigned m = mask; m; m &= m - 1) s += __shfl_sync(mask, v, __ffs(m) - 1);
    return s;
}

static __device__ __forceinline__ void flush_counters(DCounters *C, const LaneCounters &lc, double psec, bool active) {
    /* warp-aggregated atomics over the lanes that reach this point */
    unsigned long long v[17] = {lc.rk_acc, lc.rk_rej, lc.rhs, lc.fields, lc.hits, lc.bisect, lc.nodes, lc.tris, lc.subseg, lc.dense,
                                active ? 1ull : 0ull, lc.cand_calls, lc.cand_overflow, lc.cand_sum, lc.tri32, lc.dead, lc.spin};
    const unsigned mask = __activemask();
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    for (int k = 0; k < 17; ++k) v[k] = warp_sum(mask, v[k]);
    double ps = warp_sum(mask, psec);
    unsigned bm = lc.bisect_max;
    for (unsigned m = mask; m; m &= m - 1) bm = max(bm, __shfl_sync(mask, lc.bisect_max, __ffs(m) - 1));
    if (lane == leader && bm) atomicMax(&C->bisect_max, bm);
    if (lane == leader) {
        unsigned long long *dst[17] = {&C->rk_accepted, &C->rk_rejected, &C->rhs_evals, &C->field_evals, &C->hits,
                                       &C->bisection_levels, &C->bvh_nodes, &C->tri_tests, &C->subsegments,
                                       &C->dense_evals, &C->active, &C->cand_calls, &C->cand_overflow, &C->cand_sum,
                                       &C->tri32, &C->bisect_dead, &C->spin_steps};
        for (int k = 0; k < 17; ++k) if (v[k]) atomicAdd(dst[k], v[k]);
        if (ps != 0) atomicAdd(&C->particle_seconds, ps);
    }
}

/* append v to a work list (warp-aggregated atomic) */
/* The warp-synchronous spin kernels' batching of trajectory work (completing
 * a Bloch integration, the next trajectory step, its collision checks and
 * bisections): lanes that need it wait until TRAJ_BATCH of them do, or one
 * has waited TRAJ_WAIT passes, or no lane of the warp is in its Bloch
 * integration, and then run it together. */
constexpr int TRAJ_BATCH = 8, TRAJ_WAIT = 16;

static __device__ __forceinline__ void list_push(int32_t *list, int32_t *count, int32_t v) {
    const unsigned m = __activemask();
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    const int rank = __popc(m & ((1u << lane) - 1));
    int base = 0;
    if (lane == leader) base = atomicAdd(count, __popc(m));
    base = __shfl_sync(m, base, leader);
    list[base + rank] = v;
}

/* Device time of the timed kernels inside the batched form's graph: every
 * block records its start and end on %globaltimer (nanoseconds); the
 * scheduling kernel after a launch adds max(end) - min(start) to the
 * kernel's total.  sc == nullptr (host-driven loops, timed with events)
 * skips it. */
static __device__ __forceinline__ unsigned long long gtimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}
static __device__ __forceinline__ void span_begin(DSched *sc, int k) {
    if (sc && threadIdx.x == 0) atomicMin(&sc->t0[k], gtimer());
}
static __device__ __forceinline__ void span_end(DSched *sc, int k) {
    if (!sc) return;
    __syncthreads();
    if (threadIdx.x == 0) atomicMax(&sc->t1[k], gtimer());
}
static __device__ __forceinline__ void span_close(DSched *sc, int k) {
    if (sc->t1[k] > sc->t0[k] && sc->t0[k] != ~0ull) {
        sc->ns[k] += sc->t1[k] - sc->t0[k];
        sc->launches[k] += 1;
    }
    sc->t0[k] = ~0ull;
    sc->t1[k] = 0;
}

/* a committed particle keeps stepping in this advance call */
static __device__ __forceinline__ bool keeps_going(const DRun &R, const DBatch &b, const Lane &L, int i) {
    if (L.stop != PT_ID_UNKNOWN || !(L.t < R.t_pause)) return false;
    return R.max_steps <= 0 || L.nacc - b.nacc0[i] < R.max_steps;
}

} // namespace ptk
