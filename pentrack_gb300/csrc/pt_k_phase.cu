/*
 * pt_k_phase.cu -- batched form: active lists, one RK try per particle, fast step completion.
 */
#include "pt_kcommon.cuh"
#include "pt_kernels.cuh"

namespace ptk {

/* active list of a batch: particles not stopped and before t_pause */
__global__ void k_gather(const __grid_constant__ DBatch b, double t_pause, int32_t *list, int32_t *count) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.n) return;
    if (b.stop_id[i] != PT_ID_UNKNOWN) return;
    b.nacc0[i] = b.nacc[i];
    if (b.flags[i] & PT_F_PENDING) list_push(b.list[3], &b.count[3], (int32_t)i); /* resume a deferred post-step */
    else if (b.t[i] < t_pause) list_push(list, count, (int32_t)i);
}

/* The next iteration's active list rebuilt from the particle states: the same
 * set the previous iteration appended (not stopped, no post-step pending,
 * before t_pause, within the step budget), but every warp appends its active
 * particles among 32 consecutive ones in index order.  The lanes of a warp in
 * k_try then read and write neighbouring entries of the state arrays, where
 * the appends of the previous iteration had scattered them over separate
 * memory sectors. */
__global__ void k_regather(const __grid_constant__ DBatch b, double t_pause, int max_steps, int32_t *list, int32_t *count) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.n) return;
    if (b.stop_id[i] != PT_ID_UNKNOWN || (b.flags[i] & PT_F_PENDING) || !(b.t[i] < t_pause)) return;
    if (max_steps > 0 && b.nacc[i] - b.nacc0[i] >= max_steps) return;
    list_push(list, count, (int32_t)i);
}

__global__ void k_zero_counts(int32_t *count, int a, int b, int c) {
    if (threadIdx.x == 0) { count[a] = 0; count[b] = 0; count[c] = 0; }
}

/* Batched form, phase 1: exactly one Dormand-Prince try for every active
 * particle (all lanes execute the same instruction stream).  k_try_tab32 is
 * the instance with the FP32-table-only right-hand side (neutral species,
 * FP32 field mode, magnetic fields all FP32 tables).  At 3 blocks per SM
 * (168 registers) both spill part of the stage vectors to local memory;
 * the *_w instances at 2 blocks per SM (255 registers) trade a third of the
 * resident warps for fewer spills, and the autotuner picks between them. */
template <bool TAB_ONLY>
static __device__ __forceinline__ void try_phase(const DScene &S, const DRun &R, const DBatch &b, DCounters *C, int in, int out, DSched *sc) {
    span_begin(sc, PT_SPAN_TRY);
    const int n = b.count[in];
    const int32_t *lin = b.list[in];
    Lane L(S, R);
    double ksr[5][9];
    const Lane::KReg ks{ksr, L.y, L.dydt};
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int i = lin[k];
        L.load_try_input(b, i, ks);
        int r = L.rk_try_with<TAB_ONLY>(ks);
        L.store_try_output(b, i, r == 1, ks);
        if (r == 1) {
            uint32_t f = b.flags[i];
            L.flags = f;
            L.store_bc_try(b, i);
            b.flags[i] = L.flags;
            list_push(b.list[2], &b.count[2], i);
        } else if (r == 0) {
            list_push(b.list[out], &b.count[out], i);
        } else {
            b.stop_id[i] = PT_ID_ODEINT_ERROR;
        }
    }
    flush_counters(C, L.lc, 0.0, false);
    span_end(sc, PT_SPAN_TRY);
}

__global__ void __launch_bounds__(128, PT_TRY_BLOCKS_PER_SM) k_try(const __grid_constant__ DScene S, const __grid_constant__ DRun R, const __grid_constant__ DBatch b, DCounters *C, int in, int out,
                                                                  DSched *sc) {
    try_phase<false>(S, R, b, C, in, out, sc);
}
__global__ void __launch_bounds__(128, PT_TRY_BLOCKS_PER_SM) k_try_tab32(const __grid_constant__ DScene S, const __grid_constant__ DRun R, const __grid_constant__ DBatch b, DCounters *C, int in, int out,
                                                                        DSched *sc) {
    try_phase<true>(S, R, b, C, in, out, sc);
}
__global__ void __launch_bounds__(128, 2) k_try_w(const __grid_constant__ DScene S, const __grid_constant__ DRun R, const __grid_constant__ DBatch b, DCounters *C, int in, int out,
                                                  DSched *sc) {
    try_phase<false>(S, R, b, C, in, out, sc);
}
__global__ void __launch_bounds__(128, 2) k_try_tab32_w(const __grid_constant__ DScene S, const __grid_constant__ DRun R, const __grid_constant__ DBatch b, DCounters *C, int in,
                                                        int out, DSched *sc) {
    try_phase<true>(S, R, b, C, in, out, sc);
}

/* Batched form, phase 2: the common step completion (no clip, no split, no
 * collision); other steps are queued for phase 3. */
__global__ void __launch_bounds__(128) k_post(const __grid_constant__ DScene S, const __grid_constant__ DRun R, const __grid_constant__ DBatch b, DCounters *C, int out,
                                              DSched *sc) {
    span_begin(sc, PT_SPAN_POST);
    const int n = b.count[2];
    const int32_t *lp = b.list[2];
    Lane L(S, R);
    double ps = 0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int i = lp[k];
        L.load(b, i);
        L.load_try_end(b, i);
        L.load_bc(b, i);
        const double t0 = L.t;
        if (L.fast_post()) {
            ps += L.t - t0;
            L.store_bc_commit(b, i);
            L.store(b, i);
            if (keeps_going(R, b, L, i)) list_push(b.list[out], &b.count[out], i);
        } else {
            b.flags[i] |= PT_F_PENDING;
            list_push(b.list[3], &b.count[3], i);
        }
    }
    flush_counters(C, L.lc, ps, false);
    span_end(sc, PT_SPAN_POST);
}

} // namespace ptk
