/*
 * pt_k_query.cu -- initialisation, the FP64 probe and the query entry points.
 */
#include "pt_kcommon.cuh"
#include "pt_kernels.cuh"

namespace ptk {

__global__ void __launch_bounds__(128) k_init(const __grid_constant__ DScene S, const __grid_constant__ DRun R, const __grid_constant__ DBatch b, DCounters *C) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.n) return;
    Lane L(S, R);
    const int64_t n = b.n;
    L.id = b.id[i];
    L.t = b.t[i];
    for (int c = 0; c < 9; ++c) { L.y[c] = b.y[c * n + i]; L.dydt[c] = 0; }
    for (int c = 0; c < 5; ++c) L.spin[c] = b.spin[c * n + i];
    L.stop = PT_ID_UNKNOWN;
    QueryStats qs{0, 0};
    L.init(qs);
    if (R.log.track && L.stop == PT_ID_UNKNOWN) L.log_track(L.y[8], L.t, L.y); /* the track log's first point */
    L.store_bc_commit(b, i);
    L.store(b, i);
    b.hstart[i] = L.hmax;
    b.t_last[i] = L.t;
}

/* FP64 throughput probe: 8 independent dependent-FMA chains per thread */
__global__ void k_fp64_probe(double *out, int iters, double a, double b) {
    double x0 = threadIdx.x * 1e-9, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == 1.2345) out[0] = s;
}

__global__ void k_field(const __grid_constant__ DScene S, int prec, int64_t n, const double *xyzt, double *B, double *dB, double *V, double *E) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double *q = xyzt + 4 * i;
    double b[3], db[3][3], v, e[3];
    if (dB) bfield<true>(S, prec, q[0], q[1], q[2], b, db);
    else bfield<false>(S, prec, q[0], q[1], q[2], b, nullptr);
    efield(S, prec, q[0], q[1], q[2], v, e);
    if (B) for (int k = 0; k < 3; ++k) B[3 * i + k] = b[k];
    if (dB) for (int k = 0; k < 9; ++k) dB[9 * i + k] = db[k / 3][k % 3];
    if (V) V[i] = v;
    if (E) for (int k = 0; k < 3; ++k) E[3 * i + k] = e[k];
}

/* MicroRoughness of wall contacts: what 0 MRDist at (theta, phi), 1 MRProb
 * (NaN when the integration fails), 2 MRDistMax */
__global__ void k_mr(int what, int transmit, int integral, int64_t n, const double *v, const double *nrm, const double *Estep,
                     const double *b, const double *w, const double *theta, const double *phi, double *out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    MRHit h;
    mr_setup(h, v + 3 * i, nrm + 3 * i, Estep[i], b[i], w[i]);
    double r;
    if (what == 0) r = mr_dist(h, transmit != 0, integral != 0, theta[i], phi[i]);
    else if (what == 1) {
        bool ok = true;
        r = mr_prob(h, transmit != 0, ok);
        if (!ok) r = __longlong_as_double(0x7ff8000000000000ll);
    } else r = mr_distmax(h, transmit != 0);
    out[i] = r;
}

__global__ void k_collisions(const __grid_constant__ DScene S, int64_t n, const double *seg, int maxh, int *count, double *s, double *nrm, int *sid,
                             double *dn) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Coll c[PT_MAX_COLLS];
    QueryStats qs{0, 0};
    bool cp;
    int h = mesh_query<1>(S, seg + 6 * i, seg + 6 * i + 3, 0.0, 1.0, c, PT_MAX_COLLS, nullptr, qs, cp);
    if (cp) { count[i] = -1; return; }
    count[i] = h;
    int k = h < maxh ? h : maxh;
    if (k > PT_MAX_COLLS) k = PT_MAX_COLLS;
    for (int j = 0; j < k; ++j) {
        int64_t o = i * maxh + j;
        s[o] = c[j].s;
        for (int a = 0; a < 3; ++a) nrm[3 * o + a] = c[j].n[a];
        sid[o] = (int)c[j].id;
        dn[o] = c[j].dn;
    }
}

__global__ void k_point_solids(const __grid_constant__ DScene S, int64_t n, const double *p, unsigned long long *mask) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    QueryStats qs{0, 0};
    mask[i] = point_solids(S, p + 3 * i, qs);
}

} // namespace ptk
