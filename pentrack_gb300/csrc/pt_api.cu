/*
 * pt_api.cu -- host side of the GB300 tracking engine: scene upload, the
 * batched scheduler and the C ABI declared in include/pentrack_gpu.h (the
 * kernels are in pt_k_*.cu).
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "pt_kernels.cuh"
#include "pt_scene.hpp"

/* record layout of the adjoint's tapes (doubles per record; see pt_adjoint.cuh) */
namespace {
constexpr int SEG_DOUBLES = 108, CK_DOUBLES = 14, STEP_DOUBLES = 27, PT_ADJ_MAX_COEF = 16;
enum { ADJ_OVF_SEG = 1, ADJ_OVF_CK = 2, ADJ_CANCELLED = 64, ADJ_UNSUPPORTED = 8 };
}

using namespace ptk;


/* ================================================================== */
/* host side                                                          */
/* ================================================================== */
namespace {
thread_local std::string g_create_err;

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};
} // namespace

struct pt_ctx {
    int device = 0;
    std::string err;
    DScene scene;
    /* the scene's triangles in the caller's order (the surface sources pick
     * them by area in that order; the device copy is in BVH order) */
    std::vector<double> host_tris;
    std::vector<int32_t> host_tri_solid;
    std::vector<void *> allocs;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evs0 = nullptr, evs1 = nullptr;
    int *cancel_host = nullptr;
    int *cancel_dev = nullptr;
    DCounters *counters = nullptr;
    DCounters *counters_host = nullptr;
    DSched *sched_host = nullptr;   /* pinned copy of a batch's scheduler state */
    /* the autotuner's scores per kind of run (index: field precision x
     * neutral FP32-table right-hand side), kept for later batches */
    double tune_score[4][4] = {};
    int sm_count = 0;
    /* device arena kept between pt_integrate calls (their batches are
     * created and destroyed inside the call) */
    void *arena = nullptr;
    size_t arena_bytes = 0;
    /* event logs of the last run that asked for them (pt_log_read) */
    double *log_hit = nullptr, *log_snap = nullptr, *log_track = nullptr, *log_spin = nullptr, *log_snap_t = nullptr;
    unsigned long long *log_n = nullptr; /* [0] hits, [1] snapshots, [2] track points, [3] spin points */
    long long log_cap_hit = 0, log_cap_snap = 0, log_cap_track = 0, log_cap_spin = 0, log_cap = 0;
    bool log_hit_on = false, log_snap_on = false, log_track_on = false, log_spin_on = false;
};

/* Scratch of pt_segment_collisions_noalloc: a fixed device array in the
 * module's own data (allocated when the module loads, never by a call).  All
 * contexts on a device share it, so calls must not overlap.  Nothing in it
 * needs to start at zero: k_collisions writes every segment's count and the
 * result slots below min(count, max_hits); the slots after those keep values
 * from earlier calls, as the allocating entry point leaves them undefined. */
#define PT_NOALLOC_SCRATCH_BYTES (8ull << 20)
static __device__ __align__(256) unsigned char g_noalloc_scratch[PT_NOALLOC_SCRATCH_BYTES];

namespace {
/* device address of g_noalloc_scratch, resolved with that device current on
 * the first no-alloc call after a pt_create on the device (pt_create clears
 * the entry: a context created after a cudaDeviceReset must not inherit the
 * address of the module's previous load) */
std::mutex g_noalloc_mu;
unsigned char *g_noalloc_addr[64] = {};
void noalloc_forget(int device) {
    if (device < 0 || device >= 64) return;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    g_noalloc_addr[device] = nullptr;
}
cudaError_t noalloc_scratch(int device, unsigned char **out) {
    if (device < 0 || device >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e) return e;
        g_noalloc_addr[device] = (unsigned char *)p;
    }
    *out = g_noalloc_addr[device];
    return cudaSuccess;
}
} // namespace

struct pt_batch {
    pt_ctx *ctx = nullptr;
    DBatch b{};
    DRun run{};
    std::vector<double> spintimes;
    std::vector<void *> allocs;   /* owned device memory (one arena) */
    int max_launches = 0;
    double timeout_s = 0;
    int period_iters = 0;   /* persistent form: outer iterations per graph launch (0 = 64) */
    int max_run = 0;        /* persistent scheduler: consecutive steps per lane and particle (0 = budget only) */
    int scheduler = 0;      /* batched form: 0 autotuned, else SCHED_* + 1 */
    int sched_choice = 0;   /* the autotuner's choice for this batch (SCHED_* + 1; 0 = not tuned yet) */
    double tune_score[4] = {0, 0, 0, 0}; /* device ns per RK try measured for each scheduler */
    double tune_ns[4] = {0, 0, 0, 0}, tune_tries[4] = {0, 0, 0, 0}; /* trial sums per scheduler */
    int tune_windows[4] = {0, 0, 0, 0};                               /* trial windows run per scheduler */
};

namespace {

bool ck(pt_ctx *c, cudaError_t e, const char *what) {
    if (e == cudaSuccess) return true;
    if (c) c->err = std::string(what) + ": " + cudaGetErrorString(e);
    else g_create_err = std::string(what) + ": " + cudaGetErrorString(e);
    return false;
}

template <class T> T *dalloc(std::vector<void *> &list, size_t count, cudaError_t &e) {
    void *p = nullptr;
    e = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
    if (e == cudaSuccess) list.push_back(p);
    return (T *)p;
}

template <class T> T *dupload(std::vector<void *> &list, const T *src, size_t count, cudaError_t &e) {
    T *d = dalloc<T>(list, count, e);
    if (e != cudaSuccess) return nullptr;
    if (count) e = cudaMemcpy(d, src, count * sizeof(T), cudaMemcpyHostToDevice);
    return d;
}

DSpecies make_species(int s) {
    DSpecies d{};
    d.kind = s;
    if (s == PT_PROTON) {
        d.q = PT_PROTON_Q; d.m = PT_PROTON_M; d.mu = PT_PROTON_MU; d.gamma = PT_PROTON_GAMMA; d.inv_mkg = PT_PROTON_INV_MKG;
        d.fgrav = PT_PROTON_FGRAV; d.mu_over_e = PT_PROTON_MU_OVER_E; d.q_over_e = PT_PROTON_Q_OVER_E; d.mc2 = PT_PROTON_MC2; d.mg = PT_PROTON_MG;
    } else if (s == PT_ELECTRON) {
        d.q = PT_ELECTRON_Q; d.m = PT_ELECTRON_M; d.mu = PT_ELECTRON_MU; d.gamma = PT_ELECTRON_GAMMA; d.inv_mkg = PT_ELECTRON_INV_MKG;
        d.fgrav = PT_ELECTRON_FGRAV; d.mu_over_e = PT_ELECTRON_MU_OVER_E; d.q_over_e = PT_ELECTRON_Q_OVER_E; d.mc2 = PT_ELECTRON_MC2; d.mg = PT_ELECTRON_MG;
    } else {
        d.kind = PT_NEUTRON;
        d.q = PT_NEUTRON_Q; d.m = PT_NEUTRON_M; d.mu = PT_NEUTRON_MU; d.gamma = PT_NEUTRON_GAMMA; d.inv_mkg = PT_NEUTRON_INV_MKG;
        d.fgrav = PT_NEUTRON_FGRAV; d.mu_over_e = PT_NEUTRON_MU_OVER_E; d.q_over_e = PT_NEUTRON_Q_OVER_E; d.mc2 = PT_NEUTRON_MC2; d.mg = PT_NEUTRON_MG;
    }
    d.muf = (float)d.mu;
    return d;
}

/* Host-side checks of the materials (the reference's operator>> for
 * material, src/geometry.cpp:10-52): probabilities in 0..1 and at most one
 * diffuse-reflection model (Lambert, MicroRoughness, modified Lambert); run
 * by pt_create before it touches a device. */
pt_status validate_materials(const pt_scene_desc *d, std::string &err) {
    if (!d || d->n_materials < 0 || (d->n_materials > 0 && !d->materials)) { err = "materials missing"; return PT_ERR_INVALID; }
    for (int i = 0; i < d->n_materials; ++i) {
        const pt_material &m = d->materials[i];
        if (m.diff_prob < 0 || m.diff_prob > 1 || m.spinflip_prob < 0 || m.spinflip_prob > 1 || m.modified_lambert_prob < 0 ||
            m.modified_lambert_prob > 1 || m.loss_per_bounce < 0 || m.loss_per_bounce > 1) {
            err = "material " + std::to_string(i) + ": probability outside 0..1";
            return PT_ERR_INVALID;
        }
        const int models = (m.diff_prob != 0) + (m.rms_roughness != 0 || m.correl_length != 0) + (m.modified_lambert_prob != 0);
        if (models > 1) {
            err = "You have set parameters for more than one diffuse-reflection model for material " + std::to_string(i) +
                  "! Now I don't know which to use.";
            return PT_ERR_INVALID;
        }
        if (m.rms_roughness < 0 || m.correl_length < 0) {
            err = "material " + std::to_string(i) + ": negative roughness or correlation length";
            return PT_ERR_INVALID;
        }
    }
    return PT_OK;
}

pt_status build_scene(pt_ctx *c, const pt_scene_desc *d) {
    cudaError_t e = cudaSuccess;
    std::string &err = c->err;
    if (!d || d->n_solids < 1 || !d->solids || d->solids[0].id != 1) { err = "solids[0] must be the default solid with ID 1"; return PT_ERR_INVALID; }
    if (d->n_solids > PT_MAX_SOLIDS) { err = "at most 64 solids are supported"; return PT_ERR_UNSUPPORTED; }
    if (d->n_fields > PT_MAX_FIELDS) { err = "at most 8 fields are supported"; return PT_ERR_UNSUPPORTED; }
    if (d->n_triangles > 0 && (!d->triangles || !d->triangle_solid)) { err = "triangles missing"; return PT_ERR_INVALID; }
    c->host_tris.assign(d->triangles, d->triangles + 9 * d->n_triangles);
    c->host_tri_solid.assign(d->triangle_solid, d->triangle_solid + d->n_triangles);
    /* materials */
    std::vector<DMat> mats(d->n_materials);
    for (int i = 0; i < d->n_materials; ++i) {
        const pt_material &m = d->materials[i];
        mats[i] = DMat{m.fermi_real, m.fermi_imag, m.diff_prob,     m.spinflip_prob, m.internal_bfield, m.modified_lambert_prob,
                       m.loss_per_bounce, m.rms_roughness, m.correl_length};
    }
    /* solids */
    std::vector<DSolid> solids(d->n_solids);
    for (int i = 0; i < d->n_solids; ++i) {
        const pt_solid &s = d->solids[i];
        DSolid &o = solids[i];
        std::memset(&o, 0, sizeof(o));
        o.id = s.id;
        o.mat = s.material;
        if (s.material < 0 || s.material >= d->n_materials) { err = "solid references an undefined material"; return PT_ERR_INVALID; }
        if (s.n_ignore > PT_MAX_IGNORE) { err = "at most 4 ignore intervals per solid"; return PT_ERR_UNSUPPORTED; }
        o.n_ign = s.n_ignore;
        for (int k = 0; k < 2 * s.n_ignore; ++k) o.ign[k] = s.ignore_times[k];
        for (int k = 0; k < 3; ++k) { o.lo[k] = 1e300; o.hi[k] = -1e300; }
        for (int j = 0; j < i; ++j)
            if (solids[j].id == o.id) { err = "solid IDs must be unique"; return PT_ERR_INVALID; }
    }
    /* triangles */
    std::vector<pth::HostTri> tris((size_t)d->n_triangles);
    double zmax = -1e300;
    for (int64_t t = 0; t < d->n_triangles; ++t) {
        pth::HostTri &h = tris[t];
        const double *v = d->triangles + 9 * t;
        for (int k = 0; k < 3; ++k) { h.a[k] = v[k]; h.b[k] = v[3 + k]; h.c[k] = v[6 + k]; }
        double e1[3] = {h.b[0] - h.a[0], h.b[1] - h.a[1], h.b[2] - h.a[2]};
        double e2[3] = {h.c[0] - h.a[0], h.c[1] - h.a[1], h.c[2] - h.a[2]};
        double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        double nl = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        for (int k = 0; k < 3; ++k) h.n[k] = n[k] / nl;
        h.solid = d->triangle_solid[t];
        h.pad = 0;
        if (h.solid <= 0 || h.solid >= d->n_solids) { err = "triangle solid index out of range"; return PT_ERR_INVALID; }
        DSolid &so = solids[h.solid];
        for (int k = 0; k < 3; ++k) {
            so.lo[k] = std::min(so.lo[k], std::min(h.a[k], std::min(h.b[k], h.c[k])));
            so.hi[k] = std::max(so.hi[k], std::max(h.a[k], std::max(h.b[k], h.c[k])));
        }
        zmax = std::max(zmax, std::max(h.a[2], std::max(h.b[2], h.c[2])));
    }
    std::vector<pth::HostNode> nodes;
    pth::build_bvh(tris, nodes);
    static_assert(sizeof(pth::HostTri) == sizeof(DTri), "triangle layout");
    static_assert(sizeof(pth::HostNode) == sizeof(DNode), "node layout");
    DScene &S = c->scene;
    std::memset(&S, 0, sizeof(S));
    S.n_tris = (int)tris.size();
    S.n_nodes = (int)nodes.size();
    S.n_solids = d->n_solids;
    S.n_mats = d->n_materials;
    S.n_fields = d->n_fields;
    S.mesh_zmax = tris.empty() ? 0.0 : zmax;
    S.tris = (const DTri *)dupload(c->allocs, (const DTri *)tris.data(), tris.size(), e);
    if (e) return ck(c, e, "upload triangles"), PT_ERR_CUDA;
    {
        /* FP32 planes for the side pre-test, in BVH triangle order */
        std::vector<DTri32> t32(tris.size());
        for (size_t k = 0; k < tris.size(); ++k) {
            double m = 0;
            for (int a = 0; a < 3; ++a) {
                t32[k].a[a] = (float)tris[k].a[a];
                t32[k].b[a] = (float)tris[k].b[a];
                t32[k].c[a] = (float)tris[k].c[a];
                t32[k].n[a] = (float)tris[k].n[a];
                m = std::max(m, std::max(std::fabs(tris[k].a[a]), std::max(std::fabs(tris[k].b[a]), std::fabs(tris[k].c[a]))));
            }
            t32[k].m = std::nextafter((float)m, INFINITY);
            t32[k].pad[0] = t32[k].pad[1] = t32[k].pad[2] = 0;
        }
        S.tri32 = dupload(c->allocs, t32.data(), t32.size(), e);
        if (e) return ck(c, e, "upload triangle planes"), PT_ERR_CUDA;
        /* FP64 normals with error bounds and canonical edges for seg_tri64c */
        std::vector<DTriC> tc(tris.size());
        const double eps = std::ldexp(1.0, -53);
        for (size_t k = 0; k < tris.size(); ++k) {
            const pth::HostTri &h = tris[k];
            DTriC &q = tc[k];
            std::memset(&q, 0, sizeof(q));
            double e1[3], e2[3];
            for (int a = 0; a < 3; ++a) { e1[a] = h.b[a] - h.a[a]; e2[a] = h.c[a] - h.a[a]; }
            double dn = 0, n1 = 0, ea = 0;
            for (int a = 0; a < 3; ++a) {
                const int i1 = (a + 1) % 3, i2 = (a + 2) % 3;
                const double p1 = e1[i1] * e2[i2], p2 = e1[i2] * e2[i1];
                q.n[a] = p1 - p2;
                dn = std::max(dn, 5 * eps * (std::fabs(p1) + std::fabs(p2)) * (1 + 1e-10));
                n1 += std::fabs(q.n[a]);
                ea = std::max(ea, std::max(std::fabs(e1[a]), std::fabs(e2[a])));
            }
            q.dn = std::nextafter((float)dn, INFINITY);
            q.n1 = std::nextafter((float)(n1 * (1 + 1e-12)), INFINITY);
            q.ea = std::nextafter((float)ea, INFINITY);
            const double *V[3] = {h.a, h.b, h.c};
            int edges = 0;
            for (int j = 0; j < 3; ++j) {
                const int iu = j, iv = (j + 1) % 3;
                const double *u = V[iu], *v = V[iv];
                const bool swap = (v[0] != u[0]) ? v[0] < u[0] : ((v[1] != u[1]) ? v[1] < u[1] : v[2] < u[2]);
                const int cu = swap ? iv : iu, cv = swap ? iu : iv;
                edges |= cv << (2 * j);
                if (swap) edges |= 1 << (6 + j);
                double en = 0;
                for (int a = 0; a < 3; ++a) {
                    const double d = V[cu][a] - V[cv][a];
                    q.e[j][a] = (float)d;
                    en = std::max(en, std::fabs(d));
                }
                q.en[j] = std::nextafter((float)en, INFINITY);
            }
            q.edges = edges;
        }
        S.tric = dupload(c->allocs, tc.data(), tc.size(), e);
        if (e) return ck(c, e, "upload triangle certificates"), PT_ERR_CUDA;
    }
    S.nodes = (const DNode *)dupload(c->allocs, (const DNode *)nodes.data(), nodes.size(), e);
    if (e) return ck(c, e, "upload bvh"), PT_ERR_CUDA;
    S.solids = dupload(c->allocs, solids.data(), solids.size(), e);
    if (e) return ck(c, e, "upload solids"), PT_ERR_CUDA;
    S.mats = dupload(c->allocs, mats.data(), mats.size(), e);
    if (e) return ck(c, e, "upload materials"), PT_ERR_CUDA;
    /* fields */
    for (int fi = 0; fi < d->n_fields; ++fi) {
        const pt_field &f = d->fields[fi];
        DField &o = S.fields[fi];
        std::memset(&o, 0, sizeof(o));
        o.type = f.type;
        o.bscale = f.b_scale; o.escale = f.e_scale;
        o.xmax = f.xmax; o.xmin = f.xmin; o.ymax = f.ymax; o.ymin = f.ymin; o.zmax = f.zmax; o.zmin = f.zmin;
        o.bw = f.boundary_width;
        if (o.bw < 0 || (o.xmin < o.xmax && o.ymin < o.ymax && o.zmin < o.zmax &&
                         (o.bw > (o.xmax - o.xmin) / 2 || o.bw > (o.ymax - o.ymin) / 2 || o.bw > (o.zmax - o.zmin) / 2))) {
            err = "You defined a field with an invalid boundary. Check field parameters.";
            return PT_ERR_INVALID;
        }
        if (f.type == PT_FIELD_TAB3D) {
            if (f.nx < 2 || f.ny < 2 || f.nz < 2 || !f.x || !f.y || !f.z) { err = "3D table needs at least 2 points per axis"; return PT_ERR_INVALID; }
            std::vector<double> ax[3] = {std::vector<double>(f.x, f.x + f.nx), std::vector<double>(f.y, f.y + f.ny),
                                         std::vector<double>(f.z, f.z + f.nz)};
            for (int a = 0; a < 3; ++a)
                for (size_t k = 1; k < ax[a].size(); ++k)
                    if (!(ax[a][k] > ax[a][k - 1])) { err = "3D table axes must be strictly increasing"; return PT_ERR_INVALID; }
            o.has_b = (f.bx || f.by || f.bz) ? 1 : 0;
            o.has_v = f.v ? 1 : 0;
            o.ncomp = o.has_v ? 4 : 3;
            size_t tot = (size_t)f.nx * f.ny * f.nz;
            std::vector<double> nd(tot * o.ncomp * 8, 0.0);
            std::vector<double> zero(tot, 0.0);
            const double *comp[4] = {f.bx, f.by, f.bz, f.v};
            for (int k = 0; k < o.ncomp; ++k) pth::hermite_nodes(ax, comp[k] ? comp[k] : zero.data(), k, o.ncomp * 8, nd);
            o.node64 = dupload(c->allocs, nd.data(), nd.size(), e);
            if (e) return ck(c, e, "upload table"), PT_ERR_CUDA;
            {
                std::vector<float> n32;
                o.node32_stride = pth::node_table32(nd, o.ncomp, n32);
                o.node32 = dupload(c->allocs, n32.data(), n32.size(), e);
                if (e) return ck(c, e, "upload FP32 node table"), PT_ERR_CUDA;
            }
            int n3[3] = {f.nx, f.ny, f.nz};
            for (int a = 0; a < 3; ++a) {
                o.n[a] = n3[a];
                o.ax[a] = dupload(c->allocs, ax[a].data(), ax[a].size(), e);
                if (e) return ck(c, e, "upload axis"), PT_ERR_CUDA;
                o.a0[a] = ax[a][0];
                o.inv_h[a] = (double)(ax[a].size() - 1) / (ax[a].back() - ax[a][0]);
                std::vector<double> iw(ax[a].size() - 1);
                for (size_t k = 0; k + 1 < ax[a].size(); ++k) iw[k] = 1.0 / (ax[a][k + 1] - ax[a][k]);
                o.inv_w[a] = dupload(c->allocs, iw.data(), iw.size(), e);
                if (e) return ck(c, e, "upload axis"), PT_ERR_CUDA;
                std::vector<float> axf(ax[a].begin(), ax[a].end()), iwf(iw.begin(), iw.end());
                o.ax32[a] = dupload(c->allocs, axf.data(), axf.size(), e);
                if (e) return ck(c, e, "upload axis"), PT_ERR_CUDA;
                o.inv_w32[a] = dupload(c->allocs, iwf.data(), iwf.size(), e);
                if (e) return ck(c, e, "upload axis"), PT_ERR_CUDA;
                o.a0f[a] = (float)o.a0[a];
                o.inv_hf[a] = (float)o.inv_h[a];
            }
        } else if (f.type == PT_FIELD_TAB2D) {
            if (f.nx < 2 || f.nz < 2 || !f.x || !f.z) { err = "2D table needs at least 2 points per axis"; return PT_ERR_INVALID; }
            std::vector<double> ax[2] = {std::vector<double>(f.x, f.x + f.nx), std::vector<double>(f.z, f.z + f.nz)};
            for (int a = 0; a < 2; ++a)
                for (size_t k = 1; k < ax[a].size(); ++k)
                    if (!(ax[a][k] > ax[a][k - 1])) { err = "2D table axes must be strictly increasing"; return PT_ERR_INVALID; }
            /* an E map makes TabField ignore the potential (src/field_2d.cpp:262-283) */
            const bool etab = f.er || f.ephi || f.ez;
            const double *comp[PT_T2_NCOMP] = {f.bx, f.by, f.bz, etab ? nullptr : f.v, f.er, f.ephi, f.ez};
            const size_t tot = (size_t)f.nx * f.nz;
            std::vector<double> nd(tot * PT_T2_NCOMP * 4, 0.0);
            o.t2_mask = 0;
            for (int k = 0; k < PT_T2_NCOMP; ++k)
                if (comp[k]) {
                    pth::bicubic_nodes(ax[0], ax[1], comp[k], k, PT_T2_NCOMP * 4, nd);
                    o.t2_mask |= 1 << k;
                }
            o.has_b = (o.t2_mask & 7) ? 1 : 0;
            o.has_v = (o.t2_mask & 0x78) ? 1 : 0;
            o.node64 = dupload(c->allocs, nd.data(), nd.size(), e);
            if (e) return ck(c, e, "upload 2D table"), PT_ERR_CUDA;
            /* TabField::CheckTab's grid origin and first spacing give the
             * range r_lo <= r < r_lo + dr (nr - 1), likewise in z (src/field_2d.cpp:193-200, 291) */
            const double rdist = ax[0][1] - ax[0][0], zdist = ax[1][1] - ax[1][0];
            const double rspan = rdist * (double)(f.nx - 1), zspan = zdist * (double)(f.nz - 1);
            o.t2_lim[0] = ax[0][0];
            o.t2_lim[1] = ax[0][0] + rspan;
            o.t2_lim[2] = ax[1][0];
            o.t2_lim[3] = ax[1][0] + zspan;
            const int axis[2] = {0, 2};
            for (int a = 0; a < 2; ++a) {
                const int k = axis[a];
                o.n[k] = (int)ax[a].size();
                o.ax[k] = dupload(c->allocs, ax[a].data(), ax[a].size(), e);
                if (e) return ck(c, e, "upload 2D axis"), PT_ERR_CUDA;
                o.a0[k] = ax[a][0];
                o.inv_h[k] = (double)(ax[a].size() - 1) / (ax[a].back() - ax[a][0]);
            }
            o.n[1] = 1;
        } else if (f.type == PT_FIELD_HARMONIC) {
            std::vector<double> coef;
            std::vector<int> expo;
            if (!pth::harmonic_polynomial(f.n_coeff, f.l, f.m, f.g, coef, expo, err)) return PT_ERR_INVALID;
            o.has_b = 1;
            o.n_mono = (int)coef.size();
            o.mono_c = dupload(c->allocs, coef.data(), coef.size(), e);
            if (e) return ck(c, e, "upload harmonic"), PT_ERR_CUDA;
            o.mono_e = dupload(c->allocs, expo.data(), expo.size(), e);
            if (e) return ck(c, e, "upload harmonic"), PT_ERR_CUDA;
            {
                /* B = grad Phi and its Jacobian as polynomials over the
                 * monomials of degree <= deg (deg = the degree of B) */
                int deg = 0;
                for (int ex : expo) deg = std::max(deg, (ex & 15) + ((ex >> 4) & 15) + ((ex >> 8) & 15) - 1);
                deg = std::max(deg, 0);
                std::vector<int> mon;
                for (int d = 0; d <= deg; ++d)
                    for (int a = d; a >= 0; --a)
                        for (int bb = d - a; bb >= 0; --bb) mon.push_back(a | bb << 4 | (d - a - bb) << 8);
                int n1 = 0;
                for (int ex : mon) n1 += ((ex & 15) + ((ex >> 4) & 15) + ((ex >> 8) & 15)) <= deg - 1;
                const int nm = (int)mon.size();
                std::vector<double> hc(9 * (size_t)nm, 0.0);
                auto slot = [&](int a, int bb, int cc) {
                    const int key = a | bb << 4 | cc << 8;
                    for (int k = 0; k < nm; ++k) if (mon[k] == key) return k;
                    return -1;
                };
                for (size_t t = 0; t < coef.size(); ++t) {
                    const int ex = expo[t], ea = ex & 15, eb = (ex >> 4) & 15, ec = (ex >> 8) & 15;
                    const int E[3] = {ea, eb, ec};
                    for (int i = 0; i < 3; ++i) { /* dPhi/dx_i */
                        if (E[i] == 0) continue;
                        int D[3] = {ea, eb, ec};
                        D[i] -= 1;
                        const int k = slot(D[0], D[1], D[2]);
                        if (k >= 0) hc[(size_t)i * nm + k] += coef[t] * E[i];
                    }
                    const int pairs[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
                    for (int q = 0; q < 6; ++q) { /* d2Phi/dx_i dx_j */
                        const int i = pairs[q][0], j = pairs[q][1];
                        int D[3] = {ea, eb, ec};
                        double fct = D[i];
                        D[i] -= 1;
                        if (D[i] < 0) continue;
                        fct *= D[j];
                        D[j] -= 1;
                        if (D[j] < 0) continue;
                        const int k = slot(D[0], D[1], D[2]);
                        if (k >= 0) hc[(size_t)(3 + q) * nm + k] += coef[t] * fct;
                    }
                }
                o.hp_deg = deg;
                o.hp_n = nm;
                o.hp_n1 = n1;
                o.hp_c = dupload(c->allocs, hc.data(), hc.size(), e);
                if (!e) o.hp_e = dupload(c->allocs, mon.data(), mon.size(), e);
                if (e) return ck(c, e, "upload harmonic polynomials"), PT_ERR_CUDA;
            }
            {
                /* one potential per coefficient with G = 1: the basis fields of the adjoint */
                std::vector<double> bc;
                std::vector<int> be, start(1, 0);
                /* and each basis field B_k = grad Phi_k over the field's monomials */
                int deg = o.hp_deg;
                std::vector<int> mon;
                for (int d = 0; d <= deg; ++d)
                    for (int a = d; a >= 0; --a)
                        for (int bb = d - a; bb >= 0; --bb) mon.push_back(a | bb << 4 | (d - a - bb) << 8);
                const int nm = (int)mon.size();
                std::vector<double> bhp((size_t)f.n_coeff * 3 * nm, 0.0);
                for (int k = 0; k < f.n_coeff; ++k) {
                    std::vector<double> ck1;
                    std::vector<int> ek1;
                    const double one = 1.0;
                    if (!pth::harmonic_polynomial(1, f.l + k, f.m + k, &one, ck1, ek1, err)) return PT_ERR_INVALID;
                    for (size_t t = 0; t < ck1.size(); ++t) {
                        const int E[3] = {ek1[t] & 15, (ek1[t] >> 4) & 15, (ek1[t] >> 8) & 15};
                        for (int i = 0; i < 3; ++i) {
                            if (E[i] == 0) continue;
                            int D[3] = {E[0], E[1], E[2]};
                            D[i] -= 1;
                            const int key = D[0] | D[1] << 4 | D[2] << 8;
                            for (int q = 0; q < nm; ++q)
                                if (mon[q] == key) bhp[((size_t)k * 3 + i) * nm + q] += ck1[t] * E[i];
                        }
                    }
                    bc.insert(bc.end(), ck1.begin(), ck1.end());
                    be.insert(be.end(), ek1.begin(), ek1.end());
                    start.push_back((int)bc.size());
                }
                o.n_terms = f.n_coeff;
                o.term_start = dupload(c->allocs, start.data(), start.size(), e);
                if (!e) o.basis_c = dupload(c->allocs, bc.data(), bc.size(), e);
                if (!e) o.basis_e = dupload(c->allocs, be.data(), be.size(), e);
                if (!e) o.basis_hp = dupload(c->allocs, bhp.data(), bhp.size(), e);
                if (e) return ck(c, e, "upload harmonic basis"), PT_ERR_CUDA;
            }
            for (int k = 0; k < 3; ++k) o.offset[k] = f.offset[k];
        } else if (f.type == PT_FIELD_UNIFORM_E) {
            o.has_v = 1;
            for (int k = 0; k < 3; ++k) o.e[k] = f.e[k];
        } else if (f.type == PT_FIELD_SOLENOID) {
            if (!(f.sol_radius > 0) || !(f.sol_half_length > 0)) { err = "solenoid needs a positive radius and half length"; return PT_ERR_INVALID; }
            o.has_b = 1;
            o.sol_a = f.sol_radius;
            o.sol_b = f.sol_half_length;
            o.sol_B0 = f.sol_bcenter * std::sqrt(f.sol_radius * f.sol_radius + f.sol_half_length * f.sol_half_length) /
                       (PT_PI * f.sol_half_length);
            for (int k = 0; k < 3; ++k) o.offset[k] = f.offset[k];
        } else {
            err = "unsupported field type";
            return PT_ERR_UNSUPPORTED;
        }
    }
    return PT_OK;
}

void free_list(std::vector<void *> &l) {
    for (void *p : l) cudaFree(p);
    l.clear();
}

int grid_for(int64_t n, int block) { return (int)((n + block - 1) / block); }

/* Threads per block of the one-lane-per-particle kernels (k_plain,
 * k_plain_spin, k_adj_*): 128, halved down to 32 while the grid would leave
 * SMs without a block.  A small batch then spreads over the SMs one warp or
 * two per SM instead of crowding a few, which matters for the spin kernels:
 * their Bloch steps are FP64 arithmetic, and the FP64 pipes are per SM. */
int lane_block(const pt_ctx *c, int64_t n) {
    int b = 128;
    while (b > 32 && grid_for(n, b) < c->sm_count) b >>= 1;
    return b;
}

void add_counters(pt_stats &acc, const DCounters &k) {
    acc.rk_accepted += k.rk_accepted; acc.rk_rejected += k.rk_rejected; acc.rhs_evals += k.rhs_evals;
    acc.field_evals += k.field_evals; acc.hits += k.hits; acc.bisection_levels += k.bisection_levels;
    acc.bvh_nodes += k.bvh_nodes; acc.tri_tests += k.tri_tests; acc.subsegments += k.subsegments;
    acc.dense_evals += k.dense_evals; acc.particle_seconds += k.particle_seconds;
    acc.bisect_max = std::max<int64_t>(acc.bisect_max, k.bisect_max);
    acc.cand_calls += k.cand_calls; acc.cand_overflow += k.cand_overflow; acc.cand_sum += k.cand_sum; acc.tri32_tests += k.tri32; acc.bisect_dead += k.bisect_dead; acc.spin_steps += k.spin_steps;
}

int persistent_grid(pt_ctx *c, const void *fn, int block) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, block, 0);
    if (per_sm < 1) per_sm = 1;
    return per_sm * c->sm_count;
}

/* whether a run can integrate spins (IntegrateSpin's Bloch integration):
 * a species with a gyromagnetic ratio and a non-empty spin-integration
 * window [start, end) */
bool spin_run(const DRun &R) {
    if (R.sp.gamma == 0) return false;
    for (int i = 0; i + 1 < R.n_spintimes; i += 2)
        if (R.spintimes[i] < R.spintimes[i + 1]) return true;
    return false;
}

/* Plain form: k_plain launches (one lane per particle, up to steps_per_launch
 * LOOP-A iterations or the step budget) until no particle is active; also the
 * tail of the batched form (budgets counted from the call's start). */
pt_status advance_plain(pt_ctx *c, pt_batch *B, const DRun &R, pt_stats &acc, std::chrono::steady_clock::time_point w0,
                        bool &cancelled, bool &timed_out, bool from_nacc0) {
    cudaError_t e;
    const int64_t n = B->b.n;
    const int steps = R.steps_per_launch, block = lane_block(c, n);
    const int max_steps = R.max_steps;
    for (int launch = 0;; ++launch) {
        if ((e = cudaMemsetAsync(c->counters, 0, sizeof(DCounters), c->stream))) return ck(c, e, "memset"), PT_ERR_CUDA;
        cudaEventRecord(c->ev0, c->stream);
        if (spin_run(R)) k_plain_spin<<<grid_for(n, block), block, 0, c->stream>>>(c->scene, R, B->b, c->counters, steps, from_nacc0 ? 1 : 0);
        else k_plain<<<grid_for(n, block), block, 0, c->stream>>>(c->scene, R, B->b, c->counters, steps, from_nacc0 ? 1 : 0);
        cudaEventRecord(c->ev1, c->stream);
        if ((e = cudaGetLastError())) return ck(c, e, "k_plain launch"), PT_ERR_CUDA;
        if ((e = cudaMemcpyAsync(c->counters_host, c->counters, sizeof(DCounters), cudaMemcpyDeviceToHost, c->stream)))
            return ck(c, e, "counters"), PT_ERR_CUDA;
        if ((e = cudaStreamSynchronize(c->stream))) return ck(c, e, "k_plain"), PT_ERR_CUDA;
        float ms = 0;
        cudaEventElapsedTime(&ms, c->ev0, c->ev1);
        const DCounters &k = *c->counters_host;
        acc.kernel_ms += ms;
        acc.dominant_kernel_ms += ms;
        acc.dominant_launches += 1;
        acc.launches += 1;
        add_counters(acc, k);
        acc.active = (int64_t)k.active;
        if (*(volatile int *)c->cancel_host) { cancelled = true; break; }
        if (k.active == 0 || max_steps > 0) break; /* a step budget is one fixed step-batch launch */
        if (B->max_launches > 0 && launch + 1 >= B->max_launches) { timed_out = true; break; }
        if (B->timeout_s > 0 && std::chrono::duration<double>(std::chrono::steady_clock::now() - w0).count() > B->timeout_s) {
            timed_out = true;
            break;
        }
    }
    return PT_OK;
}

/* Batched (phase-split) form: per iteration one RK try for every active
 * particle (k_try), the common completion (k_post) and the full post-step
 * logic for queued steps (k_slow), over work lists in device memory. */
pt_status advance_batched(pt_ctx *c, pt_batch *B, const DRun &R, pt_stats &acc,
                          std::chrono::steady_clock::time_point w0, bool &cancelled, bool &timed_out) {
    cudaError_t e;
    DBatch &b = B->b;
    const int64_t n = b.n;
    const int block = 128;
    /* k_try without the general right-hand side when every magnetic field is
     * an FP32 table and the species is neutral in the FP32 field mode (the
     * same branch bfield32 takes per field) */
    bool tab_only = R.sp.q == 0 && R.prec == PT_PREC_FP32;
    for (int fi = 0; fi < c->scene.n_fields; ++fi) {
        const DField &f = c->scene.fields[fi];
        const bool box = f.xmin < f.xmax && f.ymin < f.ymax && f.zmin < f.zmax;
        if (f.has_b && !(f.type == PT_FIELD_TAB3D && f.node32 && !(f.bw > 0 && box))) tab_only = false;
    }
    /* the 255-register try kernel when the caller names that scheduler */
    const bool wide = B->scheduler == PT_SCHED_PHASED_WIDE;
    const void *try_fn = wide ? (tab_only ? (const void *)k_try_tab32_w : (const void *)k_try_w)
                              : (tab_only ? (const void *)k_try_tab32 : (const void *)k_try);
    const int g_try = persistent_grid(c, try_fn, block);
    const int g_post = persistent_grid(c, (const void *)k_post, block);
    const int g_slow = persistent_grid(c, (const void *)k_slow, block);
    const int g_bisect = persistent_grid(c, (const void *)k_bisect, block);
    if ((e = cudaMemsetAsync(b.count, 0, 8 * sizeof(int32_t), c->stream))) return ck(c, e, "counts"), PT_ERR_CUDA;
    k_gather<<<grid_for(n, 256), 256, 0, c->stream>>>(b, R.t_pause, b.list[0], &b.count[0]);
    if ((e = cudaGetLastError())) return ck(c, e, "gather"), PT_ERR_CUDA;
    acc.aux_launches += 1;
    cudaEvent_t ev[6];
    for (int k = 0; k < 6; ++k) cudaEventCreate(&ev[k]);
    double t_try = 0, t_post = 0, t_slow = 0, t_bisect = 0;
    int64_t l_try = 0;
    int32_t *hcount = nullptr;
    cudaHostAlloc((void **)&hcount, 8 * sizeof(int32_t), 0);
    pt_status st = PT_OK;
    /* Steps that need the full post-step logic (hits, splits, clipping) wait in
     * the slow list while the others keep stepping; k_slow runs once the list
     * is large enough to fill the GPU, or when nothing else is active.  Each
     * particle still executes its own operations in its own order, so the
     * results equal the plain form's bit for bit. */
    int64_t l_slow = 0;
    /* Once few particles remain, iterations cost mostly launch latency: the
     * queue is drained and the rest runs as plain-form lanes (same
     * per-particle arithmetic, so the same bits). */
    const int tail = (int)std::max<int64_t>(2048, n / 1000);
    bool to_plain = false;
    for (int it = 0;; ++it) {
        const int in = it & 1, out = in ^ 1;
        if ((e = cudaMemsetAsync(c->counters, 0, sizeof(DCounters), c->stream))) { ck(c, e, "memset"); st = PT_ERR_CUDA; break; }
        if (it > 0) {
            k_zero_counts<<<1, 32, 0, c->stream>>>(b.count, in, in, in);
            k_regather<<<grid_for(n, 256), 256, 0, c->stream>>>(b, R.t_pause, R.max_steps, b.list[in], &b.count[in]);
            acc.aux_launches += 2;
        }
        k_zero_counts<<<1, 32, 0, c->stream>>>(b.count, out, 2, 2);
        acc.aux_launches += 1;
        cudaEventRecord(ev[0], c->stream);
        if (wide && tab_only) k_try_tab32_w<<<g_try, block, 0, c->stream>>>(c->scene, R, b, c->counters, in, out, nullptr);
        else if (wide) k_try_w<<<g_try, block, 0, c->stream>>>(c->scene, R, b, c->counters, in, out, nullptr);
        else if (tab_only) k_try_tab32<<<g_try, block, 0, c->stream>>>(c->scene, R, b, c->counters, in, out, nullptr);
        else k_try<<<g_try, block, 0, c->stream>>>(c->scene, R, b, c->counters, in, out, nullptr);
        cudaEventRecord(ev[1], c->stream);
        k_post<<<g_post, block, 0, c->stream>>>(c->scene, R, b, c->counters, out, nullptr);
        cudaEventRecord(ev[2], c->stream);
        if ((e = cudaGetLastError())) { ck(c, e, "batched launch"); st = PT_ERR_CUDA; break; }
        cudaMemcpyAsync(hcount, b.count, 8 * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream);
        if ((e = cudaStreamSynchronize(c->stream))) { ck(c, e, "batched iteration"); st = PT_ERR_CUDA; break; }
        float a = 0, bb = 0;
        cudaEventElapsedTime(&a, ev[0], ev[1]);
        cudaEventElapsedTime(&bb, ev[1], ev[2]);
        t_try += a; t_post += bb;
        ++l_try;
        acc.kernel_ms += a + bb;
        acc.launches += 2;
        int active = hcount[out], slow = hcount[3];
        /* rounds of k_slow (each queued post-step runs to its end or to its
         * next bisection) and k_bisect, while the queue fills the GPU */
        while (slow > 0 && (slow >= std::max(2048, active / 4) || active == 0 || active <= tail)) {
            cudaEventRecord(ev[3], c->stream);
            k_slow<<<g_slow, block, 0, c->stream>>>(c->scene, R, b, c->counters, out, nullptr);
            cudaEventRecord(ev[4], c->stream);
            k_zero_counts<<<1, 32, 0, c->stream>>>(b.count, 3, 5, 5);
            k_bisect<<<g_bisect, block, 0, c->stream>>>(c->scene, R, b, c->counters, nullptr);
            cudaEventRecord(ev[5], c->stream);
            k_zero_counts<<<1, 32, 0, c->stream>>>(b.count, 4, 4, 4);
            acc.aux_launches += 2;
            if ((e = cudaGetLastError())) { ck(c, e, "k_slow launch"); st = PT_ERR_CUDA; break; }
            cudaMemcpyAsync(hcount, b.count, 8 * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream);
            if ((e = cudaStreamSynchronize(c->stream))) { ck(c, e, "k_slow"); st = PT_ERR_CUDA; break; }
            float cc = 0, cb = 0;
            cudaEventElapsedTime(&cc, ev[3], ev[4]);
            cudaEventElapsedTime(&cb, ev[4], ev[5]);
            t_slow += cc;
            t_bisect += cb;
            ++l_slow;
            acc.kernel_ms += cc + cb;
            acc.launches += 2;
            active = hcount[out];
            slow = hcount[3];
        }
        if (st != PT_OK) break;
        cudaMemcpy(c->counters_host, c->counters, sizeof(DCounters), cudaMemcpyDeviceToHost);
        add_counters(acc, *c->counters_host);
        acc.active = active + slow;
        if (*(volatile int *)c->cancel_host) { cancelled = true; break; }
        if (active == 0 && slow == 0) break;
        if (active <= tail && slow == 0) { to_plain = true; break; }
        if (B->max_launches > 0 && acc.launches >= B->max_launches) { timed_out = true; break; }
        if (B->timeout_s > 0 && std::chrono::duration<double>(std::chrono::steady_clock::now() - w0).count() > B->timeout_s) {
            timed_out = true;
            break;
        }
    }
    for (int k = 0; k < 6; ++k) cudaEventDestroy(ev[k]);
    cudaFreeHost(hcount);
    if (st == PT_OK && to_plain && !cancelled && !timed_out) {
        const double k0 = acc.kernel_ms;
        st = advance_plain(c, B, R, acc, w0, cancelled, timed_out, true);
        acc.tail_ms = acc.kernel_ms - k0;
    }
    const char *name = tab_only ? (wide ? "k_try_tab32_w" : "k_try_tab32") : (wide ? "k_try_w" : "k_try");
    double dom = t_try;
    if (t_post > dom) { dom = t_post; name = "k_post"; }
    if (t_slow > dom) { dom = t_slow; name = "k_slow"; }
    if (t_bisect > dom) { dom = t_bisect; name = "k_bisect"; }
    acc.dominant_kernel_ms = dom;
    acc.dominant_launches = (dom == t_slow || dom == t_bisect) ? l_slow : l_try;
    std::snprintf(acc.dominant_kernel, sizeof(acc.dominant_kernel), "%s", name);
    acc.try_ms = t_try;
    acc.post_ms = t_post;
    acc.slow_ms = t_slow;
    acc.bisect_ms = t_bisect;
    return st;
}

/* Adds a conditional node of `type` to the graph the stream is capturing,
 * after the captured work so far, and continues the capture after it;
 * returns the node's body graph. */
cudaError_t capture_conditional(cudaStream_t s, cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type, cudaGraph_t *body) {
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    const cudaGraphEdgeData *edges = nullptr;
    size_t nd = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, &deps, &edges, &nd);
    if (e) return e;
    if (cs != cudaStreamCaptureStatusActive) return cudaErrorIllegalState;
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = type;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    if ((e = cudaGraphAddNode(&node, g, deps, edges, nd, &p))) return e;
    *body = p.conditional.phGraph_out[0];
    return cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
}

/* The batched form's iteration bodies (schedulers), all run as a CUDA
 * graph whose loops the device schedules:
 *   SCHED_PHASED:  k_regather, k_try, k_post, slow rounds while the slow
 *                  list fills the GPU
 *   SCHED_RUN:     k_regather, k_run (persistent lanes refilled from the
 *                  active list, 168 registers), slow rounds until the slow
 *                  list is empty
 *   SCHED_RUN_WIDE: the same with the 255-register instance of k_run
 *   SCHED_PHASED_WIDE: SCHED_PHASED with the 255-register instance of k_try
 * Every body schedules each particle's own operations in its own order, so
 * all give the plain form's results bit for bit. */
enum { SCHED_PHASED = 0, SCHED_RUN = 1, SCHED_RUN_WIDE = 2, SCHED_PHASED_WIDE = 3, SCHED_VARIANTS = 4 };
static bool sched_phased(int v) { return v == SCHED_PHASED || v == SCHED_PHASED_WIDE; }

/* Builds the graph of one scheduler: a period kernel, then a WHILE node
 * over iterations with an inner WHILE node over slow rounds. */
cudaError_t build_graph(pt_ctx *c, pt_batch *B, const DRun &R, int v, bool tab_only, cudaGraph_t *gout, cudaGraphExec_t *xout) {
    DBatch &b = B->b;
    const int64_t n = b.n;
    const int block = 128;
    cudaError_t e;
    cudaGraph_t g = nullptr;
    if ((e = cudaGraphCreate(&g, 0))) return e;
    *gout = g;
    cudaGraphConditionalHandle h_outer, h_slow;
    if ((e = cudaGraphConditionalHandleCreate(&h_outer, g, 1, cudaGraphCondAssignDefault)) ||
        (e = cudaGraphConditionalHandleCreate(&h_slow, g, 0, 0)))
        return e;
    cudaGraph_t body_outer = nullptr, body_slow = nullptr, tmp = nullptr;
    if ((e = cudaStreamBeginCaptureToGraph(c->stream, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal))) return e;
    k_sched_period<<<1, 32, 0, c->stream>>>(b.sched);
    e = capture_conditional(c->stream, h_outer, cudaGraphCondTypeWhile, &body_outer);
    cudaError_t e2 = cudaStreamEndCapture(c->stream, &tmp);
    if (e || (e = e2)) return e;
    if ((e = cudaStreamBeginCaptureToGraph(c->stream, body_outer, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal))) return e;
    k_sched_begin<<<1, 32, 0, c->stream>>>(b, b.sched);
    k_regather<<<grid_for(n, 256), 256, 0, c->stream>>>(b, R.t_pause, R.max_steps, b.list[0], &b.count[0]);
    if (sched_phased(v)) {
        const bool wide = v == SCHED_PHASED_WIDE;
        const void *try_fn = wide ? (tab_only ? (const void *)k_try_tab32_w : (const void *)k_try_w)
                                  : (tab_only ? (const void *)k_try_tab32 : (const void *)k_try);
        const int g_try = persistent_grid(c, try_fn, block), g_post = persistent_grid(c, (const void *)k_post, block);
        if (wide && tab_only) k_try_tab32_w<<<g_try, block, 0, c->stream>>>(c->scene, R, b, c->counters, 0, 1, b.sched);
        else if (wide) k_try_w<<<g_try, block, 0, c->stream>>>(c->scene, R, b, c->counters, 0, 1, b.sched);
        else if (tab_only) k_try_tab32<<<g_try, block, 0, c->stream>>>(c->scene, R, b, c->counters, 0, 1, b.sched);
        else k_try<<<g_try, block, 0, c->stream>>>(c->scene, R, b, c->counters, 0, 1, b.sched);
        k_post<<<g_post, block, 0, c->stream>>>(c->scene, R, b, c->counters, 1, b.sched);
        k_sched_after_post<<<1, 32, 0, c->stream>>>(b, b.sched, h_slow);
    } else {
        const bool wide = v == SCHED_RUN_WIDE;
        const void *run_fn = wide ? (tab_only ? (const void *)k_run2_tab32 : (const void *)k_run2)
                                  : (tab_only ? (const void *)k_run_tab32 : (const void *)k_run);
        const int g_run = persistent_grid(c, run_fn, block);
        if (wide && tab_only) k_run2_tab32<<<g_run, block, 0, c->stream>>>(c->scene, R, b, c->counters, b.sched, B->max_run);
        else if (wide) k_run2<<<g_run, block, 0, c->stream>>>(c->scene, R, b, c->counters, b.sched, B->max_run);
        else if (tab_only) k_run_tab32<<<g_run, block, 0, c->stream>>>(c->scene, R, b, c->counters, b.sched, B->max_run);
        else k_run<<<g_run, block, 0, c->stream>>>(c->scene, R, b, c->counters, b.sched, B->max_run);
        k_sched_after_run<<<1, 32, 0, c->stream>>>(b, b.sched, h_slow);
    }
    e = capture_conditional(c->stream, h_slow, cudaGraphCondTypeWhile, &body_slow);
    if (!e) {
        if (sched_phased(v)) k_sched_end_phased<<<1, 32, 0, c->stream>>>(b, b.sched, R, h_outer);
        else k_sched_end<<<1, 32, 0, c->stream>>>(b, b.sched, R, h_outer);
    }
    e2 = cudaStreamEndCapture(c->stream, &tmp);
    if (e || (e = e2)) return e;
    if ((e = cudaStreamBeginCaptureToGraph(c->stream, body_slow, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal))) return e;
    const int g_slow = persistent_grid(c, (const void *)k_slow, block), g_bisect = persistent_grid(c, (const void *)k_bisect, block);
    k_slow<<<g_slow, block, 0, c->stream>>>(c->scene, R, b, c->counters, 1, b.sched);
    k_zero_counts<<<1, 32, 0, c->stream>>>(b.count, 3, 5, 5);
    k_bisect<<<g_bisect, block, 0, c->stream>>>(c->scene, R, b, c->counters, b.sched);
    k_zero_counts<<<1, 32, 0, c->stream>>>(b.count, 4, 4, 4);
    if (sched_phased(v)) k_sched_after_slow_phased<<<1, 32, 0, c->stream>>>(b, b.sched, R, h_slow);
    else k_sched_after_slow<<<1, 32, 0, c->stream>>>(b, b.sched, R, h_slow);
    if ((e = cudaStreamEndCapture(c->stream, &tmp))) return e;
    return cudaGraphInstantiate(xout, g, 0);
}

/* Batched form: the iterations run inside CUDA graphs (one launch per
 * period of at most `period_iters` iterations; the host checks
 * cancellation, launch and time limits between periods) and the last few
 * particles finish as plain-form lanes.  The scheduler is the caller's
 * choice or, when left to the autotuner, measured: the first periods of a
 * batch run a short trial of each scheduler and the one with the least
 * device time per RK try runs from then on (a choice kept by the batch). */
pt_status advance_graph(pt_ctx *c, pt_batch *B, const DRun &R, pt_stats &acc, std::chrono::steady_clock::time_point w0, bool &cancelled,
                        bool &timed_out) {
    cudaError_t e = cudaSuccess;
    DBatch &b = B->b;
    const int64_t n = b.n;
    bool tab_only = R.sp.q == 0 && R.prec == PT_PREC_FP32;
    for (int fi = 0; fi < c->scene.n_fields; ++fi) {
        const DField &f = c->scene.fields[fi];
        const bool box = f.xmin < f.xmax && f.ymin < f.ymax && f.zmin < f.zmax;
        if (f.has_b && !(f.type == PT_FIELD_TAB3D && f.node32 && !(f.bw > 0 && box))) tab_only = false;
    }
    const int tail = (int)std::max<int64_t>(2048, n / 1000);
    const int period_iters = B->period_iters > 0 ? B->period_iters : 64;
    /* Trials run in round robin, TRIAL_WINDOWS windows of trial_iters
     * iterations per scheduler, and score the sums: each scheduler is then
     * sampled over the same stretch of the batch (a step budget thins the
     * active set towards its end, and the phase split's slow rounds, one
     * every few iterations, fall into some windows and not others). */
    const int trial_iters = 4, TRIAL_WINDOWS = 2;
    /* a batch starts from the scores earlier batches of the same kind
     * measured on this context (measured again only for untried schedulers) */
    double *ctx_score = c->tune_score[(R.prec == PT_PREC_FP32 ? 2 : 0) + (tab_only ? 1 : 0)];
    if (B->scheduler == 0 && B->sched_choice == 0)
        for (int k = 0; k < SCHED_VARIANTS; ++k)
            if (!(B->tune_score[k] > 0) && ctx_score[k] > 0) B->tune_score[k] = ctx_score[k];
    DSched &hs = *c->sched_host;
    std::memset(&hs, 0, sizeof(hs));
    for (int k = 0; k < PT_SPANS; ++k) hs.t0[k] = ~0ull;
    hs.tail = tail;
    hs.max_iters = period_iters;
    if ((e = cudaMemcpyAsync(b.sched, &hs, sizeof(DSched), cudaMemcpyHostToDevice, c->stream)) ||
        (e = cudaMemsetAsync(c->counters, 0, sizeof(DCounters), c->stream)) ||
        (e = cudaMemsetAsync(b.count, 0, 8 * sizeof(int32_t), c->stream)))
        return ck(c, e, "batched setup"), PT_ERR_CUDA;
    /* budgets count from here; suspended post-steps of an earlier call go to list 3 */
    k_gather<<<grid_for(n, 256), 256, 0, c->stream>>>(b, R.t_pause, b.list[0], &b.count[0]);
    acc.aux_launches += 1;
    cudaGraph_t gr[SCHED_VARIANTS] = {};
    cudaGraphExec_t gx[SCHED_VARIANTS] = {};
    pt_status st = PT_OK;
    int64_t iters_of[SCHED_VARIANTS] = {0, 0, 0, 0};
    unsigned long long prev_tries = 0, prev_ns = 0;
    int prev_outer = 0;
    for (int period = 0;; ++period) {
        /* the scheduler of this period */
        int v;
        bool trial = false;
        if (B->scheduler > 0) v = B->scheduler - 1;
        else if (B->sched_choice > 0) v = B->sched_choice - 1;
        else {
            /* the untried scheduler with the fewest windows, in index order in
             * even rounds and in reverse order in odd ones (0 1 2 3 3 2 1 0), so
             * that no scheduler's windows all fall late in a batch */
            int wmin = TRIAL_WINDOWS;
            for (int k = 0; k < SCHED_VARIANTS; ++k)
                if (!(B->tune_score[k] > 0)) wmin = std::min(wmin, B->tune_windows[k]);
            v = -1;
            for (int k = 0; k < SCHED_VARIANTS; ++k) {
                const int kk = (wmin & 1) ? SCHED_VARIANTS - 1 - k : k;
                if (v < 0 && !(B->tune_score[kk] > 0) && B->tune_windows[kk] == wmin && wmin < TRIAL_WINDOWS) v = kk;
            }
            trial = v >= 0;
            if (!trial) {
                for (int k = 0; k < SCHED_VARIANTS; ++k) {
                    if (B->tune_score[k] > 0) continue;
                    /* trials done: score the sums (a scheduler whose windows saw no
                     * try is no candidate for this batch, and nothing is cached) */
                    B->tune_score[k] = B->tune_tries[k] > 0 ? B->tune_ns[k] / B->tune_tries[k] : 1e300;
                    if (B->tune_tries[k] > 0) ctx_score[k] = B->tune_score[k];
                }
                v = 0;
                for (int k = 1; k < SCHED_VARIANTS; ++k)
                    if (B->tune_score[k] < B->tune_score[v]) v = k;
                B->sched_choice = v + 1;
            }
        }
        if (!gx[v]) {
            e = build_graph(c, B, R, v, tab_only, &gr[v], &gx[v]);
            if (e) {
                cudaStreamCaptureStatus cs;
                if (cudaStreamIsCapturing(c->stream, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
                    cudaGraph_t junk = nullptr;
                    cudaStreamEndCapture(c->stream, &junk);
                    if (junk) cudaGraphDestroy(junk);
                }
                ck(c, e, "batched graph");
                st = PT_ERR_CUDA;
                break;
            }
        }
        const int iters = trial ? trial_iters : period_iters;
        if ((e = cudaMemcpyAsync(&b.sched->max_iters, &iters, sizeof(int), cudaMemcpyHostToDevice, c->stream)) ||
            (e = cudaGraphLaunch(gx[v], c->stream))) { ck(c, e, "graph launch"); st = PT_ERR_CUDA; break; }
        acc.graph_launches += 1;
        if ((e = cudaMemcpyAsync(c->sched_host, b.sched, sizeof(DSched), cudaMemcpyDeviceToHost, c->stream)) ||
            (e = cudaMemcpyAsync(c->counters_host, c->counters, sizeof(DCounters), cudaMemcpyDeviceToHost, c->stream)) ||
            (e = cudaStreamSynchronize(c->stream))) { ck(c, e, "batched period"); st = PT_ERR_CUDA; break; }
        unsigned long long ns = 0;
        for (int k = 0; k < PT_SPANS; ++k) ns += hs.ns[k];
        const unsigned long long tries = c->counters_host->rk_accepted + c->counters_host->rk_rejected;
        iters_of[v] += hs.outer_iters - prev_outer;
        if (trial) {
            B->tune_ns[v] += (double)(ns - prev_ns);
            B->tune_tries[v] += (double)(tries - prev_tries);
            B->tune_windows[v] += 1;
        }
        prev_tries = tries;
        prev_ns = ns;
        prev_outer = hs.outer_iters;
        if (hs.error) {
            c->err = "batched scheduler: a slow-round loop exceeded its round limit";
            st = PT_ERR_CUDA;
            break;
        }
        if (*(volatile int *)c->cancel_host) { cancelled = true; break; }
        const bool finished = hs.last_going == 0 && hs.last_slow == 0;
        if (finished || (hs.last_going <= tail && hs.last_slow == 0)) break;
        const int64_t kernels = (int64_t)hs.outer_iters * 5 + (int64_t)hs.inner_iters * 5;
        if (B->max_launches > 0 && kernels >= B->max_launches) { timed_out = true; break; }
        if (B->timeout_s > 0 && std::chrono::duration<double>(std::chrono::steady_clock::now() - w0).count() > B->timeout_s) {
            timed_out = true;
            break;
        }
    }
    for (int k = 0; k < SCHED_VARIANTS; ++k) {
        if (gx[k]) cudaGraphExecDestroy(gx[k]);
        if (gr[k]) cudaGraphDestroy(gr[k]);
    }
    if (st != PT_OK) return st;
    add_counters(acc, *c->counters_host);
    const double run_ms = hs.ns[PT_SPAN_RUN] * 1e-6, try_ms = hs.ns[PT_SPAN_TRY] * 1e-6, post_ms = hs.ns[PT_SPAN_POST] * 1e-6,
                 slow_ms = hs.ns[PT_SPAN_SLOW] * 1e-6, bisect_ms = hs.ns[PT_SPAN_BISECT] * 1e-6;
    acc.kernel_ms += run_ms + try_ms + post_ms + slow_ms + bisect_ms;
    /* kernel executions inside the graphs: the timed kernels (k_run, or k_try
     * and k_post, per iteration; k_slow + k_bisect per slow round) and the
     * bookkeeping ones (scheduling kernels, list rebuild, count resets, one
     * per period) */
    const int64_t run_it = iters_of[SCHED_RUN] + iters_of[SCHED_RUN_WIDE], ph_it = iters_of[SCHED_PHASED] + iters_of[SCHED_PHASED_WIDE];
    acc.launches += run_it + 2 * ph_it + 2 * (int64_t)hs.inner_iters;
    acc.aux_launches += (run_it + ph_it) * 4 + (int64_t)hs.inner_iters * 3 + acc.graph_launches;
    acc.sched_outer_iters = hs.outer_iters;
    acc.sched_inner_iters = hs.inner_iters;
    acc.scheduler = B->scheduler > 0 ? B->scheduler : B->sched_choice;
    for (int k = 0; k < SCHED_VARIANTS; ++k) acc.tune_ns_per_try[k] = B->tune_score[k] < 1e299 ? B->tune_score[k] : 0;
    acc.active = hs.last_going + hs.last_slow;
    if (!cancelled && !timed_out && (hs.last_going > 0 || hs.last_slow > 0)) {
        const double k0 = acc.kernel_ms;
        st = advance_plain(c, B, R, acc, w0, cancelled, timed_out, true);
        acc.tail_ms = acc.kernel_ms - k0;
    }
    /* the dominant kernel and its launches */
    const bool try_wide = iters_of[SCHED_PHASED_WIDE] > iters_of[SCHED_PHASED];
    const char *name = tab_only ? (try_wide ? "k_try_tab32_w" : "k_try_tab32") : (try_wide ? "k_try_w" : "k_try");
    double dom = try_ms;
    int64_t dl = ph_it;
    if (run_ms > dom) {
        dom = run_ms;
        dl = run_it;
        name = iters_of[SCHED_RUN_WIDE] > iters_of[SCHED_RUN] ? (tab_only ? "k_run2_tab32" : "k_run2") : (tab_only ? "k_run_tab32" : "k_run");
    }
    if (post_ms > dom) { dom = post_ms; name = "k_post"; dl = ph_it; }
    if (slow_ms > dom) { dom = slow_ms; name = "k_slow"; dl = hs.inner_iters; }
    if (bisect_ms > dom) { dom = bisect_ms; name = "k_bisect"; dl = hs.inner_iters; }
    acc.dominant_kernel_ms = dom;
    acc.dominant_launches = dl;
    std::snprintf(acc.dominant_kernel, sizeof(acc.dominant_kernel), "%s", name);
    acc.try_ms = run_ms + try_ms;
    acc.post_ms = post_ms;
    acc.slow_ms = slow_ms;
    acc.bisect_ms = bisect_ms;
    return st;
}

} // namespace

extern "C" {

const char *pt_version(void) { return "pentrack_gb300 0.1 (sm_103a)"; }

const char *pt_last_error(const pt_ctx *ctx) { return ctx ? ctx->err.c_str() : g_create_err.c_str(); }

pt_status pt_create(const pt_scene_desc *scene, int32_t device, pt_ctx **out) {
    if (!out) return PT_ERR_INVALID;
    *out = nullptr;
    {
        pt_status vs = validate_materials(scene, g_create_err);
        if (vs != PT_OK) return vs;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        g_create_err = "no CUDA device";
        return PT_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= ndev) { g_create_err = "bad device index"; return PT_ERR_INVALID; }
    std::unique_ptr<pt_ctx> c(new pt_ctx());
    c->device = device;
    if (!ck(nullptr, cudaSetDevice(device), "cudaSetDevice")) return PT_ERR_CUDA;
    noalloc_forget(device);
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    pt_status st = build_scene(c.get(), scene);
    if (st != PT_OK) {
        g_create_err = c->err;
        free_list(c->allocs);
        return st;
    }
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreate(&c->ev0)) != cudaSuccess || (e = cudaEventCreate(&c->ev1)) != cudaSuccess ||
        (e = cudaEventCreate(&c->evs0)) != cudaSuccess || (e = cudaEventCreate(&c->evs1)) != cudaSuccess ||
        (e = cudaHostAlloc((void **)&c->cancel_host, sizeof(int), cudaHostAllocMapped)) != cudaSuccess ||
        (e = cudaHostGetDevicePointer((void **)&c->cancel_dev, c->cancel_host, 0)) != cudaSuccess ||
        (e = cudaMalloc((void **)&c->counters, sizeof(DCounters))) != cudaSuccess ||
        (e = cudaHostAlloc((void **)&c->counters_host, sizeof(DCounters), 0)) != cudaSuccess ||
        (e = cudaHostAlloc((void **)&c->sched_host, sizeof(DSched), 0)) != cudaSuccess) {
        g_create_err = std::string("context setup: ") + cudaGetErrorString(e);
        free_list(c->allocs);
        return PT_ERR_CUDA;
    }
    *c->cancel_host = 0;
    *out = c.release();
    return PT_OK;
}

void pt_destroy(pt_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    free_list(c->allocs);
    if (c->arena) cudaFree(c->arena);
    if (c->log_hit) cudaFree(c->log_hit);
    if (c->log_snap) cudaFree(c->log_snap);
    if (c->log_track) cudaFree(c->log_track);
    if (c->log_spin) cudaFree(c->log_spin);
    if (c->log_snap_t) cudaFree(c->log_snap_t);
    if (c->log_n) cudaFree(c->log_n);
    if (c->counters) cudaFree(c->counters);
    if (c->counters_host) cudaFreeHost(c->counters_host);
    if (c->sched_host) cudaFreeHost(c->sched_host);
    if (c->cancel_host) cudaFreeHost(c->cancel_host);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->evs0) cudaEventDestroy(c->evs0);
    if (c->evs1) cudaEventDestroy(c->evs1);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

pt_status pt_cancel(pt_ctx *c) {
    if (!c) return PT_ERR_INVALID;
    *(volatile int *)c->cancel_host = 1;
    return PT_OK;
}

} // extern "C"

namespace {

/* Places every DBatch array in one arena (256-byte aligned blocks); with
 * base == nullptr only the size is computed. */
size_t batch_layout(DBatch &b, int64_t n, unsigned char *base) {
    size_t off = 0;
    auto take = [&](auto *&ptr, size_t count) {
        using T = std::remove_pointer_t<std::remove_reference_t<decltype(ptr)>>;
        off = (off + 255) & ~(size_t)255;
        ptr = base ? (T *)(base + off) : nullptr;
        off += std::max<size_t>(count, 1) * sizeof(T);
    };
    const size_t m = (size_t)n;
    take(b.id, m); take(b.t, m); take(b.y, 9 * m); take(b.dydt, 9 * m); take(b.dt, m);
    take(b.spin, 5 * m); take(b.tau, m); take(b.hmax, m); take(b.noflip, m); take(b.hstart, m);
    take(b.t_last, m); take(b.stop_id, m); take(b.nhit, m); take(b.nstep, m);
    take(b.nspinflip, m); take(b.nsol, m); take(b.flags, m); take(b.stack, m);
    take(b.rng_n, m); take(b.nacc, m); take(b.nrej, m); take(b.ntry, m);
    take(b.yn, 9 * m); take(b.dyn, 9 * m); take(b.kst, 36 * m); take(b.tn, m);
    take(b.bc, 14 * m); take(b.count, 8); take(b.nacc0, m);
    take(b.ps_d, 45 * m); take(b.ps_i, (7 + PT_MAX_CAND) * m);
    for (int k = 0; k < 5; ++k) take(b.list[k], m);
    take(b.sched, 1);
    return (off + 255) & ~(size_t)255;
}

pt_status batch_create(pt_ctx *c, const pt_run_params *p, const pt_particles *in, pt_batch **out, bool use_ctx_arena);

} // namespace

extern "C" pt_status pt_batch_create(pt_ctx *c, const pt_run_params *p, const pt_particles *in, pt_batch **out) {
    return batch_create(c, p, in, out, false);
}

namespace {

/* The event-log buffers of a run (context-owned, grown as asked, counts
 * reset): R.log points at them, or is empty when no log is on. */
pt_status setup_logs(pt_ctx *c, const pt_run_params *p, DRun &R) {
    std::memset(&R.log, 0, sizeof(R.log));
    c->log_hit_on = p->hitlog != 0;
    c->log_snap_on = p->snapshotlog != 0 && p->n_snapshots > 0;
    c->log_track_on = p->tracklog != 0 && p->trackloginterval > 0;
    c->log_spin_on = p->spinlog != 0 && p->spinloginterval > 0;
    if (!c->log_hit_on && !c->log_snap_on && !c->log_track_on && !c->log_spin_on) return PT_OK;
    if (c->log_snap_on && (p->n_snapshots > PT_MAX_SNAPSHOTS || !p->snapshots)) {
        c->err = "snapshotlog: 1 to 1024 snapshot times";
        return PT_ERR_INVALID;
    }
    const long long cap = p->log_capacity > 0 ? p->log_capacity : 1000000;
    cudaError_t e = cudaSuccess;
    if (!c->log_n && (e = cudaMalloc((void **)&c->log_n, 4 * sizeof(unsigned long long)))) return ck(c, e, "log counts"), PT_ERR_OOM;
    if (!c->log_snap_t && (e = cudaMalloc((void **)&c->log_snap_t, PT_MAX_SNAPSHOTS * sizeof(double)))) return ck(c, e, "log times"), PT_ERR_OOM;
    if (c->log_hit_on && c->log_cap_hit < cap) {
        if (c->log_hit) cudaFree(c->log_hit);
        c->log_hit = nullptr;
        c->log_cap_hit = 0;
        if ((e = cudaMalloc((void **)&c->log_hit, (size_t)cap * PT_HIT_RECORD * sizeof(double)))) return ck(c, e, "hit log"), PT_ERR_OOM;
        c->log_cap_hit = cap;
    }
    if (c->log_snap_on && c->log_cap_snap < cap) {
        if (c->log_snap) cudaFree(c->log_snap);
        c->log_snap = nullptr;
        c->log_cap_snap = 0;
        if ((e = cudaMalloc((void **)&c->log_snap, (size_t)cap * PT_SNAPSHOT_RECORD * sizeof(double)))) return ck(c, e, "snapshot log"), PT_ERR_OOM;
        c->log_cap_snap = cap;
    }
    if (c->log_track_on && c->log_cap_track < cap) {
        if (c->log_track) cudaFree(c->log_track);
        c->log_track = nullptr;
        c->log_cap_track = 0;
        if ((e = cudaMalloc((void **)&c->log_track, (size_t)cap * PT_TRACK_RECORD * sizeof(double)))) return ck(c, e, "track log"), PT_ERR_OOM;
        c->log_cap_track = cap;
    }
    if (c->log_spin_on && c->log_cap_spin < cap) {
        if (c->log_spin) cudaFree(c->log_spin);
        c->log_spin = nullptr;
        c->log_cap_spin = 0;
        if ((e = cudaMalloc((void **)&c->log_spin, (size_t)cap * PT_SPIN_RECORD * sizeof(double)))) return ck(c, e, "spin log"), PT_ERR_OOM;
        c->log_cap_spin = cap;
    }
    c->log_cap = cap;
    if ((e = cudaMemsetAsync(c->log_n, 0, 4 * sizeof(unsigned long long), c->stream))) return ck(c, e, "log counts"), PT_ERR_CUDA;
    if (c->log_snap_on &&
        (e = cudaMemcpyAsync(c->log_snap_t, p->snapshots, p->n_snapshots * sizeof(double), cudaMemcpyHostToDevice, c->stream)))
        return ck(c, e, "snapshot times"), PT_ERR_CUDA;
    R.log.cap = cap;
    R.log.hit_n = c->log_n;
    R.log.snap_n = c->log_n + 1;
    R.log.track_n = c->log_n + 2;
    R.log.spin_n = c->log_n + 3;
    if (c->log_spin_on) {
        R.log.spin = c->log_spin;
        R.log.spin_interval = p->spinloginterval;
    }
    if (c->log_hit_on) R.log.hit = c->log_hit;
    if (c->log_track_on) {
        R.log.track = c->log_track;
        R.log.track_interval = p->trackloginterval;
    }
    if (c->log_snap_on) {
        R.log.snap = c->log_snap;
        R.log.snap_t = c->log_snap_t;
        R.log.n_snap = p->n_snapshots;
    }
    return PT_OK;
}

pt_status batch_create(pt_ctx *c, const pt_run_params *p, const pt_particles *in, pt_batch **out, bool use_ctx_arena) {
    if (!c || !p || !in || !out || in->n < 0 || !in->id || !in->t || !in->y) return PT_ERR_INVALID;
    cudaSetDevice(c->device);
    *out = nullptr;
    if (p->n_spintimes > PT_MAX_SPINTIMES) { c->err = "at most 8 spintimes intervals"; return PT_ERR_UNSUPPORTED; }
    if (p->species < PT_NEUTRON || p->species > PT_ELECTRON) { c->err = "unknown species"; return PT_ERR_INVALID; }
    if (p->mode != PT_MODE_PLAIN && p->mode != PT_MODE_BATCHED && p->mode != PT_MODE_PHASED) { c->err = "unknown mode"; return PT_ERR_INVALID; }
    if (p->max_run < 0 || p->period_iters < 0) { c->err = "negative tuning parameter"; return PT_ERR_INVALID; }
    if (p->scheduler < 0 || p->scheduler > PT_SCHED_PHASED_WIDE) { c->err = "unknown scheduler"; return PT_ERR_INVALID; }
    std::unique_ptr<pt_batch> B(new pt_batch());
    B->ctx = c;
    B->max_launches = p->max_launches;
    B->timeout_s = p->timeout_s;
    B->max_run = p->max_run;
    B->period_iters = p->period_iters;
    B->scheduler = p->scheduler;
    DRun &R = B->run;
    std::memset(&R, 0, sizeof(R));
    R.sp = make_species(p->species);
    R.simtime = p->simtime; R.tau = p->tau; R.tmax = p->tmax; R.lmax = p->lmax; R.bmax = p->bmax;
    R.n_spintimes = p->n_spintimes;
    for (int k = 0; k < p->n_spintimes; ++k) R.spintimes[k] = p->spintimes[k];
    R.flipspin = p->flipspin;
    R.interp = p->interpolatefields != 0;
    R.mode = p->mode;
    R.prec = p->field_precision;
    R.steps_per_launch = p->steps_per_launch > 0 ? p->steps_per_launch : 64;
    R.seed = p->seed;
    R.t_pause = INFINITY;
    R.cancel = c->cancel_dev;
    if (pt_status ls = setup_logs(c, p, R)) return ls;
    const int64_t n = in->n;
    DBatch &b = B->b;
    b.n = n;
    cudaError_t e = cudaSuccess;
    const size_t bytes = batch_layout(b, n, nullptr);
    unsigned char *base = nullptr;
    if (use_ctx_arena) { /* pt_integrate: reuse the context's arena when it is large enough */
        if (c->arena_bytes < bytes) {
            if (c->arena) cudaFree(c->arena);
            c->arena = nullptr;
            c->arena_bytes = 0;
            if ((e = cudaMalloc(&c->arena, bytes))) { c->arena = nullptr; return ck(c, e, "batch alloc"), PT_ERR_OOM; }
            c->arena_bytes = bytes;
        }
        base = (unsigned char *)c->arena;
    } else {
        void *a = nullptr;
        if ((e = cudaMalloc(&a, bytes))) return ck(c, e, "batch alloc"), PT_ERR_OOM;
        B->allocs.push_back(a);
        base = (unsigned char *)a;
    }
    batch_layout(b, n, base);
    if (n > 0) {
        if ((e = cudaMemcpyAsync(b.id, in->id, n * sizeof(int64_t), cudaMemcpyHostToDevice, c->stream)) ||
            (e = cudaMemcpyAsync(b.t, in->t, n * sizeof(double), cudaMemcpyHostToDevice, c->stream)) ||
            (e = cudaMemcpyAsync(b.y, in->y, 9 * n * sizeof(double), cudaMemcpyHostToDevice, c->stream))) {
            free_list(B->allocs);
            return ck(c, e, "batch upload"), PT_ERR_CUDA;
        }
        if (in->spin) e = cudaMemcpyAsync(b.spin, in->spin, 5 * n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
        else e = cudaMemsetAsync(b.spin, 0, 5 * n * sizeof(double), c->stream);
        if (e) { free_list(B->allocs); return ck(c, e, "batch upload"), PT_ERR_CUDA; }
        k_init<<<grid_for(n, 128), 128, 0, c->stream>>>(c->scene, R, b, c->counters);
        if ((e = cudaGetLastError()) || (e = cudaStreamSynchronize(c->stream))) {
            free_list(B->allocs);
            return ck(c, e, "init kernel"), PT_ERR_CUDA;
        }
    }
    *out = B.release();
    return PT_OK;
}

} // namespace

extern "C" {

void pt_batch_destroy(pt_batch *B) {
    if (!B) return;
    if (B->ctx) cudaSetDevice(B->ctx->device);
    free_list(B->allocs);
    delete B;
}

pt_status pt_batch_advance(pt_ctx *c, pt_batch *B, double t_pause, pt_stats *stats) {
    return pt_batch_advance_steps(c, B, t_pause, 0, stats);
}

pt_status pt_batch_advance_steps(pt_ctx *c, pt_batch *B, double t_pause, int32_t max_steps, pt_stats *stats) {
    if (!c || !B || max_steps < 0) return PT_ERR_INVALID;
    cudaSetDevice(c->device);
    auto w0 = std::chrono::steady_clock::now();
    DRun R = B->run;
    R.t_pause = t_pause;
    R.max_steps = max_steps;
    pt_stats acc;
    std::memset(&acc, 0, sizeof(acc));
    std::snprintf(acc.dominant_kernel, sizeof(acc.dominant_kernel), "k_plain");
    cudaError_t e;
    int steps = R.steps_per_launch;
    const int block = 128;
    const int64_t n = B->b.n;
    bool cancelled = false, timed_out = false;
    pt_status st = PT_OK;
    cudaEventRecord(c->evs0, c->stream);
    /* Runs that integrate spins spend nearly all their time in the Bloch
     * integration, and every trajectory step of such a run needs the full
     * post-step: the batched form runs them as the warp-synchronous
     * plain-form lanes of k_plain_spin. */
    if (R.mode == PT_MODE_BATCHED && n > 0 && spin_run(R)) {
        st = advance_plain(c, B, R, acc, w0, cancelled, timed_out, false);
        if (st != PT_OK) return st;
    } else if (R.mode == PT_MODE_BATCHED && n > 0) {
        st = advance_graph(c, B, R, acc, w0, cancelled, timed_out);
        if (st != PT_OK) return st;
    }
    if (R.mode == PT_MODE_PHASED && n > 0) {
        st = advance_batched(c, B, R, acc, w0, cancelled, timed_out);
        if (st != PT_OK) return st;
    }
    if (R.mode == PT_MODE_PLAIN && n > 0) {
        st = advance_plain(c, B, R, acc, w0, cancelled, timed_out, false);
        if (st != PT_OK) return st;
    }
    cudaEventRecord(c->evs1, c->stream);
    cudaEventSynchronize(c->evs1);
    {
        float sp = 0;
        cudaEventElapsedTime(&sp, c->evs0, c->evs1);
        acc.span_ms = sp;
    }
    acc.wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - w0).count();
    if (stats) *stats = acc;
    if (cancelled) { *(volatile int *)c->cancel_host = 0; return PT_ERR_CANCELLED; }
    if (timed_out) { c->err = "particles still active at the launch or time limit"; return PT_ERR_TIMEOUT; }
    return PT_OK;
}

pt_status pt_batch_read(pt_ctx *c, pt_batch *B, pt_particles *o) {
    if (!c || !B || !o) return PT_ERR_INVALID;
    cudaSetDevice(c->device);
    const DBatch &b = B->b;
    const int64_t n = b.n;
    if (o->n != n) { c->err = "output batch size differs"; return PT_ERR_INVALID; }
    cudaError_t e = cudaSuccess;
#define GET(dst, src, T, cnt) if (o->dst && !e) e = cudaMemcpyAsync(o->dst, b.src, (size_t)(cnt) * sizeof(T), cudaMemcpyDeviceToHost, c->stream);
    GET(id, id, int64_t, n) GET(t, t, double, n) GET(y, y, double, 9 * n) GET(spin, spin, double, 5 * n)
    GET(stop_id, stop_id, int32_t, n) GET(n_hit, nhit, int32_t, n) GET(n_step, nstep, int32_t, n)
    GET(n_spinflip, nspinflip, int32_t, n) GET(h_max, hmax, double, n) GET(noflip_prob, noflip, double, n)
    GET(tau, tau, double, n) GET(h_start, hstart, double, n) GET(n_accepted, nacc, int64_t, n) GET(n_rejected, nrej, int64_t, n)
#undef GET
    if (!e) e = cudaStreamSynchronize(c->stream);
    if (e) return ck(c, e, "batch read"), PT_ERR_CUDA;
    if (o->solid) {
        /* ID of the highest-priority non-ignored solid on each particle's stack */
        std::vector<uint64_t> st(n);
        std::vector<int32_t> ns(n);
        std::vector<DSolid> solids(c->scene.n_solids);
        if ((e = cudaMemcpy(st.data(), b.stack, n * sizeof(uint64_t), cudaMemcpyDeviceToHost)) ||
            (e = cudaMemcpy(ns.data(), b.nsol, n * sizeof(int32_t), cudaMemcpyDeviceToHost)) ||
            (e = cudaMemcpy(solids.data(), c->scene.solids, solids.size() * sizeof(DSolid), cudaMemcpyDeviceToHost)))
            return ck(c, e, "batch read"), PT_ERR_CUDA;
        for (int64_t i = 0; i < n; ++i) {
            int best = 0;
            for (int k = 1; k < ns[i] && k < PT_MAX_STACK; ++k) {
                uint8_t vb = (uint8_t)(st[i] >> (8 * best)), vk = (uint8_t)(st[i] >> (8 * k));
                bool ib = vb >> 7, ik = vk >> 7;
                if (ib || (!ik && solids[vb & 63].id < solids[vk & 63].id)) best = k;
            }
            o->solid[i] = (int32_t)solids[(uint8_t)(st[i] >> (8 * best)) & 63].id;
        }
    }
    return PT_OK;
}

pt_status pt_integrate(pt_ctx *c, const pt_run_params *p, const pt_particles *in, pt_particles *out, pt_stats *stats) {
    if (!c || !p || !in || !out) return PT_ERR_INVALID;
    auto w0 = std::chrono::steady_clock::now();
    pt_batch *B = nullptr;
    pt_status st = batch_create(c, p, in, &B, true);
    if (st != PT_OK) return st;
    pt_stats s;
    std::memset(&s, 0, sizeof(s));
    st = pt_batch_advance(c, B, INFINITY, &s);
    if (st == PT_OK || st == PT_ERR_CANCELLED) {
        pt_status st2 = pt_batch_read(c, B, out);
        if (st == PT_OK) st = st2;
    }
    pt_batch_destroy(B);
    s.wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - w0).count();
    if (stats) *stats = s;
    return st;
}

pt_status pt_log_read(pt_ctx *c, int32_t kind, int64_t cap, double *rec, int64_t *total) {
    if (!c || !total || cap < 0 || (cap > 0 && !rec) || kind < PT_LOG_HIT || kind > PT_LOG_SPIN) return PT_ERR_INVALID;
    *total = 0;
    const bool on = kind == PT_LOG_HIT ? c->log_hit_on : kind == PT_LOG_SNAPSHOT ? c->log_snap_on : kind == PT_LOG_TRACK ? c->log_track_on : c->log_spin_on;
    if (!on || !c->log_n) return PT_OK;
    cudaSetDevice(c->device);
    unsigned long long cnt = 0;
    cudaError_t e = cudaMemcpyAsync(&cnt, c->log_n + kind, sizeof(cnt), cudaMemcpyDeviceToHost, c->stream);
    if (!e) e = cudaStreamSynchronize(c->stream);
    if (e) return ck(c, e, "log count"), PT_ERR_CUDA;
    *total = (int64_t)cnt;
    const int64_t kept = std::min<int64_t>((int64_t)cnt, std::min<int64_t>(cap, c->log_cap));
    const int width = kind == PT_LOG_HIT ? PT_HIT_RECORD : kind == PT_LOG_SNAPSHOT ? PT_SNAPSHOT_RECORD : kind == PT_LOG_TRACK ? PT_TRACK_RECORD : PT_SPIN_RECORD;
    const double *src = kind == PT_LOG_HIT ? c->log_hit : kind == PT_LOG_SNAPSHOT ? c->log_snap : kind == PT_LOG_TRACK ? c->log_track : c->log_spin;
    if (kept > 0) {
        e = cudaMemcpyAsync(rec, src, (size_t)kept * width * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
        if (!e) e = cudaStreamSynchronize(c->stream);
        if (e) return ck(c, e, "log read"), PT_ERR_CUDA;
    }
    return PT_OK;
}

pt_status pt_field_eval(pt_ctx *c, int64_t n, const double *xyzt, int32_t prec, double *B, double *dB, double *V, double *E) {
    if (!c || n < 0 || (!xyzt && n)) return PT_ERR_INVALID;
    if (n == 0) return PT_OK;
    cudaSetDevice(c->device);
    std::vector<void *> tmp;
    cudaError_t e = cudaSuccess;
    double *dq = dupload(tmp, xyzt, 4 * n, e);
    double *dB_ = dalloc<double>(tmp, 3 * n, e), *ddB = dalloc<double>(tmp, 9 * n, e), *dV = dalloc<double>(tmp, n, e),
           *dE = dalloc<double>(tmp, 3 * n, e);
    if (e) { free_list(tmp); return ck(c, e, "field eval alloc"), PT_ERR_OOM; }
    k_field<<<grid_for(n, 128), 128, 0, c->stream>>>(c->scene, prec, n, dq, dB_, dB ? ddB : nullptr, dV, dE);
    e = cudaGetLastError();
    if (!e && B) e = cudaMemcpyAsync(B, dB_, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (!e && dB) e = cudaMemcpyAsync(dB, ddB, 9 * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (!e && V) e = cudaMemcpyAsync(V, dV, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (!e && E) e = cudaMemcpyAsync(E, dE, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (!e) e = cudaStreamSynchronize(c->stream);
    free_list(tmp);
    if (e) return ck(c, e, "field eval"), PT_ERR_CUDA;
    return PT_OK;
}

pt_status pt_segment_collisions(pt_ctx *c, int64_t n, const double *seg, int32_t max_hits, int32_t *count, double *s,
                                double *normal, int32_t *solid_id, double *distnormal) {
    if (!c || n < 0 || max_hits < 1 || !count) return PT_ERR_INVALID;
    if (n == 0) return PT_OK;
    cudaSetDevice(c->device);
    std::vector<void *> tmp;
    cudaError_t e = cudaSuccess;
    double *dseg = dupload(tmp, seg, 6 * n, e);
    int *dc = dalloc<int>(tmp, n, e);
    double *ds = dalloc<double>(tmp, n * max_hits, e), *dn = dalloc<double>(tmp, 3 * n * max_hits, e),
           *ddn = dalloc<double>(tmp, n * max_hits, e);
    int *dsid = dalloc<int>(tmp, n * max_hits, e);
    if (e) { free_list(tmp); return ck(c, e, "collision alloc"), PT_ERR_OOM; }
    k_collisions<<<grid_for(n, 128), 128, 0, c->stream>>>(c->scene, n, dseg, max_hits, dc, ds, dn, dsid, ddn);
    e = cudaGetLastError();
    if (!e) e = cudaMemcpyAsync(count, dc, n * sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    if (!e && s) e = cudaMemcpyAsync(s, ds, n * max_hits * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (!e && normal) e = cudaMemcpyAsync(normal, dn, 3 * n * max_hits * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (!e && solid_id) e = cudaMemcpyAsync(solid_id, dsid, n * max_hits * sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    if (!e && distnormal) e = cudaMemcpyAsync(distnormal, ddn, n * max_hits * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (!e) e = cudaStreamSynchronize(c->stream);
    free_list(tmp);
    if (e) return ck(c, e, "collisions"), PT_ERR_CUDA;
    return PT_OK;
}

pt_status pt_segment_collisions_noalloc(pt_ctx *c, int64_t n, const double *seg, int32_t max_hits, int32_t *count, double *s,
                                        double *normal, int32_t *solid_id, double *distnormal) {
    if (!c || n < 0 || max_hits < 1 || !count || (n > 0 && !seg)) return PT_ERR_INVALID;
    if (n == 0) return PT_OK;
    /* scratch layout, every block 256-byte aligned: segments, counts, s, normals, distnormal, solid IDs */
    const uint64_t un = (uint64_t)n, um = (uint64_t)max_hits;
    if (un > PT_NOALLOC_SCRATCH_BYTES || um > PT_NOALLOC_SCRATCH_BYTES || un * um > PT_NOALLOC_SCRATCH_BYTES) {
        c->err = "pt_segment_collisions_noalloc: n * max_hits exceeds the static scratch of " +
                 std::to_string(PT_NOALLOC_SCRATCH_BYTES) + " bytes";
        return PT_ERR_INVALID;
    }
    auto up = [](uint64_t b) { return (b + 255) & ~(uint64_t)255; };
    const uint64_t o_cnt = up(48 * un), o_s = o_cnt + up(4 * un), o_nrm = o_s + up(8 * un * um), o_dn = o_nrm + up(24 * un * um),
                   o_sid = o_dn + up(8 * un * um), end = o_sid + up(4 * un * um);
    if (end > PT_NOALLOC_SCRATCH_BYTES) {
        c->err = "pt_segment_collisions_noalloc: " + std::to_string(end) + " bytes of scratch needed for n = " + std::to_string(n) +
                 ", max_hits = " + std::to_string(max_hits) + "; the static scratch holds " + std::to_string(PT_NOALLOC_SCRATCH_BYTES);
        return PT_ERR_INVALID;
    }
    cudaError_t e = cudaSetDevice(c->device);
    if (e) return ck(c, e, "noalloc set device"), PT_ERR_CUDA;
    unsigned char *base = nullptr;
    if ((e = noalloc_scratch(c->device, &base))) return ck(c, e, "noalloc scratch address"), PT_ERR_CUDA;
    double *dseg = (double *)base, *ds = (double *)(base + o_s), *dn = (double *)(base + o_nrm), *ddn = (double *)(base + o_dn);
    int *dc = (int *)(base + o_cnt), *dsid = (int *)(base + o_sid);
    e = cudaMemcpyAsync(dseg, seg, 48 * un, cudaMemcpyHostToDevice, c->stream);
    if (!e) {
        k_collisions<<<grid_for(n, 128), 128, 0, c->stream>>>(c->scene, n, dseg, max_hits, dc, ds, dn, dsid, ddn);
        e = cudaGetLastError();
    }
    if (!e) e = cudaMemcpyAsync(count, dc, 4 * un, cudaMemcpyDeviceToHost, c->stream);
    if (!e && s) e = cudaMemcpyAsync(s, ds, 8 * un * um, cudaMemcpyDeviceToHost, c->stream);
    if (!e && normal) e = cudaMemcpyAsync(normal, dn, 24 * un * um, cudaMemcpyDeviceToHost, c->stream);
    if (!e && solid_id) e = cudaMemcpyAsync(solid_id, dsid, 4 * un * um, cudaMemcpyDeviceToHost, c->stream);
    if (!e && distnormal) e = cudaMemcpyAsync(distnormal, ddn, 8 * un * um, cudaMemcpyDeviceToHost, c->stream);
    if (!e) e = cudaStreamSynchronize(c->stream);
    if (e) return ck(c, e, "noalloc collisions"), PT_ERR_CUDA;
    return PT_OK;
}

pt_status pt_adjoint(pt_ctx *c, const pt_run_params *p, const pt_particles *in, int32_t field, int32_t K, const double *dl_dspin,
                     const double *dl_dy, double *dl_dg, pt_particles *out, pt_stats *stats) {
    if (!c || !p || !in || !dl_dg || K < 1 || K > (1 << 20)) return PT_ERR_INVALID;
    const DScene &S = c->scene;
    if (field < 0 || field >= S.n_fields || S.fields[field].type != PT_FIELD_HARMONIC) {
        c->err = "pt_adjoint: field must index a harmonic-expansion field of the scene";
        return PT_ERR_INVALID;
    }
    const int nc = S.fields[field].n_terms;
    if (nc < 1 || nc > PT_ADJ_MAX_COEF) { c->err = "pt_adjoint: 1 to 16 coefficients"; return PT_ERR_UNSUPPORTED; }
    if (p->species != PT_NEUTRON || p->field_precision != PT_PREC_FP64) {
        c->err = "pt_adjoint: neutrons in the FP64 field mode only";
        return PT_ERR_UNSUPPORTED;
    }
    if (p->interpolatefields) {
        c->err = "pt_adjoint: the exact precession axis only (interpolatefields 0)";
        return PT_ERR_UNSUPPORTED;
    }
    for (int fi = 0; fi < S.n_fields; ++fi) {
        const DField &f = S.fields[fi];
        const bool box = f.xmin < f.xmax && f.ymin < f.ymax && f.zmin < f.zmax;
        if ((f.type != PT_FIELD_HARMONIC && f.type != PT_FIELD_UNIFORM_E) || box || f.bw > 0) {
            c->err = "pt_adjoint: the scene's fields must be harmonic expansions and uniform E fields without a box";
            return PT_ERR_UNSUPPORTED;
        }
    }
    cudaSetDevice(c->device);
    const int64_t n = in->n;
    if (n <= 0) {
        for (int k = 0; k < nc; ++k) dl_dg[k] = 0;
        return PT_OK;
    }
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    const double budget = std::min((double)free_b * 0.6, 120e9);
    const double tape_b = (double)n * K * STEP_DOUBLES * 8;
    if (tape_b > 0.5 * budget) { c->err = "pt_adjoint: the chunk tapes (n K 216 B) exceed the device memory budget"; return PT_ERR_OOM; }
    auto clampi = [](double v, double lo, double hi) { return (int)std::max(lo, std::min(hi, v)); };
    int cap_seg = clampi((budget - tape_b) * 0.7 / ((double)n * SEG_DOUBLES * 8), 64, 1 << 20);
    int cap_ck = clampi((budget - tape_b) * 0.3 / ((double)n * CK_DOUBLES * 8), 64, 1 << 22);
    pt_stats acc;
    std::memset(&acc, 0, sizeof(acc));
    std::snprintf(acc.dominant_kernel, sizeof(acc.dominant_kernel), "k_adj_reverse");
    auto w0 = std::chrono::steady_clock::now();
    pt_status st = PT_OK;
    for (int attempt = 0; attempt < 4; ++attempt) {
        pt_batch *B = nullptr;
        pt_run_params q = *p;
        q.mode = PT_MODE_PLAIN;
        if ((st = batch_create(c, &q, in, &B, false)) != PT_OK) return st;
        DRun R = B->run;
        R.t_pause = INFINITY;
        R.max_steps = 0;
        std::vector<void *> mem;
        cudaError_t e = cudaSuccess;
        DAdj A{};
        A.seg = dalloc<double>(mem, (size_t)n * cap_seg * SEG_DOUBLES, e);
        if (!e) A.ck = dalloc<double>(mem, (size_t)n * cap_ck * CK_DOUBLES, e);
        if (!e) A.tape = dalloc<double>(mem, (size_t)n * K * STEP_DOUBLES, e);
        if (!e) A.nseg = dalloc<int>(mem, n, e);
        if (!e) A.nck = dalloc<int>(mem, n, e);
        if (!e) A.status = dalloc<int>(mem, n, e);
        if (!e) A.dl_dg = dalloc<double>(mem, (size_t)n * nc, e);
        double *dspin = nullptr, *dy = nullptr;
        if (!e && dl_dspin) dspin = dupload(mem, dl_dspin, 5 * (size_t)n, e);
        if (!e && dl_dy) dy = dupload(mem, dl_dy, 9 * (size_t)n, e);
        if (e) { free_list(mem); pt_batch_destroy(B); return ck(c, e, "pt_adjoint alloc"), PT_ERR_OOM; }
        A.cap_seg = cap_seg; A.cap_ck = cap_ck; A.K = K; A.field = field; A.ncoef = nc;
        A.dl_dspin = dspin; A.dl_dy = dy;
        std::vector<int> hstat(n);
        float fms = 0, rms = 0;
        cudaMemsetAsync(c->counters, 0, sizeof(DCounters), c->stream);
        cudaEventRecord(c->ev0, c->stream);
        k_adj_forward<<<grid_for(n, lane_block(c, n)), lane_block(c, n), 0, c->stream>>>(S, R, B->b, c->counters, A);
        cudaEventRecord(c->ev1, c->stream);
        if ((e = cudaGetLastError()) || (e = cudaMemcpyAsync(hstat.data(), A.status, n * sizeof(int), cudaMemcpyDeviceToHost, c->stream)) ||
            (e = cudaStreamSynchronize(c->stream))) {
            free_list(mem); pt_batch_destroy(B);
            return ck(c, e, "pt_adjoint forward"), PT_ERR_CUDA;
        }
        cudaEventElapsedTime(&fms, c->ev0, c->ev1);
        cudaMemcpy(c->counters_host, c->counters, sizeof(DCounters), cudaMemcpyDeviceToHost);
        add_counters(acc, *c->counters_host);
        acc.adj_forward_ms += fms;
        int any = 0;
        for (int64_t i = 0; i < n; ++i) any |= hstat[i];
        if (any & ADJ_CANCELLED) {
            free_list(mem); pt_batch_destroy(B);
            *(volatile int *)c->cancel_host = 0;
            return PT_ERR_CANCELLED;
        }
        if (any & (ADJ_OVF_SEG | ADJ_OVF_CK)) { /* the tapes were too short: grow and run again */
            free_list(mem); pt_batch_destroy(B);
            if (any & ADJ_OVF_SEG) cap_seg = std::min(cap_seg * 4, 1 << 22);
            if (any & ADJ_OVF_CK) cap_ck = std::min(cap_ck * 4, 1 << 24);
            st = PT_ERR_OOM;
            c->err = "pt_adjoint: the forward tapes did not fit the device memory budget";
            continue;
        }
        if (any) {
            free_list(mem); pt_batch_destroy(B);
            c->err = "pt_adjoint: the forward pass failed";
            return PT_ERR_CUDA;
        }
        cudaMemsetAsync(c->counters, 0, sizeof(DCounters), c->stream);
        cudaEventRecord(c->ev0, c->stream);
        k_adj_reverse<<<grid_for(n, lane_block(c, n)), lane_block(c, n), 0, c->stream>>>(S, R, B->b, c->counters, A);
        cudaEventRecord(c->ev1, c->stream);
        std::vector<double> g((size_t)n * nc);
        if ((e = cudaGetLastError()) || (e = cudaMemcpyAsync(hstat.data(), A.status, n * sizeof(int), cudaMemcpyDeviceToHost, c->stream)) ||
            (e = cudaMemcpyAsync(g.data(), A.dl_dg, g.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream)) ||
            (e = cudaStreamSynchronize(c->stream))) {
            free_list(mem); pt_batch_destroy(B);
            return ck(c, e, "pt_adjoint reverse"), PT_ERR_CUDA;
        }
        cudaEventElapsedTime(&rms, c->ev0, c->ev1);
        acc.adj_reverse_ms += rms;
        any = 0;
        for (int64_t i = 0; i < n; ++i) any |= hstat[i];
        st = PT_OK;
        if (any & ADJ_UNSUPPORTED) {
            c->err = "pt_adjoint: a particle's path has a diffuse reflection or a transmission; the adjoint follows specular reflections only";
            st = PT_ERR_UNSUPPORTED;
        } else if (any) {
            c->err = "pt_adjoint: a recomputed Bloch chunk differs from the forward pass";
            st = PT_ERR_CUDA;
        }
        if (st == PT_OK) {
            /* per-particle gradients summed in particle order (deterministic) */
            for (int k = 0; k < nc; ++k) {
                double sum = 0;
                for (int64_t i = 0; i < n; ++i) sum += g[(size_t)k * n + i];
                dl_dg[k] = sum;
            }
            if (out) st = pt_batch_read(c, B, out);
        }
        free_list(mem);
        pt_batch_destroy(B);
        break;
    }
    acc.kernel_ms = acc.adj_forward_ms + acc.adj_reverse_ms;
    acc.wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - w0).count();
    acc.launches = 2;
    if (stats) *stats = acc;
    return st;
}

pt_status pt_probe_fp64(pt_ctx *c, double *tflops) {
    if (!c || !tflops) return PT_ERR_INVALID;
    cudaSetDevice(c->device);
    double *d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(double));
    if (e) return ck(c, e, "probe"), PT_ERR_CUDA;
    const int threads = 256, blocks = c->sm_count * 8, iters = 1 << 14;
    k_fp64_probe<<<blocks, threads, 0, c->stream>>>(d, 64, 0.999999, 1e-7); /* warm-up */
    cudaEventRecord(c->ev0, c->stream);
    k_fp64_probe<<<blocks, threads, 0, c->stream>>>(d, iters, 0.999999, 1e-7);
    cudaEventRecord(c->ev1, c->stream);
    e = cudaStreamSynchronize(c->stream);
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    cudaFree(d);
    if (e) return ck(c, e, "probe"), PT_ERR_CUDA;
    *tflops = 2.0 * 8.0 * (double)iters * threads * blocks / (ms * 1e-3) / 1e12;
    return PT_OK;
}

pt_status pt_source_volume(pt_ctx *c, const pt_source_params *sp, int64_t n, const int64_t *ids, pt_particles *out, double *vmin_out) {
    if (!c || !sp || n < 0 || (n && (!ids || !out || !out->id || !out->t || !out->y || !out->spin))) return PT_ERR_INVALID;
    if (sp->species < PT_NEUTRON || sp->species > PT_ELECTRON) { c->err = "pt_source_volume: unknown species"; return PT_ERR_INVALID; }
    if (sp->shape < PT_SOURCE_BOX || sp->shape > PT_SOURCE_SURFACE_STL) { c->err = "pt_source_volume: unknown shape"; return PT_ERR_INVALID; }
    const bool surface = sp->shape == PT_SOURCE_SURFACE_CYLINDER || sp->shape == PT_SOURCE_SURFACE_STL;
    const pt_ctx *reg = sp->shape == PT_SOURCE_SURFACE_STL ? sp->region : nullptr;
    if (sp->shape == PT_SOURCE_SURFACE_STL && (!reg || reg->device != c->device || reg->scene.n_solids < 2 || reg->host_tris.empty())) {
        c->err = "pt_source_volume: the STL surface source needs a region context on the same device with the STL as solid 1";
        return PT_ERR_INVALID;
    }
    if (surface && sp->phase_space) { c->err = "pt_source_volume: phase-space weighting applies to volume sources"; return PT_ERR_INVALID; }
    if (sp->shape == PT_SOURCE_SOLID && (sp->solid < 1 || sp->solid >= c->scene.n_solids)) {
        c->err = "pt_source_volume: solid must index a scene solid other than the default one";
        return PT_ERR_INVALID;
    }
    DSourceSpec Q{};
    Q.shape = sp->shape; Q.solid = sp->solid; Q.phase_space = sp->phase_space != 0;
    Q.max_rounds = sp->max_rounds > 0 ? sp->max_rounds : 100000;
    Q.seed = sp->seed;
    for (int a = 0; a < 3; ++a) { Q.lo[a] = sp->lo[a]; Q.hi[a] = sp->hi[a]; }
    Q.rmin = sp->rmin; Q.rmax = sp->rmax; Q.phimin = sp->phimin; Q.phimax = sp->phimax; Q.zmin = sp->zmin; Q.zmax = sp->zmax;
    Q.emin = sp->emin; Q.emax = sp->emax; Q.polarization = sp->polarization; Q.tmin = sp->tmin; Q.tmax = sp->tmax;
    Q.thetamin = sp->thetamin; Q.thetamax = sp->thetamax; Q.phimin_v = sp->phimin_v; Q.phimax_v = sp->phimax_v;
    Q.enormal = sp->enormal;
    const DSpecies spc = make_species(sp->species);
    cudaSetDevice(c->device);
    std::vector<void *> tmp;
    cudaError_t e = cudaSuccess;
    if (surface) { /* RandomPointOnSurface's candidates: the meshes whose box meets the source box */
        double blo[3] = {-sp->rmax, -sp->rmax, sp->zmin}, bhi[3] = {sp->rmax, sp->rmax, sp->zmax};
        if (reg) { /* the region STL's box (TSTLSurfaceSource, include/source.h:292-296) */
            for (int a = 0; a < 3; ++a) { blo[a] = INFINITY; bhi[a] = -INFINITY; }
            for (size_t k = 0; k < reg->host_tris.size(); ++k) {
                blo[k % 3] = std::min(blo[k % 3], reg->host_tris[k]);
                bhi[k % 3] = std::max(bhi[k % 3], reg->host_tris[k]);
            }
            Q.region = dupload(tmp, &reg->scene, 1, e);
            if (e) { free_list(tmp); return ck(c, e, "region upload"), PT_ERR_OOM; }
        }
        std::vector<double> tri, cum;
        const int64_t nt = (int64_t)c->host_tri_solid.size();
        double run = 0;
        for (int64_t a0 = 0; a0 < nt;) { /* one mesh: a run of triangles of one solid */
            int64_t a1 = a0;
            while (a1 < nt && c->host_tri_solid[a1] == c->host_tri_solid[a0]) ++a1;
            double mlo[3] = {INFINITY, INFINITY, INFINITY}, mhi[3] = {-INFINITY, -INFINITY, -INFINITY};
            for (int64_t k = a0; k < a1; ++k)
                for (int v = 0; v < 3; ++v)
                    for (int a = 0; a < 3; ++a) {
                        mlo[a] = std::min(mlo[a], c->host_tris[9 * k + 3 * v + a]);
                        mhi[a] = std::max(mhi[a], c->host_tris[9 * k + 3 * v + a]);
                    }
            bool meets = true;
            for (int a = 0; a < 3; ++a) meets = meets && !(mhi[a] < blo[a]) && !(mlo[a] > bhi[a]);
            if (meets)
                for (int64_t k = a0; k < a1; ++k) {
                    const double *t = &c->host_tris[9 * k];
                    const double e1[3] = {t[3] - t[0], t[4] - t[1], t[5] - t[2]}, e2[3] = {t[6] - t[0], t[7] - t[1], t[8] - t[2]};
                    const double cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2], cz = e1[0] * e2[1] - e1[1] * e2[0];
                    run = run + 0.5 * std::sqrt(cx * cx + cy * cy + cz * cz);
                    cum.push_back(run);
                    tri.insert(tri.end(), t, t + 9);
                }
            a0 = a1;
        }
        if (cum.empty()) { c->err = "pt_source_volume: no surface of the scene meets the source region"; return PT_ERR_INVALID; }
        Q.surf_tri = dupload(tmp, tri.data(), tri.size(), e);
        if (!e) Q.surf_cum = dupload(tmp, cum.data(), cum.size(), e);
        if (e) { free_list(tmp); return ck(c, e, "surface source upload"), PT_ERR_OOM; }
        Q.n_surf = (int)cum.size();
    }
    double vmin = -INFINITY;
    if (Q.phase_space) { /* FindPotentialMinimum over a fixed sample (src/source.cpp:136-156) */
        const int64_t m = sp->n_min_samples > 0 ? sp->n_min_samples : 100000;
        double *dv = dalloc<double>(tmp, m, e);
        if (e) { free_list(tmp); return ck(c, e, "source alloc"), PT_ERR_OOM; }
        k_source_vmin<<<grid_for(m, 128), 128, 0, c->stream>>>(c->scene, Q, spc, m, dv);
        std::vector<double> hv(m);
        e = cudaGetLastError();
        if (!e) e = cudaMemcpyAsync(hv.data(), dv, m * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
        if (!e) e = cudaStreamSynchronize(c->stream);
        if (e) { free_list(tmp); return ck(c, e, "source minimum potential"), PT_ERR_CUDA; }
        vmin = INFINITY;
        for (double x : hv) {
            if (x != x) { free_list(tmp); c->err = "pt_source_volume: no point inside the source volume for a sample"; return PT_ERR_INVALID; }
            vmin = std::min(vmin, x);
        }
        if (vmin > Q.emax) {
            free_list(tmp);
            c->err = "pt_source_volume: the spectrum is below the minimal potential energy in the source volume";
            return PT_ERR_INVALID;
        }
    }
    if (vmin_out) *vmin_out = vmin;
    if (n == 0) { free_list(tmp); return PT_OK; }
    const int64_t *dids = dupload(tmp, ids, n, e);
    double *dt = dalloc<double>(tmp, n, e), *dy = dalloc<double>(tmp, 9 * n, e), *ds = dalloc<double>(tmp, 5 * n, e);
    int *dst = dalloc<int>(tmp, n, e);
    if (e) { free_list(tmp); return ck(c, e, "source alloc"), PT_ERR_OOM; }
    if (surface) k_source_surface<<<grid_for(n, 128), 128, 0, c->stream>>>(c->scene, Q, spc, n, dids, dt, dy, ds, dst);
    else k_source<<<grid_for(n, 128), 128, 0, c->stream>>>(c->scene, Q, spc, n, dids, vmin, dt, dy, ds, dst);
    std::vector<int> hs(n);
    e = cudaGetLastError();
    if (!e) e = cudaMemcpyAsync(out->t, dt, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (!e) e = cudaMemcpyAsync(out->y, dy, 9 * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (!e) e = cudaMemcpyAsync(out->spin, ds, 5 * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (!e) e = cudaMemcpyAsync(hs.data(), dst, n * sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    if (!e) e = cudaStreamSynchronize(c->stream);
    free_list(tmp);
    if (e) return ck(c, e, "source"), PT_ERR_CUDA;
    if (out->id != ids) std::memcpy(out->id, ids, n * sizeof(int64_t));
    int64_t bad = 0;
    for (int64_t i = 0; i < n; ++i) bad += hs[i] != 0;
    if (bad) {
        c->err = "pt_source_volume: no accepted start point for " + std::to_string(bad) + " particles within the rounds";
        return PT_ERR_INVALID;
    }
    return PT_OK;
}

pt_status pt_neutron_decay(pt_ctx *c, uint64_t seed, int64_t n, const int64_t *ids, const double *t, const double *y,
                           pt_particles *pp, pt_particles *pe) {
    if (!c || n < 0 || !pp || !pe) return PT_ERR_INVALID;
    if (n == 0) return PT_OK;
    if (!ids || !t || !y || pp->n != n || pe->n != n || !pp->id || !pp->t || !pp->y || !pp->spin || !pe->id || !pe->t ||
        !pe->y || !pe->spin)
        return PT_ERR_INVALID;
    cudaSetDevice(c->device);
    std::vector<void *> tmp;
    cudaError_t e = cudaSuccess;
    const int64_t *did = dupload(tmp, ids, n, e);
    const double *dt = dupload(tmp, t, n, e), *dy = dupload(tmp, y, 9 * n, e);
    int64_t *dpid = dalloc<int64_t>(tmp, n, e), *deid = dalloc<int64_t>(tmp, n, e);
    double *dpt = dalloc<double>(tmp, n, e), *det = dalloc<double>(tmp, n, e);
    double *dpy = dalloc<double>(tmp, 9 * n, e), *dey = dalloc<double>(tmp, 9 * n, e);
    int *dst = dalloc<int>(tmp, n, e);
    if (e) { free_list(tmp); return ck(c, e, "decay alloc"), PT_ERR_OOM; }
    k_decay<<<grid_for(n, 128), 128, 0, c->stream>>>(seed, n, did, dt, dy, dpid, dpt, dpy, deid, det, dey, dst);
    e = cudaGetLastError();
    std::vector<int> hs(n);
    if (!e) e = cudaMemcpyAsync(pp->id, dpid, n * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream);
    if (!e) e = cudaMemcpyAsync(pe->id, deid, n * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream);
    if (!e) e = cudaMemcpyAsync(pp->t, dpt, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (!e) e = cudaMemcpyAsync(pe->t, det, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (!e) e = cudaMemcpyAsync(pp->y, dpy, 9 * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (!e) e = cudaMemcpyAsync(pe->y, dey, 9 * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (!e) e = cudaMemcpyAsync(hs.data(), dst, n * sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    if (!e) e = cudaStreamSynchronize(c->stream);
    free_list(tmp);
    if (e) return ck(c, e, "decay"), PT_ERR_CUDA;
    std::memset(pp->spin, 0, 5 * n * sizeof(double));
    std::memset(pe->spin, 0, 5 * n * sizeof(double));
    for (int64_t i = 0; i < n; ++i)
        if (hs[i]) {
            c->err = "pt_neutron_decay: proton spectrum sampling did not converge for particle " + std::to_string(ids[i]);
            return PT_ERR_INVALID;
        }
    return PT_OK;
}

namespace {
/* host SoA of m particles with every output array */
struct HostSet {
    std::vector<int64_t> id, na, nr;
    std::vector<double> t, y, spin, hmax, nf, tau, hs;
    std::vector<int32_t> stop, solid, nhit, nstep, nflip, res;
    pt_particles p{};
    explicit HostSet(int64_t m)
        : id(m), na(m), nr(m), t(m), y(9 * m), spin(5 * m), hmax(m), nf(m), tau(m), hs(m), stop(m), solid(m), nhit(m), nstep(m),
          nflip(m), res(m) {
        p.n = m;
        p.id = id.data(); p.t = t.data(); p.y = y.data(); p.spin = spin.data();
        p.stop_id = stop.data(); p.solid = solid.data(); p.n_hit = nhit.data(); p.n_step = nstep.data();
        p.n_spinflip = nflip.data(); p.reserved = res.data(); p.h_max = hmax.data(); p.noflip_prob = nf.data();
        p.tau = tau.data(); p.h_start = hs.data(); p.n_accepted = na.data(); p.n_rejected = nr.data();
    }
};

/* copies the m entries of a size-m set into `o` (stride o->n); absent output arrays are skipped */
void copy_out(const HostSet &s, pt_particles *o) {
    const int64_t m = s.p.n, n = o->n;
    for (int64_t i = 0; i < m; ++i) {
        if (o->id) o->id[i] = s.id[i];
        if (o->t) o->t[i] = s.t[i];
        if (o->y) for (int k = 0; k < 9; ++k) o->y[k * n + i] = s.y[k * m + i];
        if (o->spin) for (int k = 0; k < 5; ++k) o->spin[k * n + i] = s.spin[k * m + i];
        if (o->stop_id) o->stop_id[i] = s.stop[i];
        if (o->solid) o->solid[i] = s.solid[i];
        if (o->n_hit) o->n_hit[i] = s.nhit[i];
        if (o->n_step) o->n_step[i] = s.nstep[i];
        if (o->n_spinflip) o->n_spinflip[i] = s.nflip[i];
        if (o->h_max) o->h_max[i] = s.hmax[i];
        if (o->noflip_prob) o->noflip_prob[i] = s.nf[i];
        if (o->tau) o->tau[i] = s.tau[i];
        if (o->h_start) o->h_start[i] = s.hs[i];
        if (o->n_accepted) o->n_accepted[i] = s.na[i];
        if (o->n_rejected) o->n_rejected[i] = s.nr[i];
    }
}

void add_stats(pt_stats &a, const pt_stats &b) {
    a.kernel_ms += b.kernel_ms; a.span_ms += b.span_ms; a.particle_seconds += b.particle_seconds;
    a.launches += b.launches; a.active += b.active; a.rk_accepted += b.rk_accepted; a.rk_rejected += b.rk_rejected;
    a.rhs_evals += b.rhs_evals; a.field_evals += b.field_evals; a.hits += b.hits; a.bisection_levels += b.bisection_levels;
    a.bvh_nodes += b.bvh_nodes; a.tri_tests += b.tri_tests; a.subsegments += b.subsegments; a.dense_evals += b.dense_evals;
    a.spin_steps += b.spin_steps; a.aux_launches += b.aux_launches; a.graph_launches += b.graph_launches;
}
} // namespace

pt_status pt_integrate_secondaries(pt_ctx *c, const pt_run_params *pn, const pt_run_params *pp, const pt_run_params *pe,
                                   const pt_particles *in, pt_particles *out, pt_particles *out_p, pt_particles *out_e,
                                   int64_t *n_decayed, pt_stats *stats) {
    if (!c || !pn || !pp || !pe || !in || !out || !out_p || !out_e || !n_decayed) return PT_ERR_INVALID;
    if (pn->species != PT_NEUTRON || pp->species != PT_PROTON || pe->species != PT_ELECTRON) {
        c->err = "pt_integrate_secondaries: the runs must be neutron, proton and electron";
        return PT_ERR_INVALID;
    }
    if (!out->stop_id || !out->id || !out->t || !out->y) return PT_ERR_INVALID;
    auto w0 = std::chrono::steady_clock::now();
    *n_decayed = 0;
    pt_stats total, s;
    std::memset(&total, 0, sizeof(total));
    std::memset(&s, 0, sizeof(s));
    pt_status st = pt_integrate(c, pn, in, out, &s);
    total = s;
    if (st != PT_OK) { if (stats) *stats = total; return st; }
    std::vector<int64_t> idx;
    for (int64_t i = 0; i < out->n; ++i)
        if (out->stop_id[i] == PT_ID_DECAYED) idx.push_back(i);
    const int64_t m = (int64_t)idx.size();
    *n_decayed = m;
    if (m > out_p->n || m > out_e->n) {
        c->err = "pt_integrate_secondaries: " + std::to_string(m) + " decays exceed the secondaries' output size";
        return PT_ERR_INVALID;
    }
    if (m > 0) {
        std::vector<int64_t> ids(m);
        std::vector<double> t(m), y(9 * m);
        for (int64_t j = 0; j < m; ++j) {
            const int64_t i = idx[j];
            ids[j] = out->id[i];
            t[j] = out->t[i];
            for (int k = 0; k < 9; ++k) y[k * m + j] = out->y[k * out->n + i];
        }
        HostSet p0(m), e0(m), p1(m), e1(m);
        st = pt_neutron_decay(c, pn->seed, m, ids.data(), t.data(), y.data(), &p0.p, &e0.p);
        if (st != PT_OK) return st;
        st = pt_integrate(c, pp, &p0.p, &p1.p, &s);
        add_stats(total, s);
        if (st != PT_OK) { if (stats) *stats = total; return st; }
        st = pt_integrate(c, pe, &e0.p, &e1.p, &s);
        add_stats(total, s);
        if (st != PT_OK) { if (stats) *stats = total; return st; }
        copy_out(p1, out_p);
        copy_out(e1, out_e);
    }
    total.wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - w0).count();
    if (stats) *stats = total;
    return PT_OK;
}

pt_status pt_mr_eval(pt_ctx *c, int32_t what, int32_t transmit, int32_t integral, int64_t n, const double *v, const double *normal,
                     const double *Estep, const double *b, const double *w, const double *theta, const double *phi, double *out) {
    if (!c || n < 0 || what < 0 || what > 2) return PT_ERR_INVALID;
    if (n == 0) return PT_OK;
    if (!v || !normal || !Estep || !b || !w || !out || (what == 0 && (!theta || !phi))) return PT_ERR_INVALID;
    cudaSetDevice(c->device);
    std::vector<void *> tmp;
    cudaError_t e = cudaSuccess;
    const double *dv = dupload(tmp, v, 3 * n, e), *dn = dupload(tmp, normal, 3 * n, e), *dE = dupload(tmp, Estep, n, e);
    const double *db = dupload(tmp, b, n, e), *dw = dupload(tmp, w, n, e);
    const double *dth = what == 0 ? dupload(tmp, theta, n, e) : nullptr, *dph = what == 0 ? dupload(tmp, phi, n, e) : nullptr;
    double *dout = dalloc<double>(tmp, n, e);
    if (e) { free_list(tmp); return ck(c, e, "mr alloc"), PT_ERR_OOM; }
    k_mr<<<grid_for(n, 64), 64, 0, c->stream>>>(what, transmit, integral, n, dv, dn, dE, db, dw, dth, dph, dout);
    e = cudaGetLastError();
    if (!e) e = cudaMemcpyAsync(out, dout, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (!e) e = cudaStreamSynchronize(c->stream);
    free_list(tmp);
    if (e) return ck(c, e, "mr eval"), PT_ERR_CUDA;
    return PT_OK;
}

pt_status pt_point_solids(pt_ctx *c, int64_t n, const double *p, uint64_t *mask) {
    if (!c || n < 0 || !mask) return PT_ERR_INVALID;
    if (n == 0) return PT_OK;
    cudaSetDevice(c->device);
    std::vector<void *> tmp;
    cudaError_t e = cudaSuccess;
    double *dp = dupload(tmp, p, 3 * n, e);
    unsigned long long *dm = dalloc<unsigned long long>(tmp, n, e);
    if (e) { free_list(tmp); return ck(c, e, "point solids alloc"), PT_ERR_OOM; }
    k_point_solids<<<grid_for(n, 128), 128, 0, c->stream>>>(c->scene, n, dp, dm);
    e = cudaGetLastError();
    if (!e) e = cudaMemcpyAsync(mask, dm, n * sizeof(uint64_t), cudaMemcpyDeviceToHost, c->stream);
    if (!e) e = cudaStreamSynchronize(c->stream);
    free_list(tmp);
    if (e) return ck(c, e, "point solids"), PT_ERR_CUDA;
    return PT_OK;
}

} // extern "C"
