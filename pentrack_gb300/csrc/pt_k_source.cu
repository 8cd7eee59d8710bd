/*
 * pt_k_source.cu -- volume particle sources on the device: the initial
 * states of TVolumeSource::CreateParticle (src/source.cpp:102-194) for the
 * cuboid, cylindrical and STL volumes (TCuboidVolumeSource,
 * TCylindricalVolumeSource, TSTLVolumeSource: include/source.h:186-331),
 * with or without PhaseSpaceWeighting, written straight into the particle
 * arrays; and the proton and electron of each decayed neutron
 * (TNeutron::Decay, src/neutron.cpp:285-375).
 *
 * Every particle draws from its own Philox stream (the source stream: bit
 * 63 of the counter set, keyed by the seed and the particle id), one counter
 * per draw, in the counter layout of the host-side sources
 * (pentrack_gb300/sources.py), so a particle's start state does not depend
 * on the batch it is made in and equals the host path's.
 */
#include "pt_kcommon.cuh"
#include "pt_kernels.cuh"

namespace ptk {

namespace {

constexpr uint64_t SRC_STREAM = 1ull << 63;
constexpr uint64_t SRC_ROUND = 16;       /* counters per proposal round */
constexpr uint64_t SRC_H = 1ull << 20;   /* total-energy rounds */
constexpr uint64_t SRC_PS = 1ull << 22;  /* phase-space rounds: time, polarisation, acceptance */
constexpr int SRC_STL_ROUNDS = 10000;    /* bounding-box proposals per STL point */
constexpr uint64_t SRC_SURF = 3000;      /* surface points: triangle, two barycentric draws per round */
constexpr double REFLECT_TOLERANCE = 1e-8; /* include/trianglemesh.h:39 */

__device__ __forceinline__ double sdraw(uint64_t seed, int64_t id, uint64_t k) { return uniform(seed, id, SRC_STREAM + k); }

/* first counter of the volume point of phase-space round r (round 0: the
 * minimum-potential samples and the points of unweighted sources) */
__device__ __forceinline__ uint64_t point_base(int r) { return (uint64_t)(r + 1) << 24; }

/* a point of the source volume from draws at `base` on; false when an STL
 * volume's bounding-box proposals ran out (RandomPointInVolume,
 * include/trianglemesh.h:241-265: uniform in the box, kept when inside) */
__device__ bool volume_point(const DScene &S, const DSourceSpec &Q, uint64_t seed, int64_t id, uint64_t base, double p[3]) {
    if (Q.shape == PT_SOURCE_BOX) {
        for (int a = 0; a < 3; ++a) p[a] = Q.lo[a] + sdraw(seed, id, base + a) * (Q.hi[a] - Q.lo[a]);
        return true;
    }
    if (Q.shape == PT_SOURCE_CYLINDER) { /* r from the linear distribution, azimuth and z uniform */
        const double r = sqrt(sdraw(seed, id, base) * (Q.rmax * Q.rmax - Q.rmin * Q.rmin) + Q.rmin * Q.rmin);
        const double ph = Q.phimin + sdraw(seed, id, base + 1) * (Q.phimax - Q.phimin);
        p[0] = r * cos(ph);
        p[1] = r * sin(ph);
        p[2] = Q.zmin + sdraw(seed, id, base + 2) * (Q.zmax - Q.zmin);
        return true;
    }
    for (int r = 0; r < SRC_STL_ROUNDS; ++r) {
        const uint64_t k = base + (uint64_t)r * SRC_ROUND;
        for (int a = 0; a < 3; ++a) p[a] = Q.lo[a] + sdraw(seed, id, k + a) * (Q.hi[a] - Q.lo[a]);
        QueryStats qs{0, 0};
        if ((point_solids(S, p, qs) >> Q.solid) & 1ull) return true;
    }
    return false;
}

/* TParticle::GetInitialTotalEnergy with zero kinetic energy at (t, p) with
 * polarisation pol: the magnetic, electric and gravitational potential
 * energies and, for neutrons, the Fermi potential and internal-field term of
 * the material of the solid the point is in (the solid by
 * TGeometry::GetSolid's rule: the highest ID among the solids containing the
 * point that are not ignored at t) */
__device__ double rest_potential(const DScene &S, const DSpecies &sp, double t, const double p[3], double pol) {
    double B[3], dB[3][3], V = 0, E[3];
    bfield<true>(S, PT_PREC_FP64, p[0], p[1], p[2], B, dB);
    efield(S, PT_PREC_FP64, p[0], p[1], p[2], V, E);
    double r = 0;
    if (sp.mu != 0) r = r + (-pol * sp.mu_over_e) * sqrt(B[0] * B[0] + B[1] * B[1] + B[2] * B[2]);
    if (sp.q != 0) r = r + sp.q_over_e * V;
    r = r + sp.mg * p[2];
    if (sp.kind == PT_NEUTRON) {
        QueryStats qs{0, 0};
        const uint64_t mask = point_solids(S, p, qs);
        int best = 0;
        bool best_ign = false;
        for (int s = 1; s < S.n_solids; ++s) {
            if (!((mask >> s) & 1ull)) continue;
            const DSolid &d = S.solids[s];
            bool ign = false;
            for (int k = 0; k < d.n_ign; ++k) ign = ign || (t >= d.ign[2 * k] && t < d.ign[2 * k + 1]);
            if (best_ign || (!ign && S.solids[best].id < d.id)) {
                best = s;
                best_ign = ign;
            }
        }
        const DMat &m = S.mats[S.solids[best].mat];
        r = r + (m.fermi_real * 1e-9 - m.ibf * sp.mu_over_e * pol);
    }
    return r;
}

/* the TParticle constructor's speed from the kinetic energy
 * (src/particle.cpp:45-52): beta^2 from E / mc^2, its series below round-off */
__device__ double speed_of(double E, double m) {
    const double Eom = E / m / PT_C0 / PT_C0;
    const double series = ((((6.0 * Eom - 5.0) * Eom + 4.0) * Eom - 3.0) * Eom + 2.0) * Eom;
    const double rel = 1.0 - 1.0 / (Eom + 1) / (Eom + 1);
    const double beta2 = pow(Eom, 6.0) < 2 * 2.220446049250313e-16 ? series : rel;
    return PT_C0 * sqrt(beta2);
}

/* InSourceVolume of TCylindricalSurfaceSource: its r, phi, z ranges
 * (include/source.h:279-283, open bounds) */
__device__ bool in_surface_region(const DSourceSpec &Q, const double p[3]) {
    if (Q.shape == PT_SOURCE_SURFACE_STL) { /* TSTLSurfaceSource::InSourceVolume: inside the region STL */
        QueryStats qs{0, 0};
        return (point_solids(*Q.region, p, qs) >> 1) & 1ull;
    }
    const double r = sqrt(p[0] * p[0] + p[1] * p[1]);
    const double ph = atan2(p[1], p[0]);
    return r > Q.rmin && r < Q.rmax && ph > Q.phimin && ph < Q.phimax && p[2] > Q.zmin && p[2] < Q.zmax;
}

} // namespace

/* TSurfaceSource::CreateParticle (src/source.cpp:102-131) with
 * TTriangleMesh::RandomPointOnSurface (include/trianglemesh.h:210-232): a
 * candidate triangle by area (the first whose cumulative area exceeds u times
 * the total), a uniform point on it (barycentric draws folded back into the
 * triangle), redrawn until inside the region; then 1e-8 m off the surface
 * along the unit face normal, a cos(theta) sin(theta) direction about the
 * normal (its normal energy raised by enormal), the polarisation, kinetic
 * energy and start time from the particle's draws 3, 4 and 7 */
__global__ void k_source_surface(const __grid_constant__ DScene S, const __grid_constant__ DSourceSpec Q, DSpecies sp, int64_t n,
                                 const int64_t *ids, double *t_out, double *y, double *spin, int *status) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t id = ids[i];
    const uint64_t seed = Q.seed;
    const double total = Q.surf_cum[Q.n_surf - 1];
    double p[3] = {0, 0, 0}, nrm[3] = {0, 0, 1};
    int bad = 1;
    for (int r = 0; r < Q.max_rounds; ++r) {
        const uint64_t k = SRC_SURF + (uint64_t)r * SRC_ROUND;
        const double u = sdraw(seed, id, k) * total;
        int lo = 0, hi = Q.n_surf; /* upper bound: the first cumulative area > u */
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (Q.surf_cum[mid] > u) hi = mid;
            else lo = mid + 1;
        }
        const int j = lo < Q.n_surf ? lo : Q.n_surf - 1;
        double a = sdraw(seed, id, k + 1), b = sdraw(seed, id, k + 2);
        if (a + b > 1) {
            a = 1 - a;
            b = 1 - b;
        }
        const double *t = Q.surf_tri + 9 * (int64_t)j;
        double e1[3], e2[3], q[3];
        for (int c = 0; c < 3; ++c) {
            e1[c] = t[3 + c] - t[c];
            e2[c] = t[6 + c] - t[c];
            q[c] = t[c] + a * e1[c] + b * e2[c];
        }
        if (!in_surface_region(Q, q)) continue;
        double nv[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        const double len = sqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
        for (int c = 0; c < 3; ++c) {
            nrm[c] = nv[c] / len;
            p[c] = q[c];
        }
        bad = 0;
        break;
    }
    for (int c = 0; c < 3; ++c) p[c] = p[c] + nrm[c] * REFLECT_TOLERANCE;
    double E = Q.emin + sdraw(seed, id, 4) * (Q.emax - Q.emin);
    double ph = 2.0 * PT_PI * sdraw(seed, id, 5);
    double th = acos(sqrt(1.0 - sdraw(seed, id, 6)));
    if (Q.enormal > 0) {
        const double vn = sqrt(E * cos(th) * cos(th) + Q.enormal);
        const double vt = sqrt(E) * sin(th);
        th = atan2(vt, vn);
        E = vn * vn + vt * vt;
    }
    double v[3] = {cos(ph) * sin(th), sin(ph) * sin(th), cos(th)};
    ptd::Lane::rotate_vector(v, nrm, nullptr);
    ph = atan2(v[1], v[0]);
    th = acos(fmin(fmax(v[2], -1.0), 1.0));
    const double pol = sdraw(seed, id, 3) < 0.5 * (Q.polarization + 1) ? 1.0 : -1.0;
    const double speed = speed_of(E, sp.m);
    t_out[i] = Q.tmin + sdraw(seed, id, 7) * (Q.tmax - Q.tmin);
    y[0 * n + i] = p[0];
    y[1 * n + i] = p[1];
    y[2 * n + i] = p[2];
    y[3 * n + i] = speed * cos(ph) * sin(th);
    y[4 * n + i] = speed * sin(ph) * sin(th);
    y[5 * n + i] = speed * cos(th);
    y[6 * n + i] = 0;
    y[7 * n + i] = pol;
    y[8 * n + i] = 0;
    for (int c = 0; c < 5; ++c) spin[c * n + i] = 0;
    status[i] = bad;
}

/* FindPotentialMinimum (src/source.cpp:136-156): the rest potential at the
 * fixed sample points (ids 2^62 + k, k < n, start time and polarisation from
 * the first phase-space counters), one per thread; NaN where an STL
 * sample's proposals ran out */
__global__ void k_source_vmin(const __grid_constant__ DScene S, const __grid_constant__ DSourceSpec Q, DSpecies sp, int64_t n, double *v) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int64_t id = (int64_t)(1ull << 62) + k;
    const double t = Q.tmin + sdraw(Q.seed, id, SRC_PS + 1) * (Q.tmax - Q.tmin);
    const double pol = sdraw(Q.seed, id, SRC_PS + 2) < 0.5 * (Q.polarization + 1) ? 1.0 : -1.0;
    double p[3];
    v[k] = volume_point(S, Q, Q.seed, id, point_base(0), p) ? rest_potential(S, sp, t, p, pol) : NAN;
}

/* One particle per thread: its initial time, state (position, velocity,
 * polarisation) and zero spin.  Unweighted: the point from round 0, the
 * polarisation, kinetic energy (uniform), azimuth (uniform) and polar angle
 * (sine distribution) from draws 3-6, the start time from draw 7.
 * PhaseSpaceWeighting: a total energy H >= vmin (uniform, redrawn), then
 * rounds of (start time, polarisation, point) until the point's rest
 * potential V <= H is accepted with probability sqrt(H - V) / sqrt(H - vmin);
 * kinetic energy H - V.  status[i] = 1 when the rounds ran out. */
__global__ void k_source(const __grid_constant__ DScene S, const __grid_constant__ DSourceSpec Q, DSpecies sp, int64_t n, const int64_t *ids,
                         double vmin, double *t_out, double *y, double *spin, int *status) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t id = ids[i];
    const uint64_t seed = Q.seed;
    double p[3] = {0, 0, 0}, t0 = 0, pol = 0, ekin = 0;
    int bad = 0;
    if (!Q.phase_space) {
        if (!volume_point(S, Q, seed, id, point_base(0), p)) bad = 1;
        pol = sdraw(seed, id, 3) < 0.5 * (Q.polarization + 1) ? 1.0 : -1.0;
        ekin = Q.emin + sdraw(seed, id, 4) * (Q.emax - Q.emin);
        t0 = Q.tmin + sdraw(seed, id, 7) * (Q.tmax - Q.tmin);
    } else {
        double H = NAN;
        for (int r = 0; r < Q.max_rounds; ++r) {
            const double h = Q.emin + sdraw(seed, id, SRC_H + (uint64_t)r * SRC_ROUND) * (Q.emax - Q.emin);
            if (h >= vmin) { H = h; break; }
        }
        bool ok = H == H;
        if (!ok) bad = 1;
        for (int r = 0; ok && r < Q.max_rounds; ++r) {
            const uint64_t k = SRC_PS + (uint64_t)(r + 1) * SRC_ROUND;
            const double tt = Q.tmin + sdraw(seed, id, k + 1) * (Q.tmax - Q.tmin);
            const double pl = sdraw(seed, id, k + 2) < 0.5 * (Q.polarization + 1) ? 1.0 : -1.0;
            double q[3];
            if (!volume_point(S, Q, seed, id, point_base(r + 1), q)) { bad = 1; break; }
            const double v = rest_potential(S, sp, tt, q, pl);
            const double u = sdraw(seed, id, k + 3) * sqrt(H - vmin);
            if (H >= v && sqrt(H - v) > u) {
                p[0] = q[0]; p[1] = q[1]; p[2] = q[2];
                t0 = tt;
                pol = pl;
                ekin = H - v;
                ok = false; /* accepted */
                bad = 0;
                break;
            }
            if (r + 1 == Q.max_rounds) bad = 1;
        }
    }
    const double ph = Q.phimin_v + sdraw(seed, id, 5) * (Q.phimax_v - Q.phimin_v);
    const double u = sdraw(seed, id, 6);
    const double th = acos(cos(Q.thetamin) - u * (cos(Q.thetamin) - cos(Q.thetamax)));
    const double v = speed_of(ekin, sp.m);
    t_out[i] = t0;
    y[0 * n + i] = p[0];
    y[1 * n + i] = p[1];
    y[2 * n + i] = p[2];
    y[3 * n + i] = v * cos(ph) * sin(th);
    y[4 * n + i] = v * sin(ph) * sin(th);
    y[5 * n + i] = v * cos(th);
    y[6 * n + i] = 0;
    y[7 * n + i] = pol;
    y[8 * n + i] = 0;
    for (int c = 0; c < 5; ++c) spin[c * n + i] = 0;
    status[i] = bad;
}

/* ---- secondaries of neutron decay (TNeutron::Decay, src/neutron.cpp:285-375) ---- */

namespace {
constexpr uint64_t DECAY = 5000; /* counter offset of the decay draws in a parent's source stream */

/* ProtonBetaSpectrum (src/globals.cpp:84-92); the reference's 4/3 is integer division (= 1) */
__device__ double proton_beta_spectrum(double E) {
    const double dm = PT_M_N - PT_M_P, xi = PT_M_E / dm;
    const double sigma = 1 - 2 * E * PT_M_N / (dm * dm) / (PT_C0 * PT_C0);
    const double q = (sigma - xi * xi) / sigma;
    const double a = q * q * sqrt(1 - sigma);
    const double g1 = a * (4 * (1 + xi * xi / sigma) - 1 * (q * (1 - sigma)));
    const double g2 = a * (4 * (1 + xi * xi / sigma - 2 * sigma) - 1 * (q * (1 - sigma)));
    return 0.5 * (g1 + -0.1017 * g2);
}

/* BOOST (src/globals.cpp:67-78) of the four-vector p by the velocity beta (units of c) */
__device__ void boost4(const double beta[3], double p[4]) {
    const double b2 = beta[0] * beta[0] + beta[1] * beta[1] + beta[2] * beta[2];
    const double gamma = 1.0 / sqrt(1.0 - b2);
    const double bp = beta[0] * p[1] + beta[1] * p[2] + beta[2] * p[3];
    const double gamma2 = b2 > 0 ? (gamma - 1.0) / b2 : 0.0;
    const double q0 = gamma * (p[0] + bp);
    const double q1 = p[1] + gamma2 * bp * beta[0] + gamma * beta[0] * p[0];
    const double q2 = p[2] + gamma2 * bp * beta[1] + gamma * beta[1] * p[0];
    const double q3 = p[3] + gamma2 * bp * beta[2] + gamma * beta[2] * p[0];
    p[0] = q0; p[1] = q1; p[2] = q2; p[3] = q3;
}

/* a secondary's initial state from its four-momentum p [eV/c] and kinetic energy e [eV] */
__device__ void decay_product(const double p[4], double e, double m, double pol, const double *pos, int64_t n, int64_t i,
                              double *y) {
    const double ph = atan2(p[2], p[1]);
    const double th = acos(p[3] / sqrt(p[1] * p[1] + p[2] * p[2] + p[3] * p[3]));
    const double v = speed_of(e, m);
    y[0 * n + i] = pos[0];
    y[1 * n + i] = pos[1];
    y[2 * n + i] = pos[2];
    y[3 * n + i] = v * cos(ph) * sin(th);
    y[4 * n + i] = v * sin(ph) * sin(th);
    y[5 * n + i] = v * cos(th);
    y[6 * n + i] = 0;
    y[7 * n + i] = pol;
    y[8 * n + i] = 0;
}
} // namespace

/* One thread per decayed neutron: the proton's kinetic energy from the
 * recoil spectrum on [0, 750] eV by rejection (pairs of draws from counter
 * 5100 on, at most 256 pairs; the reference interpolates the spectrum), its
 * direction in the neutron's rest frame (azimuth uniform, polar angle from
 * the sine distribution on [0, pi/2], as the reference draws it), the
 * electron from the two-body decay of the remaining virtual state
 * (neutrino mass 1 eV/c^2) isotropic in that state's rest frame and
 * boosted, both boosted with the neutron's velocity; polarisations +-1 with
 * equal probability; start at the neutron's decay time and point.  Ids:
 * the parent's + 2^40 (proton) and + 2^41 (electron).  status 1: the
 * spectrum sampling did not converge. */
__global__ void k_decay(uint64_t seed, int64_t n, const int64_t *id, const double *t, const double *y, int64_t *pid, double *pt,
                        double *py, int64_t *eid, double *et, double *ey, int *status) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t pa = id[i];
    const double c0 = PT_C0;
    double ekin = -1;
    for (int k = 0; k < 256; ++k) {
        const double e = 0.0 + sdraw(seed, pa, DECAY + 100 + 2 * k) * (750.0 - 0.0);
        const double u = sdraw(seed, pa, DECAY + 101 + 2 * k);
        if (u < proton_beta_spectrum(e)) { ekin = e; break; }
    }
    status[i] = ekin < 0 ? 1 : 0;
    if (ekin < 0) ekin = 0;
    const double m_nue = 1 / (c0 * c0);
    const double pp0 = ekin / c0 + PT_M_P * c0;
    double pabs = sqrt(pp0 * pp0 - PT_M_P * PT_M_P * c0 * c0);
    const double b1 = 2 * PT_PI * sdraw(seed, pa, DECAY + 0), d1 = acos(1.0 - sdraw(seed, pa, DECAY + 1));
    double pp[4] = {pp0, pabs * sin(d1) * cos(b1), pabs * sin(d1) * sin(b1), pabs * cos(d1)};
    const double virt[4] = {PT_M_N * c0 - pp[0], -pp[1], -pp[2], -pp[3]};
    const double m2v = virt[0] * virt[0] - virt[1] * virt[1] - virt[2] * virt[2] - virt[3] * virt[3];
    const double pe0 = (m2v + PT_M_E * PT_M_E * c0 * c0 - m_nue * m_nue * c0 * c0) / 2 / sqrt(m2v);
    pabs = sqrt(pe0 * pe0 - PT_M_E * PT_M_E * c0 * c0);
    const double b2 = 2 * PT_PI * sdraw(seed, pa, DECAY + 2), d2 = acos(1.0 - sdraw(seed, pa, DECAY + 3));
    double pe[4] = {pe0, pabs * sin(d2) * cos(b2), pabs * sin(d2) * sin(b2), pabs * cos(d2)};
    const double bv[3] = {virt[1] / virt[0], virt[2] / virt[0], virt[3] / virt[0]};
    boost4(bv, pe);
    const double bn[3] = {y[3 * n + i] / c0, y[4 * n + i] / c0, y[5 * n + i] / c0};
    boost4(bn, pp);
    boost4(bn, pe);
    const double bp2 = (pp[1] * pp[1] + pp[2] * pp[2] + pp[3] * pp[3]) / pp[0] / pp[0];
    const double e_p = PT_M_P * c0 * c0 * bp2 * (0.5 + bp2 * (3. / 8. + bp2 * (5. / 16.)));
    const double e_e = pe[0] * c0 - PT_M_E * c0 * c0;
    const double pos[3] = {y[0 * n + i], y[1 * n + i], y[2 * n + i]};
    const double pol_p = sdraw(seed, pa, DECAY + 4) < 0.5 ? 1.0 : -1.0, pol_e = sdraw(seed, pa, DECAY + 5) < 0.5 ? 1.0 : -1.0;
    decay_product(pp, e_p, PT_M_P, pol_p, pos, n, i, py);
    decay_product(pe, e_e, PT_M_E, pol_e, pos, n, i, ey);
    pid[i] = pa + (1ll << 40);
    eid[i] = pa + (1ll << 41);
    pt[i] = t[i];
    et[i] = t[i];
}

} // namespace ptk
