/*
 * pentrack_tracker_gpu.hpp -- header-only drop-in for TTracker inside
 * PENTrack's own build: TTrackerGPU::IntegrateParticle has the signature of
 * TTracker::IntegrateParticle (include/tracking.h:46-47) and runs the
 * particle through the C ABI of include/pentrack_gpu.h.
 *
 * Include it after PENTrack's particle.h, mc.h, geometry.h and fields.h (it
 * uses TParticle, TMCGenerator, TGeometry, TFieldManager, state_type, solid
 * and stopID by name).  The scene is built from the same config file the
 * reference reads (pt_config_load: [GEOMETRY], [MATERIALS], [FIELDS],
 * [FORMULAS]), because TGeometry and TFieldManager keep their contents
 * private; the TGeometry argument is used for the final solid
 * (TGeometry::GetSolid, include/geometry.h:145), the TMCGenerator and
 * TFieldManager arguments are not needed (the random stream is Philox keyed
 * by the particle number and the constructor's seed; the fields live on the
 * device).  IntegrateParticles tracks a whole vector of particles in one
 * call, which is how the GPU should be used: the single-particle call is the
 * reference's interface, a batch of one.
 */
#ifndef PENTRACK_TRACKER_GPU_HPP
#define PENTRACK_TRACKER_GPU_HPP

#include <cstdint>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "pentrack_gpu.h"

namespace pentrack_gpu_shim {

/* the particle options TTracker::IntegrateParticle reads from its
 * particleconf (src/tracking.cpp:19-60), with `tmax` the lab-time limit it
 * is called with; spintimes is filled and out.spintimes points to it */
inline pt_run_params run_params(std::map<std::string, std::string> &conf, double tmax, int species, uint64_t seed, int mode,
                                std::vector<double> &spintimes) {
    pt_run_params p{};
    p.species = species;
    p.mode = mode;
    p.field_precision = PT_PREC_FP64;
    p.simtime = tmax;
    p.tau = 0;
    p.tmax = 9e99;
    p.lmax = 9e99;
    p.bmax = 0;
    p.flipspin = 0;
    std::istringstream(conf["tau"]) >> p.tau;
    std::istringstream(conf["tmax"]) >> p.tmax;
    std::istringstream(conf["lmax"]) >> p.lmax;
    std::istringstream(conf["flipspin"]) >> p.flipspin;
    std::istringstream(conf["Bmax"]) >> p.bmax;
    int interpolate = 0;
    std::istringstream(conf["interpolatefields"]) >> interpolate;
    p.interpolatefields = interpolate ? 1 : 0;
    spintimes.clear();
    std::istringstream st(conf["spintimes"]);
    double a, b;
    while (st >> a >> b) { spintimes.push_back(a); spintimes.push_back(b); }
    p.n_spintimes = (int32_t)spintimes.size();
    p.spintimes = spintimes.empty() ? nullptr : spintimes.data();
    p.seed = seed;
    return p;
}

inline int species_of(const std::string &name) {
    if (name == "neutron") return PT_NEUTRON;
    if (name == "proton") return PT_PROTON;
    if (name == "electron") return PT_ELECTRON;
    throw std::runtime_error("TTrackerGPU: unknown particle " + name);
}

} // namespace pentrack_gpu_shim

class TTrackerGPU {
public:
    /* config_path: the config.in of the run (its scene); seed keys the
     * particles' random streams; mode: PT_MODE_BATCHED or PT_MODE_PLAIN */
    explicit TTrackerGPU(const std::string &config_path, uint64_t seed = 1, int device = 0, int mode = PT_MODE_BATCHED)
        : seed_(seed), mode_(mode) {
        if (pt_config_load(config_path.c_str(), &scene_) != PT_OK) throw std::runtime_error(pt_config_error());
        if (pt_create(pt_config_scene_desc(scene_), device, &ctx_) != PT_OK) {
            const std::string e = pt_last_error(nullptr);
            pt_config_free(scene_);
            scene_ = nullptr;
            throw std::runtime_error(e);
        }
    }
    ~TTrackerGPU() {
        if (ctx_) pt_destroy(ctx_);
        if (scene_) pt_config_free(scene_);
    }
    TTrackerGPU(const TTrackerGPU &) = delete;
    TTrackerGPU &operator=(const TTrackerGPU &) = delete;

    /* TTracker::IntegrateParticle (include/tracking.h:46-47) */
    void IntegrateParticle(std::unique_ptr<TParticle> &p, const double tmax, std::map<std::string, std::string> &particleconf,
                           TMCGenerator &mc, const TGeometry &geom, const TFieldManager &field) {
        std::vector<std::unique_ptr<TParticle>> one;
        one.push_back(std::move(p));
        IntegrateParticles(one, tmax, particleconf, mc, geom, field);
        p = std::move(one[0]);
    }

    /* the same for a vector of particles of one species in one device call */
    void IntegrateParticles(std::vector<std::unique_ptr<TParticle>> &ps, const double tmax, std::map<std::string, std::string> &particleconf,
                            TMCGenerator &, const TGeometry &geom, const TFieldManager &) {
        const int64_t n = (int64_t)ps.size();
        if (n == 0) return;
        const int species = pentrack_gpu_shim::species_of(ps[0]->GetName());
        std::vector<int64_t> id(n);
        std::vector<double> t(n), y(9 * n), spin(5 * n);
        for (int64_t i = 0; i < n; ++i) {
            if (pentrack_gpu_shim::species_of(ps[i]->GetName()) != species)
                throw std::runtime_error("TTrackerGPU: one species per call");
            id[i] = ps[i]->GetParticleNumber();
            t[i] = ps[i]->GetInitialTime();
            const state_type y0 = ps[i]->GetInitialState(), s0 = ps[i]->GetInitialSpin();
            for (int c = 0; c < 9; ++c) y[c * n + i] = y0[c];
            for (int c = 0; c < 5; ++c) spin[c * n + i] = c < (int)s0.size() ? s0[c] : 0.0;
        }
        pt_particles in{};
        in.n = n; in.id = id.data(); in.t = t.data(); in.y = y.data(); in.spin = spin.data();
        std::vector<double> t1(n), y1(9 * n), s1(5 * n), hmax(n), noflip(n), taus(n), h0(n);
        std::vector<int32_t> stop(n), sld(n), nhit(n), nstep(n), nflip(n), res(n);
        std::vector<int64_t> nacc(n), nrej(n);
        pt_particles out{};
        out.n = n; out.id = id.data(); out.t = t1.data(); out.y = y1.data(); out.spin = s1.data();
        out.stop_id = stop.data(); out.solid = sld.data(); out.n_hit = nhit.data(); out.n_step = nstep.data();
        out.n_spinflip = nflip.data(); out.reserved = res.data(); out.h_max = hmax.data(); out.noflip_prob = noflip.data();
        out.tau = taus.data(); out.h_start = h0.data(); out.n_accepted = nacc.data(); out.n_rejected = nrej.data();
        std::vector<double> spintimes;
        pt_run_params rp = pentrack_gpu_shim::run_params(particleconf, tmax, species, seed_, mode_, spintimes);
        pt_stats st{};
        const pt_status s = pt_integrate(ctx_, &rp, &in, &out, &st);
        if (s != PT_OK) throw std::runtime_error(pt_last_error(ctx_));
        for (int64_t i = 0; i < n; ++i) {
            state_type ye(9), se(5);
            for (int c = 0; c < 9; ++c) ye[c] = y1[c * n + i];
            for (int c = 0; c < 5; ++c) se[c] = s1[c * n + i];
            const double pos[3] = {ye[0], ye[1], ye[2]};
            ps[i]->SetFinalState(t1[i], ye, se, geom.GetSolid(t1[i], pos));
            ps[i]->SetStopID(static_cast<stopID>(stop[i])); /* the same integers (include/globals.h:13-23) */
        }
        last_ = st;
    }

    /* counters and timings of the last call */
    const pt_stats &stats() const { return last_; }
    pt_ctx *context() const { return ctx_; }

private:
    pt_config_scene *scene_ = nullptr;
    pt_ctx *ctx_ = nullptr;
    uint64_t seed_;
    int mode_;
    pt_stats last_{};
};

#endif /* PENTRACK_TRACKER_GPU_HPP */
