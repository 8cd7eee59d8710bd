/* Drives TTrackerGPU (include/pentrack_tracker_gpu.hpp) with the stub
 * PENTrack types: prints the run parameters the shim reads from a particle
 * configuration, then tracks the particles of a CSV file (id t y0..y8) with
 * the single-particle IntegrateParticle and prints their end states, or the
 * error text when no context can be made (no GPU). */
#include <cstdio>
#include <fstream>
#include <iostream>

#include "stub_pentrack.h"
#include "pentrack_tracker_gpu.hpp"

int main(int argc, char **argv) {
    if (argc < 3) return 2;
    std::map<std::string, std::string> conf = {{"tau", "880"}, {"tmax", "9e99"}, {"lmax", "5e3"}, {"Bmax", "0.1"},
                                               {"flipspin", "1"}, {"spintimes", "0 10 20 30"}, {"interpolatefields", "0"}};
    std::vector<double> spt;
    pt_run_params p = pentrack_gpu_shim::run_params(conf, 100.0, PT_NEUTRON, 7, PT_MODE_PLAIN, spt);
    std::printf("params %.17g %.17g %.17g %.17g %.17g %d %d %.17g %.17g %.17g %.17g\n", p.simtime, p.tau, p.tmax, p.lmax, p.bmax,
                p.flipspin, p.n_spintimes, p.spintimes[0], p.spintimes[1], p.spintimes[2], p.spintimes[3]);
    try {
        TTrackerGPU tracker(argv[1], 1001, 0, PT_MODE_PLAIN);
        std::ifstream f(argv[2]);
        std::map<std::string, std::string> pc = {{"tau", "0"}, {"tmax", "9e99"}, {"lmax", "9e99"}, {"Bmax", "0.1"}, {"spintimes", "0 0"}};
        TMCGenerator mc;
        TGeometry geom;
        TFieldManager field;
        double simtime = 0;
        f >> simtime;
        long id;
        while (f >> id) {
            double t0;
            state_type y0(9);
            f >> t0;
            for (auto &v : y0) f >> v;
            std::unique_ptr<TParticle> part(new TParticle("neutron", (int)id, t0, y0, state_type(5, 0.0)));
            tracker.IntegrateParticle(part, simtime, pc, mc, geom, field);
            const state_type ye = part->GetFinalState();
            std::printf("end %ld %d %u %.17g", id, (int)part->GetStopID(), part->GetFinalSolid().ID, part->GetFinalTime());
            for (double v : ye) std::printf(" %.17g", v);
            std::printf("\n");
        }
    } catch (const std::exception &e) {
        std::printf("error %s\n", e.what());
        return 0;
    }
    return 0;
}
