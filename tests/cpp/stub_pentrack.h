/* Minimal stand-ins for the PENTrack types the header-only TTrackerGPU
 * shim names (TParticle, TMCGenerator, TGeometry, TFieldManager, solid,
 * state_type, stopID), with the reference's accessor names and signatures
 * (include/particle.h, include/geometry.h, include/globals.h); only for
 * compiling and running the shim in tests. */
#pragma once
#include <string>
#include <vector>

typedef double value_type;
typedef std::vector<value_type> state_type;
enum stopID { ID_UNKNOWN = 0, ID_NOT_FINISH = -1, ID_HIT_BOUNDARIES = -2, ID_ODEINT_ERROR = -3, ID_DECAYED = -4,
              ID_INITIAL_NOT_FOUND = -5, ID_CGAL_ERROR = -6, ID_GEOMETRY_ERROR = -7, ID_ABSORBED_IN_MATERIAL = 1,
              ID_ABSORBED_ON_SURFACE = 2 };
struct solid {
    std::string name;
    unsigned ID;
};
class TParticle {
public:
    TParticle(const std::string &n, int number, double t0, const state_type &y0, const state_type &s0)
        : name(n), particlenumber(number), tstart(t0), ystart(y0), spinstart(s0) {}
    std::string GetName() const { return name; }
    int GetParticleNumber() const { return particlenumber; }
    value_type GetInitialTime() const { return tstart; }
    state_type GetInitialState() const { return ystart; }
    state_type GetInitialSpin() const { return spinstart; }
    value_type GetFinalTime() const { return tend; }
    state_type GetFinalState() const { return yend; }
    state_type GetFinalSpin() const { return spinend; }
    stopID GetStopID() const { return ID; }
    solid GetFinalSolid() const { return solidend; }
    void SetStopID(const stopID aID) { ID = aID; }
    void SetFinalState(const value_type &x, const state_type &y, const state_type &spin, const solid &sld) {
        tend = x; yend = y; spinend = spin; solidend = sld;
    }

private:
    std::string name;
    int particlenumber;
    value_type tstart, tend = 0;
    state_type ystart, spinstart, yend, spinend;
    stopID ID = ID_UNKNOWN;
    solid solidend{};
};
class TMCGenerator {};
class TFieldManager {};
/* GetSolid by the +z parity of a box [-0.5, 0.5]^3: solid 2 inside, 1 outside */
class TGeometry {
public:
    solid GetSolid(const double, const double p[3]) const {
        const bool in = p[0] > -0.5 && p[0] < 0.5 && p[1] > -0.5 && p[1] < 0.5 && p[2] > -0.5 && p[2] < 0.5;
        return in ? solid{"vacuum", 2} : solid{"default", 1};
    }
};
