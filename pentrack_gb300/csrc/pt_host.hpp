/*
 * pt_host.hpp -- the reference's host-side inputs for the GPU path.
 *
 * Reads a PENTrack config.in the way TConfig::ReadFromFile does
 * (src/config.cpp:14-53: sections of "key rest-of-line" pairs, comments after
 * '#', a key defined twice is an error, keys iterate in std::map order) and
 * builds the device scene from its [GEOMETRY], [MATERIALS] (or
 * [GLOBAL] materials_file), [FIELDS] and [FORMULAS] sections, with the files
 * they name (binary STL, OPERA3D / 3Dtable text tables), as TGeometry
 * (src/geometry.cpp:93-137) and TFieldManager (src/fields.cpp:19-136) do.
 * Run parameters come from [GLOBAL] simtime and the particle options of
 * [PARTICLES] overridden by the species section (src/tracking.cpp:19-60).
 *
 * TTrackerGPU keeps the shape of TTracker for C++ callers: construct it
 * from the config, then track batches of particles through pt_integrate.
 */
#pragma once
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>
#include "../../include/pentrack_gpu.h"

namespace pth {

/* section -> key -> rest of line (comment stripped) */
using Config = std::map<std::string, std::map<std::string, std::string>>;

/* TConfig::ReadFromFile; false with a message on I/O or duplicate keys */
bool read_config(const std::string &path, Config &cfg, std::string &err);

/* binary STL as 9 doubles per triangle, |v| < 1e-8 snapped to 0
 * (TTriangleMesh::ReadFile, src/trianglemesh.cpp:17-57) */
bool read_stl(const std::string &path, std::vector<double> &tris, std::string &err);

/* OPERA3D text table (ReadOperaField3, src/field_3d.cpp:185-310): coordinates
 * scaled by lengthconv; axes sorted and unique; components [ix][iy][iz]
 * (empty vector = column absent) */
struct Table3 {
    std::vector<double> ax[3];
    std::vector<double> bx, by, bz, v;
    std::vector<double> er, ephi, ez; /* 2D tables only */
};
bool read_opera3d(const std::string &path, double lengthconv, Table3 &t, std::string &err);
/* COMSOL text export (ReadComsolField, src/field_3d.cpp:124-183): lines of x y z Bx By Bz
 * separated by spaces, tabs or commas, '%' and '#' lines skipped; the points
 * must fill a rectilinear grid */
bool read_comsol(const std::string &path, double lengthconv, Table3 &t, std::string &err);
/* OPERA2D table (TabField::ReadTabFile, src/field_2d.cpp:68-190) into ax[0] = r,
 * ax[2] = z and [ir][iz] columns bx = B_r, by = B_phi, bz = B_z, v, er, ephi, ez */
bool read_opera2d(const std::string &path, double lengthconv, Table3 &t, std::string &err);

/* Owns every array a pt_scene_desc points to. */
struct SceneStore {
    std::vector<double> triangles;
    std::vector<int32_t> triangle_solid;
    std::vector<pt_solid> solids;
    std::vector<std::vector<double>> ignore;
    std::vector<pt_material> materials;
    std::vector<std::string> material_names;
    std::vector<uint32_t> solid_ids;
    std::vector<pt_field> fields;
    std::vector<std::unique_ptr<Table3>> tables;
    std::vector<std::vector<int32_t>> hl, hm;
    std::vector<std::vector<double>> hg;
    pt_scene_desc desc{};
};

/* The scene of a config file; PT_ERR_UNSUPPORTED for field types, scale
 * formulas or materials the device path does not implement. */
pt_status load_scene(const std::string &config_path, SceneStore &store, std::string &err);

/* simtime and the options of `species` ("neutron", "proton", "electron") */
pt_status load_run_params(const std::string &config_path, const std::string &species, pt_run_params &p,
                          std::vector<double> &spintimes, std::string &err);

/* ---- end log (TLogger::Print "end", src/logger.cpp:42-126) ---- */
struct SpeciesConstants {
    const char *name;
    int kind;
    double m, q, mu, mu_over_e, q_over_e, mc2, mg;
};
/* the constants the kernels use (include/pt_constants.h); nullptr for an unknown kind */
const SpeciesConstants *species_constants(int kind);
/* TParticle::GetKineticEnergy (src/particle.cpp:237-251) and GetPotentialEnergy
 * (src/particle.cpp:254-269) + TNeutron's material potential, with the
 * kernels' operations */
double kinetic_energy(const SpeciesConstants &sp, const double v[3]);
double potential_energy(const SpeciesConstants &sp, const pt_scene_desc &scene, const double y[9], const double B[3],
                        double V, int solid);
extern const char *const END_TITLES[43];
bool end_variable_known(const std::string &name);
/* one particle's end-log variables */
struct EndRow {
    std::map<std::string, double> v;
    double get(const std::string &k) const { return v.at(k); }
};
EndRow end_row(const SpeciesConstants &sp, const pt_scene_desc &scene, const pt_particles &start, const pt_particles &end,
               int64_t i, const double *b0, double v0, int s0, const double *b1, double v1, int s1, int64_t jobnumber);

/* C++ front end with the reference's construction from a config file. */
class TTrackerGPU {
public:
    explicit TTrackerGPU(const std::string &config_path, int device = 0);
    ~TTrackerGPU();
    TTrackerGPU(const TTrackerGPU &) = delete;
    TTrackerGPU &operator=(const TTrackerGPU &) = delete;
    /* pt_integrate over host SoA arrays with the config's options for `species` */
    pt_status IntegrateParticles(const std::string &species, const pt_particles &in, pt_particles &out, pt_stats &stats,
                                 int mode = PT_MODE_BATCHED, uint64_t seed = 1);
    /* the end log of a tracked batch (pt_endlog_write): fields and solids at
     * the start and end points from this context's device queries */
    pt_status WriteEndLog(const std::string &species, const pt_particles &in, const pt_particles &out,
                          const std::string &directory, int64_t jobnumber = 0, const char *logvars = nullptr);
    const std::string &error() const { return err_; }
    pt_ctx *context() const { return ctx_; }

private:
    std::string path_, err_;
    SceneStore store_;
    pt_ctx *ctx_ = nullptr;
};

} // namespace pth
