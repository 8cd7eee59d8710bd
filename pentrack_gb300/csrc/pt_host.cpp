/*
 * pt_host.cpp -- config.in front end of the GPU path (see pt_host.hpp).
 */
#include "pt_host.hpp"
#include "../../include/pt_constants.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <sstream>

namespace fs = std::filesystem;

namespace pth {

namespace {

std::string trim(const std::string &s) {
    const char *ws = " \t\r\n";
    size_t a = s.find_first_not_of(ws);
    if (a == std::string::npos) return "";
    size_t b = s.find_last_not_of(ws);
    return s.substr(a, b - a + 1);
}

bool parse_number(const std::string &s, double &v) {
    std::string t = trim(s);
    if (t.empty()) return false;
    char *end = nullptr;
    v = std::strtod(t.c_str(), &end);
    return end && *end == '\0';
}

/* ResolveFormula (src/field.cpp) restricted to constants: a [FORMULAS] name is
 * replaced by its expression, which must then be a plain number */
bool constant_scale(const std::string &tok, const Config &cfg, double &v, std::string &err) {
    std::string e = tok;
    auto f = cfg.find("FORMULAS");
    if (f != cfg.end()) {
        auto it = f->second.find(tok);
        if (it != f->second.end()) e = it->second;
    }
    if (parse_number(e, v)) return true;
    err = "field scale '" + tok + "' is not a constant; time-dependent field scaling is not implemented on the device path";
    return false;
}

const std::map<std::string, std::string> &section(const Config &cfg, const char *name) {
    static const std::map<std::string, std::string> empty;
    auto it = cfg.find(name);
    return it == cfg.end() ? empty : it->second;
}

fs::path relative_to(const std::string &config_path, const std::string &file) {
    fs::path p(file);
    if (p.is_absolute()) return p;
    return fs::absolute(fs::path(config_path)).parent_path() / p;
}

} // namespace

bool read_config(const std::string &path, Config &cfg, std::string &err) {
    std::ifstream in(path);
    if (!in) {
        err = "Could not open " + path + "!";
        return false;
    }
    std::string line, sec;
    while (std::getline(in, line)) {
        size_t p = line.find_first_not_of(" \t\r");
        if (p == std::string::npos) continue;
        const char c = line[p];
        if (c == '[') {
            if (p + 1 < line.size() && line[p + 1] == '/') {
                sec.clear();
            } else {
                size_t q = line.find(']', p + 1);
                sec = line.substr(p + 1, q == std::string::npos ? std::string::npos : q - p - 1);
                cfg[sec];
            }
            continue;
        }
        if (c == '#' || sec.empty()) continue;
        size_t ke = line.find_first_of(" \t\r", p);
        std::string key = line.substr(p, ke == std::string::npos ? std::string::npos : ke - p);
        std::string rest = ke == std::string::npos ? "" : line.substr(ke);
        size_t h = rest.find('#');
        if (h != std::string::npos) rest = rest.substr(0, h);
        auto &m = cfg[sec];
        if (m.count(key)) {
            err = "Variable " + key + " in config file is ambiguous!";
            return false;
        }
        m[key] = rest;
    }
    return true;
}

bool read_stl(const std::string &path, std::vector<double> &tris, std::string &err) {
    std::ifstream in(path, std::ios::binary);
    if (!in) {
        err = "Could not open " + path;
        return false;
    }
    char header[80];
    uint32_t n = 0;
    if (!in.read(header, 80) || !in.read(reinterpret_cast<char *>(&n), 4)) {
        err = path + " is not a binary STL file";
        return false;
    }
    if (n == 0) {
        err = path + " contains no triangles";
        return false;
    }
    tris.resize((size_t)n * 9);
    for (uint32_t i = 0; i < n; ++i) {
        unsigned char rec[50];
        if (!in.read(reinterpret_cast<char *>(rec), 50)) {
            err = path + " should contain " + std::to_string(n) + " triangles but read " + std::to_string(i);
            return false;
        }
        for (int k = 0; k < 9; ++k) {
            float f;
            std::memcpy(&f, rec + 12 + 4 * k, 4); /* little-endian, as the STL format defines */
            double v = f;
            if (std::fabs(v) < 1e-8) v = 0.0;
            tris[(size_t)i * 9 + k] = v;
        }
    }
    return true;
}

bool read_opera3d(const std::string &path, double lengthconv, Table3 &t, std::string &err) {
    const std::string ext = fs::path(path).extension().string();
    if (ext == ".gz" || ext == ".bz2") {
        err = path + ": compressed tables are not supported; decompress the file first";
        return false;
    }
    std::ifstream in(path);
    if (!in) {
        err = "Could not open " + path;
        return false;
    }
    long xl = 0, yl = 0, zl = 0;
    std::string line;
    if (!std::getline(in, line) || !(std::istringstream(line) >> xl >> yl >> zl) || xl < 2 || yl < 2 || zl < 2) {
        err = path + ": bad table header";
        return false;
    }
    /* column lines " i NAME [UNIT]" up to " 0" */
    std::vector<std::string> cols;
    while (std::getline(in, line)) {
        std::istringstream ss(line);
        int idx = -1;
        std::string name;
        ss >> idx;
        if (idx == 0) break;
        ss >> name;
        cols.push_back(name);
    }
    if (cols.size() < 3) {
        err = path + " not found or corrupt";
        return false;
    }
    const size_t ncol = cols.size(), npts = (size_t)xl * yl * zl;
    std::vector<double> data;
    data.reserve(npts * ncol);
    double v;
    while (in >> v) data.push_back(v);
    if (data.size() != npts * ncol) {
        err = "The header says the size is " + std::to_string(npts) + ", actually it is " + std::to_string(data.size() / ncol) + "!";
        return false;
    }
    for (int a = 0; a < 3; ++a) {
        std::vector<double> &ax = t.ax[a];
        ax.resize(npts);
        for (size_t i = 0; i < npts; ++i) ax[i] = data[i * ncol + a] * lengthconv;
        std::sort(ax.begin(), ax.end());
        ax.erase(std::unique(ax.begin(), ax.end()), ax.end());
    }
    if (t.ax[0].size() != (size_t)xl || t.ax[1].size() != (size_t)yl || t.ax[2].size() != (size_t)zl) {
        err = path + ": the grid is not rectilinear with the header's dimensions";
        return false;
    }
    auto index = [](const std::vector<double> &ax, double x) { return (size_t)(std::lower_bound(ax.begin(), ax.end(), x) - ax.begin()); };
    std::vector<double> *dst[4] = {nullptr, nullptr, nullptr, nullptr};
    for (size_t c = 3; c < ncol; ++c) {
        std::string nme = cols[c];
        std::transform(nme.begin(), nme.end(), nme.begin(), ::toupper);
        std::vector<double> *d = nme == "BX" ? &t.bx : nme == "BY" ? &t.by : nme == "BZ" ? &t.bz : nme == "V" ? &t.v : nullptr;
        if (d) d->assign(npts, 0.0);
        dst[std::min<size_t>(c - 3, 3)] = d;
        if (c - 3 > 3) {
            err = path + ": more than four field columns";
            return false;
        }
    }
    for (size_t i = 0; i < npts; ++i) {
        const size_t ix = index(t.ax[0], data[i * ncol] * lengthconv), iy = index(t.ax[1], data[i * ncol + 1] * lengthconv),
                     iz = index(t.ax[2], data[i * ncol + 2] * lengthconv);
        const size_t o = (ix * yl + iy) * zl + iz;
        for (size_t c = 3; c < ncol; ++c)
            if (dst[c - 3]) (*dst[c - 3])[o] = data[i * ncol + c];
    }
    return true;
}

bool read_comsol(const std::string &path, double lengthconv, Table3 &t, std::string &err) {
    const std::string ext = fs::path(path).extension().string();
    if (ext == ".gz" || ext == ".bz2") {
        err = path + ": compressed tables are not supported; decompress the file first";
        return false;
    }
    std::ifstream in(path);
    if (!in) {
        err = "Could not open " + path;
        return false;
    }
    std::vector<double> pts; /* x y z bx by bz per point */
    std::string line;
    long num = 0;
    while (std::getline(in, line)) {
        ++num;
        if (!line.empty() && (line[0] == '%' || line[0] == '#')) continue;
        for (char &ch : line)
            if (ch == ',' || ch == '\t' || ch == '\r') ch = ' ';
        std::istringstream ss(line);
        std::vector<double> v;
        double x;
        while (ss >> x) v.push_back(x);
        if (v.empty()) continue;
        if (v.size() != 6) {
            err = "Error reading line " + std::to_string(num) + " of file " + path;
            return false;
        }
        for (int k = 0; k < 3; ++k) v[k] *= lengthconv;
        pts.insert(pts.end(), v.begin(), v.end());
    }
    const size_t np = pts.size() / 6;
    if (np == 0) {
        err = "No data read from " + path;
        return false;
    }
    for (int a = 0; a < 3; ++a) {
        std::vector<double> &ax = t.ax[a];
        ax.resize(np);
        for (size_t i = 0; i < np; ++i) ax[i] = pts[6 * i + a];
        std::sort(ax.begin(), ax.end());
        ax.erase(std::unique(ax.begin(), ax.end()), ax.end());
    }
    const size_t nx = t.ax[0].size(), ny = t.ax[1].size(), nz = t.ax[2].size();
    if (nx * ny * nz != np || nx < 2 || ny < 2 || nz < 2) {
        err = path + ": the points do not fill a rectilinear grid";
        return false;
    }
    auto index = [](const std::vector<double> &ax, double x) { return (size_t)(std::lower_bound(ax.begin(), ax.end(), x) - ax.begin()); };
    t.bx.assign(np, 0.0);
    t.by.assign(np, 0.0);
    t.bz.assign(np, 0.0);
    for (size_t i = 0; i < np; ++i) {
        const size_t o = (index(t.ax[0], pts[6 * i]) * ny + index(t.ax[1], pts[6 * i + 1])) * nz + index(t.ax[2], pts[6 * i + 2]);
        t.bx[o] = pts[6 * i + 3];
        t.by[o] = pts[6 * i + 4];
        t.bz[o] = pts[6 * i + 5];
    }
    return true;
}

bool read_opera2d(const std::string &path, double lengthconv, Table3 &t, std::string &err) {
    const std::string ext = fs::path(path).extension().string();
    if (ext == ".gz" || ext == ".bz2") {
        err = path + ": compressed tables are not supported; decompress the file first";
        return false;
    }
    std::ifstream in(path);
    if (!in) {
        err = "Could not open " + path;
        return false;
    }
    long m = 0, one = 0, n = 0;
    std::string line;
    if (!std::getline(in, line) || !(std::istringstream(line) >> m >> one >> n) || m < 2 || n < 2) {
        err = path + ": bad table header";
        return false;
    }
    /* the r line, then " 2 Y [LENGU]" and z or z alone; then the optional
     * columns in the reference's fixed order, each recognised by substring */
    std::getline(in, line);
    std::getline(in, line);
    const bool skipy = line.compare(0, 12, " 2 Y [LENGU]") != 0;
    std::getline(in, line);
    if (!skipy) std::getline(in, line);
    static const char *tags[7] = {"RBX", "RBY", "RBZ", "EX", "EY", "EZ", "RV"};
    std::vector<double> *dst[7] = {&t.bx, &t.by, &t.bz, &t.er, &t.ephi, &t.ez, &t.v};
    std::vector<int> cols;
    for (int k = 0; k < 7; ++k)
        if (line.find(tags[k]) != std::string::npos) {
            cols.push_back(k);
            dst[k]->assign((size_t)m * n, 0.0);
            std::getline(in, line);
        }
    if (!in || line.compare(0, 2, " 0") != 0) {
        err = path + " not found or corrupt";
        return false;
    }
    std::vector<double> r((size_t)m), z((size_t)n);
    std::vector<double> rowv(cols.size());
    long ri = 0, zi = -1;
    double rv, yv, zv;
    while (in >> rv) {
        if (!skipy && !(in >> yv)) break;
        if (!(in >> zv)) break;
        for (size_t c = 0; c < cols.size(); ++c)
            if (!(in >> rowv[c])) {
                err = path + ": truncated row";
                return false;
            }
        rv *= lengthconv;
        zv *= lengthconv;
        if (zi >= 0 && zv < z[(size_t)zi]) {
            ++ri;
            zi = 0;
        } else {
            ++zi;
        }
        if (ri >= m || zi >= n) {
            err = path + ": more rows than the header's " + std::to_string(m) + " by " + std::to_string(n);
            return false;
        }
        r[(size_t)ri] = rv;
        z[(size_t)zi] = zv;
        for (size_t c = 0; c < cols.size(); ++c) (*dst[cols[c]])[(size_t)ri * n + zi] = rowv[c];
    }
    if (ri + 1 != m || zi + 1 != n) {
        err = "The header says the size is " + std::to_string(m) + " by " + std::to_string(n) + ", actually it is " +
              std::to_string(ri + 1) + " by " + std::to_string(zi + 1) + "!";
        return false;
    }
    t.ax[0] = r;
    t.ax[1].clear();
    t.ax[2] = z;
    return true;
}

pt_status load_scene(const std::string &config_path, SceneStore &S, std::string &err) {
    Config cfg;
    if (!read_config(config_path, cfg, err)) return PT_ERR_IO;
    /* materials: [MATERIALS] of the config, or of [GLOBAL] materials_file */
    std::string matfile;
    {
        auto &g = section(cfg, "GLOBAL");
        auto it = g.find("materials_file");
        if (it != g.end()) matfile = trim(it->second);
    }
    Config matcfg;
    if (!matfile.empty()) {
        if (!read_config(relative_to(config_path, matfile).string(), matcfg, err)) return PT_ERR_IO;
    }
    const auto &mats = matfile.empty() ? section(cfg, "MATERIALS") : section(matcfg, "MATERIALS");
    std::map<std::string, pt_material> known;
    for (auto &kv : mats) {
        std::istringstream ss(kv.second);
        pt_material m{};
        if (!(ss >> m.fermi_real >> m.fermi_imag >> m.diff_prob >> m.spinflip_prob >> m.rms_roughness >> m.correl_length)) {
            err = "Could not read material " + kv.first + "!";
            return PT_ERR_INVALID;
        }
        if (!(ss >> m.internal_bfield)) m.internal_bfield = 0;
        if (!(ss >> m.modified_lambert_prob)) m.modified_lambert_prob = 0;
        if (!(ss >> m.loss_per_bounce)) m.loss_per_bounce = 0;
        if (m.diff_prob < 0 || m.diff_prob > 1 || m.spinflip_prob < 0 || m.spinflip_prob > 1 || m.modified_lambert_prob < 0 ||
            m.modified_lambert_prob > 1 || m.loss_per_bounce < 0 || m.loss_per_bounce > 1) {
            err = "You set a probability outside range 0..1 for material " + kv.first + "!";
            return PT_ERR_INVALID;
        }
        if ((m.diff_prob != 0) + (m.rms_roughness != 0 || m.correl_length != 0) + (m.modified_lambert_prob != 0) > 1) {
            err = "You have set parameters for more than one diffuse-reflection model for material " + kv.first +
                  "! Now I don't know which to use.";
            return PT_ERR_INVALID;
        }
        known[kv.first] = m;
    }
    auto material_index = [&](const std::string &name, int &idx) -> bool {
        auto it = known.find(name);
        if (it == known.end()) return false;
        for (size_t k = 0; k < S.material_names.size(); ++k)
            if (S.material_names[k] == name) { idx = (int)k; return true; }
        S.material_names.push_back(name);
        S.materials.push_back(it->second);
        idx = (int)S.materials.size() - 1;
        return true;
    };
    /* solids: the default solid (ID 1) first, then every other line in map order */
    const auto &geo = section(cfg, "GEOMETRY");
    bool have_default = false;
    S.solids.assign(1, pt_solid{});
    S.solid_ids.assign(1, 1);
    S.ignore.assign(1, std::vector<double>());
    for (auto &kv : geo) {
        long id = 0;
        if (!(std::istringstream(kv.first) >> id) || id < 1) {
            err = "invalid solid ID " + kv.first;
            return PT_ERR_INVALID;
        }
        std::istringstream ss(kv.second);
        std::string file, matname;
        if (!(ss >> file >> matname)) {
            err = "Could not load solid with ID " + std::to_string(id) + "! Did you define invalid parameters?";
            return PT_ERR_INVALID;
        }
        std::vector<double> ign;
        double a, b;
        char dash;
        while (ss >> a) {
            if (!(ss >> dash >> b) || dash != '-') {
                err = "Invalid ignoretimes for solid " + std::to_string(id);
                return PT_ERR_INVALID;
            }
            ign.push_back(a);
            ign.push_back(b);
        }
        int mi = -1;
        if (!material_index(matname, mi)) {
            err = "Material " + matname + " used but not defined!";
            return PT_ERR_INVALID;
        }
        pt_solid so{};
        so.id = (uint32_t)id;
        so.material = mi;
        if (id == 1) {
            have_default = true;
            S.solids[0] = so;
            S.ignore[0] = ign;
            continue;
        }
        if (std::find(S.solid_ids.begin() + 1, S.solid_ids.end(), (uint32_t)id) != S.solid_ids.end()) {
            err = "You defined solids with identical ID! IDs have to be unique!";
            return PT_ERR_INVALID;
        }
        std::vector<double> tr;
        if (!read_stl(relative_to(config_path, file).string(), tr, err)) return PT_ERR_IO;
        const int32_t sidx = (int32_t)S.solids.size();
        S.solids.push_back(so);
        S.solid_ids.push_back((uint32_t)id);
        S.ignore.push_back(ign);
        S.triangles.insert(S.triangles.end(), tr.begin(), tr.end());
        S.triangle_solid.insert(S.triangle_solid.end(), tr.size() / 9, sidx);
    }
    if (!have_default) {
        err = "the [GEOMETRY] section needs the default solid with ID 1";
        return PT_ERR_INVALID;
    }
    for (size_t k = 0; k < S.solids.size(); ++k) {
        S.solids[k].n_ignore = (int32_t)(S.ignore[k].size() / 2);
        S.solids[k].ignore_times = S.ignore[k].empty() ? nullptr : S.ignore[k].data();
    }
    /* fields */
    const auto &fl = section(cfg, "FIELDS");
    for (auto &kv : fl) {
        std::istringstream ss(kv.second);
        std::string type;
        ss >> type;
        pt_field f{};
        f.xmax = f.xmin = f.ymax = f.ymin = f.zmax = f.zmin = 0;
        if (type == "OPERA3D" || type == "3Dtable") {
            std::string file, bs, es;
            double bw = 0, lconv = 1;
            if (!(ss >> file >> bs >> es >> bw) || (type == "OPERA3D" && !(ss >> lconv))) {
                err = "Could not read all required parameters for field " + type + "!";
                return PT_ERR_INVALID;
            }
            double b = 0, e = 0;
            if (!constant_scale(bs, cfg, b, err) || !constant_scale(es, cfg, e, err)) return PT_ERR_UNSUPPORTED;
            if (type == "3Dtable") { /* centimetres, gauss and volt per centimetre */
                b *= 0.0001;
                e *= 100;
                lconv = 0.01;
            }
            auto t = std::make_unique<Table3>();
            if (!read_opera3d(relative_to(config_path, file).string(), lconv, *t, err)) return PT_ERR_IO;
            f.type = PT_FIELD_TAB3D;
            f.b_scale = b;
            f.e_scale = e;
            f.boundary_width = bw;
            f.nx = (int32_t)t->ax[0].size(); f.ny = (int32_t)t->ax[1].size(); f.nz = (int32_t)t->ax[2].size();
            f.x = t->ax[0].data(); f.y = t->ax[1].data(); f.z = t->ax[2].data();
            f.bx = t->bx.empty() ? nullptr : t->bx.data();
            f.by = t->by.empty() ? nullptr : t->by.data();
            f.bz = t->bz.empty() ? nullptr : t->bz.data();
            f.v = t->v.empty() ? nullptr : t->v.data();
            /* the container box is the table's extent (src/field_3d.cpp:308) */
            f.xmax = t->ax[0].back(); f.xmin = t->ax[0].front();
            f.ymax = t->ax[1].back(); f.ymin = t->ax[1].front();
            f.zmax = t->ax[2].back(); f.zmin = t->ax[2].front();
            S.tables.push_back(std::move(t));
        } else if (type == "COMSOL") {
            /* ReadComsolField (src/field_3d.cpp:124-183): B only, box = the data's extent */
            std::string file, bs;
            double bw = 0, lconv = 1;
            if (!(ss >> file >> bs >> bw >> lconv)) {
                err = "Could not read all required parameters for field " + type + "!";
                return PT_ERR_INVALID;
            }
            double b = 0;
            if (!constant_scale(bs, cfg, b, err)) return PT_ERR_UNSUPPORTED;
            auto t = std::make_unique<Table3>();
            if (!read_comsol(relative_to(config_path, file).string(), lconv, *t, err)) return PT_ERR_IO;
            f.type = PT_FIELD_TAB3D;
            f.b_scale = b;
            f.e_scale = 0;
            f.boundary_width = bw;
            f.nx = (int32_t)t->ax[0].size(); f.ny = (int32_t)t->ax[1].size(); f.nz = (int32_t)t->ax[2].size();
            f.x = t->ax[0].data(); f.y = t->ax[1].data(); f.z = t->ax[2].data();
            f.bx = t->bx.data(); f.by = t->by.data(); f.bz = t->bz.data(); f.v = nullptr;
            f.xmax = t->ax[0].back(); f.xmin = t->ax[0].front();
            f.ymax = t->ax[1].back(); f.ymin = t->ax[1].front();
            f.zmax = t->ax[2].back(); f.zmin = t->ax[2].front();
            S.tables.push_back(std::move(t));
        } else if (type == "OPERA2D" || type == "2Dtable") {
            /* ReadOperaField2 (src/field_2d.cpp:37-66): no box, no smoothing band */
            std::string file, bs, es;
            double lconv = 1;
            if (!(ss >> file >> bs >> es) || (type == "OPERA2D" && !(ss >> lconv))) {
                err = "Could not read all required parameters for field " + type + "!";
                return PT_ERR_INVALID;
            }
            double b = 0, e = 0;
            if (!constant_scale(bs, cfg, b, err) || !constant_scale(es, cfg, e, err)) return PT_ERR_UNSUPPORTED;
            if (type == "2Dtable") { /* centimetres, gauss and volt per centimetre */
                b *= 0.0001;
                e *= 100;
                lconv = 0.01;
            }
            auto t = std::make_unique<Table3>();
            if (!read_opera2d(relative_to(config_path, file).string(), lconv, *t, err)) return PT_ERR_IO;
            f.type = PT_FIELD_TAB2D;
            f.b_scale = b;
            f.e_scale = e;
            f.nx = (int32_t)t->ax[0].size(); f.ny = 1; f.nz = (int32_t)t->ax[2].size();
            f.x = t->ax[0].data(); f.z = t->ax[2].data();
            auto ptr = [](const std::vector<double> &v) { return v.empty() ? nullptr : v.data(); };
            f.bx = ptr(t->bx); f.by = ptr(t->by); f.bz = ptr(t->bz); f.v = ptr(t->v);
            f.er = ptr(t->er); f.ephi = ptr(t->ephi); f.ez = ptr(t->ez);
            S.tables.push_back(std::move(t));
        } else if (type == "HarmonicExpansionBField") {
            std::string bs;
            double bw;
            if (!(ss >> f.offset[0] >> f.offset[1] >> f.offset[2] >> bw >> f.xmax >> f.xmin >> f.ymax >> f.ymin >> f.zmax >> f.zmin >> bs)) {
                err = "Could not read all required parameters for field " + type + "!";
                return PT_ERR_INVALID;
            }
            double b;
            if (!constant_scale(bs, cfg, b, err)) return PT_ERR_UNSUPPORTED;
            std::vector<int32_t> L, M;
            std::vector<double> G;
            int l, m;
            double g;
            while (ss >> l >> m >> g) { L.push_back(l); M.push_back(m); G.push_back(g); }
            f.type = PT_FIELD_HARMONIC;
            f.b_scale = b;
            f.e_scale = 0;
            f.boundary_width = bw;
            S.hl.push_back(L);
            S.hm.push_back(M);
            S.hg.push_back(G);
            f.n_coeff = (int32_t)G.size();
            f.l = S.hl.back().data();
            f.m = S.hm.back().data();
            f.g = S.hg.back().data();
        } else if (type == "EDMStaticEField") {
            std::string es;
            if (!(ss >> f.e[0] >> f.e[1] >> f.e[2] >> es)) {
                err = "Could not read all required parameters for field " + type + "!";
                return PT_ERR_INVALID;
            }
            double e;
            if (!constant_scale(es, cfg, e, err)) return PT_ERR_UNSUPPORTED;
            f.type = PT_FIELD_UNIFORM_E;
            f.b_scale = 0;
            f.e_scale = e;
        } else {
            err = "field type " + type + " is not implemented on the device path";
            return PT_ERR_UNSUPPORTED;
        }
        S.fields.push_back(f);
    }
    /* the harmonic coefficient vectors moved while growing: point again */
    for (size_t k = 0, h = 0; k < S.fields.size(); ++k)
        if (S.fields[k].type == PT_FIELD_HARMONIC) {
            S.fields[k].l = S.hl[h].data();
            S.fields[k].m = S.hm[h].data();
            S.fields[k].g = S.hg[h].data();
            ++h;
        }
    pt_scene_desc &d = S.desc;
    d = pt_scene_desc{};
    d.n_triangles = (int64_t)(S.triangles.size() / 9);
    d.triangles = S.triangles.empty() ? nullptr : S.triangles.data();
    d.triangle_solid = S.triangle_solid.empty() ? nullptr : S.triangle_solid.data();
    d.n_solids = (int32_t)S.solids.size();
    d.solids = S.solids.data();
    d.n_materials = (int32_t)S.materials.size();
    d.materials = S.materials.data();
    d.n_fields = (int32_t)S.fields.size();
    d.fields = S.fields.empty() ? nullptr : S.fields.data();
    return PT_OK;
}

pt_status load_run_params(const std::string &config_path, const std::string &species, pt_run_params &p,
                          std::vector<double> &spintimes, std::string &err) {
    Config cfg;
    if (!read_config(config_path, cfg, err)) return PT_ERR_IO;
    p = pt_run_params{};
    if (species == "neutron") p.species = PT_NEUTRON;
    else if (species == "proton") p.species = PT_PROTON;
    else if (species == "electron") p.species = PT_ELECTRON;
    else {
        err = "particle type " + species + " is not implemented on the device path";
        return PT_ERR_UNSUPPORTED;
    }
    auto opt = [&](const char *key) -> std::string {
        auto &sp = section(cfg, species.c_str());
        auto it = sp.find(key);
        if (it != sp.end()) return it->second;
        auto &all = section(cfg, "PARTICLES");
        it = all.find(key);
        return it != all.end() ? it->second : std::string();
    };
    auto num = [&](const std::string &s, double dflt) {
        double v;
        return (std::istringstream(s) >> v) ? v : dflt;
    };
    {
        auto &g = section(cfg, "GLOBAL");
        auto it = g.find("simtime");
        p.simtime = it != g.end() ? num(it->second, 0) : 0;
    }
    p.tau = num(opt("tau"), 0);
    p.tmax = num(opt("tmax"), 0);
    p.lmax = num(opt("lmax"), 0);
    p.bmax = num(opt("Bmax"), 0);
    p.flipspin = (int32_t)num(opt("flipspin"), 0);
    p.interpolatefields = num(opt("interpolatefields"), 0) != 0 ? 1 : 0;
    spintimes.clear();
    {
        std::istringstream ss(opt("spintimes"));
        double t;
        while (ss >> t) spintimes.push_back(t);
    }
    p.n_spintimes = (int32_t)spintimes.size();
    p.spintimes = spintimes.empty() ? nullptr : spintimes.data();
    p.mode = PT_MODE_BATCHED;
    p.field_precision = PT_PREC_FP64;
    p.seed = 1;
    return PT_OK;
}

TTrackerGPU::TTrackerGPU(const std::string &config_path, int device) : path_(config_path) {
    pt_status st = load_scene(config_path, store_, err_);
    if (st != PT_OK) return;
    if (pt_create(&store_.desc, device, &ctx_) != PT_OK) {
        err_ = pt_last_error(nullptr);
        ctx_ = nullptr;
    }
}

TTrackerGPU::~TTrackerGPU() {
    if (ctx_) pt_destroy(ctx_);
}

pt_status TTrackerGPU::IntegrateParticles(const std::string &species, const pt_particles &in, pt_particles &out, pt_stats &stats,
                                          int mode, uint64_t seed) {
    if (!ctx_) return PT_ERR_INVALID;
    pt_run_params p;
    std::vector<double> spintimes;
    pt_status st = load_run_params(path_, species, p, spintimes, err_);
    if (st != PT_OK) return st;
    p.mode = mode;
    p.seed = seed;
    st = pt_integrate(ctx_, &p, &in, &out, &stats);
    if (st != PT_OK && st != PT_ERR_CANCELLED) err_ = pt_last_error(ctx_);
    return st;
}

pt_status TTrackerGPU::WriteEndLog(const std::string &species, const pt_particles &in, const pt_particles &out,
                                   const std::string &directory, int64_t jobnumber, const char *logvars) {
    if (!ctx_) return PT_ERR_INVALID;
    const int kind = species == "neutron" ? PT_NEUTRON : species == "proton" ? PT_PROTON : species == "electron" ? PT_ELECTRON : -1;
    if (kind < 0 || in.n != out.n) {
        err_ = "WriteEndLog: unknown species or batches of different size";
        return PT_ERR_INVALID;
    }
    const int64_t n = in.n;
    std::vector<double> q(4 * n), p(3 * n), B[2], dB(9 * n), V[2], E(3 * n);
    std::vector<uint64_t> masks(n);
    std::vector<int32_t> solid[2];
    const pt_particles *set[2] = {&in, &out};
    for (int k = 0; k < 2; ++k) {
        for (int64_t i = 0; i < n; ++i) {
            for (int c = 0; c < 3; ++c) q[4 * i + c] = p[3 * i + c] = set[k]->y[c * n + i];
            q[4 * i + 3] = set[k]->t[i];
        }
        B[k].resize(3 * n);
        V[k].resize(n);
        solid[k].resize(n);
        pt_status st = pt_field_eval(ctx_, n, q.data(), PT_PREC_FP64, B[k].data(), dB.data(), V[k].data(), E.data());
        if (st == PT_OK) st = pt_point_solids(ctx_, n, p.data(), masks.data());
        if (st != PT_OK) {
            err_ = pt_last_error(ctx_);
            return st;
        }
        if ((st = pt_current_solid(&store_.desc, n, masks.data(), set[k]->t, solid[k].data())) != PT_OK) {
            err_ = pt_config_error();
            return st;
        }
    }
    pt_status st = pt_endlog_write(directory.c_str(), jobnumber, kind, &store_.desc, &in, &out, B[0].data(), V[0].data(),
                                   solid[0].data(), B[1].data(), V[1].data(), solid[1].data(), logvars);
    if (st != PT_OK) err_ = pt_config_error();
    return st;
}

/* ---------------- end log ---------------- */
const SpeciesConstants *species_constants(int kind) {
    static const SpeciesConstants table[3] = {
        {"neutron", PT_NEUTRON, PT_NEUTRON_M, PT_NEUTRON_Q, PT_NEUTRON_MU, PT_NEUTRON_MU_OVER_E, PT_NEUTRON_Q_OVER_E,
         PT_NEUTRON_MC2, PT_NEUTRON_MG},
        {"proton", PT_PROTON, PT_PROTON_M, PT_PROTON_Q, PT_PROTON_MU, PT_PROTON_MU_OVER_E, PT_PROTON_Q_OVER_E,
         PT_PROTON_MC2, PT_PROTON_MG},
        {"electron", PT_ELECTRON, PT_ELECTRON_M, PT_ELECTRON_Q, PT_ELECTRON_MU, PT_ELECTRON_MU_OVER_E,
         PT_ELECTRON_Q_OVER_E, PT_ELECTRON_MC2, PT_ELECTRON_MG}};
    return kind >= 0 && kind < 3 ? &table[kind] : nullptr;
}

double kinetic_energy(const SpeciesConstants &sp, const double v[3]) {
    const double beta2 = (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) / PT_C0_SQ;
    const double b4 = beta2 * beta2;
    double gm1;
    if (b4 * b4 * beta2 < 2.220446049250313e-16)
        gm1 = (0.5 + (3.0 / 8.0 + (5.0 / 16.0 + 35.0 / 128.0 * beta2) * beta2) * beta2) * beta2;
    else
        gm1 = 1.0 / std::sqrt(1.0 - beta2) - 1.0;
    return sp.mc2 * gm1;
}

double potential_energy(const SpeciesConstants &sp, const pt_scene_desc &scene, const double y[9], const double B[3],
                        double V, int solid) {
    double r = 0;
    if (sp.mu != 0) r += -y[7] * sp.mu_over_e * std::sqrt(B[0] * B[0] + B[1] * B[1] + B[2] * B[2]);
    if (sp.q != 0) r += sp.q_over_e * V;
    r += sp.mg * y[2];
    if (sp.kind == PT_NEUTRON) {
        const pt_material &m = scene.materials[scene.solids[solid].material];
        r += m.fermi_real * 1e-9 - m.internal_bfield * sp.mu_over_e * y[7];
    }
    return r;
}

const char *const END_TITLES[43] = {
    "jobnumber", "particle", "tstart", "xstart", "ystart", "zstart", "vxstart", "vystart", "vzstart", "polstart",
    "Sxstart", "Systart", "Szstart", "Hstart", "Estart", "Bstart", "Ustart", "solidstart", "tend", "xend", "yend",
    "zend", "vxend", "vyend", "vzend", "polend", "Sxend", "Syend", "Szend", "Hend", "Eend", "Bend", "Uend",
    "solidend", "stopID", "Nspinflip", "spinflipprob", "Nhit", "Nstep", "propert", "trajlength", "Hmax", "wL"};

bool end_variable_known(const std::string &name) {
    if (name == "m" || name == "q" || name == "mu") return true;
    for (const char *t : END_TITLES)
        if (name == t) return true;
    return false;
}

EndRow end_row(const SpeciesConstants &sp, const pt_scene_desc &scene, const pt_particles &start, const pt_particles &end,
               int64_t i, const double *b0, double v0, int s0, const double *b1, double v1, int s1, int64_t jobnumber) {
    const int64_t n = start.n;
    double ys[9], ye[9];
    for (int c = 0; c < 9; ++c) {
        ys[c] = start.y[c * n + i];
        ye[c] = end.y[c * n + i];
    }
    const double es = kinetic_energy(sp, &ys[3]), ee = kinetic_energy(sp, &ye[3]);
    EndRow r;
    auto &v = r.v;
    v["jobnumber"] = (double)jobnumber;
    v["particle"] = (double)(start.id[i] + 1);
    v["m"] = sp.m;
    v["q"] = sp.q;
    v["mu"] = sp.mu;
    v["tstart"] = start.t[i];
    v["tend"] = end.t[i];
    const char *pos[6] = {"x", "y", "z", "vx", "vy", "vz"};
    for (int c = 0; c < 6; ++c) {
        v[std::string(pos[c]) + "start"] = ys[c];
        v[std::string(pos[c]) + "end"] = ye[c];
    }
    v["polstart"] = ys[7];
    v["polend"] = ye[7];
    const char *sn[3] = {"Sx", "Sy", "Sz"};
    for (int c = 0; c < 3; ++c) {
        v[std::string(sn[c]) + "start"] = start.spin ? start.spin[c * n + i] : 0.0;
        v[std::string(sn[c]) + "end"] = end.spin ? end.spin[c * n + i] : 0.0;
    }
    v["Hstart"] = es + potential_energy(sp, scene, ys, b0, v0, s0);
    v["Estart"] = es;
    v["Bstart"] = std::sqrt(b0[0] * b0[0] + b0[1] * b0[1] + b0[2] * b0[2]);
    v["Ustart"] = v0;
    v["solidstart"] = (double)scene.solids[s0].id;
    v["Hend"] = ee + potential_energy(sp, scene, ye, b1, v1, s1);
    v["Eend"] = ee;
    v["Bend"] = std::sqrt(b1[0] * b1[0] + b1[1] * b1[1] + b1[2] * b1[2]);
    v["Uend"] = v1;
    v["solidend"] = (double)scene.solids[s1].id;
    v["stopID"] = (double)end.stop_id[i];
    v["Nspinflip"] = (double)end.n_spinflip[i];
    v["spinflipprob"] = 1 - end.noflip_prob[i];
    v["Nhit"] = (double)end.n_hit[i];
    v["Nstep"] = (double)end.n_step[i];
    v["propert"] = ye[6];
    v["trajlength"] = ye[8];
    v["Hmax"] = end.h_max[i];
    const double s3 = end.spin ? end.spin[3 * n + i] : 0.0, s4 = end.spin ? end.spin[4 * n + i] : 0.0;
    v["wL"] = s3 > 0 ? s4 / s3 : 0.0;
    return r;
}

} // namespace pth

/* ---------------- C ABI of the config front end ---------------- */
struct pt_config_scene {
    pth::SceneStore store;
};

namespace {
thread_local std::string g_config_err;
}

extern "C" {

pt_status pt_config_load(const char *config_path, pt_config_scene **out) {
    if (!config_path || !out) return PT_ERR_INVALID;
    *out = nullptr;
    auto s = std::make_unique<pt_config_scene>();
    pt_status st = pth::load_scene(config_path, s->store, g_config_err);
    if (st != PT_OK) return st;
    *out = s.release();
    return PT_OK;
}

const pt_scene_desc *pt_config_scene_desc(const pt_config_scene *s) { return s ? &s->store.desc : nullptr; }

void pt_config_free(pt_config_scene *s) { delete s; }

pt_status pt_config_run_params(const char *config_path, const char *species, pt_run_params *out, double *spintimes,
                               int32_t max_spintimes) {
    if (!config_path || !species || !out) return PT_ERR_INVALID;
    std::vector<double> st;
    pt_status r = pth::load_run_params(config_path, species, *out, st, g_config_err);
    if (r != PT_OK) return r;
    if ((int32_t)st.size() > max_spintimes || (!spintimes && !st.empty())) {
        g_config_err = "spintimes needs " + std::to_string(st.size()) + " values";
        return PT_ERR_INVALID;
    }
    for (size_t k = 0; k < st.size(); ++k) spintimes[k] = st[k];
    out->spintimes = st.empty() ? nullptr : spintimes;
    return PT_OK;
}

const char *pt_config_error(void) { return g_config_err.c_str(); }

pt_status pt_current_solid(const pt_scene_desc *scene, int64_t n, const uint64_t *masks, const double *t,
                           int32_t *solid_index) {
    if (!scene || n < 0 || (n > 0 && (!masks || !t || !solid_index)) || scene->n_solids < 1 || scene->n_solids > 64) {
        g_config_err = "pt_current_solid: invalid arguments";
        return PT_ERR_INVALID;
    }
    auto ignored = [&](int s, double tt) {
        const pt_solid &so = scene->solids[s];
        for (int k = 0; k < so.n_ignore; ++k)
            if (tt >= so.ignore_times[2 * k] && tt < so.ignore_times[2 * k + 1]) return true;
        return false;
    };
    for (int64_t i = 0; i < n; ++i) {
        int best = 0;
        bool best_ign = false;
        for (int s = 1; s < scene->n_solids; ++s) {
            if (!((masks[i] >> s) & 1)) continue;
            const bool ign = ignored(s, t[i]);
            if (best_ign || (!ign && scene->solids[best].id < scene->solids[s].id)) {
                best = s;
                best_ign = ign;
            }
        }
        solid_index[i] = best;
    }
    return PT_OK;
}

pt_status pt_endlog_write(const char *directory, int64_t jobnumber, int32_t species, const pt_scene_desc *scene,
                          const pt_particles *start, const pt_particles *end, const double *b_start,
                          const double *v_start, const int32_t *solid_start, const double *b_end, const double *v_end,
                          const int32_t *solid_end, const char *logvars) {
    if (!directory || !scene || !start || !end || !b_start || !v_start || !solid_start || !b_end || !v_end ||
        !solid_end || start->n != end->n || !end->stop_id || !end->n_hit || !end->n_step || !end->n_spinflip ||
        !end->h_max || !end->noflip_prob) {
        g_config_err = "pt_endlog_write: missing arrays or start and end of different size";
        return PT_ERR_INVALID;
    }
    const pth::SpeciesConstants *sp = pth::species_constants(species);
    if (!sp) {
        g_config_err = "pt_endlog_write: unknown species";
        return PT_ERR_INVALID;
    }
    const int64_t n = start->n;
    for (int64_t i = 0; i < n; ++i)
        if (solid_start[i] < 0 || solid_start[i] >= scene->n_solids || solid_end[i] < 0 || solid_end[i] >= scene->n_solids) {
            g_config_err = "pt_endlog_write: solid index out of range";
            return PT_ERR_INVALID;
        }
    std::vector<std::string> titles;
    if (logvars && *logvars) {
        std::istringstream ls(logvars);
        for (std::string t; ls >> t;) titles.push_back(t);
    }
    if (titles.empty()) titles.assign(std::begin(pth::END_TITLES), std::end(pth::END_TITLES));
    for (const auto &t : titles)
        if (!pth::end_variable_known(t)) {
            g_config_err = "pt_endlog_write: end log variable '" + t + "' is not available (formulas are not evaluated)";
            return PT_ERR_UNSUPPORTED;
        }
    char name[64];
    std::snprintf(name, sizeof(name), "%012lld%send.out", (long long)jobnumber, sp->name);
    const std::string path = (std::filesystem::path(directory) / name).string();
    std::ofstream f(path);
    if (!f) {
        g_config_err = "Could not open " + path;
        return PT_ERR_IO;
    }
    f << std::setprecision(15);
    for (const auto &t : titles) f << t << ' ';
    f << '\n';
    for (int64_t i = 0; i < n; ++i) {
        const pth::EndRow row = pth::end_row(*sp, *scene, *start, *end, i, b_start + 3 * i, v_start[i], solid_start[i],
                                             b_end + 3 * i, v_end[i], solid_end[i], jobnumber);
        for (const auto &t : titles) f << row.get(t) << ' ';
        f << '\n';
    }
    if (!f) {
        g_config_err = "write error on " + path;
        return PT_ERR_IO;
    }
    return PT_OK;
}

} // extern "C"
