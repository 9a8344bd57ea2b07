// main.cpp -- the solver executable: a scene directory in, per-frame vertex
// files and checkpoints out, stepping libppf_gb300.so through the
// reference's backend entry points.
//
// Restates the frame loop of the reference's Rust driver
// (crates/ppf-cts-solver/src/main.rs:55-300, backend.rs:626-1030) for the
// part of its scene format this library simulates:
//   ppf-contact-solver --path <scene dir> --output <dir> [--load <frame>]
// Input (scene.rs:443-1110): info.toml ([count], [pin-i], [wall-i],
// [sphere-i]), param.toml ([param]), bin/vert.bin (f64 x3), bin/vel.bin
// (f32 x3), bin/displacement.bin (f64 x3 per group) with bin/vert_dmap.bin
// (u32), bin/tri.bin (u64 x3), bin/param/tri-<name>.bin (per face),
// bin/static_vert.bin / static_vert_dmap.bin / static_tri.bin and
// bin/param/static-<name>.bin (the static collision mesh), bin/pin-ind-<i>.bin
// (u64), bin/wall-pos-<i>.bin, bin/sphere-pos-<i>.bin (f64 x3) and
// bin/sphere-radius-<i>.bin (f32). Walls and spheres take their first
// keyframe. Rods, tets, stitches, pin operations and animated colliders are
// refused with a message.
// Output: <output>/vert_<frame>.bin, the surface vertices at the exact frame
// time frame / fps, linearly interpolated between the two steps that bracket
// it (backend.rs:254-480); <output>/data/time_per_frame.out and
// frame_to_time.out; the per-step SimpleLog channels in <output>/data
// (set_log_path); state_<frame>.bin checkpoints every `auto_save` frames and
// at the end, holding the positions, the time and the carried contact
// pattern (fetch_dyn), which --load <frame> restores (update_dyn).
#include "../../../include/ppf_gb300.h"
#include "../../../include/ppf_gb300_scene.h"

#include <sys/stat.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

extern "C" void print_rust(const char *msg) { std::fprintf(stdout, "%s\n", msg); }

namespace {

[[noreturn]] void die(const std::string &msg) {
    std::fprintf(stderr, "ppf-contact-solver: %s\n", msg.c_str());
    std::exit(1);
}

// ---- a TOML subset: [sections], key = value with integers, floats,
// booleans, "strings" and flat [arrays] ----------------------------------
struct TomlValue {
    std::string raw;
    std::vector<std::string> items; // for arrays
    bool is_array = false;
};
using TomlTable = std::map<std::string, std::map<std::string, TomlValue>>;

std::string trim(const std::string &s) {
    size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
    return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

TomlTable read_toml(const std::string &path) {
    std::ifstream in(path);
    if (!in) die("cannot read " + path);
    TomlTable t;
    std::string line, section;
    while (std::getline(in, line)) {
        // strip a comment outside quotes
        bool q = false;
        for (size_t i = 0; i < line.size(); ++i) {
            if (line[i] == '"') q = !q;
            if (line[i] == '#' && !q) {
                line.resize(i);
                break;
            }
        }
        line = trim(line);
        if (line.empty()) continue;
        if (line.front() == '[' && line.back() == ']') {
            section = trim(line.substr(1, line.size() - 2));
            t[section];
            continue;
        }
        size_t eq = line.find('=');
        if (eq == std::string::npos) continue;
        std::string key = trim(line.substr(0, eq)), val = trim(line.substr(eq + 1));
        if (key.size() >= 2 && key.front() == '"' && key.back() == '"')
            key = key.substr(1, key.size() - 2);
        TomlValue v;
        if (!val.empty() && val.front() == '[') {
            v.is_array = true;
            std::string body = val.substr(1, val.rfind(']') - 1);
            std::stringstream ss(body);
            std::string item;
            while (std::getline(ss, item, ','))
                if (!trim(item).empty()) v.items.push_back(trim(item));
        } else if (val.size() >= 2 && val.front() == '"' && val.back() == '"') {
            v.raw = val.substr(1, val.size() - 2);
        } else {
            v.raw = val;
        }
        t[section][key] = v;
    }
    return t;
}

const TomlValue *find(const TomlTable &t, const std::string &sec, const std::string &key) {
    auto s = t.find(sec);
    if (s == t.end()) return nullptr;
    auto k = s->second.find(key);
    return k == s->second.end() ? nullptr : &k->second;
}
double num(const TomlTable &t, const std::string &sec, const std::string &key, double dflt,
           bool required = false) {
    const TomlValue *v = find(t, sec, key);
    if (!v) {
        if (required) die("missing " + sec + "." + key);
        return dflt;
    }
    if (v->raw == "true") return 1.0;
    if (v->raw == "false") return 0.0;
    return std::strtod(v->raw.c_str(), nullptr);
}
std::string str(const TomlTable &t, const std::string &sec, const std::string &key,
                const std::string &dflt) {
    const TomlValue *v = find(t, sec, key);
    return v ? v->raw : dflt;
}

// ---- raw binary arrays ----------------------------------------------------
bool exists(const std::string &p) {
    struct stat st;
    return stat(p.c_str(), &st) == 0;
}

template <class T> std::vector<T> read_bin(const std::string &path, bool required = true) {
    std::ifstream in(path, std::ios::binary);
    if (!in) {
        if (required) die("cannot read " + path);
        return {};
    }
    in.seekg(0, std::ios::end);
    const size_t bytes = (size_t)in.tellg();
    in.seekg(0);
    if (bytes % sizeof(T)) die(path + ": size is not a multiple of the element size");
    std::vector<T> v(bytes / sizeof(T));
    if (bytes) in.read(reinterpret_cast<char *>(v.data()), (std::streamsize)bytes);
    return v;
}

void mkdirs(const std::string &p) {
    std::string cur;
    std::stringstream ss(p);
    std::string part;
    if (!p.empty() && p[0] == '/') cur = "/";
    while (std::getline(ss, part, '/')) {
        if (part.empty()) continue;
        cur += part + "/";
        mkdir(cur.c_str(), 0775);
    }
}

// ---- the scene ----------------------------------------------------------------
struct Loaded {
    PpfScene *scene = nullptr;
    unsigned n_vert = 0;     // dynamic vertices (all written to vert_<n>.bin)
    double fps = 60.0;
    int frames = 0;
    int auto_save = 0;
    float world_scaling = 1.0f;
};

PpfShellMaterial face_material(const std::map<std::string, std::vector<float>> &prm,
                               const std::vector<uint8_t> &model, unsigned i) {
    auto get = [&](const char *name, float dflt) {
        auto it = prm.find(name);
        return it == prm.end() ? dflt : it->second[i];
    };
    PpfShellMaterial m{};
    m.model = model.empty() ? PPF_MODEL_BARAFF_WITKIN : (int)model[i];
    m.density = get("density", 1.0f);
    m.young_mod = get("young-mod", 100.0f);
    m.poiss_rat = get("poiss-rat", 0.35f);
    m.bend = get("bend", 0.0f);
    m.strain_limit = get("strain-limit", 0.0f);
    m.contact_gap = get("contact-gap", 1e-3f);
    m.contact_offset = get("contact-offset", 0.0f);
    m.friction = get("friction", 0.0f);
    m.deform_damping = get("deformation-damping", 0.0f);
    m.bend_damping = get("bending-damping", 0.0f);
    return m;
}

bool same_material(const PpfShellMaterial &a, const PpfShellMaterial &b) {
    return std::memcmp(&a, &b, sizeof(a)) == 0;
}

void set_param(PpfParamSet &p, const TomlTable &t) {
    const std::string S = "param";
    auto f = [&](const char *k, float d) { return (float)num(t, S, k, d); };
    p.dt = f("dt", p.dt);
    p.playback = f("playback", p.playback);
    p.min_newton_steps = (unsigned)num(t, S, "min_newton_steps", p.min_newton_steps);
    p.max_newton_steps = (unsigned)num(t, S, "max_newton_steps", p.max_newton_steps);
    p.target_toi = f("target_toi", p.target_toi);
    p.air_friction = f("air_friction", p.air_friction);
    p.air_density = f("air_density", p.air_density);
    p.isotropic_air_friction = f("isotropic_air_friction", p.isotropic_air_friction);
    p.line_search_max_t = f("line_search_max_t", p.line_search_max_t);
    p.constraint_tol = f("constraint_tol", p.constraint_tol);
    p.cg_max_iter = (unsigned)num(t, S, "cg_max_iter", p.cg_max_iter);
    p.cg_tol = f("cg_tol", p.cg_tol);
    p.ccd_eps = f("ccd_eps", p.ccd_eps);
    p.max_dx = f("max_dx", p.max_dx);
    p.eiganalysis_eps = f("eiganalysis_eps", p.eiganalysis_eps);
    p.friction_eps = f("friction_eps", p.friction_eps);
    p.fix_xz = f("fix_xz", p.fix_xz);
    p.disable_contact = num(t, S, "disable_contact", 0.0) != 0.0;
    p.inactive_momentum = num(t, S, "inactive_momentum", 0.0) != 0.0;
    p.stitch_length_factor = f("stitch_length_factor", p.stitch_length_factor);
    if (const TomlValue *g = find(t, S, "gravity"))
        for (int d = 0; d < 3 && d < (int)g->items.size(); ++d)
            p.gravity.v[d] = std::strtof(g->items[d].c_str(), nullptr);
    if (const TomlValue *w = find(t, S, "wind"))
        for (int d = 0; d < 3 && d < (int)w->items.size(); ++d)
            p.wind.v[d] = std::strtof(w->items[d].c_str(), nullptr);
    const std::string pc = str(t, S, "precond", "none");
    p.precond = pc == "schwarz" ? 1u : 0u;
    p.schwarz_levels = (unsigned)num(t, S, "schwarz_levels", p.schwarz_levels);
    const std::string fm = str(t, S, "friction_mode", "min");
    p.friction_mode = fm == "max" ? PPF_FRICTION_MAX : fm == "mean" ? PPF_FRICTION_MEAN
                                                                    : PPF_FRICTION_MIN;
}

Loaded load_scene(const std::string &path) {
    Loaded L;
    const TomlTable info = read_toml(path + "/info.toml");
    const TomlTable prm = read_toml(path + "/param.toml");
    const std::string C = "count";
    auto count = [&](const char *k) { return (unsigned)num(info, C, k, 0.0, true); };
    const unsigned n_vert = count("vert"), n_tri = count("tri"), n_sv = count("static_vert"),
                   n_st = count("static_tri"), n_pin = count("pin_block"),
                   n_wall = count("wall"), n_sphere = count("sphere"), n_rod = count("rod");
    const unsigned n_stitch = count("stitch");
    if (count("tet")) die("tets are not read by this executable");
    const double ws = num(prm, "param", "world_scaling", 1.0);
    if (!(ws > 0.0)) die("world_scaling must be > 0");
    L.world_scaling = (float)ws;
    L.fps = num(prm, "param", "fps", 60.0);
    L.frames = (int)num(prm, "param", "frames", 0.0, true);
    L.auto_save = (int)num(prm, "param", "auto_save", 0.0);
    const std::string B = path + "/bin/";

    // dynamic vertices: vert + displacement[dmap] (scene.rs:207-217)
    const auto vert = read_bin<double>(B + "vert.bin");
    const auto disp = read_bin<double>(B + "displacement.bin");
    const auto dmap = read_bin<uint32_t>(B + "vert_dmap.bin");
    const auto vel = read_bin<float>(B + "vel.bin");
    if (vert.size() != 3 * (size_t)n_vert || dmap.size() != n_vert ||
        vel.size() != 3 * (size_t)n_vert)
        die("vert.bin / vert_dmap.bin / vel.bin do not match count.vert");
    std::vector<float> x(3 * (size_t)n_vert);
    for (unsigned i = 0; i < n_vert; ++i) {
        if (3 * (size_t)dmap[i] + 2 >= disp.size()) die("vert_dmap names a missing group");
        for (int d = 0; d < 3; ++d)
            x[3 * i + d] = (float)(vert[3 * i + d] * ws) + (float)(disp[3 * dmap[i] + d] * ws);
    }
    const auto tri64 = read_bin<uint64_t>(B + "tri.bin", n_tri > 0);
    if (tri64.size() != 3 * (size_t)n_tri) die("tri.bin does not match count.tri");
    std::vector<unsigned> tri(tri64.begin(), tri64.end());
    for (unsigned t : tri)
        if (t >= n_vert) die("tri.bin names a vertex past count.vert");

    // per-face materials (bin/param/tri-<name>.bin), deduplicated
    std::map<std::string, std::vector<float>> tp;
    for (const char *k : {"density", "young-mod", "poiss-rat", "bend", "strain-limit",
                          "contact-gap", "contact-offset", "friction"}) {
        auto v = read_bin<float>(B + "param/tri-" + k + ".bin", false);
        if (!v.empty()) {
            if (v.size() != n_tri) die(std::string("tri-") + k + ".bin does not match count.tri");
            tp[k] = v;
        }
    }
    auto model = read_bin<uint8_t>(B + "param/tri-model.bin", false);
    std::vector<PpfShellMaterial> mats;
    std::vector<unsigned> fmat(n_tri);
    for (unsigned i = 0; i < n_tri; ++i) {
        PpfShellMaterial m = face_material(tp, model, i);
        unsigned k = 0;
        while (k < mats.size() && !same_material(mats[k], m)) ++k;
        if (k == mats.size()) mats.push_back(m);
        fmat[i] = k;
    }
    L.scene = ppf_scene_create();
    L.n_vert = n_vert;
    if (!n_tri && !n_rod) die("the scene has neither shell faces nor rods");
    // every vertex is added with the shells (faces may be none)
    if (ppf_scene_add_shell_faces(L.scene, x.data(), n_vert, tri.data(), n_tri, fmat.data(),
                                  mats.data(), (unsigned)mats.size()) == 0xFFFFFFFFu)
        die("bad face material table");
    if (n_rod) {
        // rods over the shared vertex array: bin/rod.bin and the per-rod
        // bin/param/rod-<name>.bin arrays (scene.rs:512-719, 1540-1655)
        const auto rod64 = read_bin<uint64_t>(B + "rod.bin");
        if (rod64.size() != 2 * (size_t)n_rod) die("rod.bin does not match count.rod");
        std::vector<unsigned> rod(rod64.begin(), rod64.end());
        std::map<std::string, std::vector<float>> rp;
        for (const char *k : {"density", "young-mod", "bend", "length-factor", "strain-limit",
                              "contact-gap", "contact-offset", "friction", "deformation-damping",
                              "bending-damping", "bend-rest-from-geometry"}) {
            auto v = read_bin<float>(B + "param/rod-" + k + ".bin", false);
            if (!v.empty()) {
                if (v.size() != n_rod) die(std::string("rod-") + k + ".bin does not match count.rod");
                rp[k] = v;
            }
        }
        std::vector<PpfRodMaterial> rmats;
        std::vector<unsigned> rmat(n_rod);
        for (unsigned i = 0; i < n_rod; ++i) {
            auto get = [&](const char *name, float dflt) {
                auto it = rp.find(name);
                return it == rp.end() ? dflt : it->second[i];
            };
            PpfRodMaterial m{};
            m.density = get("density", 1.0f);
            m.young_mod = get("young-mod", 1000.0f);
            m.bend = get("bend", 0.0f);
            m.length_factor = get("length-factor", 1.0f);
            m.strain_limit = get("strain-limit", 0.0f);
            m.contact_gap = get("contact-gap", 1e-3f);
            m.contact_offset = get("contact-offset", 0.0f);
            m.friction = get("friction", 0.0f);
            m.deform_damping = get("deformation-damping", 0.0f);
            m.bend_damping = get("bending-damping", 0.0f);
            m.bend_rest_from_geometry = get("bend-rest-from-geometry", 0.0f) != 0.0f;
            unsigned k = 0;
            while (k < rmats.size() && std::memcmp(&rmats[k], &m, sizeof(m)) != 0) ++k;
            if (k == rmats.size()) rmats.push_back(m);
            rmat[i] = k;
        }
        if (ppf_scene_add_rod_edges(L.scene, rod.data(), n_rod, rmat.data(), rmats.data(),
                                    (unsigned)rmats.size()) != 0)
            die("rod.bin names a vertex past count.vert");
    }
    if (n_stitch) {
        // stitches (scene.rs:504-520, 748-756): six indices and weights each,
        // and a per-stitch stiffness (1 where the file is absent)
        const auto ind = read_bin<uint64_t>(B + "stitch_ind.bin");
        const auto w = read_bin<float>(B + "stitch_w.bin");
        auto k = read_bin<float>(B + "stitch_stiffness.bin", false);
        if (ind.size() != 6 * (size_t)n_stitch || w.size() != 6 * (size_t)n_stitch)
            die("stitch_ind.bin / stitch_w.bin do not match count.stitch");
        if (k.empty()) k.assign(n_stitch, 1.0f);
        if (k.size() != n_stitch) die("stitch_stiffness.bin does not match count.stitch");
        for (unsigned i = 0; i < n_stitch; ++i) {
            unsigned idx[6];
            for (int a = 0; a < 6; ++a) idx[a] = (unsigned)ind[6 * i + a];
            if (ppf_scene_add_stitch(L.scene, idx, &w[6 * i], k[i]) != 0)
                die("stitch_ind.bin names a vertex past count.vert");
        }
    }
    std::vector<float> v3(vel.begin(), vel.end());
    for (float &c : v3) c = (float)(c * ws);
    ppf_scene_set_velocity(L.scene, v3.data());

    // pins (fix pins without operations; a pull weight makes a pull pin)
    for (unsigned i = 0; i < n_pin; ++i) {
        const std::string sec = "pin-" + std::to_string(i);
        if (num(info, sec, "operation_count", 0.0) != 0.0)
            die("pin operations (moving pins) are not supported by this driver");
        auto ind64 = read_bin<uint64_t>(B + "pin-ind-" + std::to_string(i) + ".bin");
        std::vector<unsigned> ind(ind64.begin(), ind64.end());
        const float pull = (float)num(info, sec, "pull", 0.0);
        if (pull > 0.0f) ppf_scene_pull(L.scene, ind.data(), (unsigned)ind.size(), pull);
        else ppf_scene_pin(L.scene, ind.data(), (unsigned)ind.size(), 0);
    }
    // walls and spheres at their first keyframe
    for (unsigned i = 0; i < n_wall; ++i) {
        const std::string sec = "wall-" + std::to_string(i);
        if (num(info, sec, "keyframe", 0.0) < 1.0) continue;
        auto pos = read_bin<double>(B + "wall-pos-" + std::to_string(i) + ".bin");
        if (pos.size() < 3) die("wall-pos file is empty");
        float g[3] = {(float)(pos[0] * ws), (float)(pos[1] * ws), (float)(pos[2] * ws)};
        float up[3] = {(float)num(info, sec, "nx", 0.0), (float)num(info, sec, "ny", 1.0),
                       (float)num(info, sec, "nz", 0.0)};
        const float nrm = std::sqrt(up[0] * up[0] + up[1] * up[1] + up[2] * up[2]);
        for (float &c : up) c /= nrm;
        ppf_scene_add_floor(L.scene, g, up, (float)num(info, sec, "contact-gap", 1e-3),
                            (float)num(info, sec, "friction", 0.0));
    }
    for (unsigned i = 0; i < n_sphere; ++i) {
        const std::string sec = "sphere-" + std::to_string(i);
        if (num(info, sec, "keyframe", 0.0) < 1.0) continue;
        auto pos = read_bin<double>(B + "sphere-pos-" + std::to_string(i) + ".bin");
        auto rad = read_bin<float>(B + "sphere-radius-" + std::to_string(i) + ".bin");
        if (pos.size() < 3 || rad.empty()) die("sphere keyframe files are empty");
        float c[3] = {(float)(pos[0] * ws), (float)(pos[1] * ws), (float)(pos[2] * ws)};
        ppf_scene_add_sphere(L.scene, c, (float)(rad[0] * ws),
                             (float)num(info, sec, "contact-gap", 1e-3),
                             (float)num(info, sec, "friction", 0.0),
                             num(info, sec, "invert", 0.0) != 0.0,
                             num(info, sec, "hemisphere", 0.0) != 0.0);
    }
    // static collision mesh, one builder mesh per distinct contact parameter set
    if (n_st) {
        const auto sv = read_bin<double>(B + "static_vert.bin");
        const auto sdm = read_bin<uint32_t>(B + "static_vert_dmap.bin");
        const auto st64 = read_bin<uint64_t>(B + "static_tri.bin");
        if (sv.size() != 3 * (size_t)n_sv || sdm.size() != n_sv || st64.size() != 3 * (size_t)n_st)
            die("static mesh files do not match their counts");
        std::vector<float> sx(3 * (size_t)n_sv);
        for (unsigned i = 0; i < n_sv; ++i)
            for (int d = 0; d < 3; ++d)
                sx[3 * i + d] = (float)(sv[3 * i + d] * ws) + (float)(disp[3 * sdm[i] + d] * ws);
        auto sp = [&](const char *k, float dflt) {
            auto v = read_bin<float>(B + std::string("param/static-") + k + ".bin", false);
            if (v.empty()) v.assign(n_st, dflt);
            if (v.size() != n_st) die(std::string("static-") + k + ".bin does not match");
            return v;
        };
        const auto gap = sp("contact-gap", 1e-3f), off = sp("contact-offset", 0.0f),
                   fr = sp("friction", 0.0f);
        std::vector<char> done(n_st, 0);
        for (unsigned a = 0; a < n_st; ++a) {
            if (done[a]) continue;
            std::vector<unsigned> faces;
            for (unsigned b = a; b < n_st; ++b)
                if (!done[b] && gap[b] == gap[a] && off[b] == off[a] && fr[b] == fr[a]) {
                    done[b] = 1;
                    for (int k = 0; k < 3; ++k) faces.push_back((unsigned)st64[3 * b + k]);
                }
            ppf_scene_add_collision_mesh(L.scene, sx.data(), n_sv, faces.data(),
                                         (unsigned)faces.size() / 3, gap[a], off[a], fr[a]);
        }
    }
    PpfParamSet p;
    ppf_scene_default_param(&p);
    set_param(p, prm);
    // a step never spans a whole frame (builder.rs:273-275)
    p.dt = std::min(p.dt, (float)(0.9999 / L.fps));
    p.prev_dt = p.dt;
    if (ppf_scene_build(L.scene, &p) != 0) die("degenerate triangle in the scene");
    return L;
}

// ---- checkpoints ---------------------------------------------------------------
constexpr char kStateMagic[8] = {'P', 'P', 'F', 'G', 'B', '3', 'S', '1'};

struct State {
    int frame = 0;
    double time = 0.0;
    float prev_dt = 0.0f;
    std::vector<float> curr, prev;
    std::vector<unsigned> dyn_offset, dyn_index;
};

void save_state(const std::string &out, const State &s) {
    const std::string path = out + "/state_" + std::to_string(s.frame) + ".bin";
    std::ofstream f(path + ".tmp", std::ios::binary);
    auto put = [&](const void *p, size_t n) { f.write(reinterpret_cast<const char *>(p), n); };
    const uint64_t nv = s.curr.size() / 3, no = s.dyn_offset.size(), ni = s.dyn_index.size();
    put(kStateMagic, 8);
    put(&s.frame, sizeof(s.frame));
    put(&s.time, sizeof(s.time));
    put(&s.prev_dt, sizeof(s.prev_dt));
    put(&nv, 8);
    put(s.curr.data(), s.curr.size() * 4);
    put(s.prev.data(), s.prev.size() * 4);
    put(&no, 8);
    put(s.dyn_offset.data(), no * 4);
    put(&ni, 8);
    put(s.dyn_index.data(), ni * 4);
    f.close();
    std::rename((path + ".tmp").c_str(), path.c_str());
}

State load_state(const std::string &out, int frame) {
    const std::string path = out + "/state_" + std::to_string(frame) + ".bin";
    std::ifstream f(path, std::ios::binary);
    if (!f) die("no checkpoint " + path);
    auto get = [&](void *p, size_t n) {
        f.read(reinterpret_cast<char *>(p), n);
        if (!f) die("truncated checkpoint " + path);
    };
    char magic[8];
    get(magic, 8);
    if (std::memcmp(magic, kStateMagic, 8) != 0) die(path + " is not a checkpoint of this solver");
    State s;
    uint64_t nv, no, ni;
    get(&s.frame, sizeof(s.frame));
    get(&s.time, sizeof(s.time));
    get(&s.prev_dt, sizeof(s.prev_dt));
    get(&nv, 8);
    s.curr.resize(3 * nv);
    s.prev.resize(3 * nv);
    get(s.curr.data(), 12 * nv);
    get(s.prev.data(), 12 * nv);
    get(&no, 8);
    s.dyn_offset.resize(no);
    get(s.dyn_offset.data(), 4 * no);
    get(&ni, 8);
    s.dyn_index.resize(ni);
    get(s.dyn_index.data(), 4 * ni);
    return s;
}

void append_line(const std::string &path, const std::string &line) {
    std::ofstream f(path, std::ios::app);
    f << line << "\n";
}

// vert_<frame>.bin at t_frame, between the step's start (prev, t_prev) and
// end (curr, t_curr) (backend.rs:1037-1044 for the weight)
void write_frame(const std::string &out, int frame, double t_frame, double t_prev,
                 double t_curr, const float *prev, const float *curr, unsigned n,
                 float inv_world) {
    const double span = t_curr - t_prev;
    const float alpha =
        span > 1e-12 ? (float)std::min(1.0, std::max(0.0, (t_frame - t_prev) / span)) : 1.0f;
    std::vector<float> buf(3 * (size_t)n);
    for (size_t k = 0; k < buf.size(); ++k)
        buf[k] = (prev[k] + alpha * (curr[k] - prev[k])) * inv_world;
    const std::string path = out + "/vert_" + std::to_string(frame) + ".bin";
    {
        std::ofstream f(path + ".tmp", std::ios::binary);
        f.write(reinterpret_cast<const char *>(buf.data()), buf.size() * 4);
    }
    std::rename((path + ".tmp").c_str(), path.c_str());
}

} // namespace

int main(int argc, char **argv) {
    std::string path, out = "output";
    int load = 0;
    bool describe = false;
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        auto next = [&]() -> std::string {
            if (i + 1 >= argc) die("missing value for " + a);
            return argv[++i];
        };
        if (a == "--path") path = next();
        else if (a == "--output") out = next();
        else if (a == "--load") load = std::atoi(next().c_str());
        else if (a == "--describe") describe = true;
        else if (a == "--help" || a == "-h") {
            std::printf("usage: ppf-contact-solver --path <scene> --output <dir> [--load N]"
                        " [--describe]\n");
            return 0;
        } else die("unknown argument " + a);
    }
    if (path.empty() || !exists(path)) die("--path must name a scene directory");
    Loaded L = load_scene(path);
    PpfDataSet *ds = ppf_scene_dataset(L.scene);
    PpfParamSet *param = ppf_scene_param(L.scene);
    if (describe) {
        // the scene as read, without a GPU: one "key value" per line
        const PpfConstraint &c = ds->constraint;
        std::printf("vertices %u\nfaces %u\nrods %u\nstitches %u\nedges %u\nhinges %u\nfix %u\npull %u\n"
                    "spheres %u\nfloors %u\ncollision_vertices %u\ncollision_faces %u\n"
                    "face_params %u\ndt %.9g\nframes %d\nfps %.9g\nauto_save %d\n"
                    "gravity %.9g %.9g %.9g\ncg_tol %.9g\n",
                    ds->vertex.curr.size, ds->mesh.mesh.face.size, ds->rod_count,
                    c.stitch.size,
                    ds->mesh.mesh.edge.size,
                    ds->mesh.mesh.hinge.size, c.fix.size, c.pull.size, c.sphere.size,
                    c.floor.size, c.mesh.vertex.size, c.mesh.face.size,
                    ds->param_arrays.face.size, param->dt, L.frames, L.fps, L.auto_save,
                    param->gravity.v[0], param->gravity.v[1], param->gravity.v[2],
                    param->cg_tol);
        return 0;
    }
    mkdirs(out + "/data");
    const unsigned n = L.n_vert;
    int frame = 0;
    if (load < 0) {
        // resume from the latest checkpoint
        for (int f = L.frames; f >= 1 && load < 0; --f)
            if (exists(out + "/state_" + std::to_string(f) + ".bin")) load = f;
        if (load < 0) die("--load -1 but no checkpoint in " + out);
    }
    State resume;
    if (load > 0) {
        resume = load_state(out, load);
        if (resume.curr.size() != 3 * (size_t)ppf_scene_vertex_count(L.scene))
            die("the checkpoint does not match the scene");
        ppf_scene_set_positions(L.scene, resume.curr.data(), resume.prev.data());
        param->time = resume.time;
        param->prev_dt = resume.prev_dt;
        frame = resume.frame;
    }
    set_log_path((out + "/data").c_str());
    if (!initialize(ds, param)) {
        std::fprintf(stderr, "ppf-contact-solver: initialize failed (fatal code %u): %s\n",
                     (unsigned)ppf_fatal_code(), ppf_fatal_detail());
        return 1;
    }
    if (load > 0 && !param->disable_contact && !resume.dyn_offset.empty())
        update_dyn(resume.dyn_index.data(), resume.dyn_offset.data());
    const float inv_world = 1.0f / L.world_scaling;
    const unsigned nall = ppf_scene_vertex_count(L.scene);
    std::vector<float> prev_x(3 * (size_t)nall), curr_x(3 * (size_t)nall);
    ppf_scene_positions(L.scene, curr_x.data(), nullptr);
    if (load == 0) {
        write_frame(out, 0, 0.0, 0.0, 0.0, curr_x.data(), curr_x.data(), n, inv_world);
        append_line(out + "/data/frame_to_time.out", "0 0");
    }
    auto checkpoint = [&](int f) {
        State s;
        s.frame = f;
        s.time = param->time;
        s.prev_dt = param->prev_dt;
        s.curr.resize(3 * (size_t)nall);
        s.prev.resize(3 * (size_t)nall);
        ppf_scene_positions(L.scene, s.curr.data(), s.prev.data());
        unsigned nv = 0, no = 0;
        fetch_dyn_counts(&nv, &no);
        s.dyn_offset.resize(no);
        s.dyn_index.resize(nv);
        fetch_dyn(s.dyn_index.data(), nullptr, s.dyn_offset.data());
        save_state(out, s);
    };
    auto last_frame = std::chrono::steady_clock::now();
    while (frame < L.frames) {
        const double t_prev = param->time;
        prev_x = curr_x;
        PpfStepResult r{};
        advance(&r);
        if (ppf_fatal_code()) {
            std::fprintf(stderr, "ppf-contact-solver: fatal code %u: %s\n",
                         (unsigned)ppf_fatal_code(), ppf_fatal_detail());
            return 1;
        }
        if (!(r.ccd_success && r.pcg_success && r.intersection_free && r.newton_progress &&
              r.pin_feasible && r.contact_separated)) {
            std::fprintf(stderr,
                         "ppf-contact-solver: step failed at t=%g (ccd %d, pcg %d, intersection "
                         "free %d, newton progress %d, pin feasible %d, contact separated %d)\n",
                         t_prev, r.ccd_success, r.pcg_success, r.intersection_free,
                         r.newton_progress, r.pin_feasible, r.contact_separated);
            return 1;
        }
        fetch();
        ppf_scene_positions(L.scene, curr_x.data(), nullptr);
        const double t_curr = param->time;
        while (frame < L.frames && (double)(frame + 1) / L.fps <= t_curr + 1e-12) {
            ++frame;
            const double t_frame = (double)frame / L.fps;
            write_frame(out, frame, t_frame, t_prev, t_curr, prev_x.data(), curr_x.data(), n,
                        inv_world);
            const auto now = std::chrono::steady_clock::now();
            append_line(out + "/data/time_per_frame.out",
                        std::to_string(frame) + " " +
                            std::to_string(std::chrono::duration_cast<std::chrono::milliseconds>(
                                               now - last_frame)
                                               .count()));
            last_frame = now;
            char tbuf[64];
            std::snprintf(tbuf, sizeof(tbuf), "%d %.17g", frame, t_frame);
            append_line(out + "/data/frame_to_time.out", tbuf);
            if (L.auto_save > 0 && frame % L.auto_save == 0) checkpoint(frame);
        }
    }
    checkpoint(frame);
    append_line(out + "/finished.txt", "frames " + std::to_string(frame));
    return 0;
}
