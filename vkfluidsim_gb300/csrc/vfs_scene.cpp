// Scene layer of the C ABI: the scene-JSON loader and GenericScene spawn logic
// (src/util/scene_loader.cpp:42-140, src/scenes/generic_scene.cpp:10-57), the particle spawners
// of SPHModel (src/models/model.cpp:13-66, 117-137) and seeded synthetic-input generators.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "vfs_cuda.h"
#include "vfs_model.h"

namespace vfs {
namespace {

// ------------------------------------------------------------------ minimal JSON

struct Json {
    enum Type { Null, Bool, Number, String, Array, Object } type = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Json> arr;
    std::vector<std::pair<std::string, Json>> obj;

    const Json* get(const std::string& k) const {
        for (const auto& kv : obj)
            if (kv.first == k) return &kv.second;
        return nullptr;
    }
};

struct Parser {
    const std::string& s;
    size_t i = 0;
    std::string error;

    explicit Parser(const std::string& src) : s(src) {}

    void ws() {
        while (i < s.size() && (s[i] == ' ' || s[i] == '\n' || s[i] == '\r' || s[i] == '\t')) i++;
    }
    bool fail_at(const std::string& what) {
        if (error.empty()) error = what + " at offset " + std::to_string(i);
        return false;
    }
    bool literal(const char* lit) {
        const size_t n = std::strlen(lit);
        if (s.compare(i, n, lit) != 0) return fail_at(std::string("expected ") + lit);
        i += n;
        return true;
    }
    bool string(std::string& out) {
        if (i >= s.size() || s[i] != '"') return fail_at("expected string");
        i++;
        out.clear();
        while (i < s.size() && s[i] != '"') {
            char c = s[i++];
            if (c == '\\') {
                if (i >= s.size()) return fail_at("bad escape");
                const char e = s[i++];
                switch (e) {
                    case 'n': out += '\n'; break;
                    case 't': out += '\t'; break;
                    case 'r': out += '\r'; break;
                    case 'b': out += '\b'; break;
                    case 'f': out += '\f'; break;
                    case 'u':
                        if (i + 4 > s.size()) return fail_at("bad \\u escape");
                        out += '?';
                        i += 4;
                        break;
                    default: out += e;
                }
            } else {
                out += c;
            }
        }
        if (i >= s.size()) return fail_at("unterminated string");
        i++;
        return true;
    }
    bool value(Json& v, int depth) {
        if (depth > 64) return fail_at("nesting too deep");
        ws();
        if (i >= s.size()) return fail_at("unexpected end");
        const char c = s[i];
        if (c == '{') {
            v.type = Json::Object;
            i++;
            ws();
            if (i < s.size() && s[i] == '}') {
                i++;
                return true;
            }
            while (true) {
                ws();
                std::string key;
                if (!string(key)) return false;
                ws();
                if (i >= s.size() || s[i] != ':') return fail_at("expected ':'");
                i++;
                Json child;
                if (!value(child, depth + 1)) return false;
                v.obj.emplace_back(std::move(key), std::move(child));
                ws();
                if (i < s.size() && s[i] == ',') {
                    i++;
                    continue;
                }
                if (i < s.size() && s[i] == '}') {
                    i++;
                    return true;
                }
                return fail_at("expected ',' or '}'");
            }
        }
        if (c == '[') {
            v.type = Json::Array;
            i++;
            ws();
            if (i < s.size() && s[i] == ']') {
                i++;
                return true;
            }
            while (true) {
                Json child;
                if (!value(child, depth + 1)) return false;
                v.arr.push_back(std::move(child));
                ws();
                if (i < s.size() && s[i] == ',') {
                    i++;
                    continue;
                }
                if (i < s.size() && s[i] == ']') {
                    i++;
                    return true;
                }
                return fail_at("expected ',' or ']'");
            }
        }
        if (c == '"') {
            v.type = Json::String;
            return string(v.str);
        }
        if (c == 't') {
            v.type = Json::Bool;
            v.b = true;
            return literal("true");
        }
        if (c == 'f') {
            v.type = Json::Bool;
            v.b = false;
            return literal("false");
        }
        if (c == 'n') {
            v.type = Json::Null;
            return literal("null");
        }
        // number
        const size_t start = i;
        if (s[i] == '-' || s[i] == '+') i++;
        while (i < s.size() && ((s[i] >= '0' && s[i] <= '9') || s[i] == '.' || s[i] == 'e' ||
                                s[i] == 'E' || s[i] == '-' || s[i] == '+'))
            i++;
        if (i == start) return fail_at("unexpected character");
        try {
            size_t used = 0;
            v.num = std::stod(s.substr(start, i - start), &used);
            if (used != i - start) return fail_at("bad number");
        } catch (...) {
            return fail_at("bad number");
        }
        v.type = Json::Number;
        return true;
    }
};

struct SceneError {
    std::string msg;
};

const Json& need(const Json& o, const char* key) {
    if (o.type != Json::Object) throw SceneError{std::string("expected an object holding '") + key + "'"};
    const Json* v = o.get(key);
    if (!v) throw SceneError{std::string("missing key '") + key + "'"};
    return *v;
}

double num(const Json& v, const char* what) {
    if (v.type != Json::Number) throw SceneError{std::string("'") + what + "' must be a number"};
    return v.num;
}

void vec3(const Json& v, float* out, const char* what) {
    if (v.type != Json::Array || v.arr.size() < 3) throw SceneError{std::string("'") + what + "' must be an array of 3 numbers"};
    for (int a = 0; a < 3; a++) out[a] = (float)num(v.arr[a], what);
}

void uvec3(const Json& v, uint32_t* out, const char* what) {
    if (v.type != Json::Array || v.arr.size() < 3) throw SceneError{std::string("'") + what + "' must be an array of 3 integers"};
    for (int a = 0; a < 3; a++) {
        const double d = num(v.arr[a], what);
        if (d < 0 || d != std::floor(d) || d > 4294967295.0)
            throw SceneError{std::string("'") + what + "' must hold non-negative integers"};
        out[a] = (uint32_t)d;
    }
}

// ------------------------------------------------------------------ counter-based RNG

inline uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

inline double u01(uint64_t seed, uint64_t index) {
    return (double)(splitmix64(splitmix64(seed) ^ splitmix64(index ^ 0xD1B54A32D192ED03ull)) >> 11) *
           (1.0 / 9007199254740992.0);
}

// SpawnCompactParticlesInBox, src/models/model.cpp:35-66 (float arithmetic kept).
std::vector<float> spawn_compact(const float size[3], const float pos[3], uint32_t count, float density) {
    std::vector<float> out((size_t)count * 3, 0.0f);
    const float volume = 1 / density;
    const float diameter = std::cbrt(volume);
    const float nx = std::round(size[0] / diameter) - 1;
    const float ny = std::round(size[1] / diameter) - 1;
    const float nz = std::round(size[2] / diameter) - 1;
    uint32_t p = 0;
    for (uint32_t i = 0; i < nx; i++)
        for (uint32_t j = 0; j < ny; j++)
            for (uint32_t k = 0; k < nz; k++) {
                if (p >= count) return out;
                out[3 * (size_t)p] = diameter * (float)i + pos[0];
                out[3 * (size_t)p + 1] = diameter * (float)j + pos[1];
                out[3 * (size_t)p + 2] = diameter * (float)k + pos[2];
                p++;
                if (p >= count) return out;
            }
    return out;
}

// SpawnRandomParticlesInBox, src/models/model.cpp:13-33, with a seeded generator.
std::vector<float> spawn_random(const float size[3], const float pos[3], uint32_t count, uint64_t seed) {
    std::vector<float> out((size_t)count * 3);
    for (uint32_t i = 0; i < count; i++)
        for (int a = 0; a < 3; a++)
            out[3 * (size_t)i + a] = pos[a] + (float)u01(seed, 3ull * i + a) * size[a];
    return out;
}

int spawn_in_box(Model& m, uint32_t scene, const float size[3], const float pos[3],
                 uint32_t offset, int64_t count, int32_t mode, uint64_t seed) {
    if (count == 0) return VFS_OK;
    if (scene >= m.scenes.size()) return fail(VFS_ERR_INVALID_ARGUMENT, "scene index out of range");
    const SceneHost& sh = m.scenes[scene];
    const uint32_t cnt = count > 0 ? (uint32_t)count : sh.n;
    if ((uint64_t)offset + cnt > sh.n) return fail(VFS_ERR_CAPACITY, "spawn exceeds the scene's particle count");
    std::vector<float> p = mode == 1 ? spawn_random(size, pos, cnt, seed)
                                     : spawn_compact(size, pos, cnt, sh.sph.target_density);
    std::vector<float> v((size_t)cnt * 3, 0.0f);
    return m.set_state(scene, p.data(), v.data(), offset, cnt);
}

// GenericScene::Reset, src/scenes/generic_scene.cpp:42-57.
int reset_blocks(Model& m) {
    const float density = m.scenes[0].sph.target_density;
    const float particle_volume = 1 / density;
    const float particle_diam = std::cbrt(particle_volume);
    uint32_t offset = 0;
    for (const FluidBlock& b : m.scenes[0].blocks) {
        const uint32_t count = b.size[0] * b.size[1] * b.size[2];
        float size[3];
        for (int a = 0; a < 3; a++) size[a] = particle_diam * (float)(b.size[a] + 1u);
        const int rc = spawn_in_box(m, 0, size, b.pos, offset, count, 0, 0);
        if (rc) return rc;
        offset += count;
    }
    return VFS_OK;
}

}  // namespace
}  // namespace vfs

using vfs::fail;

extern "C" {

int vfs_model_set_particles_in_box(vfs_model* h, const float box_size[3], const float box_pos[3],
                                   uint32_t offset, int64_t count, int32_t mode, uint64_t seed) {
    vfs::Model* m = vfs_model_impl(h);
    if (!m || !box_size || !box_pos) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL argument");
    try {
        return vfs::spawn_in_box(*m, 0, box_size, box_pos, offset, count, mode, seed);
    } catch (const std::exception& e) {
        return fail(VFS_ERR_OUT_OF_MEMORY, e.what());
    }
}

// LoadScene (src/util/scene_loader.cpp:113-140) + GenericScene::Init (generic_scene.cpp:21-41).
int vfs_scene_load(const char* json_path, const char* resources_dir, vfs_model** out) {
    using namespace vfs;
    if (!json_path || !out) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    std::ifstream f(json_path, std::ios::binary);
    if (!f) return fail(VFS_ERR_IO, std::string("cannot open scene file '") + json_path + "'");
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string text = ss.str();
    Json root;
    Parser parser(text);
    if (!parser.value(root, 0)) return fail(VFS_ERR_PARSE, "scene JSON: " + parser.error);
    parser.ws();
    if (parser.i != text.size()) return fail(VFS_ERR_PARSE, "scene JSON: trailing characters");

    vfs_sim_params sim{};
    vfs_sph_params sph{};
    vfs_wcsph_params wc{};
    std::vector<FluidBlock> blocks;
    std::vector<vfs_analytic_object> objects;
    std::vector<std::string> mesh_paths;  // per object: the OBJ path, or empty for an analytic shape
    try {
        // Simulation::Init defaults (src/simulation.cpp:20-27), overridden when present.
        sim.gravity[0] = 0.0f;
        sim.gravity[1] = -9.81f;
        sim.gravity[2] = 0.0f;
        sim.smooth_radius = 0.2f;
        const Json& sp = need(root, "simulationParameters");
        if (const Json* g = sp.get("gravity")) vec3(*g, sim.gravity, "gravity");
        if (const Json* r = sp.get("smoothRadius")) sim.smooth_radius = (float)num(*r, "smoothRadius");
        sph.time_scale = (float)num(need(sp, "timeScale"), "timeScale");
        sph.iterations = (int32_t)num(need(sp, "iterations"), "iterations");
        sph.fixed_dt = (float)num(need(sp, "dt"), "dt");
        sph.target_density = (float)num(need(sp, "targetDensity"), "targetDensity");
        const Json& bb = need(sp, "boundingBox");
        vec3(need(bb, "pos"), sph.bbox_pos, "boundingBox.pos");
        vec3(need(bb, "size"), sph.bbox_size, "boundingBox.size");

        const Json& wp = need(root, "wcsphParameters");
        wc.stiffness = (float)num(need(wp, "stiffness"), "stiffness");
        wc.expoent = (float)num(need(wp, "expoent"), "expoent");
        wc.viscosity_strenght = (float)num(need(wp, "viscosityStrenght"), "viscosityStrenght");
        wc.wall_stiffness = (float)num(need(wp, "outerWallStiffness"), "outerWallStiffness");

        const Json& fb = need(root, "fluidBlocks");
        if (fb.type != Json::Array) throw SceneError{"'fluidBlocks' must be an array"};
        uint64_t total = 0;
        for (const Json& b : fb.arr) {
            FluidBlock blk{};
            uvec3(need(b, "size"), blk.size, "fluidBlocks.size");
            vec3(need(b, "pos"), blk.pos, "fluidBlocks.pos");
            total += (uint64_t)blk.size[0] * blk.size[1] * blk.size[2];
            blocks.push_back(blk);
        }
        if (total > kMaxParticles) throw SceneError{"fluid blocks exceed 2^30 particles"};
        sph.n_particles = (int32_t)total;

        const Json& bo = need(root, "boundaryObjects");
        if (bo.type != Json::Array) throw SceneError{"'boundaryObjects' must be an array"};
        for (const Json& o : bo.arr) {
            vfs_analytic_object a{};
            a.scale[0] = a.scale[1] = a.scale[2] = 1.0f;
            if (const Json* p = o.get("position")) vec3(*p, a.position, "position");
            if (const Json* r = o.get("rotation")) {
                a.rotation_angle_deg = (float)num(need(*r, "angle"), "rotation.angle");
                vec3(need(*r, "axis"), a.rotation_axis, "rotation.axis");
            }
            if (const Json* s = o.get("scale")) vec3(*s, a.scale, "scale");
            uvec3(need(o, "volumeMapResolution"), a.resolution, "volumeMapResolution");
            // Extension: analytic shapes in place of OBJ meshes.
            if (const Json* shape = o.get("shape")) {
                const std::string type = need(*shape, "type").str;
                if (type == "sphere") {
                    a.shape = VFS_SHAPE_SPHERE;
                    a.params[0] = num(need(*shape, "radius"), "shape.radius");
                } else if (type == "box" || type == "container") {
                    a.shape = type == "box" ? VFS_SHAPE_BOX : VFS_SHAPE_CONTAINER;
                    float he[3];
                    vec3(need(*shape, "halfExtents"), he, "shape.halfExtents");
                    for (int k = 0; k < 3; k++) a.params[k] = he[k];
                } else {
                    throw SceneError{"unknown shape type '" + type + "'"};
                }
            }
            std::string path;
            if (!o.get("shape")) {
                // Platform::Info::ResourcePath: the path is relative to the resources directory.
                path = need(o, "resourcePath").str;
                if (resources_dir && *resources_dir) path = std::string(resources_dir) + "/" + path;
            }
            objects.push_back(a);
            mesh_paths.push_back(path);
        }
    } catch (const SceneError& e) {
        return fail(VFS_ERR_PARSE, "scene JSON: " + e.msg);
    }

    vfs_model* h = nullptr;
    int rc = vfs_model_create(&sim, &sph, &wc, &h);
    if (rc) return rc;
    Model* m = vfs_model_impl(h);
    for (size_t k = 0; k < objects.size(); k++) {
        const vfs_analytic_object& a = objects[k];
        if (mesh_paths[k].empty()) {
            rc = m->add_analytic(0, a);
        } else {
            vfs_mesh_object mo{};
            mo.obj_path = mesh_paths[k].c_str();
            for (int c = 0; c < 3; c++) {
                mo.position[c] = a.position[c];
                mo.rotation_axis[c] = a.rotation_axis[c];
                mo.scale[c] = a.scale[c];
                mo.resolution[c] = a.resolution[c];
            }
            mo.rotation_angle_deg = a.rotation_angle_deg;
            rc = m->add_mesh(0, mo);
        }
        if (rc) {
            vfs_model_destroy(h);
            return rc;
        }
    }
    m->scenes[0].blocks = blocks;
    rc = reset_blocks(*m);
    if (rc) {
        vfs_model_destroy(h);
        return rc;
    }
    *out = h;
    return VFS_OK;
}

int vfs_scene_reset(vfs_model* h) {
    vfs::Model* m = vfs_model_impl(h);
    if (!m) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL model");
    return vfs::reset_blocks(*m);
}

int vfs_generate_lattice(const uint32_t dims[3], const float origin[3], float spacing, float jitter,
                         uint64_t seed, float* pos_out) {
    if (!dims || !origin || !pos_out) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL argument");
    const uint64_t nx = dims[0], ny = dims[1], nz = dims[2];
    const uint64_t total = nx * ny * nz;
    for (uint64_t lin = 0; lin < total; lin++) {
        const uint64_t idx[3] = {lin % nx, (lin / nx) % ny, lin / (nx * ny)};
        for (int a = 0; a < 3; a++) {
            const double j = (2.0 * vfs::u01(seed, 3 * lin + a) - 1.0) * (double)jitter;
            pos_out[3 * lin + a] =
                (float)((double)origin[a] + (double)spacing * ((double)idx[a] + 0.5 + j));
        }
    }
    return VFS_OK;
}

int vfs_generate_uniform_blob(uint64_t n_uniform, const float lo[3], const float hi[3],
                              uint64_t n_blob, const float center[3], float sigma, uint64_t seed,
                              float* pos_out) {
    if (!pos_out || (n_uniform && (!lo || !hi)) || (n_blob && !center))
        return fail(VFS_ERR_INVALID_ARGUMENT, "NULL argument");
    for (uint64_t i = 0; i < n_uniform; i++)
        for (int a = 0; a < 3; a++)
            pos_out[3 * i + a] =
                (float)((double)lo[a] + vfs::u01(seed, 3 * i + a) * ((double)hi[a] - (double)lo[a]));
    const uint64_t base = 3 * n_uniform;
    for (uint64_t i = 0; i < n_blob; i++)
        for (int a = 0; a < 3; a++) {
            const uint64_t r = (1ull << 62) + 6 * i + 2 * a;
            double u1 = vfs::u01(seed, r);
            const double u2 = vfs::u01(seed, r + 1);
            if (u1 < 1e-300) u1 = 1e-300;
            const double g = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
            pos_out[base + 3 * i + a] = (float)((double)center[a] + (double)sigma * g);
        }
    return VFS_OK;
}

int vfs_generate_fourier_velocity(uint64_t n, const float* pos, int32_t modes, float amplitude,
                                  uint64_t seed, float* vel_out) {
    if ((n && (!pos || !vel_out)) || modes < 1) return fail(VFS_ERR_INVALID_ARGUMENT, "bad argument");
    std::vector<double> k(3 * modes), amp(3 * modes), ph(modes);
    const double two_pi = 6.283185307179586;
    for (int m = 0; m < modes; m++) {
        for (int a = 0; a < 3; a++) {
            k[3 * m + a] = two_pi * (2.0 * vfs::u01(seed, 100 + 7 * m + a) - 1.0) * 2.0;
            amp[3 * m + a] = 2.0 * vfs::u01(seed, 100 + 7 * m + 3 + a) - 1.0;
        }
        ph[m] = two_pi * vfs::u01(seed, 100 + 7 * m + 6);
    }
    double vmax = 0.0;
    std::vector<double> v(3 * n, 0.0);
    for (uint64_t i = 0; i < n; i++) {
        for (int m = 0; m < modes; m++) {
            const double arg = k[3 * m] * pos[3 * i] + k[3 * m + 1] * pos[3 * i + 1] +
                               k[3 * m + 2] * pos[3 * i + 2] + ph[m];
            const double s = std::sin(arg);
            for (int a = 0; a < 3; a++) v[3 * i + a] += amp[3 * m + a] * s;
        }
        const double sp = std::sqrt(v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] +
                                    v[3 * i + 2] * v[3 * i + 2]);
        if (sp > vmax) vmax = sp;
    }
    const double scale = vmax > 0.0 ? (double)amplitude / vmax : 0.0;
    for (uint64_t i = 0; i < 3 * n; i++) vel_out[i] = (float)(v[i] * scale);
    return VFS_OK;
}

}  // extern "C"
