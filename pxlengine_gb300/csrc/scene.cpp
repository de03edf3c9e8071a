// Scene-JSON front end for the liquid path. The reference deserialises with serde
// (`deny_unknown_fields` on Scene, Fluid and FluidBlock) and then runs Scene::validate; this
// file does the same for the fields the liquid path reads, with the same defaults and the same
// validation messages. Scene fields outside the liquid path (nodes beyond the camera check,
// world, animation, programs, simulations, plate, materials) are accepted as any JSON value.
#include "scene.h"

#include <cerrno>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <utility>

namespace pxf {

namespace {

struct JVal {
    enum Kind { Null, Bool, Num, Str, Arr, Obj } kind = Null;
    bool b = false;
    double num = 0;
    bool integral = false;   // written without fraction or exponent
    bool negative = false;
    std::string s;           // string value, or the number's literal text
    std::vector<JVal> arr;
    std::vector<std::pair<std::string, JVal>> obj;
    const JVal* get(const char* key) const {
        for (auto& kv : obj) if (kv.first == key) return &kv.second;
        return nullptr;
    }
};

struct Parser {
    const char* p;
    const char* begin;
    std::string err;
    int depth = 0;

    void ws() { while (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r') p++; }
    bool fail(const char* m) {
        if (err.empty()) {
            int line = 1, col = 1;
            for (const char* q = begin; q < p && *q; q++) { if (*q == '\n') { line++; col = 1; } else col++; }
            err = std::string(m) + " at line " + std::to_string(line) + " column " + std::to_string(col);
        }
        return false;
    }
    bool lit(const char* w) {
        size_t n = std::strlen(w);
        if (std::strncmp(p, w, n) != 0) return fail("expected value");
        p += n;
        return true;
    }
    bool str(std::string& out) {
        if (*p != '"') return fail("expected string");
        p++;
        while (*p != '"') {
            if (!*p) return fail("EOF while parsing a string");
            if ((unsigned char)*p < 0x20) return fail("control character in string");
            if (*p == '\\') {
                p++;
                switch (*p) {
                    case '"': out += '"'; break;
                    case '\\': out += '\\'; break;
                    case '/': out += '/'; break;
                    case 'b': out += '\b'; break;
                    case 'f': out += '\f'; break;
                    case 'n': out += '\n'; break;
                    case 'r': out += '\r'; break;
                    case 't': out += '\t'; break;
                    case 'u': {
                        unsigned cp = 0;
                        for (int i = 1; i <= 4; i++) {
                            char c = p[i];
                            cp <<= 4;
                            if (c >= '0' && c <= '9') cp |= unsigned(c - '0');
                            else if (c >= 'a' && c <= 'f') cp |= unsigned(c - 'a' + 10);
                            else if (c >= 'A' && c <= 'F') cp |= unsigned(c - 'A' + 10);
                            else return fail("invalid escape");
                        }
                        p += 4;
                        if (cp < 0x80) out += char(cp);
                        else if (cp < 0x800) { out += char(0xC0 | (cp >> 6)); out += char(0x80 | (cp & 0x3F)); }
                        else { out += char(0xE0 | (cp >> 12)); out += char(0x80 | ((cp >> 6) & 0x3F)); out += char(0x80 | (cp & 0x3F)); }
                        break;
                    }
                    default: return fail("invalid escape");
                }
                p++;
            } else {
                out += *p++;
            }
        }
        p++;
        return true;
    }
    bool num(JVal& v) {
        const char* s = p;
        if (*p == '-') { v.negative = true; p++; }
        if (!(*p >= '0' && *p <= '9')) return fail("invalid number");
        if (*p == '0' && p[1] >= '0' && p[1] <= '9') return fail("invalid number");
        while (*p >= '0' && *p <= '9') p++;
        bool integral = true;
        if (*p == '.') {
            integral = false;
            p++;
            if (!(*p >= '0' && *p <= '9')) return fail("invalid number");
            while (*p >= '0' && *p <= '9') p++;
        }
        if (*p == 'e' || *p == 'E') {
            integral = false;
            p++;
            if (*p == '+' || *p == '-') p++;
            if (!(*p >= '0' && *p <= '9')) return fail("invalid number");
            while (*p >= '0' && *p <= '9') p++;
        }
        v.kind = JVal::Num;
        v.s.assign(s, p);
        v.integral = integral;
        v.num = std::strtod(v.s.c_str(), nullptr);
        return true;
    }
    bool value(JVal& v) {
        if (++depth > 128) return fail("recursion limit exceeded");
        ws();
        bool ok = true;
        switch (*p) {
            case 'n': ok = lit("null"); v.kind = JVal::Null; break;
            case 't': ok = lit("true"); v.kind = JVal::Bool; v.b = true; break;
            case 'f': ok = lit("false"); v.kind = JVal::Bool; v.b = false; break;
            case '"': v.kind = JVal::Str; ok = str(v.s); break;
            case '[': {
                v.kind = JVal::Arr;
                p++;
                ws();
                if (*p == ']') { p++; break; }
                while (true) {
                    v.arr.emplace_back();
                    if (!value(v.arr.back())) { ok = false; break; }
                    ws();
                    if (*p == ',') { p++; continue; }
                    if (*p == ']') { p++; break; }
                    ok = fail("expected `,` or `]`");
                    break;
                }
                break;
            }
            case '{': {
                v.kind = JVal::Obj;
                p++;
                ws();
                if (*p == '}') { p++; break; }
                while (true) {
                    ws();
                    std::string key;
                    if (!str(key)) { ok = false; break; }
                    ws();
                    if (*p != ':') { ok = fail("expected `:`"); break; }
                    p++;
                    v.obj.emplace_back(std::move(key), JVal());
                    if (!value(v.obj.back().second)) { ok = false; break; }
                    ws();
                    if (*p == ',') { p++; continue; }
                    if (*p == '}') { p++; break; }
                    ok = fail("expected `,` or `}`");
                    break;
                }
                break;
            }
            default:
                if (*p == '-' || (*p >= '0' && *p <= '9')) ok = num(v);
                else ok = fail("expected value");
        }
        depth--;
        return ok;
    }
};

// serde-style type errors ("invalid type: ..., expected ...").
std::string unexpected(const JVal& v) {
    switch (v.kind) {
        case JVal::Null: return "null";
        case JVal::Bool: return std::string("boolean `") + (v.b ? "true" : "false") + "`";
        case JVal::Num:
            if (v.integral) return "integer `" + v.s + "`";
            return "floating point `" + v.s + "`";
        case JVal::Str: return "string \"" + v.s + "\"";
        case JVal::Arr: return "sequence";
        default: return "map";
    }
}

bool get_f32(const JVal& v, float& out, std::string& err) {
    if (v.kind != JVal::Num) { err = "invalid type: " + unexpected(v) + ", expected f32"; return false; }
    out = float(v.num);   // serde_json: f64 then `as f32`
    return true;
}

bool get_u32(const JVal& v, uint32_t& out, std::string& err) {
    if (v.kind != JVal::Num || !v.integral) { err = "invalid type: " + unexpected(v) + ", expected u32"; return false; }
    if (v.negative) {
        if (v.s == "-0") { out = 0; return true; }
        err = "invalid value: integer `" + v.s + "`, expected u32";
        return false;
    }
    errno = 0;
    unsigned long long x = std::strtoull(v.s.c_str(), nullptr, 10);
    if (errno || x > 0xffffffffull) { err = "invalid value: integer `" + v.s + "`, expected u32"; return false; }
    out = uint32_t(x);
    return true;
}

bool get_vec3(const JVal& v, float out[3], std::string& err) {
    if (v.kind != JVal::Arr) { err = "invalid type: " + unexpected(v) + ", expected an array of length 3"; return false; }
    if (v.arr.size() != 3) { err = "invalid length " + std::to_string(v.arr.size()) + ", expected an array of length 3"; return false; }
    for (int i = 0; i < 3; i++) if (!get_f32(v.arr[i], out[i], err)) return false;
    return true;
}

bool check_fields(const JVal& o, const char* const* known, int n, std::string& err) {
    for (auto& kv : o.obj) {
        bool ok = false;
        for (int i = 0; i < n; i++) if (kv.first == known[i]) ok = true;
        if (!ok) {
            err = "unknown field `" + kv.first + "`, expected ";
            if (n == 1) {
                err += std::string("`") + known[0] + "`";
            } else {
                err += "one of ";
                for (int i = 0; i < n; i++) err += std::string(i ? ", `" : "`") + known[i] + "`";
            }
            return false;
        }
    }
    // serde rejects duplicate keys in a struct.
    for (size_t i = 0; i < o.obj.size(); i++)
        for (size_t j = i + 1; j < o.obj.size(); j++)
            if (o.obj[i].first == o.obj[j].first) { err = "duplicate field `" + o.obj[i].first + "`"; return false; }
    return true;
}

bool parse_block(const JVal& v, pxf_fill_block& b, std::string& err) {
    static const char* const known[] = {"min", "max", "velocity"};
    if (v.kind != JVal::Obj) { err = "invalid type: " + unexpected(v) + ", expected struct FluidBlock"; return false; }
    if (!check_fields(v, known, 3, err)) return false;
    const JVal* mn = v.get("min");
    const JVal* mx = v.get("max");
    if (!mn) { err = "missing field `min`"; return false; }
    if (!mx) { err = "missing field `max`"; return false; }
    if (!get_vec3(*mn, b.min, err) || !get_vec3(*mx, b.max, err)) return false;
    b.velocity[0] = b.velocity[1] = b.velocity[2] = 0.0f;
    if (const JVal* vel = v.get("velocity")) if (!get_vec3(*vel, b.velocity, err)) return false;
    return true;
}

bool parse_fluid(const JVal& v, FluidCfg& f, std::string& err) {
    static const char* const known[] = {"name", "bounds", "resolution", "fill", "particles_per_cell", "substeps",
                                        "flip", "gravity", "pressure_iterations", "surface_refine",
                                        "particle_radius", "warmup", "max_triangles", "materials"};
    if (v.kind != JVal::Obj) { err = "invalid type: " + unexpected(v) + ", expected struct Fluid"; return false; }
    if (!check_fields(v, known, 14, err)) return false;
    const JVal* name = v.get("name");
    if (!name) { err = "missing field `name`"; return false; }
    if (name->kind != JVal::Str) { err = "invalid type: " + unexpected(*name) + ", expected a string"; return false; }
    f.name = name->s;
    const JVal* bounds = v.get("bounds");
    if (!bounds) { err = "missing field `bounds`"; return false; }
    if (bounds->kind != JVal::Arr) { err = "invalid type: " + unexpected(*bounds) + ", expected an array of length 2"; return false; }
    if (bounds->arr.size() != 2) { err = "invalid length " + std::to_string(bounds->arr.size()) + ", expected an array of length 2"; return false; }
    if (!get_vec3(bounds->arr[0], f.bounds[0], err) || !get_vec3(bounds->arr[1], f.bounds[1], err)) return false;
    const JVal* fill = v.get("fill");
    if (!fill) { err = "missing field `fill`"; return false; }
    if (fill->kind != JVal::Arr) { err = "invalid type: " + unexpected(*fill) + ", expected a sequence"; return false; }
    f.fill.clear();
    for (auto& b : fill->arr) {
        pxf_fill_block blk;
        if (!parse_block(b, blk, err)) return false;
        f.fill.push_back(blk);
    }
    struct U { const char* k; uint32_t* dst; } us[] = {
        {"resolution", &f.resolution}, {"particles_per_cell", &f.particles_per_cell}, {"substeps", &f.substeps},
        {"pressure_iterations", &f.pressure_iterations}, {"surface_refine", &f.surface_refine},
        {"max_triangles", &f.max_triangles}};
    for (auto& u : us) if (const JVal* x = v.get(u.k)) if (!get_u32(*x, *u.dst, err)) return false;
    struct F { const char* k; float* dst; } fs[] = {{"flip", &f.flip}, {"particle_radius", &f.particle_radius}, {"warmup", &f.warmup}};
    for (auto& q : fs) if (const JVal* x = v.get(q.k)) if (!get_f32(*x, *q.dst, err)) return false;
    if (const JVal* g = v.get("gravity")) if (!get_vec3(*g, f.gravity, err)) return false;
    if (const JVal* m = v.get("materials"))
        if (m->kind != JVal::Arr) { err = "invalid type: " + unexpected(*m) + ", expected a sequence"; return false; }
    return true;
}

bool has_camera(const JVal* nodes) {
    if (!nodes || nodes->kind != JVal::Arr) return false;
    for (auto& n : nodes->arr) {
        if (n.kind != JVal::Obj) continue;
        const JVal* t = n.get("type");
        if (t && t->kind == JVal::Str && t->s == "camera") return true;
    }
    return false;
}

}  // namespace

void FluidCfg::from_desc(const pxf_fluid_desc& d) {
    name = d.name ? d.name : "";
    std::memcpy(bounds, d.bounds, sizeof(bounds));
    resolution = d.resolution;
    fill.assign(d.fill, d.fill + (d.fill ? d.fill_count : 0));
    particles_per_cell = d.particles_per_cell;
    substeps = d.substeps;
    flip = d.flip;
    std::memcpy(gravity, d.gravity, sizeof(gravity));
    pressure_iterations = d.pressure_iterations;
    surface_refine = d.surface_refine;
    particle_radius = d.particle_radius;
    warmup = d.warmup;
    max_triangles = d.max_triangles;
}

void FluidCfg::to_desc(pxf_fluid_desc& d) const {
    d.name = name.c_str();
    std::memcpy(d.bounds, bounds, sizeof(bounds));
    d.resolution = resolution;
    d.fill = fill.data();
    d.fill_count = uint32_t(fill.size());
    d.particles_per_cell = particles_per_cell;
    d.substeps = substeps;
    d.flip = flip;
    std::memcpy(d.gravity, gravity, sizeof(gravity));
    d.pressure_iterations = pressure_iterations;
    d.surface_refine = surface_refine;
    d.particle_radius = particle_radius;
    d.warmup = warmup;
    d.max_triangles = max_triangles;
}

// Vec3::round is round-half-away-from-zero (std::round); `as u32` saturates.
void fluid_grid(const float bounds[2][3], uint32_t resolution, uint32_t n[3], float& h) {
    float size[3];
    for (int a = 0; a < 3; a++) size[a] = bounds[1][a] - bounds[0][a];
    float mx = size[0];
    if (size[1] > mx) mx = size[1];
    if (size[2] > mx) mx = size[2];
    h = mx / float(resolution);
    for (int a = 0; a < 3; a++) {
        float v = std::round(size[a] / h);
        v = v > 4.0f ? v : 4.0f;   // Vec3::max(splat(4)); a NaN gives 4 like f32::max
        n[a] = v >= 4294967295.0f ? 0xffffffffu : uint32_t(v);
    }
}

bool validate_fluid(const FluidCfg& f, uint32_t i, bool lift, std::string& msg) {
    const std::string ctx = "fluids[" + std::to_string(i) + "] '" + f.name + "': ";
    for (int a = 0; a < 3; a++) {
        if (!(f.bounds[1][a] > f.bounds[0][a])) {
            msg = ctx + "bounds must be [min, max] with max > min on every axis";
            return false;
        }
    }
    const bool res_ok = lift ? f.resolution >= 16 : (f.resolution >= 16 && f.resolution <= 256);
    if (!res_ok || !(f.particles_per_cell >= 1 && f.particles_per_cell <= 64) || !(f.substeps >= 1 && f.substeps <= 64) ||
        !(f.surface_refine >= 1 && f.surface_refine <= 3) || !(f.flip >= 0.0f && f.flip <= 1.0f) ||
        f.pressure_iterations == 0) {
        msg = ctx + "resolution 16..256, particles_per_cell 1..64, substeps 1..64, surface_refine 1..3, flip 0..1";
        return false;
    }
    if (f.fill.empty()) {
        msg = ctx + "needs at least one `fill` block of liquid";
        return false;
    }
    for (auto& b : f.fill) {
        bool bad = false;
        for (int a = 0; a < 3; a++) {
            if (!(b.max[a] > b.min[a])) bad = true;
            if (b.min[a] < f.bounds[0][a] || b.max[a] > f.bounds[1][a]) bad = true;
        }
        if (bad) {
            msg = ctx + "each fill block must have max > min and lie inside `bounds`";
            return false;
        }
    }
    uint32_t n[3];
    float h;
    fluid_grid(f.bounds, f.resolution, n, h);
    const uint64_t cells = uint64_t(n[0]) * n[1] * n[2];
    if (!lift && cells > 16000000ull) {
        msg = ctx + "grid too large (lower resolution)";
        return false;
    }
    // Faces are indexed with 32-bit integers on the device.
    const uint64_t faces = uint64_t(n[0] + 1) * n[1] * n[2] + uint64_t(n[0]) * (n[1] + 1) * n[2] + uint64_t(n[0]) * n[1] * (n[2] + 1);
    if (faces >= 0xffffffffull) {
        msg = ctx + "grid too large (lower resolution)";
        return false;
    }
    return true;
}

bool parse_scene(const char* text, SceneFluids& out, std::string& msg) {
    if (!text) { msg = "invalid scene: null text"; return false; }
    Parser ps{text, text, std::string(), 0};
    JVal root;
    if (!ps.value(root)) { msg = "invalid scene: " + ps.err; return false; }
    ps.ws();
    if (*ps.p) { ps.fail("trailing characters"); msg = "invalid scene: " + ps.err; return false; }
    static const char* const known[] = {"version", "nodes", "world", "render", "animation", "programs",
                                        "simulations", "plate", "fluids"};
    std::string err;
    if (root.kind != JVal::Obj) { msg = "invalid scene: invalid type: " + unexpected(root) + ", expected struct Scene"; return false; }
    if (!check_fields(root, known, 9, err)) { msg = "invalid scene: " + err; return false; }
    const JVal* ver = root.get("version");
    if (!ver) { msg = "invalid scene: missing field `version`"; return false; }
    uint32_t version = 0;
    if (!get_u32(*ver, version, err)) { msg = "invalid scene: " + err; return false; }
    out.fluids.clear();
    out.seed = 0;
    out.fps = 24.0f;
    if (const JVal* r = root.get("render")) {
        if (r->kind != JVal::Obj) { msg = "invalid scene: invalid type: " + unexpected(*r) + ", expected struct RenderSettings"; return false; }
        static const char* const rk[] = {"resolution", "samples", "bounces", "exposure", "view", "seed", "fps",
                                         "motion_blur", "denoise", "transparent"};
        if (!check_fields(*r, rk, 10, err)) { msg = "invalid scene: " + err; return false; }
        if (const JVal* s = r->get("seed")) if (!get_u32(*s, out.seed, err)) { msg = "invalid scene: " + err; return false; }
        if (const JVal* f = r->get("fps")) if (!get_f32(*f, out.fps, err)) { msg = "invalid scene: " + err; return false; }
    }
    if (const JVal* fl = root.get("fluids")) {
        if (fl->kind != JVal::Arr) { msg = "invalid scene: invalid type: " + unexpected(*fl) + ", expected a sequence"; return false; }
        for (auto& fv : fl->arr) {
            FluidCfg f;
            if (!parse_fluid(fv, f, err)) { msg = "invalid scene: " + err; return false; }
            out.fluids.push_back(std::move(f));
        }
    }
    // Scene::validate (lib.rs:650-735), the checks that apply before and to fluids.
    if (version != 1) {
        msg = "scene version " + std::to_string(version) + " is not supported (expected 1)";
        return false;
    }
    if (!has_camera(root.get("nodes"))) {
        msg = "scene has no camera node; add {\"type\":\"camera\",\"translation\":[x,y,z],\"target\":[0,0,0]}";
        return false;
    }
    if (!(out.fps > 0.0f)) {
        msg = "render.fps must be > 0";
        return false;
    }
    for (size_t i = 0; i < out.fluids.size(); i++)
        if (!validate_fluid(out.fluids[i], uint32_t(i), false, msg)) return false;
    return true;
}

}  // namespace pxf
