// lt_json.cpp -- Lantern scene JSON + LMF loading for lt_scene_load_json.
//
// Follows Scene::ParseJSON (source/core/scene/scene.cpp:215-446) and AddLMF
// (:502-582) for the parts this library renders: background colour, the
// orbiting pinhole camera with the reference's defaults, lambert / mirror /
// ideal_specular_dielectric BSDFs with constant albedo, non_scattering and
// isotropic_scattering media (plus the henyey_greenstein extension), materials,
// and "lmf", "grid" and "geosphere" primitives with an optional row-major 4x4
// transform and emission.
// Numbers are read as double and narrowed to float, as nlohmann's get<float>()
// does. Unlike the reference, which prints and skips a primitive it cannot
// load, every problem here is returned as an error.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "lt_scene.h"

namespace lt {
namespace {

struct Json {
    enum Type { Null, Bool, Number, String, Array, Object } type = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Json> arr;
    std::vector<std::pair<std::string, Json>> obj;

    const Json *get(const char *key) const {
        if (type != Object) return nullptr;
        for (auto &kv : obj)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
};

struct Parser {
    const char *p, *end;
    std::string err;

    void ws() {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
    }
    bool fail(const char *m) {
        if (err.empty()) err = m;
        return false;
    }
    bool parse_string(std::string &out) {
        if (p >= end || *p != '"') return fail("expected string");
        ++p;
        while (p < end && *p != '"') {
            char ch = *p++;
            if (ch == '\\') {
                if (p >= end) return fail("bad escape");
                char e = *p++;
                switch (e) {
                    case 'n': out += '\n'; break;
                    case 't': out += '\t'; break;
                    case 'r': out += '\r'; break;
                    case 'b': out += '\b'; break;
                    case 'f': out += '\f'; break;
                    case 'u': {
                        if (end - p < 4) return fail("bad unicode escape");
                        unsigned cp = (unsigned)strtoul(std::string(p, p + 4).c_str(), nullptr, 16);
                        p += 4;
                        if (cp < 0x80) out += (char)cp;
                        else if (cp < 0x800) { out += (char)(0xC0 | (cp >> 6)); out += (char)(0x80 | (cp & 0x3F)); }
                        else { out += (char)(0xE0 | (cp >> 12)); out += (char)(0x80 | ((cp >> 6) & 0x3F)); out += (char)(0x80 | (cp & 0x3F)); }
                        break;
                    }
                    default: out += e;
                }
            } else {
                out += ch;
            }
        }
        if (p >= end) return fail("unterminated string");
        ++p;
        return true;
    }
    bool parse(Json &v, int depth = 0) {
        if (depth > 64) return fail("nesting too deep");
        ws();
        if (p >= end) return fail("unexpected end");
        char c = *p;
        if (c == '{') {
            ++p;
            v.type = Json::Object;
            ws();
            if (p < end && *p == '}') { ++p; return true; }
            for (;;) {
                ws();
                std::string k;
                if (!parse_string(k)) return false;
                ws();
                if (p >= end || *p != ':') return fail("expected ':'");
                ++p;
                v.obj.emplace_back(k, Json());
                if (!parse(v.obj.back().second, depth + 1)) return false;
                ws();
                if (p < end && *p == ',') { ++p; continue; }
                if (p < end && *p == '}') { ++p; return true; }
                return fail("expected ',' or '}'");
            }
        }
        if (c == '[') {
            ++p;
            v.type = Json::Array;
            ws();
            if (p < end && *p == ']') { ++p; return true; }
            for (;;) {
                v.arr.emplace_back();
                if (!parse(v.arr.back(), depth + 1)) return false;
                ws();
                if (p < end && *p == ',') { ++p; continue; }
                if (p < end && *p == ']') { ++p; return true; }
                return fail("expected ',' or ']'");
            }
        }
        if (c == '"') {
            v.type = Json::String;
            return parse_string(v.str);
        }
        if (!strncmp(p, "true", 4) && end - p >= 4) { p += 4; v.type = Json::Bool; v.b = true; return true; }
        if (!strncmp(p, "false", 5) && end - p >= 5) { p += 5; v.type = Json::Bool; v.b = false; return true; }
        if (!strncmp(p, "null", 4) && end - p >= 4) { p += 4; v.type = Json::Null; return true; }
        char *q = nullptr;
        std::string tok(p, std::min<size_t>((size_t)(end - p), 64));
        double d = strtod(tok.c_str(), &q);
        if (q == tok.c_str()) return fail("unexpected character");
        p += (q - tok.c_str());
        v.type = Json::Number;
        v.num = d;
        return true;
    }
};

bool read_file(const std::string &path, std::vector<char> &out) {
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) return false;
    fseek(f, 0, SEEK_END);
    long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    out.resize(n > 0 ? (size_t)n : 0);
    size_t got = n > 0 ? fread(out.data(), 1, (size_t)n, f) : 0;
    fclose(f);
    return got == out.size();
}

bool num(const Json *j, float *out) {
    if (!j || j->type != Json::Number) return false;
    *out = (float)j->num;
    return true;
}

bool float3(const Json *j, float out[3]) {
    if (!j || j->type != Json::Array || j->arr.size() != 3) return false;
    for (int i = 0; i < 3; ++i)
        if (!num(&j->arr[i], &out[i])) return false;
    return true;
}

// ReadLMF (io/lantern_model_file.cpp:33-65) with bounds checks
// CreateGrid (geometry_generator.cpp:515-566): m rows of n vertices in the xz
// plane, row i at z = -(depth/2 - i * dz), normals +y, two triangles per cell.
void make_grid(float width, float depth, uint32_t m, uint32_t n, std::vector<float> &pos, std::vector<float> &nrm,
               std::vector<float> &tex, std::vector<uint32_t> &idx) {
    const float half_w = 0.5f * width, half_d = 0.5f * depth;
    const float dx = width / (float)(n - 1), dz = depth / (float)(m - 1);
    const float du = 1.0f / (float)(n - 1), dv = 1.0f / (float)(m - 1);
    pos.resize(3 * (size_t)m * n);
    nrm.resize(3 * (size_t)m * n);
    tex.resize(2 * (size_t)m * n);
    for (uint32_t i = 0; i < m; ++i) {
        const float z = half_d - (float)i * dz;
        for (uint32_t j = 0; j < n; ++j) {
            const float x = -half_w + (float)j * dx;
            float *p = &pos[3 * ((size_t)i * n + j)], *q = &nrm[3 * ((size_t)i * n + j)];
            p[0] = x; p[1] = 0.0f; p[2] = -z;
            q[0] = 0.0f; q[1] = 1.0f; q[2] = 0.0f;
            tex[2 * ((size_t)i * n + j)] = (float)j * du;  // stretched over the grid
            tex[2 * ((size_t)i * n + j) + 1] = (float)i * dv;
        }
    }
    idx.clear();
    idx.reserve(6 * (size_t)(m - 1) * (n - 1));
    for (uint32_t i = 0; i + 1 < m; ++i)
        for (uint32_t j = 0; j + 1 < n; ++j) {
            const uint32_t a = i * n + j, b = (i + 1) * n + j;
            idx.insert(idx.end(), {a, a + 1, b, b, a + 1, b + 1});
        }
}

// CreateGeosphere (geometry_generator.cpp:306-356) with Subdivide (:214-283):
// the icosahedron below, each subdivision replacing every triangle by four with
// six fresh vertices (no sharing), then every vertex projected to the sphere:
// n = v * (1 / sqrt(dot(v, v))), position = radius * n, normal = n.
void make_geosphere(float radius, uint32_t subdivisions, std::vector<float> &pos, std::vector<float> &nrm,
                    std::vector<uint32_t> &idx) {
    const float X = 0.525731f, Z = 0.850651f;
    const float base[12][3] = {{-X, 0.0f, -Z}, {X, 0.0f, -Z}, {-X, 0.0f, Z}, {X, 0.0f, Z},
                               {0.0f, Z, -X},  {0.0f, Z, X},  {0.0f, -Z, -X}, {0.0f, -Z, X},
                               {Z, X, 0.0f},   {-Z, X, 0.0f}, {Z, -X, 0.0f},  {-Z, -X, 0.0f}};
    const uint32_t tri[60] = {1, 4, 0, 4, 9, 0, 4, 5, 9, 8, 5, 4, 1, 8, 4, 1, 10, 8, 10, 3, 8, 8, 3, 5, 3, 2, 5,
                              3, 7, 2, 3, 10, 7, 10, 6, 7, 6, 11, 7, 6, 0, 11, 6, 1, 0, 10, 1, 6, 11, 0, 9, 2, 11, 9,
                              5, 2, 9, 11, 2, 7};
    pos.assign(&base[0][0], &base[0][0] + 36);
    idx.assign(tri, tri + 60);
    for (uint32_t s = 0; s < subdivisions; ++s) {
        std::vector<float> p2;
        std::vector<uint32_t> i2;
        const size_t nt = idx.size() / 3;
        p2.reserve(18 * nt);
        i2.reserve(12 * nt);
        for (size_t t = 0; t < nt; ++t) {
            const float *v0 = &pos[3 * (size_t)idx[3 * t]], *v1 = &pos[3 * (size_t)idx[3 * t + 1]],
                        *v2 = &pos[3 * (size_t)idx[3 * t + 2]];
            float m0[3], m1[3], m2[3];
            for (int c = 0; c < 3; ++c) {
                m0[c] = 0.5f * (v0[c] + v1[c]);
                m1[c] = 0.5f * (v1[c] + v2[c]);
                m2[c] = 0.5f * (v0[c] + v2[c]);
            }
            const float *vs[6] = {v0, v1, v2, m0, m1, m2};
            for (const float *v : vs) p2.insert(p2.end(), v, v + 3);
            const uint32_t b = (uint32_t)(6 * t);
            i2.insert(i2.end(), {b, b + 3, b + 5, b + 3, b + 4, b + 5, b + 5, b + 4, b + 2, b + 3, b + 1, b + 4});
        }
        pos.swap(p2);
        idx.swap(i2);
    }
    const size_t nv = pos.size() / 3;
    nrm.resize(pos.size());
    for (size_t v = 0; v < nv; ++v) {
        float *p = &pos[3 * v];
        const float inv = 1.0f / sqrtf((p[0] * p[0] + p[1] * p[1]) + p[2] * p[2]);
        for (int c = 0; c < 3; ++c) {
            nrm[3 * v + c] = p[c] * inv;
            p[c] = radius * nrm[3 * v + c];
        }
    }
}

lt_status read_lmf(const std::string &path, uint8_t *vpp, std::vector<float> &pos, std::vector<uint32_t> &idx,
                   std::vector<float> &nrm, std::vector<float> &tex, std::string *err) {
    std::vector<char> buf;
    if (!read_file(path, buf)) {
        *err = "cannot read LMF file " + path;
        return LT_ERR_IO;
    }
    size_t off = 0;
    auto take = [&](void *dst, size_t n) -> bool {
        if (off + n > buf.size()) return false;
        memcpy(dst, buf.data() + off, n);
        off += n;
        return true;
    };
    uint32_t magic = 0, flags = 0;
    uint64_t n = 0;
    if (!take(&magic, 4) || magic != (uint32_t)('L' | ('M' << 8) | ('F' << 16))) {
        *err = path + ": not an LMF file";
        return LT_ERR_PARSE;
    }
    if (!take(vpp, 1) || !take(&flags, 4) || !take(&n, 8) || n > (buf.size() / 12)) {
        *err = path + ": truncated LMF header";
        return LT_ERR_PARSE;
    }
    pos.resize(n * 3);
    if (!take(pos.data(), n * 12)) { *err = path + ": truncated positions"; return LT_ERR_PARSE; }
    uint64_t ni = 0;
    if (!take(&ni, 8) || ni > buf.size() / 4) { *err = path + ": truncated index count"; return LT_ERR_PARSE; }
    idx.resize(ni);
    if (!take(idx.data(), ni * 4)) { *err = path + ": truncated indices"; return LT_ERR_PARSE; }
    nrm.clear();
    if (flags & 1u) {
        uint64_t nn = 0;
        if (!take(&nn, 8) || nn > buf.size() / 4) { *err = path + ": truncated normal count"; return LT_ERR_PARSE; }
        nrm.resize(nn);
        if (!take(nrm.data(), nn * 4)) { *err = path + ": truncated normals"; return LT_ERR_PARSE; }
    }
    tex.clear();
    if (flags & 2u) {
        uint64_t nt = 0;
        if (!take(&nt, 8) || nt > buf.size() / 4) { *err = path + ": truncated texcoord count"; return LT_ERR_PARSE; }
        tex.resize(nt);
        if (!take(tex.data(), nt * 4)) { *err = path + ": truncated texcoords"; return LT_ERR_PARSE; }
    }
    return LT_OK;
}

bool file_exists(const std::string &path) {
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) return false;
    fclose(f);
    return true;
}

}  // namespace

lt_status load_scene_json(const char *path, lt_scene_desc *desc, JsonSceneStorage *st, std::string *err) {
    std::vector<char> text;
    if (!read_file(path, text)) {
        *err = std::string("cannot read scene file ") + path;
        return LT_ERR_IO;
    }
    Parser ps{text.data(), text.data() + text.size(), ""};
    Json root;
    if (!ps.parse(root) || root.type != Json::Object) {
        *err = std::string("scene JSON parse error: ") + (ps.err.empty() ? "not an object" : ps.err);
        return LT_ERR_PARSE;
    }
    std::string dir(path);
    size_t slash = dir.find_last_of('/');
    dir = slash == std::string::npos ? std::string(".") : dir.substr(0, slash);

    memset(desc, 0, sizeof *desc);
    if (const Json *bg = root.get("background_color")) {
        if (!float3(bg, desc->background)) { *err = "background_color must be 3 numbers"; return LT_ERR_PARSE; }
    }
    const Json *cam = root.get("camera");
    if (!cam || cam->type != Json::Object) {
        *err = "JSON parse error: \"camera\" is required";
        return LT_ERR_PARSE;
    }
    lt_camera_desc &c = desc->camera;
    c.phi = 0.785398163397448309616f;   // (float)M_PI_4, scene.cpp:229
    c.theta = 0.0f;
    c.radius = 10.0f;
    c.fov = 0.785398163397448309616f;
    float w = 0, h = 0;
    if (!num(cam->get("client_width"), &w) || !num(cam->get("client_height"), &h) || w < 1 || h < 1) {
        *err = "camera client_width and client_height are required";
        return LT_ERR_PARSE;
    }
    c.width = (uint32_t)cam->get("client_width")->num;
    c.height = (uint32_t)cam->get("client_height")->num;
    num(cam->get("phi"), &c.phi);
    num(cam->get("theta"), &c.theta);
    num(cam->get("radius"), &c.radius);
    num(cam->get("fov"), &c.fov);
    if (const Json *t = cam->get("target")) float3(t, c.target);

    std::map<std::string, int> medium_ix, material_ix;
    std::map<std::string, uint32_t> image_ix;
    if (const Json *media = root.get("media")) {
        for (const Json &m : media->arr) {
            const Json *name = m.get("name"), *type = m.get("type");
            if (!name || !type) { *err = "medium needs name and type"; return LT_ERR_PARSE; }
            lt_medium_desc md;
            memset(&md, 0, sizeof md);
            if (type->str == "henyey_greenstein") {
                md.type = LT_MEDIUM_HG;
                if (!float3(m.get("sigma_a"), md.sigma_a) || !float3(m.get("sigma_s"), md.sigma_s)) {
                    *err = "henyey_greenstein medium needs sigma_a and sigma_s";
                    return LT_ERR_PARSE;
                }
                num(m.get("g"), &md.g);
            } else if (type->str == "non_scattering" || type->str == "isotropic_scattering") {
                // Medium ctor (medium.h:19-23): sigma_a = -log(color) / distance;
                // isotropic (isotropic_scattering_medium.h:22-25): sigma_s = 1 / distance
                float col[3], at = 1.0f, sd = 1.0f;
                if (!float3(m.get("absorption_color"), col) || !num(m.get("absorption_at_distance"), &at)) {
                    *err = "medium needs absorption_color and absorption_at_distance";
                    return LT_ERR_PARSE;
                }
                for (int k = 0; k < 3; ++k) md.sigma_a[k] = -logf(col[k]) / at;
                if (type->str == "isotropic_scattering") {
                    if (!num(m.get("scattering_distance"), &sd)) {
                        *err = "isotropic_scattering medium needs scattering_distance";
                        return LT_ERR_PARSE;
                    }
                    md.type = LT_MEDIUM_ISOTROPIC;
                    for (int k = 0; k < 3; ++k) md.sigma_s[k] = 1 / sd;
                } else {
                    md.type = LT_MEDIUM_NON_SCATTERING;
                }
            } else {
                continue;  // unknown medium types are ignored, as the reference does
            }
            medium_ix[name->str] = (int)st->media.size();
            st->media.push_back(md);
        }
    }
    std::map<std::string, const Json *> bsdfs;
    if (const Json *b = root.get("bsdfs"))
        for (const Json &x : b->arr)
            if (const Json *n = x.get("name")) bsdfs[n->str] = &x;
    if (const Json *mats = root.get("materials")) {
        for (const Json &m : mats->arr) {
            const Json *name = m.get("name"), *bn = m.get("bsdf");
            if (!name || !bn) { *err = "material needs name and bsdf"; return LT_ERR_PARSE; }
            auto it = bsdfs.find(bn->str);
            if (it == bsdfs.end()) continue;  // scene.cpp:346-349 skips it
            const Json &b = *it->second;
            lt_material_desc md;
            memset(&md, 0, sizeof md);
            md.medium = -1;
            const std::string type = b.get("type") ? b.get("type")->str : "";
            if (type == "lambert") md.bsdf = LT_BSDF_LAMBERT;
            else if (type == "mirror") md.bsdf = LT_BSDF_MIRROR;
            else if (type == "ideal_specular_dielectric") {
                md.bsdf = LT_BSDF_DIELECTRIC;
                if (!num(b.get("ior"), &md.ior)) { *err = "dielectric needs ior"; return LT_ERR_PARSE; }
            } else {
                *err = "unknown bsdf type " + type;
                return LT_ERR_PARSE;
            }
            // albedo texture (scene.cpp:266-318): constant, uv or image
            const Json *alb = b.get("albedo");
            const Json *at = alb ? alb->get("type") : nullptr;
            const std::string akind = at ? at->str : "";
            if (akind == "constant") {
                md.albedo_kind = LT_ALBEDO_CONSTANT;
                if (!float3(alb->get("value"), md.albedo)) { *err = "constant albedo needs value"; return LT_ERR_PARSE; }
            } else if (akind == "uv") {
                md.albedo_kind = LT_ALBEDO_UV;
            } else if (akind == "image") {
                const Json *ip = alb->get("file_path");
                if (!ip || ip->str.empty()) { *err = "image albedo needs file_path"; return LT_ERR_PARSE; }
                // as given (the reference's image cache opens it from the working
                // directory), else next to the scene file
                std::string ipath = ip->str;
                if (ipath[0] != '/' && !file_exists(ipath)) ipath = dir + "/" + ipath;
                auto found = image_ix.find(ipath);
                if (found == image_ix.end()) {
                    lt_image_desc id;
                    std::vector<uint8_t> texels;
                    lt_status rs = load_png(ipath, &texels, &id.width, &id.height, &id.channels, err);
                    if (rs != LT_OK) return rs;
                    st->bytes.push_back(std::move(texels));
                    id.texels = st->bytes.back().data();
                    found = image_ix.emplace(ipath, (uint32_t)st->images.size()).first;
                    st->images.push_back(id);
                }
                md.albedo_kind = LT_ALBEDO_IMAGE;
                md.image = found->second;
            } else {
                *err = "bsdf " + bn->str + ": unknown albedo type " + akind;
                return LT_ERR_UNSUPPORTED;
            }
            if (const Json *mn = m.get("medium")) {
                auto mi = medium_ix.find(mn->str);
                if (mi == medium_ix.end()) continue;  // scene.cpp:354-357 skips it
                md.medium = mi->second;
            }
            material_ix[name->str] = (int)st->materials.size();
            st->materials.push_back(md);
        }
    }
    if (const Json *prims = root.get("primitives")) {
        for (const Json &p : prims->arr) {
            const Json *type = p.get("type");
            const std::string pname = p.get("name") ? p.get("name")->str : "";
            std::vector<float> pos, nrm, tex;
            std::vector<uint32_t> idx;
            if (type && type->str == "lmf") {
                const Json *fp = p.get("file_path");
                if (!fp) { *err = "lmf primitive needs file_path"; return LT_ERR_PARSE; }
                std::string file = fp->str;
                if (file.empty() || file[0] != '/') file = dir + "/" + file;
                uint8_t vpp = 0;
                lt_status rs = read_lmf(file, &vpp, pos, idx, nrm, tex, err);
                if (rs != LT_OK) return rs;
                if (vpp != 3) {
                    *err = file + ": only triangle LMF files are supported";
                    return LT_ERR_UNSUPPORTED;
                }
            } else if (type && type->str == "grid") {
                float width = 0.0f, depth = 0.0f, n = 0.0f, m = 0.0f;
                if (!num(p.get("width"), &width) || !num(p.get("depth"), &depth) || !num(p.get("n"), &n) ||
                    !num(p.get("m"), &m)) {
                    *err = "grid primitive " + pname + " needs width, depth, n, m";
                    return LT_ERR_PARSE;
                }
                if (n < 2.0f || m < 2.0f || n > 65536.0f || m > 65536.0f) {
                    *err = "grid primitive " + pname + ": n and m must be 2..65536";
                    return LT_ERR_INVALID;
                }
                make_grid(width, depth, (uint32_t)m, (uint32_t)n, pos, nrm, tex, idx);
            } else if (type && type->str == "geosphere") {
                float radius = 0.0f, n = 0.0f;
                if (!num(p.get("radius"), &radius) || !num(p.get("n"), &n)) {
                    *err = "geosphere primitive " + pname + " needs radius and n";
                    return LT_ERR_PARSE;
                }
                if (n < 0.0f || n > 10.0f) {
                    *err = "geosphere primitive " + pname + ": n (subdivisions) must be 0..10";
                    return LT_ERR_INVALID;
                }
                make_geosphere(radius, (uint32_t)n, pos, nrm, idx);
            } else {
                *err = "primitive " + pname + ": unknown type (lmf, grid and geosphere are supported)";
                return LT_ERR_UNSUPPORTED;
            }
            const size_t nv = pos.size() / 3;
            std::vector<float> xform;
            if (const Json *t = p.get("transform")) {  // applied by lt_scene_create (transform_points)
                if (t->type != Json::Array || t->arr.size() != 16) { *err = "transform needs 16 numbers"; return LT_ERR_PARSE; }
                xform.resize(16);
                for (int k = 0; k < 16; ++k)
                    if (!num(&t->arr[k], &xform[k])) { *err = "transform needs 16 numbers"; return LT_ERR_PARSE; }
            }
            const Json *mn = p.get("material");
            auto mi = mn ? material_ix.find(mn->str) : material_ix.end();
            if (mi == material_ix.end()) {
                *err = "primitive " + pname + ": unknown material";
                return LT_ERR_PARSE;
            }
            lt_mesh_desc md;
            memset(&md, 0, sizeof md);
            md.num_vertices = (uint32_t)nv;
            md.num_triangles = (uint32_t)(idx.size() / 3);
            md.material = mi->second;
            if (const Json *em = p.get("emission")) {
                md.emissive = 1;
                if (!float3(em->get("color"), md.emission_color) || !num(em->get("radiant_power"), &md.radiant_power)) {
                    *err = "emission needs color and radiant_power";
                    return LT_ERR_PARSE;
                }
            }
            st->floats.push_back(std::move(pos));
            md.positions = st->floats.back().data();
            if (nrm.size() == nv * 3 && nv) {
                st->floats.push_back(std::move(nrm));
                md.normals = st->floats.back().data();
            }
            if (tex.size() == nv * 2 && nv) {
                st->floats.push_back(std::move(tex));
                md.texcoords = st->floats.back().data();
            }
            if (!xform.empty()) {
                st->floats.push_back(std::move(xform));
                md.transform = st->floats.back().data();
            }
            st->uints.push_back(std::move(idx));
            md.indices = st->uints.back().data();
            st->meshes.push_back(md);
        }
    }
    desc->materials = st->materials.data();
    desc->num_materials = (uint32_t)st->materials.size();
    desc->media = st->media.data();
    desc->num_media = (uint32_t)st->media.size();
    desc->meshes = st->meshes.data();
    desc->num_meshes = (uint32_t)st->meshes.size();
    desc->images = st->images.data();
    desc->num_images = (uint32_t)st->images.size();
    return LT_OK;
}

}  // namespace lt
