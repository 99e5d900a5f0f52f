// lt_scene.cpp -- scene description -> flat host arrays, light setup and the
// binned-SAH BVH2 that the traversal kernels read.
#include "lt_scene.h"

#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>

namespace lt {

// transform * float3a(p, 1) (scene.cpp:456-461, 517-522; linearspace4.h:43-47,165):
// row r = ((x*m[4r] + y*m[4r+1]) + z*m[4r+2]) + 1*m[4r+3].
void transform_points(const float *m, const float *in, uint32_t n, float *out) {
    for (uint32_t v = 0; v < n; ++v) {
        const float x = in[3 * (size_t)v], y = in[3 * (size_t)v + 1], z = in[3 * (size_t)v + 2];
        for (int r = 0; r < 3; ++r)
            out[3 * (size_t)v + r] = ((x * m[4 * r] + y * m[4 * r + 1]) + z * m[4 * r + 2]) + 1.0f * m[4 * r + 3];
    }
}

lt_status build_host_scene(const lt_scene_desc *d, HostScene *s, std::string *err, bool host_setup) {
    const lt_camera_desc &cd = d->camera;
    if (cd.width == 0 || cd.height == 0) {
        *err = "camera width and height must be positive";
        return LT_ERR_INVALID;
    }
    s->camera = make_camera(cd.phi, cd.theta, cd.radius, cd.width, cd.height, ld3(cd.target), cd.fov);
    s->filter = make_tent_filter();
    s->background = ld3(d->background);

    s->media.clear();
    for (uint32_t i = 0; i < d->num_media; ++i) {
        const lt_medium_desc &m = d->media[i];
        if (m.type < LT_MEDIUM_NON_SCATTERING || m.type > LT_MEDIUM_HG) {
            *err = "unknown medium type";
            return LT_ERR_INVALID;
        }
        MediumInfo mi;
        memset(&mi, 0, sizeof mi);
        mi.type = m.type;
        mi.g = m.g;
        for (int c = 0; c < 3; ++c) { mi.sigma_a[c] = m.sigma_a[c]; mi.sigma_s[c] = m.sigma_s[c]; }
        mi.sigma_s_mean = (m.sigma_s[0] + m.sigma_s[1] + m.sigma_s[2]) / 3.0f;
        s->media.push_back(mi);
    }
    s->materials.clear();
    for (uint32_t i = 0; i < d->num_materials; ++i) {
        const lt_material_desc &m = d->materials[i];
        if (m.bsdf < LT_BSDF_LAMBERT || m.bsdf > LT_BSDF_DIELECTRIC) {
            *err = "unknown bsdf type";
            return LT_ERR_INVALID;
        }
        if (m.medium < -1 || m.medium >= (int32_t)d->num_media) {
            *err = "material medium index out of range";
            return LT_ERR_INVALID;
        }
        MaterialInfo mi;
        memset(&mi, 0, sizeof mi);
        mi.bsdf = m.bsdf;
        mi.medium = m.medium;
        mi.ior = m.ior;
        for (int c = 0; c < 3; ++c) mi.albedo[c] = m.albedo[c];
        if (m.albedo_kind == LT_ALBEDO_CONSTANT) {
            mi.tex = kAlbedoConstant;
        } else if (m.albedo_kind == LT_ALBEDO_UV) {
            mi.tex = kAlbedoUV;
        } else if (m.albedo_kind == LT_ALBEDO_IMAGE) {
            if (m.image >= d->num_images) {
                *err = "material image index out of range";
                return LT_ERR_INVALID;
            }
            mi.tex = (int32_t)m.image;
        } else {
            *err = "unknown albedo kind";
            return LT_ERR_INVALID;
        }
        s->materials.push_back(mi);
    }
    s->images.clear();
    s->texels.clear();
    for (uint32_t i = 0; i < d->num_images; ++i) {
        const lt_image_desc &im = d->images[i];
        if (!im.texels || im.width == 0 || im.height == 0 || im.channels < 1 || im.channels > 4 ||
            im.width > 65536 || im.height > 65536) {
            *err = "image " + std::to_string(i) + ": texels, size or channel count invalid";
            return LT_ERR_INVALID;
        }
        ImageInfo ii;
        memset(&ii, 0, sizeof ii);
        ii.offset = s->texels.size();
        ii.width = im.width;
        ii.height = im.height;
        ii.channels = im.channels;
        s->texels.insert(s->texels.end(), im.texels, im.texels + (size_t)im.width * im.height * im.channels);
        s->images.push_back(ii);
    }

    size_t ntri = 0, nvert = 0;
    for (uint32_t g = 0; g < d->num_meshes; ++g) {
        ntri += d->meshes[g].num_triangles;
        nvert += d->meshes[g].num_vertices;
    }
    if (ntri >= (1u << (31 - kLeafBits)) || nvert >= 0xFFFFFFFFu) {
        *err = "scene too large: at most 2^28 triangles";
        return LT_ERR_INVALID;
    }
    s->geoms.clear();
    s->lights.clear();
    s->light_tris.clear();
    s->light_src.clear();
    s->tri_geom.assign(ntri, 0);
    if (host_setup) {
        s->tri_v0e1e2.assign(ntri * 9, 0.0f);
        s->tri_vidx.assign(ntri * 3, 0);
        s->vnormal.assign(nvert * 3, 0.0f);
        s->vtex.assign(nvert * 2, 0.0f);
    } else {  // the device builds these (lt_setup.cu)
        s->tri_v0e1e2.clear();
        s->tri_vidx.clear();
        s->vnormal.clear();
        s->vtex.clear();
    }
    size_t t0 = 0, vbase = 0;
    uint32_t light_tri_count = 0;
    std::vector<float> moved;
    for (uint32_t g = 0; g < d->num_meshes; ++g) {
        const lt_mesh_desc &m = d->meshes[g];
        if (m.material < 0 || m.material >= (int32_t)d->num_materials) {
            *err = "mesh material index out of range";
            return LT_ERR_INVALID;
        }
        if ((m.num_triangles && (!m.indices || !m.positions)) || (m.num_vertices && !m.positions)) {
            *err = "mesh arrays missing";
            return LT_ERR_INVALID;
        }
        for (size_t k = 0; k < 3 * (size_t)m.num_triangles; ++k)
            if (m.indices[k] >= m.num_vertices) {
                *err = "triangle index out of range in mesh " + std::to_string(g);
                return LT_ERR_INVALID;
            }
        GeomInfo gi;
        gi.material = m.material;
        gi.light = -1;
        gi.has_normals = m.normals != nullptr;
        gi.has_texcoords = m.texcoords != nullptr;
        gi.first_tri = (uint32_t)t0;
        for (uint32_t t = 0; t < m.num_triangles; ++t) s->tri_geom[t0 + t] = g;
        // world-space positions on the host: every mesh for a host setup, else
        // only the lights' (area, bounding sphere, light triangles)
        const float *pos = m.positions;
        if (m.transform && host_setup) {
            moved.resize(3 * (size_t)m.num_vertices);
            transform_points(m.transform, m.positions, m.num_vertices, moved.data());
            pos = moved.data();
        }
        if (host_setup) {
            for (uint32_t t = 0; t < m.num_triangles; ++t) {
                uint32_t i0 = m.indices[3 * t], i1 = m.indices[3 * t + 1], i2 = m.indices[3 * t + 2];
                v3 a = ld3(pos + 3 * (size_t)i0), b = ld3(pos + 3 * (size_t)i1), c = ld3(pos + 3 * (size_t)i2);
                float *dst = &s->tri_v0e1e2[9 * (t0 + t)];
                v3 e1 = a - b, e2 = c - a;
                dst[0] = a.x; dst[1] = a.y; dst[2] = a.z;
                dst[3] = e1.x; dst[4] = e1.y; dst[5] = e1.z;
                dst[6] = e2.x; dst[7] = e2.y; dst[8] = e2.z;
                s->tri_vidx[3 * (t0 + t)] = (uint32_t)(vbase + i0);
                s->tri_vidx[3 * (t0 + t) + 1] = (uint32_t)(vbase + i1);
                s->tri_vidx[3 * (t0 + t) + 2] = (uint32_t)(vbase + i2);
            }
            if (m.normals)
                memcpy(&s->vnormal[3 * vbase], m.normals, (size_t)m.num_vertices * 3 * sizeof(float));
            if (m.texcoords)
                memcpy(&s->vtex[2 * vbase], m.texcoords, (size_t)m.num_vertices * 2 * sizeof(float));
        }
        if (m.emissive) {
            LightInfo li;
            memset(&li, 0, sizeof li);
            li.geom = (int32_t)g;
            li.tri_first = light_tri_count;
            li.tri_count = m.num_triangles;
            light_tri_count += m.num_triangles;
            if (host_setup) {
                for (uint32_t t = 0; t < m.num_triangles; ++t) {
                    uint32_t i0 = m.indices[3 * t], i1 = m.indices[3 * t + 1], i2 = m.indices[3 * t + 2];
                    v3 a = ld3(pos + 3 * (size_t)i0), b = ld3(pos + 3 * (size_t)i1), c = ld3(pos + 3 * (size_t)i2);
                    v3 e1 = a - b, e2 = c - a;
                    const float row[12] = {a.x, a.y, a.z, bits_to_float((uint32_t)(t0 + t)),
                                           e1.x, e1.y, e1.z, 0.0f, e2.x, e2.y, e2.z, 0.0f};
                    s->light_tris.insert(s->light_tris.end(), row, row + 12);
                }
                li.area = light_area(pos, m.indices, m.num_triangles);
                if (m.num_vertices) light_bounding_sphere(pos, m.num_vertices, li.sphere);
                const v3 rad = light_radiance(m.emission_color, m.radiant_power, li.area);
                li.radiance[0] = rad.x; li.radiance[1] = rad.y; li.radiance[2] = rad.z;
            } else {
                LightSource src;
                memset(&src, 0, sizeof src);
                src.geom = g;
                src.vbase = (uint32_t)vbase;
                src.tbase = (uint32_t)t0;
                src.nverts = m.num_vertices;
                src.ntris = m.num_triangles;
                src.tri_first = li.tri_first;
                memcpy(src.color, m.emission_color, sizeof src.color);
                src.power = m.radiant_power;
                s->light_src.push_back(src);
            }
            gi.light = (int32_t)s->lights.size();
            s->lights.push_back(li);
        }
        s->geoms.push_back(gi);
        t0 += m.num_triangles;
        vbase += m.num_vertices;
    }
    return LT_OK;
}

// ------------------------------------------------------------------ BVH build
namespace {

struct Box {
    float lo[3], hi[3];
    void reset() {
        for (int c = 0; c < 3; ++c) {
            lo[c] = std::numeric_limits<float>::infinity();
            hi[c] = -std::numeric_limits<float>::infinity();
        }
    }
    void grow(const Box &o) {
        for (int c = 0; c < 3; ++c) {
            lo[c] = fminf(lo[c], o.lo[c]);
            hi[c] = fmaxf(hi[c], o.hi[c]);
        }
    }
    void grow(const float *p) {
        for (int c = 0; c < 3; ++c) {
            lo[c] = fminf(lo[c], p[c]);
            hi[c] = fmaxf(hi[c], p[c]);
        }
    }
    float area() const {
        float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        if (!(dx >= 0.0f)) return 0.0f;
        return 2.0f * (dx * dy + dy * dz + dz * dx);
    }
};

struct TNode {
    Box box;
    int32_t left, right;  // -1 for a leaf
    uint32_t first, count;
};

constexpr int kBins = 32;
constexpr uint32_t kLeafMax = 4;

}  // namespace

void build_bvh(HostScene *s) {
    auto t_start = std::chrono::steady_clock::now();
    const size_t n = s->tri_geom.size();
    std::vector<Box> tb(n);
    std::vector<float> cen(3 * n);
    std::vector<uint32_t> idx(n);
    for (size_t t = 0; t < n; ++t) {
        const float *d = &s->tri_v0e1e2[9 * t];
        float p[3][3];
        for (int c = 0; c < 3; ++c) {
            p[0][c] = d[c];
            p[1][c] = d[c] - d[3 + c];
            p[2][c] = d[c] + d[6 + c];
        }
        tb[t].reset();
        for (int k = 0; k < 3; ++k) tb[t].grow(p[k]);
        for (int c = 0; c < 3; ++c) cen[3 * t + c] = 0.5f * (tb[t].lo[c] + tb[t].hi[c]);
        idx[t] = (uint32_t)t;
    }

    std::vector<TNode> tn;
    tn.reserve(n ? 2 * n / kLeafMax + 16 : 1);
    struct Task { uint32_t node, begin, end, depth; };
    std::vector<Task> stack;
    tn.push_back(TNode());
    stack.push_back({0, 0, (uint32_t)n, 0});
    uint32_t max_depth = 0;
    while (!stack.empty()) {
        Task task = stack.back();
        stack.pop_back();
        Box nb, cb;
        nb.reset();
        cb.reset();
        for (uint32_t i = task.begin; i < task.end; ++i) {
            nb.grow(tb[idx[i]]);
            cb.grow(&cen[3 * (size_t)idx[i]]);
        }
        TNode &node = tn[task.node];
        node.box = nb;
        if (task.depth > max_depth) max_depth = task.depth;
        uint32_t count = task.end - task.begin;
        if (count <= kLeafMax) {
            node.left = node.right = -1;
            node.first = task.begin;
            node.count = count;
            continue;
        }
        int best_axis = -1, best_bin = -1;
        float best_cost = std::numeric_limits<float>::infinity();
        Box bins[3][kBins];
        uint32_t bcnt[3][kBins];
        float scale[3];
        for (int ax = 0; ax < 3; ++ax) {
            float ext = cb.hi[ax] - cb.lo[ax];
            scale[ax] = ext > 0.0f ? (float)kBins / ext : 0.0f;
            for (int b = 0; b < kBins; ++b) { bins[ax][b].reset(); bcnt[ax][b] = 0; }
        }
        for (uint32_t i = task.begin; i < task.end; ++i) {
            uint32_t t = idx[i];
            for (int ax = 0; ax < 3; ++ax) {
                if (scale[ax] == 0.0f) continue;
                int b = (int)((cen[3 * (size_t)t + ax] - cb.lo[ax]) * scale[ax]);
                b = b < 0 ? 0 : (b >= kBins ? kBins - 1 : b);
                bins[ax][b].grow(tb[t]);
                bcnt[ax][b]++;
            }
        }
        for (int ax = 0; ax < 3; ++ax) {
            if (scale[ax] == 0.0f) continue;
            float rarea[kBins];
            uint32_t rc[kBins];
            Box acc;
            acc.reset();
            uint32_t c = 0;
            for (int b = kBins - 1; b > 0; --b) {
                acc.grow(bins[ax][b]);
                c += bcnt[ax][b];
                rarea[b] = acc.area();
                rc[b] = c;
            }
            acc.reset();
            c = 0;
            for (int b = 0; b < kBins - 1; ++b) {
                acc.grow(bins[ax][b]);
                c += bcnt[ax][b];
                if (c == 0 || rc[b + 1] == 0) continue;
                float cost = acc.area() * (float)c + rarea[b + 1] * (float)rc[b + 1];
                if (cost < best_cost) { best_cost = cost; best_axis = ax; best_bin = b; }
            }
        }
        uint32_t mid;
        if (best_axis < 0) {
            mid = task.begin + count / 2;
        } else {
            uint32_t i = task.begin, j = task.end;
            while (i < j) {
                uint32_t t = idx[i];
                int b = (int)((cen[3 * (size_t)t + best_axis] - cb.lo[best_axis]) * scale[best_axis]);
                b = b < 0 ? 0 : (b >= kBins ? kBins - 1 : b);
                if (b <= best_bin) ++i;
                else std::swap(idx[i], idx[--j]);
            }
            mid = i;
            if (mid == task.begin || mid == task.end) mid = task.begin + count / 2;
        }
        int32_t l = (int32_t)tn.size();
        tn.push_back(TNode());
        tn.push_back(TNode());
        tn[task.node].left = l;
        tn[task.node].right = l + 1;
        tn[task.node].first = tn[task.node].count = 0;
        stack.push_back({(uint32_t)l + 1, mid, task.end, task.depth + 1});
        stack.push_back({(uint32_t)l, task.begin, mid, task.depth + 1});
    }

    // device layout: inner nodes only, depth-first, each holding both child boxes
    s->nodes.clear();
    s->nodes.reserve(tn.size() / 2 + 1);
    auto child_ref = [&](int32_t c, int32_t assigned) -> int32_t {
        return tn[c].left < 0 ? leaf_ref(tn[c].first, tn[c].count) : assigned;
    };
    auto set_box = [&](BvhNode &g, int k, const Box &b) {
        if (k == 0) {
            g.a[0] = b.lo[0]; g.a[1] = b.hi[0]; g.a[2] = b.lo[1]; g.a[3] = b.hi[1];
            g.c[0] = b.lo[2]; g.c[1] = b.hi[2];
        } else {
            g.b[0] = b.lo[0]; g.b[1] = b.hi[0]; g.b[2] = b.lo[1]; g.b[3] = b.hi[1];
            g.c[2] = b.lo[2]; g.c[3] = b.hi[2];
        }
    };
    if (tn[0].left < 0) {
        BvhNode g;
        memset(&g, 0, sizeof g);
        set_box(g, 0, tn[0].box);
        set_box(g, 1, tn[0].box);
        g.ref[0] = leaf_ref(tn[0].first, tn[0].count);
        g.ref[1] = leaf_ref(0, 0);
        g.count[0] = tn[0].count;
        g.count[1] = 0;
        s->nodes.push_back(g);
    } else {
        struct Item { int32_t tnode; uint32_t slot; };
        std::vector<Item> st;
        s->nodes.push_back(BvhNode());
        st.push_back({0, 0});
        while (!st.empty()) {
            Item it = st.back();
            st.pop_back();
            const TNode &t = tn[it.tnode];
            BvhNode g;
            memset(&g, 0, sizeof g);
            int32_t kids[2] = {t.left, t.right};
            uint32_t slots[2] = {0, 0};
            for (int k = 0; k < 2; ++k) {
                const TNode &c = tn[kids[k]];
                set_box(g, k, c.box);
                if (c.left >= 0) {
                    slots[k] = (uint32_t)s->nodes.size();
                    s->nodes.push_back(BvhNode());
                }
                g.ref[k] = child_ref(kids[k], (int32_t)slots[k]);
                g.count[k] = c.left < 0 ? c.count : 0;
            }
            s->nodes[it.slot] = g;
            for (int k = 1; k >= 0; --k)
                if (tn[kids[k]].left >= 0) st.push_back({kids[k], slots[k]});
        }
    }

    s->leaf_tris.assign(12 * n, 0.0f);
    for (size_t k = 0; k < n; ++k) {
        const float *d = &s->tri_v0e1e2[9 * (size_t)idx[k]];
        float *o = &s->leaf_tris[12 * k];
        o[0] = d[0]; o[1] = d[1]; o[2] = d[2]; o[3] = bits_to_float(idx[k]);
        o[4] = d[3]; o[5] = d[4]; o[6] = d[5]; o[7] = 0.0f;
        o[8] = d[6]; o[9] = d[7]; o[10] = d[8]; o[11] = 0.0f;
    }
    s->max_depth = max_depth;
    s->build_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t_start).count();
}

}  // namespace lt
