// lt_bvh8.cpp -- collapse of the binned-SAH BVH2 into compressed 8-wide nodes
// (layout in lt_scene.h). Host code; the scene's BVH2 is built first (on the
// GPU or the host) and read back.
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "lt_scene.h"

namespace lt {

namespace {

// A BVH2 child: inner node index (ref >= 0) or leaf (first, count), with its box.
struct Item {
    int32_t ref;
    uint32_t first, count;
    float lo[3], hi[3];
    bool inner() const { return ref >= 0; }
    uint32_t slots() const { return inner() ? 1u : (count + 2u) / 3u; }
    float area() const {
        float d[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
        return 2.0f * (d[0] * d[1] + d[1] * d[2] + d[2] * d[0]);
    }
};

Item child_item(const BvhNode &n, int k) {
    Item it;
    it.ref = n.ref[k];
    if (it.ref < 0) {
        uint32_t code = ~(uint32_t)it.ref;
        it.first = code >> kLeafBits;
        it.count = code & ((1u << kLeafBits) - 1u);
    } else {
        it.first = it.count = 0;
    }
    const float *xy = k == 0 ? n.a : n.b;
    it.lo[0] = xy[0]; it.hi[0] = xy[1];
    it.lo[1] = xy[2]; it.hi[1] = xy[3];
    it.lo[2] = n.c[2 * k]; it.hi[2] = n.c[2 * k + 1];
    return it;
}

// Smallest biased exponent E (cell 2^(E-127)) with p + 255 * cell >= hi in float.
uint8_t grid_exponent(float lo, float hi) {
    float ext = hi - lo;
    int e = -126;
    if (ext > 0.0f) {
        int ex = 0;
        std::frexp(ext / 255.0f, &ex);  // ext/255 = m * 2^ex, m in [0.5, 1)
        e = std::max(ex, -126);
    }
    while (e < 127 && lo + 255.0f * std::ldexp(1.0f, e) < hi) ++e;
    return (uint8_t)(e + 127);
}

// Quantises [clo, chi] on the grid (p, cell) outward; the traversal
// dequantises with the same float expression p + q * cell.
void quantise(float p, float cell, float clo, float chi, uint8_t *qlo, uint8_t *qhi) {
    float fl = std::floor((clo - p) / cell), fh = std::ceil((chi - p) / cell);
    int a = (int)std::min(std::max(fl, 0.0f), 255.0f), b = (int)std::min(std::max(fh, 0.0f), 255.0f);
    while (a > 0 && p + (float)a * cell > clo) --a;
    while (b < 255 && p + (float)b * cell < chi) ++b;
    *qlo = (uint8_t)a;
    *qhi = (uint8_t)b;
}

}  // namespace

uint32_t build_bvh8(const std::vector<BvhNode> &nodes, const std::vector<float> &leaf_tris,
                    std::vector<Bvh8Node> *out, std::vector<float> *tris8) {
    out->clear();
    tris8->clear();
    out->reserve(nodes.size() / 3 + 1);
    tris8->reserve(leaf_tris.size());
    struct Task { uint32_t wide, node, depth; };
    std::vector<Task> stack;
    out->push_back(Bvh8Node());
    stack.push_back({0, 0, 1});
    uint32_t max_depth = 0;
    while (!stack.empty()) {
        const Task task = stack.back();
        stack.pop_back();
        max_depth = std::max(max_depth, task.depth);
        // children of the BVH2 node, opened largest-area-first while they fit
        std::vector<Item> items;
        for (int k = 0; k < 2; ++k) {
            Item it = child_item(nodes[task.node], k);
            if (it.inner() || it.count > 0) items.push_back(it);
        }
        for (;;) {
            uint32_t used = 0;
            for (const Item &it : items) used += it.slots();
            int best = -1;
            float best_area = -1.0f;
            for (size_t i = 0; i < items.size(); ++i) {
                if (!items[i].inner()) continue;
                const BvhNode &n = nodes[items[i].ref];
                uint32_t add = 0;
                for (int k = 0; k < 2; ++k) {
                    Item c = child_item(n, k);
                    if (c.inner() || c.count > 0) add += c.slots();
                }
                if (used - 1 + add > 8) continue;
                if (items[i].area() > best_area) {
                    best_area = items[i].area();
                    best = (int)i;
                }
            }
            if (best < 0) break;
            const BvhNode &n = nodes[items[best].ref];
            items.erase(items.begin() + best);
            for (int k = 0; k < 2; ++k) {
                Item c = child_item(n, k);
                if (c.inner() || c.count > 0) items.push_back(c);
            }
        }
        // one entry per slot: leaves of more than 3 triangles split (same box)
        std::vector<Item> ent;
        for (const Item &it : items) {
            if (it.inner()) {
                ent.push_back(it);
                continue;
            }
            for (uint32_t f = 0; f < it.count; f += 3) {
                Item part = it;
                part.first = it.first + f;
                part.count = std::min(3u, it.count - f);
                ent.push_back(part);
            }
        }
        // parent box and octant placement
        float plo[3] = {INFINITY, INFINITY, INFINITY}, phi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (const Item &it : ent)
            for (int c = 0; c < 3; ++c) {
                plo[c] = std::min(plo[c], it.lo[c]);
                phi[c] = std::max(phi[c], it.hi[c]);
            }
        float pc[3] = {0.5f * (plo[0] + phi[0]), 0.5f * (plo[1] + phi[1]), 0.5f * (plo[2] + phi[2])};
        struct Cand { float score; int e, s; };
        std::vector<Cand> cand;
        for (size_t i = 0; i < ent.size(); ++i)
            for (int s = 0; s < 8; ++s) {
                float sc = 0.0f;
                for (int c = 0; c < 3; ++c) {
                    float d = 0.5f * (ent[i].lo[c] + ent[i].hi[c]) - pc[c];
                    sc += (s >> c & 1) ? -d : d;
                }
                cand.push_back({sc, (int)i, s});
            }
        std::stable_sort(cand.begin(), cand.end(), [](const Cand &x, const Cand &y) { return x.score > y.score; });
        int slot_of[8];
        int ent_in[8];
        for (int s = 0; s < 8; ++s) ent_in[s] = -1;
        for (size_t i = 0; i < ent.size(); ++i) slot_of[i] = -1;
        for (const Cand &c : cand)
            if (slot_of[c.e] < 0 && ent_in[c.s] < 0) {
                slot_of[c.e] = c.s;
                ent_in[c.s] = c.e;
            }
        // the wide node
        Bvh8Node w;
        memset(&w, 0, sizeof w);
        float cell[3];
        for (int c = 0; c < 3; ++c) {
            w.p[c] = plo[c];
            w.e[c] = grid_exponent(plo[c], phi[c]);
            uint32_t bits = (uint32_t)w.e[c] << 23;
            memcpy(&cell[c], &bits, 4);
        }
        w.base_child = (uint32_t)out->size();
        w.base_tri = (uint32_t)(tris8->size() / 12);
        std::vector<Task> kids;
        uint32_t tri_off = 0;
        for (int s = 0; s < 8; ++s) {
            const int i = ent_in[s];
            if (i < 0) continue;
            const Item &it = ent[i];
            for (int c = 0; c < 3; ++c) quantise(w.p[c], cell[c], it.lo[c], it.hi[c], &w.qlo[c][s], &w.qhi[c][s]);
            if (it.inner()) {
                w.imask |= (uint8_t)(1u << s);
                w.meta[s] = (uint8_t)((1u << 5) | (24u + (uint32_t)s));
                kids.push_back({(uint32_t)out->size(), (uint32_t)it.ref, task.depth + 1});
                out->push_back(Bvh8Node());
            } else {
                w.meta[s] = (uint8_t)((((1u << it.count) - 1u) << 5) | tri_off);
                tris8->insert(tris8->end(), leaf_tris.begin() + 12 * (size_t)it.first,
                              leaf_tris.begin() + 12 * (size_t)(it.first + it.count));
                tri_off += it.count;
            }
        }
        (*out)[task.wide] = w;
        for (auto k = kids.rbegin(); k != kids.rend(); ++k) stack.push_back(*k);
    }
    return max_depth;
}


uint32_t build_bvh4(const std::vector<BvhNode> &nodes, std::vector<Bvh4Node> *out) {
    out->clear();
    if (nodes.empty()) return 0;
    struct Child {
        float lo[3], hi[3];
        int32_t ref;
    };
    auto child_of = [&](const BvhNode &n, int k) {
        Child c;
        const float *xy = k == 0 ? n.a : n.b;
        c.lo[0] = xy[0]; c.hi[0] = xy[1]; c.lo[1] = xy[2]; c.hi[1] = xy[3];
        c.lo[2] = n.c[2 * k]; c.hi[2] = n.c[2 * k + 1];
        c.ref = n.ref[k];
        return c;
    };
    struct Task {
        int32_t bvh2;   // BVH2 node whose children form the 4-wide node
        uint32_t slot;  // its index in *out
        uint32_t depth;
    };
    std::vector<Task> stack;
    out->push_back(Bvh4Node());
    stack.push_back({0, 0, 1});
    uint32_t depth = 0;
    while (!stack.empty()) {
        const Task t = stack.back();
        stack.pop_back();
        if (t.depth > depth) depth = t.depth;
        Child ch[4];
        int n = 0;
        const BvhNode &b = nodes[(size_t)t.bvh2];
        for (int k = 0; k < 2; ++k) {
            const Child c = child_of(b, k);
            if (c.ref >= 0) {  // open an inner child into its two children
                const BvhNode &g = nodes[(size_t)c.ref];
                ch[n++] = child_of(g, 0);
                ch[n++] = child_of(g, 1);
            } else {
                ch[n++] = c;
            }
        }
        Bvh4Node w;
        memset(&w, 0, sizeof w);
        w.count = (uint32_t)n;
        for (int s = 0; s < 4; ++s) {
            if (s >= n) {
                w.lo_x[s] = w.lo_y[s] = w.lo_z[s] = 0.0f;
                w.hi_x[s] = w.hi_y[s] = w.hi_z[s] = 0.0f;
                w.ref[s] = kEmptyRef4;
                continue;
            }
            w.lo_x[s] = ch[s].lo[0]; w.hi_x[s] = ch[s].hi[0];
            w.lo_y[s] = ch[s].lo[1]; w.hi_y[s] = ch[s].hi[1];
            w.lo_z[s] = ch[s].lo[2]; w.hi_z[s] = ch[s].hi[2];
            if (ch[s].ref >= 0) {
                const uint32_t slot = (uint32_t)out->size();
                out->push_back(Bvh4Node());
                w.ref[s] = (int32_t)slot;
                stack.push_back({ch[s].ref, slot, t.depth + 1});
            } else {
                w.ref[s] = ch[s].ref;
            }
        }
        (*out)[t.slot] = w;
    }
    return depth;
}
}  // namespace lt
