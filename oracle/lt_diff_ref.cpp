// lt_diff_ref.cpp -- host restatement of the differentiable estimator and of
// its path-replay gradient, in double (the FP64 reference) or float.
//
// TEST INFRASTRUCTURE ONLY (checker for lt_render_diff / lt_render_adjoint).
// The estimator: Integrator::RenderPixel's loop (integrator.cpp:98-250) with
// per-triangle albedo and emission, the RGB medium form (distance sampled with
// the mean of sigma_s; isotropic media with sigma_s[0]; weight = transmittance
// x sigma_s / pdf) and roulette on the throughput. Geometry comes from the
// oracle's Embree-rule intersector (lt_oracle.c): hits are float, every
// shading, weight and gradient operation runs in R. The gradient of a loss
// with d loss / d film = dI is, per path, sum over factors w of
// dI * (radiance collected after w) * dlog(w)/dtheta plus, for every emission
// term e, dI * throughput * de/dtheta -- written here directly from the
// estimator, independently of the GPU code.
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include "lt_oracle.h"

namespace {

template <typename R> struct V {
    R x, y, z;
};
template <typename R> V<R> mk(R x, R y, R z) { return V<R>{x, y, z}; }
template <typename R> V<R> operator+(V<R> a, V<R> b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
template <typename R> V<R> operator-(V<R> a, V<R> b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
template <typename R> V<R> operator*(V<R> a, V<R> b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
template <typename R> V<R> operator*(V<R> a, R s) { return mk(a.x * s, a.y * s, a.z * s); }
template <typename R> V<R> operator/(V<R> a, R s) { return mk(a.x / s, a.y / s, a.z / s); }
template <typename R> V<R> operator-(V<R> a) { return mk(-a.x, -a.y, -a.z); }
template <typename R> R dot(V<R> a, V<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename R> V<R> cross(V<R> a, V<R> b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <typename R> R len(V<R> a) { return std::sqrt(dot(a, a)); }
template <typename R> V<R> nrm(V<R> a) { return a * (R(1) / std::sqrt(dot(a, a))); }
template <typename R> V<R> ld(const float *p) { return mk<R>(R(p[0]), R(p[1]), R(p[2])); }

// PCG32 (math/uniform_sampler.h:17-57), seeded with MurmurHash3(pixel, frame)
struct Pcg {
    uint64_t state, inc;
    uint32_t next() {
        uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return (xs >> rot) | (xs << ((0u - rot) & 31u));
    }
    float nextf() {
        uint32_t b = (next() >> 9u) | 0x3F800000u;
        float f;
        std::memcpy(&f, &b, 4);
        return f - 1.0f;
    }
};

template <typename R> V<R> rotate_to_world(R x, R y, R z, V<R> n) {
    V<R> major = std::fabs(n.x) < R(0.57735026919) ? mk<R>(1, 0, 0)
               : (std::fabs(n.y) < R(0.57735026919) ? mk<R>(0, 1, 0) : mk<R>(0, 0, 1));
    V<R> u = nrm(cross(n, major));
    V<R> v = cross(n, u);
    return (u * x + v * y) + n * z;
}

template <typename R> struct Ctx {
    const orc_scene *s;
    const float *albedo, *emission, *sa, *ss;
    uint32_t w, h, spp, first, max_depth, rr_depth;
    float cam[14];
    V<R> bg;
    int nlights;
};

struct Hit {
    bool ok;
    float t, u, v;
    uint32_t prim;
};

template <typename R> Hit closest(const Ctx<R> &c, V<R> o, V<R> d, float tnear) {
    float of[3] = {(float)o.x, (float)o.y, (float)o.z}, df[3] = {(float)d.x, (float)d.y, (float)d.z};
    Hit h;
    uint32_t g, lp;
    h.ok = orc_intersect1(c.s, of, df, tnear, INFINITY, &h.t, &h.u, &h.v, &h.prim, &g, &lp) != 0;
    return h;
}

template <typename R> V<R> shading_normal(const Ctx<R> &c, uint32_t prim, float u, float v) {
    float n[9];
    orc_tri_normals(c.s, prim, n);
    R w = R(1) - R(u) - R(v);
    return nrm((ld<R>(n) * w + ld<R>(n + 3) * R(u)) + ld<R>(n + 6) * R(v));
}

template <typename R> struct Grad {
    std::vector<double> a, e, sa, ss;
};

// one path; kGrad: add gradient terms with path radiance I and adjoint delta
template <typename R, bool kGrad>
V<R> path(const Ctx<R> &c, uint32_t pixel, uint32_t frame, V<R> I, V<R> delta, Grad<R> *G) {
    uint32_t x = pixel % c.w, y = pixel / c.w;
    Pcg g;
    g.state = orc_tile_seed(pixel, frame);
    g.inc = (uint64_t)frame | 1u;
    (void)g.next();
    R fu = R(orc_filter_sample(g.nextf())), fv = R(orc_filter_sample(g.nextf()));
    V<R> view = mk<R>(((R(x) + R(0.5) + fu) / R(c.w) * R(2) - R(1)) * R(c.cam[12]),
                      -((R(y) + R(0.5) + fv) / R(c.h) * R(2) - R(1)) * R(c.cam[13]), R(-1));
    V<R> org = ld<R>(c.cam);
    V<R> dir = mk(dot(view, ld<R>(c.cam + 3)), dot(view, ld<R>(c.cam + 6)), dot(view, ld<R>(c.cam + 9)));
    float tnear = 0.0f;
    V<R> T = mk<R>(1, 1, 1), C = mk<R>(0, 0, 0);
    int lobe = 0, med = -1;
    R iori = 1;
    for (uint32_t b = 0; b < c.max_depth; ++b) {
        Hit h = closest(c, org, dir, tnear);
        if (!h.ok) {
            C = C + T * c.bg;
            break;
        }
        V<R> origin = org, direction = nrm(dir);
        bool surface = true;
        if (med >= 0) {
            int type;
            float sa3[3], ss3[3], gg;
            orc_medium_info(c.s, med, &type, sa3, ss3, &gg);
            V<R> sa = ld<R>(c.sa + 3 * med), ss = ld<R>(c.ss + 3 * med);
            R dist, t = R(h.t);
            bool scat = false;
            V<R> wt;
            if (type == ORC_MED_NON_SCATTERING) {
                dist = t;
                wt = mk(std::exp(-sa.x * dist), std::exp(-sa.y * dist), std::exp(-sa.z * dist));
            } else {
                R sbar = type == ORC_MED_ISOTROPIC ? ss.x : (ss.x + ss.y + ss.z) / R(3);
                dist = -std::log(R(g.nextf())) / sbar;
                scat = dist < t;
                if (!scat) dist = t;
                wt = mk(std::exp(-(sa.x + ss.x - sbar) * dist), std::exp(-(sa.y + ss.y - sbar) * dist),
                        std::exp(-(sa.z + ss.z - sbar) * dist));
                if (scat) wt = wt * (ss / sbar);
            }
            if (kGrad) {
                V<R> Rr = (I - C) * delta;
                for (int k = 0; k < 3; ++k) {
                    R r = k == 0 ? Rr.x : (k == 1 ? Rr.y : Rr.z);
                    R s_k = k == 0 ? ss.x : (k == 1 ? ss.y : ss.z);
                    G->sa[3 * med + k] += double(r * -dist);
                    if (type != ORC_MED_NON_SCATTERING)
                        G->ss[3 * med + k] += double(r * (-dist + (scat ? R(1) / s_k : R(0))));
                }
            }
            T = T * wt;
            if (scat) {
                surface = false;
                org = origin + direction * dist;
                tnear = 0.001f;
                if (type == ORC_MED_HG && gg != 0.0f) {
                    R G0 = R(gg), u1 = R(g.nextf()), u2 = R(g.nextf());
                    R sq = (R(1) - G0 * G0) / (R(1) - G0 + R(2) * G0 * u1);
                    R ct = (R(1) + G0 * G0 - sq * sq) / (R(2) * G0);
                    ct = ct < R(-1) ? R(-1) : (ct > R(1) ? R(1) : ct);
                    R st = std::sqrt(std::max(R(0), R(1) - ct * ct));
                    R ph = R(2) * R(M_PI) * u2;
                    dir = nrm(rotate_to_world(st * std::cos(ph), st * std::sin(ph), ct, direction));
                } else {
                    R cp = R(2) * R(g.nextf()) - R(1);
                    R sp = std::sqrt(R(1) - cp * cp);
                    R th = R(2) * R(M_PI) * R(g.nextf());
                    dir = mk(sp * std::sin(th), cp, sp * std::cos(th));
                }
            }
        }
        if (surface) {
            uint32_t gid = orc_tri_geom(c.s, h.prim);
            int mat, light, has_n;
            orc_geom_info(c.s, gid, &mat, &light, &has_n);
            int bsdf, mmed;
            float alb_m[3], ior_f;
            orc_material_info(c.s, mat, &bsdf, alb_m, &ior_f, &mmed);
            const R ior = R(ior_f);
            V<R> alb = ld<R>(c.albedo + 3 * h.prim);
            if ((b == 0 || (lobe & 3)) && light >= 0) {
                C = C + T * ld<R>(c.emission + 3 * h.prim);
                if (kGrad) {
                    V<R> d = T * delta;
                    G->e[3 * h.prim] += double(d.x);
                    G->e[3 * h.prim + 1] += double(d.y);
                    G->e[3 * h.prim + 2] += double(d.z);
                }
            }
            V<R> P = origin + direction * R(h.t);
            V<R> N = has_n ? shading_normal(c, h.prim, h.u, h.v) : nrm(mk<R>(0, 0, 0));
            V<R> wo = -direction;
            int nl = c.nlights;
            auto bsdf_sample = [&](V<R> &n, V<R> &wi, int &lb, R &ioro) {
                if (bsdf == ORC_BSDF_LAMBERT) {
                    R rnd = R(g.nextf());
                    R r = std::sqrt(rnd), th = R(g.nextf()) * R(2) * R(M_PI);
                    R dx = r * std::cos(th), dy = r * std::sin(th);
                    wi = nrm(rotate_to_world(dx, dy, std::sqrt(R(1) - dx * dx - dy * dy), n));
                    lb = 4;
                } else if (bsdf == ORC_BSDF_MIRROR) {
                    wi = n * (R(2) * dot(wo, n)) - wo;
                    lb = 1;
                } else {
                    R vdn = dot(wo, n), io = ior;
                    if (vdn < 0) { io = 1; n = -n; vdn = -vdn; }
                    R eta = iori / io, s2 = eta * eta * (R(1) - vdn * vdn), F;
                    if (s2 > 1) F = 1;
                    else {
                        R ct = std::sqrt(R(1) - s2);
                        R rp = (iori * vdn - io * ct) / (iori * vdn + io * ct);
                        R rl = (io * vdn - iori * ct) / (io * vdn + iori * ct);
                        F = R(0.5) * (rp * rp + rl * rl);
                    }
                    if (R(g.nextf()) <= F) { wi = n * (R(2) * dot(wo, n)) - wo; lb = 1; ioro = iori; }
                    else { wi = n * (eta * vdn - std::sqrt(R(1) - s2)) - wo * eta; lb = 2; ioro = io; }
                }
            };
            auto light_pdf = [&](int li, V<R> wi, Hit &lh) -> R {
                lh = closest(c, P, wi, 0.001f);
                if (!lh.ok || (int)orc_tri_geom(c.s, lh.prim) != orc_light_geom(c.s, li)) return R(0);
                float area, sph[4], rad[3];
                orc_light_info(c.s, li, &area, sph, rad);
                V<R> d = (P + nrm(wi) * R(lh.t)) - P;
                return dot(d, d) / (std::fabs(dot(shading_normal(c, lh.prim, lh.u, lh.v), wi)) * R(area));
            };
            if (!(nl == 0 || (nl == 1 && light >= 0))) {
                int li;
                do {
                    li = (int)(uint32_t)((float)nl * g.nextf());
                } while (li == light);
                float area, sph[4], rad[3];
                orc_light_info(c.s, li, &area, sph, rad);
                const R fn = R(nl);
                V<R> n2 = N;
                if (bsdf == ORC_BSDF_LAMBERT) {
                    R rnd = R(g.nextf());
                    R r = std::sqrt(rnd) * R(sph[3]), th = R(g.nextf()) * R(2) * R(M_PI);
                    V<R> cd = mk<R>(R(sph[0]), R(sph[1]), R(sph[2])) - P;
                    V<R> ldir = nrm(rotate_to_world(r * std::cos(th), r * std::sin(th), len(cd) - R(sph[3]), nrm(cd)));
                    R cosl = dot(ldir, N);
                    Hit lh;
                    R lpdf = cosl > 0 ? light_pdf(li, ldir, lh) : R(0);
                    R spdf = cosl * R(M_1_PI);
                    if (lpdf != 0 && spdf != 0) {
                        V<R> Li = ld<R>(c.emission + 3 * lh.prim);
                        V<R> f = (alb * R(M_1_PI)) * cosl;
                        R wgt = (lpdf * lpdf) / (lpdf * lpdf + spdf * spdf);
                        C = C + T * ((((f * Li) * wgt) / lpdf) * fn);
                        if (kGrad) {
                            V<R> dga = T * delta * Li * (fn * (cosl * R(M_1_PI)) * wgt / lpdf);
                            V<R> dge = T * delta * f * (fn * wgt / lpdf);
                            G->a[3 * h.prim] += double(dga.x); G->a[3 * h.prim + 1] += double(dga.y);
                            G->a[3 * h.prim + 2] += double(dga.z);
                            G->e[3 * lh.prim] += double(dge.x); G->e[3 * lh.prim + 1] += double(dge.y);
                            G->e[3 * lh.prim + 2] += double(dge.z);
                        }
                    }
                }
                V<R> wi2;
                int lb2 = 0;
                R ioro2 = 0;
                bsdf_sample(n2, wi2, lb2, ioro2);
                R cosb = dot(wi2, n2);
                R spdf = bsdf == ORC_BSDF_LAMBERT ? cosb * R(M_1_PI) : R(1);
                Hit bh;
                R lpdf = (spdf != 0 && cosb > 0) ? light_pdf(li, wi2, bh) : R(0);
                if (lpdf != 0) {
                    V<R> Le = ld<R>(c.emission + 3 * bh.prim);
                    R dfa = bsdf == ORC_BSDF_LAMBERT ? R(M_1_PI) * cosb : R(1);
                    V<R> f = bsdf == ORC_BSDF_LAMBERT ? (alb * R(M_1_PI)) * cosb : alb;
                    R wgt = (spdf * spdf) / (spdf * spdf + lpdf * lpdf);
                    C = C + T * ((((f * Le) * wgt) / spdf) * fn);
                    if (kGrad) {
                        V<R> dga = T * delta * Le * (fn * dfa * wgt / spdf);
                        V<R> dge = T * delta * f * (fn * wgt / spdf);
                        G->a[3 * h.prim] += double(dga.x); G->a[3 * h.prim + 1] += double(dga.y);
                        G->a[3 * h.prim + 2] += double(dga.z);
                        G->e[3 * bh.prim] += double(dge.x); G->e[3 * bh.prim + 1] += double(dge.y);
                        G->e[3 * bh.prim + 2] += double(dge.z);
                    }
                }
            }
            V<R> wi;
            R ioro = 0;
            int lb = 0;
            bsdf_sample(N, wi, lb, ioro);
            if (kGrad) {
                V<R> Rr = (I - C) * delta;
                if (alb.x > 0) G->a[3 * h.prim] += double(Rr.x / alb.x);
                if (alb.y > 0) G->a[3 * h.prim + 1] += double(Rr.y / alb.y);
                if (alb.z > 0) G->a[3 * h.prim + 2] += double(Rr.z / alb.z);
            }
            if (bsdf == ORC_BSDF_LAMBERT) {
                R cw = dot(wi, N);
                T = (T * ((alb * R(M_1_PI)) * cw)) / (cw * R(M_1_PI));
            } else {
                T = (T * alb) / R(1);
            }
            if (lb == 2) { iori = ioro; med = mmed; }
            lobe = lb;
            org = P;
            dir = wi;
            tnear = 0.001f;
        }
        if (b > c.rr_depth) {
            R p = std::max(T.x, std::max(T.y, T.z));
            if (R(g.nextf()) > p) break;
            T = T * (R(1) / p);
        }
    }
    return C;
}

template <typename R>
void run(const Ctx<R> &c, const uint32_t crop[4], const float *dI, double *rgb, Grad<R> *Gtot, int threads) {
    std::atomic<uint32_t> next(0);
    const uint32_t cw = crop[2] - crop[0], chh = crop[3] - crop[1], n = cw * chh;
    std::mutex mu;
    auto body = [&]() {
        Grad<R> G;
        G.a.assign(Gtot->a.size(), 0.0);
        G.e.assign(Gtot->e.size(), 0.0);
        G.sa.assign(Gtot->sa.size(), 0.0);
        G.ss.assign(Gtot->ss.size(), 0.0);
        for (;;) {
            uint32_t k = next.fetch_add(1);
            if (k >= n) break;
            uint32_t pixel = (crop[1] + k / cw) * c.w + crop[0] + k % cw;
            V<R> delta = dI ? ld<R>(dI + 3 * (size_t)pixel) : mk<R>(0, 0, 0);
            V<R> sum = mk<R>(0, 0, 0);
            for (uint32_t s = 0; s < c.spp; ++s) {
                V<R> I = path<R, false>(c, pixel, c.first + s, mk<R>(0, 0, 0), mk<R>(0, 0, 0), nullptr);
                sum = sum + I;
                if (dI && (delta.x != 0 || delta.y != 0 || delta.z != 0))
                    path<R, true>(c, pixel, c.first + s, I, delta, &G);
            }
            if (rgb) {
                rgb[3 * (size_t)pixel] += double(sum.x);
                rgb[3 * (size_t)pixel + 1] += double(sum.y);
                rgb[3 * (size_t)pixel + 2] += double(sum.z);
            }
        }
        std::lock_guard<std::mutex> lock(mu);
        for (size_t i = 0; i < G.a.size(); ++i) Gtot->a[i] += G.a[i];
        for (size_t i = 0; i < G.e.size(); ++i) Gtot->e[i] += G.e[i];
        for (size_t i = 0; i < G.sa.size(); ++i) Gtot->sa[i] += G.sa[i];
        for (size_t i = 0; i < G.ss.size(); ++i) Gtot->ss[i] += G.ss[i];
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t) pool.emplace_back(body);
    body();
    for (auto &t : pool) t.join();
}

template <typename R>
void render_grad(const orc_scene *s, const float *albedo, const float *emission, const float *sa, const float *ss,
                 uint32_t spp, uint32_t first, uint32_t max_depth, uint32_t rr_depth, const uint32_t crop[4],
                 const float *dI, double *rgb, double *ga, double *ge, double *gsa, double *gss, int threads) {
    Ctx<R> c;
    c.s = s;
    c.albedo = albedo;
    c.emission = emission;
    c.sa = sa;
    c.ss = ss;
    c.spp = spp;
    c.first = first;
    c.max_depth = max_depth;
    c.rr_depth = rr_depth;
    orc_camera_info(s, c.cam, &c.w, &c.h);
    float bg[3];
    orc_background_info(s, bg);
    c.bg = ld<R>(bg);
    c.nlights = orc_num_lights(s);
    uint32_t ntri = orc_num_triangles(s), nmed = (uint32_t)orc_num_media(s);
    Grad<R> G;
    G.a.assign(3 * (size_t)ntri, 0.0);
    G.e.assign(3 * (size_t)ntri, 0.0);
    G.sa.assign(3 * (size_t)nmed, 0.0);
    G.ss.assign(3 * (size_t)nmed, 0.0);
    run(c, crop, dI, rgb, &G, threads < 1 ? 1 : threads);
    for (size_t i = 0; i < G.a.size(); ++i) {
        if (ga) ga[i] += G.a[i];
        if (ge) ge[i] += G.e[i];
    }
    for (size_t i = 0; i < G.sa.size(); ++i) {
        if (gsa) gsa[i] += G.sa[i];
        if (gss) gss[i] += G.ss[i];
    }
}

}  // namespace

extern "C" void orc_diff_render(const orc_scene *s, int fp64, const float *albedo, const float *emission,
                                const float *sigma_a, const float *sigma_s, uint32_t spp, uint32_t first_frame,
                                uint32_t max_depth, uint32_t rr_depth, const uint32_t crop[4], const float *dI,
                                double *rgb, double *g_albedo, double *g_emission, double *g_sigma_a,
                                double *g_sigma_s, int threads) {
    if (fp64)
        render_grad<double>(s, albedo, emission, sigma_a, sigma_s, spp, first_frame, max_depth, rr_depth, crop, dI,
                            rgb, g_albedo, g_emission, g_sigma_a, g_sigma_s, threads);
    else
        render_grad<float>(s, albedo, emission, sigma_a, sigma_s, spp, first_frame, max_depth, rr_depth, crop, dI,
                           rgb, g_albedo, g_emission, g_sigma_a, g_sigma_s, threads);
}
