// gbpt_oracle.cpp -- CPU oracle of the globillum path-tracing hot path.
//
// TEST INFRASTRUCTURE ONLY.  This library is loaded by tests/, by
// __graft_entry__.smoke() and by bench.py's CPU-baseline / reference arm as
// the checker and the timed CPU path; the product (libgbpt.so) never links,
// loads or calls it.
//
// It restates the reference's CPU hot path frame-synchronously, exactly as
// the hybrid bouncer sequences it (hybrid-pt.h:115-249): for every path
// sample, camera rays for all pixels (raygen.h:122-181 / raygen.cu:61-118),
// then per bounce a closest-hit trace of all pixels, the area-light sample
// of all pixels (rta::generate_arealight_sample,
// arealight-sampler-cpu.cpp:144-156), an any-hit trace of all shadow rays
// and compute_path_contribution_and_bounce over all pixels
// (hybrid-pt.cpp:450-584, OpenMP over rows as at :462), followed by the
// moving average of new_path (hybrid-pt.h:123-131, util-kernels.cu:17-25).
// Random numbers come in as pools, as the reference downloads them from
// the device (hybrid-pt.h:112-113, :232-233): pool update u of pixel i holds
// three uniforms; path p uses update p for the camera jitter and update
// p*L+b for both the light and the path draws of bounce b (the three
// reference pools are seeded identically, util-kernels.cu:284).
//
// Traversal: its own binary binned-SAH BVH (or brute force), with the
// closest-hit rule "minimum (t, canonical id) over all triangles with
// 0 < t <= t_max" (tracers.cu:113 up to exact ties), so results do not
// depend on the tree.  The per-ray arithmetic (triangle test, light sample,
// BRDFs, camera) is the shared gbpt_math.h, compiled with
// -ffp-contract=off so that every value equals the device's bit for bit.
#include <omp.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../globillum_gb300/csrc/gbpt_host.h"
#include "../globillum_gb300/csrc/gbpt_math.h"
#include "../include/gbpt.h"

using namespace gb;

namespace {

struct OBox {
    float lo[3], hi[3];
};

struct ONode {
    OBox b;
    int left, right;   // inner: children
    int first, count;  // leaf: range in idx
};

struct OScene {
    int n = 0;
    std::vector<float> pos, nrm;  // 9 per triangle
    std::vector<int> mat;
    std::vector<MaterialRec> mats;
    std::vector<LightRec> lights;
    float overall = 0.0f;
    bool use_bvh = true;
    std::vector<ONode> nodes;
    std::vector<int> idx;
    // sky light tables (sky.light = -1 without one)
    SkyTables sky_tab;
    SkyRec sky{};
    // textures (orc_scene_set_textures): 6 texture coordinates per triangle,
    // mip chains; textured = some material has a diffuse texture
    bool textured = false;
    std::vector<float> tc;
    std::vector<std::vector<uint8_t>> tex_data;
    std::vector<TexRec> tex;
    // descriptions the differentiable parameters come from
    std::vector<gb_material> mats_in;
    std::vector<gb_principled_params> params_in;
    std::vector<gb_light> lights_in;
};

void box_grow(OBox& b, const float* p) {
    for (int a = 0; a < 3; ++a) { b.lo[a] = std::min(b.lo[a], p[a]); b.hi[a] = std::max(b.hi[a], p[a]); }
}
void box_grow(OBox& b, const OBox& c) {
    for (int a = 0; a < 3; ++a) { b.lo[a] = std::min(b.lo[a], c.lo[a]); b.hi[a] = std::max(b.hi[a], c.hi[a]); }
}
OBox box_empty() {
    OBox b;
    for (int a = 0; a < 3; ++a) { b.lo[a] = 3e38f; b.hi[a] = -3e38f; }
    return b;
}
float box_area(const OBox& b) {
    float d0 = std::max(0.0f, b.hi[0] - b.lo[0]), d1 = std::max(0.0f, b.hi[1] - b.lo[1]),
          d2 = std::max(0.0f, b.hi[2] - b.lo[2]);
    return d0 * d1 + d1 * d2 + d2 * d0;
}

// Binned SAH (12 bins), leaves of at most 4 triangles.
int build_node(OScene& s, std::vector<OBox>& tb, std::vector<float>& cen, int b, int e) {
    OBox nb = box_empty(), cb = box_empty();
    for (int i = b; i < e; ++i) { box_grow(nb, tb[s.idx[i]]); box_grow(cb, &cen[3 * s.idx[i]]); }
    int me = (int)s.nodes.size();
    s.nodes.push_back(ONode{nb, -1, -1, b, 0});
    int cnt = e - b;
    if (cnt <= 4) { s.nodes[me].count = cnt; return me; }
    const int K = 12;
    float best = 3e38f; int ba = -1, bk = -1;
    for (int a = 0; a < 3; ++a) {
        float ext = cb.hi[a] - cb.lo[a];
        if (!(ext > 0.0f)) continue;
        OBox bins[K]; int bc[K];
        for (int k = 0; k < K; ++k) { bins[k] = box_empty(); bc[k] = 0; }
        for (int i = b; i < e; ++i) {
            int t = s.idx[i];
            int k = std::min(K - 1, (int)((cen[3 * t + a] - cb.lo[a]) / ext * K));
            box_grow(bins[k], tb[t]); bc[k]++;
        }
        for (int k = 0; k < K - 1; ++k) {
            OBox l = box_empty(), r = box_empty(); int nl = 0, nr = 0;
            for (int j = 0; j <= k; ++j) { box_grow(l, bins[j]); nl += bc[j]; }
            for (int j = k + 1; j < K; ++j) { box_grow(r, bins[j]); nr += bc[j]; }
            if (!nl || !nr) continue;
            float c = box_area(l) * nl + box_area(r) * nr;
            if (c < best) { best = c; ba = a; bk = k; }
        }
    }
    int mid = b + cnt / 2;
    if (ba >= 0) {
        float ext = cb.hi[ba] - cb.lo[ba];
        int* p = std::partition(&s.idx[b], &s.idx[b] + cnt, [&](int t) {
            return std::min(K - 1, (int)((cen[3 * t + ba] - cb.lo[ba]) / ext * K)) <= bk;
        });
        mid = (int)(p - &s.idx[0]);
        if (mid == b || mid == e) mid = b + cnt / 2;
    }
    int l = build_node(s, tb, cen, b, mid);
    int r = build_node(s, tb, cen, mid, e);
    s.nodes[me].left = l; s.nodes[me].right = r;
    return me;
}

void build_bvh(OScene& s) {
    std::vector<OBox> tb(s.n);
    std::vector<float> cen(3 * (size_t)s.n);
    for (int t = 0; t < s.n; ++t) {
        OBox b = box_empty();
        for (int v = 0; v < 3; ++v) box_grow(b, &s.pos[9 * (size_t)t + 3 * v]);
        // pad outward by 2^-18 of the magnitude so that slab tests stay
        // conservative under rounding
        float m = 0.0f;
        for (int a = 0; a < 3; ++a) m = std::max(m, std::max(std::fabs(b.lo[a]), std::fabs(b.hi[a])));
        float d = m * (1.0f / 262144.0f) + 1e-30f;
        for (int a = 0; a < 3; ++a) { b.lo[a] -= d; b.hi[a] += d; cen[3 * (size_t)t + a] = 0.5f * (b.lo[a] + b.hi[a]); }
        tb[t] = b;
    }
    s.idx.resize(s.n);
    for (int i = 0; i < s.n; ++i) s.idx[i] = i;
    s.nodes.clear();
    s.nodes.reserve(2 * (size_t)s.n);
    build_node(s, tb, cen, 0, s.n);
}

// Slab test with a relative slack of 1e-5 on the interval (conservative).
inline bool slab(const OBox& b, const v3& o, const v3& inv, float bound, float* tentry) {
    float t0x = (b.lo[0] - o.x) * inv.x, t1x = (b.hi[0] - o.x) * inv.x;
    float t0y = (b.lo[1] - o.y) * inv.y, t1y = (b.hi[1] - o.y) * inv.y;
    float t0z = (b.lo[2] - o.z) * inv.z, t1z = (b.hi[2] - o.z) * inv.z;
    float tmin = std::max(std::max(std::min(t0x, t1x), std::min(t0y, t1y)), std::min(t0z, t1z));
    float tmax = std::min(std::min(std::max(t0x, t1x), std::max(t0y, t1y)), std::max(t0z, t1z));
    float lo = std::max(tmin * 0.99999f, 0.0f);
    float hi = std::min(tmax * 1.00001f, bound);
    *tentry = lo;
    return lo <= hi;
}

inline bool tri_test(const OScene& s, int t, const v3& o, const v3& d, float* tt, float* u, float* v) {
    const float* p = &s.pos[9 * (size_t)t];
    v3 a = mk(p[0], p[1], p[2]);
    v3 e1 = mk(p[3] - p[0], p[4] - p[1], p[5] - p[2]);
    v3 e2 = mk(p[6] - p[0], p[7] - p[1], p[8] - p[2]);
    return intersect_tri(o, d, a, e1, e2, tt, u, v);
}

// Closest hit: minimum (t, id) over 0 < t <= tmax.
gb_hit trace_closest(const OScene& s, v3 o, v3 d, float tmax, uint64_t* visits, uint64_t* tests) {
    gb_hit h{FLT_MAX, 0.0f, 0.0f, 0xffffffffu};
    if (!(tmax >= 0.0f)) return h;
    if (!s.use_bvh) {
        for (int t = 0; t < s.n; ++t) {
            float tt, u, v;
            if (tests) ++*tests;
            if (tri_test(s, t, o, d, &tt, &u, &v) && tt <= tmax && closer(tt, (uint32_t)t, h.t, h.ref))
                h = gb_hit{tt, u, v, (uint32_t)t};
        }
        return h;
    }
    const float ooeps = 8.271806125530277e-25f;
    v3 inv = mk(1.0f / (std::fabs(d.x) > ooeps ? d.x : std::copysign(ooeps, d.x)),
                1.0f / (std::fabs(d.y) > ooeps ? d.y : std::copysign(ooeps, d.y)),
                1.0f / (std::fabs(d.z) > ooeps ? d.z : std::copysign(ooeps, d.z)));
    int stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const ONode& nd = s.nodes[stack[--sp]];
        float te;
        if (visits) ++*visits;
        if (!slab(nd.b, o, inv, std::min(h.t, tmax), &te)) continue;
        if (nd.count > 0) {
            for (int i = 0; i < nd.count; ++i) {
                int t = s.idx[nd.first + i];
                float tt, u, v;
                if (tests) ++*tests;
                if (tri_test(s, t, o, d, &tt, &u, &v) && tt <= tmax && closer(tt, (uint32_t)t, h.t, h.ref))
                    h = gb_hit{tt, u, v, (uint32_t)t};
            }
            continue;
        }
        float tl, tr;
        bool hl = slab(s.nodes[nd.left].b, o, inv, std::min(h.t, tmax), &tl);
        bool hr = slab(s.nodes[nd.right].b, o, inv, std::min(h.t, tmax), &tr);
        if (hl && hr) {
            if (sp + 2 > 128) break;
            if (tl <= tr) { stack[sp++] = nd.right; stack[sp++] = nd.left; }
            else { stack[sp++] = nd.left; stack[sp++] = nd.right; }
        } else if (hl) { stack[sp++] = nd.left; }
        else if (hr) { stack[sp++] = nd.right; }
    }
    return h;
}

bool trace_any(const OScene& s, v3 o, v3 d, float tmax) {
    if (!(tmax >= 0.0f)) return false;
    if (!s.use_bvh) {
        for (int t = 0; t < s.n; ++t) {
            float tt, u, v;
            if (tri_test(s, t, o, d, &tt, &u, &v) && tt <= tmax) return true;
        }
        return false;
    }
    const float ooeps = 8.271806125530277e-25f;
    v3 inv = mk(1.0f / (std::fabs(d.x) > ooeps ? d.x : std::copysign(ooeps, d.x)),
                1.0f / (std::fabs(d.y) > ooeps ? d.y : std::copysign(ooeps, d.y)),
                1.0f / (std::fabs(d.z) > ooeps ? d.z : std::copysign(ooeps, d.z)));
    int stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const ONode& nd = s.nodes[stack[--sp]];
        float te;
        if (!slab(nd.b, o, inv, tmax, &te)) continue;
        if (nd.count > 0) {
            for (int i = 0; i < nd.count; ++i) {
                float tt, u, v;
                if (tri_test(s, s.idx[nd.first + i], o, d, &tt, &u, &v) && tt <= tmax) return true;
            }
            continue;
        }
        if (sp + 2 > 128) break;
        stack[sp++] = nd.left;
        stack[sp++] = nd.right;
    }
    return false;
}

inline v3 tri_interp(const std::vector<float>& a, int t, float beta, float gamma) {
    const float* p = &a[9 * (size_t)t];
    return bary(beta, gamma, mk(p[0], p[1], p[2]), mk(p[3], p[4], p[5]), mk(p[6], p[7], p[8]));
}

// pixel_generate_arealight_sample_cpu (arealight-sampler-cpu.cpp:25-143).
// *sd holds the buffer's direction on entry (read by the miss branch).
void nee_pixel(const OScene& s, int id, const gb_hit& h, v3 rnd, float shadow_offset, v3* so, v3* sd, float* smax,
               v3* psc) {
    if (h.ref != 0xffffffffu && !s.lights.empty()) {
        int l = pick_light(s.lights.data(), (int)s.lights.size(), s.overall, rnd.z);
        v3 P = tri_interp(s.pos, (int)h.ref, h.beta, h.gamma);
        v3 N = tri_interp(s.nrm, (int)h.ref, h.beta, h.gamma);
        if (s.lights[l].type == 1)
            sky_light_sample(s.sky, s.lights[l].power, s.overall, P, N, rnd.x, rnd.y, shadow_offset, so, sd, smax,
                             psc);
        else
            rect_light_sample(s.lights[l], s.lights[l].col, s.overall, P, N, rnd.x, rnd.y, shadow_offset, so, sd,
                              smax, psc);
    } else {
        v3 d = *sd;
        *so = mk(FLT_MAX, FLT_MAX, FLT_MAX);
        *sd = mk(0.0f, 0.0f, 0.0f);
        *smax = -1.0f;
        *psc = s.sky.light >= 0 ? s.sky.scale * sky_eval(s.sky, d) : mk(0.0f, 0.0f, 0.0f);
    }
    (void)id;
}

// ---------------------------------------------------- FP64 adjoint reference --
// Forward-mode dual numbers in double: value and derivative with respect to
// one parameter.
struct Dd {
    double v, d;
};
inline Dd cst(double x) { return Dd{x, 0.0}; }
inline Dd operator+(Dd a, Dd b) { return Dd{a.v + b.v, a.d + b.d}; }
inline Dd operator-(Dd a, Dd b) { return Dd{a.v - b.v, a.d - b.d}; }
inline Dd operator*(Dd a, Dd b) { return Dd{a.v * b.v, a.d * b.v + a.v * b.d}; }
inline Dd operator/(Dd a, Dd b) { return Dd{a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)}; }
inline Dd powc(Dd a, double e) {  // a^e for a >= 0
    if (a.v <= 0.0) return Dd{0.0, 0.0};
    return Dd{std::pow(a.v, e), e * std::pow(a.v, e - 1.0) * a.d};
}
inline Dd mixd(Dd x, Dd y, Dd t) { return (cst(1.0) - t) * x + t * y; }

struct MatD {
    int kind;
    Dd diffuse[3], metallic, subsurface, roughness, sheen, clearcoat;
    Dd cdlin[3], csheen[3], cspec0[3];
    double cc_a, cc_a2m1, cc_pilog;
};

// make_material (principledMaterial.h:178-252 constants) in dual numbers;
// `seed` = 0..4 marks colour r, g, b, roughness or metallic as the variable.
MatD make_material_d(const gb_material& m, const gb_principled_params* params, int seed) {
    MatD r{};
    if (m.principled < 0) {
        r.kind = MAT_LAMBERT;
        for (int c = 0; c < 3; ++c) r.diffuse[c] = Dd{m.diffuse[c], seed == c ? 1.0 : 0.0};
        return r;
    }
    const gb_principled_params& p = params[m.principled];
    r.kind = MAT_PRINCIPLED;
    Dd col[3];
    for (int c = 0; c < 3; ++c) col[c] = Dd{p.color[c], seed == c ? 1.0 : 0.0};
    r.roughness = Dd{p.roughness, seed == 3 ? 1.0 : 0.0};
    r.metallic = Dd{p.metallic, seed == 4 ? 1.0 : 0.0};
    r.subsurface = cst(p.subsurface);
    r.sheen = cst(p.sheen);
    r.clearcoat = cst(p.clearcoat);
    Dd cd[3];
    for (int c = 0; c < 3; ++c) cd[c] = powc(col[c], 2.2);
    Dd lum = cst(.3) * cd[0] + cst(.6) * cd[1] + cst(.1) * cd[2];
    for (int c = 0; c < 3; ++c) {
        Dd ct = lum.v > 0.0 ? cd[c] / lum : cst(1.0);
        r.cdlin[c] = cd[c];
        r.csheen[c] = cst(1.0 - p.sheen_tint) + cst(p.sheen_tint) * ct;
        Dd st = cst(1.0 - p.specular_tint) + cst(p.specular_tint) * ct;
        r.cspec0[c] = (cst(1.0) - r.metallic) * cst(p.specular * .08) * st + r.metallic * cd[c];
    }
    double a = (1.0 - p.clearcoat_gloss) * 0.1 + p.clearcoat_gloss * 0.001;
    r.cc_a = a;
    r.cc_a2m1 = a * a - 1.0;
    r.cc_pilog = M_PI * std::log(a * a);
    return r;
}

struct V3d {
    double x, y, z;
};
inline V3d vd(v3 a) { return V3d{a.x, a.y, a.z}; }
inline double dotd(V3d a, V3d b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double schlickd(double u) {
    double m = std::min(1.0, std::max(0.0, 1.0 - u));
    return m * m * m * m * m;
}
inline double smithd(double ndv, double ag) {
    double a = ag * ag, b = ndv * ndv;
    return 1.0 / (ndv + std::sqrt(a + b - a * b));
}

// material_eval (principledMaterial.h:210-301, simpleMaterial.h:82-113) in double.
void eval_d(const MatD& m, int lobe, V3d V, V3d L, V3d N, Dd out[3]) {
    for (int c = 0; c < 3; ++c) out[c] = cst(0.0);
    if (m.kind == MAT_LAMBERT) {
        double f = std::fabs(dotd(L, N)) / M_PI;
        for (int c = 0; c < 3; ++c) out[c] = m.diffuse[c] * cst(f);
        return;
    }
    if (lobe == LOBE_SPECULAR_REFLECTION) { for (int c = 0; c < 3; ++c) out[c] = cst(1.0); return; }
    if (lobe == LOBE_SPECULAR_TRANSMISSION) {
        for (int c = 0; c < 3; ++c) out[c] = cst(1.0 / std::fabs(dotd(L, N)));
        return;
    }
    double NdotL = dotd(N, L), NdotV = dotd(N, V);
    if (NdotL < 0.0 || NdotV < 0.0) return;
    V3d H{L.x + V.x, L.y + V.y, L.z + V.z};
    double hl = std::sqrt(dotd(H, H));
    H = V3d{H.x / hl, H.y / hl, H.z / hl};
    double LdotH = dotd(L, H), FH = schlickd(LdotH);
    if (lobe == LOBE_DISNEY_REFLECTION) {
        double NdotH = dotd(N, H), cg = 0.0;
        if (m.clearcoat.v > 0.0) {
            double Dr = m.cc_a >= 1.0 ? 1.0 / M_PI : m.cc_a2m1 / (m.cc_pilog * (1.0 + m.cc_a2m1 * NdotH * NdotH));
            double Fr = (1.0 - FH) * 0.04 + FH;
            cg = 0.25 * m.clearcoat.v * smithd(NdotL, 0.25) * smithd(NdotV, 0.25) * Fr * Dr;
        }
        for (int c = 0; c < 3; ++c)
            out[c] = (cst(1.0 - FH) * m.cspec0[c] + cst(FH + cg)) * cst(NdotL) * m.metallic;
        return;
    }
    double FL = schlickd(NdotL), FV = schlickd(NdotV);
    Dd Fd90 = cst(0.5) + cst(2.0 * LdotH * LdotH) * m.roughness;
    Dd Fd = mixd(cst(1.0), Fd90, cst(FL)) * mixd(cst(1.0), Fd90, cst(FV));
    Dd Fss90 = cst(LdotH * LdotH) * m.roughness;
    Dd Fss = mixd(cst(1.0), Fss90, cst(FL)) * mixd(cst(1.0), Fss90, cst(FV));
    Dd ss = cst(1.25) * (Fss * cst(1.0 / (NdotL + NdotV) - 0.5) + cst(0.5));
    Dd k = cst(1.0 / M_PI) * mixd(Fd, ss, m.subsurface);
    for (int c = 0; c < 3; ++c)
        out[c] = (k * m.cdlin[c] + cst(FH) * m.sheen * m.csheen[c]) * (cst(1.0) - m.metallic) * cst(NdotL);
}

// One shaded vertex of a replayed path.
constexpr int kReplayBounces = 64;  // bounces orc_adjoint_f64 replays per path at most

struct AdjVertex {
    int mi, light, lobe;
    bool nee;
    float pdf, q, scale;
    v3 wo, wi, N, ld;
    uint32_t flags;  // SAMPLE_* of the vertex's BRDF sample
};

int shade_stage(const OScene& s, int w, int h, const gb_render_desc* desc, float* ray_orig, float* ray_dir,
                float* max_t, const gb_hit* hits, const uint8_t* occl, const float* rnd, float* tp, float* accum,
                const float* to_light, const float* psc, int path, int bounce, int pixel_base, RayDiff* rdiff);

}  // namespace

extern "C" {

void* orc_scene_create(int n, const float* pos, const float* nrm, const int* mat, int nmat, const gb_material* mats,
                       int nparams, const gb_principled_params* params, int nl, const gb_light* lights, int use_bvh) {
    if (n <= 0 || !pos || !mat || nmat <= 0 || !mats) return nullptr;
    OScene* s = new OScene();
    s->n = n;
    s->pos.assign(pos, pos + 9 * (size_t)n);
    if (nrm) s->nrm.assign(nrm, nrm + 9 * (size_t)n);
    else {
        s->nrm.resize(9 * (size_t)n);
        for (int t = 0; t < n; ++t) {
            const float* p = pos + 9 * (size_t)t;
            v3 fn = normalize_div(cross(mk(p[3] - p[0], p[4] - p[1], p[5] - p[2]), mk(p[6] - p[0], p[7] - p[1], p[8] - p[2])));
            for (int k = 0; k < 3; ++k) { s->nrm[9 * t + 3 * k] = fn.x; s->nrm[9 * t + 3 * k + 1] = fn.y; s->nrm[9 * t + 3 * k + 2] = fn.z; }
        }
    }
    s->mat.assign(mat, mat + n);
    (void)nparams;
    for (int m = 0; m < nmat; ++m) {
        // the round trip through the 32-float record is what the device sees
        float f[kMaterialFloats];
        pack_material(make_material(mats[m], params), f);
        s->mats.push_back(unpack_material(f));
    }
    s->sky.light = -1;
    for (int l = 0; l < nl; ++l) {
        s->lights.push_back(make_light(lights[l]));
        if (lights[l].type == GB_LIGHT_SKY && lights[l].sky_rgb && lights[l].sky_w > 0 && lights[l].sky_h > 0) {
            make_sky_tables(lights[l].sky_rgb, lights[l].sky_w, lights[l].sky_h, &s->sky_tab);
            s->sky.light = l;
        }
    }
    if (s->sky.light >= 0) {
        SkyTables& t = s->sky_tab;
        s->sky.texel = t.texel.data();
        s->sky.row_cdf = t.row_cdf.data();
        s->sky.row_pdf = t.row_pdf.data();
        s->sky.col_cdf = t.col_cdf.data();
        s->sky.col_pdf = t.col_pdf.data();
        s->sky.w = t.w;
        s->sky.h = t.h;
        s->sky.scale = s->lights[s->sky.light].scale;
    }
    s->overall = overall_power(s->lights.data(), (int)s->lights.size());
    s->mats_in.assign(mats, mats + nmat);
    if (nparams > 0 && params) s->params_in.assign(params, params + nparams);
    if (nl > 0) s->lights_in.assign(lights, lights + nl);
    s->use_bvh = use_bvh != 0;
    if (s->use_bvh) build_bvh(*s);
    return s;
}

void orc_scene_destroy(void* s) { delete (OScene*)s; }

// Diffuse textures of a scene (gb_scene_desc's texture fields): mip chains
// by make_mipmaps, texture index per material.  Returns 1 for bad input.
int orc_scene_set_textures(void* sp, int ntex, const gb_texture* tex, const float* texcoords, const int* dtex) {
    OScene& s = *(OScene*)sp;
    if (ntex < 0 || (ntex > 0 && !tex)) return 1;
    s.tex_data.assign((size_t)ntex, std::vector<uint8_t>());
    s.tex.assign((size_t)ntex, TexRec{});
    for (int k = 0; k < ntex; ++k) {
        if (!tex[k].rgba || tex[k].w <= 0 || tex[k].h <= 0) return 1;
        make_mipmaps(tex[k].rgba, tex[k].w, tex[k].h, &s.tex_data[k], &s.tex[k].max_mm, &s.tex[k].size);
        s.tex[k].texels = s.tex_data[k].data();
        s.tex[k].w = tex[k].w;
        s.tex[k].h = tex[k].h;
    }
    s.textured = false;
    for (size_t m = 0; m < s.mats.size(); ++m) {
        const int v = dtex ? dtex[m] : -1;
        if (v < -1 || v >= ntex) return 1;
        s.mats[m].dtex = v;
        s.textured = s.textured || v >= 0;
    }
    if (s.textured) {
        if (!texcoords) return 1;
        s.tc.assign(texcoords, texcoords + 6 * (size_t)s.n);
    }
    return 0;
}

int orc_trace_closest(void* sp, int n, const float* o, const float* d, const float* tmax, gb_hit* hits,
                      uint64_t* counts) {
    const OScene& s = *(const OScene*)sp;
    uint64_t vis = 0, tst = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : vis, tst)
    for (int i = 0; i < n; ++i) {
        uint64_t v = 0, t = 0;
        hits[i] = trace_closest(s, mk(o[3 * i], o[3 * i + 1], o[3 * i + 2]), mk(d[3 * i], d[3 * i + 1], d[3 * i + 2]),
                                tmax[i], &v, &t);
        vis += v; tst += t;
    }
    if (counts) { counts[0] = vis; counts[1] = tst; }
    return 0;
}

int orc_trace_any(void* sp, int n, const float* o, const float* d, const float* tmax, uint8_t* occl) {
    const OScene& s = *(const OScene*)sp;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < n; ++i)
        occl[i] = trace_any(s, mk(o[3 * i], o[3 * i + 1], o[3 * i + 2]), mk(d[3 * i], d[3 * i + 1], d[3 * i + 2]),
                            tmax[i]) ? 1 : 0;
    return 0;
}

// rta::generate_arealight_sample on a w x h grid (host buffers, reference
// layout).  Serial when `serial` (the reference's `omp prallel` typo at
// arealight-sampler-cpu.cpp:148), else OpenMP over rows.
int orc_generate_arealight_sample(void* sp, int w, int h, float shadow_offset, const float* rnd, const gb_hit* hits,
                                  float* ray_orig, float* ray_dir, float* max_t, float* psc, int serial) {
    const OScene& s = *(const OScene*)sp;
#pragma omp parallel for schedule(dynamic, 1) if (!serial)
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            int id = y * w + x;
            v3 so, ps; float sm;
            v3 sd = mk(ray_dir[3 * id], ray_dir[3 * id + 1], ray_dir[3 * id + 2]);
            nee_pixel(s, id, hits[id], mk(rnd[3 * id], rnd[3 * id + 1], rnd[3 * id + 2]), shadow_offset, &so, &sd, &sm, &ps);
            ray_orig[3 * id] = so.x; ray_orig[3 * id + 1] = so.y; ray_orig[3 * id + 2] = so.z;
            ray_dir[3 * id] = sd.x; ray_dir[3 * id + 1] = sd.y; ray_dir[3 * id + 2] = sd.z;
            max_t[id] = sm;
            psc[3 * id] = ps.x; psc[3 * id + 1] = ps.y; psc[3 * id + 2] = ps.z;
        }
    return 0;
}

// compute_path_contribution_and_bounce (hybrid-pt.cpp:450-584), host buffers.
int orc_compute_path_contribution_and_bounce(void* sp, int w, int h, const gb_render_desc* desc, float* ray_orig,
                                             float* ray_dir, float* max_t, const gb_hit* hits,
                                             const uint8_t* occl, const float* rnd, float* tp, float* accum,
                                             const float* to_light, const float* psc, int path, int bounce,
                                             int pixel_base) {
    return shade_stage(*(const OScene*)sp, w, h, desc, ray_orig, ray_dir, max_t, hits, occl, rnd, tp, accum, to_light,
                       psc, path, bounce, pixel_base, nullptr);
}

}  // extern "C"

namespace {

// compute_path_contribution_and_bounce (hybrid-pt.cpp:450-584) over a
// w x h block; rdiff (textured scenes) holds each pixel's ray
// differentials, moved to the hit by computeRayDiffs (:300-328) before the
// material is set up with the texture's colour.
int shade_stage(const OScene& s, int w, int h, const gb_render_desc* desc, float* ray_orig, float* ray_dir,
                float* max_t, const gb_hit* hits, const uint8_t* occl, const float* rnd, float* tp, float* accum,
                const float* to_light, const float* psc, int path, int bounce, int pixel_base, RayDiff* rdiff) {
    ShadeParams par = make_shade_params(*desc);
#pragma omp parallel for schedule(dynamic, 1)
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            int id = y * w + x;
            const gb_hit& hh = hits[id];
            v3 t = mk(tp[3 * id], tp[3 * id + 1], tp[3 * id + 2]);
            v3 ac = mk(accum[3 * id], accum[3 * id + 1], accum[3 * id + 2]);
            bool alive = false;
            if (hh.ref != 0xffffffffu) {
                v3 P = tri_interp(s.pos, (int)hh.ref, hh.beta, hh.gamma);
                v3 N = tri_interp(s.nrm, (int)hh.ref, hh.beta, hh.gamma);
                MaterialRec m = s.mats[s.mat[hh.ref]];
                if (s.textured && rdiff) {
                    const float* p = &s.pos[9 * (size_t)hh.ref];
                    const float* tcs = &s.tc[6 * (size_t)hh.ref];
                    float ts, tt;
                    bary2(hh.beta, hh.gamma, tcs, &ts, &tt);
                    const float diff = ray_diff_hit(&rdiff[id], mk(p[0], p[1], p[2]), mk(p[3], p[4], p[5]),
                                                    mk(p[6], p[7], p[8]), tcs, ts, tt, normalize_div(N));
                    if (m.dtex >= 0 && m.dtex < (int)s.tex.size())
                        m = textured_material(m, tex_sample_bilin_lod(s.tex[m.dtex], ts, tt, diff));
                }
                ShadeOut o = shade_hit(m, P, N, mk(ray_dir[3 * id], ray_dir[3 * id + 1], ray_dir[3 * id + 2]), t,
                                       mk(rnd[3 * id], rnd[3 * id + 1], rnd[3 * id + 2]), occl[id] == 0,
                                       mk(to_light[3 * id], to_light[3 * id + 1], to_light[3 * id + 2]),
                                       mk(psc[3 * id], psc[3 * id + 1], psc[3 * id + 2]), par,
                                       (uint32_t)(pixel_base + id), (uint32_t)path, bounce);
                ac = ac + o.accum_add;
                t = o.tp;
                alive = o.alive;
                if (alive) {
                    ray_orig[3 * id] = o.org.x; ray_orig[3 * id + 1] = o.org.y; ray_orig[3 * id + 2] = o.org.z;
                    ray_dir[3 * id] = o.dir.x; ray_dir[3 * id + 1] = o.dir.y; ray_dir[3 * id + 2] = o.dir.z;
                    max_t[id] = FLT_MAX;
                }
            } else {
                if (max_t[id] != -1.0f)
                    ac = ac + miss_contribution(t, mk(ray_dir[3 * id], ray_dir[3 * id + 1], ray_dir[3 * id + 2]), par,
                                                &s.sky);
                t = mk(0.0f, 0.0f, 0.0f);
            }
            if (!alive) {
                ray_orig[3 * id] = FLT_MAX; ray_orig[3 * id + 1] = FLT_MAX; ray_orig[3 * id + 2] = FLT_MAX;
                ray_dir[3 * id] = 0.0f; ray_dir[3 * id + 1] = 0.0f; ray_dir[3 * id + 2] = 0.0f;
                max_t[id] = -1.0f;
            }
            tp[3 * id] = t.x; tp[3 * id + 1] = t.y; tp[3 * id + 2] = t.z;
            accum[3 * id] = ac.x; accum[3 * id + 1] = ac.y; accum[3 * id + 2] = ac.z;
        }
    return 0;
}


}  // namespace

extern "C" {

// Full progressive frame over rows [row0, row1) of a w x h image.
// pool: `pool_updates` updates of the rows' pixels, layout
// [update][pixel - row0*w][3]; needs spp*L updates.  out_rgb: (row1-row0)*w*3.
// stats (optional): camera, extension, shadow rays, node visits, tri tests.
int orc_render(void* sp, const gb_camera* cam, const gb_render_desc* d, int row0, int row1, const float* pool,
               int pool_updates, float* out_rgb, int serial_nee, uint64_t* stats) {
    const OScene& s = *(const OScene*)sp;
    const int W = d->width, H = d->height, L = d->max_bounces;
    if (row0 < 0 || row1 > H || row0 >= row1) return 1;
    if (pool_updates < d->spp * L) return 2;
    if (cam->aperture != 0.0f && (row0 != 0 || row1 != H)) return 3;
    const int h = row1 - row0, n = W * h, base = row0 * W;
    CameraRec C = make_camera(*cam, W, H);
    ShadeParams par = make_shade_params(*d);
    std::vector<float> ro(3 * (size_t)n), rd(3 * (size_t)n), mt(n), so(3 * (size_t)n), sd(3 * (size_t)n), sm(n),
        ps(3 * (size_t)n), tp(3 * (size_t)n), ac(3 * (size_t)n), lr(3 * (size_t)n), rnd(3 * (size_t)n);
    std::vector<gb_hit> hits(n);
    std::vector<uint8_t> occl(n);
    std::vector<RayDiff> rdf(s.textured ? (size_t)n : 0);
    std::fill(out_rgb, out_rgb + 3 * (size_t)n, 0.0f);
    uint64_t n_cam = 0, n_ext = 0, n_sh = 0, n_vis = 0, n_tst = 0;
    for (int p = 0; p < d->spp; ++p) {
        // new_path: throughput 1, accumulation 0, camera rays with jitter update p
        const float* jp = pool + (size_t)p * n * 3;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            int id = base + i;
            int x = id % W, y = id / W;
            float lx = 0.0f, ly = 0.0f;
            if (C.aperture != 0.0f) {
                int o = (id + 17) % (W * H);
                lx = jp[3 * o + 2] - 0.5f;
                ly = jp[3 * o + 1] - 0.5f;
            }
            v3 o, dd;
            camera_ray(C, x, y, jp[3 * i], jp[3 * i + 1], lx, ly, &o, &dd);
            ro[3 * i] = o.x; ro[3 * i + 1] = o.y; ro[3 * i + 2] = o.z;
            rd[3 * i] = dd.x; rd[3 * i + 1] = dd.y; rd[3 * i + 2] = dd.z;
            mt[i] = FLT_MAX;
            if (s.textured) rdf[i] = camera_diff(C, x, y);
            tp[3 * i] = tp[3 * i + 1] = tp[3 * i + 2] = 1.0f;
            ac[3 * i] = ac[3 * i + 1] = ac[3 * i + 2] = 0.0f;
        }
        n_cam += n;
        for (int b = 0; b < L; ++b) {
            const float* up = pool + ((size_t)p * L + b) * n * 3;
            // closest hit of every live ray (dead rays: max_t == -1)
            uint64_t ce = 0, cv = 0, ct = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : ce, cv, ct)
            for (int i = 0; i < n; ++i) {
                if (mt[i] < 0.0f) { hits[i] = gb_hit{FLT_MAX, 0.0f, 0.0f, 0xffffffffu}; continue; }
                uint64_t v = 0, t = 0;
                hits[i] = trace_closest(s, mk(ro[3 * i], ro[3 * i + 1], ro[3 * i + 2]),
                                        mk(rd[3 * i], rd[3 * i + 1], rd[3 * i + 2]), mt[i], &v, &t);
                ce += 1; cv += v; ct += t;
            }
            if (b > 0) n_ext += ce;
            n_vis += cv; n_tst += ct;
            // light draws: the light pool, or Halton (h2(i+1), h3(i+1), h3(i+1))
            for (int i = 0; i < n; ++i) {
                if (d->rng_mode == GB_RNG_HALTON_LIGHT) {
                    float hy = halton(base + i + 1, 3);
                    lr[3 * i] = halton(base + i + 1, 2); lr[3 * i + 1] = hy; lr[3 * i + 2] = hy;
                } else {
                    lr[3 * i] = up[3 * i]; lr[3 * i + 1] = up[3 * i + 1]; lr[3 * i + 2] = up[3 * i + 2];
                }
                rnd[3 * i] = up[3 * i]; rnd[3 * i + 1] = up[3 * i + 1]; rnd[3 * i + 2] = up[3 * i + 2];
            }
            orc_generate_arealight_sample(sp, W, h, d->shadow_offset, lr.data(), hits.data(), so.data(), sd.data(),
                                          sm.data(), ps.data(), serial_nee);
            uint64_t cs = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : cs)
            for (int i = 0; i < n; ++i) {
                if (hits[i].ref == 0xffffffffu) { occl[i] = 1; continue; }
                occl[i] = (sm[i] >= 0.0f) ? (trace_any(s, mk(so[3 * i], so[3 * i + 1], so[3 * i + 2]),
                                                       mk(sd[3 * i], sd[3 * i + 1], sd[3 * i + 2]), sm[i]) ? 1 : 0)
                                          : 1;
                cs += 1;
            }
            n_sh += cs;
            shade_stage(s, W, h, d, ro.data(), rd.data(), mt.data(), hits.data(), occl.data(), rnd.data(), tp.data(),
                        ac.data(), sd.data(), ps.data(), p, b, base, s.textured ? rdf.data() : nullptr);
        }
        // new_path: moving average
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            v3 c = combine_sample(mk(out_rgb[3 * i], out_rgb[3 * i + 1], out_rgb[3 * i + 2]),
                                  mk(ac[3 * i], ac[3 * i + 1], ac[3 * i + 2]), p);
            out_rgb[3 * i] = c.x; out_rgb[3 * i + 1] = c.y; out_rgb[3 * i + 2] = c.z;
        }
    }
    (void)par;
    if (stats) { stats[0] = n_cam; stats[1] = n_ext; stats[2] = n_sh; stats[3] = n_vis; stats[4] = n_tst; }
    return 0;
}

// FP64 reference gradient of sum(dimg * image) over rows [row0, row1) with
// respect to the parameters `sel` (gb_scene_param_count layout: 5 per
// material, then 3 per light): every path is replayed in float exactly as
// orc_render traces and shades it (same pools), its vertices are recorded,
// and the path value C = sum_k T_k bl_k col s_k with
// T_{k+1} = clamp1(T_k brdf_k / pdf_k) / q_k is differentiated in double by
// forward-mode dual numbers, one parameter at a time, through
// make_material and the BRDF formulas (directions, pdfs and roulette held
// at their sampled values).  dimg: rows' pixels x 3 (not divided by spp).
int orc_adjoint_f64(void* sp, const gb_camera* cam, const gb_render_desc* d, int row0, int row1, const float* pool,
                    int pool_updates, const float* dimg, int n_sel, const int* sel, double* out, int sampling_terms) {
    const OScene& s = *(const OScene*)sp;
    const int W = d->width, H = d->height, L = d->max_bounces;
    if (row0 < 0 || row1 > H || row0 >= row1) return 1;
    if (pool_updates < d->spp * L) return 2;
    if (cam->aperture != 0.0f && (row0 != 0 || row1 != H)) return 3;
    if (s.sky.light >= 0) return 4;  // the adjoint covers rect lights only
    if (L > kReplayBounces) return 5;
    const int n = W * (row1 - row0), base = row0 * W;
    const int nm = (int)s.mats_in.size();
    CameraRec C = make_camera(*cam, W, H);
    ShadeParams par = make_shade_params(*d);
    for (int j = 0; j < n_sel; ++j) out[j] = 0.0;
    const gb_principled_params* prm = s.params_in.empty() ? nullptr : s.params_in.data();
#pragma omp parallel
    {
        std::vector<double> acc(n_sel, 0.0);
        std::vector<AdjVertex> vs;
#pragma omp for schedule(dynamic, 16)
        for (int i = 0; i < n; ++i) {
            const int id = base + i, x = id % W, y = id / W;
            const v3 g = mk(dimg[3 * i], dimg[3 * i + 1], dimg[3 * i + 2]);
            if (g.x == 0.0f && g.y == 0.0f && g.z == 0.0f) continue;
            for (int p = 0; p < d->spp; ++p) {
                const float* jp = pool + (size_t)p * n * 3;
                float lx = 0.0f, ly = 0.0f;
                if (C.aperture != 0.0f) {
                    int o = (id + 17) % (W * H);
                    lx = jp[3 * o + 2] - 0.5f;
                    ly = jp[3 * o + 1] - 0.5f;
                }
                v3 o, dd;
                camera_ray(C, x, y, jp[3 * i], jp[3 * i + 1], lx, ly, &o, &dd);
                float tmax = FLT_MAX;
                v3 tp = mk(1.0f, 1.0f, 1.0f);
                vs.clear();
                v3 miss_end = mk(0.0f, 0.0f, 0.0f);  // what the path's final miss adds
                for (int b = 0; b < L; ++b) {
                    gb_hit h = trace_closest(s, o, dd, tmax, nullptr, nullptr);
                    if (h.ref == 0xffffffffu) {
                        if (b > 0) miss_end = miss_contribution(tp, dd, par, &s.sky);
                        break;
                    }
                    const float* up = pool + ((size_t)p * L + b) * n * 3;
                    v3 rnd = mk(up[3 * i], up[3 * i + 1], up[3 * i + 2]);
                    v3 lr = rnd;
                    if (d->rng_mode == GB_RNG_HALTON_LIGHT) {
                        float hy = halton(id + 1, 3);
                        lr = mk(halton(id + 1, 2), hy, hy);
                    }
                    v3 P = tri_interp(s.pos, (int)h.ref, h.beta, h.gamma);
                    v3 Nr = tri_interp(s.nrm, (int)h.ref, h.beta, h.gamma);
                    v3 so = mk(0.0f, 0.0f, 0.0f), sd = so, psc = so;
                    float smax = -1.0f, scale = 0.0f;
                    int light = 0;
                    if (!s.lights.empty()) {
                        light = pick_light(s.lights.data(), (int)s.lights.size(), s.overall, lr.z);
                        rect_light_sample(s.lights[light], s.lights[light].col, s.overall, P, Nr, lr.x, lr.y,
                                          d->shadow_offset, &so, &sd, &smax, &psc, &scale);
                    }
                    bool occl = smax < 0.0f || trace_any(s, so, sd, smax);
                    const int mi = s.mat[h.ref];
                    ShadeTrace tr;
                    ShadeOut so2 = shade_hit(s.mats[mi], P, Nr, dd, tp, rnd, !occl, sd, psc, par, (uint32_t)id,
                                             (uint32_t)p, b, nullptr, nullptr, &tr);
                    vs.push_back(AdjVertex{mi, light, tr.lobe, tr.nee, tr.pdf, tr.q, scale, tr.wo, tr.wi, tr.N, tr.ld,
                                           tr.flags});
                    if (!so2.alive || b + 1 >= L) break;
                    tp = so2.tp;
                    o = so2.org;
                    dd = so2.dir;
                    tmax = FLT_MAX;
                }
                const int K = (int)vs.size();
                for (int j = 0; j < n_sel; ++j) {
                    const int pi = sel[j];
                    int pm = -1, pk = -1, pl = -1, pc = -1;
                    if (pi < 5 * nm) { pm = pi / 5; pk = pi % 5; }
                    else { pl = (pi - 5 * nm) / 3; pc = (pi - 5 * nm) % 3; }
                    bool touched = false;
                    for (const AdjVertex& v : vs)
                        if ((pm >= 0 && v.mi == pm) || (pl >= 0 && v.nee && v.light == pl)) touched = true;
                    if (!touched) continue;
                    Dd T[3] = {cst(1.0), cst(1.0), cst(1.0)}, Cc[3] = {cst(0.0), cst(0.0), cst(0.0)};
                    double gnee[kReplayBounces] = {}, sm[kReplayBounces] = {}, sr[kReplayBounces] = {};
                    for (int k = 0; k < K; ++k) {
                        const AdjVertex& v = vs[k];
                        MatD m = make_material_d(s.mats_in[v.mi], prm, v.mi == pm ? pk : -1);
                        float fsm = 0.0f, fsr = 0.0f, fwr = 0.0f;
                        if (sampling_terms && v.mi == pm) {
                            float zlo = 0.0f, zhi = 1.0f;
                            if (d->rng_mode == GB_RNG_MRG32K3A_POOL && !s.lights.empty())
                                light_pick_interval(s.lights.data(), (int)s.lights.size(), s.overall, v.light, &zlo,
                                                    &zhi);
                            sampling_scores(s.mats[v.mi], v.lobe, v.flags, v.wo, v.wi, v.N, v.pdf, zlo, zhi, &fsm,
                                            &fsr, &fwr);
                        }
                        sm[k] = fsm;
                        sr[k] = fsr;
                        if (v.nee) {
                            Dd bl[3];
                            eval_d(m, v.lobe, vd(v.wo), vd(v.ld), vd(v.N), bl);
                            const gb_light& li = s.lights_in[v.light];
                            for (int c = 0; c < 3; ++c) {
                                Dd col{li.col[c], (v.light == pl && c == pc) ? 1.0 : 0.0};
                                Dd term = T[c] * bl[c] * col * cst(v.scale);
                                Cc[c] = Cc[c] + term;
                                gnee[k] += (double)(c == 0 ? g.x : (c == 1 ? g.y : g.z)) * term.v;
                            }
                        }
                        if (k + 1 < K) {
                            Dd br[3];
                            eval_d(m, v.lobe, vd(v.wo), vd(v.wi), vd(v.N), br);
                            // the Walter weight's roughness dependence (sampling terms)
                            const Dd pdf{v.pdf, pk == 3 ? (double)v.pdf * (double)fwr : 0.0};
                            for (int c = 0; c < 3; ++c) {
                                Dd t = T[c] * br[c] / pdf;
                                if (t.v > 1.0) t = cst(1.0);
                                T[c] = t / cst(v.q);
                            }
                        }
                    }
                    double dval = (double)g.x * Cc[0].d + (double)g.y * Cc[1].d + (double)g.z * Cc[2].d;
                    if (sampling_terms && (pk == 3 || pk == 4)) {
                        // scores times the path terms each decision moves
                        double after = (double)g.x * miss_end.x + (double)g.y * miss_end.y + (double)g.z * miss_end.z;
                        for (int k = K - 1; k >= 0; --k) {
                            if (vs[k].mi == pm) dval += pk == 4 ? sm[k] * (gnee[k] + after) : sr[k] * after;
                            after += gnee[k];
                        }
                    }
                    acc[j] += dval / d->spp;
                }
            }
        }
#pragma omp critical
        for (int j = 0; j < n_sel; ++j) out[j] += acc[j];
    }
    return 0;
}

// gpu_area_lights (direct-lighting.cpp:29-104): pixel-centre camera rays,
// first-hit material colour (MTL diffuse colour, background for a miss),
// `samples` GPU-sampler light samples averaged; sample k uses pool update
// max(0, k - 1).  pool: [update][pixel][3], at least max(1, samples - 1)
// updates.  out_rgb: w*h*3.
int orc_render_direct(void* sp, const gb_camera* cam, const gb_render_desc* d, int samples, const float* pool,
                      int pool_updates, float* out_rgb) {
    const OScene& s = *(const OScene*)sp;
    const int W = d->width, H = d->height, n = W * H;
    if (samples <= 0 || pool_updates < std::max(1, samples - 1)) return 1;
    CameraRec C = make_camera(*cam, W, H);
    const v3 bg = mk(d->background[0], d->background[1], d->background[2]);
#pragma omp parallel for schedule(dynamic, 64)
    for (int g = 0; g < n; ++g) {
        v3 o, dd;
        camera_ray(C, g % W, g / W, 0.5f, 0.5f, 0.0f, 0.0f, &o, &dd);
        gb_hit h = trace_closest(s, o, dd, FLT_MAX, nullptr, nullptr);
        const bool hit = h.ref != 0xffffffffu;
        v3 P = mk(0.0f, 0.0f, 0.0f), N = P, mcol = bg;
        if (hit) {
            P = tri_interp(s.pos, (int)h.ref, h.beta, h.gamma);
            N = tri_interp(s.nrm, (int)h.ref, h.beta, h.gamma);
            const MaterialRec& m = s.mats[s.mat[h.ref]];
            mcol = mk(m.kd[0], m.kd[1], m.kd[2]);
            if (s.textured && m.dtex >= 0 && m.dtex < (int)s.tex.size()) {
                // pixel_evaluate_material_bilin_lod_cpu (material-cpu.cpp:36-77)
                const float* p = &s.pos[9 * (size_t)h.ref];
                const float* tcs = &s.tc[6 * (size_t)h.ref];
                float ts, tt;
                bary2(h.beta, h.gamma, tcs, &ts, &tt);
                RayDiff df = camera_diff(C, g % W, g / W);
                const float diff = ray_diff_hit(&df, mk(p[0], p[1], p[2]), mk(p[3], p[4], p[5]), mk(p[6], p[7], p[8]),
                                                tcs, ts, tt, N);
                mcol = mcol * tex_sample_bilin_lod(s.tex[m.dtex], ts, tt, diff);
            }
        }
        v3 buf_dir = dd, acc = mk(0.0f, 0.0f, 0.0f);
        for (int k = 0; k < samples; ++k) {
            const float* up = pool + ((size_t)std::max(0, k - 1) * n + g) * 3;
            const v3 rnd = mk(up[0], up[1], up[2]);
            v3 weight = mk(0.0f, 0.0f, 0.0f);
            bool occluded = false;
            if (hit && !s.lights.empty()) {
                const int l = pick_light(s.lights.data(), (int)s.lights.size(), s.overall, rnd.z);
                const LightRec& L = s.lights[l];
                v3 so, sd;
                float smax;
                if (L.type == 1)
                    sky_light_sample_uniform(s.sky, L.power, s.overall, P, N, rnd.x, rnd.y, d->shadow_offset, &so, &sd,
                                             &smax, &weight);
                else
                    rect_light_sample(L, L.col, s.overall, P, N, rnd.x, rnd.y, d->shadow_offset, &so, &sd, &smax,
                                      &weight, nullptr, false);
                buf_dir = sd;
                occluded = smax >= 0.0f && trace_any(s, so, sd, smax);
            } else {
                if (s.sky.light >= 0) weight = s.sky.scale * sky_eval(s.sky, buf_dir);
                buf_dir = mk(0.0f, 0.0f, 0.0f);
            }
            const v3 mat = occluded ? mk(0.0f, 0.0f, 0.0f) : mcol;
            acc = (float(k) * acc + weight * mat) / (float(k) + 1.0f);
        }
        out_rgb[3 * (size_t)g] = acc.x;
        out_rgb[3 * (size_t)g + 1] = acc.y;
        out_rgb[3 * (size_t)g + 2] = acc.z;
    }
    return 0;
}

// hybrid_area_lights (direct-lighting.cpp:203-316, direct-lighting.h:137-215)
// on pools [update][pixel][3]: camera sample c takes jitter update c (and the
// lens jitter of pixel (g + 17) mod n, update c), light sample j of camera
// sample c takes update c*L + max(0, j-1); needs max(C, C*L) updates.
int orc_render_hybrid_direct(void* sp, const gb_camera* cam, const gb_render_desc* d, int cam_samples,
                             int light_samples, const float* pool, int pool_updates, float* out_rgb) {
    const OScene& s = *(const OScene*)sp;
    const int W = d->width, H = d->height, n = W * H, L = light_samples;
    if (cam_samples <= 0 || L <= 0 || pool_updates < std::max(cam_samples, cam_samples * L)) return 1;
    CameraRec C = make_camera(*cam, W, H);
    const v3 bg = mk(d->background[0], d->background[1], d->background[2]);
#pragma omp parallel for schedule(dynamic, 64)
    for (int g = 0; g < n; ++g) {
        const int x = g % W, y = g / W;
        v3 acc = mk(0.0f, 0.0f, 0.0f);
        for (int c = 0; c < cam_samples; ++c) {
            const float* jp = pool + ((size_t)c * n + g) * 3;
            float lx = 0.0f, ly = 0.0f;
            if (C.aperture != 0.0f) {
                const float* lp = pool + ((size_t)c * n + (g + 17) % n) * 3;
                lx = lp[2] - 0.5f;
                ly = lp[1] - 0.5f;
            }
            v3 o, dd;
            camera_ray(C, x, y, jp[0], jp[1], lx, ly, &o, &dd);
            gb_hit h = trace_closest(s, o, dd, FLT_MAX, nullptr, nullptr);
            const bool hit = h.ref != 0xffffffffu;
            v3 mcol = bg;
            if (hit) {
                const v3 N = tri_interp(s.nrm, (int)h.ref, h.beta, h.gamma);
                const MaterialRec& m = s.mats[s.mat[h.ref]];
                mcol = mk(m.kd[0], m.kd[1], m.kd[2]);
                if (s.textured && m.dtex >= 0 && m.dtex < (int)s.tex.size()) {
                    const float* p = &s.pos[9 * (size_t)h.ref];
                    const float* tcs = &s.tc[6 * (size_t)h.ref];
                    float ts, tt;
                    bary2(h.beta, h.gamma, tcs, &ts, &tt);
                    RayDiff df = camera_diff(C, x, y);
                    const float diff = ray_diff_hit(&df, mk(p[0], p[1], p[2]), mk(p[3], p[4], p[5]),
                                                    mk(p[6], p[7], p[8]), tcs, ts, tt, N);
                    mcol = mcol * tex_sample_bilin_lod(s.tex[m.dtex], ts, tt, diff);
                }
            }
            v3 buf_dir = dd;
            for (int j = 0; j < L; ++j) {
                const float* up = pool + ((size_t)(c * L + std::max(0, j - 1)) * n + g) * 3;
                v3 so, sd = buf_dir, psc;
                float smax;
                nee_pixel(s, g, h, mk(up[0], up[1], up[2]), d->shadow_offset, &so, &sd, &smax, &psc);
                buf_dir = sd;
                const bool occluded = hit && !s.lights.empty() && smax >= 0.0f && trace_any(s, so, sd, smax);
                const v3 mat = occluded ? mk(0.0f, 0.0f, 0.0f) : mcol;
                const float sc = float(c * L + j);
                acc = (sc * acc + psc * mat) / (sc + 1.0f);
            }
        }
        out_rgb[3 * (size_t)g] = acc.x;
        out_rgb[3 * (size_t)g + 1] = acc.y;
        out_rgb[3 * (size_t)g + 2] = acc.z;
    }
    return 0;
}

// Halton pool of util.cpp:38-51 for pixels [0, n): (h2(i+1), h3(i+1)).
int orc_halton_pool(int n, float* out) {
    for (int i = 0; i < n; ++i) { out[2 * i] = halton(i + 1, 2); out[2 * i + 1] = halton(i + 1, 3); }
    return 0;
}

// Exposed per-ray functions for the pinning tests against the reference's
// own BRDF / light code.
int orc_material_sample_eval(const gb_material* mat, const gb_principled_params* params, const float* wo_ts,
                             const float* rnd, const float* N, const float* wo_world, const float* wi_eval,
                             float* wi_out, float* pdf_out, int* lobe_out, float* f_sampled, float* f_eval) {
    float f[kMaterialFloats];
    pack_material(make_material(*mat, params), f);
    MaterialRec m = unpack_material(f);
    v3 wi; float pdf; int lobe;
    material_sample(m, mk(wo_ts[0], wo_ts[1], wo_ts[2]), mk(rnd[0], rnd[1], rnd[2]), &wi, &pdf, &lobe);
    wi_out[0] = wi.x; wi_out[1] = wi.y; wi_out[2] = wi.z;
    *pdf_out = pdf; *lobe_out = lobe;
    v3 n = mk(N[0], N[1], N[2]), wo = mk(wo_world[0], wo_world[1], wo_world[2]);
    v3 fs = material_eval(m, lobe, wo, wi, n);
    v3 fe = material_eval(m, lobe, wo, mk(wi_eval[0], wi_eval[1], wi_eval[2]), n);
    f_sampled[0] = fs.x; f_sampled[1] = fs.y; f_sampled[2] = fs.z;
    f_eval[0] = fe.x; f_eval[1] = fe.y; f_eval[2] = fe.z;
    return 0;
}

// sample_bsdf + the two evaluations of evaluate_material, for the pinning
// tests against the reference's own materialBRDF (same outputs as
// ref_shade_eval in oracle/ref_glue.cpp): out[0..2] wi, [3] pdf, [4..6]
// brdf(wi), [7..9] brdf(to_light), [10] glass.
int orc_shade_eval(const gb_material* mat, const gb_principled_params* params, const float* n_raw,
                   const float* ray_dir, const float* rnd, const float* to_light, float* out) {
    float f[kMaterialFloats];
    pack_material(make_material(*mat, params), f);
    MaterialRec m = unpack_material(f);
    BsdfSample s = sample_bsdf(m, mk(n_raw[0], n_raw[1], n_raw[2]), mk(ray_dir[0], ray_dir[1], ray_dir[2]),
                               mk(rnd[0], rnd[1], rnd[2]));
    v3 ld = normalize_div(mk(to_light[0], to_light[1], to_light[2]));
    v3 fw = material_eval(m, s.lobe, s.inv_org_dir, s.wi, s.N);
    v3 fl = material_eval(m, s.lobe, s.inv_org_dir, ld, s.N);
    out[0] = s.wi.x; out[1] = s.wi.y; out[2] = s.wi.z;
    out[3] = s.pdf;
    out[4] = fw.x; out[5] = fw.y; out[6] = fw.z;
    out[7] = fl.x; out[8] = fl.y; out[9] = fl.z;
    out[10] = s.glass ? 1.0f : 0.0f;
    return 0;
}

int orc_sincos_2pi(int n, const float* u, float* s, float* c) {
    for (int i = 0; i < n; ++i) sincos_2pi(u[i], &s[i], &c[i]);
    return 0;
}

// MRG32k3a jump of `steps` generator steps (mrg_jump_matrices + mrg_jump of
// the library's shared headers) applied to s1[3], s2[3] in place.
int orc_mrg_jump(unsigned long long steps, uint32_t* s1, uint32_t* s2) {
    uint32_t J1[9], J2[9];
    mrg_jump_matrices(steps, J1, J2);
    mrg_jump(s1, s2, J1, J2);
    return 0;
}

// The shared atan2 / acos (sky texel lookup) for accuracy tests.
int orc_atan2_acos(int n, const float* y, const float* x, float* atan2_out, float* acos_out) {
    for (int i = 0; i < n; ++i) {
        atan2_out[i] = atan2_ex(y[i], x[i]);
        acos_out[i] = acos_ex(x[i]);
    }
    return 0;
}

// Distribution1D::init + sample on the host tables (sky sampling tests).
int orc_dist1d(int n, const float* data, int m, const float* u, float* x, float* p) {
    std::vector<float> pdf(n), cdf(n + 1);
    dist1d_init(data, n, pdf.data(), cdf.data());
    for (int i = 0; i < m; ++i) dist1d_sample(cdf.data(), pdf.data(), n, u[i], &x[i], &p[i]);
    return 0;
}

// Texture helpers for the known-answer tests: the mip chain of make_mipmaps
// (out must hold 4 * (total + w + 1) bytes; returns the texel count in
// *size), sample_bilin_lod of n points, and pow22.
int orc_mipmaps(const uint8_t* rgba, int w, int h, uint8_t* out, long long cap_bytes, int* max_mm, int* size) {
    std::vector<uint8_t> v;
    make_mipmaps(rgba, w, h, &v, max_mm, size);
    if ((long long)v.size() > cap_bytes) return 1;
    std::memcpy(out, v.data(), v.size());
    return 0;
}
int orc_tex_sample(const uint8_t* rgba, int w, int h, int n, const float* sc, const float* tc, const float* diff,
                   float* out) {
    std::vector<uint8_t> v;
    TexRec t;
    make_mipmaps(rgba, w, h, &v, &t.max_mm, &t.size);
    t.texels = v.data();
    t.w = w;
    t.h = h;
    for (int i = 0; i < n; ++i) {
        v3 c = tex_sample_bilin_lod(t, sc[i], tc[i], diff[i]);
        out[3 * i] = c.x; out[3 * i + 1] = c.y; out[3 * i + 2] = c.z;
    }
    return 0;
}
int orc_pow22(int n, const double* x, double* out) {
    for (int i = 0; i < n; ++i) out[i] = pow22(x[i]);
    return 0;
}

int orc_threads(void) { return omp_get_max_threads(); }
void orc_set_threads(int n) { if (n > 0) omp_set_num_threads(n); }

}  // extern "C"
