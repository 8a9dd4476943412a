// fp64_render.cpp -- TEST INFRASTRUCTURE ONLY (CPU, C++17 + OpenMP).
//
// An independent double-precision restatement of the reference's hybrid
// path tracer.  It renders the converged high-spp image against which the
// RMSE of every GPU frame is stated, and it checks the expectation of the
// float path (gbpt_oracle.cpp and the kernels) without sharing their code:
// it has its own binned-SAH binary BVH and traversal in double, its own
// counter-based random numbers, and every per-path formula is re-derived
// from the reference sources:
//   camera            raygen.cu:61-118 (jittered Shirley camera, thin lens)
//   light pick        arealight-sampler-cpu.cpp:30-39 (stops at the last light)
//   rect light sample arealight-sampler-cpu.cpp:40-86, :114-119
//   shading / bounce  hybrid-pt.cpp:330-371 (sample / evaluate),
//                     :421-448 (hit data), :450-575 (NEE, next ray, clamp,
//                     misses), :196-206 (handle_no_hit)
//   BRDFs             principledMaterial.h:21-390, simpleMaterial.h:82-113,
//                     materialBase.h:16-24
//   light power       lights.cpp:92
//   Halton            util.cpp:22-51, util.h:120-123
// The helpers of the absent rta / libhyb libraries follow the conventions
// the library defines for them: make_tangent_frame is the orthonormal basis
// of Duff et al. 2017, make_tangential(v, n) maps a z-up vector into that
// frame, reflect(v, n) = v - 2 (v.n) n, barycentrics are (1-b-g, b, g), the
// triangle test is double-sided with t > 0.  The library's deviations are
// kept: the light pick stops at the last light, a path whose BRDF pdf is 0
// or whose throughput is NaN ends, a NaN light-sample term is dropped.  The
// Russian-roulette extension follows the library's rule (from bounce
// rr_start on, survival q = clamp(max channel of the clamped throughput,
// 0.05, 1), throughput / q) with its own uniform draws.  Sky lights and
// textures are not covered (rect lights, untextured materials).
//
// Sample streams keep the reference's structure with another generator:
// pixel i owns a sequence of uniform triplets U(i, k) in (0, 1]; path p's
// camera jitter is U(i, p), its lens sample U((i + 17) mod n, p), bounce b
// draws U(i, p L + b) for the light sample and the BRDF sample alike (the
// reference's identically seeded light and path pools,
// hybrid-pt.cpp:83-95); the Halton light mode uses (h2(i+1), h3(i+1),
// h3(i+1)) for every light sample of pixel i.
#include <omp.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../include/gbpt.h"

namespace {

struct d3 {
    double x, y, z;
};
inline d3 D(double x, double y, double z) { return d3{x, y, z}; }
inline d3 operator+(d3 a, d3 b) { return D(a.x + b.x, a.y + b.y, a.z + b.z); }
inline d3 operator-(d3 a, d3 b) { return D(a.x - b.x, a.y - b.y, a.z - b.z); }
inline d3 operator-(d3 a) { return D(-a.x, -a.y, -a.z); }
inline d3 operator*(d3 a, d3 b) { return D(a.x * b.x, a.y * b.y, a.z * b.z); }
inline d3 operator*(double s, d3 a) { return D(s * a.x, s * a.y, s * a.z); }
inline d3 operator*(d3 a, double s) { return D(a.x * s, a.y * s, a.z * s); }
inline d3 operator/(d3 a, double s) { return D(a.x / s, a.y / s, a.z / s); }
inline double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline d3 cross(d3 a, d3 b) { return D(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline double len(d3 a) { return std::sqrt(dot(a, a)); }
inline d3 unit(d3 a) { return a / len(a); }
inline bool any_nan(d3 a) { return std::isnan(a.x) || std::isnan(a.y) || std::isnan(a.z); }
inline double comp(d3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }
inline d3 from3(const float* p) { return D(p[0], p[1], p[2]); }

const double kPi = 3.14159265358979323846;

// ------------------------------------------------------------ random draws
// SplitMix64 finaliser over a key built from (seed, pixel, counter, lane);
// the top 53 bits give a double in (0, 1], the range curand_uniform has.
inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline double unit01(uint64_t seed, uint64_t pixel, uint64_t k, uint64_t lane) {
    uint64_t h = mix64(seed * 0x9E3779B97F4A7C15ull ^ mix64(pixel + 0x632BE59BD9B4E019ull) ^
                       mix64((k << 2 | lane) * 0xD1B54A32D192ED03ull + 0x8CB92BA72F3D8DD7ull));
    return (double)((h >> 11) + 1) * (1.0 / 9007199254740992.0);
}
inline d3 U3(uint64_t seed, uint64_t pixel, uint64_t k) {
    return D(unit01(seed, pixel, k, 0), unit01(seed, pixel, k, 1), unit01(seed, pixel, k, 2));
}

// radical inverse of util.cpp:22-32
double halton(int index, int base) {
    double r = 0.0, f = 1.0 / base;
    for (int i = index; i > 0; i /= base) {
        r += f * (i % base);
        f /= base;
    }
    return r;
}

// ------------------------------------------------------------ helpers
// orthonormal basis around a unit n (Duff et al. 2017)
inline void tangent_frame(d3 n, d3* T, d3* B) {
    const double s = std::copysign(1.0, n.z);
    const double a = -1.0 / (s + n.z);
    const double b = n.x * n.y * a;
    *T = D(1.0 + s * n.x * n.x * a, s * b, -s * n.x);
    *B = D(b, s + n.y * n.y * a, -n.y);
}
inline d3 tangential(d3 v, d3 n) {
    d3 T, B;
    tangent_frame(n, &T, &B);
    return v.x * T + v.y * B + v.z * n;
}
inline d3 reflect_v(d3 v, d3 n) { return v - 2.0 * dot(v, n) * n; }

// ------------------------------------------------------------ scene
struct Mat {
    bool principled = false;
    d3 color{0, 0, 0};  // Lambert diffuse_color, or PrincipledBRDFParameters::color
    double metallic = 0, subsurface = 0, specular = 0, roughness = 0, specular_tint = 0, anisotropic = 0;
    double sheen = 0, sheen_tint = 0, clearcoat = 0, clearcoat_gloss = 0, opacity = 1;
};

struct Light {
    d3 center, dir, col;
    double w, h, power;
};

struct Node {
    double lo[3], hi[3];
    int first;  // leaf: first triangle of `order`; inner: left child (right = first + 1)
    int count;  // > 0: leaf
};

// Trees deeper than this are refused at creation, so the traversal stack
// (at most depth + 1 entries) cannot overflow.
constexpr int kMaxDepth = 120;

struct Scene {
    int n = 0;
    std::vector<d3> a, b, c, na, nb, nc;
    std::vector<int> mat;
    std::vector<Mat> mats;
    std::vector<Light> lights;
    double overall = 0.0;
    std::vector<Node> nodes;
    std::vector<int> order;
};

// Binned-SAH build (16 bins over the centroid bounds of each node).
struct Builder {
    Scene& s;
    std::vector<double> lo, hi, cen;  // 3 per triangle
    explicit Builder(Scene& sc) : s(sc) {}

    void box(int first, int count, double* blo, double* bhi) const {
        for (int k = 0; k < 3; ++k) { blo[k] = DBL_MAX; bhi[k] = -DBL_MAX; }
        for (int i = first; i < first + count; ++i) {
            const int t = s.order[i];
            for (int k = 0; k < 3; ++k) {
                blo[k] = std::min(blo[k], lo[3 * t + k]);
                bhi[k] = std::max(bhi[k], hi[3 * t + k]);
            }
        }
    }
    static double area(const double* l, const double* h) {
        const double dx = h[0] - l[0], dy = h[1] - l[1], dz = h[2] - l[2];
        return dx < 0 ? 0.0 : 2.0 * (dx * dy + dy * dz + dz * dx);
    }

    void build() {
        const int n = s.n;
        lo.resize(3 * (size_t)n);
        hi.resize(3 * (size_t)n);
        cen.resize(3 * (size_t)n);
        s.order.resize(n);
        for (int t = 0; t < n; ++t) {
            s.order[t] = t;
            for (int k = 0; k < 3; ++k) {
                const double va = comp(s.a[t], k), vb = comp(s.b[t], k), vc = comp(s.c[t], k);
                lo[3 * t + k] = std::min(va, std::min(vb, vc));
                hi[3 * t + k] = std::max(va, std::max(vb, vc));
                cen[3 * t + k] = 0.5 * (lo[3 * t + k] + hi[3 * t + k]);
            }
        }
        s.nodes.reserve(2 * (size_t)std::max(n, 1));
        s.nodes.push_back(Node{});
        split(0, 0, n);
        // pad every box by a margin far above double rounding of the slab test
        double ext = 0.0;
        for (int k = 0; k < 3; ++k) ext = std::max(ext, s.nodes[0].hi[k] - s.nodes[0].lo[k]);
        const double pad = 1e-9 * std::max(ext, 1.0);
        for (Node& nd : s.nodes)
            for (int k = 0; k < 3; ++k) { nd.lo[k] -= pad; nd.hi[k] += pad; }
    }

    int max_depth = 0;

    void split(int ni, int first, int count, int depth = 0) {
        max_depth = std::max(max_depth, depth);
        double blo[3], bhi[3];
        box(first, count, blo, bhi);
        for (int k = 0; k < 3; ++k) { s.nodes[ni].lo[k] = blo[k]; s.nodes[ni].hi[k] = bhi[k]; }
        s.nodes[ni].first = first;
        s.nodes[ni].count = count;
        if (count <= 2) return;
        double clo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, chi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
        for (int i = first; i < first + count; ++i)
            for (int k = 0; k < 3; ++k) {
                clo[k] = std::min(clo[k], cen[3 * s.order[i] + k]);
                chi[k] = std::max(chi[k], cen[3 * s.order[i] + k]);
            }
        constexpr int kBins = 16;
        double best = DBL_MAX;
        int best_axis = -1, best_bin = 0;
        for (int ax = 0; ax < 3; ++ax) {
            const double ext = chi[ax] - clo[ax];
            if (!(ext > 0.0)) continue;
            int cnt[kBins] = {};
            double bl[kBins][3], bh[kBins][3];
            for (int b = 0; b < kBins; ++b)
                for (int k = 0; k < 3; ++k) { bl[b][k] = DBL_MAX; bh[b][k] = -DBL_MAX; }
            for (int i = first; i < first + count; ++i) {
                const int t = s.order[i];
                int b = (int)((cen[3 * t + ax] - clo[ax]) / ext * kBins);
                b = std::min(std::max(b, 0), kBins - 1);
                ++cnt[b];
                for (int k = 0; k < 3; ++k) {
                    bl[b][k] = std::min(bl[b][k], lo[3 * t + k]);
                    bh[b][k] = std::max(bh[b][k], hi[3 * t + k]);
                }
            }
            double rl[kBins][3], rh[kBins][3];
            int rc[kBins];
            double al[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, ah[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
            int acc = 0;
            for (int b = kBins - 1; b >= 0; --b) {
                acc += cnt[b];
                for (int k = 0; k < 3; ++k) { al[k] = std::min(al[k], bl[b][k]); ah[k] = std::max(ah[k], bh[b][k]); }
                rc[b] = acc;
                for (int k = 0; k < 3; ++k) { rl[b][k] = al[k]; rh[b][k] = ah[k]; }
            }
            double ll[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, lh[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
            int lc = 0;
            for (int b = 0; b < kBins - 1; ++b) {
                lc += cnt[b];
                for (int k = 0; k < 3; ++k) { ll[k] = std::min(ll[k], bl[b][k]); lh[k] = std::max(lh[k], bh[b][k]); }
                if (lc == 0 || rc[b + 1] == 0) continue;
                const double cost = lc * area(ll, lh) + rc[b + 1] * area(rl[b + 1], rh[b + 1]);
                if (cost < best) { best = cost; best_axis = ax; best_bin = b; }
            }
        }
        const double leaf_cost = count * area(blo, bhi);
        if (best_axis < 0 || (count <= 4 && best >= leaf_cost)) return;
        const double ext = chi[best_axis] - clo[best_axis];
        int* beg = s.order.data() + first;
        int* mid = std::partition(beg, beg + count, [&](int t) {
            int b = (int)((cen[3 * t + best_axis] - clo[best_axis]) / ext * kBins);
            return std::min(std::max(b, 0), kBins - 1) <= best_bin;
        });
        const int nl = (int)(mid - beg);
        if (nl == 0 || nl == count) return;
        const int left = (int)s.nodes.size();
        s.nodes.push_back(Node{});
        s.nodes.push_back(Node{});
        s.nodes[ni].first = left;
        s.nodes[ni].count = 0;
        split(left, first, nl, depth + 1);
        split(left + 1, first + nl, count - nl, depth + 1);
    }
};

// ------------------------------------------------------------ traversal
struct Ray {
    d3 o, d, inv;
    int neg[3];
};
inline Ray make_ray(d3 o, d3 d) {
    Ray r;
    r.o = o;
    r.d = d;
    for (int k = 0; k < 3; ++k) {
        const double dk = comp(d, k);
        const double iv = dk != 0.0 ? 1.0 / dk : (std::signbit(dk) ? -INFINITY : INFINITY);
        (k == 0 ? r.inv.x : (k == 1 ? r.inv.y : r.inv.z)) = iv;
        r.neg[k] = iv < 0.0;
    }
    return r;
}

// entry distance of the ray into the node's box within (0, tmax], or -1
inline double box_enter(const Node& n, const Ray& r, double tmax) {
    double t0 = 0.0, t1 = tmax;
    for (int k = 0; k < 3; ++k) {
        const double o = comp(r.o, k), iv = comp(r.inv, k);
        if (std::isinf(iv)) {  // parallel to the slabs of this axis
            if (o < n.lo[k] || o > n.hi[k]) return -1.0;
            continue;
        }
        double a = (n.lo[k] - o) * iv, b = (n.hi[k] - o) * iv;
        if (a > b) std::swap(a, b);
        t0 = std::max(t0, a);
        t1 = std::min(t1, b);
        if (t0 > t1) return -1.0;
    }
    return t0;
}

// double-sided Moller-Trumbore, t in (0, tmax]
inline bool tri_hit(const Scene& s, int t, const Ray& r, double tmax, double* tt, double* bb, double* gg) {
    const d3 e1 = s.b[t] - s.a[t], e2 = s.c[t] - s.a[t];
    const d3 p = cross(r.d, e2);
    const double det = dot(e1, p);
    if (det == 0.0 || std::isnan(det)) return false;
    const double inv = 1.0 / det;
    const d3 q0 = r.o - s.a[t];
    const double u = dot(q0, p) * inv;
    if (u < 0.0 || u > 1.0) return false;
    const d3 q = cross(q0, e1);
    const double v = dot(r.d, q) * inv;
    if (v < 0.0 || u + v > 1.0) return false;
    const double th = dot(e2, q) * inv;
    if (!(th > 0.0) || th > tmax) return false;
    *tt = th;
    *bb = u;
    *gg = v;
    return true;
}

struct Hit {
    int id = -1;
    double t = 0, beta = 0, gamma = 0;
};

// Ties: hits whose distances differ by at most kTie * t count as equally
// near, and the lower triangle id wins -- the library's closest-hit rule
// (the (t, id) minimum), which decides e.g. between a floor and the
// coplanar bottom face of a box standing on it.
constexpr double kTie = 1e-9;

// closest hit (any = false) or any hit within (0, tmax]
Hit trace(const Scene& s, const Ray& r, double tmax, bool any) {
    Hit h;
    double bound = tmax;  // farthest distance still worth visiting
    if (s.nodes.empty()) return h;
    int stack[kMaxDepth + 2];  // one entry per level plus the current node's sibling
    int sp = 0;
    if (box_enter(s.nodes[0], r, bound) < 0.0) return h;
    stack[sp++] = 0;
    while (sp > 0) {
        const Node& n = s.nodes[stack[--sp]];
        if (box_enter(n, r, bound) < 0.0) continue;
        if (n.count > 0) {
            for (int i = n.first; i < n.first + n.count; ++i) {
                const int t = s.order[i];
                double tt, bb, gg;
                if (!tri_hit(s, t, r, std::min(bound, tmax), &tt, &bb, &gg)) continue;
                if (any) {
                    h.id = t; h.t = tt; h.beta = bb; h.gamma = gg;
                    return h;
                }
                const bool nearer = h.id < 0 || tt < h.t * (1.0 - kTie) ||
                                    (tt <= h.t * (1.0 + kTie) && t < h.id);
                if (nearer) {
                    h.id = t; h.t = tt; h.beta = bb; h.gamma = gg;
                    bound = tt * (1.0 + kTie);
                }
            }
            continue;
        }
        const double tl = box_enter(s.nodes[n.first], r, bound), tr = box_enter(s.nodes[n.first + 1], r, bound);
        if (tl >= 0.0 && tr >= 0.0) {
            // nearer child on top
            if (tl <= tr) { stack[sp++] = n.first + 1; stack[sp++] = n.first; }
            else { stack[sp++] = n.first; stack[sp++] = n.first + 1; }
        } else if (tl >= 0.0) {
            stack[sp++] = n.first;
        } else if (tr >= 0.0) {
            stack[sp++] = n.first + 1;
        }
    }
    return h;
}

// ------------------------------------------------------------ BRDFs
enum Lobe { DIFFUSE = 0, DISNEY_REFLECTION = 1, SPECULAR_REFLECTION = 2, SPECULAR_TRANSMISSION = 3 };

inline double saturate(double a) { return std::min(std::max(a, 0.0), 1.0); }
inline double schlick(double u) {
    const double m = saturate(1.0 - u);
    return m * m * m * m * m;
}
inline double mixd(double x, double y, double s) { return (1.0 - s) * x + s * y; }
inline d3 mix3(d3 x, d3 y, double s) { return (1.0 - s) * x + s * y; }
inline d3 mon2lin(d3 c) { return D(std::pow(c.x, 2.2), std::pow(c.y, 2.2), std::pow(c.z, 2.2)); }
inline double smith_ggx(double ndv, double ag) {
    const double a = ag * ag, b = ndv * ndv;
    return 1.0 / (ndv + std::sqrt(a + b - a * b));
}
inline double gtr1(double ndh, double a) {
    if (a >= 1.0) return 1.0 / kPi;
    const double a2 = a * a, t = 1.0 + (a2 - 1.0) * ndh * ndh;
    return (a2 - 1.0) / (kPi * std::log(a2) * t);
}

// evaluatePrincipledBRDF_specular (principledMaterial.h:210-252), N dot L included
d3 principled_specular(const Mat& m, d3 wo, d3 N, d3 wi) {
    const double ndl = dot(N, wi), ndv = dot(N, wo);
    if (ndl < 0.0 || ndv < 0.0) return D(0, 0, 0);
    const d3 H = unit(wi + wo);
    const double ndh = dot(N, H), ldh = dot(wi, H);
    const d3 cd = mon2lin(m.color);
    const double lum = .3 * cd.x + .6 * cd.y + .1 * cd.z;
    const d3 white = D(1, 1, 1);
    const d3 tint = lum > 0.0 ? cd / lum : white;
    const d3 spec0 = mix3(m.specular * .08 * mix3(white, tint, m.specular_tint), cd, m.metallic);
    const double fh = schlick(ldh);
    const d3 fs = mix3(spec0, white, fh);
    double cg = 0.0;
    if (m.clearcoat > 0.0) {
        const double dr = gtr1(ndh, mixd(.1, .001, m.clearcoat_gloss));
        const double fr = mixd(0.04, 1.0, fh);
        const double gr = smith_ggx(ndl, 0.25) * smith_ggx(ndv, 0.25);
        cg = 0.25 * m.clearcoat * gr * fr * dr;
    }
    return (fs + D(cg, cg, cg)) * ndl * m.metallic;
}

// evaluatePrincipledBRDF_diffuse (principledMaterial.h:254-301), N dot L included
d3 principled_diffuse(const Mat& m, d3 wo, d3 N, d3 wi) {
    const double ndl = dot(N, wi), ndv = dot(N, wo);
    if (ndl < 0.0 || ndv < 0.0) return D(0, 0, 0);
    const d3 H = unit(wi + wo);
    const double ldh = dot(wi, H);
    const d3 cd = mon2lin(m.color);
    const double lum = .3 * cd.x + .6 * cd.y + .1 * cd.z;
    const d3 white = D(1, 1, 1);
    const d3 tint = lum > 0.0 ? cd / lum : white;
    const d3 csheen = mix3(white, tint, m.sheen_tint);
    const double fl = schlick(ndl), fv = schlick(ndv);
    const double fd90 = 0.5 + 2.0 * ldh * ldh * m.roughness;
    const double fd = mixd(1.0, fd90, fl) * mixd(1.0, fd90, fv);
    const double fh = schlick(ldh);
    const d3 fsheen = fh * m.sheen * csheen;
    const double fss90 = ldh * ldh * m.roughness;
    const double fss = mixd(1.0, fss90, fl) * mixd(1.0, fss90, fv);
    const double ss = 1.25 * (fss * (1.0 / (ndl + ndv) - .5) + .5);
    return ((1.0 / kPi) * mixd(fd, ss, m.subsurface) * cd + fsheen) * (1.0 - m.metallic) * ndl;
}

// materialBRDF::evaluate (material-wrapper.h:33-37) with the lobe sample() chose
d3 brdf_eval(const Mat& m, int lobe, d3 wo, d3 wi, d3 N) {
    if (!m.principled) return m.color * (1.0 / kPi) * std::fabs(dot(wi, N));
    if (lobe == DISNEY_REFLECTION) return principled_specular(m, wo, N, wi);
    if (lobe == SPECULAR_REFLECTION) return D(1, 1, 1);
    if (lobe == SPECULAR_TRANSMISSION) return D(1, 1, 1) * (1.0 / std::fabs(dot(wi, N)));
    return principled_diffuse(m, wo, N, wi);
}

inline d3 cosine_hemisphere(double u, double v) {
    const double r = std::sqrt(u), phi = 2.0 * kPi * v;
    return D(r * std::cos(phi), r * std::sin(phi), std::sqrt(std::max(0.0, 1.0 - u)));
}

// G1 of Walter et al. (principledMaterial.h:75-79)
inline double walter_g1(d3 v, d3 m, d3 n, double a2, double tan_v) {
    const double fac = (dot(v, m) / dot(v, n)) > 0.0 ? 1.0 : 0.0;
    return fac * 2.0 / (1.0 + std::sqrt(1.0 + a2 * tan_v * tan_v));
}

// materialBRDF::sample in tangent space (wo = the inverted ray direction):
// the direction, its "pdf" and the lobe evaluate() will use.
void brdf_sample(const Mat& m, d3 wo, d3 rnd, d3* wi, double* pdf, int* lobe) {
    if (!m.principled) {  // LambertianMaterial::sample
        *wi = cosine_hemisphere(rnd.x, rnd.y);
        *pdf = std::fabs(wi->z) / kPi;
        *lobe = DIFFUSE;
        return;
    }
    const d3 n = D(0, 0, 1);
    if (m.opacity < 1.0) {  // sampleGlass, ior 1.9 (principledMaterial.h:86-118)
        const double ior = 1.9, c = dot(n, wo);
        const double fres = schlick(c);
        *pdf = 1.0;
        if (rnd.x > fres) {
            *wi = -wo;
            *lobe = SPECULAR_REFLECTION;
            return;
        }
        const double ti = 1.0 + ior * (c * c - 1.0);
        if (ti <= 0.0) {
            *wi = reflect_v(wo, n);
            *lobe = SPECULAR_REFLECTION;
            return;
        }
        const double sg = dot(wo, n) > 0.0 ? 1.0 : -1.0;
        *wi = (ior * c - sg * std::sqrt(ti)) * n - ior * wo;
        *lobe = SPECULAR_TRANSMISSION;
        return;
    }
    if (rnd.z < m.metallic) {  // GTR2-aniso half vector + Walter weight (:121-176, :304-310)
        const double aspect = std::sqrt(1.0 - m.anisotropic * .9);
        const double r2 = m.roughness * m.roughness;
        const double ax = std::max(.001, r2 / aspect), ay = std::max(.001, r2 * aspect);
        const double sn = std::sin(2.0 * kPi * rnd.x), cs = std::cos(2.0 * kPi * rnd.x);
        const double fac = std::sqrt(rnd.y / (1.0 - rnd.y));
        const d3 h = unit(fac * D(ax * cs, ay * sn, 0.0) + n);
        d3 L = wo - 2.0 * dot(wo, h) * h;  // reflectR(V, m)
        if (dot(L, n) < 0.0) L = -L;
        const double rg = (ax * ay * .5 + .5) * (ax * ay * .5 + .5);
        const double dlm = dot(L, h), dvm = dot(wo, h);
        const double tl = std::sqrt(1.0 - dlm * dlm) / dlm, tv = std::sqrt(1.0 - dvm * dvm) / dvm;
        const double gs = walter_g1(L, h, n, rg * rg, tl) * walter_g1(wo, h, n, rg * rg, tv);
        double w = (std::fabs(dot(L, h)) * gs) / (std::fabs(dot(L, n)) * std::fabs(dot(n, h)));
        if (w < 0.01) w = 0.01;
        if (w == 0.0 || std::isnan(w)) {  // diffuse fallback (principledMaterial.h:374-378)
            *wi = cosine_hemisphere(rnd.x, rnd.y);
            *pdf = std::max(wi->z, 0.0) / kPi;
            *lobe = DIFFUSE;
            return;
        }
        *wi = L;
        *pdf = w;
        *lobe = DISNEY_REFLECTION;
        return;
    }
    *wi = cosine_hemisphere(rnd.x, rnd.y);
    *pdf = std::max(wi->z, 0.0) * (1.0 / kPi);
    *lobe = DIFFUSE;
}

// ------------------------------------------------------------ one path
struct Cam {
    d3 pos, view, U, V, W;
    double width, height, aperture, focus;
    int w, h;
};

Cam make_cam(const gb_camera& c, int w, int h) {
    Cam r;
    r.pos = from3(c.pos);
    r.view = from3(c.dir);
    const d3 up = from3(c.up);
    r.W = r.view / len(r.view);
    const d3 txw = cross(up, r.W);
    r.U = txw / len(txw);
    r.V = cross(r.W, r.U);
    r.height = std::tan(kPi * ((double)c.fovy_deg / 2.0) / 180.0);
    r.width = (double)w / (double)h * r.height;
    r.aperture = c.aperture;
    r.focus = c.focus_distance;
    r.w = w;
    r.h = h;
    return r;
}

struct Params {
    int L, rr_start, halton;
    double ray_offset, shadow_offset;
    d3 background;
    uint64_t seed;
};

// One path sample of pixel `id` (path index p): its radiance.
d3 path_sample(const Scene& s, const Cam& C, const Params& P, int id, int p) {
    const int npx = C.w * C.h;
    const int x = id % C.w, y = id / C.w;
    // camera (raygen.cu:61-118)
    const d3 j = U3(P.seed, (uint64_t)id, (uint64_t)p);
    const double us = ((x + j.x) / C.w * 2.0 - 1.0) * C.width;
    const double vs = ((y + j.y) / C.h * 2.0 - 1.0) * C.height;
    d3 dir = unit(C.U * us + C.V * vs + C.W);
    d3 org = C.pos;
    if (C.aperture != 0.0) {
        const d3 lj = U3(P.seed, (uint64_t)((id + 17) % npx), (uint64_t)p);
        const d3 focal = C.pos + dir * (1.0 / dot(dir, C.view)) * C.focus;
        org = C.pos + C.U * ((lj.z - 0.5) * C.aperture) + C.V * ((lj.y - 0.5) * C.aperture);
        dir = unit(focal - org);
    }
    d3 tp = D(1, 1, 1), acc = D(0, 0, 0);
    d3 halton_l = D(0, 0, 0);
    if (P.halton) {
        const double hy = halton(id + 1, 3);
        halton_l = D(halton(id + 1, 2), hy, hy);
    }
    for (int b = 0; b < P.L; ++b) {
        const Ray ray = make_ray(org, dir);
        const Hit h = trace(s, ray, DBL_MAX, false);
        if (h.id < 0) {
            // handle_no_hit under NO_BACKGROUND (hybrid-pt.cpp:45, :567-575):
            // throughput (1,1,1) marks a camera ray; no sky light here
            if (tp.x == 1.0 && tp.y == 1.0 && tp.z == 1.0) acc = acc + tp * P.background;
            break;
        }
        const int t = h.id;
        const double wa = 1.0 - h.beta - h.gamma;
        const d3 Ph = wa * s.a[t] + h.beta * s.b[t] + h.gamma * s.c[t];
        const d3 Nraw = wa * s.na[t] + h.beta * s.nb[t] + h.gamma * s.nc[t];
        const Mat& m = s.mats[s.mat[t]];
        const d3 rnd = U3(P.seed, (uint64_t)id, (uint64_t)p * P.L + (uint64_t)b);
        const d3 lr = P.halton ? halton_l : rnd;
        // area-light sample (arealight-sampler-cpu.cpp:25-119): raw
        // interpolated normal, shadow ray from P + offset along the sample
        // direction with max_t = the distance from P
        d3 sdir = D(0, 0, 0), psc = D(0, 0, 0);
        double smax = -1.0;
        d3 sorg = Ph;
        const int nl = (int)s.lights.size();
        if (nl > 0) {
            const double choice = lr.z * s.overall;
            double lacc = 0.0;
            int l = 0;
            while (l < nl - 1 && choice > lacc + s.lights[l].power) {
                lacc += s.lights[l].power;
                ++l;
            }
            const Light& Lt = s.lights[l];
            const d3 right = tangential(D(1, 0, 0), Lt.dir), up = tangential(D(0, 1, 0), Lt.dir);
            const d3 sp = Lt.center + ((lr.x - 0.5) * Lt.w) * right + ((lr.y - 0.5) * Lt.h) * up;
            d3 v = sp - Ph;
            const double dist = len(v);
            v = v / dist;
            const double ndotl = std::max(dot(Nraw, v), 0.0);
            const double lcos = std::max(dot(Lt.dir, -v), 0.0);
            const double f = Lt.w * Lt.h * ndotl * lcos / (dist * dist);
            psc = Lt.col * f * (s.overall / Lt.power);
            sdir = v;
            sorg = Ph + P.shadow_offset * v;
            smax = dist;
        }
        // shading (hybrid-pt.cpp:421-562)
        const d3 org_dir = unit(dir);
        d3 N = unit(Nraw);
        d3 T, B;
        tangent_frame(N, &T, &B);
        T = unit(T);
        B = unit(B);
        const d3 wo = -org_dir;
        const bool glass = m.principled && m.opacity < 1.0;
        if (dot(org_dir, N) > 0.0) N = -N;
        const d3 wo_ts = D(dot(wo, T), dot(wo, B), dot(wo, N));
        d3 wi_ts;
        double pdf;
        int lobe;
        brdf_sample(m, wo_ts, rnd, &wi_ts, &pdf, &lobe);
        const d3 wi = unit(wi_ts.x * T + wi_ts.y * B + wi_ts.z * N);
        if (!glass && smax >= 0.0) {
            const bool occluded = trace(s, make_ray(sorg, sdir), smax, true).id >= 0;
            if (!occluded) {
                const d3 add = brdf_eval(m, lobe, wo, unit(sdir), N) * (tp * psc);
                if (!any_nan(add)) acc = acc + add;
            }
        }
        const d3 f = brdf_eval(m, lobe, wo, wi, N);
        d3 ntp = tp * f / pdf;
        ntp = D(std::min(ntp.x, 1.0), std::min(ntp.y, 1.0), std::min(ntp.z, 1.0));
        if (!(pdf > 0.0) || any_nan(ntp)) break;
        if (P.rr_start >= 0 && b >= P.rr_start) {
            const double q = std::min(std::max(std::max(std::max(ntp.x, ntp.y), ntp.z), 0.05), 1.0);
            if (unit01(P.seed ^ 0x5DEECE66Dull, (uint64_t)id, (uint64_t)p * P.L + (uint64_t)b, 3) >= q) break;
            ntp = ntp / q;
        }
        tp = ntp;
        org = glass ? Ph + P.ray_offset * org_dir : Ph + P.ray_offset * N;
        dir = wi;
    }
    return acc;
}

}  // namespace

extern "C" {

// Scene from the public description (rect lights and untextured materials
// only).  Returns NULL for a description this restatement does not cover.
void* orc64_scene_create(const gb_scene_desc* d) {
    if (!d || d->num_triangles < 0 || !d->positions || !d->material_index) return nullptr;
    Scene* s = new Scene();
    const int n = d->num_triangles;
    s->n = n;
    s->a.resize(n); s->b.resize(n); s->c.resize(n);
    s->na.resize(n); s->nb.resize(n); s->nc.resize(n);
    s->mat.resize(n);
    for (int t = 0; t < n; ++t) {
        const float* p = d->positions + 9 * (size_t)t;
        s->a[t] = from3(p); s->b[t] = from3(p + 3); s->c[t] = from3(p + 6);
        if (d->normals) {
            const float* q = d->normals + 9 * (size_t)t;
            s->na[t] = from3(q); s->nb[t] = from3(q + 3); s->nc[t] = from3(q + 6);
        } else {
            const d3 fn = cross(s->b[t] - s->a[t], s->c[t] - s->a[t]);
            s->na[t] = s->nb[t] = s->nc[t] = fn;
        }
        s->mat[t] = d->material_index[t];
        if (s->mat[t] < 0 || s->mat[t] >= d->num_materials) { delete s; return nullptr; }
    }
    for (int i = 0; i < d->num_materials; ++i) {
        const gb_material& gm = d->materials[i];
        Mat m;
        if (gm.principled >= 0) {
            if (gm.principled >= d->num_params) { delete s; return nullptr; }
            const gb_principled_params& pp = d->params[gm.principled];
            m.principled = true;
            m.color = from3(pp.color);
            m.metallic = pp.metallic; m.subsurface = pp.subsurface; m.specular = pp.specular;
            m.roughness = pp.roughness; m.specular_tint = pp.specular_tint; m.anisotropic = pp.anisotropic;
            m.sheen = pp.sheen; m.sheen_tint = pp.sheen_tint; m.clearcoat = pp.clearcoat;
            m.clearcoat_gloss = pp.clearcoat_gloss; m.opacity = pp.opacity;
        } else {
            m.color = from3(gm.diffuse);
        }
        s->mats.push_back(m);
    }
    if (d->num_textures > 0 && d->diffuse_texture) {
        for (int i = 0; i < d->num_materials; ++i)
            if (d->diffuse_texture[i] >= 0) { delete s; return nullptr; }
    }
    for (int i = 0; i < d->num_lights; ++i) {
        const gb_light& gl = d->lights[i];
        if (gl.type != GB_LIGHT_RECT) { delete s; return nullptr; }
        Light l;
        l.center = from3(gl.center); l.dir = from3(gl.dir); l.col = from3(gl.col);
        l.w = gl.wh[0]; l.h = gl.wh[1];
        // add-rectlight's power rule (lights.cpp:92) unless given
        l.power = gl.power >= 0.0f ? (double)gl.power : l.w * l.h * (l.col.x + l.col.y + l.col.z) * .333;
        s->overall += l.power;
        s->lights.push_back(l);
    }
    Builder bld(*s);
    bld.build();
    if (bld.max_depth > kMaxDepth) { delete s; return nullptr; }
    return s;
}

void orc64_scene_destroy(void* s) { delete (Scene*)s; }

// Mean radiance over `spp` path samples of the pixels of rows [row0, row1)
// (mean_rgb: (row1-row0)*w*3 doubles) and, when var_rgb is given, each
// pixel's sample variance of one path sample (same layout).  desc gives the
// resolution, bounces, roulette start, offsets, background and light mode;
// `seed` selects the random numbers.
int orc64_render(void* sp, const gb_camera* cam, const gb_render_desc* d, int row0, int row1, int spp,
                 unsigned long long seed, double* mean_rgb, double* var_rgb) {
    const Scene* s = (const Scene*)sp;
    if (!s || !cam || !d || !mean_rgb || spp <= 0) return 1;
    const int W = d->width, H = d->height;
    if (W <= 0 || H <= 0 || row0 < 0 || row1 > H || row0 >= row1 || d->max_bounces <= 0) return 2;
    if (d->rng_mode != GB_RNG_MRG32K3A_POOL && d->rng_mode != GB_RNG_HALTON_LIGHT) return 3;
    const Cam C = make_cam(*cam, W, H);
    Params P;
    P.L = d->max_bounces;
    P.rr_start = d->rr_start;
    P.halton = d->rng_mode == GB_RNG_HALTON_LIGHT;
    P.ray_offset = d->ray_offset;
    P.shadow_offset = d->shadow_offset;
    P.background = from3(d->background);
    P.seed = seed;
    const int n = (row1 - row0) * W;
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < n; ++i) {
        const int id = row0 * W + i;
        double sum[3] = {0, 0, 0}, sq[3] = {0, 0, 0};
        for (int p = 0; p < spp; ++p) {
            const d3 v = path_sample(*s, C, P, id, p);
            for (int k = 0; k < 3; ++k) {
                const double c = comp(v, k);
                sum[k] += c;
                sq[k] += c * c;
            }
        }
        for (int k = 0; k < 3; ++k) {
            const double mean = sum[k] / spp;
            mean_rgb[3 * (size_t)i + k] = mean;
            if (var_rgb) var_rgb[3 * (size_t)i + k] = spp > 1 ? std::max(0.0, (sq[k] - spp * mean * mean) / (spp - 1)) : 0.0;
        }
    }
    return 0;
}

// Closest hit of n rays with this restatement's own tree (ids -1 for a miss;
// t as double), for checking its traversal against the float tracers.
int orc64_trace_closest(void* sp, int n, const float* o, const float* d, const float* tmax, int* ids, double* t) {
    const Scene* s = (const Scene*)sp;
    if (!s) return 1;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < n; ++i) {
        const Hit h = trace(*s, make_ray(from3(o + 3 * (size_t)i), from3(d + 3 * (size_t)i)), (double)tmax[i], false);
        ids[i] = h.id;
        t[i] = h.id >= 0 ? h.t : 0.0;
    }
    return 0;
}

}  // extern "C"
