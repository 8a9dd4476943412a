// gbpt_math.h -- per-ray arithmetic of the globillum path-tracing hot path.
//
// One definition of every formula the path evaluates (camera ray, triangle
// test, light sample, principled/Lambert BRDF sample + eval, throughput
// update), compiled both into the sm_103a kernels (nvcc, -fmad=false) and
// into the CPU oracle (g++, -ffp-contract=off).  Only IEEE-exact operations
// are used (+ - * / sqrt and explicit fmaf); the two transcendentals the
// per-ray path needs (sin/cos of 2*pi*u) are evaluated by a quadrant
// reduction plus the Taylor series of sin/cos(pi/2 * r) in Horner form, so
// host and device produce the same bits.  Per-material constants that need
// pow/log (mon2lin, GTR1 normalisation) are precomputed on the host.
//
// Reference formulas followed (file:line in kiselgra/globillum src/):
//   camera ray          raygen.cu:61-118 (setup_jittered_dof_shirley)
//   area-light sample   arealight-sampler-cpu.cpp:25-143
//   shade / bounce      hybrid-pt.cpp:330-371, 421-448, 450-584
//   principled BRDF     principledMaterial.h:27-401
//   Lambert BRDF        simpleMaterial.h:162-193, materialBase.h:16-24
//   Halton              util.cpp:22-32
//   moving average      util-kernels.cu:17-25
// Helpers that live in the (absent) rta/libhyb libraries -- the triangle
// test, make_tangent_frame, make_tangential, barycentric interpolation,
// normalize_vec3f, cross -- are defined here once (see each function).
#pragma once

#include <stdint.h>
#include <math.h>
#include <float.h>

#if defined(__CUDACC__)
#define GB_HD __host__ __device__ __forceinline__
#else
#define GB_HD static inline
#endif

namespace gb {

// ---------------------------------------------------------------- vectors --
struct v3 { float x, y, z; };

GB_HD v3 mk(float x, float y, float z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
GB_HD v3 operator+(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
GB_HD v3 operator-(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
GB_HD v3 operator-(v3 a) { return mk(-a.x, -a.y, -a.z); }
GB_HD v3 operator*(v3 a, v3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
GB_HD v3 operator*(float s, v3 a) { return mk(s * a.x, s * a.y, s * a.z); }
GB_HD v3 operator*(v3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
GB_HD v3 operator/(v3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
GB_HD v3 operator/(v3 a, v3 b) { return mk(a.x / b.x, a.y / b.y, a.z / b.z); }

// dot product in the reference's operator| order (left to right, no fma).
GB_HD float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// cross product as rta's cross_vec3f (plain products, no fma).
GB_HD v3 cross(v3 a, v3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
GB_HD float length(v3 a) { return sqrtf(dot(a, a)); }
// libhyb normalize_vec3f: divide by the length.
GB_HD v3 normalize_div(v3 a) { float l = length(a); return a / l; }
// principledMaterial.h:34-37 normalize: multiply by 1/sqrt.
GB_HD v3 normalize_rcp(v3 a) { float b = 1.0f / sqrtf(dot(a, a)); return a * b; }

// fused forms used only by the ray/triangle and ray/box tests.
GB_HD float fdot(v3 a, v3 b) { return fmaf(a.x, b.x, fmaf(a.y, b.y, a.z * b.z)); }
GB_HD v3 fcross(v3 a, v3 b) {
    return mk(fmaf(a.y, b.z, -(a.z * b.y)), fmaf(a.z, b.x, -(a.x * b.z)), fmaf(a.x, b.y, -(a.y * b.x)));
}

GB_HD float clampf(float a, float lo, float hi) { return fminf(fmaxf(a, lo), hi); }
GB_HD float sqr(float a) { return a * a; }

static const float kPi = 3.14159265358979f;
static const float kInvPi = 0.318309873342514f;

// --------------------------------------------------------- sin/cos(2*pi*u) --
// Quadrant reduction: 4u = q + r with q integral and r in [-1/2, 1/2] (both
// steps exact in binary floating point), then sin/cos(pi/2 * r) from the
// Taylor series of sin and cos (coefficients (-1)^k (pi/2)^n / n!, rounded
// to float) in Horner form with fmaf.  Error below 2 ulp for u in [0, 1].
GB_HD void sincos_2pi(float u, float* s, float* c) {
    float u4 = u * 4.0f;
    float q = rintf(u4);
    float r = u4 - q;
    int qi = ((int)q) & 3;
    float r2 = r * r;
    float sp = fmaf(r2, -3.598843250074424e-06f, 0.00016044118092395365f);
    sp = fmaf(r2, sp, -0.004681753925979137f);
    sp = fmaf(r2, sp, 0.07969262450933456f);
    sp = fmaf(r2, sp, -0.6459640860557556f);
    sp = fmaf(r2, sp, 1.5707963705062866f);
    float sn = r * sp;
    float cp = fmaf(r2, 4.710874748070637e-07f, -2.520204179745633e-05f);
    cp = fmaf(r2, cp, 0.0009192602592520416f);
    cp = fmaf(r2, cp, -0.020863480865955353f);
    cp = fmaf(r2, cp, 0.25366950035095215f);
    cp = fmaf(r2, cp, -1.2337005138397217f);
    float cs = fmaf(r2, cp, 1.0f);
    float so, co;
    if (qi == 0) { so = sn; co = cs; }
    else if (qi == 1) { so = cs; co = -sn; }
    else if (qi == 2) { so = -sn; co = -cs; }
    else { so = -cs; co = sn; }
    *s = so; *c = co;
}

// ------------------------------------------------------------ tangent frame --
// make_tangent_frame (libhyb, absent): orthonormal basis around a unit N by
// Duff et al., "Building an Orthonormal Basis, Revisited", JCGT 6(1) 2017.
GB_HD void make_tangent_frame(v3 n, v3* T, v3* B) {
    float sign = copysignf(1.0f, n.z);
    float a = -1.0f / (sign + n.z);
    float b = n.x * n.y * a;
    *T = mk(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x);
    *B = mk(b, sign + n.y * n.y * a, -n.y);
}
// make_tangential(v, N) (libhyb, absent): local z-up vector v to world space
// around N (arealight-sampler-cpu.cpp:72-73, :93 use it this way).
GB_HD v3 make_tangential(v3 v, v3 n) {
    v3 T, B; make_tangent_frame(n, &T, &B);
    return (v.x * T + v.y * B) + v.z * n;
}
GB_HD v3 to_tangent(v3 v, v3 T, v3 B, v3 N) { return mk(dot(v, T), dot(v, B), dot(v, N)); }
GB_HD v3 from_tangent(v3 v, v3 T, v3 B, v3 N) { return (v.x * T + v.y * B) + v.z * N; }
// materialBase.h:36-38 reflectR; libhyb reflect uses the same convention.
GB_HD v3 reflect(v3 v, v3 n) { return v - (2.0f * dot(v, n)) * n; }

// barycentric_coord / barycentric_interpolation (rta, absent):
// bc = (1 - beta - gamma, beta, gamma); value = bc.x*a + bc.y*b + bc.z*c.
GB_HD v3 bary(float beta, float gamma, v3 a, v3 b, v3 c) {
    float w = (1.0f - beta) - gamma;
    return (w * a + beta * b) + gamma * c;
}
// The same for texture coordinates: t = 6 floats (ta, tb, tc), out (s, t).
GB_HD void bary2(float beta, float gamma, const float* t, float* s_out, float* t_out) {
    float w = (1.0f - beta) - gamma;
    *s_out = (w * t[0] + beta * t[2]) + gamma * t[4];
    *t_out = (w * t[1] + beta * t[3]) + gamma * t[5];
}

// ------------------------------------------------------ ray/triangle test --
// Moller-Trumbore (intersect_tri_opt in rta is not available; this is the
// published test of Moller & Trumbore 1997, double sided, strict t > 0).
// e1 = v1 - v0 and e2 = v2 - v0 are passed precomputed (same float bits as
// computing them from the corners).
GB_HD bool intersect_tri(v3 o, v3 d, v3 v0, v3 e1, v3 e2, float* t, float* beta, float* gamma) {
    v3 p = fcross(d, e2);
    float det = fdot(e1, p);
    if (det == 0.0f) return false;
    float inv = 1.0f / det;
    v3 s = o - v0;
    float u = fdot(s, p) * inv;
    if (!(u >= 0.0f && u <= 1.0f)) return false;
    v3 q = fcross(s, e1);
    float v = fdot(d, q) * inv;
    if (!(v >= 0.0f && u + v <= 1.0f)) return false;
    float tt = fdot(e2, q) * inv;
    if (!(tt > 0.0f)) return false;
    *t = tt; *beta = u; *gamma = v;
    return true;
}

// intersect_tri_opt_nocheck (rta, absent; "actually just a plane
// intersection", hybrid-pt.cpp:308-313): the same arithmetic without any
// range check, so the barycentrics of the hit with the triangle's plane.
GB_HD void plane_bary(v3 o, v3 d, v3 v0, v3 e1, v3 e2, float* beta, float* gamma) {
    v3 p = fcross(d, e2);
    float inv = 1.0f / fdot(e1, p);
    v3 s = o - v0;
    *beta = fdot(s, p) * inv;
    v3 q = fcross(s, e1);
    *gamma = fdot(d, q) * inv;
}

// closest-hit acceptance: lexicographic minimum of (t, canonical id) over
// all triangles with 0 < t <= t_max; the result is independent of the BVH
// layout and traversal order (tracers.cu:113 keeps `is.t < closest.t &&
// is.t <= t_max`, which is the same except at exact ties in t).
GB_HD bool closer(float t, uint32_t id, float best_t, uint32_t best_id) {
    return t < best_t || (t == best_t && id < best_id);
}

// ----------------------------------------------------------- sample streams --
// util.cpp:22-32
GB_HD float halton(int index, int base) {
    float result = 0.0f;
    float f = 1.0f / float(base);
    int i = index;
    while (i > 0) {
        result += f * float(i % base);
        i = i / base;
        f = f / float(base);
    }
    return result;
}

// Integer hash for the Russian-roulette extension (not in the reference):
// "lowbias32" integer finaliser (C. Wellons, hash-prospector, 2018).
GB_HD uint32_t hash32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}
GB_HD float rr_uniform(uint32_t seed, uint32_t pixel, uint32_t path, uint32_t bounce) {
    uint32_t h = hash32(seed ^ hash32(pixel ^ hash32(path * 0x9e3779b9U ^ hash32(bounce + 0x632be5abU))));
    return float(h >> 8) * (1.0f / 16777216.0f);
}

// MRG32k3a jump-ahead (L'Ecuyer 1999, "Good parameters and implementations
// for combined multiple recursive random number generators"; jumps by matrix
// powers as in L'Ecuyer, Simard, Chen and Kelton 2002, "An object-oriented
// random-number package with many long streams and substreams").  The two
// component states are kept oldest value first, (x[n-3], x[n-2], x[n-1]);
// one step maps them with
//   A1 = [[0, 1, 0], [0, 0, 1], [-810728, 1403580, 0]]   mod m1 = 2^32 - 209
//   A2 = [[0, 1, 0], [0, 0, 1], [-1370589, 0, 527612]]   mod m2 = 2^32 - 22853
// and k steps with A1^k, A2^k (row-major, entries reduced mod m).
constexpr uint32_t kMrgM1 = 4294967087u;
constexpr uint32_t kMrgM2 = 4294944443u;

// x mod m for m = 2^32 - c (x < 2^64): 2^32 = c (mod m) folds the high word
// into the low word twice, then at most two subtractions remain.
GB_HD uint32_t mrg_reduce(uint64_t x, uint32_t c, uint32_t m) {
    x = (x >> 32) * c + (x & 0xffffffffull);
    x = (x >> 32) * c + (x & 0xffffffffull);
    while (x >= m) x -= m;
    return (uint32_t)x;
}

GB_HD void mrg_apply(uint32_t s[3], const uint32_t* J, uint32_t c, uint32_t m) {
    uint32_t r[3];
    for (int i = 0; i < 3; ++i) {
        uint64_t acc = 0;
        for (int j = 0; j < 3; ++j) acc += mrg_reduce((uint64_t)J[3 * i + j] * s[j], c, m);
        r[i] = mrg_reduce(acc, c, m);  // acc < 3 m
    }
    s[0] = r[0]; s[1] = r[1]; s[2] = r[2];
}

// One step of the two component recurrences as 3x3 matrices on the state
// vectors (L'Ecuyer 1999: x_n = (1403580 x_{n-2} - 810728 x_{n-3}) mod m1,
// y_n = (527612 y_{n-1} - 1370589 y_{n-3}) mod m2), in the state order
// s[0] oldest .. s[2] newest.
constexpr uint32_t kMrgA1[9] = {0, 1, 0, 0, 0, 1, kMrgM1 - 810728u, 1403580u, 0};
constexpr uint32_t kMrgA2[9] = {0, 1, 0, 0, 0, 1, kMrgM2 - 1370589u, 0, 527612u};

// C = A B mod m (3x3); C may alias A or B.
GB_HD void mrg_matmul(const uint32_t* A, const uint32_t* B, uint32_t* C, uint32_t c, uint32_t m) {
    uint32_t r[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            uint64_t acc = 0;
            for (int k = 0; k < 3; ++k) acc += mrg_reduce((uint64_t)A[3 * i + k] * B[3 * k + j], c, m);
            r[3 * i + j] = mrg_reduce(acc, c, m);
        }
    for (int i = 0; i < 9; ++i) C[i] = r[i];
}

// out = A^k mod m by square-and-multiply.
GB_HD void mrg_power(const uint32_t* A, uint64_t k, uint32_t* out, uint32_t c, uint32_t m) {
    uint32_t base[9], acc[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    for (int i = 0; i < 9; ++i) base[i] = A[i];
    while (k) {
        if (k & 1) mrg_matmul(acc, base, acc, c, m);
        mrg_matmul(base, base, base, c, m);
        k >>= 1;
    }
    for (int i = 0; i < 9; ++i) out[i] = acc[i];
}

// Jumps between the subsequences of curand_init(seed, subsequence, 0):
// subsequence i starts i * 2^76 steps after subsequence 0 (cuRAND's
// documented MRG32k3a subsequence spacing).  j1[k], j2[k] = A1^(2^(76+k)),
// A2^(2^(76+k)), so subsequence i is reached by applying the matrices of
// the set bits of i.
struct MrgSubseqTable {
    uint32_t j1[32][9], j2[32][9];
};

static inline void mrg_subsequence_table(MrgSubseqTable* T) {
    uint32_t a1[9], a2[9];
    for (int i = 0; i < 9; ++i) { a1[i] = kMrgA1[i]; a2[i] = kMrgA2[i]; }
    for (int s = 0; s < 76; ++s) {  // A^(2^76)
        mrg_matmul(a1, a1, a1, 209u, kMrgM1);
        mrg_matmul(a2, a2, a2, 22853u, kMrgM2);
    }
    for (int k = 0; k < 32; ++k) {
        for (int i = 0; i < 9; ++i) { T->j1[k][i] = a1[i]; T->j2[k][i] = a2[i]; }
        mrg_matmul(a1, a1, a1, 209u, kMrgM1);
        mrg_matmul(a2, a2, a2, 22853u, kMrgM2);
    }
}

// Advances a state (s1, s2) by the steps J1 = A1^k, J2 = A2^k stand for.
GB_HD void mrg_jump(uint32_t s1[3], uint32_t s2[3], const uint32_t* J1, const uint32_t* J2) {
    mrg_apply(s1, J1, 209u, kMrgM1);
    mrg_apply(s2, J2, 22853u, kMrgM2);
}

// ----------------------------------------------------------------- camera --
// Per-frame constants of setup_jittered_dof_shirley (raygen.cu:61-118); the
// host fills them once (W, U, V are the same for every ray).
struct CameraRec {
    v3 pos, view, U, V, W;
    float width, height;      // aspect*tan(fovy/2), tan(fovy/2)
    float aperture, focus;
    int w, h;
};

GB_HD void camera_frame(v3 view, v3 up, v3* U, v3* V, v3* W) {
    *W = view / length(view);
    v3 TxW = cross(up, *W);
    *U = TxW / length(TxW);
    *V = cross(*W, *U);
}

// jitter = (rnd.x, rnd.y) of the jitter stream; lens = aperture sample
// (zero when aperture == 0, where it is multiplied by zero in the reference).
// Shirley direction through the image-plane point (jx, jy) in pixels.
GB_HD v3 camera_dir(const CameraRec& c, float jx, float jy) {
    float u_s = ((jx) / (float)c.w) * 2.0f - 1.0f;
    float v_s = ((jy) / (float)c.h) * 2.0f - 1.0f;
    u_s = c.width * u_s;
    v_s = c.height * v_s;
    v3 d = c.U * u_s;
    d = d + c.V * v_s;
    d = d + c.W;
    return normalize_div(d);
}

GB_HD void camera_ray(const CameraRec& c, int x, int y, float jx_r, float jy_r, float lens_x, float lens_y,
                      v3* org, v3* dir) {
    v3 d = camera_dir(c, float(x) + jx_r, float(y) + jy_r);
    v3 focal = c.pos + (d * (1.0f / dot(d, c.view))) * c.focus;
    v3 jp = (c.pos + (c.U * lens_x) * c.aperture) + (c.V * lens_y) * c.aperture;
    d = focal - jp;
    *dir = normalize_div(d);
    *org = jp;
}

// Ray differentials of a path (hybrid-pt.cpp:300-328): origin and
// direction of the "upper" and "right" neighbour rays.
struct RayDiff { v3 uo, ud, ro, rd; };

// The camera's differentials.  They come from rta's
// camera_ray_generator_shirley<gpu_ray_generator_with_differentials>, which
// the jittered lens generator runs first and which "generates ray
// differentials based on a uniform ray distribution" (raygen.h:49-52, :86-90);
// rta is not available, so the uniform generator is taken to be the
// pixel-centre Shirley camera and the neighbours to be pixels (x, y+1) and
// (x+1, y), both from the eye.
GB_HD RayDiff camera_diff(const CameraRec& c, int x, int y) {
    RayDiff r;
    r.uo = c.pos;
    r.ud = camera_dir(c, float(x) + 0.5f, float(y + 1) + 0.5f);
    r.ro = c.pos;
    r.rd = camera_dir(c, float(x + 1) + 0.5f, float(y) + 0.5f);
    return r;
}

// ----------------------------------------------------------------- lights --
// gi::light (lights.h:94-154) restricted to rectangular lights; right/up are
// make_tangential((1,0,0)|(0,1,0), dir) (arealight-sampler-cpu.cpp:72-73),
// fixed per light and filled by the host.
struct LightRec {
    v3 center, dir, col, right, up;
    float w, h, power;
    int type;        // 0 rect, 1 sky (gi::light::type_t, lights.h:147-149)
    float scale;     // sky: radiance scale (sky_light::scale)
};

// --------------------------------------------------------------- sky light --
// atan / atan2 / acos from IEEE-exact operations: the Taylor series
// atan(z) = z - z^3/3 + z^5/5 - ... (terms to z^17) on |z| <= tan(pi/12),
// the addition formula atan(z) = pi/6 + atan((sqrt(3) z - 1) / (z + sqrt(3)))
// above it, and atan(z) = pi/2 - atan(1/z) for z > 1.  Used only to find the
// texel of a direction in a sky map.
GB_HD float atan_pos(float z) {  // z >= 0
    bool inv = z > 1.0f;
    if (inv) z = 1.0f / z;
    bool shift = z > 0.267949192f;  // tan(pi/12)
    if (shift) z = (1.73205081f * z - 1.0f) / (z + 1.73205081f);
    float z2 = z * z;
    // q = -1/3 + z^2/5 - z^4/7 + ... + z^14/17, atan(z) = z (1 + z^2 q)
    float q = 1.0f / 17.0f;
    q = q * z2 - 1.0f / 15.0f;
    q = q * z2 + 1.0f / 13.0f;
    q = q * z2 - 1.0f / 11.0f;
    q = q * z2 + 1.0f / 9.0f;
    q = q * z2 - 1.0f / 7.0f;
    q = q * z2 + 1.0f / 5.0f;
    q = q * z2 - 1.0f / 3.0f;
    float a = z + z * (z2 * q);
    if (shift) a = a + 0.523598776f;  // pi/6
    if (inv) a = 1.57079633f - a;     // pi/2
    return a;
}
GB_HD float atan2_ex(float y, float x) {
    if (x == 0.0f && y == 0.0f) return 0.0f;
    float ax = fabsf(x), ay = fabsf(y);
    float a = ax >= ay ? atan_pos(ay / ax) : 1.57079633f - atan_pos(ax / ay);
    if (x < 0.0f) a = 3.14159265f - a;
    return y < 0.0f ? -a : a;
}
GB_HD float acos_ex(float x) {
    x = fminf(1.0f, fmaxf(-1.0f, x));
    return atan2_ex(sqrtf((1.0f - x) * (1.0f + x)), x);
}

// A lat-long radiance map (rows theta = 0 .. pi, columns phi = 0 .. 2 pi)
// with the two-level sampling tables of Distribution2D (lights.h:18-90):
// a row CDF/PDF over the summed row importance and one column CDF/PDF per
// row, built on the host (gbpt_host.h, make_sky_tables).
struct SkyRec {
    const float* texel;    // w*h radiance, 4 floats per texel (rgb, 0)
    const float* row_cdf;  // h + 1
    const float* row_pdf;  // h
    const float* col_cdf;  // h * (w + 1)
    const float* col_pdf;  // h * w
    int w, h;
    float scale;
    int light;             // index of the sky light, -1 = none
};

// Distribution1D::sample (lights.h:49-56): index with CDF[i] <= u < CDF[i+1]
// (upper_bound - 1, clamped), then x = (1 - t) i + t (i + 1) with
// t = (CDF[i+1] - u) / (CDF[i+1] - CDF[i]) as written there.
GB_HD void dist1d_sample(const float* cdf, const float* pdf, int n, float u, float* x, float* p) {
    int lo = 0, hi = n;
    while (lo < hi) {  // upper_bound over cdf[0 .. n-1]
        int mid = (lo + hi) >> 1;
        if (cdf[mid] <= u) lo = mid + 1;
        else hi = mid;
    }
    int idx = lo - 1;
    idx = idx < 0 ? 0 : (idx > n - 1 ? n - 1 : idx);
    float t = (cdf[idx + 1] - u) / (cdf[idx + 1] - cdf[idx]);
    *x = (1.0f - t) * float(idx) + t * float(idx + 1);
    *p = pdf[idx];
}

// sky_light::sample (lights.h:107-126) with Distribution2D::sample
// (lights.h:73-79): (u, v) from the tables, direction
// (sin t cos p, sin t sin p, cos t) for t = u pi / h, p = v 2 pi / w, pdf
// (pdf_row pdf_col w h) / (2 pi^2 sin t), radiance of texel (int u, int v).
GB_HD v3 sky_sample(const SkyRec& s, float ru, float rv, float* pdf_out, v3* dir) {
    float u, v, pu, pv;
    dist1d_sample(s.row_cdf, s.row_pdf, s.h, ru, &u, &pu);
    int yi = (int)u;
    yi = yi < 0 ? 0 : (yi > s.h - 1 ? s.h - 1 : yi);
    dist1d_sample(s.col_cdf + (size_t)yi * (s.w + 1), s.col_pdf + (size_t)yi * s.w, s.w, rv, &v, &pv);
    float st, ct, sp, cp;
    sincos_2pi(u * (0.5f / float(s.h)), &st, &ct);
    sincos_2pi(v / float(s.w), &sp, &cp);
    *dir = mk(st * cp, st * sp, ct);
    *pdf_out = (pu * pv * float(s.w * s.h)) / (19.7392088f * st);  // 2 pi^2
    int xi = (int)v;
    xi = xi < 0 ? 0 : (xi > s.w - 1 ? s.w - 1 : xi);
    const float* t = s.texel + 4 * ((size_t)yi * s.w + xi);
    return mk(t[0], t[1], t[2]);
}

// evaluateSkyLight (hybrid-pt.cpp:175-189): the texel of a direction,
// theta = acos(d.y), phi = atan2(d.z, d.x) in [0, 2 pi); no scale applied.
GB_HD v3 sky_eval(const SkyRec& s, v3 d) {
    float theta = acos_ex(d.y);
    float phi = atan2_ex(d.z, d.x);
    if (phi < 0.0f) phi += 6.28318531f;
    float su = phi / 6.28318531f, tv = theta / 3.14159265f;
    long long idx = (long long)(int)(tv * float(s.h)) * s.w + (int)(su * float(s.w));
    if (idx < 0 || idx >= (long long)s.h * s.w) return mk(0.0f, 0.0f, 0.0f);
    const float* t = s.texel + 4 * idx;
    return mk(t[0], t[1], t[2]);
}

// Sky branch of the GPU sampler k::pixel_generate_arealight_sample
// (arealight-sampler.cu:213-229): a uniform hemisphere direction
// (sqrt(1 - x^2) cos 2 pi y, sqrt(1 - x^2) sin 2 pi y, x) mapped around the
// (unnormalised) normal, weighted by scale * texel(dir) * (dir . N); the
// direction is not renormalised there and the shadow ray is unbounded.
GB_HD void sky_light_sample_uniform(const SkyRec& s, float power, float overall_power, v3 P, v3 N, float rx,
                                    float ry, float shadow_offset, v3* so, v3* sd, float* smax, v3* psc) {
    float sq = sqrtf(1.0f - rx * rx);
    float sn, cs;
    sincos_2pi(ry, &sn, &cs);
    v3 dir = make_tangential(mk(sq * cs, sq * sn, rx), N);
    float theta = acos_ex(dir.y);
    float phi = atan2_ex(dir.z, dir.x);
    if (phi < 0.0f) phi += 6.28318531f;
    float su = phi / 6.28318531f, tv = theta / 3.14159265f;
    long long idx = (long long)(int)(tv * float(s.h)) * s.w + (int)(su * float(s.w));
    v3 L = mk(0.0f, 0.0f, 0.0f);
    if (idx >= 0 && idx < (long long)s.h * s.w) L = mk(s.texel[4 * idx], s.texel[4 * idx + 1], s.texel[4 * idx + 2]);
    v3 contribution = (s.scale * L) * dot(dir, N);
    *so = P + shadow_offset * dir;
    *sd = dir;
    *smax = FLT_MAX;
    *psc = contribution * (overall_power / power);
}

// Sky branch of pixel_generate_arealight_sample_cpu with USE_SKY_SAMPLING
// (arealight-sampler-cpu.cpp:87-96, 113-119): the sampled direction is
// mapped around the (unnormalised) normal with make_tangential, weighted by
// scale / pdf * |dir . N|; the shadow ray is unbounded.
GB_HD void sky_light_sample(const SkyRec& s, float power, float overall_power, v3 P, v3 N, float rx, float ry,
                            float shadow_offset, v3* so, v3* sd, float* smax, v3* psc) {
    float pdf;
    v3 dir;
    v3 L = sky_sample(s, rx, ry, &pdf, &dir);
    dir = make_tangential(dir, N);
    float a = 1.0f / pdf;
    v3 contribution = (s.scale * L) * (a * fabsf(dot(dir, N)));
    dir = normalize_div(dir);
    *so = P + shadow_offset * dir;
    *sd = dir;
    *smax = FLT_MAX;
    *psc = contribution * (overall_power / power);
}

// lights.cpp:92: power = w*h*(r+g+b)*.333
GB_HD float rect_light_power(float w, float h, v3 col) {
    return (float)((double)(w * h * (col.x + col.y + col.z)) * .333);
}

// Light pick (arealight-sampler-cpu.cpp:32-39).  The reference reads
// lights[n] when the accumulated power falls short of choice by rounding;
// here the index stops at n-1.
// The interval (lo, hi] of the uniform draw rnd_z that pick_light maps to
// light l (choice = rnd_z * overall_power, the light pick of
// arealight-sampler-cpu.cpp:32-39; the last light takes the rest).
GB_HD void light_pick_interval(const LightRec* L, int n, float overall_power, int l, float* lo, float* hi) {
    float acc = 0.0f;
    for (int i = 0; i < l; ++i) acc += L[i].power;
    *lo = acc / overall_power;
    *hi = l + 1 < n ? (acc + L[l].power) / overall_power : 1.0f;
}

GB_HD int pick_light(const LightRec* L, int n, float overall_power, float rnd_z) {
    float choice = rnd_z * overall_power;
    float acc = 0.0f;
    int l = 0;
    while (l < n - 1 && choice > acc + L[l].power) {
        acc += L[l].power;
        ++l;
    }
    return l;
}

// Rectangular-light sample at a hit (arealight-sampler-cpu.cpp:65-86, 114-119).
// P, N: interpolated hit point and (unnormalised) normal.  Outputs the
// shadow ray and potential_sample_contribution = col * scale, where col is
// the light's emission (l.col, or the emission being differentiated) and
// scale the geometry term over the light's pick probability.
GB_HD void rect_light_sample(const LightRec& l, v3 col, float overall_power, v3 P, v3 N, float rx, float ry,
                             float shadow_offset, v3* so, v3* sd, float* smax, v3* psc, float* scale = nullptr,
                             bool renormalize = true) {
    float offx = (rx - 0.5f) * l.w;
    float offy = (ry - 0.5f) * l.h;
    v3 ls = (l.center + offx * l.right) + offy * l.up;
    v3 dir = ls - P;
    float len = length(dir);
    dir = dir / len;
    float ndotl = fmaxf(dot(N, dir), 0.0f);
    float light_cos = fmaxf(dot(l.dir, -dir), 0.0f);
    float factor = l.w * l.h * ndotl * light_cos / (len * len);
    v3 contribution = col * factor;
    if (renormalize) dir = normalize_div(dir);  // the CPU sampler normalises again (:113)
    *so = P + shadow_offset * dir;
    *sd = dir;
    *smax = len;
    float inv_pick = overall_power / l.power;
    *psc = contribution * inv_pick;
    if (scale) *scale = factor * inv_pick;
}

// -------------------------------------------------------------- materials --
// material_t (material.h:142-184) + PrincipledBRDFParameters
// (principledParameters.h:7-24), flattened with the per-material constants
// of principledMaterial.h:178-252 precomputed on the host.
// --------------------------------------------------------------- textures --
// texture_data (material.h:21-137) after convert_texture
// (material-conversion.cpp:18-35): RGBA8 texels, row 0 at t = 1, mip levels
// stored one after the other (level i+1 is ((W+1)/2) x ((H+1)/2) of level
// i; compute_mipmaps, material.cu:259-275).  The buffer holds `size`
// texels: the levels and a zero tail, so that the reads sample_bilin_lod
// makes one row or one texel past a level (t = 0 gives y = H; x = W for the
// right neighbour of the last column) stay inside it.
struct TexRec {
    const uint8_t* texels;   // 4 bytes per texel
    int w, h, max_mm;        // max_mm = floor(log2(min(w, h)))
    int size;                // texels in the buffer
};

GB_HD v3 tex_texel(const TexRec& t, int i) {
    i = i < 0 ? 0 : (i >= t.size ? t.size - 1 : i);  // never taken by the reads below
#ifdef __CUDA_ARCH__
    uchar4 q = __ldg((const uchar4*)t.texels + i);
    return mk(float(q.x) / 255.0f, float(q.y) / 255.0f, float(q.z) / 255.0f);
#else
    const uint8_t* p = t.texels + 4 * (size_t)i;
    return mk(float(p[0]) / 255.0f, float(p[1]) / 255.0f, float(p[2]) / 255.0f);
#endif
}

// Mip levels sample_bilin_lod steps down: its loop `for (i = 0; i < lod; ++i)`
// with lod = fminf(log2f(x), max_mm) runs min(ceil(log2 x), max_mm) times
// when x > 1, max_mm times for NaN, none otherwise.  ceil(log2 x) is taken
// from the binary exponent of x, which is exact; a rounded log2f differs
// from it only for x within about an ulp above a power of two.
GB_HD int tex_levels(float x, int max_mm) {
    if (x != x) return max_mm;
    if (!(x > 1.0f)) return 0;
    if (x > FLT_MAX) return max_mm;
    int e;
    float m = frexpf(x, &e);  // x = m 2^e, m in [0.5, 1)
    int c = m == 0.5f ? e - 1 : e;
    return c < max_mm ? c : max_mm;
}

// texture_data::sample_bilin_lod (material.h:88-137): level chosen by the
// footprint `diff` in texture space, coordinates wrapped into [0, 1), the
// nearest texel and its neighbour towards the sample point blended with
// weights |neighbour centre - x|.  The neighbour index wraps only when it
// is negative or more than one past the level (`other_x > W`), as in the
// reference, so x = W and y = H read the texel after the row / level.
GB_HD v3 tex_sample_bilin_lod(const TexRec& t, float s, float tt, float diff) {
    int W = t.w, H = t.h;
    int levels = tex_levels(diff * fmaxf((float)t.w, (float)t.h), t.max_mm);
    int offset = 0;
    for (int i = 0; i < levels; ++i) {
        offset += W * H;
        W = (W + 1) / 2;
        H = (H + 1) / 2;
    }
    if (s < 0) s += -truncf(s) + 1;
    if (s >= 1) s -= truncf(s);
    if (tt < 0) tt += -truncf(tt) + 1;
    if (tt >= 1) tt -= truncf(tt);
    float x = s * (float)W;
    float y = (1.0f - tt) * (float)H;
    int nx = int(x), ny = int(y);
    int ox = nx + 1, oy = ny + 1;
    if (x - floorf(x) < .5f) ox = nx - 1;
    if (y - floorf(y) < .5f) oy = ny - 1;
    // (float(o) + .5 - x) of the reference is exact in double; its float
    // rounding equals this float subtraction
    float wx = fabsf(((float)ox + .5f) - x);
    float wy = fabsf(((float)oy + .5f) - y);
    if (ox > W) ox -= W;
    if (ox < 0) ox += W;
    if (oy > H) oy -= H;
    if (oy < 0) oy += H;
    v3 a00 = tex_texel(t, offset + ny * W + nx);
    v3 a01 = tex_texel(t, offset + ny * W + ox);
    v3 a10 = tex_texel(t, offset + oy * W + nx);
    v3 a11 = tex_texel(t, offset + oy * W + ox);
    v3 a0x = wx * a00 + (1.0f - wx) * a01;
    v3 a1x = wx * a10 + (1.0f - wx) * a11;
    return wy * a0x + (1.0f - wy) * a1x;
}

// computeRayDiffs (hybrid-pt.cpp:300-328) and the footprint of
// material_t::diffuseColor (material.h:159-170) at a hit on triangle
// (a, b, c) with texture coordinates tcs (6 floats), hit texture
// coordinate (ts, tt) and normalised normal N: both neighbour rays meet the
// triangle's plane, their texture coordinates give the footprint; the
// origins move to those points and the upper direction is reflected about
// N (the right direction is left as it was, as in the reference).
GB_HD float ray_diff_hit(RayDiff* rd, v3 a, v3 b, v3 c, const float* tcs, float ts, float tt, v3 N) {
    v3 e1 = b - a, e2 = c - a;
    float ub, ug, rb, rg, us, ut, rs, rt;
    plane_bary(rd->uo, rd->ud, a, e1, e2, &ub, &ug);
    bary2(ub, ug, tcs, &us, &ut);
    v3 up = bary(ub, ug, a, b, c);
    plane_bary(rd->ro, rd->rd, a, e1, e2, &rb, &rg);
    bary2(rb, rg, tcs, &rs, &rt);
    v3 rp = bary(rb, rg, a, b, c);
    rd->uo = up;
    rd->ro = rp;
    rd->ud = reflect(rd->ud, N);
    float dx = fabsf(ts - us);
    float dy = fabsf(tt - ut);
    dx = fmaxf(fabsf(ts - rs), dx);
    dy = fmaxf(fabsf(tt - rt), dy);
    return fmaxf(dx, dy);
}

// x^2.2 in double for the textured colours of principled materials
// (mon2lin, principledMaterial.h:226): ln x from the atanh series of the
// mantissa reduced to [sqrt(1/2), sqrt(2)), exp by reduction to
// |r| <= ln(2)/2 and its Taylor polynomial.  Written out here (not pow) so
// that host and device give the same bits; error below 1e-14 relative.
GB_HD double pow22(double x) {
    if (x != x || x < 0.0) return (x - x) / (x - x);  // NaN, as pow of a negative base
    if (x == 0.0) return 0.0;
    const double kLn2 = 0.69314718055994530942;
    int e;
    double m = frexp(x, &e);
    if (m < 0.70710678118654752440) { m *= 2.0; e -= 1; }
    double z = (m - 1.0) / (m + 1.0), z2 = z * z, p = 1.0 / 25.0;
    for (int k = 23; k >= 1; k -= 2) p = p * z2 + 1.0 / (double)k;
    double y = 2.2 * (2.0 * z * p + (double)e * kLn2);
    double kf = floor(y / kLn2 + 0.5);
    double r = y - kf * kLn2, q = 1.0;
    for (int k = 18; k >= 1; --k) q = q * (r / (double)k) + 1.0;
    return ldexp(q, (int)kf);
}

enum { MAT_LAMBERT = 0, MAT_PRINCIPLED = 1 };
struct MaterialRec {
    int kind;
    float diffuse[3];          // Lambert: diffuse_color; principled: parameters->color
    float metallic, subsurface, roughness, sheen, clearcoat, opacity;
    float ax, ay, roughg2;     // principledMaterial.h:179-181, :158, :166
    float cdlin[3];            // mon2lin(color)           :226
    float csheen[3];           // mix(1, Ctint, sheenTint) :276
    float cspec0[3];           // :231
    float cc_a, cc_a2m1, cc_pilog;  // GTR1 constants        :186-192, :241
    float kd[3];               // material_t::diffuse_color (evaluate_material, material-cpu.cpp:20-80)
    float sheen_tint, specular_tint, specular;  // to recompute the colour terms for a texture
    int dtex;                  // diffuse texture (index into the scene's textures) or -1
};
static const int kMaterialFloats = 32;  // padded device record size

// Inverse of pack_material (gbpt_host.h): record from its 32-float form.
GB_HD MaterialRec unpack_material(const float* f) {
    MaterialRec r;
    r.kind = (int)f[0];
    r.diffuse[0] = f[1]; r.diffuse[1] = f[2]; r.diffuse[2] = f[3];
    r.metallic = f[4]; r.subsurface = f[5]; r.roughness = f[6]; r.sheen = f[7];
    r.clearcoat = f[8]; r.opacity = f[9]; r.ax = f[10]; r.ay = f[11]; r.roughg2 = f[12];
    for (int k = 0; k < 3; ++k) { r.cdlin[k] = f[13 + k]; r.csheen[k] = f[16 + k]; r.cspec0[k] = f[19 + k]; }
    r.cc_a = f[22]; r.cc_a2m1 = f[23]; r.cc_pilog = f[24];
    r.kd[0] = f[25]; r.kd[1] = f[26]; r.kd[2] = f[27];
    r.sheen_tint = f[28]; r.specular_tint = f[29]; r.specular = f[30];
    r.dtex = (int)f[31];
    return r;
}

// The colour terms of a principled record (make_material) for base colour
// c, principledMaterial.h:226-231, :276.  Shared by the host set-up and the
// texture path so both give the same bits.
GB_HD void material_colour_terms(MaterialRec* r, const float* c, bool own_pow) {
    float cdlin[3];
    for (int k = 0; k < 3; ++k) {
        r->diffuse[k] = c[k];
#ifdef __CUDA_ARCH__
        cdlin[k] = (float)pow22((double)c[k]);
        (void)own_pow;
#else
        cdlin[k] = own_pow ? (float)pow22((double)c[k]) : (float)pow((double)c[k], 2.2);
#endif
    }
    float cdlum = (float)(.3 * cdlin[0] + .6 * cdlin[1] + .1 * cdlin[2]);
    float ctint[3];
    for (int k = 0; k < 3; ++k) ctint[k] = cdlum > 0 ? cdlin[k] / cdlum : 1.0f;
    float spec08 = (float)((double)r->specular * .08);
    for (int k = 0; k < 3; ++k) {
        r->cdlin[k] = cdlin[k];
        r->csheen[k] = (1.0f - r->sheen_tint) * 1.0f + r->sheen_tint * ctint[k];
        float st = (1.0f - r->specular_tint) * 1.0f + r->specular_tint * ctint[k];
        float a = spec08 * st;
        r->cspec0[k] = (1.0f - r->metallic) * a + r->metallic * cdlin[k];
    }
}

// material_t::diffuseColor with a diffuse texture (material.h:159-170): the
// base colour (diffuse_color, or parameters->color for principled
// materials) times the texture sample, used by both the Lambert and the
// principled model (simpleMaterial.h:95, principledMaterial.h:327).
GB_HD MaterialRec textured_material(const MaterialRec& m, v3 tex) {
    MaterialRec r = m;
    float c[3] = {m.diffuse[0] * tex.x, m.diffuse[1] * tex.y, m.diffuse[2] * tex.z};
    if (m.kind == MAT_PRINCIPLED) material_colour_terms(&r, c, true);
    else for (int k = 0; k < 3; ++k) r.diffuse[k] = c[k];
    return r;
}

enum { LOBE_DIFFUSE = 0, LOBE_SPECULAR = 1, LOBE_DISNEY_REFLECTION = 2,
       LOBE_SPECULAR_REFLECTION = 3, LOBE_SPECULAR_TRANSMISSION = 4 };

GB_HD float schlick(float u) {
    float m = clampf(1.0f - u, 0.0f, 1.0f);
    float m2 = m * m;
    return m2 * m2 * m;
}
GB_HD float mixf(float x, float y, float s) { return (1.0f - s) * x + s * y; }

// materialBase.h:16-24
GB_HD v3 cosine_sample_hemisphere(float u, float v) {
    float r = sqrtf(u);
    float sn, cs; sincos_2pi(v, &sn, &cs);
    return mk(r * cs, r * sn, sqrtf(fmaxf(0.0f, 1.0f - u)));
}

// principledMaterial.h:64-69
GB_HD float smithG_GGX(float ndv, float alphaG) {
    float a = alphaG * alphaG;
    float b = ndv * ndv;
    return 1.0f / (ndv + sqrtf(a + b - a * b));
}
// principledMaterial.h:76-80 (Walter et al. G1 with the Xi indicator)
GB_HD float G1(v3 v, v3 m, v3 n, float a2, float tanv) {
    float fac = (dot(v, m) / dot(v, n)) > 0.0f ? 1.0f : 0.0f;
    return fac * 2.0f / (1.0f + sqrtf(1.0f + a2 * tanv * tanv));
}

// principledMaterial.h:121-176 with T=(1,0,0), B=(0,1,0), n=(0,0,1) in
// tangent space (:369-371).  Returns the Walter weight (>= 0.01 or NaN).
GB_HD float sample_gtr2_aniso(float u, float v, float ax, float ay, float roughg2, v3 V, v3* Lout,
                              bool* flipped = nullptr) {
    float sn, cs; sincos_2pi(u, &sn, &cs);
    float fac = sqrtf(v / (1.0f - v));
    v3 t = mk(ax * cs, 0.0f, 0.0f);
    t = t + mk(0.0f, ay * sn, 0.0f);
    v3 h = normalize_rcp(fac * t + mk(0.0f, 0.0f, 1.0f));
    v3 n = mk(0.0f, 0.0f, 1.0f);
    v3 L = reflect(V, h);
    const bool flip = dot(L, n) < 0.0f;
    if (flip) L = -1.0f * L;
    if (flipped) *flipped = flip;
    float dotLm = dot(L, h);
    float dotVm = dot(V, h);
    float tanL = sqrtf(1.0f - dotLm * dotLm) / dotLm;
    float tanV = sqrtf(1.0f - dotVm * dotVm) / dotVm;
    float Gs = G1(L, h, n, roughg2, tanL) * G1(V, h, n, roughg2, tanV);
    float w = (fabsf(dot(L, h)) * Gs) / (fabsf(dot(L, n)) * fabsf(dot(n, h)));
    if (w < 0.01f) w = 0.01f;
    *Lout = L;
    return w;
}

// principledMaterial.h:86-118
GB_HD v3 sample_glass(float u, v3 V, float ior, int* lobe) {
    v3 n = mk(0.0f, 0.0f, 1.0f);
    float c = dot(n, V);
    float fresnel = schlick(c);
    if (u > fresnel) {
        *lobe = LOBE_SPECULAR_REFLECTION;
        return -V;
    }
    float ti = 1.0f + ior * (c * c - 1.0f);
    if (ti <= 0.0f) {
        *lobe = LOBE_SPECULAR_REFLECTION;
        return reflect(V, n);
    }
    *lobe = LOBE_SPECULAR_TRANSMISSION;
    float sg = dot(V, n) > 0.0f ? 1.0f : -1.0f;
    return (ior * c - sg * sqrtf(ti)) * n - ior * V;
}

GB_HD bool is_glass(const MaterialRec& m) { return m.kind == MAT_PRINCIPLED && m.opacity < 1.0f; }

// Flags of a sampled vertex (for the derivatives of the sampling
// decisions): the metallic branch was taken (rnd.z < metallic), the GTR2
// reflection was flipped to the upper side, the shading normal was flipped
// to face the incoming ray.
enum { SAMPLE_METAL_BRANCH = 1u, SAMPLE_L_FLIPPED = 2u, SAMPLE_N_FLIPPED = 4u };

// materialBRDF::sample (material-wrapper.h:224-227) -> LambertianMaterial::sample
// (simpleMaterial.h:183-186) or PrincipledMaterial::sample
// (principledMaterial.h:354-390).  wo, wi in tangent space.
GB_HD void material_sample(const MaterialRec& m, v3 wo, v3 rnd, v3* wi, float* pdf, int* lobe,
                           uint32_t* flags = nullptr) {
    if (flags) *flags = 0u;
    if (m.kind == MAT_LAMBERT) {
        v3 w = cosine_sample_hemisphere(rnd.x, rnd.y);
        *wi = w;
        *pdf = fabsf(w.z) * kInvPi;
        *lobe = LOBE_DIFFUSE;
        return;
    }
    if (m.opacity < 1.0f) {
        *wi = sample_glass(rnd.x, wo, 1.9f, lobe);
        *pdf = 1.0f;
        return;
    }
    if (rnd.z < m.metallic) {
        v3 L;
        bool flip = false;
        float p = sample_gtr2_aniso(rnd.x, rnd.y, m.ax, m.ay, m.roughg2, wo, &L, &flip);
        if (flags) *flags = SAMPLE_METAL_BRANCH | (flip ? SAMPLE_L_FLIPPED : 0u);
        *lobe = LOBE_DISNEY_REFLECTION;
        *wi = L;
        *pdf = p;
        if (p == 0.0f || p != p) {
            v3 w = cosine_sample_hemisphere(rnd.x, rnd.y);
            *wi = w;
            *lobe = LOBE_DIFFUSE;
            *pdf = clampf(w.z, 0.0f, FLT_MAX) * kInvPi;
        }
        return;
    }
    v3 w = cosine_sample_hemisphere(rnd.x, rnd.y);
    *wi = w;
    *lobe = LOBE_DIFFUSE;
    *pdf = fmaxf(w.z, 0.0f) * kInvPi;
}

// principledMaterial.h:254-301
GB_HD v3 principled_diffuse(const MaterialRec& m, v3 V, v3 N, v3 L) {
    float NdotL = dot(N, L);
    float NdotV = dot(N, V);
    if (NdotL < 0.0f || NdotV < 0.0f) return mk(0.0f, 0.0f, 0.0f);
    v3 H = normalize_rcp(L + V);
    float LdotH = dot(L, H);
    float FL = schlick(NdotL), FV = schlick(NdotV);
    float Fd90 = 0.5f + 2.0f * LdotH * LdotH * m.roughness;
    float Fd = mixf(1.0f, Fd90, FL) * mixf(1.0f, Fd90, FV);
    float FH = schlick(LdotH);
    float fs = FH * m.sheen;
    v3 Fsheen = fs * mk(m.csheen[0], m.csheen[1], m.csheen[2]);
    float Fss90 = LdotH * LdotH * m.roughness;
    float Fss = mixf(1.0f, Fss90, FL) * mixf(1.0f, Fss90, FV);
    float ss = 1.25f * (Fss * (1.0f / (NdotL + NdotV) - 0.5f) + 0.5f);
    float k = kInvPi * mixf(Fd, ss, m.subsurface);
    v3 dcol = (k * mk(m.cdlin[0], m.cdlin[1], m.cdlin[2]) + Fsheen) * (1.0f - m.metallic);
    return dcol * NdotL;
}

// principledMaterial.h:210-252
GB_HD v3 principled_specular(const MaterialRec& m, v3 V, v3 N, v3 L) {
    float NdotL = dot(N, L);
    float NdotV = dot(N, V);
    if (NdotL < 0.0f || NdotV < 0.0f) return mk(0.0f, 0.0f, 0.0f);
    v3 H = normalize_rcp(L + V);
    float NdotH = dot(N, H);
    float LdotH = dot(L, H);
    float FH = schlick(LdotH);
    v3 Fs = (1.0f - FH) * mk(m.cspec0[0], m.cspec0[1], m.cspec0[2]) + FH * mk(1.0f, 1.0f, 1.0f);
    float cg = 0.0f;
    if (m.clearcoat > 0.0f) {
        float Dr;
        if (m.cc_a >= 1.0f) Dr = kInvPi;
        else {
            float t = 1.0f + m.cc_a2m1 * NdotH * NdotH;
            Dr = m.cc_a2m1 / (m.cc_pilog * t);
        }
        float Fr = mixf(0.04f, 1.0f, FH);
        float Gr = smithG_GGX(NdotL, 0.25f) * smithG_GGX(NdotV, 0.25f);
        cg = 0.25f * m.clearcoat * Gr * Fr * Dr;
    }
    v3 sum = Fs + mk(cg, cg, cg);
    return (sum * NdotL) * m.metallic;
}

// materialBRDF::evaluate (material-wrapper.h:228-232) with the lobe chosen by
// the preceding sample() (principledMaterial.h:336-352); world space.
GB_HD v3 material_eval(const MaterialRec& m, int lobe, v3 wo, v3 wi, v3 N) {
    if (m.kind == MAT_LAMBERT)
        return (mk(m.diffuse[0], m.diffuse[1], m.diffuse[2]) * kInvPi) * fabsf(dot(wi, N));
    if (lobe == LOBE_DISNEY_REFLECTION) return principled_specular(m, wo, N, wi);
    if (lobe == LOBE_SPECULAR_REFLECTION) return mk(1.0f, 1.0f, 1.0f);
    if (lobe == LOBE_SPECULAR_TRANSMISSION) return mk(1.0f, 1.0f, 1.0f) * (1.0f / fabsf(dot(wi, N)));
    return principled_diffuse(m, wo, N, wi);
}

// Derivatives of a vertex's sampling decisions (PrincipledMaterial::sample,
// principledMaterial.h:354-390: the metallic lobe when rnd.z < metallic,
// then the GTR2-aniso half vector of :46-61 and the Walter weight of
// :121-176 as the sample's "pdf"):
//   sm  d log P(branch | the other uses of rnd.z) / d metallic.  rnd.z is
//       uniform on (zlo, zhi] given the vertex's other decisions that read
//       it: with MRG32k3a light draws the light pick reads the same value
//       (the light and path pools are seeded alike), so it is the picked
//       light's power interval; otherwise (0, 1].  P(metallic branch) =
//       clamp((metallic - zlo) / (zhi - zlo), 0, 1), so the score is
//       1 / (metallic - zlo) for the metallic branch and
//       -1 / (zhi - metallic) for the diffuse one while metallic lies in
//       the interval (derivatives from inside the interval at its ends),
//       0 otherwise; 0 for Lambert and glass
//   sr  d log p(h) / d roughness of the sampled half vector, with
//       p(h) = D_GTR2(h) cos(theta_h) (the density of the sampling formula)
//       and h held fixed; the density of the second half vector that
//       reflects to the same flipped direction is neglected
//   wr  d log w / d roughness of the Walter weight the throughput is
//       divided by (0 where it was clamped at 0.01)
// sr and wr are nonzero for a successful metallic sample only.  The half
// vector is recovered from the recorded directions: L = +-(V - 2 (V.h) h),
// so h is parallel to V - L, or to V + L when L was flipped.
GB_HD void sampling_scores(const MaterialRec& m, int lobe, uint32_t flags, v3 wo, v3 wi, v3 N, float pdf,
                           float zlo, float zhi, float* sm, float* sr, float* wr) {
    *sm = 0.0f;
    *sr = 0.0f;
    *wr = 0.0f;
    if (m.kind != MAT_PRINCIPLED || m.opacity < 1.0f) return;
    const float mt = m.metallic;
    if (flags & SAMPLE_METAL_BRANCH) *sm = (mt > zlo && mt <= zhi) ? 1.0f / (mt - zlo) : 0.0f;
    else *sm = (mt >= zlo && mt < zhi) ? -1.0f / (zhi - mt) : 0.0f;
    if (lobe != LOBE_DISNEY_REFLECTION) return;
    const float r = m.roughness;
    if (!(r > 0.0f)) return;
    // the sampling frame: tangents of the unflipped normal, z = N
    const v3 Nu = (flags & SAMPLE_N_FLIPPED) ? -1.0f * N : N;
    v3 T, B;
    make_tangent_frame(Nu, &T, &B);
    T = normalize_div(T);
    B = normalize_div(B);
    v3 h = (flags & SAMPLE_L_FLIPPED) ? wo + wi : wo - wi;
    const float hl = length(h);
    if (!(hl > 0.0f)) return;
    h = h / hl;
    float hz = dot(h, N);
    if (hz < 0.0f) {
        h = -1.0f * h;
        hz = -hz;
    }
    const float hx = dot(h, T), hy = dot(h, B);
    const float ax = m.ax, ay = m.ay;
    // ax = max(.001, r^2 / aspect), ay = max(.001, r^2 aspect)
    const float dax = ax > 0.001f ? 2.0f * ax / r : 0.0f;
    const float day = ay > 0.001f ? 2.0f * ay / r : 0.0f;
    // log D = -log(pi ax ay) - 2 log Q, Q = (hx / ax)^2 + (hy / ay)^2 + hz^2
    const float qx = hx / ax, qy = hy / ay;
    const float Q = qx * qx + qy * qy + hz * hz;
    const float dlx = -1.0f / ax + 4.0f * qx * qx / (ax * Q);
    const float dly = -1.0f / ay + 4.0f * qy * qy / (ay * Q);
    *sr = dlx * dax + dly * day;
    if (!(pdf > 0.01f)) return;
    // w = |L.h| G1(L) G1(V) / (|L.n| |n.h|), G1 = Xi 2 / (1 + S),
    // S = sqrt(1 + a2 tan^2): d log G1 / d a2 = -(tan^2 / (2 S)) / (1 + S)
    const float a2 = m.roughg2;
    float dlw = 0.0f;
    for (int side = 0; side < 2; ++side) {
        const float d = side ? dot(wo, h) : dot(wi, h);
        const float t2 = (1.0f - d * d) / (d * d);
        const float S = sqrtf(1.0f + a2 * t2);
        dlw += -(t2 / (2.0f * S)) / (1.0f + S);
    }
    // a2 = roughg^2, roughg = b^2, b = ax ay / 2 + 1 / 2
    const float b = ax * ay * 0.5f + 0.5f;
    const float roughg = b * b;
    *wr = dlw * (2.0f * roughg * b * (dax * ay + ax * day));
}

// ---------------------------------------------------------------- adjoint --
// Gradient of the differentiable fields of a material record.  Sampling
// quantities (ax, ay, roughg2, lobe choice) are held fixed by the
// path-replay adjoint, so roughness enters through the diffuse lobe only.
struct MatGrad {
    float cdlin[3], csheen[3], cspec0[3];
    float metallic, roughness;
    float diffuse[3];
};
static const int kMatGradFloats = 14;  // cdlin[3], csheen[3], cspec0[3], metallic, roughness, diffuse[3]

GB_HD void matgrad_zero(MatGrad* g) {
    for (int c = 0; c < 3; ++c) { g->cdlin[c] = 0.0f; g->csheen[c] = 0.0f; g->cspec0[c] = 0.0f; g->diffuse[c] = 0.0f; }
    g->metallic = 0.0f;
    g->roughness = 0.0f;
}
GB_HD float v3c(v3 v, int c) { return c == 0 ? v.x : (c == 1 ? v.y : v.z); }

// a^T d(principled_diffuse)/d(cdlin, csheen, metallic, roughness), added to g.
GB_HD void principled_diffuse_vjp(const MaterialRec& m, v3 V, v3 N, v3 L, v3 a, MatGrad* g) {
    float NdotL = dot(N, L);
    float NdotV = dot(N, V);
    if (NdotL < 0.0f || NdotV < 0.0f) return;
    v3 H = normalize_rcp(L + V);
    float LdotH = dot(L, H);
    float FL = schlick(NdotL), FV = schlick(NdotV);
    float l2 = LdotH * LdotH;
    float Fd90 = 0.5f + 2.0f * l2 * m.roughness;
    float Ad = mixf(1.0f, Fd90, FL), Bd = mixf(1.0f, Fd90, FV);
    float Fd = Ad * Bd;
    float FH = schlick(LdotH);
    float Fss90 = l2 * m.roughness;
    float As = mixf(1.0f, Fss90, FL), Bs = mixf(1.0f, Fss90, FV);
    float Fss = As * Bs;
    float css = 1.25f * (1.0f / (NdotL + NdotV) - 0.5f);  // d ss / d Fss
    float ss = css * Fss + 0.625f;
    float k = kInvPi * mixf(Fd, ss, m.subsurface);
    float om = 1.0f - m.metallic;
    float fsh = FH * m.sheen;
    v3 ad = a * NdotL;  // adjoint of dcol
    float ak = 0.0f, am = 0.0f;
    for (int c = 0; c < 3; ++c) {
        float adc = v3c(ad, c);
        g->cdlin[c] += adc * k * om;
        g->csheen[c] += adc * fsh * om;
        ak += adc * m.cdlin[c] * om;
        am -= adc * (k * m.cdlin[c] + fsh * m.csheen[c]);
    }
    g->metallic += am;
    float dFd = (FL * Bd + Ad * FV) * 2.0f * l2;
    float dss = css * (FL * Bs + As * FV) * l2;
    g->roughness += ak * kInvPi * ((1.0f - m.subsurface) * dFd + m.subsurface * dss);
}

// a^T d(principled_specular)/d(cspec0, metallic), added to g.
GB_HD void principled_specular_vjp(const MaterialRec& m, v3 V, v3 N, v3 L, v3 a, MatGrad* g) {
    float NdotL = dot(N, L);
    float NdotV = dot(N, V);
    if (NdotL < 0.0f || NdotV < 0.0f) return;
    v3 H = normalize_rcp(L + V);
    float NdotH = dot(N, H);
    float LdotH = dot(L, H);
    float FH = schlick(LdotH);
    float cg = 0.0f;
    if (m.clearcoat > 0.0f) {
        float Dr;
        if (m.cc_a >= 1.0f) Dr = kInvPi;
        else {
            float t = 1.0f + m.cc_a2m1 * NdotH * NdotH;
            Dr = m.cc_a2m1 / (m.cc_pilog * t);
        }
        float Fr = mixf(0.04f, 1.0f, FH);
        float Gr = smithG_GGX(NdotL, 0.25f) * smithG_GGX(NdotV, 0.25f);
        cg = 0.25f * m.clearcoat * Gr * Fr * Dr;
    }
    float am = 0.0f;
    for (int c = 0; c < 3; ++c) {
        float ac = v3c(a, c);
        float Fs = (1.0f - FH) * m.cspec0[c] + FH;
        g->cspec0[c] += ac * NdotL * m.metallic * (1.0f - FH);
        am += ac * (Fs + cg) * NdotL;
    }
    g->metallic += am;
}

// a^T d(material_eval)/d(record fields), added to g.
GB_HD void material_eval_vjp(const MaterialRec& m, int lobe, v3 wo, v3 wi, v3 N, v3 a, MatGrad* g) {
    if (m.kind == MAT_LAMBERT) {
        float f = kInvPi * fabsf(dot(wi, N));
        g->diffuse[0] += a.x * f; g->diffuse[1] += a.y * f; g->diffuse[2] += a.z * f;
        return;
    }
    if (lobe == LOBE_DISNEY_REFLECTION) { principled_specular_vjp(m, wo, N, wi, a, g); return; }
    if (lobe == LOBE_SPECULAR_REFLECTION || lobe == LOBE_SPECULAR_TRANSMISSION) return;
    principled_diffuse_vjp(m, wo, N, wi, a, g);
}

// ------------------------------------------------------------ shade/bounce --
// Parameters of compute_path_contribution_and_bounce that the reference hard
// codes (hybrid-pt.cpp:45, :52, :551; arealight-sampler-cpu.cpp:115).
struct ShadeParams {
    float ray_offset;       // 0.3 in the reference
    float shadow_offset;    // 0.9 in the reference
    v3 background;          // (1,1,1), added for primary misses (NO_BACKGROUND)
    int rr_start;           // Russian roulette from this bounce (extension); <0 = off
    uint32_t seed;
};

struct ShadeOut {
    v3 org, dir;     // next ray
    v3 tp;           // new throughput
    v3 accum_add;    // added to col_accum this bounce
    bool alive;
};

// sample_material of hybrid-pt.cpp:330-349 with the normal and tangent
// frame of :430 and :525-528: the sampled world direction, its pdf and lobe,
// and the (possibly flipped) shading normal.
struct BsdfSample {
    v3 org_dir, inv_org_dir, N, wi;
    float pdf;
    int lobe;
    bool glass;
    uint32_t flags;  // SAMPLE_*
};

GB_HD BsdfSample sample_bsdf(const MaterialRec& m, v3 Nraw, v3 ray_dir, v3 rnd) {
    BsdfSample s;
    s.org_dir = normalize_div(ray_dir);
    v3 N = normalize_div(Nraw);
    v3 T, B;
    make_tangent_frame(N, &T, &B);
    T = normalize_div(T);
    B = normalize_div(B);
    s.inv_org_dir = -1.0f * s.org_dir;
    s.glass = is_glass(m);
    const bool nflip = dot(s.org_dir, N) > 0.0f;
    if (nflip) N = N * -1.0f;
    v3 wo_ts = to_tangent(s.inv_org_dir, T, B, N);
    v3 wi;
    material_sample(m, wo_ts, rnd, &wi, &s.pdf, &s.lobe, &s.flags);
    if (nflip) s.flags |= SAMPLE_N_FLIPPED;
    wi = from_tangent(wi, T, B, N);
    s.wi = normalize_div(wi);
    s.N = N;
    return s;
}

// What the path-replay adjoint needs of one shaded vertex: the directions
// and normal the BRDF was evaluated with, the sampling pdf and roulette
// probability (both held fixed when differentiating), the lobe, which
// throughput channels were clamped at 1, and whether the NEE term counted.
struct ShadeTrace {
    v3 wo, wi, N, ld;
    float pdf, q;
    int lobe;
    uint32_t clamp_mask;  // bit c: channel c of the new throughput was clamped
    bool nee;
    uint32_t flags;       // SAMPLE_* of the vertex's BRDF sample
};

GB_HD v3 clamp_one(v3 t, uint32_t* mask) {
    uint32_t mk_ = 0;
    if (t.x > 1.0f) { t.x = 1.0f; mk_ |= 1u; }
    if (t.y > 1.0f) { t.y = 1.0f; mk_ |= 2u; }
    if (t.z > 1.0f) { t.z = 1.0f; mk_ |= 4u; }
    *mask = mk_;
    return t;
}
GB_HD bool has_nan(v3 t) { return t.x != t.x || t.y != t.y || t.z != t.z; }

// One pixel of compute_path_contribution_and_bounce (hybrid-pt.cpp:465-564)
// for a valid hit.  P, Nraw: interpolated hit point / normal; ray_dir: the
// ray direction; rnd: the path-stream draw; unoccluded: shadow result;
// to_light, psc: the NEE outputs of this bounce.
// Frozen-sampling replay (me, tp0 given): directions, lobes and pdfs come
// from m, the BRDF values from me; tp0 carries the throughput under m, which
// makes the roulette and path-end decisions, so the path's random choices
// are those of m while its value is that of me.  trace (optional) receives
// the vertex record of the adjoint.
GB_HD ShadeOut shade_hit(const MaterialRec& m, v3 P, v3 Nraw, v3 ray_dir, v3 tp, v3 rnd,
                         bool unoccluded, v3 to_light, v3 psc, const ShadeParams& sp,
                         uint32_t pixel, uint32_t path, int bounce, const MaterialRec* me = nullptr,
                         v3* tp0 = nullptr, ShadeTrace* trace = nullptr) {
    ShadeOut o;
    const MaterialRec& E = me ? *me : m;
    BsdfSample bs = sample_bsdf(m, Nraw, ray_dir, rnd);
    const v3 org_dir = bs.org_dir, inv_org_dir = bs.inv_org_dir, N = bs.N, wi = bs.wi;
    const float pdf = bs.pdf;
    const int lobe = bs.lobe;
    const bool glass = bs.glass;
    // evaluate_material (hybrid-pt.cpp:351-371)
    o.accum_add = mk(0.0f, 0.0f, 0.0f);
    bool nee = false;
    v3 ld = mk(0.0f, 0.0f, 0.0f);
    if (!glass && unoccluded) {
        v3 currTP = tp * psc;
        ld = normalize_div(to_light);
        v3 bl = material_eval(E, lobe, inv_org_dir, ld, N);
        v3 add = bl * currTP;
        if (!has_nan(add)) { o.accum_add = add; nee = true; }
    }
    v3 brdf = material_eval(E, lobe, inv_org_dir, wi, N);
    // next ray (hybrid-pt.cpp:550-562)
    v3 Pn = glass ? P + sp.ray_offset * org_dir : P + sp.ray_offset * N;
    o.org = Pn;
    o.dir = wi;
    uint32_t cmask = 0;
    v3 ntp = clamp_one((tp * brdf) / pdf, &cmask);
    v3 ntp0 = ntp;  // throughput that makes the decisions
    if (tp0) {
        uint32_t unused;
        ntp0 = clamp_one((*tp0 * material_eval(m, lobe, inv_org_dir, wi, N)) / pdf, &unused);
    }
    o.alive = true;
    // pdf == 0 or a NaN throughput would poison the pixel forever in the
    // reference; such paths end here.
    if (!(pdf > 0.0f) || has_nan(ntp0)) {
        o.alive = false;
        ntp = ntp0 = mk(0.0f, 0.0f, 0.0f);
    } else if (has_nan(ntp)) {
        ntp = mk(0.0f, 0.0f, 0.0f);
    }
    // Russian roulette (extension, off when rr_start < 0)
    float q = 1.0f;
    if (o.alive && sp.rr_start >= 0 && bounce >= sp.rr_start) {
        q = fmaxf(fmaxf(ntp0.x, ntp0.y), ntp0.z);
        q = clampf(q, 0.05f, 1.0f);
        float u = rr_uniform(sp.seed, pixel, path, (uint32_t)bounce);
        if (u >= q) { o.alive = false; ntp = ntp0 = mk(0.0f, 0.0f, 0.0f); }
        else { ntp = ntp / q; ntp0 = ntp0 / q; }
    }
    o.tp = ntp;
    if (tp0) *tp0 = ntp0;
    if (trace) {
        trace->wo = inv_org_dir; trace->wi = wi; trace->N = N; trace->ld = ld;
        trace->pdf = pdf; trace->q = q; trace->lobe = lobe; trace->clamp_mask = cmask; trace->nee = nee;
        trace->flags = bs.flags;
    }
    return o;
}

// handle_no_hit (hybrid-pt.cpp:196-206, :567-575): primary misses are
// recognised by throughput == (1,1,1) and add the background; other misses
// add throughput * the sky texel of the normalised ray direction
// (evaluateSkyLight, hybrid-pt.cpp:175-189, unscaled), or nothing when the
// scene has no sky light.
GB_HD v3 miss_contribution(v3 tp, v3 ray_dir, const ShadeParams& sp, const SkyRec* sky = nullptr) {
    if (tp.x == 1.0f && tp.y == 1.0f && tp.z == 1.0f) return tp * sp.background;
    if (sky && sky->light >= 0) return tp * sky_eval(*sky, normalize_div(ray_dir));
    return tp * mk(0.0f, 0.0f, 0.0f);
}

// util-kernels.cu:17-25
GB_HD v3 combine_sample(v3 sofar, v3 sample, int k) {
    return (float(k) * sofar + sample) / float(k + 1);
}

}  // namespace gb
