// gbpt_host.h -- host-side preparation of the per-frame / per-scene records
// that the per-ray arithmetic of gbpt_math.h consumes.  Used by libgbpt and
// by the CPU oracle so both see the same constants.
#pragma once

#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/gbpt.h"
#include "gbpt_math.h"

namespace gb {

// Per-material constants of principledMaterial.h:178-252 (mon2lin, Ctint,
// Cspec0, Csheen, anisotropic alphas, the remapped roughness of :158 and the
// GTR1 normalisation of :186-192), from a material_t-like description.
static inline MaterialRec make_material(const gb_material& m, const gb_principled_params* params) {
    MaterialRec r;
    std::memset(&r, 0, sizeof(r));
    for (int k = 0; k < 3; ++k) r.kd[k] = m.diffuse[k];
    r.dtex = -1;
    if (m.principled < 0) {
        r.kind = MAT_LAMBERT;
        for (int k = 0; k < 3; ++k) r.diffuse[k] = m.diffuse[k];
        r.opacity = 1.0f;
        return r;
    }
    const gb_principled_params& p = params[m.principled];
    r.kind = MAT_PRINCIPLED;
    for (int k = 0; k < 3; ++k) r.diffuse[k] = p.color[k];
    r.metallic = p.metallic; r.subsurface = p.subsurface; r.roughness = p.roughness;
    r.sheen = p.sheen; r.clearcoat = p.clearcoat; r.opacity = p.opacity;
    float aspect = (float)std::sqrt(1.0 - (double)p.anisotropic * .9);
    float r2 = p.roughness * p.roughness;
    r.ax = std::max(.001f, r2 / aspect);
    r.ay = std::max(.001f, r2 * aspect);
    float roughg = (float)((double)(r.ax * r.ay) * .5 + .5);
    roughg = roughg * roughg;
    r.roughg2 = roughg * roughg;
    r.sheen_tint = p.sheen_tint;
    r.specular_tint = p.specular_tint;
    r.specular = p.specular;
    material_colour_terms(&r, p.color, false);
    float a = (1.0f - p.clearcoat_gloss) * 0.1f + p.clearcoat_gloss * 0.001f;
    float a2 = a * a;
    r.cc_a = a;
    r.cc_a2m1 = a2 - 1.0f;
    r.cc_pilog = kPi * (float)std::log((double)a2);
    return r;
}

// Differentiable parameters of a material: base colour (3), roughness,
// metallic; of a light: emission (3).
static const int kMatParams = 5;
static const int kLightParams = 3;

// Chain rule from the record-field gradient of a material (MatGrad order,
// kMatGradFloats doubles) to its parameters (kMatParams doubles), following
// make_material: cdlin = color^2.2, Ctint = cdlin / lum(cdlin), csheen =
// mix(1, Ctint, sheenTint), cspec0 = mix(0.08 specular mix(1, Ctint,
// specularTint), cdlin, metallic).  Lambert materials take the colour
// gradient from `diffuse`; their roughness and metallic entries are 0.
static inline void material_param_vjp(const gb_material& mat, const gb_principled_params* params,
                                      const double* gr, double* out) {
    for (int k = 0; k < kMatParams; ++k) out[k] = 0.0;
    if (mat.principled < 0) {
        for (int c = 0; c < 3; ++c) out[c] = gr[11 + c];
        return;
    }
    const gb_principled_params& p = params[mat.principled];
    double cd[3], dcd[3];
    for (int c = 0; c < 3; ++c) {
        cd[c] = std::pow((double)p.color[c], 2.2);
        dcd[c] = p.color[c] > 0.0f ? 2.2 * std::pow((double)p.color[c], 1.2) : 0.0;
    }
    const double w[3] = {.3, .6, .1};
    const double lum = w[0] * cd[0] + w[1] * cd[1] + w[2] * cd[2];
    const double met = p.metallic, st = p.specular_tint, sh = p.sheen_tint, spec08 = (double)p.specular * .08;
    // gradient with respect to cdlin[i]
    double gcd[3];
    for (int i = 0; i < 3; ++i) gcd[i] = gr[0 + i] + met * gr[6 + i];
    if (lum > 0.0) {
        for (int k = 0; k < 3; ++k) {
            double gt = sh * gr[3 + k] + (1.0 - met) * spec08 * st * gr[6 + k];  // gradient of Ctint[k]
            for (int i = 0; i < 3; ++i) {
                double dct = ((k == i ? lum : 0.0) - cd[k] * w[i]) / (lum * lum);
                gcd[i] += gt * dct;
            }
        }
    }
    for (int c = 0; c < 3; ++c) out[c] = gcd[c] * dcd[c];
    out[3] = gr[10];
    double gm = gr[9];
    for (int k = 0; k < 3; ++k) {
        double ctint = lum > 0.0 ? cd[k] / lum : 1.0;
        gm += gr[6 + k] * (cd[k] - spec08 * ((1.0 - st) + st * ctint));
    }
    out[4] = gm;
}

// Flattened device record (kMaterialFloats floats).
static inline void pack_material(const MaterialRec& r, float* f) {
    std::memset(f, 0, sizeof(float) * kMaterialFloats);
    f[0] = (float)r.kind;
    f[1] = r.diffuse[0]; f[2] = r.diffuse[1]; f[3] = r.diffuse[2];
    f[4] = r.metallic; f[5] = r.subsurface; f[6] = r.roughness; f[7] = r.sheen;
    f[8] = r.clearcoat; f[9] = r.opacity; f[10] = r.ax; f[11] = r.ay; f[12] = r.roughg2;
    for (int k = 0; k < 3; ++k) { f[13 + k] = r.cdlin[k]; f[16 + k] = r.csheen[k]; f[19 + k] = r.cspec0[k]; }
    f[22] = r.cc_a; f[23] = r.cc_a2m1; f[24] = r.cc_pilog;
    f[25] = r.kd[0]; f[26] = r.kd[1]; f[27] = r.kd[2];
    f[28] = r.sheen_tint; f[29] = r.specular_tint; f[30] = r.specular;
    f[31] = (float)r.dtex;
}

// Mip chain of a texture (texture_data's constructor and compute_mipmaps,
// material.h:27-36, material.cu:231-275): max_mm = floor(log2(min(w, h)))
// levels after the image, texel (x, y) of level i+1 the integer mean
// (truncated) of the 2x2 block at (2x, 2y) of level i.  Parts of the block
// outside an odd-sized level are left out of the mean; the reference's
// kernel drops the wrong weight there (w00 instead of w01) and reads an
// uninitialised texel, which is not reproduced.  Integer floor(log2) is
// exact where log2f of the size is not (sizes near 2^k above 2^17).
// Output: all levels, then a zero tail of w + 1 texels (see TexRec).
static inline void make_mipmaps(const uint8_t* rgba, int w, int h, std::vector<uint8_t>* out, int* max_mm,
                                int* size) {
    int mn = w < h ? w : h, mm = 0;
    while ((2 << mm) <= mn) ++mm;
    std::vector<int> off(1, 0), lw(1, w), lh(1, h);
    for (int i = 0; i < mm; ++i) {
        off.push_back(off.back() + lw.back() * lh.back());
        lw.push_back((lw.back() + 1) / 2);
        lh.push_back((lh.back() + 1) / 2);
    }
    const int total = off.back() + lw.back() * lh.back();
    out->assign(4 * (size_t)(total + w + 1), 0);
    uint8_t* d = out->data();
    std::memcpy(d, rgba, 4 * (size_t)w * h);
    for (int i = 0; i < mm; ++i) {
        const int sw = lw[i], sh = lh[i], tw = lw[i + 1], th = lh[i + 1];
        const uint8_t* src = d + 4 * (size_t)off[i];
        uint8_t* dst = d + 4 * (size_t)off[i + 1];
        for (int y = 0; y < th; ++y)
            for (int x = 0; x < tw; ++x) {
                const int X = 2 * x, Y = 2 * y;
                const bool rx = X + 1 < sw, ry = Y + 1 < sh;
                const unsigned W = 1u + (rx ? 1u : 0u) + (ry ? 1u : 0u) + (rx && ry ? 1u : 0u);
                for (int k = 0; k < 4; ++k) {
                    unsigned t = src[4 * ((size_t)Y * sw + X) + k];
                    if (rx) t += src[4 * ((size_t)Y * sw + X + 1) + k];
                    if (ry) t += src[4 * ((size_t)(Y + 1) * sw + X) + k];
                    if (rx && ry) t += src[4 * ((size_t)(Y + 1) * sw + X + 1) + k];
                    dst[4 * ((size_t)y * tw + x) + k] = (uint8_t)(t / W);
                }
            }
    }
    *max_mm = mm;
    *size = total + w + 1;
}

// gi::light: a rect light with its fixed basis (arealight-sampler-cpu.cpp:70-73),
// or a sky light with add-skylight's power rule scale * 4 pi (d / 2)^2
// (lights.cpp:98-104).
static inline LightRec make_light(const gb_light& l) {
    LightRec r;
    std::memset(&r, 0, sizeof(r));
    r.type = l.type == GB_LIGHT_SKY ? 1 : 0;
    if (r.type == 1) {
        r.scale = l.sky_scale;
        float d = l.sky_diameter;
        r.power = l.power >= 0.0f ? l.power : l.sky_scale * 4.0f * (float)M_PI * (d * 0.5f) * (d * 0.5f);
        return r;
    }
    r.center = mk(l.center[0], l.center[1], l.center[2]);
    r.dir = mk(l.dir[0], l.dir[1], l.dir[2]);
    r.col = mk(l.col[0], l.col[1], l.col[2]);
    r.w = l.wh[0]; r.h = l.wh[1];
    r.right = make_tangential(mk(1.0f, 0.0f, 0.0f), r.dir);
    r.up = make_tangential(mk(0.0f, 1.0f, 0.0f), r.dir);
    r.power = l.power >= 0.0f ? l.power : rect_light_power(r.w, r.h, r.col);
    return r;
}

// Host copy of a sky map and its sampling tables (SkyRec's arrays).
struct SkyTables {
    std::vector<float> texel;    // 4 floats per texel (rgb, 0)
    std::vector<float> row_cdf, row_pdf, col_cdf, col_pdf;
    int w = 0, h = 0;
};

// Distribution1D::init (lights.h:28-45) in float: PDF = data / sum (0 when
// the sum is 0), CDF[0] = 0, CDF[i] = CDF[i-1] + PDF[i-1], CDF[n] = 1.
static inline float dist1d_init(const float* data, int n, float* pdf, float* cdf) {
    float sum = 0.0f;
    for (int i = 0; i < n; ++i) sum += data[i];
    float scale = sum > 0.0f ? 1.0f / sum : 0.0f;
    cdf[0] = 0.0f;
    for (int i = 0; i < n; ++i) {
        pdf[i] = data[i] * scale;
        if (i > 0) cdf[i] = cdf[i - 1] + pdf[i - 1];
    }
    cdf[n] = 1.0f;
    return sum;
}

// sky_light::initSkylight (lights.h:100-110): importance of texel (x, y) =
// sin(pi (y + 0.5) / h) * (r + g + b), one row distribution per row and a
// distribution over the row sums (Distribution2D, lights.h:62-72).
static inline void make_sky_tables(const float* rgb, int w, int h, SkyTables* t) {
    t->w = w;
    t->h = h;
    t->texel.assign(4 * (size_t)w * h, 0.0f);
    std::vector<float> imp((size_t)w * h);
    for (int y = 0; y < h; ++y) {
        float sy = std::sin((float)(M_PI * (y + 0.5f) / h));
        for (int x = 0; x < w; ++x) {
            const float* c = rgb + 3 * ((size_t)y * w + x);
            for (int k = 0; k < 3; ++k) t->texel[4 * ((size_t)y * w + x) + k] = c[k];
            imp[(size_t)y * w + x] = sy * ((c[0] + c[1]) + c[2]);
        }
    }
    t->col_pdf.assign((size_t)w * h, 0.0f);
    t->col_cdf.assign((size_t)(w + 1) * h, 0.0f);
    std::vector<float> rows(h);
    for (int y = 0; y < h; ++y)
        rows[y] = dist1d_init(&imp[(size_t)y * w], w, &t->col_pdf[(size_t)y * w], &t->col_cdf[(size_t)y * (w + 1)]);
    t->row_pdf.assign(h, 0.0f);
    t->row_cdf.assign(h + 1, 0.0f);
    dist1d_init(rows.data(), h, t->row_pdf.data(), t->row_cdf.data());
}

// hybrid-pt.cpp:74-78
static inline float overall_power(const LightRec* L, int n) {
    float p = 0.0f;
    for (int i = 0; i < n; ++i) p += L[i].power;
    return p;
}

// Per-frame camera constants (raygen.cu:71-90).  aspect = w/h; the half
// field of view tangent is taken in double on the host.
static inline CameraRec make_camera(const gb_camera& c, int w, int h) {
    CameraRec r;
    r.pos = mk(c.pos[0], c.pos[1], c.pos[2]);
    r.view = mk(c.dir[0], c.dir[1], c.dir[2]);
    v3 up = mk(c.up[0], c.up[1], c.up[2]);
    camera_frame(r.view, up, &r.U, &r.V, &r.W);
    double half = (double)c.fovy_deg / 2.0;
    r.height = (float)std::tan(3.14159265358979323846 * half / 180.0);
    float aspect = (float)w / (float)h;
    r.width = aspect * r.height;
    r.aperture = c.aperture;
    r.focus = c.focus_distance;
    r.w = w; r.h = h;
    return r;
}

// Jump matrices for `steps` MRG32k3a steps (mrg_power of the one-step
// matrices, gbpt_math.h).
static inline void mrg_jump_matrices(uint64_t steps, uint32_t J1[9], uint32_t J2[9]) {
    mrg_power(kMrgA1, steps, J1, 209u, kMrgM1);
    mrg_power(kMrgA2, steps, J2, 22853u, kMrgM2);
}

static inline ShadeParams make_shade_params(const gb_render_desc& d) {
    ShadeParams s;
    s.ray_offset = d.ray_offset;
    s.shadow_offset = d.shadow_offset;
    s.background = mk(d.background[0], d.background[1], d.background[2]);
    s.rr_start = d.rr_start;
    s.seed = d.seed;
    return s;
}

}  // namespace gb
