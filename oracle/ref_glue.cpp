// ref_glue.cpp -- C entry points around the reference's own code, compiled
// in place from the reference tree by oracle/build_ref.py together with
// arealight-sampler-cpu.cpp (TEST INFRASTRUCTURE ONLY: used by the pinning
// tests and by tests/golden/make_golden.py, never by the product).
//
// The shading entry point repeats the reference's per-pixel call sequence
// of sample_material + evaluate_material (hybrid-pt.cpp:330-371, with the
// tangent frame of :525-528) around the reference's materialBRDF
// (material-wrapper.h:15-51, principledMaterial.h, simpleMaterial.h); the
// light entry point calls rta::generate_arealight_sample
// (arealight-sampler-cpu.cpp:144-156) unchanged.
#include "config.h"

#include <librta/cuda-kernels.h>
#include <librta/cuda-vec.h>
#include <libhyb/trav-util.h>

#include "util.h"
#include "lights.h"
#include "material.h"
#include "material-wrapper.h"
#include "arealight-sampler.h"

#include <vector>

namespace {
// Field order of gb_principled_params (include/gbpt.h).
struct Params {
    float metallic, subsurface, specular, roughness, specular_tint, anisotropic;
    float sheen, sheen_tint, clearcoat, clearcoat_gloss, opacity, transmiss;
    float color[3];
    float tangent[3];
};
// Field order of gb_light.
struct Light {
    int type;
    float power;
    float center[3], dir[3], up[3], col[3];
    float wh[2];
};
inline float3 f3(const float* p) { return make_float3(p[0], p[1], p[2]); }
inline void put(float* p, const float3& v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }
}  // namespace

extern "C" {

// One shading evaluation: out[0..2] sampled world direction, out[3] pdf,
// out[4..6] brdf towards it, out[7..9] brdf towards `to_light`, out[10]
// glass flag.  n_raw: interpolated normal; ray_dir: incoming ray.
int ref_shade_eval(const float* diffuse, int principled, const Params* pp, const float* n_raw,
                   const float* ray_dir, const float* rnd, const float* to_light, float* out) {
    rta::cuda::material_t mat;
    rta::PrincipledBRDFParameters params;
    mat.diffuse_color = f3(diffuse);
    if (principled) {
        params.metallic = pp->metallic; params.subsurface = pp->subsurface; params.specular = pp->specular;
        params.roughness = pp->roughness; params.specularTint = pp->specular_tint;
        params.anisotropic = pp->anisotropic; params.sheen = pp->sheen; params.sheenTint = pp->sheen_tint;
        params.clearcoat = pp->clearcoat; params.clearcoatGloss = pp->clearcoat_gloss;
        params.opacity = pp->opacity; params.transmiss = pp->transmiss;
        params.color = f3(pp->color); params.tangent = f3(pp->tangent);
        mat.parameters = &params;
    }
    // hybrid-pt.cpp:430, :470-472, :525-530
    float3 N = f3(n_raw);
    normalize_vec3f(&N);
    float3 org_dir = f3(ray_dir);
    normalize_vec3f(&org_dir);
    float3 T, B;
    make_tangent_frame(N, T, B);
    normalize_vec3f(&T);
    normalize_vec3f(&B);
    float2 tc = make_float2(0.0f, 0.0f);
    materialBRDF m;
    m.init(principled != 0, false, &mat, tc, tc, tc, T, B);
    // sample_material (hybrid-pt.cpp:330-349)
    float3 random = f3(rnd);
    float pdf = 1.f;
    bool enterGlass = true;
    float3 inv_org_dir = -1.0f * org_dir;
    if ((org_dir | N) > 0.0f) {
        if (m.isGlass()) { enterGlass = false; N *= -1.f; }
        else N *= -1.f;
    }
    float3 wo_ts = transform_to_tangent_frame(inv_org_dir, T, B, N);
    float3 wi;
    m.sample(wo_ts, wi, random, pdf, enterGlass);
    wi = transform_from_tangent_frame(wi, T, B, N);
    normalize_vec3f(&wi);
    // evaluate_material (hybrid-pt.cpp:351-371)
    float3 ld = f3(to_light);
    normalize_vec3f(&ld);
    float3 fl = m.evaluate(inv_org_dir, ld, N);
    float3 fw = m.evaluate(inv_org_dir, wi, N);
    put(out, wi);
    out[3] = pdf;
    put(out + 4, fw);
    put(out + 7, fl);
    out[10] = m.isGlass() ? 1.0f : 0.0f;
    return 0;
}

// rta::generate_arealight_sample on n pixels (a 1 x n grid).  tris: 18
// floats per triangle (a, b, c, na, nb, nc); hits: (t, beta, gamma, ref).
int ref_generate_arealight_sample(int n, const Light* lights, int nl, float overall_power, const float* tris,
                                  int ntris, const void* hits, const float* rnd, float* ray_orig, float* ray_dir,
                                  float* max_t, float* psc) {
    std::vector<gi::light> L(nl);
    for (int i = 0; i < nl; ++i) {
        L[i].type = gi::light::rect;
        L[i].power = lights[i].power;
        L[i].rectlight.center = f3(lights[i].center);
        L[i].rectlight.dir = f3(lights[i].dir);
        L[i].rectlight.up = f3(lights[i].up);
        L[i].rectlight.col = f3(lights[i].col);
        L[i].rectlight.wh = make_float2(lights[i].wh[0], lights[i].wh[1]);
    }
    std::vector<rta::cuda::simple_triangle> T(ntris);
    for (int t = 0; t < ntris; ++t) {
        const float* p = tris + 18 * (size_t)t;
        T[t].a = f3(p); T[t].b = f3(p + 3); T[t].c = f3(p + 6);
        T[t].na = f3(p + 9); T[t].nb = f3(p + 12); T[t].nc = f3(p + 15);
        T[t].ta = T[t].tb = T[t].tc = make_float2(0.0f, 0.0f);
        T[t].material_index = 0;
    }
    typedef rta::triangle_intersection<rta::cuda::simple_triangle> ti_t;
    std::vector<ti_t> H(n);
    const float* h = (const float*)hits;
    for (int i = 0; i < n; ++i) {
        H[i].t = h[4 * i]; H[i].beta = h[4 * i + 1]; H[i].gamma = h[4 * i + 2];
        H[i].ref = ((const uint32_t*)h)[4 * i + 3];
    }
    rta::generate_arealight_sample(n, 1, L.data(), nl, overall_power, (float3*)ray_orig, (float3*)ray_dir, max_t,
                                   H.data(), T.data(), (float3*)rnd, (float3*)psc);
    return 0;
}

}  // extern "C"
