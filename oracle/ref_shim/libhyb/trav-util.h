// Shim for libhyb's trav-util.h: the vector helpers the reference sources
// call, with the definitions of globillum_gb300/csrc/gbpt_math.h (Duff et
// al. 2017 tangent frame; bc.x*a + bc.y*b + bc.z*c; division by the length).
// Test infrastructure only.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include "../librta/cuda-vec.h"

namespace rta {
inline float clamp(float a, float lo, float hi) { return fminf(fmaxf(a, lo), hi); }
}  // namespace rta

inline void make_tangent_frame(const float3 &n, float3 &T, float3 &B) {
    float sign = copysignf(1.0f, n.z);
    float a = -1.0f / (sign + n.z);
    float b = n.x * n.y * a;
    T = make_float3(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x);
    B = make_float3(b, sign + n.y * n.y * a, -n.y);
}
inline float3 make_tangential(const float3 &v, const float3 &n) {
    float3 T, B;
    make_tangent_frame(n, T, B);
    return (v.x * T + v.y * B) + v.z * n;
}
inline float3 transform_to_tangent_frame(const float3 &v, const float3 &T, const float3 &B, const float3 &N) {
    return make_float3(v | T, v | B, v | N);
}
inline float3 transform_from_tangent_frame(const float3 &v, const float3 &T, const float3 &B, const float3 &N) {
    return (v.x * T + v.y * B) + v.z * N;
}
inline float3 reflect(const float3 &v, const float3 &n) { return v - (2.0f * (v | n)) * n; }
inline float length_of_vector(const float3 &v) { return sqrtf(v | v); }
inline void normalize_vec3f(float3 *v) { float l = length_of_vector(*v); *v = *v / l; }
inline void barycentric_interpolation(float3 *out, const float3 *bc, const float3 *a, const float3 *b, const float3 *c) {
    *out = (bc->x * *a + bc->y * *b) + bc->z * *c;
}
inline void barycentric_interpolation(float2 *out, const float3 *bc, const float2 *a, const float2 *b, const float2 *c) {
    *out = make_float2((bc->x * a->x + bc->y * b->x) + bc->z * c->x, (bc->x * a->y + bc->y * b->y) + bc->z * c->y);
}
