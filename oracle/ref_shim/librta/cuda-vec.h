// Shim for rta's cuda-vec.h: float2/float3 operators as used by the
// reference sources (operator| is the dot product).  Test infrastructure only.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

inline float3 operator+(const float3 &a, const float3 &b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline float3 operator-(const float3 &a, const float3 &b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline float3 operator-(const float3 &a) { return make_float3(-a.x, -a.y, -a.z); }
inline float3 operator*(const float3 &a, const float3 &b) { return make_float3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline float3 operator*(float s, const float3 &a) { return make_float3(s * a.x, s * a.y, s * a.z); }
inline float3 operator*(const float3 &a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
inline float3 operator/(const float3 &a, float s) { return make_float3(a.x / s, a.y / s, a.z / s); }
inline float3 operator/(const float3 &a, const float3 &b) { return make_float3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline float3 &operator+=(float3 &a, const float3 &b) { a = a + b; return a; }
inline float3 &operator-=(float3 &a, const float3 &b) { a = a - b; return a; }
inline float3 &operator*=(float3 &a, float s) { a = a * s; return a; }
inline float3 &operator*=(float3 &a, const float3 &b) { a = a * b; return a; }
inline float3 &operator/=(float3 &a, float s) { a = a / s; return a; }
inline float operator|(const float3 &a, const float3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float2 operator+(const float2 &a, const float2 &b) { return make_float2(a.x + b.x, a.y + b.y); }
inline float2 operator*(float s, const float2 &a) { return make_float2(s * a.x, s * a.y); }
