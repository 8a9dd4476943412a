// Shim for rta's cuda-kernels.h: the triangle / hit records the reference
// sources use.  Test infrastructure only.
#pragma once
#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>
#include <stdexcept>
#include <string>

#define heterogenous
#define checked_cuda(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) throw std::runtime_error(cudaGetErrorString(e_)); } while (0)
typedef unsigned int uint;

namespace rta {
namespace cuda {
struct simple_triangle {
    float3 a, b, c, na, nb, nc;
    float2 ta, tb, tc;
    int material_index;
};
}  // namespace cuda

template <typename tri_t> struct triangle_intersection {
    float t, beta, gamma;
    uint ref;
    triangle_intersection() : t(FLT_MAX), beta(0), gamma(0), ref(0xffffffffu) {}
    explicit triangle_intersection(uint r) : t(FLT_MAX), beta(0), gamma(0), ref(r) {}
    bool valid() const { return t < FLT_MAX; }
    // bc = (1 - beta - gamma, beta, gamma)
    void barycentric_coord(float3 *bc) const { bc->x = (1.0f - beta) - gamma; bc->y = beta; bc->z = gamma; }
};
}  // namespace rta
