// gbpt_kernels.h -- device data views and launch wrappers of the sm_103a
// kernels (gbpt_kernels.cu).  Host code only sees plain pointers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gbpt_math.h"

namespace gb {

// Resident scene (device pointers).
struct DevScene {
    const float4* nodes;     // 5 float4 per 8-wide node
    const float4* tris;      // 3 float4 per triangle (v0|id, e1, e2), leaf order
    const float4* shade;     // 6 float4 per canonical triangle: a|mat, b, c, na, nb, nc
    const float* mats;       // kMaterialFloats per material
    const LightRec* lights;
    int n_lights;
    float overall_power;
    int n_nodes, n_tris;
};

// Status bits written by the kernels (never a trap).
enum { ST_STACK_OVERFLOW = 1u, ST_ITER_LIMIT = 2u };

// Per-pixel wavefront state (SoA, one entry per pixel of the frame).
struct Frame {
    int w, h, n;
    float4* ray_o;     // origin xyz, t_max
    float4* ray_d;     // direction xyz
    float4* tp;        // throughput
    float4* accum;     // col_accum of the current path
    float4* out;       // output_color (moving average)
    float4* sh_o;      // shadow origin xyz, max_t
    float4* sh_d;      // shadow direction xyz (to_light)
    float4* psc;       // potential_sample_contribution
    float4* rnd;       // path draw of this bounce
    float4* hit_p;     // hit point xyz | material index bits
    float4* hit_n;     // interpolated (unnormalised) normal
    void* rng;         // curandStateMRG32k3a[n], light/path stream
    void* rngj;        // curandStateMRG32k3a[n], camera-jitter stream
    int* draws;        // updates consumed by `rng`
    float4* jpool;     // jitter pool (thin lens only)
    uint32_t* q[3];    // ray queues: extension (ping/pong) and shadow
    uint32_t* ctr;     // per bounce: [4*b+0] ext count, +1 ext head, +2 shadow count, +3 shadow head
    unsigned long long* stats;  // 0 camera, 1 ext, 2 shadow rays; 3/4 closest, 5/6 shadow node visits / tri tests
    uint32_t* status;
};

struct RenderParams {
    CameraRec cam;
    ShadeParams sp;
    int spp, L, rng_mode;
    uint32_t seed;
};

int launch_grid_size();  // persistent grid (blocks) for the queue kernels

cudaError_t k_launch_trace(const DevScene& S, int n, const float* orig, const float* dir, const float* tmax,
                           float4* hits, uint8_t* occluded, bool any, uint32_t* status, cudaStream_t st);
cudaError_t k_launch_rng_init(const Frame& F, uint32_t seed, cudaStream_t st);
cudaError_t k_launch_raygen(const Frame& F, const RenderParams& P, int path, cudaStream_t st);
cudaError_t k_launch_extend(const DevScene& S, const Frame& F, const RenderParams& P, int path, int bounce,
                            bool instrument, cudaStream_t st);
cudaError_t k_launch_shade(const DevScene& S, const Frame& F, const RenderParams& P, int path, int bounce,
                           bool instrument, cudaStream_t st);
cudaError_t k_launch_finalize(const Frame& F, int path, cudaStream_t st);
cudaError_t k_launch_pack_rgb(const float4* src, int n, float* dst, cudaStream_t st);
cudaError_t k_launch_mrg_pool(int npix, uint32_t seed, int first_update, int num_updates, float* out,
                              cudaStream_t st);
cudaError_t k_launch_nee_stage(const DevScene& S, int n, float shadow_offset, const float* rnd, const float4* hits,
                               float* ray_orig, float* ray_dir, float* max_t, float* psc, cudaStream_t st);
cudaError_t k_launch_shade_stage(const DevScene& S, int n, const ShadeParams& sp, float* ray_orig, float* ray_dir,
                                 float* max_t, const float4* hits, const uint8_t* occl, const float* rnd,
                                 float* tp, float* accum, const float* to_light, const float* psc, int path,
                                 int bounce, cudaStream_t st);

}  // namespace gb
