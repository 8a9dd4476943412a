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
    // records the BRDF values and light emission are evaluated with: the same
    // as mats / lights, except in a frozen-sampling replay (directions,
    // lobes, pdfs and light picks still come from mats / lights)
    const float* mats_eval;
    const LightRec* lights_eval;
    SkyRec sky;  // the scene's sky light (sky.light = -1 when it has none)
    // textures: 6 texture coordinates per canonical triangle (null when the
    // scene has none; then no ray differentials are kept either)
    const float* texcoord;
    const TexRec* tex;
    int n_tex;
};

// The six 32-bit component words of a curandStateMRG32k3a (s1[3], s2[3]):
// all a uniform draw reads and writes, stored in 24 bytes instead of 48.
struct MrgState {
    uint32_t s1[3], s2[3];
};

// Status bits written by the kernels (never a trap).
enum { ST_STACK_OVERFLOW = 1u, ST_ITER_LIMIT = 2u };

// One scene of a frame (single renders are a frame of one scene; batches
// have many): geometry, camera, shading parameters and its pixel range.
struct SceneRec {
    DevScene S;
    CameraRec cam;
    ShadeParams sp;
    int w, h, n;        // resolution, pixels
    int spp, L, rng_mode;
    uint32_t pixel_base;  // first global pixel of the scene
    uint32_t seed;
    uint32_t jump1[9], jump2[9];  // MRG32k3a jump by the 3 L draws of one path
    int n_mats;
    uint32_t grad_base;   // first record-gradient float of the scene (adjoint)
};

// Render modes of a chunk.
enum { MODE_FORWARD = 0, MODE_FROZEN = 1, MODE_ADJOINT = 2 };
constexpr int kAdjPlanes = 5;        // float4 planes of one adjoint vertex record
constexpr int kMaxAdjBounces = 16;   // bounces the adjoint records per path
constexpr int kAdjMaxSlots = 1 << 22;  // slots of an adjoint chunk (vertex records: 80 B x bounces each)

constexpr int kMaxRounds = 64;  // path samples per chunk

// Per-slot state of the wavefront: one 256-byte record per path slot.
// Slots are visited in queue order, which is not slot order, so every field
// access of a slot is a scattered access.  A record keeps what one stage
// reads or writes together in one 128-byte line, so that a stage touches a
// few whole 32-byte sectors of a slot instead of one partly used sector per
// field, and the kernels write whole sectors (a partly written sector costs
// DRAM a read-modify-write when it leaves the L2):
//   line 0 (path state: written by path start and by shading)
//     0 ray_o, 16 ray_d (w: pb), 32 tp, 48 accum, 64 pix, 68 ps, 72 zero,
//     80 rdiff[0..2] (ray differentials of textured scenes; rdiff[0] is
//     zeroed at path start otherwise)
//   line 1 (hit record: written by the closest-hit kernel)
//     128 hit_p, 144 hit_n, 160 sh_o, 176 sh_d, 192 psc, 208 rnd,
//     224 rng (+ 8 zero bytes)
constexpr size_t kSlotBytes = 256;
// GB_SHADOW_SPLIT: shadow rays (sh_o, sh_d) in their own 32-byte-per-slot
// array instead of the hit line
#ifndef GB_SHADOW_SPLIT
#define GB_SHADOW_SPLIT 0
#endif
constexpr size_t kShadowStride = GB_SHADOW_SPLIT ? 32 : kSlotBytes;
enum : size_t {
    kSlotRayO = 0, kSlotRayD = 16, kSlotPb = 28, kSlotTp = 32, kSlotAccum = 48, kSlotPix = 64, kSlotPs = 68,
    kSlotRdiff = 80, kSlotHitP = 128, kSlotHitN = 144, kSlotShO = 160, kSlotShD = 176, kSlotPsc = 192,
    kSlotRnd = 208, kSlotRng = 224
};
static_assert(kSlotRdiff + 48 <= 128 && kSlotRng + 24 <= kSlotBytes, "slot record layout");

// Loads and stores of the per-iteration state stream (slot records, samples,
// jitter pool, stream cursors) carry the cache-streaming hint (ld.cs /
// st.cs: lines allocated evict-first in L1 and L2), so that the state
// streaming through every iteration -- several times the L2 -- is evicted
// before the scene's nodes and triangles.  GB_REC_EVICT_FIRST=0 makes them
// plain accesses.
#ifndef GB_REC_EVICT_FIRST
#define GB_REC_EVICT_FIRST 1
#endif
#ifndef GB_HIT_LINE_KEEP
#define GB_HIT_LINE_KEEP 0
#endif
#ifdef __CUDACC__
template <class T>
__device__ __forceinline__ T rec_ld(const T* p) {
#if GB_REC_EVICT_FIRST
    return __ldcs(p);
#else
    return *p;
#endif
}
template <class T>
__device__ __forceinline__ void rec_st(T* p, const T& v) {
#if GB_REC_EVICT_FIRST
    __stcs(p, v);
#else
    *p = v;
#endif
}
#endif

// One field of the slot records: f[slot] is that field of record `slot`;
// f.ld(slot) / f.st(slot, v) are the stream accesses (rec_ld / rec_st).
template <class T, size_t Stride = kSlotBytes>
struct SlotField {
    unsigned char* base = nullptr;  // the field in record 0
#ifdef __CUDACC__
    __host__ __device__
#endif
    inline T& operator[](size_t slot) const {
        return *reinterpret_cast<T*>(base + slot * Stride);
    }
#ifdef __CUDACC__
    __device__ inline T ld(size_t slot) const { return rec_ld(reinterpret_cast<const T*>(base + slot * Stride)); }
    __device__ inline void st(size_t slot, const T& v) const {
        rec_st(reinterpret_cast<T*>(base + slot * Stride), v);
    }
    // the hit line the closest-hit kernel writes and the any-hit and
    // shading kernels of the same iteration read back (GB_HIT_LINE_KEEP:
    // with normal L2 priority instead of evict-first)
    __device__ inline void st_hit(size_t slot, const T& v) const {
#if GB_HIT_LINE_KEEP
        *reinterpret_cast<T*>(base + slot * Stride) = v;
#else
        rec_st(reinterpret_cast<T*>(base + slot * Stride), v);
#endif
    }
#endif
};

// Wavefront state: per path slot (records above) and per global pixel.
struct Frame {
    int ntot;          // pixels of all scenes
    int nslots;        // path slots in flight
    const SceneRec* scenes;  // device array
    int nscenes;
    // per slot: nslots records of kSlotBytes at `slots`, viewed field by field
    unsigned char* slots;
    SlotField<float4> ray_o;     // origin xyz, t_max
    SlotField<float4> ray_d;     // direction xyz
    SlotField<float4> tp;        // throughput
    SlotField<float4> accum;     // col_accum of the slot's path
    SlotField<float4, kShadowStride> sh_o;  // shadow origin xyz, max_t
    SlotField<float4, kShadowStride> sh_d;  // shadow direction xyz (to_light), w = occluded
    unsigned char* shadow;       // the shadow-ray array (GB_SHADOW_SPLIT), else null
    SlotField<float4> psc;       // potential_sample_contribution
    SlotField<float4> rnd;       // path draw of this bounce
    SlotField<float4> hit_p;     // hit point xyz | material index bits
    SlotField<float4> hit_n;     // interpolated (unnormalised) normal | hit triangle id bits
    SlotField<float4> rdiff[3];  // ray differentials of textured scenes (RayDiff packed)
    SlotField<MrgState> rng;     // light/path stream of the slot's path
    SlotField<uint32_t> pix;     // global pixel of the slot's path
    SlotField<uint32_t> ps;      // scene of the slot's path
    SlotField<uint32_t> pb;      // path index << 10 | bounce (the bits of ray_d.w)
    SlotField<uint4> pixw;       // (pix, ps, 0, 0) as one 16-byte word
    uint32_t* q[4];    // queues: extension (ping/pong), shadow, ended paths; nslots entries each
    // per global pixel
    float4* out;       // output_color (moving average)
    MrgState* pristine;  // stream after curand_init(seed, pixel, 0)
    MrgState* cursor;    // light/path stream at the pixel's next chunk
    MrgState* jcursor;   // camera-jitter stream at the pixel's next chunk
    uint32_t* pscene;  // scene of each pixel
    float4* samples;   // sample of path l of the chunk (l = round_start[r] + pixel)
    float4* jpool;     // camera jitter of path l of the chunk
    MrgState* spool;   // light/path stream state at the start of path l of the chunk
    // control
    uint32_t* ctr;     // 3 sets of 8 (by iteration % 3): count, ext head, shadow count, shadow head, ended
    uint32_t* path_ctr;  // next path of the chunk to start
    int* iter;         // iteration index of the chunk's slot-pool loop
    unsigned long long* stats;  // 0 camera, 1 ext, 2 shadow rays; 3/4 closest, 5/6 shadow node visits / tri tests;
                                // 7 iterations; 8 closest hits (light samples); 16 words
    uint32_t* status;
    // frozen-sampling replay: throughput of the path under the sampling records
    float4* tp0;
    // adjoint: vertex records [bounce][plane][slot], per-pixel loss gradient
    // (already divided by spp), per-block gradient replicas of the record fields
    float4* adj;
    float4* dimg;
    float* grad;
    int grad_stride;   // floats per replica
    int grad_replicas;
};

// Points the slot fields of F at the records at `slots` (kSlotBytes-aligned)
// and, with GB_SHADOW_SPLIT, the shadow rays at `shadow` (nslots * 32 bytes).
inline void bind_slots(Frame& F, unsigned char* slots, unsigned char* shadow) {
    F.slots = slots;
    auto at = [slots](size_t off) { return slots ? slots + off : nullptr; };
    F.ray_o.base = at(kSlotRayO);
    F.ray_d.base = at(kSlotRayD);
    F.tp.base = at(kSlotTp);
    F.accum.base = at(kSlotAccum);
    F.pix.base = at(kSlotPix);
    F.ps.base = at(kSlotPs);
    F.pb.base = at(kSlotPb);
    F.pixw.base = at(kSlotPix);
    for (int k = 0; k < 3; ++k) F.rdiff[k].base = at(kSlotRdiff + 16 * (size_t)k);
    F.hit_p.base = at(kSlotHitP);
    F.hit_n.base = at(kSlotHitN);
    F.shadow = GB_SHADOW_SPLIT ? shadow : nullptr;
    F.sh_o.base = GB_SHADOW_SPLIT ? shadow : at(kSlotShO);
    F.sh_d.base = GB_SHADOW_SPLIT ? (shadow ? shadow + 16 : nullptr) : at(kSlotShD);
    F.psc.base = at(kSlotPsc);
    F.rnd.base = at(kSlotRnd);
    F.rng.base = at(kSlotRng);
}

// Launch-wide parameters of one chunk.
struct RenderParams {
    int refill;        // refill a warp's lanes once this many are idle (1..32)
    int tri_mode;      // 0: all pending triangles then a node; 1/2: triangle postponing, one / all triangles;
                       // 3: warp-cooperative triangle tests, then a node
    int blocks_per_sm; // resident blocks per SM of the traversal kernels (0 = occupancy limit)
    int sampling_terms; // adjoint: add the derivatives of the sampling decisions (sampling_scores)
    int trav_variant;  // traversal kernels of the default triangle policy: stack entries / threads per
                       // block 0: 32 / 128, 1: 24 / 128, 2: 32 / 64, 3: 24 / 64
    int mode;          // MODE_*
    int textured;      // some scene of the frame has textures (k_shade's texture variant)
    int p0, rounds;    // path samples p0 .. p0+rounds-1
    // L2 window of the traversal launches (GB_NODE_L2_PERSIST, frames of one
    // scene): the scene's node array, accessed as persisting
    const void* l2_nodes;
    unsigned long long l2_nodes_bytes;
    float l2_hit_ratio;  // fraction of the window's accesses that persist
    uint32_t chunk_paths;  // paths of the chunk
    uint32_t round_start[kMaxRounds + 1];  // first path index of each round (prefix sums of N_p)
};

cudaError_t k_launch_trace(const DevScene& S, int n, const float* orig, const float* dir, const float* tmax,
                           float4* hits, uint8_t* occluded, bool any, uint32_t* status, cudaStream_t st);
cudaError_t k_launch_frame_init(const Frame& F, bool rng, cudaStream_t st);
cudaError_t k_launch_start(const Frame& F, const RenderParams& P, int nstart, cudaStream_t st);
cudaError_t k_launch_extend(const Frame& F, const RenderParams& P, bool instrument, cudaStream_t st);
cudaError_t k_launch_shadow(const Frame& F, const RenderParams& P, bool instrument, cudaStream_t st);
cudaError_t k_launch_shade(const Frame& F, const RenderParams& P, cudaStream_t st);
cudaError_t k_launch_regen(const Frame& F, const RenderParams& P, cudaStream_t st);
cudaError_t k_launch_step(const Frame& F, const RenderParams& P, unsigned long long cond, bool has_cond,
                          int max_iters, cudaStream_t st);
cudaError_t k_launch_jitter_pool(const Frame& F, const RenderParams& P, cudaStream_t st);
cudaError_t k_launch_combine(const Frame& F, const RenderParams& P, cudaStream_t st);
cudaError_t k_launch_pack_rgb(const float4* src, int n, float* dst, cudaStream_t st);
cudaError_t k_launch_adjoint(const Frame& F, const RenderParams& P, cudaStream_t st);
cudaError_t k_launch_direct(const DevScene& S, const CameraRec& cam, int w, int h, int samples, uint32_t seed,
                            float shadow_offset, v3 background, float* out, uint32_t* status, cudaStream_t st);
cudaError_t k_launch_direct_hybrid(const DevScene& S, const CameraRec& cam, int w, int h, int cam_samples,
                                   int light_samples, uint32_t seed, float shadow_offset, v3 background, float* out,
                                   uint32_t* status, cudaStream_t st);
int k_adjoint_grid();
cudaError_t k_launch_dimg_pack(const float* src, int n, float scale, float4* dst, cudaStream_t st);
cudaError_t k_launch_grad_reduce(const float* grad, int replicas, int stride, double* out, cudaStream_t st);
cudaError_t k_launch_l2_loss(const float* img, const float* target, int n, float scale, float4* dimg, double* loss,
                             cudaStream_t st);
// Kernel launches of one slot-pool iteration in a render mode.
int k_launches_per_iteration(int mode);
cudaError_t k_launch_mrg_states(uint32_t seed, const uint32_t* sub, int n, int method, uint32_t* out,
                                cudaStream_t st);
cudaError_t k_launch_mrg_pool(int pixel0, int npix, uint32_t seed, int first_update, int num_updates, float* out,
                              cudaStream_t st);
cudaError_t k_launch_nee_stage(const DevScene& S, int n, float shadow_offset, const float* rnd, const float4* hits,
                               float* ray_orig, float* ray_dir, float* max_t, float* psc, cudaStream_t st);
cudaError_t k_launch_shade_stage(const DevScene& S, int n, const ShadeParams& sp, float* ray_orig, float* ray_dir,
                                 float* max_t, const float4* hits, const uint8_t* occl, const float* rnd,
                                 float* tp, float* accum, const float* to_light, const float* psc, int path,
                                 int bounce, cudaStream_t st);

}  // namespace gb
