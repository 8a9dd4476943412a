// gbpt_api.cpp -- C ABI of libgbpt.so (include/gbpt.h): contexts, resident
// scenes, the progressive wavefront frame, tracing and per-stage entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/gbpt.h"
#include "gbpt_build.h"
#include "gbpt_bvh.h"
#include "gbpt_host.h"
#include "gbpt_kernels.h"

using namespace gb;

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

static const int kSnaps = 16;
static const size_t kMaxGraphs = 16;

// One scene of a frame as the host sees it.
struct BatchScene {
    gb_scene* scene = nullptr;
    gb_camera cam{};
    gb_render_desc desc{};
    float* out = nullptr;   // gb_render_batch output (host or device)
    int n = 0;              // pixels
    uint32_t base = 0;      // first pixel of the scene in the frame
    // frozen-sampling replay: records the BRDFs / emission are evaluated with
    const float* mats_eval = nullptr;
    const LightRec* lights_eval = nullptr;
    // adjoint: loss gradient of the image, parameter gradient output and the
    // scene's first record-gradient float
    const float* dimg = nullptr;
    float* grad_out = nullptr;
    uint32_t grad_base = 0;
    // fitting step (gb_fit_*): target image (device), image output (device or
    // null) and the scene's index in the caller's list
    const float* target = nullptr;
    float* image = nullptr;
    int user = 0;
};

// An instantiated chunk graph and everything it was captured with.
struct ChunkGraph {
    std::vector<uint64_t> key;
    cudaGraphExec_t exec;
};

// A prepared fitting step (gb_fit_prepare): the scenes in layout order, the
// one graph of a step, and the pinned buffers it copies from and to.
struct FitState {
    bool ready = false;
    std::vector<BatchScene> items;      // layout order
    std::vector<gb_fit_item> user;      // as the caller gave them
    cudaGraphExec_t exec = nullptr;
    std::vector<uint64_t> key;          // device buffers the graph was captured with
    SceneRec* h_recs = nullptr;         // scene records of the frame
    float* h_mats = nullptr;            // material records of every scene
    LightRec* h_lights = nullptr;       // light records of every scene
    std::vector<size_t> mat_off, light_off;
    double* h_out = nullptr;            // gradient sums (stride), then one loss per scene
    double* d_loss = nullptr;
    int stride = 0, replicas = 0;
    size_t mats_total = 0, lights_total = 0;
};

struct gb_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t aux = nullptr;         // capture stream of the chunk graphs
    bool own_stream = false;
    std::string err;
    // frame: per-slot, per-pixel, sample-buffer and scene-record capacities
    Frame F{};
    size_t slot_cap = 0, pixel_cap = 0, sample_cap = 0, scenes_cap = 0;
    std::vector<void*> slot_allocs, pixel_allocs, sample_allocs;
    SceneRec* d_scenes = nullptr;
    // current frame: one scene (gb_render*) or a batch, in layout order (spp descending)
    std::vector<BatchScene> items;
    std::vector<SceneRec> recs;
    int max_spp = 0, max_L = 0;
    int paths_done = 0;                 // rounds done
    bool active = false;
    bool instrument = false;
    bool use_graph = true;              // run chunks as CUDA graphs (conditional while loop)
    int mode = MODE_FORWARD;            // render mode of the next chunks
    // frozen-sampling replay and adjoint buffers
    std::vector<void*> adj_allocs;
    size_t tp0_cap = 0, adj_cap = 0, dimg_cap = 0, grad_cap = 0, gsum_cap = 0;
    double* d_gsum = nullptr;
    float* d_eval_mats = nullptr;
    LightRec* d_eval_lights = nullptr;
    size_t eval_mats_cap = 0, eval_lights_cap = 0;
    std::vector<ChunkGraph> graphs;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    uint32_t* d_status = nullptr;
    unsigned long long* d_stats = nullptr;
    gb_stats stats{};
    uint64_t launches = 0;              // launches outside the slot-pool iterations
    bool stage_timing = false;
    int refill = 20;                    // idle lanes that trigger a warp refill
    int tri_mode = 0;                   // traversal triangle policy (see gb_tuning)
    int blocks_per_sm = 0;              // resident traversal blocks per SM (0 = occupancy limit)
    int stack_depth = 32;               // traversal stack entries (24 or 32)
    int sampling_terms = 0;             // adjoint: add the derivatives of the sampling decisions
    size_t l2_persist = 0;              // persisting L2 set-aside this context asked for (GB_NODE_L2_PERSIST)
    int block_threads = 128;            // threads per traversal block (64 or 128)
    int slots = 1 << 24;                // path slots in flight (upper bound)
    int sample_mb = 1024;               // sample buffer budget (chunk size)
    // queue-count snapshots: pinned ring + events (host stays a few iterations ahead)
    uint32_t* snap_host = nullptr;
    cudaEvent_t snap_ev[kSnaps] = {};
    std::vector<cudaEvent_t> ev_pool;   // stage timing events (pairs)
    std::vector<int> ev_stage;          // stage of each recorded pair
    size_t ev_used = 0;
    // layout (pixels and seed of each scene, in order) whose initial RNG
    // states F.pristine and scene map F.pscene hold
    std::vector<uint64_t> pristine_key;
    // scratch for API calls with host pointers
    DevBuf scratch[4];
    float* d_rgb = nullptr;
    size_t rgb_cap = 0;
    // fitting steps: the loop bodies of the step graph are captured on fit_aux
    cudaStream_t fit_aux = nullptr;
    FitState fit;
};

struct gb_scene {
    gb_ctx* ctx = nullptr;
    DevScene S{};
    std::vector<void*> allocs;
    gb_scene_info info{};
    // host copies of the descriptions the differentiable parameters change
    std::vector<gb_material> mats;
    std::vector<gb_principled_params> params;
    std::vector<gb_light> lights;
    // device-built tree (GB_BVH_DEVICE_PLOC) and what a refit rewrites
    GpuBvh gbvh;
    std::vector<int> material_index;
    void* shade_buf = nullptr;
    size_t tree_bytes = 0;  // host-built tree: nodes then triangles in one allocation at S.nodes
    std::vector<int> mat_dtex;  // diffuse texture of each material (-1 = none)
};

// GB_NODE_L2_PERSIST: a frame of one scene keeps the scene's node array in a
// persisting L2 set-aside (cudaLimitPersistingL2CacheSize, released when the
// context is destroyed), given to the traversal launches as an access-policy
// window
#ifndef GB_NODE_L2_PERSIST
#define GB_NODE_L2_PERSIST 1
#endif
#ifndef GB_TREE_WINDOW
#define GB_TREE_WINDOW 0
#endif

namespace {

int fail(gb_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

int cuda_fail(gb_ctx* c, cudaError_t e, const char* what) {
    cudaGetLastError();
    int code = e == cudaErrorMemoryAllocation ? GB_ERR_OOM : GB_ERR_CUDA;
    return fail(c, code, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                             \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    } while (0)

// Host-side fault injection (gb_set_fault_injection): the k-th device
// allocation from the moment it is armed fails as if the device were full.
std::atomic<long long> g_alloc_countdown{-1};

cudaError_t dalloc(std::vector<void*>& list, void** p, size_t bytes) {
    *p = nullptr;
    if (g_alloc_countdown.load() >= 0 && g_alloc_countdown.fetch_sub(1) == 0) return cudaErrorMemoryAllocation;
    cudaError_t e = cudaMalloc(p, bytes == 0 ? 16 : bytes);
    if (e == cudaSuccess) list.push_back(*p);
    return e;
}

void free_all(std::vector<void*>& list) {
    for (void* p : list) cudaFree(p);
    list.clear();
}

// Allocations of a device BVH build: kept buffers join the scene's list,
// temporaries are freed when the build is done.
struct SceneAllocator : DevAllocator {
    std::vector<void*>& keep;
    std::vector<void*> tmp;
    explicit SceneAllocator(std::vector<void*>& k) : keep(k) {}
    cudaError_t alloc(void** p, size_t bytes, bool k) override { return dalloc(k ? keep : tmp, p, bytes); }
    void release_temps() override { free_all(tmp); }
    ~SceneAllocator() override { free_all(tmp); }
};

// Shading records, canonical triangle order, 24 floats each: the three
// vertices (w of the first = material index bits) and the three normals
// (face normal when none are given).
void make_shade_records(const float* pos, const float* normals, const int* material_index, int n,
                        std::vector<float>* out) {
    std::vector<float>& shade = *out;
    shade.assign((size_t)n * 24, 0.0f);
    for (int t = 0; t < n; ++t) {
        float* s = &shade[(size_t)t * 24];
        const float* p = pos + 9 * (size_t)t;
        float nrm[9];
        if (normals) std::memcpy(nrm, normals + 9 * (size_t)t, sizeof(nrm));
        else {
            v3 fn = normalize_div(cross(mk(p[3] - p[0], p[4] - p[1], p[5] - p[2]), mk(p[6] - p[0], p[7] - p[1], p[8] - p[2])));
            for (int k = 0; k < 3; ++k) { nrm[3 * k] = fn.x; nrm[3 * k + 1] = fn.y; nrm[3 * k + 2] = fn.z; }
        }
        uint32_t mi = (uint32_t)material_index[t];
        for (int v = 0; v < 3; ++v) {
            s[4 * v] = p[3 * v]; s[4 * v + 1] = p[3 * v + 1]; s[4 * v + 2] = p[3 * v + 2]; s[4 * v + 3] = 0.0f;
            s[12 + 4 * v] = nrm[3 * v]; s[12 + 4 * v + 1] = nrm[3 * v + 1]; s[12 + 4 * v + 2] = nrm[3 * v + 2];
            s[12 + 4 * v + 3] = 0.0f;
        }
        std::memcpy(&s[3], &mi, 4);
    }
}

cudaError_t ensure_scratch(gb_ctx* ctx, int k, size_t bytes) {
    if (ctx->scratch[k].bytes >= bytes) return cudaSuccess;
    if (ctx->scratch[k].p) cudaFree(ctx->scratch[k].p);
    ctx->scratch[k].p = nullptr;
    ctx->scratch[k].bytes = 0;
    cudaError_t e = cudaMalloc(&ctx->scratch[k].p, bytes);
    if (e == cudaSuccess) ctx->scratch[k].bytes = bytes;
    return e;
}

// Per-slot buffers for `nslots` slots, per-pixel buffers for `n` pixels,
// sample and jitter buffers of `samples` float4 entries and `nscenes` scene
// records; grown on demand.
cudaError_t ensure_frame(gb_ctx* ctx, int n, int nslots, size_t samples, int nscenes) {
    Frame& F = ctx->F;
    cudaError_t e;
    if ((size_t)nslots > ctx->slot_cap) {
        cudaStreamSynchronize(ctx->stream);
        free_all(ctx->slot_allocs);
        ctx->slot_cap = 0;
        unsigned char *recs = nullptr, *shadow = nullptr;
        if ((e = dalloc(ctx->slot_allocs, (void**)&recs, kSlotBytes * (size_t)nslots)) != cudaSuccess) return e;
        if (GB_SHADOW_SPLIT && (e = dalloc(ctx->slot_allocs, (void**)&shadow, 32 * (size_t)nslots)) != cudaSuccess)
            return e;
        bind_slots(F, recs, shadow);
        for (int k = 0; k < 4; ++k)
            if ((e = dalloc(ctx->slot_allocs, (void**)&F.q[k], 4 * (size_t)nslots)) != cudaSuccess) return e;
        if ((e = dalloc(ctx->slot_allocs, (void**)&F.ctr, 4 * 32)) != cudaSuccess) return e;
        if ((e = dalloc(ctx->slot_allocs, (void**)&F.path_ctr, 4 * 8)) != cudaSuccess) return e;
        if ((e = dalloc(ctx->slot_allocs, (void**)&F.iter, 4 * 8)) != cudaSuccess) return e;
        ctx->slot_cap = (size_t)nslots;
    }
    if ((size_t)n > ctx->pixel_cap) {
        cudaStreamSynchronize(ctx->stream);
        free_all(ctx->pixel_allocs);
        ctx->pixel_cap = 0;
        ctx->pristine_key.clear();
        if ((e = dalloc(ctx->pixel_allocs, (void**)&F.out, sizeof(float4) * (size_t)n)) != cudaSuccess) return e;
        if ((e = dalloc(ctx->pixel_allocs, (void**)&F.pscene, 4 * (size_t)n)) != cudaSuccess) return e;
        if ((e = dalloc(ctx->pixel_allocs, (void**)&F.pristine, sizeof(MrgState) * (size_t)n)) != cudaSuccess) return e;
        if ((e = dalloc(ctx->pixel_allocs, (void**)&F.cursor, sizeof(MrgState) * (size_t)n)) != cudaSuccess) return e;
        if ((e = dalloc(ctx->pixel_allocs, (void**)&F.jcursor, sizeof(MrgState) * (size_t)n)) != cudaSuccess) return e;
        ctx->pixel_cap = (size_t)n;
    }
    if ((size_t)nscenes > ctx->scenes_cap) {
        cudaStreamSynchronize(ctx->stream);
        if (ctx->d_scenes) cudaFree(ctx->d_scenes);
        ctx->d_scenes = nullptr;
        ctx->scenes_cap = 0;
        std::vector<void*> tmp;
        if ((e = dalloc(tmp, (void**)&ctx->d_scenes, sizeof(SceneRec) * (size_t)nscenes)) != cudaSuccess) return e;
        ctx->scenes_cap = (size_t)nscenes;
    }
    if (samples > ctx->sample_cap) {
        cudaStreamSynchronize(ctx->stream);
        free_all(ctx->sample_allocs);
        ctx->sample_cap = 0;
        if ((e = dalloc(ctx->sample_allocs, (void**)&F.samples, sizeof(float4) * samples)) != cudaSuccess) return e;
        if ((e = dalloc(ctx->sample_allocs, (void**)&F.jpool, sizeof(float4) * samples)) != cudaSuccess) return e;
        if ((e = dalloc(ctx->sample_allocs, (void**)&F.spool, sizeof(MrgState) * samples)) != cudaSuccess) return e;
        ctx->sample_cap = samples;
    }
    return cudaSuccess;
}

int check_render_desc(gb_ctx* ctx, const gb_camera* cam, const gb_render_desc* d) {
    if (!cam || !d) return fail(ctx, GB_ERR_INVALID, "null camera or render desc");
    if (d->width <= 0 || d->height <= 0 || (long long)d->width * d->height > (1ll << 28))
        return fail(ctx, GB_ERR_INVALID, "bad resolution");
    if (d->spp <= 0 || d->max_bounces <= 0 || d->max_bounces > 1024)
        return fail(ctx, GB_ERR_INVALID, "bad spp / max_bounces");
    if (d->rng_mode != GB_RNG_MRG32K3A_POOL && d->rng_mode != GB_RNG_HALTON_LIGHT)
        return fail(ctx, GB_ERR_INVALID, "bad rng_mode");
    if (!(cam->fovy_deg > 0.0f && cam->fovy_deg < 180.0f)) return fail(ctx, GB_ERR_INVALID, "bad fovy");
    return GB_OK;
}

int check_status(gb_ctx* ctx) {
    uint32_t st = 0;
    CK(cudaMemcpyAsync(&st, ctx->d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (st) {
        CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(uint32_t), ctx->stream));
        return fail(ctx, GB_ERR_TRAVERSAL,
                    (st & ST_STACK_OVERFLOW) ? "traversal stack overflow" : "traversal iteration bound exceeded");
    }
    return GB_OK;
}

// Stage timing: an event pair around a stage launch (only when enabled).
cudaError_t stage_mark(gb_ctx* ctx, int stage, bool begin) {
    if (!ctx->stage_timing) return cudaSuccess;
    size_t k = begin ? 2 * ctx->ev_used : 2 * ctx->ev_used + 1;
    while (ctx->ev_pool.size() <= k) {
        cudaEvent_t e;
        cudaError_t err = cudaEventCreate(&e);
        if (err != cudaSuccess) return err;
        ctx->ev_pool.push_back(e);
    }
    cudaError_t err = cudaEventRecord(ctx->ev_pool[k], ctx->stream);
    if (!begin) {
        if (ctx->ev_stage.size() <= ctx->ev_used) ctx->ev_stage.resize(ctx->ev_used + 1);
        ctx->ev_stage[ctx->ev_used] = stage;
        ctx->ev_used++;
    }
    return err;
}

}  // namespace

extern "C" {

int gb_ctx_create(const gb_ctx_desc* desc, gb_ctx** out) {
    if (!out) return GB_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return GB_ERR_UNSUPPORTED;
    }
    int dev = desc ? desc->device : 0;
    if (dev < 0 || dev >= ndev) return GB_ERR_INVALID;
    gb_ctx* ctx = new (std::nothrow) gb_ctx();
    if (!ctx) return GB_ERR_OOM;
    ctx->device = dev;
    cudaError_t e = cudaSetDevice(dev);
    if (e == cudaSuccess) {
        if (desc && desc->stream) ctx->stream = (cudaStream_t)desc->stream;
        else { e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking); ctx->own_stream = true; }
    }
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->aux, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_status, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_stats, sizeof(unsigned long long) * 16);
    if (e == cudaSuccess) e = cudaMemset(ctx->d_status, 0, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(ctx->d_stats, 0, sizeof(unsigned long long) * 16);
    if (e == cudaSuccess) e = cudaHostAlloc((void**)&ctx->snap_host, sizeof(uint32_t) * kSnaps, cudaHostAllocDefault);
    for (int k = 0; k < kSnaps && e == cudaSuccess; ++k) e = cudaEventCreateWithFlags(&ctx->snap_ev[k], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        cudaGetLastError();
        gb_ctx_destroy(ctx);
        return e == cudaErrorMemoryAllocation ? GB_ERR_OOM : GB_ERR_CUDA;
    }
    *out = ctx;
    return GB_OK;
}

void gb_ctx_destroy(gb_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    free_all(ctx->slot_allocs);
    free_all(ctx->pixel_allocs);
    free_all(ctx->sample_allocs);
    for (ChunkGraph& g : ctx->graphs) cudaGraphExecDestroy(g.exec);
    if (ctx->fit.exec) cudaGraphExecDestroy(ctx->fit.exec);
    if (ctx->fit.h_recs) cudaFreeHost(ctx->fit.h_recs);
    if (ctx->fit.h_mats) cudaFreeHost(ctx->fit.h_mats);
    if (ctx->fit.h_lights) cudaFreeHost(ctx->fit.h_lights);
    if (ctx->fit.h_out) cudaFreeHost(ctx->fit.h_out);
    if (ctx->fit.d_loss) cudaFree(ctx->fit.d_loss);
    if (ctx->fit_aux) cudaStreamDestroy(ctx->fit_aux);
    free_all(ctx->adj_allocs);
    if (ctx->d_scenes) cudaFree(ctx->d_scenes);
    if (ctx->aux) cudaStreamDestroy(ctx->aux);
    for (auto& s : ctx->scratch) if (s.p) cudaFree(s.p);
    if (ctx->snap_host) cudaFreeHost(ctx->snap_host);
    for (int k = 0; k < kSnaps; ++k) if (ctx->snap_ev[k]) cudaEventDestroy(ctx->snap_ev[k]);
    if (ctx->d_rgb) cudaFree(ctx->d_rgb);
    if (ctx->d_status) cudaFree(ctx->d_status);
    if (ctx->d_stats) cudaFree(ctx->d_stats);
    if (ctx->l2_persist) {
        // give back the persisting L2 set-aside this context asked for
        cudaCtxResetPersistingL2Cache();
        cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, 0);
        cudaGetLastError();
    }
    for (cudaEvent_t e : ctx->ev_pool) cudaEventDestroy(e);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char* gb_last_error(const gb_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int gb_ctx_set_stream(gb_ctx* ctx, void* stream) {
    if (!ctx) return GB_ERR_INVALID;
    if (ctx->own_stream && ctx->stream) {
        cudaStreamSynchronize(ctx->stream);
        cudaStreamDestroy(ctx->stream);
        ctx->own_stream = false;
    }
    if (stream) ctx->stream = (cudaStream_t)stream;
    else {
        CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
        ctx->own_stream = true;
    }
    return GB_OK;
}

// 8-wide grouping and binned-SAH options of gb_build_options (defaults:
// SAH-optimal grouping with a triangle test worth 1.2 node visits, 32 bins).
static bool wide_options(const gb_build_options* opts, WideCollapse* wide, std::string* why) {
    wide->sah = true;
    wide->prim_cost = 1.2;
    wide->bins = 0;
    if (!opts) return true;
    if (opts->wide_collapse < 0 || opts->wide_collapse > 2 || !(opts->prim_cost >= 0.0f)) {
        *why = "wide_collapse must be 0, 1 or 2 and prim_cost >= 0";
        return false;
    }
    if (opts->sah_bins < 0 || opts->sah_bins == 1 || opts->sah_bins > 64) {
        *why = "sah_bins must be 2 .. 64 (0 = 32)";
        return false;
    }
    if (opts->wide_collapse == 2) wide->sah = false;
    if (opts->prim_cost > 0.0f) wide->prim_cost = opts->prim_cost;
    wide->bins = opts->sah_bins;
    return true;
}

int gb_bvh_build_stats(const float* positions, int n, const gb_build_options* opts, gb_bvh_stats* out) {
    if (!positions || !out || n <= 0 || n > (1 << 28)) return GB_ERR_INVALID;
    if (opts && opts->builder != GB_BVH_HOST_SAH) return GB_ERR_UNSUPPORTED;
    WideCollapse wide;
    std::string why;
    if (!wide_options(opts, &wide, &why)) return GB_ERR_INVALID;
    CwBvh bvh;
    if (!build_cwbvh(positions, n, &bvh, &why, &wide)) return GB_ERR_INVALID;
    out->num_nodes = bvh.n_nodes;
    out->depth = bvh.depth;
    out->binary_nodes = bvh.binary_nodes;
    out->num_triangles = bvh.n_tris;
    out->build_ms = bvh.build_ms;
    return GB_OK;
}

int gb_scene_create(gb_ctx* ctx, const gb_scene_desc* d, gb_scene** out) {
    return gb_scene_create_ex(ctx, d, nullptr, out);
}

int gb_scene_create_ex(gb_ctx* ctx, const gb_scene_desc* d, const gb_build_options* opts, gb_scene** out) {
    if (!ctx || !d || !out) return fail(ctx, GB_ERR_INVALID, "null argument");
    *out = nullptr;
    const int builder = opts ? opts->builder : GB_BVH_HOST_SAH;
    if (builder != GB_BVH_HOST_SAH && builder != GB_BVH_DEVICE_PLOC) return fail(ctx, GB_ERR_INVALID, "unknown BVH builder");
    if (opts && (opts->ploc_radius < 0 || opts->ploc_radius > 32))
        return fail(ctx, GB_ERR_INVALID, "clustering radius must be 0 (default) .. 32");
    const int radius = opts && opts->ploc_radius > 0 ? opts->ploc_radius : 16;
    CK(cudaSetDevice(ctx->device));
    int n = d->num_triangles;
    if (n <= 0 || !d->positions || !d->material_index) return fail(ctx, GB_ERR_INVALID, "no triangles");
    if (n > (1 << 28)) return fail(ctx, GB_ERR_INVALID, "too many triangles");
    if (d->num_materials <= 0 || !d->materials) return fail(ctx, GB_ERR_INVALID, "no materials");
    if (d->num_lights < 0 || (d->num_lights > 0 && !d->lights)) return fail(ctx, GB_ERR_INVALID, "bad lights");
    for (int i = 0; i < n; ++i)
        if (d->material_index[i] < 0 || d->material_index[i] >= d->num_materials)
            return fail(ctx, GB_ERR_INVALID, "material index out of range");
    for (int m = 0; m < d->num_materials; ++m) {
        int p = d->materials[m].principled;
        if (p >= 0 && (p >= d->num_params || !d->params)) return fail(ctx, GB_ERR_INVALID, "parameter index out of range");
    }
    std::vector<LightRec> lights;
    SkyTables sky_tab;
    int sky_light = -1;
    for (int l = 0; l < d->num_lights; ++l) {
        const gb_light& gl = d->lights[l];
        if (gl.type == GB_LIGHT_SKY) {
            if (sky_light >= 0) return fail(ctx, GB_ERR_UNSUPPORTED, "at most one sky light per scene");
            if (!gl.sky_rgb || gl.sky_w <= 0 || gl.sky_h <= 0 || (long long)gl.sky_w * gl.sky_h > (1ll << 26))
                return fail(ctx, GB_ERR_INVALID, "sky light without a valid map");
            for (long long i = 0; i < 3ll * gl.sky_w * gl.sky_h; ++i)
                if (!std::isfinite(gl.sky_rgb[i]) || gl.sky_rgb[i] < 0.0f)
                    return fail(ctx, GB_ERR_INVALID, "sky map values must be finite and non-negative");
            make_sky_tables(gl.sky_rgb, gl.sky_w, gl.sky_h, &sky_tab);
            sky_light = l;
        } else if (gl.type != GB_LIGHT_RECT) {
            return fail(ctx, GB_ERR_UNSUPPORTED, "unknown light type");
        }
        lights.push_back(make_light(gl));
        if (!(lights.back().power > 0.0f)) return fail(ctx, GB_ERR_INVALID, "light power must be positive");
    }
    CwBvh bvh;
    std::string err;
    WideCollapse wide;
    {
        std::string why;
        if (!wide_options(opts, &wide, &why)) return fail(ctx, GB_ERR_INVALID, why);
    }
    if (builder == GB_BVH_HOST_SAH && !build_cwbvh(d->positions, n, &bvh, &err, &wide))
        return fail(ctx, GB_ERR_INVALID, "BVH build: " + err);

    std::vector<float> shade;
    make_shade_records(d->positions, d->normals, d->material_index, n, &shade);
    // textures: checked here, mip chains made on the host (shared with the oracle)
    if (d->num_textures < 0 || (d->num_textures > 0 && !d->textures)) return fail(ctx, GB_ERR_INVALID, "bad textures");
    for (int k = 0; k < d->num_textures; ++k) {
        const gb_texture& t = d->textures[k];
        if (!t.rgba || t.w <= 0 || t.h <= 0 || t.w > 65536 || t.h > 65536 || (long long)t.w * t.h > (1ll << 26))
            return fail(ctx, GB_ERR_INVALID, "texture size must be 1 .. 65536 per side and at most 2^26 texels");
    }
    std::vector<int> dtex((size_t)d->num_materials, -1);
    bool any_tex = false;
    if (d->diffuse_texture)
        for (int m = 0; m < d->num_materials; ++m) {
            const int v = d->diffuse_texture[m];
            if (v < -1 || v >= d->num_textures) return fail(ctx, GB_ERR_INVALID, "diffuse texture index out of range");
            dtex[m] = v;
            any_tex = any_tex || v >= 0;
        }
    if (any_tex) {
        if (!d->texcoords) return fail(ctx, GB_ERR_INVALID, "textured materials need texture coordinates");
        for (size_t i = 0; i < 6 * (size_t)n; ++i)
            if (!std::isfinite(d->texcoords[i])) return fail(ctx, GB_ERR_INVALID, "non-finite texture coordinate");
    }
    std::vector<float> mats((size_t)d->num_materials * kMaterialFloats);
    for (int m = 0; m < d->num_materials; ++m) {
        MaterialRec r = make_material(d->materials[m], d->params);
        r.dtex = dtex[m];
        pack_material(r, &mats[(size_t)m * kMaterialFloats]);
    }

    gb_scene* sc = new (std::nothrow) gb_scene();
    if (!sc) return fail(ctx, GB_ERR_OOM, "host allocation");
    sc->ctx = ctx;
    void *pn = nullptr, *pt = nullptr, *ps, *pm, *pl;
    size_t bn = bvh.nodes.size() * 4, bt = bvh.tris.size() * 4, bs = shade.size() * 4, bm = mats.size() * 4,
           bl = sizeof(LightRec) * std::max<size_t>(1, lights.size());
    cudaError_t e;
    if (builder == GB_BVH_DEVICE_PLOC) {
        // positions to the device, tree built there; kept buffers join the scene
        auto tb = std::chrono::steady_clock::now();
        SceneAllocator SA(sc->allocs);
        float* dpos = nullptr;
        e = SA.alloc((void**)&dpos, sizeof(float) * 9 * (size_t)n, false);
        if (e == cudaSuccess) e = cudaMemcpy(dpos, d->positions, sizeof(float) * 9 * (size_t)n, cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = gpu_build_cwbvh(dpos, n, radius, SA, &sc->gbvh, &err, ctx->stream, wide.sah, (float)wide.prim_cost);
        if (e != cudaSuccess) {
            SA.release_temps();
            free_all(sc->allocs);
            delete sc;
            if (e == cudaErrorInvalidValue && !err.empty()) return fail(ctx, GB_ERR_INVALID, "BVH build: " + err);
            return cuda_fail(ctx, e, "device BVH build");
        }
        bvh.n_nodes = sc->gbvh.n_nodes;
        bvh.n_tris = sc->gbvh.n_tris;
        bvh.depth = sc->gbvh.depth;
        bvh.binary_nodes = sc->gbvh.binary_nodes;
        bvh.build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tb).count();
        pn = sc->gbvh.nodes;
        pt = sc->gbvh.tris;
        bn = sc->gbvh.device_bytes;
        bt = 0;
        sc->material_index.assign(d->material_index, d->material_index + n);
    }
    // a host-built tree is one allocation (nodes, then triangles at a
    // 256-byte boundary), so that one L2 access-policy window can cover it
    const size_t bn_al = (bn + 255) & ~(size_t)255;
    if ((builder == GB_BVH_HOST_SAH && (e = dalloc(sc->allocs, &pn, bn_al + bt)) != cudaSuccess) ||
        (e = dalloc(sc->allocs, &ps, bs)) != cudaSuccess || (e = dalloc(sc->allocs, &pm, bm)) != cudaSuccess ||
        (e = dalloc(sc->allocs, &pl, bl)) != cudaSuccess) {
        free_all(sc->allocs);
        delete sc;
        return cuda_fail(ctx, e, "scene allocation");
    }
    sc->shade_buf = ps;
    if (builder == GB_BVH_HOST_SAH) {
        pt = (unsigned char*)pn + bn_al;
        sc->tree_bytes = bn_al + bt;
    }
    e = cudaSuccess;
    if (builder == GB_BVH_HOST_SAH) {
        e = cudaMemcpy(pn, bvh.nodes.data(), bn, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(pt, bvh.tris.data(), bt, cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaMemcpy(ps, shade.data(), bs, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(pm, mats.data(), bm, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !lights.empty())
        e = cudaMemcpy(pl, lights.data(), sizeof(LightRec) * lights.size(), cudaMemcpyHostToDevice);
    sc->S.sky = SkyRec{};
    sc->S.sky.light = -1;
    if (e == cudaSuccess && sky_light >= 0) {
        const std::vector<float>* src[5] = {&sky_tab.texel, &sky_tab.row_cdf, &sky_tab.row_pdf, &sky_tab.col_cdf,
                                            &sky_tab.col_pdf};
        const float* dst[5] = {};
        for (int k = 0; k < 5 && e == cudaSuccess; ++k) {
            void* p = nullptr;
            e = dalloc(sc->allocs, &p, sizeof(float) * src[k]->size());
            if (e == cudaSuccess) e = cudaMemcpy(p, src[k]->data(), sizeof(float) * src[k]->size(), cudaMemcpyHostToDevice);
            dst[k] = (const float*)p;
            bs += sizeof(float) * src[k]->size();
        }
        sc->S.sky.texel = dst[0];
        sc->S.sky.row_cdf = dst[1];
        sc->S.sky.row_pdf = dst[2];
        sc->S.sky.col_cdf = dst[3];
        sc->S.sky.col_pdf = dst[4];
        sc->S.sky.w = sky_tab.w;
        sc->S.sky.h = sky_tab.h;
        sc->S.sky.scale = lights[sky_light].scale;
        sc->S.sky.light = sky_light;
    }
    sc->S.texcoord = nullptr;
    sc->S.tex = nullptr;
    sc->S.n_tex = 0;
    if (e == cudaSuccess && any_tex) {
        void* ptc = nullptr;
        e = dalloc(sc->allocs, &ptc, sizeof(float) * 6 * (size_t)n);
        if (e == cudaSuccess) e = cudaMemcpy(ptc, d->texcoords, sizeof(float) * 6 * (size_t)n, cudaMemcpyHostToDevice);
        bs += sizeof(float) * 6 * (size_t)n;
        std::vector<TexRec> recs((size_t)d->num_textures);
        std::vector<uint8_t> chain;
        for (int k = 0; k < d->num_textures && e == cudaSuccess; ++k) {
            const gb_texture& t = d->textures[k];
            make_mipmaps(t.rgba, t.w, t.h, &chain, &recs[k].max_mm, &recs[k].size);
            void* pt_ = nullptr;
            e = dalloc(sc->allocs, &pt_, chain.size());
            if (e == cudaSuccess) e = cudaMemcpy(pt_, chain.data(), chain.size(), cudaMemcpyHostToDevice);
            recs[k].texels = (const uint8_t*)pt_;
            recs[k].w = t.w;
            recs[k].h = t.h;
            bs += chain.size();
        }
        void* prec = nullptr;
        if (e == cudaSuccess) e = dalloc(sc->allocs, &prec, sizeof(TexRec) * std::max<size_t>(1, recs.size()));
        if (e == cudaSuccess && !recs.empty())
            e = cudaMemcpy(prec, recs.data(), sizeof(TexRec) * recs.size(), cudaMemcpyHostToDevice);
        sc->S.texcoord = (const float*)ptc;
        sc->S.tex = (const TexRec*)prec;
        sc->S.n_tex = d->num_textures;
    }
    if (e != cudaSuccess) {
        free_all(sc->allocs);
        delete sc;
        return cuda_fail(ctx, e, "scene upload");
    }
    sc->mat_dtex = dtex;
    sc->S.nodes = (const float4*)pn;
    sc->S.tris = (const float4*)pt;
    sc->S.shade = (const float4*)ps;
    sc->S.mats = (const float*)pm;
    sc->S.lights = (const LightRec*)pl;
    sc->S.n_lights = (int)lights.size();
    sc->S.overall_power = overall_power(lights.data(), (int)lights.size());
    sc->S.n_nodes = bvh.n_nodes;
    sc->S.n_tris = bvh.n_tris;
    sc->S.mats_eval = sc->S.mats;
    sc->S.lights_eval = sc->S.lights;
    sc->mats.assign(d->materials, d->materials + d->num_materials);
    if (d->num_params > 0) sc->params.assign(d->params, d->params + d->num_params);
    if (d->num_lights > 0) sc->lights.assign(d->lights, d->lights + d->num_lights);
    for (gb_light& l : sc->lights) l.sky_rgb = nullptr;  // the map was copied; the caller owns its memory
    sc->info.num_triangles = n;
    sc->info.num_nodes = bvh.n_nodes;
    sc->info.depth = bvh.depth;
    sc->info.binary_nodes = bvh.binary_nodes;
    sc->info.build_ms = bvh.build_ms;
    sc->info.builder = builder;
    sc->info.build_passes = sc->gbvh.iterations;
    sc->info.device_bytes = bn + bt + bs + bm + bl;
    sc->info.overall_light_power = sc->S.overall_power;
    *out = sc;
    return GB_OK;
}

void gb_scene_destroy(gb_scene* scene) {
    if (!scene) return;
    if (scene->ctx) {
        cudaSetDevice(scene->ctx->device);
        for (const BatchScene& b : scene->ctx->items)
            if (b.scene == scene) { scene->ctx->active = false; scene->ctx->items.clear(); break; }
        cudaStreamSynchronize(scene->ctx->stream);
    }
    free_all(scene->allocs);
    delete scene;
}

int gb_scene_get_info(const gb_scene* scene, gb_scene_info* info) {
    if (!scene || !info) return GB_ERR_INVALID;
    *info = scene->info;
    return GB_OK;
}

int gb_scene_refit(gb_scene* scene, const float* positions, const float* normals) {
    if (!scene || !positions) return fail(scene ? scene->ctx : nullptr, GB_ERR_INVALID, "null argument");
    gb_ctx* ctx = scene->ctx;
    if (scene->info.builder != GB_BVH_DEVICE_PLOC)
        return fail(ctx, GB_ERR_UNSUPPORTED, "refit needs a scene built with GB_BVH_DEVICE_PLOC");
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));  // frames in flight still read the old tree
    const int n = scene->gbvh.n;
    SceneAllocator SA(scene->allocs);
    float* dpos = nullptr;
    std::string err;
    cudaError_t e = SA.alloc((void**)&dpos, sizeof(float) * 9 * (size_t)n, false);
    if (e == cudaSuccess) e = cudaMemcpy(dpos, positions, sizeof(float) * 9 * (size_t)n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = gpu_refit_cwbvh(dpos, SA, &scene->gbvh, &err, ctx->stream);
    if (e != cudaSuccess) {
        if (e == cudaErrorInvalidValue && !err.empty()) return fail(ctx, GB_ERR_INVALID, "refit: " + err);
        return cuda_fail(ctx, e, "refit");
    }
    std::vector<float> shade;
    make_shade_records(positions, normals, scene->material_index.data(), n, &shade);
    CK(cudaMemcpy(scene->shade_buf, shade.data(), sizeof(float) * shade.size(), cudaMemcpyHostToDevice));
    return GB_OK;
}

namespace {

// Pixels of the frame that take a sample in round p.  Scenes are laid out by
// spp, largest first, so these pixels are a prefix of the frame.
long long round_pixels(const gb_ctx* ctx, int p) {
    long long n = 0;
    for (const BatchScene& b : ctx->items) {
        if (b.desc.spp <= p) break;
        n += b.n;
    }
    return n;
}

// Path samples in the sample and jitter buffers (sample_mb budget).
long long sample_budget(const gb_ctx* ctx) { return std::max(1ll, ((long long)ctx->sample_mb << 20) / 16); }

// End of the chunk that starts at round p0 (exclusive, <= end): rounds are
// added while the chunk's paths fit the sample budget and 2^31, and the
// chunk has at most kMaxRounds rounds.
int chunk_end(const gb_ctx* ctx, int p0, int end, long long* paths) {
    const long long budget = sample_budget(ctx);
    const long long n0 = round_pixels(ctx, p0);
    long long tot = n0;
    int p1 = p0 + 1;
    while (p1 < end && p1 - p0 < kMaxRounds) {
        long long np = round_pixels(ctx, p1);
        if (tot + np > budget || tot + np >= (1ll << 31)) break;
        tot += np;
        ++p1;
    }
    *paths = tot;
    return p1;
}

// The device part of starting a frame, on stream `st`: counters, the scene
// records (copied from `recs`, ctx->recs.size() of them), the layout's
// initial RNG states when the layout changed, and both stream cursors of
// every pixel reset to them.  Captured into the fitting graph as well.
int enqueue_frame_setup(gb_ctx* ctx, cudaStream_t st, const SceneRec* recs, bool record_start) {
    const Frame& F = ctx->F;
    CK(cudaMemsetAsync(ctx->d_stats, 0, sizeof(unsigned long long) * 16, st));
    CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(uint32_t), st));
    if (record_start) CK(cudaEventRecord(ctx->ev0, st));
    CK(cudaMemcpyAsync(ctx->d_scenes, recs, sizeof(SceneRec) * ctx->recs.size(), cudaMemcpyHostToDevice, st));
    // F.pscene and the initial RNG states depend on the pixel counts, their
    // order and the seeds only
    std::vector<uint64_t> key;
    key.push_back((uint64_t)F.ntot);
    for (const BatchScene& b : ctx->items) key.push_back(((uint64_t)b.desc.seed << 32) | (uint32_t)b.n);
    if (key != ctx->pristine_key) {
        CK(k_launch_frame_init(F, true, st));
        ctx->launches += 2;
        ctx->pristine_key = key;
    }
    // both streams of every pixel restart at curand_init(seed, pixel, 0)
    CK(cudaMemcpyAsync(F.cursor, F.pristine, sizeof(MrgState) * (size_t)F.ntot, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(F.jcursor, F.pristine, sizeof(MrgState) * (size_t)F.ntot, cudaMemcpyDeviceToDevice, st));
    return GB_OK;
}

// Lays out the scenes of a render (one scene, or a batch) in HBM and starts
// it: scene records, pixel ranges, RNG streams.
int begin_frame(gb_ctx* ctx, std::vector<BatchScene>& items) {
    ctx->active = false;
    if (items.empty()) return fail(ctx, GB_ERR_INVALID, "empty batch");
    long long ntot = 0, total_paths = 0;
    int max_spp = 0, max_L = 0;
    for (BatchScene& b : items) {
        if (!b.scene) return fail(ctx, GB_ERR_INVALID, "null scene");
        if (b.scene->ctx != ctx) return fail(ctx, GB_ERR_INVALID, "scene belongs to another context");
        int rc = check_render_desc(ctx, &b.cam, &b.desc);
        if (rc != GB_OK) return rc;
        b.n = b.desc.width * b.desc.height;
        ntot += b.n;
        total_paths += (long long)b.n * b.desc.spp;
        max_spp = std::max(max_spp, b.desc.spp);
        max_L = std::max(max_L, b.desc.max_bounces);
    }
    if (ntot > (1ll << 28)) return fail(ctx, GB_ERR_INVALID, "more than 2^28 pixels in one frame");
    std::stable_sort(items.begin(), items.end(),
                     [](const BatchScene& a, const BatchScene& b) { return a.desc.spp > b.desc.spp; });
    CK(cudaSetDevice(ctx->device));
    const long long samples = std::min(total_paths, std::max(ntot, sample_budget(ctx)));
    const int nslots = (int)std::max(1ll, std::min<long long>(total_paths, ctx->slots));
    CK(ensure_frame(ctx, (int)ntot, nslots, (size_t)samples, (int)items.size()));
    ctx->recs.assign(items.size(), SceneRec{});
    uint32_t base = 0;
    for (size_t i = 0; i < items.size(); ++i) {
        BatchScene& b = items[i];
        SceneRec& R = ctx->recs[i];
        R.S = b.scene->S;
        R.cam = make_camera(b.cam, b.desc.width, b.desc.height);
        R.sp = make_shade_params(b.desc);
        R.w = b.desc.width;
        R.h = b.desc.height;
        R.n = b.n;
        R.spp = b.desc.spp;
        R.L = b.desc.max_bounces;
        R.rng_mode = b.desc.rng_mode;
        R.pixel_base = base;
        R.seed = b.desc.seed;
        mrg_jump_matrices(3ull * (uint64_t)R.L, R.jump1, R.jump2);
        if (b.mats_eval) R.S.mats_eval = b.mats_eval;
        if (b.lights_eval) R.S.lights_eval = b.lights_eval;
        R.n_mats = (int)b.scene->mats.size();
        R.grad_base = b.grad_base;
        b.base = base;
        base += (uint32_t)b.n;
    }
    ctx->items.swap(items);
    ctx->max_spp = max_spp;
    ctx->max_L = max_L;
    Frame& F = ctx->F;
    F.ntot = (int)ntot;
    F.scenes = ctx->d_scenes;
    F.nscenes = (int)ctx->items.size();
    F.stats = ctx->d_stats;
    F.status = ctx->d_status;
    ctx->paths_done = 0;
    ctx->launches = 0;
    ctx->ev_used = 0;
    int rc = enqueue_frame_setup(ctx, ctx->stream, ctx->recs.data(), true);
    if (rc != GB_OK) return rc;
    ctx->active = true;
    return GB_OK;
}

// Slot-pool loop of one chunk driven by the host: every iteration launches
// extend, shadow, shade, regen and step; the host reads the next queue count
// through snapshots and stays at most kLead iterations ahead of the GPU.
int run_chunk_loop(gb_ctx* ctx, const RenderParams& P, int nstart, int max_iters) {
    const Frame& F = ctx->F;
    CK(cudaMemsetAsync(F.ctr, 0, sizeof(uint32_t) * 24, ctx->stream));
    CK(stage_mark(ctx, 0, true));
    CK(k_launch_jitter_pool(F, P, ctx->stream));
    CK(k_launch_start(F, P, nstart, ctx->stream));
    CK(stage_mark(ctx, 0, false));
    ctx->launches += 2;
    const int kEvery = 2, kLead = 12;
    int snap_it[kSnaps];
    int head = 0, tail = 0;  // pending snapshots [tail, head)
    bool done = false;
    for (int it = 0; !done; ++it) {
        if (it >= max_iters) return fail(ctx, GB_ERR_TRAVERSAL, "path iteration bound exceeded");
        CK(stage_mark(ctx, 1, true));
        CK(k_launch_extend(F, P, ctx->instrument, ctx->stream));
        CK(stage_mark(ctx, 1, false));
        CK(stage_mark(ctx, 2, true));
        CK(k_launch_shadow(F, P, ctx->instrument, ctx->stream));
        CK(stage_mark(ctx, 2, false));
        CK(stage_mark(ctx, 3, true));
        CK(k_launch_shade(F, P, ctx->stream));
        CK(stage_mark(ctx, 3, false));
        CK(stage_mark(ctx, 4, true));
        if (P.mode == MODE_ADJOINT) CK(k_launch_adjoint(F, P, ctx->stream));
        CK(k_launch_regen(F, P, ctx->stream));
        CK(k_launch_step(F, P, 0, false, max_iters, ctx->stream));
        CK(stage_mark(ctx, 4, false));
        if (it % kEvery == kEvery - 1) {
            int k = head % kSnaps;
            CK(cudaMemcpyAsync(ctx->snap_host + k, F.ctr + 8 * ((it + 1) % 3), sizeof(uint32_t),
                               cudaMemcpyDeviceToHost, ctx->stream));
            CK(cudaEventRecord(ctx->snap_ev[k], ctx->stream));
            snap_it[k] = it;
            ++head;
        }
        while (tail < head) {
            int k = tail % kSnaps;
            bool must_wait = (it - snap_it[k] >= kLead) || head - tail >= kSnaps;
            if (must_wait) CK(cudaEventSynchronize(ctx->snap_ev[k]));
            else {
                cudaError_t q = cudaEventQuery(ctx->snap_ev[k]);
                if (q == cudaErrorNotReady) break;
                if (q != cudaSuccess) return cuda_fail(ctx, q, "snapshot event");
            }
            if (ctx->snap_host[k] == 0u) done = true;
            ++tail;
        }
    }
    CK(stage_mark(ctx, 5, true));
    CK(k_launch_combine(F, P, ctx->stream));
    CK(stage_mark(ctx, 5, false));
    ctx->launches += 1;
    return GB_OK;
}

// Everything a captured chunk graph depends on: the frame's buffers and
// sizes, the chunk parameters and the kernel variants.
std::vector<uint64_t> graph_key(const gb_ctx* ctx, const RenderParams& P, int nstart, int max_iters) {
    const Frame& F = ctx->F;
    std::vector<uint64_t> k;
    k.push_back(((uint64_t)(uint32_t)F.ntot << 32) | (uint32_t)F.nslots);
    k.push_back(((uint64_t)(uint32_t)F.nscenes << 32) | (uint32_t)nstart);
    k.push_back(((uint64_t)(uint32_t)max_iters << 32) | (ctx->instrument ? 1u : 0u));
    const void* ptrs[] = {F.scenes, F.slots, F.shadow, F.q[0], F.q[1], F.q[2], F.q[3], F.out,
                          F.pristine, F.cursor, F.jcursor, F.pscene, F.samples, F.jpool, F.spool, F.ctr, F.path_ctr,
                          F.iter, F.stats, F.status, F.tp0, F.adj, F.dimg, F.grad};
    for (const void* p : ptrs) k.push_back((uint64_t)(uintptr_t)p);
    k.push_back(((uint64_t)(uint32_t)F.grad_stride << 32) | (uint32_t)F.grad_replicas);
    static_assert(sizeof(RenderParams) % 4 == 0, "RenderParams is made of 32-bit words");
    uint32_t w[sizeof(RenderParams) / 4];
    std::memcpy(w, &P, sizeof(P));
    for (uint32_t x : w) k.push_back(x);
    return k;
}

// One chunk as a CUDA graph: counter reset, jitter pool and first paths,
// then a conditional WHILE node whose body (extend, shadow, shade, regen,
// step) repeats until k_step finds the next extension queue empty, then the
// moving average.  Captured on the context's second stream.
int build_chunk_graph(gb_ctx* ctx, const RenderParams& P, int nstart, int max_iters, cudaGraphExec_t* out) {
    const Frame& F = ctx->F;
    cudaStream_t a = ctx->aux;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(a, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "graph capture");
    cudaGraphNodeParams np{};
    if (e == cudaSuccess) e = cudaMemsetAsync(F.ctr, 0, sizeof(uint32_t) * 24, a);
    if (e == cudaSuccess) e = k_launch_jitter_pool(F, P, a);
    if (e == cudaSuccess) e = k_launch_start(F, P, nstart, a);
    cudaStreamCaptureStatus cs;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    if (e == cudaSuccess) e = cudaStreamGetCaptureInfo(a, &cs, nullptr, &cg, &deps, nullptr, &nd);
    cudaGraphConditionalHandle h = 0;
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, cg, 1, cudaGraphCondAssignDefault);
    cudaGraphNode_t loop = nullptr;
    if (e == cudaSuccess) {
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = h;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        e = cudaGraphAddNode(&loop, cg, deps, nullptr, nd, &np);
    }
    if (e == cudaSuccess) e = cudaStreamUpdateCaptureDependencies(a, &loop, nullptr, 1, cudaStreamSetCaptureDependencies);
    if (e == cudaSuccess) e = k_launch_combine(F, P, a);
    cudaError_t e2 = cudaStreamEndCapture(a, &g);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) {
        cudaGraph_t body = np.conditional.phGraph_out[0];
        e = cudaStreamBeginCaptureToGraph(a, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
        if (e == cudaSuccess) {
            e = k_launch_extend(F, P, ctx->instrument, a);
            if (e == cudaSuccess) e = k_launch_shadow(F, P, ctx->instrument, a);
            if (e == cudaSuccess) e = k_launch_shade(F, P, a);
            if (e == cudaSuccess && P.mode == MODE_ADJOINT) e = k_launch_adjoint(F, P, a);
            if (e == cudaSuccess) e = k_launch_regen(F, P, a);
            if (e == cudaSuccess) e = k_launch_step(F, P, (unsigned long long)h, true, max_iters, a);
            cudaGraph_t body_out = nullptr;
            e2 = cudaStreamEndCapture(a, &body_out);
            if (e == cudaSuccess) e = e2;
        }
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(out, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "chunk graph");
    return GB_OK;
}

// The same chunk appended to the capture in progress on stream `a`; the
// loop body is captured on stream `b` while `a` keeps capturing.
int append_chunk(gb_ctx* ctx, const RenderParams& P, int nstart, int max_iters, cudaStream_t a, cudaStream_t b) {
    const Frame& F = ctx->F;
    cudaError_t e = cudaMemsetAsync(F.ctr, 0, sizeof(uint32_t) * 24, a);
    if (e == cudaSuccess) e = k_launch_jitter_pool(F, P, a);
    if (e == cudaSuccess) e = k_launch_start(F, P, nstart, a);
    cudaStreamCaptureStatus cs;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    if (e == cudaSuccess) e = cudaStreamGetCaptureInfo(a, &cs, nullptr, &cg, &deps, nullptr, &nd);
    cudaGraphConditionalHandle h = 0;
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, cg, 1, cudaGraphCondAssignDefault);
    cudaGraphNodeParams np{};
    cudaGraphNode_t loop = nullptr;
    if (e == cudaSuccess) {
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = h;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        e = cudaGraphAddNode(&loop, cg, deps, nullptr, nd, &np);
    }
    if (e == cudaSuccess) e = cudaStreamUpdateCaptureDependencies(a, &loop, nullptr, 1, cudaStreamSetCaptureDependencies);
    if (e == cudaSuccess) {
        e = cudaStreamBeginCaptureToGraph(b, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                          cudaStreamCaptureModeRelaxed);
        if (e == cudaSuccess) {
            e = k_launch_extend(F, P, ctx->instrument, b);
            if (e == cudaSuccess) e = k_launch_shadow(F, P, ctx->instrument, b);
            if (e == cudaSuccess) e = k_launch_shade(F, P, b);
            if (e == cudaSuccess && P.mode == MODE_ADJOINT) e = k_launch_adjoint(F, P, b);
            if (e == cudaSuccess) e = k_launch_regen(F, P, b);
            if (e == cudaSuccess) e = k_launch_step(F, P, (unsigned long long)h, true, max_iters, b);
            cudaGraph_t body_out = nullptr;
            cudaError_t e2 = cudaStreamEndCapture(b, &body_out);
            if (e == cudaSuccess) e = e2;
        }
    }
    if (e == cudaSuccess) e = k_launch_combine(F, P, a);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "step graph chunk");
    return GB_OK;
}

int run_chunk_graph(gb_ctx* ctx, const RenderParams& P, int nstart, int max_iters) {
    std::vector<uint64_t> key = graph_key(ctx, P, nstart, max_iters);
    size_t hit = ctx->graphs.size();
    for (size_t i = 0; i < ctx->graphs.size(); ++i)
        if (ctx->graphs[i].key == key) { hit = i; break; }
    if (hit == ctx->graphs.size()) {
        cudaGraphExec_t ex = nullptr;
        int rc = build_chunk_graph(ctx, P, nstart, max_iters, &ex);
        if (rc != GB_OK) return rc;
        if (ctx->graphs.size() >= kMaxGraphs) {
            cudaGraphExecDestroy(ctx->graphs.front().exec);
            ctx->graphs.erase(ctx->graphs.begin());
        }
        ctx->graphs.push_back(ChunkGraph{std::move(key), ex});
        hit = ctx->graphs.size() - 1;
    }
    CK(cudaGraphLaunch(ctx->graphs[hit].exec, ctx->stream));
    ctx->launches += 3;
    return GB_OK;
}

// Launch parameters of the chunk of rounds [p0, p1): sets the frame's slot
// count and returns the paths started first and the iteration bound.
void make_chunk(gb_ctx* ctx, int p0, int p1, RenderParams* out, int* nstart_out, int* max_iters_out) {
    RenderParams P{};
    P.refill = ctx->refill;
    P.tri_mode = ctx->tri_mode;
    P.blocks_per_sm = ctx->blocks_per_sm;
    P.trav_variant = (ctx->stack_depth == 24 ? 1 : 0) + (ctx->block_threads == 64 ? 2 : 0);
    P.sampling_terms = ctx->sampling_terms;
    P.mode = ctx->mode;
    P.textured = 0;
    for (const BatchScene& b : ctx->items)
        if (b.scene->S.texcoord) P.textured = 1;
    P.p0 = p0;
    P.rounds = p1 - p0;
#if GB_NODE_L2_PERSIST
    // a frame of one scene keeps its node array in a persisting L2 set-aside
    if (ctx->items.size() == 1) {
        const DevScene& S = ctx->items[0].scene->S;
        int dev = 0, max_persist = 0, max_window = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, dev);
        cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, dev);
        // the window: the node array, or the whole host-built tree (GB_TREE_WINDOW)
        const size_t tree = ctx->items[0].scene->tree_bytes;
        const size_t want = (GB_TREE_WINDOW && tree) ? tree : (size_t)80 * (size_t)S.n_nodes;
        const size_t window = std::min(want, (size_t)max_window);
        const size_t bytes = std::min(window, (size_t)max_persist);
        // the set-aside is a device limit: raised only outside a stream capture
        // (a fitting step is captured whole), the window is used once it is there
        cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone, cap_aux = cudaStreamCaptureStatusNone;
        cudaStreamIsCapturing(ctx->stream, &cap);
        if (ctx->aux) cudaStreamIsCapturing(ctx->aux, &cap_aux);
        if (bytes > ctx->l2_persist && cap == cudaStreamCaptureStatusNone && cap_aux == cudaStreamCaptureStatusNone &&
            cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, bytes) == cudaSuccess)
            ctx->l2_persist = bytes;
        cudaGetLastError();
        if (bytes > 0 && ctx->l2_persist >= bytes) {
            P.l2_nodes = S.nodes;
            P.l2_nodes_bytes = window;
            P.l2_hit_ratio = (float)((double)bytes / (double)window);
        }
    }
#endif
    long long acc = 0;
    for (int r = 0; r < P.rounds; ++r) {
        P.round_start[r] = (uint32_t)acc;
        acc += round_pixels(ctx, p0 + r);
    }
    P.round_start[P.rounds] = (uint32_t)acc;
    P.chunk_paths = (uint32_t)acc;
    // paths start in order on the free slots, several per pixel at once
    // (each from its own jump of the pixel's stream)
    Frame& F = ctx->F;
    F.nslots = (int)std::max(1ll, std::min({(long long)ctx->slot_cap, (long long)ctx->slots, acc}));
    // the adjoint's vertex records take 80 B x bounces per slot
    if (ctx->mode == MODE_ADJOINT) F.nslots = std::min(F.nslots, kAdjMaxSlots);
    const int nstart = (int)std::min<long long>(F.nslots, acc);
    // Every iteration moves each busy slot's path one bounce (at most L + 1
    // per path), and all slots stay busy until the chunk's last path has
    // started, so the loop ends within acc (L + 1) / nslots + L + 1
    // iterations; twice that (plus slack) bounds it.
    const long long L1 = ctx->max_L + 1;
    const int max_iters =
        (int)std::min<long long>(1ll << 30, 2 * ((acc * L1 + F.nslots - 1) / F.nslots + L1) + 16);
    *out = P;
    *nstart_out = nstart;
    *max_iters_out = max_iters;
}

// Rounds [p0, p1) of every pixel that takes them, through the slot pool.
int run_chunk(gb_ctx* ctx, int p0, int p1) {
    RenderParams P{};
    int nstart = 0, max_iters = 0;
    make_chunk(ctx, p0, p1, &P, &nstart, &max_iters);
    if (ctx->use_graph && !ctx->stage_timing) return run_chunk_graph(ctx, P, nstart, max_iters);
    return run_chunk_loop(ctx, P, nstart, max_iters);
}

int step_frame(gb_ctx* ctx, int paths) {
    if (!ctx || !ctx->active || ctx->items.empty()) return fail(ctx, GB_ERR_INVALID, "no render in progress");
    if (paths < 0) return fail(ctx, GB_ERR_INVALID, "negative path count");
    CK(cudaSetDevice(ctx->device));
    const int end = (int)std::min<long long>(ctx->max_spp, (long long)ctx->paths_done + paths);
    while (ctx->paths_done < end) {
        long long cp = 0;
        int p1 = chunk_end(ctx, ctx->paths_done, end, &cp);
        int rc = run_chunk(ctx, ctx->paths_done, p1);
        if (rc != GB_OK) return rc;
        ctx->paths_done = p1;
    }
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    return GB_OK;
}

// The packed-colour scratch for the frame (3 * ntot floats).
int ensure_rgb(gb_ctx* ctx) {
    const size_t bytes = sizeof(float) * 3 * (size_t)ctx->F.ntot;
    if (ctx->rgb_cap < bytes) {
        CK(cudaStreamSynchronize(ctx->stream));
        if (ctx->d_rgb) cudaFree(ctx->d_rgb);
        ctx->d_rgb = nullptr;
        ctx->rgb_cap = 0;
        std::vector<void*> tmp;
        CK(dalloc(tmp, (void**)&ctx->d_rgb, bytes));
        ctx->rgb_cap = bytes;
    }
    return GB_OK;
}

// Packs the frame's colours into RGB triples (device scratch of 3 * ntot floats).
int pack_frame(gb_ctx* ctx) {
    int rc = ensure_rgb(ctx);
    if (rc != GB_OK) return rc;
    if (ctx->paths_done == 0) CK(cudaMemsetAsync(ctx->F.out, 0, sizeof(float4) * (size_t)ctx->F.ntot, ctx->stream));
    CK(k_launch_pack_rgb(ctx->F.out, ctx->F.ntot, ctx->d_rgb, ctx->stream));
    ctx->launches += 1;
    return GB_OK;
}

// Copies the packed colours of one scene of the frame to `out`.
int copy_scene(gb_ctx* ctx, const BatchScene& b, float* out, int out_is_device) {
    CK(cudaMemcpyAsync(out, ctx->d_rgb + 3 * (size_t)b.base, sizeof(float) * 3 * (size_t)b.n,
                       out_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, ctx->stream));
    return GB_OK;
}

// Waits for the frame, gathers its statistics and reports kernel status.
int finish_frame(gb_ctx* ctx) {
    CK(cudaStreamSynchronize(ctx->stream));
    unsigned long long st[16];
    CK(cudaMemcpy(st, ctx->d_stats, sizeof(st), cudaMemcpyDeviceToHost));
    ctx->stats.camera_rays = st[0];
    ctx->stats.extension_rays = st[1];
    ctx->stats.shadow_rays = st[2];
    ctx->stats.closest_node_visits = st[3];
    ctx->stats.closest_tri_tests = st[4];
    ctx->stats.shadow_node_visits = st[5];
    ctx->stats.shadow_tri_tests = st[6];
    ctx->stats.light_samples = st[8];
    // every slot-pool iteration (counted by k_step in st[7]) is 4 launches
    // (extend, shadow, shade, step), 6 with the adjoint sweep
    ctx->stats.kernel_launches = ctx->launches + (uint64_t)k_launches_per_iteration(ctx->mode) * st[7];
    ctx->stats.paths_done = ctx->paths_done;
    for (int k = 0; k < 6; ++k) { ctx->stats.stage_ms[k] = 0.0; ctx->stats.stage_launches[k] = 0; }
    for (size_t i = 0; i < ctx->ev_used; ++i) {
        float ems = 0.0f;
        if (cudaEventElapsedTime(&ems, ctx->ev_pool[2 * i], ctx->ev_pool[2 * i + 1]) == cudaSuccess) {
            ctx->stats.stage_ms[ctx->ev_stage[i]] += ems;
            ctx->stats.stage_launches[ctx->ev_stage[i]] += 1;
        }
    }
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1) == cudaSuccess) ctx->stats.render_ms = ms;
    cudaGetLastError();
    return check_status(ctx);
}

}  // namespace

int gb_render_begin(gb_ctx* ctx, gb_scene* scene, const gb_camera* cam, const gb_render_desc* d) {
    if (!ctx || !scene) return fail(ctx, GB_ERR_INVALID, "null context or scene");
    if (!cam || !d) return fail(ctx, GB_ERR_INVALID, "null camera or render desc");
    std::vector<BatchScene> items(1);
    items[0].scene = scene;
    items[0].cam = *cam;
    items[0].desc = *d;
    return begin_frame(ctx, items);
}

int gb_render_step(gb_ctx* ctx, int paths) { return step_frame(ctx, paths); }

int gb_render_paths_done(const gb_ctx* ctx, int* done) {
    if (!ctx || !done) return GB_ERR_INVALID;
    *done = ctx->paths_done;
    return GB_OK;
}

int gb_render_read(gb_ctx* ctx, float* out_rgb, int out_is_device) {
    if (!ctx || !ctx->active || ctx->items.empty()) return fail(ctx, GB_ERR_INVALID, "no render in progress");
    if (!out_rgb) return fail(ctx, GB_ERR_INVALID, "null output");
    if (ctx->items.size() != 1) return fail(ctx, GB_ERR_INVALID, "gb_render_read reads single-scene renders");
    CK(cudaSetDevice(ctx->device));
    int rc = pack_frame(ctx);
    if (rc == GB_OK) rc = copy_scene(ctx, ctx->items[0], out_rgb, out_is_device);
    if (rc != GB_OK) return rc;
    return finish_frame(ctx);
}

int gb_render(gb_ctx* ctx, gb_scene* scene, const gb_camera* cam, const gb_render_desc* desc, float* out_rgb,
              int out_is_device) {
    int rc = gb_render_begin(ctx, scene, cam, desc);
    if (rc != GB_OK) return rc;
    rc = gb_render_step(ctx, desc->spp);
    if (rc != GB_OK) return rc;
    return gb_render_read(ctx, out_rgb, out_is_device);
}

int gb_render_instrumented(gb_ctx* ctx, gb_scene* scene, const gb_camera* cam, const gb_render_desc* desc,
                           float* out_rgb, int out_is_device) {
    if (!ctx) return GB_ERR_INVALID;
    ctx->instrument = true;
    int rc = gb_render(ctx, scene, cam, desc, out_rgb, out_is_device);
    ctx->instrument = false;
    return rc;
}

int gb_render_batch(gb_ctx* ctx, int n, const gb_batch_item* items, int out_is_device, int graph_capture) {
    if (!ctx) return GB_ERR_INVALID;
    if (n <= 0 || !items) return fail(ctx, GB_ERR_INVALID, "empty batch");
    std::vector<BatchScene> v((size_t)n);
    for (int i = 0; i < n; ++i) {
        if (!items[i].out_rgb) return fail(ctx, GB_ERR_INVALID, "null output");
        v[i].scene = items[i].scene;
        v[i].cam = items[i].camera;
        v[i].desc = items[i].desc;
        v[i].out = items[i].out_rgb;
    }
    const bool saved = ctx->use_graph;
    if (graph_capture >= 0) ctx->use_graph = graph_capture != 0;
    int rc = begin_frame(ctx, v);
    if (rc == GB_OK) rc = step_frame(ctx, ctx->max_spp);
    ctx->use_graph = saved;
    if (rc == GB_OK) rc = pack_frame(ctx);
    for (size_t i = 0; rc == GB_OK && i < ctx->items.size(); ++i)
        rc = copy_scene(ctx, ctx->items[i], ctx->items[i].out, out_is_device);
    if (rc != GB_OK) return rc;
    return finish_frame(ctx);
}

namespace {

int param_count(const gb_scene* s) {
    return kMatParams * (int)s->mats.size() + kLightParams * (int)s->lights.size();
}

size_t grad_floats(const gb_scene* s) { return kMatGradFloats * s->mats.size() + 3 * s->lights.size(); }

// Copies of the scene's descriptions with the parameter vector x applied
// (base colour, roughness, metallic per material; emission per light).  A
// principled parameter set shared by several materials takes the values of
// the last of them.
void apply_params(const gb_scene* s, const float* x, std::vector<gb_material>* mats,
                  std::vector<gb_principled_params>* params, std::vector<gb_light>* lights) {
    *mats = s->mats;
    *params = s->params;
    *lights = s->lights;
    for (size_t m = 0; m < mats->size(); ++m) {
        const float* v = x + kMatParams * m;
        gb_material& mt = (*mats)[m];
        if (mt.principled >= 0) {
            gb_principled_params& p = (*params)[mt.principled];
            for (int c = 0; c < 3; ++c) p.color[c] = v[c];
            p.roughness = v[3];
            p.metallic = v[4];
        } else {
            for (int c = 0; c < 3; ++c) mt.diffuse[c] = v[c];
        }
    }
    const float* lx = x + kMatParams * mats->size();
    for (size_t l = 0; l < lights->size(); ++l)
        for (int c = 0; c < 3; ++c) (*lights)[l].col[c] = lx[kLightParams * l + c];
}

void build_records(const std::vector<gb_material>& mats, const std::vector<gb_principled_params>& params,
                   const std::vector<gb_light>& lights, std::vector<float>* mrec, std::vector<LightRec>* lrec,
                   const std::vector<int>* dtex = nullptr) {
    mrec->assign(mats.size() * kMaterialFloats, 0.0f);
    for (size_t m = 0; m < mats.size(); ++m) {
        MaterialRec r = make_material(mats[m], params.empty() ? nullptr : params.data());
        if (dtex && m < dtex->size()) r.dtex = (*dtex)[m];
        pack_material(r, &(*mrec)[m * kMaterialFloats]);
    }
    lrec->clear();
    for (const gb_light& l : lights) lrec->push_back(make_light(l));
}

bool all_finite(const float* x, int n) {
    for (int i = 0; i < n; ++i)
        if (!std::isfinite(x[i])) return false;
    return true;
}

cudaError_t ensure_buf(gb_ctx* ctx, void** p, size_t* cap, size_t bytes) {
    if (bytes <= *cap) return cudaSuccess;
    cudaStreamSynchronize(ctx->stream);
    if (*p) {
        auto it = std::find(ctx->adj_allocs.begin(), ctx->adj_allocs.end(), *p);
        if (it != ctx->adj_allocs.end()) ctx->adj_allocs.erase(it);
        cudaFree(*p);
    }
    *p = nullptr;
    *cap = 0;
    cudaError_t e = dalloc(ctx->adj_allocs, p, bytes);
    if (e == cudaSuccess) *cap = bytes;
    return e;
}

}  // namespace

int gb_scene_param_count(const gb_scene* scene, int* n) {
    if (!scene || !n) return GB_ERR_INVALID;
    *n = param_count(scene);
    return GB_OK;
}

int gb_scene_get_params(const gb_scene* scene, float* x) {
    if (!scene || !x) return GB_ERR_INVALID;
    for (size_t m = 0; m < scene->mats.size(); ++m) {
        float* v = x + kMatParams * m;
        const gb_material& mt = scene->mats[m];
        if (mt.principled >= 0) {
            const gb_principled_params& p = scene->params[mt.principled];
            for (int c = 0; c < 3; ++c) v[c] = p.color[c];
            v[3] = p.roughness;
            v[4] = p.metallic;
        } else {
            for (int c = 0; c < 3; ++c) v[c] = mt.diffuse[c];
            v[3] = 0.0f;
            v[4] = 0.0f;
        }
    }
    float* lx = x + kMatParams * scene->mats.size();
    for (size_t l = 0; l < scene->lights.size(); ++l)
        for (int c = 0; c < 3; ++c) lx[kLightParams * l + c] = scene->lights[l].col[c];
    return GB_OK;
}

int gb_scene_set_params(gb_scene* scene, const float* x) {
    if (!scene || !x) return GB_ERR_INVALID;
    gb_ctx* ctx = scene->ctx;
    if (!all_finite(x, param_count(scene))) return fail(ctx, GB_ERR_INVALID, "non-finite parameter");
    std::vector<gb_material> mats;
    std::vector<gb_principled_params> params;
    std::vector<gb_light> lights;
    apply_params(scene, x, &mats, &params, &lights);
    std::vector<float> mrec;
    std::vector<LightRec> lrec;
    build_records(mats, params, lights, &mrec, &lrec, &scene->mat_dtex);
    for (const LightRec& l : lrec)
        if (!(l.power > 0.0f)) return fail(ctx, GB_ERR_INVALID, "light power must be positive");
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));  // kernels in flight read the records
    CK(cudaMemcpy((void*)scene->S.mats, mrec.data(), sizeof(float) * mrec.size(), cudaMemcpyHostToDevice));
    if (!lrec.empty())
        CK(cudaMemcpy((void*)scene->S.lights, lrec.data(), sizeof(LightRec) * lrec.size(), cudaMemcpyHostToDevice));
    scene->mats.swap(mats);
    scene->params.swap(params);
    scene->lights.swap(lights);
    scene->S.overall_power = overall_power(lrec.data(), (int)lrec.size());
    scene->info.overall_light_power = scene->S.overall_power;
    return GB_OK;
}

int gb_forward(gb_ctx* ctx, gb_scene* scene, const gb_camera* cam, const gb_render_desc* desc,
               const float* eval_params, float* out_rgb, int out_is_device) {
    if (!eval_params) return gb_render(ctx, scene, cam, desc, out_rgb, out_is_device);
    if (!ctx || !scene || !cam || !desc) return fail(ctx, GB_ERR_INVALID, "null argument");
    if (scene->ctx != ctx) return fail(ctx, GB_ERR_INVALID, "scene belongs to another context");
    if (!all_finite(eval_params, param_count(scene))) return fail(ctx, GB_ERR_INVALID, "non-finite parameter");
    if (scene->S.texcoord)
        return fail(ctx, GB_ERR_UNSUPPORTED, "frozen-sampling replay covers scenes without textures only");
    CK(cudaSetDevice(ctx->device));
    std::vector<gb_material> mats;
    std::vector<gb_principled_params> params;
    std::vector<gb_light> lights;
    apply_params(scene, eval_params, &mats, &params, &lights);
    std::vector<float> mrec;
    std::vector<LightRec> lrec;
    build_records(mats, params, lights, &mrec, &lrec);
    CK(ensure_buf(ctx, (void**)&ctx->d_eval_mats, &ctx->eval_mats_cap, sizeof(float) * mrec.size()));
    CK(ensure_buf(ctx, (void**)&ctx->d_eval_lights, &ctx->eval_lights_cap,
                  sizeof(LightRec) * std::max<size_t>(1, lrec.size())));
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(ctx->d_eval_mats, mrec.data(), sizeof(float) * mrec.size(), cudaMemcpyHostToDevice));
    if (!lrec.empty())
        CK(cudaMemcpy(ctx->d_eval_lights, lrec.data(), sizeof(LightRec) * lrec.size(), cudaMemcpyHostToDevice));
    std::vector<BatchScene> items(1);
    items[0].scene = scene;
    items[0].cam = *cam;
    items[0].desc = *desc;
    items[0].mats_eval = ctx->d_eval_mats;
    items[0].lights_eval = ctx->d_eval_lights;
    int rc = begin_frame(ctx, items);
    if (rc == GB_OK) {
        cudaError_t e = ensure_buf(ctx, (void**)&ctx->F.tp0, &ctx->tp0_cap, sizeof(float4) * ctx->slot_cap);
        if (e != cudaSuccess) rc = cuda_fail(ctx, e, "replay buffers");
    }
    ctx->mode = MODE_FROZEN;
    if (rc == GB_OK) rc = step_frame(ctx, ctx->max_spp);
    ctx->mode = MODE_FORWARD;
    if (rc == GB_OK) rc = pack_frame(ctx);
    if (rc == GB_OK) rc = copy_scene(ctx, ctx->items[0], out_rgb, out_is_device);
    if (rc == GB_OK) rc = finish_frame(ctx);
    ctx->active = false;  // the frame's records are the context's scratch
    return rc;
}

int gb_backward_batch(gb_ctx* ctx, int n, const gb_adjoint_item* items, int dimg_is_device, int graph_capture) {
    if (!ctx) return GB_ERR_INVALID;
    if (n <= 0 || !items) return fail(ctx, GB_ERR_INVALID, "empty batch");
    std::vector<BatchScene> v((size_t)n);
    std::vector<uint32_t> gbase((size_t)n);
    uint32_t gtot = 0;
    for (int i = 0; i < n; ++i) {
        if (!items[i].scene || !items[i].dL_dimg || !items[i].dL_dparams)
            return fail(ctx, GB_ERR_INVALID, "null scene, image gradient or parameter gradient");
        if (items[i].desc.max_bounces > kMaxAdjBounces)
            return fail(ctx, GB_ERR_INVALID, "the adjoint records at most 16 bounces per path");
        if (items[i].scene->S.sky.light >= 0)
            return fail(ctx, GB_ERR_UNSUPPORTED, "the adjoint covers scenes with rectangular lights only");
        if (items[i].scene->S.texcoord)
            return fail(ctx, GB_ERR_UNSUPPORTED, "the adjoint covers scenes without textures only");
        v[i].scene = items[i].scene;
        v[i].cam = items[i].camera;
        v[i].desc = items[i].desc;
        v[i].dimg = items[i].dL_dimg;
        v[i].grad_out = items[i].dL_dparams;
        v[i].grad_base = gtot;
        gtot += (uint32_t)grad_floats(items[i].scene);
    }
    CK(cudaSetDevice(ctx->device));
    int rc = begin_frame(ctx, v);
    if (rc != GB_OK) return rc;
    Frame& F = ctx->F;
    const int replicas = k_adjoint_grid();
    const int stride = (int)std::max<uint32_t>(1, gtot);
    cudaError_t e = ensure_buf(ctx, (void**)&F.adj, &ctx->adj_cap,
                               sizeof(float4) * kAdjPlanes * (size_t)ctx->max_L *
                                   std::min(ctx->slot_cap, (size_t)kAdjMaxSlots));
    if (e == cudaSuccess) e = ensure_buf(ctx, (void**)&F.dimg, &ctx->dimg_cap, sizeof(float4) * (size_t)F.ntot);
    if (e == cudaSuccess)
        e = ensure_buf(ctx, (void**)&F.grad, &ctx->grad_cap, sizeof(float) * (size_t)replicas * (size_t)stride);
    if (e == cudaSuccess) e = ensure_buf(ctx, (void**)&ctx->d_gsum, &ctx->gsum_cap, sizeof(double) * (size_t)stride);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "adjoint buffers");
    F.grad_stride = stride;
    F.grad_replicas = replicas;
    for (const BatchScene& b : ctx->items) {
        const float* src = b.dimg;
        if (!dimg_is_device) {
            CK(ensure_scratch(ctx, 0, sizeof(float) * 3 * (size_t)b.n));
            CK(cudaMemcpyAsync(ctx->scratch[0].p, b.dimg, sizeof(float) * 3 * (size_t)b.n, cudaMemcpyHostToDevice,
                               ctx->stream));
            src = (const float*)ctx->scratch[0].p;
        }
        CK(k_launch_dimg_pack(src, b.n, 1.0f / (float)b.desc.spp, F.dimg + b.base, ctx->stream));
        ctx->launches += 1;
    }
    CK(cudaMemsetAsync(F.grad, 0, sizeof(float) * (size_t)replicas * (size_t)stride, ctx->stream));
    const bool saved = ctx->use_graph;
    if (graph_capture >= 0) ctx->use_graph = graph_capture != 0;
    ctx->mode = MODE_ADJOINT;
    rc = step_frame(ctx, ctx->max_spp);
    ctx->use_graph = saved;
    std::vector<double> gsum((size_t)stride);
    if (rc == GB_OK) {
        cudaError_t e2 = k_launch_grad_reduce(F.grad, replicas, stride, ctx->d_gsum, ctx->stream);
        if (e2 == cudaSuccess) e2 = cudaMemcpyAsync(gsum.data(), ctx->d_gsum, sizeof(double) * (size_t)stride,
                                                    cudaMemcpyDeviceToHost, ctx->stream);
        if (e2 != cudaSuccess) rc = cuda_fail(ctx, e2, "gradient reduction");
        ctx->launches += 1;
    }
    if (rc == GB_OK) rc = finish_frame(ctx);
    ctx->mode = MODE_FORWARD;
    ctx->active = false;
    if (rc != GB_OK) return rc;
    // record-field gradients to parameter gradients (host, double)
    for (const BatchScene& b : ctx->items) {
        const gb_scene* sc = b.scene;
        const double* gm = gsum.data() + b.grad_base;
        for (size_t m = 0; m < sc->mats.size(); ++m) {
            double out[kMatParams];
            material_param_vjp(sc->mats[m], sc->params.empty() ? nullptr : sc->params.data(),
                               gm + kMatGradFloats * m, out);
            for (int k = 0; k < kMatParams; ++k) b.grad_out[kMatParams * m + k] = (float)out[k];
        }
        const double* gl = gm + kMatGradFloats * sc->mats.size();
        float* lo = b.grad_out + kMatParams * sc->mats.size();
        for (size_t l = 0; l < sc->lights.size(); ++l)
            for (int c = 0; c < 3; ++c) lo[kLightParams * l + c] = (float)gl[3 * l + c];
    }
    return GB_OK;
}

int gb_backward(gb_ctx* ctx, gb_scene* scene, const gb_camera* cam, const gb_render_desc* desc,
                const float* dL_dimg, int dimg_is_device, float* dL_dparams) {
    if (!ctx || !scene || !cam || !desc) return fail(ctx, GB_ERR_INVALID, "null argument");
    gb_adjoint_item it;
    it.scene = scene;
    it.camera = *cam;
    it.desc = *desc;
    it.dL_dimg = dL_dimg;
    it.dL_dparams = dL_dparams;
    return gb_backward_batch(ctx, 1, &it, dimg_is_device, -1);
}

namespace {

// Device buffers and launch knobs a fitting graph was captured with; a
// change (another render grew the frame, a new tuning) means a new graph.
std::vector<uint64_t> fit_key(const gb_ctx* ctx) {
    const Frame& F = ctx->F;
    std::vector<uint64_t> k;
    const void* ptrs[] = {ctx->d_scenes, F.slots, F.shadow, F.q[0], F.q[1], F.q[2], F.q[3], F.out, F.pristine,
                          F.cursor, F.jcursor, F.pscene, F.samples, F.jpool, F.spool, F.ctr, F.path_ctr, F.iter, F.stats,
                          F.status, F.adj, F.dimg, F.grad, ctx->d_gsum, ctx->d_rgb, ctx->fit.d_loss};
    for (const void* p : ptrs) k.push_back((uint64_t)(uintptr_t)p);
    k.push_back(((uint64_t)ctx->slot_cap << 32) ^ (uint64_t)ctx->sample_cap);
    k.push_back(((uint64_t)(uint32_t)ctx->slots << 32) | (uint32_t)ctx->sample_mb);
    k.push_back(((uint64_t)(uint32_t)ctx->refill << 32) | (uint32_t)ctx->tri_mode);
    k.push_back(((uint64_t)(uint32_t)ctx->blocks_per_sm << 32) | (uint32_t)(ctx->stack_depth * 1000 + ctx->block_threads));
    k.push_back((uint64_t)ctx->sampling_terms);
    for (const gb_fit_item& u : ctx->fit.user)
        k.push_back((uint64_t)(uintptr_t)u.scene->S.mats ^ ((uint64_t)(uintptr_t)u.scene->S.lights << 1));
    return k;
}

cudaError_t host_buf(void** p, size_t* cap, size_t bytes) {
    if (bytes <= *cap && *p) return cudaSuccess;
    if (*p) cudaFreeHost(*p);
    *p = nullptr;
    *cap = 0;
    cudaError_t e = cudaHostAlloc(p, std::max<size_t>(bytes, 16), cudaHostAllocDefault);
    if (e == cudaSuccess) *cap = bytes;
    return e;
}

// Lays the fitting frame out (an ordinary start of the forward frame: scene
// order, buffers, the layout's initial RNG states), allocates everything a
// step touches, and captures the step graph on the context's capture
// streams.
int fit_build(gb_ctx* ctx) {
    FitState& f = ctx->fit;
    f.ready = false;
    if (f.exec) { cudaGraphExecDestroy(f.exec); f.exec = nullptr; }
    std::vector<BatchScene> v(f.user.size());
    uint32_t gtot = 0;
    for (size_t i = 0; i < f.user.size(); ++i) {
        const gb_fit_item& u = f.user[i];
        v[i].scene = u.scene;
        v[i].cam = u.camera;
        v[i].desc = u.desc;
        v[i].target = u.target;
        v[i].image = u.image;
        v[i].user = (int)i;
        v[i].grad_base = gtot;
        gtot += (uint32_t)grad_floats(u.scene);
    }
    CK(cudaSetDevice(ctx->device));
    ctx->mode = MODE_FORWARD;
    int rc = begin_frame(ctx, v);
    ctx->active = false;
    if (rc != GB_OK) return rc;
    f.items = ctx->items;
    Frame& F = ctx->F;
    f.replicas = k_adjoint_grid();
    f.stride = (int)std::max<uint32_t>(1, gtot);
    const size_t ns = f.items.size();
    cudaError_t e = ensure_buf(ctx, (void**)&F.adj, &ctx->adj_cap,
                               sizeof(float4) * kAdjPlanes * (size_t)ctx->max_L *
                                   std::min(ctx->slot_cap, (size_t)kAdjMaxSlots));
    if (e == cudaSuccess) e = ensure_buf(ctx, (void**)&F.dimg, &ctx->dimg_cap, sizeof(float4) * (size_t)F.ntot);
    if (e == cudaSuccess)
        e = ensure_buf(ctx, (void**)&F.grad, &ctx->grad_cap, sizeof(float) * (size_t)f.replicas * (size_t)f.stride);
    if (e == cudaSuccess) e = ensure_buf(ctx, (void**)&ctx->d_gsum, &ctx->gsum_cap, sizeof(double) * (size_t)f.stride);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "fitting buffers");
    rc = ensure_rgb(ctx);
    if (rc != GB_OK) return rc;
    if (f.d_loss) { cudaFree(f.d_loss); f.d_loss = nullptr; }
    std::vector<void*> tmp;
    CK(dalloc(tmp, (void**)&f.d_loss, sizeof(double) * ns));
    f.mat_off.assign(ns, 0);
    f.light_off.assign(ns, 0);
    f.mats_total = f.lights_total = 0;
    for (size_t k = 0; k < ns; ++k) {
        f.mat_off[k] = f.mats_total;
        f.light_off[k] = f.lights_total;
        f.mats_total += f.items[k].scene->mats.size() * kMaterialFloats;
        f.lights_total += f.items[k].scene->lights.size();
    }
    size_t c0 = 0, c1 = 0, c2 = 0, c3 = 0;
    if (f.h_recs) { cudaFreeHost(f.h_recs); f.h_recs = nullptr; }
    if (f.h_mats) { cudaFreeHost(f.h_mats); f.h_mats = nullptr; }
    if (f.h_lights) { cudaFreeHost(f.h_lights); f.h_lights = nullptr; }
    if (f.h_out) { cudaFreeHost(f.h_out); f.h_out = nullptr; }
    CK(host_buf((void**)&f.h_recs, &c0, sizeof(SceneRec) * ns));
    CK(host_buf((void**)&f.h_mats, &c1, sizeof(float) * f.mats_total));
    CK(host_buf((void**)&f.h_lights, &c2, sizeof(LightRec) * std::max<size_t>(1, f.lights_total)));
    CK(host_buf((void**)&f.h_out, &c3, sizeof(double) * ((size_t)f.stride + ns)));
    std::memcpy(f.h_recs, ctx->recs.data(), sizeof(SceneRec) * ns);
    F.grad_stride = f.stride;
    F.grad_replicas = f.replicas;
    CK(cudaStreamSynchronize(ctx->stream));  // the layout's RNG states are in place
    if (!ctx->fit_aux) CK(cudaStreamCreateWithFlags(&ctx->fit_aux, cudaStreamNonBlocking));
    // capture: parameters -> forward frame -> loss and image gradient ->
    // adjoint frame -> gradient reduction -> results to pinned memory
    cudaStream_t a = ctx->aux, b = ctx->fit_aux;
    e = cudaStreamBeginCapture(a, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "step graph capture");
    rc = GB_OK;
    for (size_t k = 0; k < ns && rc == GB_OK; ++k) {
        gb_scene* sc = f.items[k].scene;
        e = cudaMemcpyAsync((void*)sc->S.mats, f.h_mats + f.mat_off[k], sizeof(float) * sc->mats.size() * kMaterialFloats,
                            cudaMemcpyHostToDevice, a);
        if (e == cudaSuccess && !sc->lights.empty())
            e = cudaMemcpyAsync((void*)sc->S.lights, f.h_lights + f.light_off[k], sizeof(LightRec) * sc->lights.size(),
                                cudaMemcpyHostToDevice, a);
        if (e != cudaSuccess) rc = cuda_fail(ctx, e, "step graph parameters");
    }
    if (rc == GB_OK) rc = enqueue_frame_setup(ctx, a, f.h_recs, false);
    for (int pass = 0; pass < 2 && rc == GB_OK; ++pass) {
        ctx->mode = pass == 0 ? MODE_FORWARD : MODE_ADJOINT;
        if (pass == 1) {
            // the adjoint replays the same paths: both streams of every pixel restart
            e = cudaMemcpyAsync(F.cursor, F.pristine, sizeof(MrgState) * (size_t)F.ntot, cudaMemcpyDeviceToDevice, a);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(F.jcursor, F.pristine, sizeof(MrgState) * (size_t)F.ntot, cudaMemcpyDeviceToDevice, a);
            if (e == cudaSuccess) e = cudaMemsetAsync(F.grad, 0, sizeof(float) * (size_t)f.replicas * (size_t)f.stride, a);
            if (e != cudaSuccess) { rc = cuda_fail(ctx, e, "step graph adjoint set-up"); break; }
        }
        for (int p0 = 0; p0 < ctx->max_spp && rc == GB_OK;) {
            long long cp = 0;
            const int p1 = chunk_end(ctx, p0, ctx->max_spp, &cp);
            RenderParams P{};
            int nstart = 0, max_iters = 0;
            make_chunk(ctx, p0, p1, &P, &nstart, &max_iters);
            rc = append_chunk(ctx, P, nstart, max_iters, a, b);
            p0 = p1;
        }
        if (rc != GB_OK) break;
        if (pass == 0) {
            e = k_launch_pack_rgb(F.out, F.ntot, ctx->d_rgb, a);
            for (size_t k = 0; k < ns && e == cudaSuccess; ++k) {
                const BatchScene& it = f.items[k];
                const float* img = ctx->d_rgb + 3 * (size_t)it.base;
                e = k_launch_l2_loss(img, it.target, it.n, 1.0f / (float)it.desc.spp, F.dimg + it.base, f.d_loss + k, a);
                if (e == cudaSuccess && it.image)
                    e = cudaMemcpyAsync(it.image, img, sizeof(float) * 3 * (size_t)it.n, cudaMemcpyDeviceToDevice, a);
            }
        } else {
            e = k_launch_grad_reduce(F.grad, f.replicas, f.stride, ctx->d_gsum, a);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(f.h_out, ctx->d_gsum, sizeof(double) * (size_t)f.stride, cudaMemcpyDeviceToHost, a);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(f.h_out + f.stride, f.d_loss, sizeof(double) * ns, cudaMemcpyDeviceToHost, a);
        }
        if (e != cudaSuccess) rc = cuda_fail(ctx, e, "step graph");
    }
    ctx->mode = MODE_FORWARD;
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(a, &g);
    if (rc == GB_OK && e != cudaSuccess) rc = cuda_fail(ctx, e, "step graph capture");
    if (rc == GB_OK) {
        e = cudaGraphInstantiate(&f.exec, g, 0);
        if (e != cudaSuccess) rc = cuda_fail(ctx, e, "step graph instantiation");
    }
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    if (rc != GB_OK) return rc;
    f.key = fit_key(ctx);
    f.ready = true;
    return GB_OK;
}

}  // namespace

int gb_fit_prepare(gb_ctx* ctx, int n, const gb_fit_item* items) {
    if (!ctx) return GB_ERR_INVALID;
    if (n <= 0 || n > 1024 || !items) return fail(ctx, GB_ERR_INVALID, "a fitting step takes 1..1024 scenes");
    for (int i = 0; i < n; ++i) {
        const gb_fit_item& u = items[i];
        if (!u.scene || !u.target) return fail(ctx, GB_ERR_INVALID, "null scene or target");
        if (u.scene->ctx != ctx) return fail(ctx, GB_ERR_INVALID, "scene belongs to another context");
        if (u.desc.max_bounces > kMaxAdjBounces)
            return fail(ctx, GB_ERR_INVALID, "the adjoint records at most 16 bounces per path");
        if (u.scene->S.sky.light >= 0)
            return fail(ctx, GB_ERR_UNSUPPORTED, "the adjoint covers scenes with rectangular lights only");
        if (u.scene->S.texcoord) return fail(ctx, GB_ERR_UNSUPPORTED, "the adjoint covers scenes without textures only");
        for (int j = 0; j < i; ++j)
            if (items[j].scene == u.scene) return fail(ctx, GB_ERR_INVALID, "a scene appears twice in a fitting step");
        int rc = check_render_desc(ctx, &u.camera, &u.desc);
        if (rc != GB_OK) return rc;
    }
    ctx->fit.user.assign(items, items + n);
    return fit_build(ctx);
}

int gb_fit_step(gb_ctx* ctx, const float* const* params, float* const* dL_dparams, double* loss) {
    if (!ctx) return GB_ERR_INVALID;
    FitState& f = ctx->fit;
    if (f.user.empty()) return fail(ctx, GB_ERR_INVALID, "no fitting step prepared");
    if (!params || !dL_dparams) return fail(ctx, GB_ERR_INVALID, "null parameter or gradient list");
    const size_t ns = f.user.size();
    for (size_t i = 0; i < ns; ++i) {
        if (!params[i] || !dL_dparams[i]) return fail(ctx, GB_ERR_INVALID, "null parameter or gradient vector");
        if (!all_finite(params[i], param_count(f.user[i].scene))) return fail(ctx, GB_ERR_INVALID, "non-finite parameter");
    }
    CK(cudaSetDevice(ctx->device));
    // parameters -> records (host, as gb_scene_set_params); a frame of
    // another call may still read the scenes' records
    CK(cudaStreamSynchronize(ctx->stream));
    std::vector<std::vector<float>> mrecs(ns);
    std::vector<std::vector<LightRec>> lrecs(ns);
    std::vector<std::vector<gb_material>> mats(ns);
    std::vector<std::vector<gb_principled_params>> pars(ns);
    std::vector<std::vector<gb_light>> lights(ns);
    for (size_t i = 0; i < ns; ++i) {
        gb_scene* sc = f.user[i].scene;
        apply_params(sc, params[i], &mats[i], &pars[i], &lights[i]);
        build_records(mats[i], pars[i], lights[i], &mrecs[i], &lrecs[i], &sc->mat_dtex);
        for (const LightRec& l : lrecs[i])
            if (!(l.power > 0.0f)) return fail(ctx, GB_ERR_INVALID, "light power must be positive");
    }
    for (size_t i = 0; i < ns; ++i) {
        gb_scene* sc = f.user[i].scene;
        sc->mats.swap(mats[i]);
        sc->params.swap(pars[i]);
        sc->lights.swap(lights[i]);
        sc->S.overall_power = overall_power(lrecs[i].data(), (int)lrecs[i].size());
        sc->info.overall_light_power = sc->S.overall_power;
    }
    if (!f.ready || fit_key(ctx) != f.key) {
        int rc = fit_build(ctx);
        if (rc != GB_OK) return rc;
    }
    for (size_t k = 0; k < f.items.size(); ++k) {
        const BatchScene& it = f.items[k];
        std::memcpy(f.h_mats + f.mat_off[k], mrecs[it.user].data(), sizeof(float) * mrecs[it.user].size());
        if (!lrecs[it.user].empty())
            std::memcpy(f.h_lights + f.light_off[k], lrecs[it.user].data(), sizeof(LightRec) * lrecs[it.user].size());
        f.h_recs[k].S = it.scene->S;  // the light power sum follows the emissions
    }
    CK(cudaGraphLaunch(f.exec, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    int rc = check_status(ctx);
    if (rc != GB_OK) return rc;
    for (size_t k = 0; k < f.items.size(); ++k) {
        const BatchScene& it = f.items[k];
        const gb_scene* sc = it.scene;
        const double* gm = f.h_out + it.grad_base;
        float* go = dL_dparams[it.user];
        for (size_t m = 0; m < sc->mats.size(); ++m) {
            double out[kMatParams];
            material_param_vjp(sc->mats[m], sc->params.empty() ? nullptr : sc->params.data(), gm + kMatGradFloats * m, out);
            for (int j = 0; j < kMatParams; ++j) go[kMatParams * m + j] = (float)out[j];
        }
        const double* gl = gm + kMatGradFloats * sc->mats.size();
        float* lo = go + kMatParams * sc->mats.size();
        for (size_t l = 0; l < sc->lights.size(); ++l)
            for (int c = 0; c < 3; ++c) lo[kLightParams * l + c] = (float)gl[3 * l + c];
        if (loss) loss[it.user] = f.h_out[f.stride + k];
    }
    return GB_OK;
}

namespace {

// One autotuner trial: the frame runs as gb_render_batch runs it, without
// writing images; one warm-up frame (buffers, graph capture), then the
// median device time of `repeats` frames.
int tune_trial(gb_ctx* ctx, const std::vector<BatchScene>& base, int repeats, double* ms) {
    std::vector<double> t;
    for (int r = 0; r <= repeats; ++r) {
        std::vector<BatchScene> v = base;
        int rc = begin_frame(ctx, v);
        if (rc == GB_OK) rc = step_frame(ctx, ctx->max_spp);
        if (rc == GB_OK) rc = finish_frame(ctx);
        if (rc != GB_OK) return rc;
        if (r > 0) t.push_back(ctx->stats.render_ms);
    }
    std::sort(t.begin(), t.end());
    *ms = t[t.size() / 2];
    return GB_OK;
}

}  // namespace

int gb_autotune(gb_ctx* ctx, int n, const gb_batch_item* items, int proxy_spp, int repeats, gb_tuning* best,
                double* best_ms) {
    if (!ctx) return GB_ERR_INVALID;
    if (n <= 0 || !items) return fail(ctx, GB_ERR_INVALID, "empty batch");
    if (repeats < 1) repeats = 1;
    std::vector<BatchScene> v((size_t)n);
    for (int i = 0; i < n; ++i) {
        v[i].scene = items[i].scene;
        v[i].cam = items[i].camera;
        v[i].desc = items[i].desc;
        if (proxy_spp > 0) v[i].desc.spp = std::min(v[i].desc.spp, proxy_spp);
    }
    gb_tuning cur{};
    gb_ctx_get_tuning(ctx, &cur);
    double cur_ms = 0.0;
    int rc = tune_trial(ctx, v, repeats, &cur_ms);
    if (rc != GB_OK) return rc;
    // coordinate descent: one knob at a time over its candidates (gb_tuning
    // encoding), keeping a value only when it is at least 1% faster
    struct Knob {
        int gb_tuning::*field;
        std::vector<int> vals;
    };
    const Knob knobs[] = {
        {&gb_tuning::graph, {1, 2}},
        {&gb_tuning::slots, {1 << 20, 1 << 22, 1 << 23, 1 << 24, 1 << 25}},
        {&gb_tuning::refill, {8, 16, 24, 32}},
        {&gb_tuning::tri_mode, {1, 2, 3, 4}},
        {&gb_tuning::blocks_per_sm, {1, 3, 4, 5, 6}},
        {&gb_tuning::stack_depth, {24, 32}},
        {&gb_tuning::block_threads, {64, 128}},
    };
    for (int pass = 0; pass < 2; ++pass) {
        bool changed = false;
        for (const Knob& k : knobs) {
            for (int val : k.vals) {
                if (cur.*(k.field) == val) continue;
                gb_tuning t = cur;
                t.*(k.field) = val;
                gb_ctx_set_tuning(ctx, &t);
                double ms = 0.0;
                rc = tune_trial(ctx, v, repeats, &ms);
                if (rc == GB_ERR_TRAVERSAL) continue;  // e.g. a stack too shallow for a tree: not a candidate
                if (rc != GB_OK) {
                    gb_ctx_set_tuning(ctx, &cur);
                    return rc;
                }
                if (ms < 0.99 * cur_ms) {
                    cur = t;
                    cur_ms = ms;
                    changed = true;
                }
            }
            gb_ctx_set_tuning(ctx, &cur);
        }
        if (!changed) break;
    }
    gb_ctx_set_tuning(ctx, &cur);
    ctx->active = false;
    ctx->items.clear();
    if (best) *best = cur;
    if (best_ms) *best_ms = cur_ms;
    return GB_OK;
}

int gb_render_direct(gb_ctx* ctx, gb_scene* scene, const gb_camera* cam, const gb_render_desc* d,
                     int light_samples, float* out_rgb, int out_is_device) {
    if (!ctx || !scene) return fail(ctx, GB_ERR_INVALID, "null context or scene");
    if (scene->ctx != ctx) return fail(ctx, GB_ERR_INVALID, "scene belongs to another context");
    int rc = check_render_desc(ctx, cam, d);
    if (rc != GB_OK) return rc;
    if (light_samples <= 0 || light_samples > (1 << 20)) return fail(ctx, GB_ERR_INVALID, "bad light sample count");
    if (!out_rgb) return fail(ctx, GB_ERR_INVALID, "null output");
    CK(cudaSetDevice(ctx->device));
    const int n = d->width * d->height;
    const size_t bytes = sizeof(float) * 3 * (size_t)n;
    float* dst = out_rgb;
    if (!out_is_device) {
        CK(ensure_scratch(ctx, 0, bytes));
        dst = (float*)ctx->scratch[0].p;
    }
    CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(uint32_t), ctx->stream));
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    CK(k_launch_direct(scene->S, make_camera(*cam, d->width, d->height), d->width, d->height, light_samples, d->seed,
                       d->shadow_offset, mk(d->background[0], d->background[1], d->background[2]), dst,
                       ctx->d_status, ctx->stream));
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    if (!out_is_device) CK(cudaMemcpyAsync(out_rgb, dst, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1) == cudaSuccess) ctx->stats.render_ms = ms;
    ctx->stats.kernel_launches = 1;
    cudaGetLastError();
    return check_status(ctx);
}

int gb_render_hybrid_direct(gb_ctx* ctx, gb_scene* scene, const gb_camera* cam, const gb_render_desc* d,
                            int camera_samples, int light_samples, float* out_rgb, int out_is_device) {
    if (!ctx || !scene) return fail(ctx, GB_ERR_INVALID, "null context or scene");
    if (scene->ctx != ctx) return fail(ctx, GB_ERR_INVALID, "scene belongs to another context");
    int rc = check_render_desc(ctx, cam, d);
    if (rc != GB_OK) return rc;
    if (camera_samples <= 0 || light_samples <= 0 || (long long)camera_samples * light_samples > (1 << 20))
        return fail(ctx, GB_ERR_INVALID, "bad camera / light sample counts");
    if (!out_rgb) return fail(ctx, GB_ERR_INVALID, "null output");
    CK(cudaSetDevice(ctx->device));
    const int n = d->width * d->height;
    const size_t bytes = sizeof(float) * 3 * (size_t)n;
    float* dst = out_rgb;
    if (!out_is_device) {
        CK(ensure_scratch(ctx, 0, bytes));
        dst = (float*)ctx->scratch[0].p;
    }
    CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(uint32_t), ctx->stream));
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    CK(k_launch_direct_hybrid(scene->S, make_camera(*cam, d->width, d->height), d->width, d->height, camera_samples,
                              light_samples, d->seed, d->shadow_offset,
                              mk(d->background[0], d->background[1], d->background[2]), dst, ctx->d_status,
                              ctx->stream));
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    if (!out_is_device) CK(cudaMemcpyAsync(out_rgb, dst, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1) == cudaSuccess) ctx->stats.render_ms = ms;
    ctx->stats.kernel_launches = 1;
    cudaGetLastError();
    return check_status(ctx);
}

int gb_get_stats(const gb_ctx* ctx, gb_stats* stats) {
    if (!ctx || !stats) return GB_ERR_INVALID;
    *stats = ctx->stats;
    return GB_OK;
}

int gb_set_fault_injection(int alloc_fail_after) {
    g_alloc_countdown.store(alloc_fail_after < 0 ? -1 : (long long)alloc_fail_after);
    return GB_OK;
}

int gb_ctx_set_tuning(gb_ctx* ctx, const gb_tuning* t) {
    if (!ctx || !t) return fail(ctx, GB_ERR_INVALID, "null argument");
    if (t->refill < 0 || t->refill > 32) return fail(ctx, GB_ERR_INVALID, "refill must be in 1..32");
    if (t->slots < 0 || t->sample_mb < 0) return fail(ctx, GB_ERR_INVALID, "negative tuning value");
    if (t->tri_mode < 0 || t->tri_mode > 4) return fail(ctx, GB_ERR_INVALID, "tri_mode must be 1..4 (0 keeps)");
    if (t->graph < 0 || t->graph > 2) return fail(ctx, GB_ERR_INVALID, "graph must be 1 or 2 (0 keeps)");
    if (t->blocks_per_sm < 0 || t->blocks_per_sm > 65)
        return fail(ctx, GB_ERR_INVALID, "blocks_per_sm must be 1..65 (0 keeps)");
    if (t->stack_depth != 0 && t->stack_depth != 24 && t->stack_depth != 32)
        return fail(ctx, GB_ERR_INVALID, "stack_depth must be 24 or 32 (0 keeps)");
    if (t->block_threads != 0 && t->block_threads != 64 && t->block_threads != 128)
        return fail(ctx, GB_ERR_INVALID, "block_threads must be 64 or 128 (0 keeps)");
    if (t->blocks_per_sm) ctx->blocks_per_sm = t->blocks_per_sm - 1;
    if (t->stack_depth) ctx->stack_depth = t->stack_depth;
    if (t->block_threads) ctx->block_threads = t->block_threads;
    if (t->tri_mode) ctx->tri_mode = t->tri_mode - 1;
    if (t->graph) ctx->use_graph = t->graph == 2;
    if (t->refill) ctx->refill = t->refill;
    if (t->slots) ctx->slots = t->slots;
    if (t->sample_mb) ctx->sample_mb = t->sample_mb;
    return GB_OK;
}

int gb_ctx_get_tuning(const gb_ctx* ctx, gb_tuning* t) {
    if (!ctx || !t) return GB_ERR_INVALID;
    t->refill = ctx->refill;
    t->slots = ctx->slots;
    t->sample_mb = ctx->sample_mb;
    t->tri_mode = ctx->tri_mode + 1;
    t->graph = ctx->use_graph ? 2 : 1;
    t->blocks_per_sm = ctx->blocks_per_sm + 1;
    t->stack_depth = ctx->stack_depth;
    t->block_threads = ctx->block_threads;
    return GB_OK;
}

int gb_ctx_set_gradient_terms(gb_ctx* ctx, int sampling) {
    if (!ctx) return GB_ERR_INVALID;
    if (sampling != 0 && sampling != 1) return fail(ctx, GB_ERR_INVALID, "sampling must be 0 or 1");
    ctx->sampling_terms = sampling;
    return GB_OK;
}

int gb_ctx_set_stage_timing(gb_ctx* ctx, int on) {
    if (!ctx) return GB_ERR_INVALID;
    ctx->stage_timing = on != 0;
    return GB_OK;
}

int gb_layout_sizes(int* node_bytes, int* tri_bytes) {
    if (node_bytes) *node_bytes = kNodeWords * 4;
    if (tri_bytes) *tri_bytes = kTriWords * 4;
    return GB_OK;
}

static int trace_common(gb_ctx* ctx, gb_scene* scene, int n, const float* orig, const float* dir,
                        const float* max_t, gb_hit* hits, uint8_t* occl, int device_ptrs, bool any) {
    if (!ctx || !scene) return fail(ctx, GB_ERR_INVALID, "null context or scene");
    if (n < 0) return fail(ctx, GB_ERR_INVALID, "negative ray count");
    if (n == 0) return GB_OK;
    if (!orig || !dir || !max_t || (any ? !occl : !hits)) return fail(ctx, GB_ERR_INVALID, "null buffer");
    CK(cudaSetDevice(ctx->device));
    const float *d_o = orig, *d_d = dir, *d_t = max_t;
    float4* d_h = (float4*)hits;
    uint8_t* d_oc = occl;
    size_t b3 = sizeof(float) * 3 * (size_t)n;
    if (!device_ptrs) {
        CK(ensure_scratch(ctx, 0, b3));
        CK(ensure_scratch(ctx, 1, b3));
        CK(ensure_scratch(ctx, 2, sizeof(float) * (size_t)n));
        CK(ensure_scratch(ctx, 3, sizeof(float4) * (size_t)n));
        CK(cudaMemcpyAsync(ctx->scratch[0].p, orig, b3, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(ctx->scratch[1].p, dir, b3, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(ctx->scratch[2].p, max_t, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, ctx->stream));
        d_o = (const float*)ctx->scratch[0].p;
        d_d = (const float*)ctx->scratch[1].p;
        d_t = (const float*)ctx->scratch[2].p;
        d_h = (float4*)ctx->scratch[3].p;
        d_oc = (uint8_t*)ctx->scratch[3].p;
    }
    CK(k_launch_trace(scene->S, n, d_o, d_d, d_t, d_h, d_oc, any, ctx->d_status, ctx->stream));
    if (!device_ptrs) {
        if (any) CK(cudaMemcpyAsync(occl, d_oc, (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
        else CK(cudaMemcpyAsync(hits, d_h, sizeof(gb_hit) * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
    }
    return check_status(ctx);
}

int gb_trace_closest(gb_ctx* ctx, gb_scene* scene, int n, const float* orig, const float* dir, const float* max_t,
                     gb_hit* hits, int device_ptrs) {
    return trace_common(ctx, scene, n, orig, dir, max_t, hits, nullptr, device_ptrs, false);
}

int gb_trace_any(gb_ctx* ctx, gb_scene* scene, int n, const float* orig, const float* dir, const float* max_t,
                 uint8_t* occluded, int device_ptrs) {
    return trace_common(ctx, scene, n, orig, dir, max_t, nullptr, occluded, device_ptrs, true);
}

int gb_generate_arealight_sample(gb_ctx* ctx, gb_scene* scene, int w, int h, float shadow_offset, const float* rnd,
                                 const gb_hit* hits, float* ray_orig, float* ray_dir, float* max_t, float* psc) {
    if (!ctx || !scene || w < 0 || h < 0) return fail(ctx, GB_ERR_INVALID, "bad arguments");
    if (!rnd || !hits || !ray_orig || !ray_dir || !max_t || !psc) return fail(ctx, GB_ERR_INVALID, "null buffer");
    CK(cudaSetDevice(ctx->device));
    CK(k_launch_nee_stage(scene->S, w * h, shadow_offset, rnd, (const float4*)hits, ray_orig, ray_dir, max_t, psc,
                          ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return GB_OK;
}

int gb_compute_path_contribution_and_bounce(gb_ctx* ctx, gb_scene* scene, int w, int h, const gb_render_desc* desc,
                                            float* ray_orig, float* ray_dir, float* max_t, const gb_hit* hits,
                                            const uint8_t* shadow_occluded, const float* rnd, float* throughput,
                                            float* col_accum, const float* to_light, const float* psc, int path,
                                            int bounce) {
    if (!ctx || !scene || !desc || w < 0 || h < 0) return fail(ctx, GB_ERR_INVALID, "bad arguments");
    if (!ray_orig || !ray_dir || !max_t || !hits || !shadow_occluded || !rnd || !throughput || !col_accum ||
        !to_light || !psc)
        return fail(ctx, GB_ERR_INVALID, "null buffer");
    if (scene->S.texcoord)
        return fail(ctx, GB_ERR_UNSUPPORTED, "the stage call has no ray-differential buffers; textured scenes need gb_render");
    CK(cudaSetDevice(ctx->device));
    ShadeParams sp = make_shade_params(*desc);
    CK(k_launch_shade_stage(scene->S, w * h, sp, ray_orig, ray_dir, max_t, (const float4*)hits, shadow_occluded, rnd,
                            throughput, col_accum, to_light, psc, path, bounce, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return GB_OK;
}

int gb_mrg_pool(gb_ctx* ctx, int npix, uint32_t seed, int first_update, int num_updates, float* out) {
    return gb_mrg_pool_range(ctx, 0, npix, seed, first_update, num_updates, out);
}

int gb_mrg_pool_range(gb_ctx* ctx, int pixel0, int npix, uint32_t seed, int first_update, int num_updates,
                      float* out) {
    if (!ctx || pixel0 < 0 || npix <= 0 || npix > INT32_MAX - pixel0 || first_update < 0 || num_updates <= 0 || !out)
        return fail(ctx, GB_ERR_INVALID, "bad arguments");
    CK(cudaSetDevice(ctx->device));
    size_t bytes = sizeof(float) * 3 * (size_t)npix * (size_t)num_updates;
    void* d = nullptr;
    CK(cudaMalloc(&d, bytes));
    cudaError_t e = k_launch_mrg_pool(pixel0, npix, seed, first_update, num_updates, (float*)d, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "mrg pool");
    return GB_OK;
}

int gb_mrg_states(gb_ctx* ctx, uint32_t seed, const uint32_t* subsequences, int n, int method, uint32_t* out) {
    if (!ctx || n <= 0 || !subsequences || !out || (method != 0 && method != 1))
        return fail(ctx, GB_ERR_INVALID, "bad arguments");
    CK(cudaSetDevice(ctx->device));
    void* d = nullptr;
    CK(cudaMalloc(&d, 7 * 4 * (size_t)n));
    uint32_t* dsub = (uint32_t*)d;
    uint32_t* dout = dsub + n;
    cudaError_t e = cudaMemcpyAsync(dsub, subsequences, 4 * (size_t)n, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = k_launch_mrg_states(seed, dsub, n, method, dout, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, 6 * 4 * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "mrg states");
    return GB_OK;
}

}  // extern "C"

namespace gb {
// Internal views used by gb_render_noalloc (gbpt_noalloc.cu).
const DevScene* scene_device_view(const gb_scene* s) { return s ? &s->S : nullptr; }
int scene_device(const gb_scene* s) { return s && s->ctx ? s->ctx->device : -1; }
void scene_set_error(const gb_scene* s, const char* msg) {
    if (s && s->ctx) s->ctx->err = msg;
}
}  // namespace gb
