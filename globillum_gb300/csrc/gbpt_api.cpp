// gbpt_api.cpp -- C ABI of libgbpt.so (include/gbpt.h): contexts, resident
// scenes, the progressive wavefront frame, tracing and per-stage entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/gbpt.h"
#include "gbpt_bvh.h"
#include "gbpt_host.h"
#include "gbpt_kernels.h"

using namespace gb;

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

static const int kSnaps = 16;

struct gb_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string err;
    // frame: per-slot, per-pixel and sample-buffer capacities
    Frame F{};
    size_t slot_cap = 0, pixel_cap = 0, sample_cap = 0;
    std::vector<void*> slot_allocs, pixel_allocs, sample_allocs;
    int chunk = 1;                      // path samples per chunk of the current render
    // progressive render
    gb_scene* scene = nullptr;
    RenderParams P{};
    int paths_done = 0;
    bool active = false;
    bool instrument = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    uint32_t* d_status = nullptr;
    unsigned long long* d_stats = nullptr;
    gb_stats stats{};
    uint64_t launches = 0;
    bool stage_timing = false;
    int refill = 16;                    // idle lanes that trigger a warp refill
    int tri_mode = 0;                   // traversal triangle policy (see gb_tuning)
    int slots = 1 << 20;                // path slots in flight (upper bound; at most one per pixel)
    int sample_mb = 1024;               // sample buffer budget (chunk size)
    // queue-count snapshots: pinned ring + events (host stays a few iterations ahead)
    uint32_t* snap_host = nullptr;
    cudaEvent_t snap_ev[kSnaps] = {};
    std::vector<cudaEvent_t> ev_pool;   // stage timing events (pairs)
    std::vector<int> ev_stage;          // stage of each recorded pair
    size_t ev_used = 0;
    // curand states right after curand_init(seed, pixel, 0) are kept in
    // F.pristine while the seed and pixel buffer stay the same
    size_t pristine_n = 0;
    uint32_t pristine_seed = 0;
    // scratch for API calls with host pointers
    DevBuf scratch[4];
    float* d_rgb = nullptr;
    size_t rgb_cap = 0;
};

struct gb_scene {
    gb_ctx* ctx = nullptr;
    DevScene S{};
    std::vector<void*> allocs;
    gb_scene_info info{};
};

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

cudaError_t ensure_scratch(gb_ctx* ctx, int k, size_t bytes) {
    if (ctx->scratch[k].bytes >= bytes) return cudaSuccess;
    if (ctx->scratch[k].p) cudaFree(ctx->scratch[k].p);
    ctx->scratch[k].p = nullptr;
    ctx->scratch[k].bytes = 0;
    cudaError_t e = cudaMalloc(&ctx->scratch[k].p, bytes);
    if (e == cudaSuccess) ctx->scratch[k].bytes = bytes;
    return e;
}

// Per-slot buffers for `nslots` slots, per-pixel buffers for `n` pixels and a
// sample buffer of `samples` float4 entries; grown on demand.
cudaError_t ensure_frame(gb_ctx* ctx, int n, int nslots, size_t samples) {
    Frame& F = ctx->F;
    cudaError_t e;
    if ((size_t)nslots > ctx->slot_cap) {
        cudaStreamSynchronize(ctx->stream);
        free_all(ctx->slot_allocs);
        ctx->slot_cap = 0;
        size_t v4 = sizeof(float4) * (size_t)nslots;
        float4** bufs[] = {&F.ray_o, &F.ray_d, &F.tp, &F.accum, &F.sh_o, &F.sh_d, &F.psc, &F.rnd, &F.hit_p, &F.hit_n};
        for (float4** b : bufs)
            if ((e = dalloc(ctx->slot_allocs, (void**)b, v4)) != cudaSuccess) return e;
        if ((e = dalloc(ctx->slot_allocs, &F.rng, 48 * (size_t)nslots)) != cudaSuccess) return e;
        if ((e = dalloc(ctx->slot_allocs, (void**)&F.pix, 4 * (size_t)nslots)) != cudaSuccess) return e;
        if ((e = dalloc(ctx->slot_allocs, (void**)&F.pb, 4 * (size_t)nslots)) != cudaSuccess) return e;
        for (int k = 0; k < 4; ++k)
            if ((e = dalloc(ctx->slot_allocs, (void**)&F.q[k], 4 * (size_t)nslots)) != cudaSuccess) return e;
        if ((e = dalloc(ctx->slot_allocs, (void**)&F.ctr, 4 * 32)) != cudaSuccess) return e;
        if ((e = dalloc(ctx->slot_allocs, (void**)&F.path_ctr, 4 * 8)) != cudaSuccess) return e;
        ctx->slot_cap = (size_t)nslots;
    }
    if ((size_t)n > ctx->pixel_cap) {
        cudaStreamSynchronize(ctx->stream);
        free_all(ctx->pixel_allocs);
        ctx->pixel_cap = 0;
        ctx->pristine_n = 0;
        if ((e = dalloc(ctx->pixel_allocs, (void**)&F.out, sizeof(float4) * (size_t)n)) != cudaSuccess) return e;
        if ((e = dalloc(ctx->pixel_allocs, &F.pristine, 48 * (size_t)n)) != cudaSuccess) return e;
        if ((e = dalloc(ctx->pixel_allocs, &F.cursor, 48 * (size_t)n)) != cudaSuccess) return e;
        if ((e = dalloc(ctx->pixel_allocs, &F.jcursor, 48 * (size_t)n)) != cudaSuccess) return e;
        ctx->pixel_cap = (size_t)n;
    }
    if (samples > ctx->sample_cap) {
        cudaStreamSynchronize(ctx->stream);
        free_all(ctx->sample_allocs);
        ctx->sample_cap = 0;
        if ((e = dalloc(ctx->sample_allocs, (void**)&F.samples, sizeof(float4) * samples)) != cudaSuccess) return e;
        if ((e = dalloc(ctx->sample_allocs, (void**)&F.jpool, sizeof(float4) * samples)) != cudaSuccess) return e;
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
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_status, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_stats, sizeof(unsigned long long) * 8);
    if (e == cudaSuccess) e = cudaMemset(ctx->d_status, 0, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(ctx->d_stats, 0, sizeof(unsigned long long) * 8);
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
    for (auto& s : ctx->scratch) if (s.p) cudaFree(s.p);
    if (ctx->snap_host) cudaFreeHost(ctx->snap_host);
    for (int k = 0; k < kSnaps; ++k) if (ctx->snap_ev[k]) cudaEventDestroy(ctx->snap_ev[k]);
    if (ctx->d_rgb) cudaFree(ctx->d_rgb);
    if (ctx->d_status) cudaFree(ctx->d_status);
    if (ctx->d_stats) cudaFree(ctx->d_stats);
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

int gb_scene_create(gb_ctx* ctx, const gb_scene_desc* d, gb_scene** out) {
    if (!ctx || !d || !out) return fail(ctx, GB_ERR_INVALID, "null argument");
    *out = nullptr;
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
    for (int l = 0; l < d->num_lights; ++l) {
        if (d->lights[l].type != GB_LIGHT_RECT) return fail(ctx, GB_ERR_UNSUPPORTED, "only rectangular lights are supported");
        lights.push_back(make_light(d->lights[l]));
        if (!(lights.back().power > 0.0f)) return fail(ctx, GB_ERR_INVALID, "light power must be positive");
    }
    CwBvh bvh;
    std::string err;
    if (!build_cwbvh(d->positions, n, &bvh, &err)) return fail(ctx, GB_ERR_INVALID, "BVH build: " + err);

    std::vector<float> shade((size_t)n * 24);
    for (int t = 0; t < n; ++t) {
        float* s = &shade[(size_t)t * 24];
        const float* p = d->positions + 9 * (size_t)t;
        float nrm[9];
        if (d->normals) std::memcpy(nrm, d->normals + 9 * (size_t)t, sizeof(nrm));
        else {
            v3 fn = normalize_div(cross(mk(p[3] - p[0], p[4] - p[1], p[5] - p[2]), mk(p[6] - p[0], p[7] - p[1], p[8] - p[2])));
            for (int k = 0; k < 3; ++k) { nrm[3 * k] = fn.x; nrm[3 * k + 1] = fn.y; nrm[3 * k + 2] = fn.z; }
        }
        uint32_t mi = (uint32_t)d->material_index[t];
        for (int v = 0; v < 3; ++v) {
            s[4 * v] = p[3 * v]; s[4 * v + 1] = p[3 * v + 1]; s[4 * v + 2] = p[3 * v + 2]; s[4 * v + 3] = 0.0f;
            s[12 + 4 * v] = nrm[3 * v]; s[12 + 4 * v + 1] = nrm[3 * v + 1]; s[12 + 4 * v + 2] = nrm[3 * v + 2];
            s[12 + 4 * v + 3] = 0.0f;
        }
        std::memcpy(&s[3], &mi, 4);
    }
    std::vector<float> mats((size_t)d->num_materials * kMaterialFloats);
    for (int m = 0; m < d->num_materials; ++m)
        pack_material(make_material(d->materials[m], d->params), &mats[(size_t)m * kMaterialFloats]);

    gb_scene* sc = new (std::nothrow) gb_scene();
    if (!sc) return fail(ctx, GB_ERR_OOM, "host allocation");
    sc->ctx = ctx;
    void *pn, *pt, *ps, *pm, *pl;
    size_t bn = bvh.nodes.size() * 4, bt = bvh.tris.size() * 4, bs = shade.size() * 4, bm = mats.size() * 4,
           bl = sizeof(LightRec) * std::max<size_t>(1, lights.size());
    cudaError_t e;
    if ((e = dalloc(sc->allocs, &pn, bn)) != cudaSuccess || (e = dalloc(sc->allocs, &pt, bt)) != cudaSuccess ||
        (e = dalloc(sc->allocs, &ps, bs)) != cudaSuccess || (e = dalloc(sc->allocs, &pm, bm)) != cudaSuccess ||
        (e = dalloc(sc->allocs, &pl, bl)) != cudaSuccess) {
        free_all(sc->allocs);
        delete sc;
        return cuda_fail(ctx, e, "scene allocation");
    }
    e = cudaMemcpy(pn, bvh.nodes.data(), bn, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(pt, bvh.tris.data(), bt, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(ps, shade.data(), bs, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(pm, mats.data(), bm, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !lights.empty())
        e = cudaMemcpy(pl, lights.data(), sizeof(LightRec) * lights.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        free_all(sc->allocs);
        delete sc;
        return cuda_fail(ctx, e, "scene upload");
    }
    sc->S.nodes = (const float4*)pn;
    sc->S.tris = (const float4*)pt;
    sc->S.shade = (const float4*)ps;
    sc->S.mats = (const float*)pm;
    sc->S.lights = (const LightRec*)pl;
    sc->S.n_lights = (int)lights.size();
    sc->S.overall_power = overall_power(lights.data(), (int)lights.size());
    sc->S.n_nodes = bvh.n_nodes;
    sc->S.n_tris = bvh.n_tris;
    sc->info.num_triangles = n;
    sc->info.num_nodes = bvh.n_nodes;
    sc->info.depth = bvh.depth;
    sc->info.binary_nodes = bvh.binary_nodes;
    sc->info.build_ms = bvh.build_ms;
    sc->info.device_bytes = bn + bt + bs + bm + bl;
    sc->info.overall_light_power = sc->S.overall_power;
    *out = sc;
    return GB_OK;
}

void gb_scene_destroy(gb_scene* scene) {
    if (!scene) return;
    if (scene->ctx) {
        cudaSetDevice(scene->ctx->device);
        if (scene->ctx->scene == scene) { scene->ctx->scene = nullptr; scene->ctx->active = false; }
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

int gb_render_begin(gb_ctx* ctx, gb_scene* scene, const gb_camera* cam, const gb_render_desc* d) {
    if (!ctx || !scene) return fail(ctx, GB_ERR_INVALID, "null context or scene");
    int rc = check_render_desc(ctx, cam, d);
    if (rc != GB_OK) return rc;
    CK(cudaSetDevice(ctx->device));
    const int n = d->width * d->height;
    // chunk: path samples per pass of the slot pool (bounded by the sample
    // buffer budget and by 2^31 paths); slots: paths in flight
    long long budget = (long long)ctx->sample_mb << 20;
    int chunk = (int)std::max(1ll, std::min<long long>(d->spp, budget / (16ll * n)));
    chunk = (int)std::min<long long>(chunk, std::max(1ll, (1ll << 31) / n - 1));
    long long chunk_paths = (long long)chunk * n;
    // at most one slot per pixel: a launch then starts at most one path per
    // pixel, which keeps the per-pixel stream cursors unshared
    int nslots = (int)std::max(1ll, std::min<long long>(std::min<long long>(chunk_paths, n), ctx->slots));
    CK(ensure_frame(ctx, n, nslots, (size_t)chunk_paths));
    Frame& F = ctx->F;
    F.w = d->width; F.h = d->height; F.n = n;
    F.nslots = nslots;
    F.stats = ctx->d_stats;
    F.status = ctx->d_status;
    ctx->chunk = chunk;
    RenderParams& P = ctx->P;
    P.cam = make_camera(*cam, d->width, d->height);
    P.sp = make_shade_params(*d);
    P.spp = d->spp;
    P.L = d->max_bounces;
    P.rng_mode = d->rng_mode;
    P.seed = d->seed;
    P.refill = ctx->refill;
    P.tri_mode = ctx->tri_mode;
    ctx->scene = scene;
    ctx->paths_done = 0;
    ctx->active = true;
    ctx->launches = 0;
    ctx->ev_used = 0;
    CK(cudaMemsetAsync(ctx->d_stats, 0, sizeof(unsigned long long) * 8, ctx->stream));
    CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(uint32_t), ctx->stream));
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    if (!(ctx->pristine_seed == d->seed && ctx->pristine_n >= (size_t)n)) {
        CK(k_launch_rng_init(n, d->seed, F.pristine, ctx->stream));
        ctx->launches += 1;
        ctx->pristine_n = (size_t)n;
        ctx->pristine_seed = d->seed;
    }
    // both streams of pixel i restart at curand_init(seed, i, 0)
    CK(cudaMemcpyAsync(F.cursor, F.pristine, 48 * (size_t)n, cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaMemcpyAsync(F.jcursor, F.pristine, 48 * (size_t)n, cudaMemcpyDeviceToDevice, ctx->stream));
    return GB_OK;
}

namespace {

// Path samples [p0, p1) of every pixel through the slot pool.
int run_chunk(gb_ctx* ctx, int p0, int p1) {
    RenderParams& P = ctx->P;
    const Frame& F = ctx->F;
    const DevScene& S = ctx->scene->S;
    P.p0 = p0;
    P.chunk_paths = (p1 - p0) * F.n;
    const int nstart = std::min(F.nslots, P.chunk_paths);
    CK(cudaMemsetAsync(F.ctr, 0, sizeof(uint32_t) * 24, ctx->stream));
    CK(stage_mark(ctx, 0, true));
    CK(k_launch_jitter_pool(F, p0, p1, ctx->stream));
    CK(k_launch_start(F, P, nstart, ctx->stream));
    CK(stage_mark(ctx, 0, false));
    ctx->launches += 2;
    // iterations until the next extension queue is empty; the host checks
    // that count through snapshots and stays at most kLead iterations ahead
    const long long max_iters = (long long)P.chunk_paths * P.L + 8;
    const int kEvery = 2, kLead = 12;
    int snap_it[kSnaps];
    int head = 0, tail = 0;  // pending snapshots [tail, head)
    bool done = false;
    for (long long it = 0; !done; ++it) {
        if (it >= max_iters) return fail(ctx, GB_ERR_TRAVERSAL, "path iteration bound exceeded");
        const int ii = (int)(it % 3000000);
        CK(cudaMemsetAsync(F.ctr + 8 * ((ii + 1) % 3), 0, sizeof(uint32_t) * 8, ctx->stream));
        CK(stage_mark(ctx, 1, true));
        CK(k_launch_extend(S, F, P, ii, ctx->instrument, ctx->stream));
        CK(stage_mark(ctx, 1, false));
        CK(stage_mark(ctx, 2, true));
        CK(k_launch_shadow(S, F, P, ii, ctx->instrument, ctx->stream));
        CK(stage_mark(ctx, 2, false));
        CK(stage_mark(ctx, 3, true));
        CK(k_launch_shade(S, F, P, ii, ctx->stream));
        CK(stage_mark(ctx, 3, false));
        CK(stage_mark(ctx, 4, true));
        CK(k_launch_regen(F, P, ii, ctx->stream));
        CK(stage_mark(ctx, 4, false));
        ctx->launches += 4;
        if (it % kEvery == kEvery - 1) {
            int k = head % kSnaps;
            CK(cudaMemcpyAsync(ctx->snap_host + k, F.ctr + 8 * ((ii + 1) % 3), sizeof(uint32_t),
                               cudaMemcpyDeviceToHost, ctx->stream));
            CK(cudaEventRecord(ctx->snap_ev[k], ctx->stream));
            snap_it[k] = (int)it;
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
    CK(k_launch_combine(F, p0, p1, ctx->stream));
    CK(stage_mark(ctx, 5, false));
    ctx->launches += 1;
    return GB_OK;
}

}  // namespace

int gb_render_step(gb_ctx* ctx, int paths) {
    if (!ctx || !ctx->active || !ctx->scene) return fail(ctx, GB_ERR_INVALID, "no render in progress");
    if (paths < 0) return fail(ctx, GB_ERR_INVALID, "negative path count");
    CK(cudaSetDevice(ctx->device));
    int end = std::min(ctx->P.spp, ctx->paths_done + paths);
    while (ctx->paths_done < end) {
        int p1 = std::min(end, ctx->paths_done + ctx->chunk);
        int rc = run_chunk(ctx, ctx->paths_done, p1);
        if (rc != GB_OK) return rc;
        ctx->paths_done = p1;
    }
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    return GB_OK;
}

int gb_render_paths_done(const gb_ctx* ctx, int* done) {
    if (!ctx || !done) return GB_ERR_INVALID;
    *done = ctx->paths_done;
    return GB_OK;
}

int gb_render_read(gb_ctx* ctx, float* out_rgb, int out_is_device) {
    if (!ctx || !ctx->active) return fail(ctx, GB_ERR_INVALID, "no render in progress");
    if (!out_rgb) return fail(ctx, GB_ERR_INVALID, "null output");
    CK(cudaSetDevice(ctx->device));
    int n = ctx->F.n;
    size_t bytes = sizeof(float) * 3 * (size_t)n;
    if (ctx->paths_done == 0) CK(cudaMemsetAsync(ctx->F.out, 0, sizeof(float4) * (size_t)n, ctx->stream));
    if (out_is_device) {
        CK(k_launch_pack_rgb(ctx->F.out, n, out_rgb, ctx->stream));
        ctx->launches += 1;
    } else {
        if (ctx->rgb_cap < bytes) {
            if (ctx->d_rgb) cudaFree(ctx->d_rgb);
            ctx->d_rgb = nullptr;
            ctx->rgb_cap = 0;
            CK(cudaMalloc(&ctx->d_rgb, bytes));
            ctx->rgb_cap = bytes;
        }
        CK(k_launch_pack_rgb(ctx->F.out, n, ctx->d_rgb, ctx->stream));
        ctx->launches += 1;
        CK(cudaMemcpyAsync(out_rgb, ctx->d_rgb, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    unsigned long long st[8];
    CK(cudaMemcpy(st, ctx->d_stats, sizeof(st), cudaMemcpyDeviceToHost));
    ctx->stats.camera_rays = st[0];
    ctx->stats.extension_rays = st[1];
    ctx->stats.shadow_rays = st[2];
    ctx->stats.closest_node_visits = st[3];
    ctx->stats.closest_tri_tests = st[4];
    ctx->stats.shadow_node_visits = st[5];
    ctx->stats.shadow_tri_tests = st[6];
    ctx->stats.kernel_launches = ctx->launches;
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
    if (t->tri_mode < 0 || t->tri_mode > 3) return fail(ctx, GB_ERR_INVALID, "tri_mode must be 1..3 (0 keeps)");
    if (t->tri_mode) ctx->tri_mode = t->tri_mode - 1;
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
    CK(cudaSetDevice(ctx->device));
    ShadeParams sp = make_shade_params(*desc);
    CK(k_launch_shade_stage(scene->S, w * h, sp, ray_orig, ray_dir, max_t, (const float4*)hits, shadow_occluded, rnd,
                            throughput, col_accum, to_light, psc, path, bounce, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return GB_OK;
}

int gb_mrg_pool(gb_ctx* ctx, int npix, uint32_t seed, int first_update, int num_updates, float* out) {
    if (!ctx || npix <= 0 || first_update < 0 || num_updates <= 0 || !out)
        return fail(ctx, GB_ERR_INVALID, "bad arguments");
    CK(cudaSetDevice(ctx->device));
    size_t bytes = sizeof(float) * 3 * (size_t)npix * (size_t)num_updates;
    void* d = nullptr;
    CK(cudaMalloc(&d, bytes));
    cudaError_t e = k_launch_mrg_pool(npix, seed, first_update, num_updates, (float*)d, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "mrg pool");
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
