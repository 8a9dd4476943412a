// gbpt_noalloc.cu -- gb_render_noalloc: the progressive frame of gb_render
// without any device allocation.
//
// gb_render keeps its per-pixel wavefront state (rays, throughput,
// accumulators, RNG streams, queues) in buffers a context allocates with
// cudaMalloc on first use.  Some callers cannot allow that: a render loop
// that runs while other work owns the device's memory through its own pool
// (cudaMalloc and cudaFree synchronise the whole device and fragment such a
// pool), or code on a path where the host must not block in the CUDA
// driver's allocator.  For them this entry point keeps that state in one
// file-scope __device__ array of fixed size instead.  Every GPU that loads
// the library holds the array until the process exits.
//
// Limits: at most kNoAllocMaxPixels pixels (a 256 x 256 frame) and at most
// kNoAllocMaxBounces bounces per call; larger requests return
// GB_ERR_INVALID.  All calls share the one array, so calls whose work
// overlaps on the GPU (two streams, or two host threads) race and corrupt
// each other's frames: serialise them.
//
// Set-up: the first call on a device, with that device current, looks up the
// array's device address (cudaGetSymbolAddress) and caches it.  The call
// synchronises its stream and reads counters back to the host on every pass,
// so it must never be called while its stream is capturing (it returns
// GB_ERR_INVALID then).  It makes the scene's device current for its work
// and gives the caller's current device back before it returns.  Errors are
// recorded in the scene's context (gb_last_error): do not run other calls on
// that context from another thread at the same time.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/gbpt.h"
#include "gbpt_host.h"
#include "gbpt_kernels.h"

namespace gb {
const DevScene* scene_device_view(const gb_scene* s);
int scene_device(const gb_scene* s);
void scene_set_error(const gb_scene* s, const char* msg);
}  // namespace gb

using namespace gb;

namespace {

constexpr int kNoAllocMaxPixels = 65536;
constexpr int kNoAllocMaxBounces = 64;
constexpr int kMaxDevices = 64;
constexpr size_t kAlign = 256;

constexpr size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }
constexpr size_t kV4 = align_up(sizeof(float4) * (size_t)kNoAllocMaxPixels);  // one float4 per slot / pixel
constexpr size_t kRng = align_up(sizeof(MrgState) * (size_t)kNoAllocMaxPixels);  // MRG32k3a words per slot / pixel
constexpr size_t kU32 = align_up(4 * (size_t)kNoAllocMaxPixels);              // one 32-bit word per slot
constexpr size_t kCtr = align_up(4 * 32);
constexpr size_t kStats = align_up(16 * 8);
constexpr size_t kStatus = align_up(4);
constexpr size_t kRec = align_up(sizeof(SceneRec));
constexpr size_t kSlots = kSlotBytes * (size_t)kNoAllocMaxPixels;  // slot records
constexpr size_t kShadow = GB_SHADOW_SPLIT ? 32 * (size_t)kNoAllocMaxPixels : 0;  // shadow rays
// One slot per pixel and one path sample per pass: the slot records and
// 4 queues; per pixel the image, the
// initial RNG states, the two stream cursors, the scene word, one sample,
// one stream state and
// one jitter value; counters, path counter, iteration, stats, status and the
// scene record.
constexpr size_t kScratchBytes = kSlots + kShadow + 4 * kU32 + kV4 + 4 * kRng + kU32 + 2 * kV4 + kCtr +
                                 kCtr + kCtr + kStats + kStatus + kRec;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mutex;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

// Device address of the array on `dev` (current device), looked up once.
cudaError_t scratch_on_device(int dev, unsigned char** out) {
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = (unsigned char*)p;
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

Frame carve(unsigned char* base, int n, SceneRec** rec) {
    Frame F{};
    F.ntot = n;
    F.nslots = n;
    F.nscenes = 1;
    size_t off = 0;
    bind_slots(F, base + off, base + off + kSlots); off += kSlots + kShadow;
    for (int k = 0; k < 4; ++k) { F.q[k] = (uint32_t*)(base + off); off += kU32; }
    F.out = (float4*)(base + off); off += kV4;
    F.pristine = (MrgState*)(base + off); off += kRng;
    F.cursor = (MrgState*)(base + off); off += kRng;
    F.spool = (MrgState*)(base + off); off += kRng;
    F.jcursor = (MrgState*)(base + off); off += kRng;
    F.pscene = (uint32_t*)(base + off); off += kU32;
    F.samples = (float4*)(base + off); off += kV4;
    F.jpool = (float4*)(base + off); off += kV4;
    F.ctr = (uint32_t*)(base + off); off += kCtr;
    F.path_ctr = (uint32_t*)(base + off); off += kCtr;
    F.iter = (int*)(base + off); off += kCtr;
    F.stats = (unsigned long long*)(base + off); off += kStats;
    F.status = (uint32_t*)(base + off); off += kStatus;
    *rec = (SceneRec*)(base + off);
    F.scenes = *rec;
    return F;
}

int fail(const gb_scene* s, int code, const char* msg) {
    scene_set_error(s, msg);
    return code;
}

// The caller's current device, made current again when the call returns.
struct DeviceRestore {
    int prev = -1;
    DeviceRestore() {
        if (cudaGetDevice(&prev) != cudaSuccess) { cudaGetLastError(); prev = -1; }
    }
    ~DeviceRestore() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

int render_noalloc(const gb_scene* scene, const gb_camera* cam, const gb_render_desc* d, float* out_rgb,
                   void* stream);

}  // namespace

extern "C" int gb_render_noalloc(const gb_scene* scene, const gb_camera* cam, const gb_render_desc* d,
                                 float* out_rgb, void* stream) {
    DeviceRestore restore;
    return render_noalloc(scene, cam, d, out_rgb, stream);
}

namespace {

int render_noalloc(const gb_scene* scene, const gb_camera* cam, const gb_render_desc* d, float* out_rgb,
                   void* stream) {
    if (!scene || !cam || !d || !out_rgb) return fail(scene, GB_ERR_INVALID, "gb_render_noalloc: null argument");
    if (d->width <= 0 || d->height <= 0 || d->spp <= 0 || d->max_bounces <= 0)
        return fail(scene, GB_ERR_INVALID, "gb_render_noalloc: bad resolution / spp / bounces");
    if ((long long)d->width * d->height > kNoAllocMaxPixels)
        return fail(scene, GB_ERR_INVALID, "gb_render_noalloc: more than 65536 pixels (256 x 256) per call");
    if (d->max_bounces > kNoAllocMaxBounces)
        return fail(scene, GB_ERR_INVALID, "gb_render_noalloc: more than 64 bounces");
    if (d->rng_mode != GB_RNG_MRG32K3A_POOL && d->rng_mode != GB_RNG_HALTON_LIGHT)
        return fail(scene, GB_ERR_INVALID, "gb_render_noalloc: bad rng_mode");
    if (!(cam->fovy_deg > 0.0f && cam->fovy_deg < 180.0f))
        return fail(scene, GB_ERR_INVALID, "gb_render_noalloc: bad fovy");
    int dev = scene_device(scene);
    if (dev < 0 || dev >= kMaxDevices) return fail(scene, GB_ERR_INVALID, "gb_render_noalloc: bad scene device");
    if (scene_device_view(scene)->texcoord)
        return fail(scene, GB_ERR_UNSUPPORTED, "gb_render_noalloc: scenes with texture coordinates need gb_render");
    if (cudaSetDevice(dev) != cudaSuccess) { cudaGetLastError(); return fail(scene, GB_ERR_CUDA, "cudaSetDevice failed"); }
    unsigned char* base = nullptr;
    if (scratch_on_device(dev, &base) != cudaSuccess) {
        cudaGetLastError();
        return fail(scene, GB_ERR_CUDA, "gb_render_noalloc: cudaGetSymbolAddress of the scratch array failed");
    }
    cudaStream_t st = (cudaStream_t)stream;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) {
        cudaGetLastError();
        return fail(scene, GB_ERR_CUDA, "gb_render_noalloc: cudaStreamIsCapturing failed");
    }
    if (cap != cudaStreamCaptureStatusNone)
        return fail(scene, GB_ERR_INVALID, "gb_render_noalloc: the stream is capturing (the call synchronises it)");
    const int n = d->width * d->height;
    SceneRec* d_rec = nullptr;
    Frame F = carve(base, n, &d_rec);
    SceneRec R{};
    R.S = *scene_device_view(scene);
    R.cam = make_camera(*cam, d->width, d->height);
    R.sp = make_shade_params(*d);
    R.w = d->width;
    R.h = d->height;
    R.n = n;
    R.spp = d->spp;
    R.L = d->max_bounces;
    R.rng_mode = d->rng_mode;
    R.pixel_base = 0;
    R.seed = d->seed;
    mrg_jump_matrices(3ull * (uint64_t)R.L, R.jump1, R.jump2);
    RenderParams P{};
    P.refill = 16;
    P.tri_mode = 0;
    P.blocks_per_sm = 0;
    P.rounds = 1;
    P.round_start[0] = 0;
    P.round_start[1] = (uint32_t)n;
    P.chunk_paths = (uint32_t)n;
    cudaError_t e = cudaMemcpyAsync(d_rec, &R, sizeof(R), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(F.stats, 0, 16 * 8, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(F.status, 0, 4, st);
    if (e == cudaSuccess) e = k_launch_frame_init(F, true, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(F.cursor, F.pristine, sizeof(MrgState) * (size_t)n, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(F.jcursor, F.pristine, sizeof(MrgState) * (size_t)n, cudaMemcpyDeviceToDevice, st);
    // one path sample of every pixel per pass, one slot per pixel: a path
    // has at most max_bounces segments, so the queue is empty after
    // max_bounces + 1 iterations; the host checks the queue count every 8
    // iterations and the device flags a queue still non-empty after
    // max_bounces + 2 iterations (ST_ITER_LIMIT)
    const int max_iters = d->max_bounces + 2;
    uint32_t left = 0;
    for (int p = 0; p < d->spp && e == cudaSuccess; ++p) {
        P.p0 = p;
        e = cudaMemsetAsync(F.ctr, 0, sizeof(uint32_t) * 24, st);
        if (e == cudaSuccess) e = k_launch_jitter_pool(F, P, st);
        if (e == cudaSuccess) e = k_launch_start(F, P, n, st);
        left = 1;
        for (int it = 0; e == cudaSuccess && left != 0u && it < max_iters; ++it) {
            e = k_launch_extend(F, P, false, st);
            if (e == cudaSuccess) e = k_launch_shadow(F, P, false, st);
            if (e == cudaSuccess) e = k_launch_shade(F, P, st);
            if (e == cudaSuccess) e = k_launch_regen(F, P, st);
            if (e == cudaSuccess) e = k_launch_step(F, P, 0, false, max_iters, st);
            if (e == cudaSuccess && (it % 8 == 7 || it == d->max_bounces || it == max_iters - 1)) {
                e = cudaMemcpyAsync(&left, F.ctr + 8 * ((it + 1) % 3), sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
                if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            }
        }
        if (e == cudaSuccess && left != 0u) break;  // paths still queued: reported below
        if (e == cudaSuccess) e = k_launch_combine(F, P, st);
    }
    if (e == cudaSuccess) e = k_launch_pack_rgb(F.out, n, out_rgb, st);
    uint32_t status = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&status, F.status, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(scene, GB_ERR_CUDA, cudaGetErrorString(e));
    }
    if (status || left != 0u) return fail(scene, GB_ERR_TRAVERSAL, "gb_render_noalloc: traversal bound exceeded");
    return GB_OK;
}

}  // namespace
