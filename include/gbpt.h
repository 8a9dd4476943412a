/* gbpt.h -- C ABI of the GB300 path-tracing hot path (libgbpt.so).
 *
 * Drop-in boundary for globillum's `hybrid_pt` integrator: the library owns
 * the device memory of a scene and of a frame, runs the whole progressive
 * frame (camera rays, closest-hit, area-light sample, any-hit shadow ray,
 * BRDF sample/eval, moving-average accumulation) as a wavefront of
 * hand-written sm_103a kernels, and exposes the per-stage entry points the
 * reference's hybrid bouncer calls on the CPU.  Plain C types only; every
 * call returns a status code, no exception crosses the ABI, and
 * gb_last_error() gives the message of the last failing call of a context.
 * One context per host thread.
 *
 * Reference interfaces replaced (kiselgra/globillum, src/):
 *   gi_algorithm / hybrid_pt          gi_algorithm.h:12-68, hybrid-pt.h:256-288
 *   hybrid_pt::activate/compute/update hybrid-pt.cpp:65-174
 *   hybrid_pt_bouncer (bounce loop)   hybrid-pt.h:16-253
 *   rta::generate_arealight_sample    arealight-sampler-cpu.cpp:144-156
 *   compute_path_contribution_and_bounce hybrid-pt.cpp:450-584
 *   closest / any-hit tracers (rta bbvh-cuda) hl-main.cpp:375-385, tracers.cu:38-140
 *   gi::cuda::generate_mt_pool_on_gpu / update_mt_pool util-kernels.cu:277-333
 *   gi::cuda::generate_halton_pool_on_gpu util.cpp:38-51
 */
#ifndef GBPT_H
#define GBPT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ status codes */
enum {
    GB_OK = 0,
    GB_ERR_INVALID = 1,     /* bad argument / handle / size                       */
    GB_ERR_CUDA = 2,        /* a CUDA runtime call failed                         */
    GB_ERR_OOM = 3,         /* device or host allocation failed                   */
    GB_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up                 */
    GB_ERR_TRAVERSAL = 5,   /* traversal stack or iteration bound exceeded         */
    GB_ERR_UNSUPPORTED = 6  /* feature not available (e.g. no CUDA device)         */
};

typedef struct gb_ctx gb_ctx;
typedef struct gb_scene gb_scene;

/* --------------------------------------------------------------- context */
typedef struct {
    int device;             /* CUDA device ordinal                                */
    void* stream;           /* cudaStream_t to launch on; NULL = library-owned    */
} gb_ctx_desc;

/* Creates a context on `device`.  Replaces the implicit global CUDA state of
 * the reference (checked_cuda + cudaDeviceSynchronize after every launch). */
int gb_ctx_create(const gb_ctx_desc* desc, gb_ctx** out);
void gb_ctx_destroy(gb_ctx* ctx);
/* Message of the last failing call on this context ("" if none). */
const char* gb_last_error(const gb_ctx* ctx);
/* Switches the stream later launches of this context use. */
int gb_ctx_set_stream(gb_ctx* ctx, void* stream);

/* ------------------------------------------------------------------ scene */
/* PrincipledBRDFParameters (principledParameters.h:7-22), same field order. */
typedef struct {
    float metallic, subsurface, specular, roughness, specular_tint, anisotropic;
    float sheen, sheen_tint, clearcoat, clearcoat_gloss, opacity, transmiss;
    float color[3];
    float tangent[3];
} gb_principled_params;

/* rta::cuda::material_t (material.h:142-184) without textures: a material is
 * principled when `principled` >= 0 (index into gb_scene_desc.params), else
 * Lambert with `diffuse` (ALL_MATERIAL_LAMBERT, material-wrapper.h:11). */
typedef struct {
    float diffuse[3];
    int principled;
} gb_material;

enum { GB_LIGHT_RECT = 0, GB_LIGHT_SKY = 1 };
/* gi::light with rect_light / sky_light (lights.h:94-154).
 * Rect: center, dir, up, col, wh; power < 0 means "compute it with the
 * add-rectlight rule" w*h*(r+g+b)*.333 (lights.cpp:92).
 * Sky: sky_rgb is a lat-long radiance map of sky_h rows (theta 0 .. pi) by
 * sky_w columns (phi 0 .. 2 pi), float RGB, copied at scene creation (the
 * texture add-skylight loads, lights.cpp:98-111); sky_scale scales the
 * light samples; power < 0 means scale * 4 pi (sky_diameter / 2)^2
 * (lights.cpp:104).  At most one sky light per scene. */
typedef struct {
    int type;
    float power;
    float center[3], dir[3], up[3], col[3];
    float wh[2];
    const float* sky_rgb;
    int sky_w, sky_h;
    float sky_scale, sky_diameter;
} gb_light;

/* An RGBA8 image of w x h texels (4 bytes each, rows top first). */
typedef struct {
    int w, h;
    const uint8_t* rgba;
} gb_texture;

typedef struct {
    int num_triangles;
    const float* positions;       /* 9 floats per triangle: a, b, c           */
    const float* normals;         /* 9 floats per triangle: na, nb, nc        */
    const int* material_index;    /* per triangle, into `materials`           */
    int num_materials;
    const gb_material* materials;
    int num_params;
    const gb_principled_params* params;
    int num_lights;
    const gb_light* lights;
    /* Diffuse textures (material_t::diffuse_texture, material.h:142-170):
     * textures[k] is RGBA8 with row 0 at t = 1 (texture_data after
     * convert_texture, material-conversion.cpp:18-35); mip levels are made at
     * scene creation (compute_mipmaps, material.cu:259-275).  texcoords holds
     * 6 floats per triangle (ta, tb, tc as (s, t)); diffuse_texture holds one
     * texture index or -1 per material.  All three may be 0 / NULL; a
     * description must be zero-initialised for callers without textures. */
    int num_textures;
    const gb_texture* textures;
    const float* texcoords;
    const int* diffuse_texture;
} gb_scene_desc;

typedef struct {
    int num_triangles, num_nodes, depth, binary_nodes;
    double build_ms;              /* BVH build wall time (GB_BVH_* below)     */
    size_t device_bytes;          /* resident scene bytes                     */
    float overall_light_power;    /* sum of light powers (hybrid-pt.cpp:74-78) */
    int builder;                  /* GB_BVH_* the tree was built with         */
    int build_passes;             /* clustering passes of GB_BVH_DEVICE_PLOC  */
} gb_scene_info;

/* BVH builders.  The reference builds a binary binned-SAH tree on the host
 * through rta (`-b bsah`, hl-main.cpp:375-385).
 *   GB_BVH_HOST_SAH     binned SAH on the host, collapsed to 8-wide nodes.
 *   GB_BVH_DEVICE_PLOC  on the GPU: Morton order, parallel locally-ordered
 *                       clustering, then the same 8-wide collapse rules, level
 *                       by level; scenes built this way can be refitted.
 * Both trees give identical frames (closest hits are the minimum (t, id)). */
enum { GB_BVH_HOST_SAH = 0, GB_BVH_DEVICE_PLOC = 1 };
typedef struct {
    int builder;                  /* GB_BVH_*                                 */
    int ploc_radius;              /* clustering search radius, 1 .. 32; 0 = 16 */
    int wide_collapse;            /* grouping of binary nodes into 8-wide nodes (both
                                     builders): 0 / 1 = SAH-optimal grouping by dynamic
                                     programming over slot counts (Ylitie et al. 2017; the
                                     default), 2 = open the largest child until 8 */
    float prim_cost;              /* triangle test cost against a node visit for the
                                     SAH-optimal grouping; 0 = 1.2 */
    int sah_bins;                 /* GB_BVH_HOST_SAH: bins per axis of the binned SAH,
                                     2 .. 64; 0 = 32 */
} gb_build_options;

/* Host BVH build alone (GB_BVH_HOST_SAH; no device needed): the tree
 * gb_scene_create_ex would upload, summarised.  For inspecting build options
 * before a scene is made. */
typedef struct {
    int num_nodes, depth, binary_nodes, num_triangles;
    double build_ms;
} gb_bvh_stats;
int gb_bvh_build_stats(const float* positions, int num_triangles, const gb_build_options* opts, gb_bvh_stats* out);

/* Uploads triangles, materials and lights and builds the BVH (replaces
 * setup_rta's plugin_create_rt_set + convert_and_upload_materials,
 * hl-main.cpp:357-464, and hybrid_pt::activate's light copy).
 * gb_scene_create uses GB_BVH_HOST_SAH. */
int gb_scene_create(gb_ctx* ctx, const gb_scene_desc* desc, gb_scene** out);
int gb_scene_create_ex(gb_ctx* ctx, const gb_scene_desc* desc, const gb_build_options* opts, gb_scene** out);
void gb_scene_destroy(gb_scene* scene);
int gb_scene_get_info(const gb_scene* scene, gb_scene_info* info);

/* Moves the vertices of a GB_BVH_DEVICE_PLOC scene: positions (9 floats per
 * triangle, same count and order as at creation) and optional normals (NULL:
 * face normals).  The tree keeps its topology; boxes are recomputed bottom-up
 * and the nodes re-quantised on the GPU.  No counterpart in the reference,
 * which rebuilds (plugin_create_rt_set).  GB_ERR_UNSUPPORTED for host-built
 * scenes. */
int gb_scene_refit(gb_scene* scene, const float* positions, const float* normals);

/* ----------------------------------------------------------------- camera */
/* crgs->setup(pos, dir, up, fovy) + jittered_lens_ray_generator
 * (hybrid-pt.cpp:86, :169; raygen.cu:61-118).  fovy_deg is the full
 * vertical field of view; aperture 0 gives the jittered pinhole. */
typedef struct {
    float pos[3], dir[3], up[3];
    float fovy_deg;
    float aperture, focus_distance, eye_to_lens;
} gb_camera;

/* ----------------------------------------------------------------- render */
enum {
    GB_RNG_MRG32K3A_POOL = 0,  /* light and path draws from the per-pixel MRG32k3a
                                  streams (curand_init(seed, pixel, 0)), 3 per bounce */
    GB_RNG_HALTON_LIGHT = 1    /* light draws (h2(i+1), h3(i+1), h3(i+1)) per pixel,
                                  path draws from MRG32k3a (util.cpp:38-51)        */
};

typedef struct {
    int width, height;
    int spp;                 /* path samples (init_path_samples)                   */
    int max_bounces;         /* path length (init_path_length)                     */
    int rng_mode;            /* GB_RNG_*                                            */
    uint32_t seed;           /* curand seed (0 in the reference)                    */
    float ray_offset;        /* 0.3 in the reference (hybrid-pt.cpp:551)            */
    float shadow_offset;     /* 0.9 in the reference (arealight-sampler-cpu.cpp:115) */
    float background[3];     /* (1,1,1) in the reference (hybrid-pt.cpp:52)          */
    int rr_start;            /* Russian roulette from this bounce; -1 = off (parity) */
} gb_render_desc;

/* Renders a full progressive frame (spp paths of max_bounces bounces per
 * pixel) and writes the moving-average image (float RGB, w*h*3, pixel
 * (x,y) at index y*w+x as output_color in hybrid-pt.h:35).  `out_rgb` may be
 * host memory (copied back inside the call) or device memory
 * (out_is_device = 1). */
int gb_render(gb_ctx* ctx, gb_scene* scene, const gb_camera* cam, const gb_render_desc* desc,
              float* out_rgb, int out_is_device);

/* Progressive form mirroring gi_algorithm::compute/update: begin sets up a
 * pass (new_pass, hybrid-pt.h:115-122), each step renders `paths` further
 * path samples (one update() of the reference advances half a bounce; here
 * a step is whole paths), read copies the current image. */
int gb_render_begin(gb_ctx* ctx, gb_scene* scene, const gb_camera* cam, const gb_render_desc* desc);
int gb_render_step(gb_ctx* ctx, int paths);
int gb_render_paths_done(const gb_ctx* ctx, int* done);
int gb_render_read(gb_ctx* ctx, float* out_rgb, int out_is_device);

/* ------------------------------------------------------- direct lighting */
/* The reference's GPU direct-lighting integrator gpu_area_lights
 * (direct-lighting.cpp:29-104; samples as in arealight-sampler.cu:156-260,
 * :340-364): per pixel the material colour of the pixel-centre camera ray's
 * first hit (the MTL diffuse colour; desc->background for a miss) times
 * the moving average of `light_samples` area-light samples that reach their
 * light.  Uses width, height, seed, shadow_offset (0.01 in the reference)
 * and background of desc; light sample k draws update max(0, k-1) of the
 * pixel's MRG32k3a stream, as the reference's pool updates fall. */
int gb_render_direct(gb_ctx* ctx, gb_scene* scene, const gb_camera* cam, const gb_render_desc* desc,
                     int light_samples, float* out_rgb, int out_is_device);
/* The reference's hybrid direct-lighting integrator hybrid_area_lights
 * (direct-lighting.cpp:203-316, direct-lighting.h:137-215): per pixel
 * `camera_samples` jittered camera rays (the jittered lens generator of
 * hybrid_pt, jitter update c for camera sample c), the material colour of
 * each camera hit as in gb_render_direct, and per camera sample
 * `light_samples` samples of the CPU area-light sampler (the one hybrid_pt's
 * light samples use: desc->shadow_offset, 0.9 in the reference, and
 * importance-sampled sky), averaged over all camera x light samples.  Light
 * sample j of camera sample c draws update c*L + max(0, j-1) of the pixel's
 * MRG32k3a stream, as the reference's pool updates fall; jitter and light
 * draws come from the same stream (the reference seeds all its pools alike). */
int gb_render_hybrid_direct(gb_ctx* ctx, gb_scene* scene, const gb_camera* cam, const gb_render_desc* desc,
                            int camera_samples, int light_samples, float* out_rgb, int out_is_device);

/* ------------------------------------------------------------ batching */
/* One scene of a batch: its own camera, resolution, spp, bounces, RNG mode
 * and seed; out_rgb receives width*height*3 floats as in gb_render. */
typedef struct {
    gb_scene* scene;
    gb_camera camera;
    gb_render_desc desc;
    float* out_rgb;
} gb_batch_item;

/* Renders n scenes of one context as one wavefront frame: their pixels share
 * the slot pool, so small scenes fill the GPU together and every traversal
 * lane carries the geometry of its own scene.  Each scene's image is
 * bit-identical to a gb_render of that scene alone.  graph_capture = 1 runs
 * each chunk of path samples as one CUDA graph whose slot-pool loop is a
 * conditional while node (captured once per frame layout and reused);
 * 0 drives the loop from the host; -1 follows the context's tuning.  The reference renders one scene per
 * gi_algorithm (hybrid_pt::activate/compute, hybrid-pt.cpp:65-174); this
 * call has no counterpart there. */
int gb_render_batch(gb_ctx* ctx, int n, const gb_batch_item* items, int out_is_device, int graph_capture);

/* ------------------------------------------------------ differentiation */
/* Differentiable parameters of a scene, as one float vector: per material
 * (in gb_scene_desc order) base colour r, g, b, roughness, metallic (the
 * principled set's color / roughness / metallic, or a Lambert material's
 * diffuse colour with two unused entries), then per light emission r, g, b.
 * The reference has no derivatives; these calls have no counterpart there. */
int gb_scene_param_count(const gb_scene* scene, int* n);
int gb_scene_get_params(const gb_scene* scene, float* params);
/* Replaces the parameters (materials and light emission; a light described
 * with power < 0 gets its power recomputed by the add-rectlight rule). */
int gb_scene_set_params(gb_scene* scene, const float* params);

/* Forward pass of the path-replay adjoint.  eval_params = NULL renders
 * exactly as gb_render.  Otherwise the frame is replayed with every random
 * choice (camera jitter, light pick and point, BRDF lobe and direction,
 * roulette) made with the scene's current parameters while the BRDF values
 * and emission are evaluated with eval_params: the function whose
 * derivative gb_backward returns, so finite differences of it at common
 * random numbers check the adjoint. */
int gb_forward(gb_ctx* ctx, gb_scene* scene, const gb_camera* cam, const gb_render_desc* desc,
               const float* eval_params, float* out_rgb, int out_is_device);

/* Backward pass: gradient of a loss with respect to the scene's parameters,
 * given dL_dimg = dLoss/d(image) (w*h*3 floats, host or device).  The frame
 * is replayed from its random-number streams (no path is stored between the
 * passes); each path slot records its vertices (80 bytes per bounce, at
 * most 16 bounces) and, when the path ends, a reverse sweep adds
 * hand-written vector-Jacobian products of the BRDF evaluations and the
 * emission to per-block gradient copies, which are summed in double.  Pdfs,
 * lobe choices and roulette probabilities are held at their sampled values
 * (the derivative of gb_forward(eval_params) at eval_params = current).
 * dL_dparams receives gb_scene_param_count floats. */
int gb_backward(gb_ctx* ctx, gb_scene* scene, const gb_camera* cam, const gb_render_desc* desc,
                const float* dL_dimg, int dimg_is_device, float* dL_dparams);

typedef struct {
    gb_scene* scene;
    gb_camera camera;
    gb_render_desc desc;
    const float* dL_dimg;   /* width*height*3 */
    float* dL_dparams;      /* gb_scene_param_count of the scene (host) */
} gb_adjoint_item;

/* gb_backward for several scenes in one wavefront frame (as gb_render_batch;
 * graph_capture 1 / 0 / -1 as there). */
int gb_backward_batch(gb_ctx* ctx, int n, const gb_adjoint_item* items, int dimg_is_device, int graph_capture);

/* ---------------------------------------------------------------- ingest */
/* Scene assets gathered on the host into one gb_scene_desc, as the
 * reference's loader does (add_objfile_to_flat_tri_list, hl-main.cpp:277-354;
 * convert_and_upload_materials, material-conversion.cpp:59-148; the light /
 * add-rectlight forms, lights.scm:4-9 and lights.cpp:84-96).  Diffuse
 * texture maps (MTL map_Kd) are read when they are PPM files (P6 or P3, maxval
 * <= 255); other image formats are left out (the material keeps its Kd).
 * Sky forms of scene scripts are skipped. */
typedef struct gb_asset gb_asset;
int gb_asset_create(gb_asset** out);
void gb_asset_destroy(gb_asset* asset);
const char* gb_asset_last_error(const gb_asset* asset);
/* Appends the triangles of a Wavefront OBJ file (polygons fanned into
 * triangles; per-corner normals, or the face normal where a corner has none)
 * transformed by `trafo` (16 floats, row-major, NULL = identity; normals by
 * its inverse transpose).  Materials follow the OBJ's MTL library: a name
 * becomes a principled material when material_dir/<name>.pbrdf exists
 * (material_dir may be NULL), else Lambert with the MTL's Kd; faces without a
 * known material use the fallback material 0 (Lambert (1, 0, 0), created with
 * the first OBJ).  Texture coordinates (vt, "v/vt/vn" corners) are kept, 0 for
 * corners without one. */
int gb_asset_add_obj(gb_asset* asset, const char* obj_path, const char* material_dir, const float* trafo);
/* Appends the rectangular lights of a scene script: every (light "name"
 * :type :rect :color (list r g b) :pos (list ...) :dir (list ...) :up (list ...)
 * :dim (list w h)) form, with add-rectlight's power rule.  Other light types
 * are counted in *skipped_lights (may be NULL). */
int gb_asset_add_lights(gb_asset* asset, const char* script_path, int* skipped_lights);
int gb_asset_add_light(gb_asset* asset, const gb_light* light);
/* A description of everything gathered so far; its pointers stay valid
 * until the asset is changed or destroyed. */
int gb_asset_get_desc(const gb_asset* asset, gb_scene_desc* desc);
int gb_asset_material_name(const gb_asset* asset, int index, const char** name);
/* One .pbrdf parameter file (principledParameters.h:64-125): "key value"
 * pairs; keys absent from the file take the defaults of
 * principledParameters.h:23-24 (0, opacity 1, transmission 1). */
int gb_read_pbrdf(const char* path, gb_principled_params* out);

/* -------------------------------------------------------------- tracing */
/* triangle_intersection (t, beta, gamma, ref): ref = canonical triangle id,
 * 0xffffffff and t = FLT_MAX for a miss. */
typedef struct {
    float t, beta, gamma;
    uint32_t ref;
} gb_hit;

/* Closest hit for n rays (origin/direction 3 floats each, AoS; max_t per
 * ray).  Pointers are host memory unless `device_ptrs` is 1. */
int gb_trace_closest(gb_ctx* ctx, gb_scene* scene, int n, const float* orig, const float* dir,
                     const float* max_t, gb_hit* hits, int device_ptrs);
/* Any hit with 0 < t <= max_t: occluded[i] = 1 / 0.  max_t < 0 = no ray. */
int gb_trace_any(gb_ctx* ctx, gb_scene* scene, int n, const float* orig, const float* dir,
                 const float* max_t, uint8_t* occluded, int device_ptrs);

/* --------------------------------------------------------- hybrid stages */
/* GPU form of rta::generate_arealight_sample (arealight-sampler-cpu.cpp:144-156)
 * for a w x h pixel grid, device pointers, float3 = 3 packed floats:
 *   rnd[3*i]        light-stream draw of pixel i
 *   hits[i]         closest hits of this bounce
 *   ray_dir[3*i]    in: path ray direction (used for misses); out: shadow dir
 *   ray_orig, max_t out: shadow ray (max_t = -1 for misses)
 *   psc[3*i]        out: potential_sample_contribution */
int gb_generate_arealight_sample(gb_ctx* ctx, gb_scene* scene, int w, int h, float shadow_offset,
                                 const float* rnd, const gb_hit* hits, float* ray_orig,
                                 float* ray_dir, float* max_t, float* psc);

/* GPU form of compute_path_contribution_and_bounce (hybrid-pt.cpp:450-584),
 * device pointers, same buffers as the reference:
 *   ray_orig/ray_dir/max_t  path rays (in: this bounce, out: next bounce)
 *   hits, shadow_occluded   closest hits and any-hit results (1 = blocked)
 *   rnd                     path-stream draw; throughput, col_accum in/out
 *   to_light, psc           outputs of gb_generate_arealight_sample
 * `path` and `bounce` only feed the Russian-roulette extension. */
int gb_compute_path_contribution_and_bounce(gb_ctx* ctx, gb_scene* scene, int w, int h,
                                            const gb_render_desc* desc, float* ray_orig,
                                            float* ray_dir, float* max_t, const gb_hit* hits,
                                            const uint8_t* shadow_occluded, const float* rnd,
                                            float* throughput, float* col_accum,
                                            const float* to_light, const float* psc,
                                            int path, int bounce);

/* ----------------------------------------------------------- sample pools */
/* Draws of the per-pixel MRG32k3a streams: out[(u*npix + i)*3 + k] is draw
 * 3*(first_update+u)+k of pixel i's stream, i.e. what update_mt_pool
 * (util-kernels.cu:287-302) leaves in the pool at update first_update+u
 * (curand_init(seed, i, 0), 3 curand_uniform per update).  Host `out`. */
int gb_mrg_pool(gb_ctx* ctx, int npix, uint32_t seed, int first_update, int num_updates, float* out);
/* The same for pixels pixel0 .. pixel0 + npix - 1 (a band of rows of a
 * frame): out[(u*npix + i)*3 + k] is draw 3*(first_update+u)+k of pixel
 * pixel0 + i's stream, the pool slice the reference's bouncer downloads for
 * those pixels (hybrid-pt.h:232-233).  Host `out`. */
int gb_mrg_pool_range(gb_ctx* ctx, int pixel0, int npix, uint32_t seed, int first_update, int num_updates,
                      float* out);
/* The MRG32k3a states curand_init(seed, subsequences[i], 0) leaves, as
 * out[6 i .. 6 i + 5] = s1[0..2], s2[0..2].  method 0: curand_init itself
 * (the reference's seeding call, util-kernels.cu:284); method 1: the
 * library's own jump-ahead, which the frame, gpu_area_lights and
 * hybrid_area_lights kernels use to start their pixel streams.  Host
 * buffers. */
int gb_mrg_states(gb_ctx* ctx, uint32_t seed, const uint32_t* subsequences, int n, int method, uint32_t* out);

/* ------------------------------------------------------------- statistics */
typedef struct {
    uint64_t camera_rays, extension_rays, shadow_rays;  /* traced in the last render  */
    /* traversal work, only counted by gb_render_instrumented                        */
    uint64_t closest_node_visits, closest_tri_tests;    /* camera + extension rays    */
    uint64_t shadow_node_visits, shadow_tri_tests;      /* shadow (any-hit) rays      */
    uint64_t kernel_launches;                           /* launches of the last render */
    double render_ms;                                   /* device time, begin -> last step */
    /* per-stage device time when stage timing is on (gb_ctx_set_stage_timing):
     * 0 path start, 1 closest-hit + light sample, 2 any-hit, 3 shade,
     * 4 path end + restart, 5 moving average                                   */
    double stage_ms[6];
    uint64_t stage_launches[6];
    int paths_done;
    uint64_t light_samples;  /* closest hits, each with its light sample; only
                              * counted by gb_render_instrumented          */
} gb_stats;

/* Knobs of the wavefront (chosen by the autotuner); 0 keeps a value:
 *   refill    idle lanes (1..32) at which a closest-hit traversal warp
 *             fetches new rays, default 20 (any-hit warps refill at 12)
 *   slots     paths in flight (queue capacity), default 2^24 (a frame
 *             allocates min(its paths, slots); 256 B of path state per slot;
 *             the adjoint replay uses at most 2^22)
 *   sample_mb budget of the per-path sample buffer, which bounds how many
 *             path samples per pixel one pass of the slot pool covers */
typedef struct {
    int refill;
    int slots;
    int sample_mb;
    int tri_mode;   /* traversal triangle policy + 1: 1 = every pending triangle then a
                       node; 2 / 3 = postpone triangle groups when fewer than a fifth of a
                       warp's active lanes have any, else test one (2) / all (3);
                       4 = the warp tests all lanes' pending triangles together
                       (32 at a time), then every lane visits one node */
    int graph;      /* 1 = the host drives the slot-pool loop of single renders; 2 = each
                       chunk runs as one CUDA graph with a conditional while loop (default) */
    int blocks_per_sm; /* resident 128-thread blocks per SM of the persistent traversal
                          kernels + 1: 1 = as many as occupancy allows, k + 1 = at most k */
    int stack_depth;   /* node-group stack entries of the traversal kernels: 24 or 32
                          (default 32; the reference's tracers keep 32, tracers.cu:55).  A
                          ray that needs more ends the render with GB_ERR_TRAVERSAL */
    int block_threads; /* threads per block of the traversal kernels: 64 or 128 (default;
                          the reference launches 16x16 blocks).  stack_depth and
                          block_threads apply to triangle policy 1; the others run 32 / 128 */
} gb_tuning;
int gb_ctx_set_tuning(gb_ctx* ctx, const gb_tuning* tuning);
int gb_ctx_get_tuning(const gb_ctx* ctx, gb_tuning* tuning);

/* Which derivative the adjoint computes (no counterpart in the reference).
 * sampling = 0 (default): the derivative of the frame with every random
 * decision frozen at the current parameters -- exactly the derivative of
 * gb_forward(eval_params), with the BRDF "pdf" (the Walter weight of the
 * metallic lobe) held fixed.  sampling = 1: also the derivatives of the
 * sampling decisions that depend on the parameters, so that the gradient
 * estimates the derivative of the expected frame:
 *  - the metallic lobe choice (rnd.z < metallic, principledMaterial.h:365)
 *    by its score times everything the choice moves.  With MRG32k3a light
 *    draws the light pick reads the same rnd.z, so the score is taken given
 *    the picked light's interval (lo, hi] of rnd.z: 1/(metallic - lo) for
 *    the metallic branch, -1/(hi - metallic) for the diffuse one, 0 when
 *    metallic lies outside the interval; with Halton light draws lo = 0,
 *    hi = 1;
 *  - the roughness dependence of the GTR2 half-vector density (:46-61) by
 *    its score times what follows the vertex;
 *  - the roughness dependence of the Walter weight (:121-176) through the
 *    throughput.
 * The survival probability q of the Russian-roulette extension is held
 * fixed in both forms; for the expected frame that is exact (the survival
 * score d log q cancels the derivative of the 1/q weight).  Not covered:
 * the jump of a miss's contribution where a throughput reaches the clamp to
 * exactly (1, 1, 1) (hybrid-pt.cpp:567-572 add the white background then),
 * a discontinuity in the parameters.  Applies to gb_backward,
 * gb_backward_batch and gb_fit_step. */
int gb_ctx_set_gradient_terms(gb_ctx* ctx, int sampling);

/* ------------------------------------------------ batched fitting steps */
/* One scene of a fitting step: the frame it renders and the image it is
 * fitted to. */
typedef struct {
    gb_scene* scene;
    gb_camera camera;
    gb_render_desc desc;
    const float* target;    /* device, width*height*3 floats: the image to match */
    float* image;           /* device, width*height*3 floats, or NULL: receives the frame */
} gb_fit_item;

/* Batched inverse rendering as one CUDA graph launch per step (no
 * counterpart in the reference, which has no derivatives).  A step sets
 * every scene's parameters, renders the scenes as one batched frame,
 * computes each scene's L2 loss sum over pixels and channels of
 * (image - target)^2 and its image gradient on the device, runs the
 * path-replay adjoint of that gradient over the same batch (as
 * gb_backward_batch) and reduces the parameter gradients: the parameter
 * upload, both frames, the loss and the reduction are one captured graph,
 * launched once per step; the image gradients never leave the device.
 * gb_fit_prepare(ctx, n, items) lays the batch out and captures the graph
 * (1..1024 scenes, each at most once; the restrictions of
 * gb_backward_batch apply).  The targets and images must stay valid and the
 * scenes must not be used by other calls while steps run.  Renders on the
 * same context in between may grow its buffers; the next step then
 * captures the graph again by itself. */
int gb_fit_prepare(gb_ctx* ctx, int n, const gb_fit_item* items);
/* One step: params[i] (host, gb_scene_param_count floats) become item i's
 * scene parameters, as gb_scene_set_params sets them; dL_dparams[i] (host)
 * receives the gradient of item i's loss and loss[i] (host, or NULL) the
 * loss. */
int gb_fit_step(gb_ctx* ctx, const float* const* params, float* const* dL_dparams, double* loss);

/* Autotuner of the wavefront knobs (gb_tuning: graph capture, slot-pool
 * capacity, refill threshold, triangle policy, resident traversal blocks per
 * SM, traversal stack depth and block shape) for a batch (or one scene, n = 1): coordinate descent from the
 * context's current tuning, two passes at most, each candidate timed as the
 * median device time of `repeats` frames after a warm-up frame.  With
 * proxy_spp > 0 every scene renders min(spp, proxy_spp) samples per trial
 * (a cheaper frame of the same layout).  A candidate whose frame fails (a
 * traversal stack too shallow for a tree) is skipped.  Leaves the best tuning set on the
 * context and returns it with its frame time; out_rgb of the items is not
 * used.  The reference has no tunable launch parameters; no counterpart. */
int gb_autotune(gb_ctx* ctx, int n, const gb_batch_item* items, int proxy_spp, int repeats,
                gb_tuning* best, double* best_ms);

/* Records CUDA events around every stage launch of later renders on the
 * context's stream (for per-kernel timing); off by default. */
int gb_ctx_set_stage_timing(gb_ctx* ctx, int on);
int gb_get_stats(const gb_ctx* ctx, gb_stats* stats);
/* Same as gb_render but counts 8-wide node visits and triangle tests of
 * every traced ray (slower; used for the roofline's algorithmic bytes). */
int gb_render_instrumented(gb_ctx* ctx, gb_scene* scene, const gb_camera* cam,
                           const gb_render_desc* desc, float* out_rgb, int out_is_device);

/* Allocation-free gb_render (no counterpart in the reference).  For callers
 * that must not allocate device memory while rendering -- e.g. a loop that
 * shares the GPU with work whose memory lives in its own pool, where
 * cudaMalloc/cudaFree would synchronise the device and fragment that pool.
 * The scene is created beforehand (gb_scene_create allocates); this call
 * renders the same frame as gb_render into the caller's device buffer
 * `out_rgb` (w*h*3 floats) on `stream` (NULL = legacy default stream), with
 * its wavefront state in one fixed file-scope device array (about 27 MB,
 * held by every GPU that loads the library until exit) instead of cudaMalloc.
 * Limits: w*h <= 65536 pixels and max_bounces <= 64, else GB_ERR_INVALID;
 * scenes with texture coordinates return GB_ERR_UNSUPPORTED (use gb_render).
 * The first call on a device looks the array up (cudaGetSymbolAddress) with
 * the scene's device current; the caller's current device is restored
 * before the call returns.  Every call synchronises `stream` and reads
 * counters back to the host, so it must never be called while `stream` is
 * capturing (GB_ERR_INVALID).  All calls share the array: calls that overlap
 * on the GPU race; serialise them.  Returns after the frame is finished;
 * errors are reported through the scene's context (gb_last_error), so do
 * not run other calls on that context from another thread meanwhile. */
int gb_render_noalloc(const gb_scene* scene, const gb_camera* cam, const gb_render_desc* desc,
                      float* out_rgb, void* stream);

/* Test hook (host-side fault injection): after `alloc_fail_after` further
 * device allocations made by the library, the next one fails as if the
 * device were out of memory (the call returns GB_ERR_OOM and the context
 * stays usable).  A negative value disarms it.  Process-wide. */
int gb_set_fault_injection(int alloc_fail_after);

/* Bytes of one stored 8-wide node / triangle (for roofline arithmetic). */
int gb_layout_sizes(int* node_bytes, int* tri_bytes);

#ifdef __cplusplus
}
#endif

#endif /* GBPT_H */
