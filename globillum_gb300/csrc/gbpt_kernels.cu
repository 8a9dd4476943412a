// gbpt_kernels.cu -- sm_103a kernels of the GB300 path-tracing hot path.
//
// Wavefront per path sample (one "generation" = path p of every pixel):
//   k_raygen   camera rays (raygen.cu:61-118), jitter stream, stream skip
//   per bounce b:
//     k_extend  closest-hit traversal of the extension queue; misses add
//               handle_no_hit's contribution (hybrid-pt.cpp:196-206); hits
//               draw the bounce's 3 uniforms and emit the area-light shadow
//               ray (arealight-sampler-cpu.cpp:25-143) into the shadow queue
//     k_shade   any-hit traversal of the shadow queue fused with the
//               BRDF sample/eval and throughput update of
//               compute_path_contribution_and_bounce (hybrid-pt.cpp:450-584);
//               surviving paths go to the next extension queue
//   k_finalize moving average of the finished path into the image
//              (new_path -> combine_color_samples, util-kernels.cu:17-25)
// Queues are compacted with one warp ballot + one atomic per warp; queue
// kernels run a persistent grid that fetches 32 rays per warp at a time.
//
// Traversal: compressed 8-wide BVH (80 B nodes, 8-bit quantised child
// boxes), node-group stack of 32 entries, octant-ordered child visits,
// conservative slab tests (relative slack 1e-5 on top of outward-rounded
// boxes), so the result equals the (t, id)-minimum over all triangles.
#include "gbpt_kernels.h"

#include <curand_kernel.h>

namespace gb {

namespace {

constexpr int kBlock = 128;
constexpr int kStack = 32;
constexpr int kIterLimit = 1 << 22;

__device__ __forceinline__ v3 ld3(const float4 a) { return mk(a.x, a.y, a.z); }

__device__ __forceinline__ float byte_f(uint32_t w, int sh) { return (float)((w >> sh) & 0xffu); }

struct RayInv {
    v3 o, d, idir;
    uint32_t oxor;
};

__device__ __forceinline__ RayInv make_ray(v3 o, v3 d) {
    RayInv r;
    r.o = o; r.d = d;
    const float ooeps = 8.271806125530277e-25f;  // 2^-80 (tracers.cu:48-51)
    r.idir.x = 1.0f / (fabsf(d.x) > ooeps ? d.x : copysignf(ooeps, d.x));
    r.idir.y = 1.0f / (fabsf(d.y) > ooeps ? d.y : copysignf(ooeps, d.y));
    r.idir.z = 1.0f / (fabsf(d.z) > ooeps ? d.z : copysignf(ooeps, d.z));
    uint32_t oct = (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
    r.oxor = oct ^ 7u;
    return r;
}

// Intersects the 8 children of node `ni`; returns the node group (child
// base, hit bits 24-31 in visit order | imask) and the triangle group.
__device__ __forceinline__ void intersect_node(const float4* __restrict__ nodes, uint32_t ni, const RayInv& r,
                                               float bound, uint2* ng, uint2* tg) {
    const float4* n = nodes + 5 * (size_t)ni;
    float4 n0 = __ldg(n + 0), n1 = __ldg(n + 1), n2 = __ldg(n + 2), n3 = __ldg(n + 3), n4 = __ldg(n + 4);
    uint32_t ew = __float_as_uint(n0.w);
    float sx = __uint_as_float((ew & 0xffu) << 23);
    float sy = __uint_as_float(((ew >> 8) & 0xffu) << 23);
    float sz = __uint_as_float(((ew >> 16) & 0xffu) << 23);
    uint32_t imask = ew >> 24;
    float aix = sx * r.idir.x, aiy = sy * r.idir.y, aiz = sz * r.idir.z;
    float aox = (n0.x - r.o.x) * r.idir.x, aoy = (n0.y - r.o.y) * r.idir.y, aoz = (n0.z - r.o.z) * r.idir.z;
    uint32_t hits_n = 0, hits_t = 0;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        uint32_t meta_w = __float_as_uint(half ? n1.w : n1.z);
        uint32_t qlx = __float_as_uint(half ? n2.y : n2.x), qly = __float_as_uint(half ? n2.w : n2.z);
        uint32_t qlz = __float_as_uint(half ? n3.y : n3.x), qhx = __float_as_uint(half ? n3.w : n3.z);
        uint32_t qhy = __float_as_uint(half ? n4.y : n4.x), qhz = __float_as_uint(half ? n4.w : n4.z);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int sh = 8 * j;
            const int slot = 4 * half + j;
            uint32_t meta = (meta_w >> sh) & 0xffu;
            float x0 = fmaf(byte_f(qlx, sh), aix, aox), x1 = fmaf(byte_f(qhx, sh), aix, aox);
            float y0 = fmaf(byte_f(qly, sh), aiy, aoy), y1 = fmaf(byte_f(qhy, sh), aiy, aoy);
            float z0 = fmaf(byte_f(qlz, sh), aiz, aoz), z1 = fmaf(byte_f(qhz, sh), aiz, aoz);
            float tmin = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fminf(z0, z1));
            float tmax = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fmaxf(z0, z1));
            float lo = fmaxf(tmin * 0.99999f, 0.0f);
            float hi = fminf(tmax * 1.00001f, bound);
            if (meta != 0u && lo <= hi) {
                if ((imask >> slot) & 1u) hits_n |= 1u << (24 + (slot ^ r.oxor));
                else hits_t |= (meta >> 5) << (meta & 31u);
            }
        }
    }
    *ng = make_uint2(__float_as_uint(n1.x), hits_n | imask);
    *tg = make_uint2(__float_as_uint(n1.y), hits_t);
}

struct TraceOut {
    float t, beta, gamma;
    uint32_t id;
};

// Closest (ANY=false) or any (ANY=true) hit with 0 < t <= tmax.
template <bool ANY, bool INSTR>
__device__ __forceinline__ bool traverse(const DevScene& S, const RayInv& r, float tmax, TraceOut* out,
                                         uint32_t* status, uint32_t* nvis, uint32_t* ntri) {
    float best_t = FLT_MAX;
    uint32_t best_id = 0xffffffffu;
    float bb = 0.0f, bg = 0.0f;
    uint2 stack[kStack];
    int sp = 0;
    uint32_t oct = r.oxor ^ 7u;
    uint2 ng = make_uint2(0u, 0x80000000u | (1u << oct));
    uint2 tg = make_uint2(0u, 0u);
    int iters = 0;
    bool found = false;
    while (true) {
        while (tg.y != 0u) {
            int b = __ffs(tg.y) - 1;
            tg.y &= tg.y - 1u;
            const float4* tp = S.tris + 3 * (size_t)(tg.x + (uint32_t)b);
            float4 a0 = __ldg(tp + 0), a1 = __ldg(tp + 1), a2 = __ldg(tp + 2);
            if (INSTR) ++*ntri;
            float t, u, v;
            if (intersect_tri(r.o, r.d, ld3(a0), ld3(a1), ld3(a2), &t, &u, &v) && t <= tmax) {
                uint32_t id = __float_as_uint(a0.w);
                if (ANY) { found = true; tg.y = 0u; ng.y = 0u; sp = 0; break; }
                if (closer(t, id, best_t, best_id)) { best_t = t; best_id = id; bb = u; bg = v; }
            }
        }
        if (ANY && found) break;
        if (ng.y > 0x00ffffffu) {
            uint32_t k = 31u - (uint32_t)__clz(ng.y);
            ng.y &= ~(1u << k);
            uint32_t slot = (k - 24u) ^ r.oxor;
            uint32_t imask = ng.y & 0xffu;
            uint32_t child = ng.x + (uint32_t)__popc(imask & ((1u << slot) - 1u));
            if (ng.y > 0x00ffffffu) {
                if (sp >= kStack) { atomicOr(status, ST_STACK_OVERFLOW); break; }
                stack[sp++] = ng;
            }
            if (INSTR) ++*nvis;
            intersect_node(S.nodes, child, r, fminf(best_t, tmax), &ng, &tg);
        } else if (sp > 0) {
            ng = stack[--sp];
        } else {
            break;
        }
        if (++iters > kIterLimit) { atomicOr(status, ST_ITER_LIMIT); break; }
    }
    if (ANY) return found;
    out->t = best_t; out->beta = bb; out->gamma = bg; out->id = best_id;
    return best_id != 0xffffffffu;
}

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// Warp-aggregated append of `id` (when pred) to queue q with counter c.
__device__ __forceinline__ void push(bool pred, uint32_t id, uint32_t* q, uint32_t* c) {
    uint32_t mask = __ballot_sync(0xffffffffu, pred);
    if (mask == 0u) return;
    uint32_t leader = (uint32_t)__ffs(mask) - 1u;
    uint32_t base = 0u;
    if (lane_id() == leader) base = atomicAdd(c, (uint32_t)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, (int)leader);
    if (pred) q[base + (uint32_t)__popc(mask & ((1u << lane_id()) - 1u))] = id;
}

__device__ __forceinline__ void add_stats(unsigned long long* s, uint32_t v) {
    uint32_t w = __reduce_add_sync(0xffffffffu, v);
    if (lane_id() == 0u && w) atomicAdd(s, (unsigned long long)w);
}

// ----------------------------------------------------------------- kernels

__global__ void __launch_bounds__(kBlock) k_trace(DevScene S, int n, const float* __restrict__ orig,
                                                  const float* __restrict__ dir, const float* __restrict__ tmaxv,
                                                  float4* hits, uint8_t* occluded, int any, uint32_t* status) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    v3 o = mk(orig[3 * i], orig[3 * i + 1], orig[3 * i + 2]);
    v3 d = mk(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]);
    float tmax = tmaxv[i];
    RayInv r = make_ray(o, d);
    uint32_t nv = 0, nt = 0;
    if (any) {
        bool f = (tmax >= 0.0f) && traverse<true, false>(S, r, tmax, nullptr, status, &nv, &nt);
        occluded[i] = f ? 1 : 0;
    } else {
        TraceOut h;
        if (tmax >= 0.0f) traverse<false, false>(S, r, tmax, &h, status, &nv, &nt);
        else { h.t = FLT_MAX; h.beta = 0.0f; h.gamma = 0.0f; h.id = 0xffffffffu; }
        hits[i] = make_float4(h.t, h.beta, h.gamma, __uint_as_float(h.id));
    }
}

__global__ void k_rng_init(int n, uint32_t seed, curandStateMRG32k3a* rng, curandStateMRG32k3a* rngj, int* draws) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    curandStateMRG32k3a s;
    curand_init((unsigned long long)seed, (unsigned long long)i, 0ull, &s);
    rng[i] = s;
    rngj[i] = s;
    draws[i] = 0;
}

__device__ __forceinline__ v3 draw3(curandStateMRG32k3a* s) {
    float x = curand_uniform(s);
    float y = curand_uniform(s);
    float z = curand_uniform(s);
    return mk(x, y, z);
}

// Jitter pool for the thin-lens camera (the lens sample reads another pixel).
__global__ void k_jitter_pool(Frame F) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= F.n) return;
    curandStateMRG32k3a* js = (curandStateMRG32k3a*)F.rngj;
    curandStateMRG32k3a s = js[i];
    v3 j = draw3(&s);
    js[i] = s;
    F.jpool[i] = make_float4(j.x, j.y, j.z, 0.0f);
}

__global__ void __launch_bounds__(kBlock) k_raygen(Frame F, RenderParams P, int path, int use_pool) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) atomicAdd(&F.stats[0], (unsigned long long)F.n);
    if (i >= F.n) return;
    if (path == 0) F.out[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    F.tp[i] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
    F.accum[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    v3 j;
    float lx = 0.0f, ly = 0.0f;
    if (use_pool) {
        float4 jp = F.jpool[i];
        j = mk(jp.x, jp.y, jp.z);
        // raygen.cu:100-106: one lens sample from pixel (id+17)%n (the loop
        // condition never holds since |(z-.5, y-.5)| < 1)
        float4 lp = F.jpool[(i + 17) % F.n];
        lx = lp.z - 0.5f;
        ly = lp.y - 0.5f;
    } else {
        curandStateMRG32k3a* js = (curandStateMRG32k3a*)F.rngj;
        curandStateMRG32k3a s = js[i];
        j = draw3(&s);
        js[i] = s;
    }
    // position the light/path stream at update path*L (paths that ended
    // early still consume their remaining updates, as the pools do)
    int target = path * P.L;
    int d = F.draws[i];
    if (d < target) {
        curandStateMRG32k3a* rs = (curandStateMRG32k3a*)F.rng;
        curandStateMRG32k3a s = rs[i];
        for (; d < target; ++d) (void)draw3(&s);
        rs[i] = s;
        F.draws[i] = d;
    }
    int x = i % F.w, y = i / F.w;
    v3 o, dir;
    camera_ray(P.cam, x, y, j.x, j.y, lx, ly, &o, &dir);
    F.ray_o[i] = make_float4(o.x, o.y, o.z, FLT_MAX);
    F.ray_d[i] = make_float4(dir.x, dir.y, dir.z, 0.0f);
}

template <bool INSTR>
__global__ void __launch_bounds__(kBlock) k_extend(DevScene S, Frame F, RenderParams P, int path, int bounce) {
    uint32_t* ctr = F.ctr + 4 * bounce;
    const uint32_t count = bounce == 0 ? (uint32_t)F.n : ctr[0];
    const uint32_t* qin = F.q[bounce & 1];
    uint32_t* qsh = F.q[2];
    uint32_t* csh = ctr + 2;
    if (blockIdx.x == 0 && threadIdx.x == 0 && bounce > 0) atomicAdd(&F.stats[1], (unsigned long long)count);
    uint32_t nvis = 0, ntri = 0;
    curandStateMRG32k3a* rs = (curandStateMRG32k3a*)F.rng;
    while (true) {
        uint32_t base = 0;
        if (lane_id() == 0) base = atomicAdd(ctr + 1, 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= count) break;
        uint32_t qi = base + lane_id();
        bool valid = qi < count;
        uint32_t id = 0;
        bool hit = false;
        if (valid) {
            id = bounce == 0 ? qi : qin[qi];
            float4 ro = F.ray_o[id], rd = F.ray_d[id];
            RayInv r = make_ray(ld3(ro), ld3(rd));
            TraceOut h;
            hit = traverse<false, INSTR>(S, r, ro.w, &h, F.status, &nvis, &ntri);
            if (!hit) {
                float4 tp4 = F.tp[id], ac = F.accum[id];
                v3 add = miss_contribution(ld3(tp4), P.sp);
                F.accum[id] = make_float4(ac.x + add.x, ac.y + add.y, ac.z + add.z, 0.0f);
            } else {
                const float4* sh = S.shade + 6 * (size_t)h.id;
                float4 a = __ldg(sh + 0), b = __ldg(sh + 1), c = __ldg(sh + 2);
                float4 na = __ldg(sh + 3), nb = __ldg(sh + 4), nc = __ldg(sh + 5);
                v3 Pp = bary(h.beta, h.gamma, ld3(a), ld3(b), ld3(c));
                v3 Nr = bary(h.beta, h.gamma, ld3(na), ld3(nb), ld3(nc));
                curandStateMRG32k3a s = rs[id];
                v3 rnd = draw3(&s);
                rs[id] = s;
                F.draws[id] += 1;
                v3 lr = rnd;
                if (P.rng_mode == 1) {
                    float hy = halton((int)id + 1, 3);
                    lr = mk(halton((int)id + 1, 2), hy, hy);
                }
                v3 so = mk(0.0f, 0.0f, 0.0f), sd = mk(0.0f, 0.0f, 0.0f), psc = mk(0.0f, 0.0f, 0.0f);
                float smax = -1.0f;
                if (S.n_lights > 0) {
                    int l = pick_light(S.lights, S.n_lights, S.overall_power, lr.z);
                    LightRec L = S.lights[l];
                    rect_light_sample(L, S.overall_power, Pp, Nr, lr.x, lr.y, P.sp.shadow_offset, &so, &sd, &smax,
                                      &psc);
                }
                F.sh_o[id] = make_float4(so.x, so.y, so.z, smax);
                F.sh_d[id] = make_float4(sd.x, sd.y, sd.z, 0.0f);
                F.psc[id] = make_float4(psc.x, psc.y, psc.z, 0.0f);
                F.rnd[id] = make_float4(rnd.x, rnd.y, rnd.z, 0.0f);
                F.hit_p[id] = make_float4(Pp.x, Pp.y, Pp.z, a.w);
                F.hit_n[id] = make_float4(Nr.x, Nr.y, Nr.z, 0.0f);
            }
        }
        push(valid && hit, id, qsh, csh);
    }
    if (INSTR) { add_stats(&F.stats[3], nvis); add_stats(&F.stats[4], ntri); }
}

template <bool INSTR>
__global__ void __launch_bounds__(kBlock) k_shade(DevScene S, Frame F, RenderParams P, int path, int bounce) {
    uint32_t* ctr = F.ctr + 4 * bounce;
    const uint32_t count = ctr[2];
    const uint32_t* qsh = F.q[2];
    uint32_t* qout = F.q[(bounce + 1) & 1];
    uint32_t* cout_ = F.ctr + 4 * (bounce + 1);
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&F.stats[2], (unsigned long long)count);
    uint32_t nvis = 0, ntri = 0;
    const bool last = bounce + 1 >= P.L;
    while (true) {
        uint32_t base = 0;
        if (lane_id() == 0) base = atomicAdd(ctr + 3, 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= count) break;
        uint32_t qi = base + lane_id();
        bool valid = qi < count;
        uint32_t id = 0;
        bool alive = false;
        if (valid) {
            id = qsh[qi];
            float4 so = F.sh_o[id], sd = F.sh_d[id];
            bool occl = true;
            if (so.w >= 0.0f) {
                RayInv r = make_ray(ld3(so), ld3(sd));
                occl = traverse<true, INSTR>(S, r, so.w, nullptr, F.status, &nvis, &ntri);
            }
            float4 hp = F.hit_p[id], hn = F.hit_n[id];
            uint32_t mi = __float_as_uint(hp.w);
            float mf[kMaterialFloats];
            const float4* mp = (const float4*)(S.mats + (size_t)kMaterialFloats * mi);
#pragma unroll
            for (int k = 0; k < 7; ++k) {
                float4 q = __ldg(mp + k);
                mf[4 * k] = q.x; mf[4 * k + 1] = q.y; mf[4 * k + 2] = q.z; mf[4 * k + 3] = q.w;
            }
            MaterialRec m = unpack_material(mf);
            float4 rd = F.ray_d[id], tp4 = F.tp[id], rn = F.rnd[id], ps = F.psc[id], ac = F.accum[id];
            ShadeOut o = shade_hit(m, ld3(hp), ld3(hn), ld3(rd), ld3(tp4), ld3(rn), !occl, ld3(sd), ld3(ps), P.sp,
                                   id, (uint32_t)path, bounce);
            F.accum[id] = make_float4(ac.x + o.accum_add.x, ac.y + o.accum_add.y, ac.z + o.accum_add.z, 0.0f);
            F.tp[id] = make_float4(o.tp.x, o.tp.y, o.tp.z, 0.0f);
            F.ray_o[id] = make_float4(o.org.x, o.org.y, o.org.z, FLT_MAX);
            F.ray_d[id] = make_float4(o.dir.x, o.dir.y, o.dir.z, 0.0f);
            alive = o.alive && !last;
        }
        push(alive, id, qout, cout_);
    }
    if (INSTR) { add_stats(&F.stats[5], nvis); add_stats(&F.stats[6], ntri); }
}

__global__ void k_finalize(Frame F, int path) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= F.n) return;
    float4 o = F.out[i], a = F.accum[i];
    v3 c = combine_sample(mk(o.x, o.y, o.z), mk(a.x, a.y, a.z), path);
    F.out[i] = make_float4(c.x, c.y, c.z, 0.0f);
}

__global__ void k_pack_rgb(const float4* __restrict__ src, int n, float* dst) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 v = src[i];
    dst[3 * i] = v.x; dst[3 * i + 1] = v.y; dst[3 * i + 2] = v.z;
}

__global__ void k_mrg_pool(int npix, uint32_t seed, int first_update, int num_updates, float* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npix) return;
    curandStateMRG32k3a s;
    curand_init((unsigned long long)seed, (unsigned long long)i, 0ull, &s);
    for (int u = 0; u < first_update; ++u) (void)draw3(&s);
    for (int u = 0; u < num_updates; ++u) {
        v3 r = draw3(&s);
        size_t o = ((size_t)u * npix + i) * 3;
        out[o] = r.x; out[o + 1] = r.y; out[o + 2] = r.z;
    }
}

// rta::generate_arealight_sample on a pixel grid (device buffers).
__global__ void k_nee_stage(DevScene S, int n, float shadow_offset, const float* __restrict__ rnd,
                            const float4* __restrict__ hits, float* ray_orig, float* ray_dir, float* max_t,
                            float* psc) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 h = hits[i];
    uint32_t id = __float_as_uint(h.w);
    v3 r = mk(rnd[3 * i], rnd[3 * i + 1], rnd[3 * i + 2]);
    if (id != 0xffffffffu && S.n_lights > 0) {
        int l = pick_light(S.lights, S.n_lights, S.overall_power, r.z);
        const float4* sh = S.shade + 6 * (size_t)id;
        v3 Pp = bary(h.y, h.z, ld3(sh[0]), ld3(sh[1]), ld3(sh[2]));
        v3 Nr = bary(h.y, h.z, ld3(sh[3]), ld3(sh[4]), ld3(sh[5]));
        v3 so, sd, ps; float sm;
        rect_light_sample(S.lights[l], S.overall_power, Pp, Nr, r.x, r.y, shadow_offset, &so, &sd, &sm, &ps);
        ray_orig[3 * i] = so.x; ray_orig[3 * i + 1] = so.y; ray_orig[3 * i + 2] = so.z;
        ray_dir[3 * i] = sd.x; ray_dir[3 * i + 1] = sd.y; ray_dir[3 * i + 2] = sd.z;
        max_t[i] = sm;
        psc[3 * i] = ps.x; psc[3 * i + 1] = ps.y; psc[3 * i + 2] = ps.z;
    } else {
        // arealight-sampler-cpu.cpp:121-142 without a sky light
        ray_orig[3 * i] = FLT_MAX; ray_orig[3 * i + 1] = FLT_MAX; ray_orig[3 * i + 2] = FLT_MAX;
        ray_dir[3 * i] = 0.0f; ray_dir[3 * i + 1] = 0.0f; ray_dir[3 * i + 2] = 0.0f;
        max_t[i] = -1.0f;
        psc[3 * i] = 0.0f; psc[3 * i + 1] = 0.0f; psc[3 * i + 2] = 0.0f;
    }
}

// compute_path_contribution_and_bounce on a pixel grid (device buffers).
__global__ void k_shade_stage(DevScene S, int n, ShadeParams sp, float* ray_orig, float* ray_dir, float* max_t,
                              const float4* __restrict__ hits, const uint8_t* __restrict__ occl,
                              const float* __restrict__ rnd, float* tp, float* accum,
                              const float* __restrict__ to_light, const float* __restrict__ psc, int path,
                              int bounce) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 h = hits[i];
    uint32_t id = __float_as_uint(h.w);
    v3 t = mk(tp[3 * i], tp[3 * i + 1], tp[3 * i + 2]);
    v3 ac = mk(accum[3 * i], accum[3 * i + 1], accum[3 * i + 2]);
    if (id != 0xffffffffu) {
        const float4* sh = S.shade + 6 * (size_t)id;
        float4 a = sh[0];
        v3 Pp = bary(h.y, h.z, ld3(a), ld3(sh[1]), ld3(sh[2]));
        v3 Nr = bary(h.y, h.z, ld3(sh[3]), ld3(sh[4]), ld3(sh[5]));
        MaterialRec m = unpack_material(S.mats + (size_t)kMaterialFloats * __float_as_uint(a.w));
        v3 rd = mk(ray_dir[3 * i], ray_dir[3 * i + 1], ray_dir[3 * i + 2]);
        ShadeOut o = shade_hit(m, Pp, Nr, rd, t, mk(rnd[3 * i], rnd[3 * i + 1], rnd[3 * i + 2]), occl[i] == 0,
                               mk(to_light[3 * i], to_light[3 * i + 1], to_light[3 * i + 2]),
                               mk(psc[3 * i], psc[3 * i + 1], psc[3 * i + 2]), sp, (uint32_t)i, (uint32_t)path,
                               bounce);
        ac = ac + o.accum_add;
        t = o.tp;
        if (o.alive) {
            ray_orig[3 * i] = o.org.x; ray_orig[3 * i + 1] = o.org.y; ray_orig[3 * i + 2] = o.org.z;
            ray_dir[3 * i] = o.dir.x; ray_dir[3 * i + 1] = o.dir.y; ray_dir[3 * i + 2] = o.dir.z;
            max_t[i] = FLT_MAX;
        } else {
            ray_orig[3 * i] = FLT_MAX; ray_orig[3 * i + 1] = FLT_MAX; ray_orig[3 * i + 2] = FLT_MAX;
            ray_dir[3 * i] = 0.0f; ray_dir[3 * i + 1] = 0.0f; ray_dir[3 * i + 2] = 0.0f;
            max_t[i] = -1.0f;
        }
    } else {
        // handle_no_hit (hybrid-pt.cpp:196-206); dead rays (max_t == -1) add 0
        if (max_t[i] != -1.0f) ac = ac + miss_contribution(t, sp);
        ray_orig[3 * i] = FLT_MAX; ray_orig[3 * i + 1] = FLT_MAX; ray_orig[3 * i + 2] = FLT_MAX;
        ray_dir[3 * i] = 0.0f; ray_dir[3 * i + 1] = 0.0f; ray_dir[3 * i + 2] = 0.0f;
        max_t[i] = -1.0f;
        t = mk(0.0f, 0.0f, 0.0f);
    }
    tp[3 * i] = t.x; tp[3 * i + 1] = t.y; tp[3 * i + 2] = t.z;
    accum[3 * i] = ac.x; accum[3 * i + 1] = ac.y; accum[3 * i + 2] = ac.z;
}

inline int blocks_for(int n) { return (n + kBlock - 1) / kBlock; }

template <typename K>
int persistent_blocks(K kernel) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, kBlock, 0);
    if (per < 1) per = 1;
    return sms * per;
}

}  // namespace

int launch_grid_size() { return persistent_blocks(k_extend<false>); }

cudaError_t k_launch_trace(const DevScene& S, int n, const float* orig, const float* dir, const float* tmax,
                           float4* hits, uint8_t* occluded, bool any, uint32_t* status, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_trace<<<blocks_for(n), kBlock, 0, st>>>(S, n, orig, dir, tmax, hits, occluded, any ? 1 : 0, status);
    return cudaGetLastError();
}

cudaError_t k_launch_rng_init(const Frame& F, uint32_t seed, cudaStream_t st) {
    k_rng_init<<<blocks_for(F.n), kBlock, 0, st>>>(F.n, seed, (curandStateMRG32k3a*)F.rng,
                                                   (curandStateMRG32k3a*)F.rngj, F.draws);
    return cudaGetLastError();
}

cudaError_t k_launch_raygen(const Frame& F, const RenderParams& P, int path, cudaStream_t st) {
    bool lens = P.cam.aperture != 0.0f;
    if (lens) k_jitter_pool<<<blocks_for(F.n), kBlock, 0, st>>>(F);
    k_raygen<<<blocks_for(F.n), kBlock, 0, st>>>(F, P, path, lens ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t k_launch_extend(const DevScene& S, const Frame& F, const RenderParams& P, int path, int bounce,
                            bool instrument, cudaStream_t st) {
    static int g0 = persistent_blocks(k_extend<false>);
    static int g1 = persistent_blocks(k_extend<true>);
    if (instrument) k_extend<true><<<g1, kBlock, 0, st>>>(S, F, P, path, bounce);
    else k_extend<false><<<g0, kBlock, 0, st>>>(S, F, P, path, bounce);
    return cudaGetLastError();
}

cudaError_t k_launch_shade(const DevScene& S, const Frame& F, const RenderParams& P, int path, int bounce,
                           bool instrument, cudaStream_t st) {
    static int g0 = persistent_blocks(k_shade<false>);
    static int g1 = persistent_blocks(k_shade<true>);
    if (instrument) k_shade<true><<<g1, kBlock, 0, st>>>(S, F, P, path, bounce);
    else k_shade<false><<<g0, kBlock, 0, st>>>(S, F, P, path, bounce);
    return cudaGetLastError();
}

cudaError_t k_launch_finalize(const Frame& F, int path, cudaStream_t st) {
    k_finalize<<<blocks_for(F.n), kBlock, 0, st>>>(F, path);
    return cudaGetLastError();
}

cudaError_t k_launch_pack_rgb(const float4* src, int n, float* dst, cudaStream_t st) {
    k_pack_rgb<<<blocks_for(n), kBlock, 0, st>>>(src, n, dst);
    return cudaGetLastError();
}

cudaError_t k_launch_mrg_pool(int npix, uint32_t seed, int first_update, int num_updates, float* out,
                              cudaStream_t st) {
    k_mrg_pool<<<blocks_for(npix), kBlock, 0, st>>>(npix, seed, first_update, num_updates, out);
    return cudaGetLastError();
}

cudaError_t k_launch_nee_stage(const DevScene& S, int n, float shadow_offset, const float* rnd, const float4* hits,
                               float* ray_orig, float* ray_dir, float* max_t, float* psc, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_nee_stage<<<blocks_for(n), kBlock, 0, st>>>(S, n, shadow_offset, rnd, hits, ray_orig, ray_dir, max_t, psc);
    return cudaGetLastError();
}

cudaError_t k_launch_shade_stage(const DevScene& S, int n, const ShadeParams& sp, float* ray_orig, float* ray_dir,
                                 float* max_t, const float4* hits, const uint8_t* occl, const float* rnd,
                                 float* tp, float* accum, const float* to_light, const float* psc, int path,
                                 int bounce, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_shade_stage<<<blocks_for(n), kBlock, 0, st>>>(S, n, sp, ray_orig, ray_dir, max_t, hits, occl, rnd, tp, accum,
                                                    to_light, psc, path, bounce);
    return cudaGetLastError();
}

}  // namespace gb
