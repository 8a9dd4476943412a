// gbpt_kernels.cu -- sm_103a kernels of the GB300 path-tracing hot path.
//
// The progressive frame runs as a wavefront over a pool of path slots.  The
// paths of a chunk (samples p0..p1-1 of every pixel) are handed out to the
// slots in path order; a slot whose path ends stores the path's sample and
// takes the next path, so every iteration works on a full queue until the
// chunk runs dry.  One iteration:
//   k_extend  closest-hit traversal of the extension queue; misses add
//             handle_no_hit's contribution (hybrid-pt.cpp:196-206) and end
//             the path; hits draw the bounce's uniforms and emit the
//             area-light shadow ray (arealight-sampler-cpu.cpp:25-143)
//   k_shadow  any-hit traversal of the shadow queue
//   k_shade   BRDF sample/eval, NEE accumulation, throughput and next ray of
//             compute_path_contribution_and_bounce (hybrid-pt.cpp:450-584)
// then k_combine folds the chunk's samples into the image with new_path's
// moving average (util-kernels.cu:17-25), in path order per pixel, so the
// image equals the reference's pixel-sequential one bit for bit.
// Queues are compacted with one warp ballot + one atomic per warp; traversal
// kernels run persistent warps that refill idle lanes from the queue.
//
// Traversal: compressed 8-wide BVH (80 B nodes, 8-bit quantised child
// boxes), node-group stack of 32 entries, octant-ordered child visits,
// conservative slab tests (relative slack 1e-5 on top of outward-rounded
// boxes), so the result equals the (t, id)-minimum over all triangles.
#include "gbpt_kernels.h"

#include <curand_kernel.h>

#include <algorithm>

namespace gb {

namespace {

constexpr int kBlock = 128;
// Resident 128-thread blocks per SM the traversal kernels are compiled for:
// 7 (72 registers, 28 warps per SM) measured fastest on the 1 M-triangle
// frame (8 blocks spill more; the compiler's own choice of 80 registers
// gives 6 blocks).
#ifndef GB_TRAV_MIN_BLOCKS
#define GB_TRAV_MIN_BLOCKS 7
#endif
constexpr int kStack = 32;
constexpr int kIterLimit = 1 << 22;
// Experimental build options, each off by default (measured in the design
// notes): traversal stack entries kept in shared memory, L2 prefetch of hit
// child nodes, light samples in a kernel of their own, register budgets and
// grid of the streaming kernels.
#ifndef GB_SMEM_STACK
#define GB_SMEM_STACK 0
#endif
#ifndef GB_PREFETCH
#define GB_PREFETCH 0
#endif
#ifndef GB_SPLIT_NEE
#define GB_SPLIT_NEE 0
#endif
#ifndef GB_SHADE_MIN_BLOCKS
#define GB_SHADE_MIN_BLOCKS 5  // resident k_shade blocks per SM (register budget 102)
#endif
#ifndef GB_STREAM_MIN_BLOCKS
#define GB_STREAM_MIN_BLOCKS 1
#endif
#ifndef GB_NODE_FOLD
#define GB_NODE_FOLD 0  // 1: plane bias folded into the per-node origin term
#endif
#ifndef GB_FUSED_RESTART
#define GB_FUSED_RESTART 1  // paths ended by a miss restart in k_shadow's warps
#endif
#ifndef GB_WIDE_STREAM_GRIDS
#define GB_WIDE_STREAM_GRIDS 0
#endif
constexpr int kSmemStack = GB_SMEM_STACK;

// A thread's traversal stack: entry e < kSmemStack at top[e * stride]
// (a column of a shared-memory array), deeper entries in deep[e - kSmemStack].
struct StackRef {
    uint2* top;
    uint2* deep;
    int stride;
};
__device__ __forceinline__ void stack_put(const StackRef& k, int e, uint2 v) {
    if (e < kSmemStack) k.top[e * k.stride] = v;
    else k.deep[e - kSmemStack] = v;
}
__device__ __forceinline__ uint2 stack_get(const StackRef& k, int e) {
    return e < kSmemStack ? k.top[e * k.stride] : k.deep[e - kSmemStack];
}

__device__ __forceinline__ v3 ld3(const float4 a) { return mk(a.x, a.y, a.z); }

// Byte j of w as a float, exactly: the byte is placed in the mantissa of
// 2^23 (one PRMT) and 2^23 is subtracted (one FADD).
__device__ __forceinline__ float byte_f(uint32_t w, uint32_t j) {
    return __uint_as_float(__byte_perm(w, 0x4b000000u, 0x7440u | j)) - 8388608.0f;
}

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

// Read-only 16-byte loads of the tree with cache hints: triangles without L1
// allocation (GB_TRI_NOALLOC), nodes with a 128-byte L2 fetch (GB_NODE_L2_128);
// plain __ldg otherwise.
#ifndef GB_SHADOW_MIN_BLOCKS
#define GB_SHADOW_MIN_BLOCKS 8  // resident any-hit blocks per SM (register budget)
#endif
#ifndef GB_SHADOW_REFILL
#define GB_SHADOW_REFILL 12  // refill threshold of the any-hit kernel (0: the frame's refill)
#endif
#ifndef GB_TRI_NOALLOC
#define GB_TRI_NOALLOC 0
#endif
#ifndef GB_NODE_L2_128
#define GB_NODE_L2_128 0
#endif
__device__ __forceinline__ float4 ld_tri(const float4* p) {
#if GB_TRI_NOALLOC
    float4 v;
    asm("ld.global.nc.L1::no_allocate.v4.f32 {%0, %1, %2, %3}, [%4];"
        : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(__cvta_generic_to_global(p)));
    return v;
#else
    return __ldg(p);
#endif
}
// The hit triangle's shading record (positions and normals for the hit
// point), read once per hit with little reuse across a frame: with
// GB_SHADE_EVICT_FIRST the load is marked evict-first (ld.global.cs), so
// that the 98 MB array streaming past does not push the tree out of L2.
#ifndef GB_SHADE_EVICT_FIRST
#define GB_SHADE_EVICT_FIRST 0
#endif
__device__ __forceinline__ float4 ld_shade(const float4* p) {
#if GB_SHADE_EVICT_FIRST
    return __ldcs(p);
#else
    return __ldg(p);
#endif
}
__device__ __forceinline__ float4 ld_node(const float4* p) {
#if GB_NODE_L2_128
    float4 v;
    asm("ld.global.nc.L2::128B.v4.f32 {%0, %1, %2, %3}, [%4];"
        : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(__cvta_generic_to_global(p)));
    return v;
#else
    return __ldg(p);
#endif
}

// Packed FP32 (two lanes per 64-bit register) and 3-input min/max of sm_100+.
__device__ __forceinline__ uint64_t pack2(float a, float b) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void unpack2(uint64_t v, float& a, float& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ uint64_t fma2(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ uint64_t add2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t mul2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ float max3(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float min3(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// Bits of an 8-bit mask moved from position i to i ^ x (x in 0..7).
__device__ __forceinline__ uint32_t xor_permute8(uint32_t m, uint32_t x) {
    if (x & 1u) m = ((m & 0x55u) << 1) | ((m >> 1) & 0x55u);
    if (x & 2u) m = ((m & 0x33u) << 2) | ((m >> 2) & 0x33u);
    if (x & 4u) m = ((m & 0x0fu) << 4) | ((m >> 4) & 0x0fu);
    return m;
}

// Intersects the 8 children of node `ni`; returns the node group (child
// base, hit bits 24-31 in visit order | imask) and the triangle group.
// Per axis the near and far planes are chosen once per node from the sign
// of the inverse direction (fma is monotonic in the plane index, so this
// equals taking min/max of the two plane distances per child); children are
// tested two at a time with packed FP32.  The test is conservative: the
// entry distance is shrunk and the exit distance grown by 1e-5 relative on
// top of the outward-rounded boxes.  Empty slots (meta 0, imask bit 0) may
// test positive; they add neither a node nor a triangle.
// Plane distances (GB_NODE_FOLD): q a + o is evaluated as one packed FMA
// (2^15 + q) a + (o - 2^15 a).  One PRMT places byte q in bits 8-15 of the
// float 2^15, which is then exactly 2^15 + q; the bias -2^15 a is folded
// into the per-node origin term, whose rounding (at most |a| 2^-9 per
// rounding, two roundings) is covered by moving near planes down and far
// planes up by |a| / 64, a 64th of a quantisation step.  Without the fold,
// byte q is made exact as (2^23 + q) - 2^23 (PRMT + packed FADD).
__device__ __forceinline__ void intersect_node(const float4* __restrict__ nodes, uint32_t ni, const RayInv& r,
                                               float bound, uint2* ng, uint2* tg) {
    const float4* n = nodes + 5 * (size_t)ni;
    float4 n0 = ld_node(n + 0), n1 = ld_node(n + 1), n2 = ld_node(n + 2), n3 = ld_node(n + 3), n4 = ld_node(n + 4);
    uint32_t ew = __float_as_uint(n0.w);
    float sx = __uint_as_float((ew & 0xffu) << 23);
    float sy = __uint_as_float(((ew >> 8) & 0xffu) << 23);
    float sz = __uint_as_float(((ew >> 16) & 0xffu) << 23);
    const uint32_t imask = ew >> 24;
    const float aix = sx * r.idir.x, aiy = sy * r.idir.y, aiz = sz * r.idir.z;
    const uint64_t AX = pack2(aix, aix), AY = pack2(aiy, aiy), AZ = pack2(aiz, aiz);
    const float aox = (n0.x - r.o.x) * r.idir.x, aoy = (n0.y - r.o.y) * r.idir.y, aoz = (n0.z - r.o.z) * r.idir.z;
#if GB_NODE_FOLD
    const float bx = fmaf(-32768.0f, aix, aox), by = fmaf(-32768.0f, aiy, aoy), bz = fmaf(-32768.0f, aiz, aoz);
    const float ex = fabsf(aix) * 0.015625f, ey = fabsf(aiy) * 0.015625f, ez = fabsf(aiz) * 0.015625f;
    const uint64_t ONX = pack2(bx - ex, bx - ex), ONY = pack2(by - ey, by - ey), ONZ = pack2(bz - ez, bz - ez);
    const uint64_t OFX = pack2(bx + ex, bx + ex), OFY = pack2(by + ey, by + ey), OFZ = pack2(bz + ez, bz + ez);
#else
    const uint64_t OX = pack2(aox, aox), OY = pack2(aoy, aoy), OZ = pack2(aoz, aoz);
    const uint64_t ONX = OX, ONY = OY, ONZ = OZ, OFX = OX, OFY = OY, OFZ = OZ;
    const uint64_t BIAS = pack2(-8388608.0f, -8388608.0f);
#endif
    const uint64_t KN = pack2(0.99999f, 0.99999f), KF = pack2(1.00001f, 1.00001f);
    const bool fx = r.idir.x < 0.0f, fy = r.idir.y < 0.0f, fz = r.idir.z < 0.0f;
    uint32_t hm = 0;  // child hits by slot
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        uint32_t qlx = __float_as_uint(half ? n2.y : n2.x), qly = __float_as_uint(half ? n2.w : n2.z);
        uint32_t qlz = __float_as_uint(half ? n3.y : n3.x), qhx = __float_as_uint(half ? n3.w : n3.z);
        uint32_t qhy = __float_as_uint(half ? n4.y : n4.x), qhz = __float_as_uint(half ? n4.w : n4.z);
        uint32_t nx = fx ? qhx : qlx, fxw = fx ? qlx : qhx;
        uint32_t ny = fy ? qhy : qly, fyw = fy ? qly : qhy;
        uint32_t nz = fz ? qhz : qlz, fzw = fz ? qlz : qhz;
#pragma unroll
        for (uint32_t j = 0; j < 4; j += 2) {
            // plane index bytes j, j+1 as floats 2^23 + q (PRMT), minus 2^23
            // (exact), then the plane distance q * a + o (packed FMA)
#if GB_NODE_FOLD
#define GB_PLANES(w, A, O) fma2(pack2(__uint_as_float(__byte_perm(w, 0x47000000u, 0x7604u | (j << 4))),          \
                                      __uint_as_float(__byte_perm(w, 0x47000000u, 0x7604u | ((j + 1u) << 4)))), \
                                A, O)
#else
#define GB_PLANES(w, A, O) fma2(add2(pack2(__uint_as_float(__byte_perm(w, 0x4b000000u, 0x7440u | j)),          \
                                            __uint_as_float(__byte_perm(w, 0x4b000000u, 0x7440u | (j + 1u)))), \
                                      BIAS), A, O)
#endif
            float tnx0, tnx1, tny0, tny1, tnz0, tnz1, tfx0, tfx1, tfy0, tfy1, tfz0, tfz1;
            unpack2(GB_PLANES(nx, AX, ONX), tnx0, tnx1);
            unpack2(GB_PLANES(ny, AY, ONY), tny0, tny1);
            unpack2(GB_PLANES(nz, AZ, ONZ), tnz0, tnz1);
            unpack2(GB_PLANES(fxw, AX, OFX), tfx0, tfx1);
            unpack2(GB_PLANES(fyw, AY, OFY), tfy0, tfy1);
            unpack2(GB_PLANES(fzw, AZ, OFZ), tfz0, tfz1);
#undef GB_PLANES
            float lo0, lo1, hi0, hi1;
            unpack2(mul2(pack2(max3(tnx0, tny0, fmaxf(tnz0, 0.0f)), max3(tnx1, tny1, fmaxf(tnz1, 0.0f))), KN), lo0,
                    lo1);
            unpack2(mul2(pack2(min3(tfx0, tfy0, tfz0), min3(tfx1, tfy1, tfz1)), KF), hi0, hi1);
            const int slot = 4 * half + (int)j;
            if (lo0 <= fminf(hi0, bound)) hm |= 1u << slot;
            if (lo1 <= fminf(hi1, bound)) hm |= 2u << slot;
        }
    }
    const uint32_t inner = hm & imask;
    uint32_t leaf = hm & ~imask;
    uint32_t hits_t = 0;
    const uint32_t meta_lo = __float_as_uint(n1.z), meta_hi = __float_as_uint(n1.w);
    while (leaf) {
        uint32_t slot = (uint32_t)__ffs(leaf) - 1u;
        leaf &= leaf - 1u;
        uint32_t meta = __byte_perm(slot < 4u ? meta_lo : meta_hi, 0u, 0x4440u | (slot & 3u));
        hits_t |= (meta >> 5) << (meta & 31u);
    }
#if GB_PREFETCH
    // the hit inner children will be visited: start their fetch into L2 now
    for (uint32_t m = inner; m; m &= m - 1u) {
        const uint32_t s = (uint32_t)__ffs(m) - 1u;
        const float4* cp = nodes + 5 * (size_t)(__float_as_uint(n1.x) + (uint32_t)__popc(imask & ((1u << s) - 1u)));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(__cvta_generic_to_global(cp)));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(__cvta_generic_to_global(cp + 4)));
    }
#endif
    *ng = make_uint2(__float_as_uint(n1.x), (xor_permute8(inner, r.oxor) << 24) | imask);
    *tg = make_uint2(__float_as_uint(n1.y), hits_t);
}

// Resumable traversal state of one ray (the node-group stack lives beside it).
struct Trav {
    uint2 ng, tg;
    int sp;
    float best_t, bb, bg;
    uint32_t best_id;
};

__device__ __forceinline__ void trav_init(Trav& s, const RayInv& r) {
    s.ng = make_uint2(0u, 0x80000000u | (1u << (r.oxor ^ 7u)));
    s.tg = make_uint2(0u, 0u);
    s.sp = 0;
    s.best_t = FLT_MAX;
    s.best_id = 0xffffffffu;
    s.bb = 0.0f;
    s.bg = 0.0f;
}

// Traversal steps.  The stack holds node groups (hit bits 24-31 set) and
// postponed triangle groups (24-bit triangle mask, bits 24-31 clear).
//
// tri_step: one triangle of the current triangle group.  Returns true when
// an any-hit query has found its hit.
template <bool ANY, bool INSTR>
__device__ __forceinline__ bool tri_step(const float4* __restrict__ tris, const RayInv& r, float tmax, Trav& s,
                                         uint32_t* ntri) {
    int b = __ffs(s.tg.y) - 1;
    s.tg.y &= s.tg.y - 1u;
    const float4* tp = tris + 3 * (size_t)(s.tg.x + (uint32_t)b);
    float4 a0 = ld_tri(tp + 0), a1 = ld_tri(tp + 1), a2 = ld_tri(tp + 2);
    if (INSTR) ++*ntri;
    float t, u, v;
    if (intersect_tri(r.o, r.d, ld3(a0), ld3(a1), ld3(a2), &t, &u, &v) && t <= tmax) {
        uint32_t id = __float_as_uint(a0.w);
        if (ANY) { s.best_t = t; s.best_id = id; return true; }
        if (closer(t, id, s.best_t, s.best_id)) { s.best_t = t; s.best_id = id; s.bb = u; s.bg = v; }
    }
    return false;
}

// node_step (current triangle group empty): one node of the current node
// group, or a stack pop.  Returns true when the ray is finished; the result
// is the (t, id)-minimum in s (any-hit: best_id != none when found).
template <bool INSTR, int STACK = kStack>
__device__ __forceinline__ bool node_step(const float4* __restrict__ nodes, const RayInv& r, float tmax, Trav& s,
                                          const StackRef& stack, uint32_t* status, uint32_t* nvis) {
    if (s.ng.y > 0x00ffffffu) {
        uint32_t k = 31u - (uint32_t)__clz(s.ng.y);
        s.ng.y &= ~(1u << k);
        uint32_t slot = (k - 24u) ^ r.oxor;
        uint32_t imask = s.ng.y & 0xffu;
        uint32_t child = s.ng.x + (uint32_t)__popc(imask & ((1u << slot) - 1u));
        if (s.ng.y > 0x00ffffffu) {
            if (s.sp >= STACK) { atomicOr(status, ST_STACK_OVERFLOW); return true; }
            stack_put(stack, s.sp++, s.ng);
        }
        if (INSTR) ++*nvis;
        intersect_node(nodes, child, r, fminf(s.best_t, tmax), &s.ng, &s.tg);
        return false;
    }
    if (s.sp > 0) {
        uint2 g = stack_get(stack, --s.sp);
        if (g.y > 0x00ffffffu) s.ng = g;
        else s.tg = g;
        return false;
    }
    return true;
}

// Whole traversal of one ray without warp cooperation.
template <bool ANY, bool INSTR, int STACK = kStack>
__device__ __forceinline__ bool trav_step(const float4* __restrict__ nodes, const float4* __restrict__ tris,
                                          const RayInv& r, float tmax, Trav& s, const StackRef& stack, uint32_t* status,
                                          uint32_t* nvis, uint32_t* ntri) {
    while (s.tg.y != 0u)
        if (tri_step<ANY, INSTR>(tris, r, tmax, s, ntri)) return true;
    return node_step<INSTR, STACK>(nodes, r, tmax, s, stack, status, nvis);
}

struct TraceOut {
    float t, beta, gamma;
    uint32_t id;
};

// Whole traversal of one ray (API tracing kernel).
template <bool ANY>
__device__ __forceinline__ bool traverse(const DevScene& S, const RayInv& r, float tmax, TraceOut* out,
                                         uint32_t* status) {
    Trav s;
    trav_init(s, r);
    uint2 lstack[kStack];
    const StackRef stack{lstack, lstack + kSmemStack, 1};
    uint32_t nv = 0, nt = 0;
    int iters = 0;
    while (!trav_step<ANY, false>(S.nodes, S.tris, r, tmax, s, stack, status, &nv, &nt)) {
        if (++iters > kIterLimit) { atomicOr(status, ST_ITER_LIMIT); break; }
    }
    if (out) { out->t = s.best_t; out->beta = s.bb; out->gamma = s.bg; out->id = s.best_id; }
    return s.best_id != 0xffffffffu;
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

// Warp-aggregated counter increment: the lane's index among the warp's
// increments, counted from the counter's value (0 where pred is false).
__device__ __forceinline__ uint32_t warp_inc(bool pred, uint32_t* c) {
    uint32_t mask = __ballot_sync(0xffffffffu, pred);
    if (mask == 0u) return 0u;
    uint32_t leader = (uint32_t)__ffs(mask) - 1u;
    uint32_t base = 0u;
    if (lane_id() == leader) base = atomicAdd(c, (uint32_t)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, (int)leader);
    return base + (uint32_t)__popc(mask & ((1u << lane_id()) - 1u));
}

__device__ __forceinline__ void add_stats(unsigned long long* s, uint32_t v) {
    uint32_t w = __reduce_add_sync(0xffffffffu, v);
    if (lane_id() == 0u && w) atomicAdd(s, (unsigned long long)w);
}

// One count from a (possibly divergent) lane.
__device__ __forceinline__ void add_stats_lane(unsigned long long* s) {
    uint32_t m = __activemask();
    if (lane_id() == (uint32_t)__ffs(m) - 1u) atomicAdd(s, (unsigned long long)__popc(m));
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
    if (any) {
        bool f = (tmax >= 0.0f) && traverse<true>(S, r, tmax, nullptr, status);
        occluded[i] = f ? 1 : 0;
    } else {
        TraceOut h;
        if (tmax >= 0.0f) traverse<false>(S, r, tmax, &h, status);
        else { h.t = FLT_MAX; h.beta = 0.0f; h.gamma = 0.0f; h.id = 0xffffffffu; }
        hits[i] = make_float4(h.t, h.beta, h.gamma, __uint_as_float(h.id));
    }
}

__device__ __forceinline__ v3 draw3(curandStateMRG32k3a* s) {
    float x = curand_uniform(s);
    float y = curand_uniform(s);
    float z = curand_uniform(s);
    return mk(x, y, z);
}

// MrgState <-> curandStateMRG32k3a (the Box-Muller caches are unused by
// uniform draws and start cleared, as after curand_init).
__device__ __forceinline__ curandStateMRG32k3a mrg_expand(const MrgState& m) {
    curandStateMRG32k3a st;
    for (int k = 0; k < 3; ++k) { st.s1[k] = m.s1[k]; st.s2[k] = m.s2[k]; }
    st.boxmuller_flag = 0;
    st.boxmuller_flag_double = 0;
    st.boxmuller_extra = 0.0f;
    st.boxmuller_extra_double = 0.0;
    return st;
}
__device__ __forceinline__ MrgState mrg_pack(const curandStateMRG32k3a& st) {
    MrgState m;
    for (int k = 0; k < 3; ++k) { m.s1[k] = st.s1[k]; m.s2[k] = st.s2[k]; }
    return m;
}
// 24-byte states as three 8-byte accesses.
__device__ __forceinline__ MrgState ld_mrg(const MrgState* base, size_t i) {
    const uint2* q = reinterpret_cast<const uint2*>(base + i);
    uint2 a = rec_ld(q), b = rec_ld(q + 1), c = rec_ld(q + 2);
    MrgState m;
    m.s1[0] = a.x; m.s1[1] = a.y; m.s1[2] = b.x; m.s2[0] = b.y; m.s2[1] = c.x; m.s2[2] = c.y;
    return m;
}
__device__ __forceinline__ void st_mrg(MrgState* base, size_t i, const MrgState& m) {
    uint2* q = reinterpret_cast<uint2*>(base + i);
    rec_st(q, make_uint2(m.s1[0], m.s1[1]));
    rec_st(q + 1, make_uint2(m.s1[2], m.s2[0]));
    rec_st(q + 2, make_uint2(m.s2[1], m.s2[2]));
}
// the same for the stream of a slot record, stored as its whole 32-byte
// sector (the state and 8 zero bytes)
__device__ __forceinline__ MrgState ld_mrg(const SlotField<MrgState>& f, size_t slot) { return ld_mrg(&f[slot], 0); }
__device__ __forceinline__ void st_mrg(const SlotField<MrgState>& f, size_t slot, const MrgState& m,
                                       bool hit_line = false) {
    uint4* q = reinterpret_cast<uint4*>(&f[slot]);
    const uint4 a = make_uint4(m.s1[0], m.s1[1], m.s1[2], m.s2[0]), b = make_uint4(m.s2[1], m.s2[2], 0u, 0u);
    if (GB_HIT_LINE_KEEP && hit_line) {
        q[0] = a;
        q[1] = b;
    } else {
        rec_st(q, a);
        rec_st(q + 1, b);
    }
}
__device__ __forceinline__ v3 draw3(MrgState* m) {
    curandStateMRG32k3a st = mrg_expand(*m);
    v3 r = draw3(&st);
    *m = mrg_pack(st);
    return r;
}

// The state curand_init(seed, sub, 0) leaves: curand_init of subsequence 0
// (no skip-ahead) advanced by sub * 2^76 steps with the table's jumps, one
// 3x3 matrix product per component for each set bit of sub, in exact
// integer arithmetic mod m1 / m2.
__device__ __forceinline__ MrgState mrg_stream(const MrgSubseqTable& T, uint32_t seed, uint32_t sub) {
    curandStateMRG32k3a s;
    curand_init((unsigned long long)seed, 0ull, 0ull, &s);
    MrgState m = mrg_pack(s);
    for (int k = 0; sub != 0u; ++k, sub >>= 1)
        if (sub & 1u) {
            mrg_apply(m.s1, T.j1[k], 209u, kMrgM1);
            mrg_apply(m.s2, T.j2[k], 22853u, kMrgM2);
        }
    return m;
}

// curand states right after curand_init(seed, pixel, 0) (util-kernels.cu:277-285)
// for every pixel of every scene of the frame (pixel = index within its scene).
__global__ void k_rng_init_frame(Frame F, const MrgSubseqTable T) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= F.ntot) return;
    const SceneRec& R = F.scenes[F.pscene[g]];
    st_mrg(F.pristine, (size_t)g, mrg_stream(T, R.seed, (uint32_t)(g - (int)R.pixel_base)));
}

// States of curand_init(seed, sub[i], 0): method 0 by curand_init itself,
// 1 by mrg_stream.
__global__ void k_mrg_states(const MrgSubseqTable T, uint32_t seed, const uint32_t* sub, int n, int method,
                             uint32_t* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    MrgState m;
    if (method == 0) {
        curandStateMRG32k3a s;
        curand_init((unsigned long long)seed, (unsigned long long)sub[i], 0ull, &s);
        m = mrg_pack(s);
    } else {
        m = mrg_stream(T, seed, sub[i]);
    }
    for (int k = 0; k < 3; ++k) { out[6 * i + k] = m.s1[k]; out[6 * i + 3 + k] = m.s2[k]; }
}

// Scene of every global pixel.
__global__ void k_fill_pscene(Frame F) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= F.ntot) return;
    int lo = 0, hi = F.nscenes - 1;
    while (lo < hi) {  // last scene whose pixel_base <= g
        int mid = (lo + hi + 1) >> 1;
        if ((int)F.scenes[mid].pixel_base <= g) lo = mid;
        else hi = mid - 1;
    }
    F.pscene[g] = (uint32_t)lo;
}

// ------------------------------------------------------------ path slots --
// A slot carries one path (scene, pixel, sample p) at a time.  The frame's
// pixels are laid out scene after scene with scenes sorted by spp (largest
// first), so the pixels that still take a sample in round p form the prefix
// [0, N_p) and a chunk's paths enumerate without holes: path l of the chunk
// is (p0 + r, l - round_start[r]) for the round r holding l.  The
// reference's three identically seeded per-pixel pools
// (hybrid-pt.cpp:83-95, util-kernels.cu:284) become:
//   camera jitter  = update p of the pixel's stream, read from the chunk's
//                    jitter pool (k_jitter_pool walks each pixel's stream)
//   lens sample    = update p of pixel (pixel+17)%n (raygen.cu:100-106)
//   light/path     = updates pL, pL+1, ... one per bounce (hybrid-pt.h:229-233):
//                    k_jitter_pool walks the pixel's stream cursor over the
//                    chunk's paths (a jump of L updates, 3L generator steps,
//                    mrg_jump, per path) and leaves each path's start state
//                    in the chunk's stream pool.
// A path's stream therefore depends only on (pixel, p): a launch may start
// several paths of one pixel, in any order, on any slots.
// Per pixel at the start of a chunk, for every path p of the pixel in the
// chunk (path l = round_start[p - p0] + pixel): its camera jitter (update p
// of the pixel's jitter stream) and the state of its light/path stream
// (L updates per path: one jump of 3 L generator steps from the previous
// path's).  Paths then start from their own pool entries, in any order and
// several per pixel at once.
__global__ void k_jitter_pool(Frame F, RenderParams P) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= F.ntot) return;
    const SceneRec& R = F.scenes[F.nscenes == 1 ? 0u : F.pscene[g]];
    MrgState s = ld_mrg(F.jcursor, (size_t)g);
    MrgState c = ld_mrg(F.cursor, (size_t)g);
    const int pe = min(P.p0 + P.rounds, R.spp);
    for (int p = P.p0; p < pe; ++p) {
        const uint32_t l = P.round_start[p - P.p0] + (uint32_t)g;
        v3 j = draw3(&s);
        rec_st(&F.jpool[l], make_float4(j.x, j.y, j.z, 0.0f));
        st_mrg(F.spool, l, c);
        mrg_jump(c.s1, c.s2, R.jump1, R.jump2);  // = L draw3 calls
    }
    st_mrg(F.jcursor, (size_t)g, s);
    st_mrg(F.cursor, (size_t)g, c);
}

// Ray differentials of a slot, 12 floats in 3 planes of nslots float4.
__device__ __forceinline__ RayDiff ld_rdiff(const Frame& F, uint32_t slot) {
    const float4 a = F.rdiff[0][slot], b = F.rdiff[1][slot], c = F.rdiff[2][slot];
    RayDiff r;
    r.uo = mk(a.x, a.y, a.z);
    r.ud = mk(a.w, b.x, b.y);
    r.ro = mk(b.z, b.w, c.x);
    r.rd = mk(c.y, c.z, c.w);
    return r;
}
__device__ __forceinline__ void st_rdiff(const Frame& F, uint32_t slot, const RayDiff& r) {
    F.rdiff[0][slot] = make_float4(r.uo.x, r.uo.y, r.uo.z, r.ud.x);
    F.rdiff[1][slot] = make_float4(r.ud.y, r.ud.z, r.ro.x, r.ro.y);
    F.rdiff[2][slot] = make_float4(r.ro.z, r.rd.x, r.rd.y, r.rd.z);
}

__device__ __forceinline__ void start_path(const Frame& F, const RenderParams& P, uint32_t slot, uint32_t l) {
    int lo = 0, hi = P.rounds - 1;
    while (lo < hi) {  // round holding path l
        int mid = (lo + hi + 1) >> 1;
        if (P.round_start[mid] <= l) lo = mid;
        else hi = mid - 1;
    }
    const uint32_t gpix = l - P.round_start[lo];
    const uint32_t sc = F.nscenes == 1 ? 0u : F.pscene[gpix];
    const SceneRec& R = F.scenes[sc];
    const uint32_t lp = gpix - R.pixel_base;
    const float4* jp = F.jpool + P.round_start[lo];
    float4 j = rec_ld(&jp[gpix]);
    float lx = 0.0f, ly = 0.0f;
    if (R.cam.aperture != 0.0f) {
        float4 lj = rec_ld(&jp[R.pixel_base + (lp + 17u) % (uint32_t)R.n]);
        lx = lj.z - 0.5f;
        ly = lj.y - 0.5f;
    }
    st_mrg(F.rng, slot, ld_mrg(F.spool, l));
    v3 o, d;
    camera_ray(R.cam, (int)(lp % (uint32_t)R.w), (int)(lp / (uint32_t)R.w), j.x, j.y, lx, ly, &o, &d);
    F.ray_o.st(slot, make_float4(o.x, o.y, o.z, FLT_MAX));
    F.ray_d.st(slot, make_float4(d.x, d.y, d.z, __uint_as_float(((uint32_t)P.p0 + (uint32_t)lo) << 10)));  // w: pb
    F.tp.st(slot, make_float4(1.0f, 1.0f, 1.0f, 0.0f));
    if (P.mode == MODE_FROZEN) F.tp0[slot] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
    F.accum.st(slot, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    F.pixw.st(slot, make_uint4(gpix, sc, 0u, 0u));
    if (R.S.texcoord) st_rdiff(F, slot, camera_diff(R.cam, (int)(lp % (uint32_t)R.w), (int)(lp / (uint32_t)R.w)));
    else F.rdiff[0][slot] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);  // completes the sector of pix / ps
}

// The scene record of a slot's path; a frame of one scene needs no load of
// the slot's scene word.
__device__ __forceinline__ const SceneRec& scene_of(const Frame& F, uint32_t slot) {
    return F.scenes[F.nscenes == 1 ? 0u : F.ps.ld(slot)];
}

// Counter set of iteration `it`: [0] queue count, [1] extension head,
// [2] shadow count, [3] shadow head, [4] ended paths (free queue count).
// The iteration index lives in F.iter (device), so an iteration's launches
// are the same every time (graph-capturable).
__device__ __forceinline__ uint32_t* ctr_set(const Frame& F, int it) { return F.ctr + 8 * (it % 3); }

// The sample of a path that ended (new_path's input to the moving average):
// path p's colour at sample index round_start[p - p0] + pixel.
__device__ __forceinline__ void store_sample(const Frame& F, const RenderParams& P, uint32_t slot, uint32_t pbv,
                                             float4 acc) {
    rec_st(&F.samples[P.round_start[(pbv >> 10) - (uint32_t)P.p0] + F.pix.ld(slot)], acc);
}

// Slots whose path ended go to the free queue; k_regen starts the next
// paths on them.
__device__ __forceinline__ void end_paths(const Frame& F, bool ended, uint32_t slot, uint32_t* cn) {
    push(ended, slot, F.q[3], cn + 4);
}

// Stores the sample of every ended path (new_path's input to the moving
// average) and starts the next paths of the chunk on the freed slots,
// appending them to the next extension queue.
__global__ void __launch_bounds__(kBlock, GB_STREAM_MIN_BLOCKS) k_regen(Frame F, RenderParams P) {
    const int it = *F.iter;
    const uint32_t* cn = ctr_set(F, it + 1);
    // free-queue entries before cn[5] were restarted by k_shadow (cn[7]
    // paths started); the rest are the paths k_shade ended (all of them
    // when k_shadow restarted none)
    const uint32_t first = cn[5];
    const uint32_t count = cn[4] - first;
    const uint32_t next0 = cn[0];   // paths already queued for the next iteration
    const uint32_t l0 = *F.path_ctr + cn[7];
    const uint32_t avail = l0 < P.chunk_paths ? P.chunk_paths - l0 : 0u;
    uint32_t* qout = F.q[(it + 1) & 1];
    const uint32_t stride = gridDim.x * blockDim.x;
    // free-queue entry first + qi takes path l0 + qi and next-queue entry
    // next0 + qi: no counter round trip; k_step advances both counters
    // afterwards.  The ended paths' samples were stored where they ended
    // (store_sample).
    const uint32_t nstart = min(count, avail);
    for (uint32_t qi = blockIdx.x * blockDim.x + threadIdx.x; qi < nstart; qi += stride) {
        const uint32_t slot = F.q[3][first + qi];
        start_path(F, P, slot, l0 + qi);
        qout[next0 + qi] = slot;
    }
}

// Restart of the paths k_extend ended (misses), run by the warps of
// k_shadow once the shadow queue has no rays left for them, so that it
// fills the tail of the any-hit launch.  Free-queue entry qi < nA takes
// path l0 + qi and next-queue entry qi; k_shade appends the continuing
// paths after them, k_regen restarts the paths k_shade ends.  Not in the
// adjoint mode, whose sweep reads the ended paths' records first.
__device__ __forceinline__ void restart_misses(const Frame& F, const RenderParams& P) {
    const int it = *F.iter;
    uint32_t* cn = ctr_set(F, it + 1);
    const uint32_t count = cn[4];  // misses of k_extend (k_shade has not run)
    const uint32_t l0 = *F.path_ctr;
    const uint32_t avail = l0 < P.chunk_paths ? P.chunk_paths - l0 : 0u;
    const uint32_t nA = min(count, avail);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        cn[0] = nA;     // next-queue entries taken (k_shade appends after them)
        cn[5] = count;  // free-queue entries consumed
        cn[7] = nA;     // paths started
    }
    uint32_t* qout = F.q[(it + 1) & 1];
    const uint32_t lane = lane_id();
    while (true) {
        uint32_t base = 0;
        if (lane == 0u) base = atomicAdd(&cn[6], 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= nA) break;
        const uint32_t qi = base + lane;
        if (qi < nA) {
            const uint32_t slot = F.q[3][qi];
            start_path(F, P, slot, l0 + qi);
            qout[qi] = slot;
        }
    }
}

// First paths of a chunk: slot s takes path s.  Resets the iteration index.
__global__ void __launch_bounds__(kBlock) k_start(Frame F, RenderParams P, int nstart) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s == 0) { *F.path_ctr = (uint32_t)nstart; *F.iter = 0; }
    bool go = s < (uint32_t)nstart;
    if (go) start_path(F, P, s, s);
    add_stats(&F.stats[0], go ? 1u : 0u);
    push(go, s, F.q[0], F.ctr + 0);  // queue of iteration 0
}

// End of an iteration: accounts the paths k_regen started (path counter,
// next queue count, camera rays), clears the counter set two iterations
// ahead, moves the iteration index, counts the iteration (stats[7]) and
// tells the graph's loop (when there is one) whether the next extension
// queue has work.
__global__ void k_step(Frame F, RenderParams P, unsigned long long cond, int has_cond, int max_iters) {
    const int it = *F.iter;
    uint32_t* cn = ctr_set(F, it + 1);
    const uint32_t l0 = *F.path_ctr;
    const uint32_t avail = l0 < P.chunk_paths ? P.chunk_paths - l0 : 0u;
    // restarts in k_shadow and k_shade (cn[7] attempts, already queued), or
    // in k_regen (the free queue, queued at cn[0] + qi)
    const bool fused = GB_FUSED_RESTART && P.mode != MODE_ADJOINT;
    const uint32_t started = fused ? min(cn[7], avail) : min(cn[4], avail);
    *F.path_ctr = l0 + started;
    if (!fused) cn[0] += started;
    F.stats[0] += (unsigned long long)started;
    uint32_t* c2 = ctr_set(F, it + 2);
    for (int k = 0; k < 8; ++k) c2[k] = 0u;
    const uint32_t next = cn[0];
    *F.iter = it + 1;
    F.stats[7] += 1ull;
    if (next != 0u && it + 1 >= max_iters) atomicOr(F.status, (uint32_t)ST_ITER_LIMIT);
    if (has_cond) cudaGraphSetConditional((cudaGraphConditionalHandle)cond, (next != 0u && it + 1 < max_iters) ? 1u : 0u);
}

// (t, canonical id) as one 64-bit key whose unsigned order is the
// lexicographic closest-hit order: t > 0, so its bits order like its value.
__device__ __forceinline__ unsigned long long hit_key(float t, uint32_t id) {
    return ((unsigned long long)__float_as_uint(t) << 32) | id;
}

// Warp-cooperative triangle phase (triangle policy 3): the pending triangles
// of all active lanes are tested by the whole warp, 32 at a time.  A warp
// scan of the per-lane counts numbers the (lane, triangle) pairs; tester
// lane g finds its owner (the last lane whose exclusive count is <= g), the
// owner's k-th pending triangle, and the owner's ray through shuffles.  Hits
// resolve per owner by an atomicMin of hit_key in shared memory, so the
// result is the same lexicographic minimum as testing sequentially.  A new
// closest hit's barycentrics are recomputed by its owner from the shading
// record with the same (v0, v1 - v0, v2 - v0) arithmetic as the triangle
// layout, so they are bit-identical too.  All 32 lanes must call this.
template <bool ANY, bool INSTR>
__device__ __forceinline__ bool coop_triangles(bool act, const float4* tris, const float4* shade, const RayInv& r,
                                               float tmax, Trav& s, unsigned long long* skey, uint32_t* ntri) {
    const uint32_t lane = lane_id();
    const uint32_t cnt = act ? (uint32_t)__popc(s.tg.y) : 0u;
    uint32_t incl = cnt;
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    if (total == 0u) return false;
    const uint32_t excl = incl - cnt;
    const unsigned long long mine = act ? hit_key(s.best_t, s.best_id) : ~0ull;
    skey[lane] = mine;
    __syncwarp();
    for (uint32_t base = 0; base < total; base += 32u) {
        const uint32_t g = base + lane;
        uint32_t o = 0;
#pragma unroll
        for (uint32_t step = 16; step >= 1; step >>= 1) {
            uint32_t c = o + step;
            if (__shfl_sync(0xffffffffu, excl, (int)c) <= g) o = c;
        }
        const uint32_t om = __shfl_sync(0xffffffffu, s.tg.y, (int)o);
        const uint32_t ob = __shfl_sync(0xffffffffu, s.tg.x, (int)o);
        const uint32_t oe = __shfl_sync(0xffffffffu, excl, (int)o);
        const v3 ro = mk(__shfl_sync(0xffffffffu, r.o.x, (int)o), __shfl_sync(0xffffffffu, r.o.y, (int)o),
                         __shfl_sync(0xffffffffu, r.o.z, (int)o));
        const v3 rd = mk(__shfl_sync(0xffffffffu, r.d.x, (int)o), __shfl_sync(0xffffffffu, r.d.y, (int)o),
                         __shfl_sync(0xffffffffu, r.d.z, (int)o));
        const float otmax = __shfl_sync(0xffffffffu, tmax, (int)o);
        const float4* otris = (const float4*)__shfl_sync(0xffffffffu, (unsigned long long)tris, (int)o);
        if (g < total) {
            const uint32_t bit = __fns(om, 0u, (int)(g - oe) + 1);
            if (bit < 32u && ((om >> bit) & 1u)) {
                const float4* tp = otris + 3 * (size_t)(ob + bit);
                float4 a0 = ld_tri(tp + 0), a1 = ld_tri(tp + 1), a2 = ld_tri(tp + 2);
                if (INSTR) ++*ntri;
                float t, u, v;
                if (intersect_tri(ro, rd, ld3(a0), ld3(a1), ld3(a2), &t, &u, &v) && t <= otmax)
                    atomicMin(skey + o, hit_key(t, __float_as_uint(a0.w)));
            }
        }
    }
    __syncwarp();
    bool found = false;
    if (act) {
        const unsigned long long k = skey[lane];
        s.tg.y = 0u;
        if (k != mine) {
            const float t = __uint_as_float((uint32_t)(k >> 32));
            const uint32_t id = (uint32_t)k;
            s.best_t = t;
            s.best_id = id;
            found = true;
            if (!ANY) {
                const float4* sh = shade + 6 * (size_t)id;
                const v3 a = ld3(__ldg(sh + 0)), b = ld3(__ldg(sh + 1)), c = ld3(__ldg(sh + 2));
                float tt, u, v;
                if (intersect_tri(r.o, r.d, a, b - a, c - a, &tt, &u, &v)) { s.bb = u; s.bg = v; }
            }
        }
    }
    __syncwarp();
    return found;
}

// Persistent-warp ray loop shared by the traversal kernels: lanes whose ray
// has finished run `finish` together, idle lanes are refilled from the queue
// as soon as `refill` lanes are idle (all lanes once the queue is
// exhausted), and traversal resumes where each lane stopped.  The first
// wave is assigned by warp index (warp w takes entries [32w, 32w+32)); later
// fetches take one atomic per warp on `head`.  Each lane carries the
// geometry of its own scene.  fetch(q, &handle, ...) loads queue entry q's
// ray and sets the handle that finish(fin, handle, trav, t_max) gets back
// when the ray is done.
template <bool ANY, bool INSTR, int MODE, int STACK, int BT, typename Fetch, typename Finish>
__device__ __forceinline__ void ray_loop(uint32_t count, uint32_t* head, int refill, uint32_t* status, Fetch fetch,
                                         Finish finish, uint32_t* nvis, uint32_t* ntri) {
    const uint32_t lane = lane_id();
    const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
    const uint32_t dyn0 = nwarps * 32u;
    const uint32_t gwarp = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    bool act = false, fin = false, exhausted = false, first = true;
    uint32_t qi = 0;  // the lane's handle for finish, as fetch sets it
    int iters = 0;
    RayInv r;
    float tmax = 0.0f;
    Trav s;
    __shared__ uint2 s_stack[kSmemStack > 0 ? kSmemStack * BT : 1];
    uint2 deep[STACK - kSmemStack];
    const StackRef stack{s_stack + threadIdx.x, deep, BT};
    const float4* nodes = nullptr;
    const float4* tris = nullptr;
    const float4* shade = nullptr;
    __shared__ unsigned long long s_key[MODE == 3 ? BT : 1];
    unsigned long long* skey = s_key + (MODE == 3 ? (threadIdx.x & ~31u) : 0u);
    while (true) {
        finish(fin, qi, s, tmax);
        fin = false;
        uint32_t idle = __ballot_sync(0xffffffffu, !act);
        if (!exhausted && idle) {
            uint32_t n = (uint32_t)__popc(idle);
            uint32_t base;
            if (first) {
                base = gwarp * 32u;
                first = false;
                if (dyn0 >= count) exhausted = true;
            } else {
                uint32_t leader = (uint32_t)__ffs(idle) - 1u;
                base = 0;
                if (lane == leader) base = atomicAdd(head, n);
                base = dyn0 + __shfl_sync(0xffffffffu, base, (int)leader);
                if (base + n >= count) exhausted = true;
            }
            if (!act) {
                uint32_t q = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
                if (q < count) {
                    v3 o, d;
                    if (fetch(q, &qi, &o, &d, &tmax, &nodes, &tris, &shade)) {
                        r = make_ray(o, d);
                        trav_init(s, r);
                        iters = 0;
                        act = true;
                    } else {
                        trav_init(s, make_ray(o, d));
                        fin = true;  // nothing to trace (e.g. no light): finish directly
                    }
                }
            }
        }
        if (!__any_sync(0xffffffffu, act || fin)) break;
        while (true) {
            if (MODE == 3) {
                // the warp tests every lane's pending triangles together, then
                // each lane visits one node
                bool hit = coop_triangles<ANY, INSTR>(act, tris, shade, r, tmax, s, skey, ntri);
                if (ANY && act && hit) { act = false; fin = true; }
                if (act) {
                    bool done = node_step<INSTR, STACK>(nodes, r, tmax, s, stack, status, nvis);
                    if (!done && ++iters > kIterLimit) { atomicOr(status, ST_ITER_LIMIT); done = true; }
                    if (done) { act = false; fin = true; }
                }
            } else if (MODE == 0) {
                // every pending triangle, then one node
                if (act) {
                    bool done = trav_step<ANY, INSTR, STACK>(nodes, tris, r, tmax, s, stack, status, nvis, ntri);
                    if (!done && ++iters > kIterLimit) { atomicOr(status, ST_ITER_LIMIT); done = true; }
                    if (done) { act = false; fin = true; }
                }
            } else {
                // triangle postponing: when fewer than a fifth of the active
                // lanes have triangles pending, those lanes stack their
                // triangle group and keep traversing nodes with the rest of
                // the warp; otherwise they test one (MODE 1) or all (MODE 2)
                // of their pending triangles
                const bool want_tri = act && s.tg.y != 0u;
                const uint32_t mt = __ballot_sync(0xffffffffu, want_tri);
                const uint32_t ma = __ballot_sync(0xffffffffu, act);
                bool do_tri = want_tri;
                if (want_tri && 5u * (uint32_t)__popc(mt) < (uint32_t)__popc(ma) && s.sp < STACK) {
                    stack_put(stack, s.sp++, s.tg);
                    s.tg.y = 0u;
                    do_tri = false;
                }
                if (act) {
                    bool done = false;
                    if (do_tri) {
                        if (MODE == 1) done = tri_step<ANY, INSTR>(tris, r, tmax, s, ntri);
                        else
                            while (s.tg.y != 0u && !done) done = tri_step<ANY, INSTR>(tris, r, tmax, s, ntri);
                    } else {
                        done = node_step<INSTR, STACK>(nodes, r, tmax, s, stack, status, nvis);
                    }
                    if (!done && ++iters > kIterLimit) { atomicOr(status, ST_ITER_LIMIT); done = true; }
                    if (done) { act = false; fin = true; }
                }
            }
            uint32_t nidle = (uint32_t)__popc(__ballot_sync(0xffffffffu, !act));
            if (nidle == 32u || (!exhausted && nidle >= (uint32_t)refill)) break;
        }
    }
}

// Closest hit of the extension queue.  Misses add handle_no_hit's
// contribution and end their path; hits draw the bounce's uniforms and emit
// the area-light shadow ray (arealight-sampler-cpu.cpp:25-143).
// The light sample of a hit (generate_arealight_sample,
// arealight-sampler-cpu.cpp:25-143) on the path's light draw: shadow ray,
// potential_sample_contribution and the path draw of this bounce.
// skip_dark: a sample whose potential contribution is exactly zero (the
// surface or the light faces away) gets no shadow ray (max_t = -1, read as
// occluded).  Its visibility cannot change the path: shading adds
// bl * (tp * psc) = +-0 when unoccluded (or nothing, when that is NaN), and
// the accumulation is never -0, so the sum is the same bits either way.
__device__ __forceinline__ void nee_at_hit(const Frame& F, const SceneRec& R, uint32_t slot, v3 Pp, v3 Nr,
                                           bool skip_dark) {
    const DevScene& S = R.S;
    MrgState st = ld_mrg(F.rng, slot);
    v3 rnd = draw3(&st);
    st_mrg(F.rng, slot, st, true);
    v3 lr = rnd;
    if (R.rng_mode == 1) {
        int pid = (int)(F.pix.ld(slot) - R.pixel_base) + 1;
        float hy = halton(pid, 3);
        lr = mk(halton(pid, 2), hy, hy);
    }
    v3 so = mk(0.0f, 0.0f, 0.0f), sd = mk(0.0f, 0.0f, 0.0f), psc = mk(0.0f, 0.0f, 0.0f);
    float smax = -1.0f, scale = 0.0f;
    if (S.n_lights > 0) {
        int l = pick_light(S.lights, S.n_lights, S.overall_power, lr.z);
        LightRec L = S.lights[l];
        if (L.type == 1)
            sky_light_sample(S.sky, L.power, S.overall_power, Pp, Nr, lr.x, lr.y, R.sp.shadow_offset, &so, &sd,
                             &smax, &psc);
        else
            rect_light_sample(L, S.lights_eval[l].col, S.overall_power, Pp, Nr, lr.x, lr.y, R.sp.shadow_offset,
                              &so, &sd, &smax, &psc, &scale);
    }
    if (skip_dark && psc.x == 0.0f && psc.y == 0.0f && psc.z == 0.0f) smax = -1.0f;
    F.sh_o.st_hit(slot, make_float4(so.x, so.y, so.z, smax));
    F.sh_d.st_hit(slot, make_float4(sd.x, sd.y, sd.z, 0.0f));
    F.psc.st_hit(slot, make_float4(psc.x, psc.y, psc.z, scale));
    F.rnd.st_hit(slot, make_float4(rnd.x, rnd.y, rnd.z, 0.0f));
}

// STACK: traversal stack entries; BT: threads per block (the register
// budget stays that of GB_TRAV_MIN_BLOCKS blocks of 128 threads).
template <bool INSTR, int MODE, int STACK, int BT>
__global__ void __launch_bounds__(BT, GB_TRAV_MIN_BLOCKS * 128 / BT) k_extend(Frame F, RenderParams P) {
    const int it = *F.iter;
    uint32_t* cs = ctr_set(F, it);
    uint32_t* cn = ctr_set(F, it + 1);
    const uint32_t count = cs[0];
    const uint32_t* qin = F.q[it & 1];
    uint32_t* qsh = F.q[2];
    uint32_t nvis = 0, ntri = 0, nhit = 0;
    // the handle finish gets back is the queue entry: re-reading the slot
    // there costs less than keeping it live through the traversal
    auto fetch = [&](uint32_t q, uint32_t* handle, v3* o, v3* d, float* tmax, const float4** nodes,
                     const float4** tris, const float4** shade) {
        const uint32_t slot = qin[q];
        *handle = q;
        float4 ro = F.ray_o.ld(slot), rd = F.ray_d.ld(slot);
        const SceneRec& R = scene_of(F, slot);
        *nodes = R.S.nodes;
        *tris = R.S.tris;
        *shade = R.S.shade;
        *o = ld3(ro); *d = ld3(rd); *tmax = ro.w;
        return true;
    };
    auto finish = [&](bool fin, uint32_t q, const Trav& h, float) {
        bool hit = false, ended = false;
        uint32_t slot = 0;
        if (fin) {
            slot = qin[q];
            hit = h.best_id != 0xffffffffu;
            const SceneRec& R = scene_of(F, slot);
            uint32_t pbv = F.pb.ld(slot);
            if ((pbv & 1023u) > 0u) add_stats_lane(&F.stats[1]);
            if (!hit) {
                float4 tp4 = F.tp.ld(slot);
                float4 acc = F.accum.ld(slot);
                v3 add = miss_contribution(ld3(tp4), ld3(F.ray_d.ld(slot)), R.sp, &R.S.sky);
                store_sample(F, P, slot, pbv, make_float4(acc.x + add.x, acc.y + add.y, acc.z + add.z, 0.0f));
                ended = true;
            } else {
                const DevScene& S = R.S;
                if (INSTR) ++nhit;
                const float4* sh = S.shade + 6 * (size_t)h.best_id;
                float4 a = ld_shade(sh + 0), b = ld_shade(sh + 1), c = ld_shade(sh + 2);
                float4 na = ld_shade(sh + 3), nb = ld_shade(sh + 4), nc = ld_shade(sh + 5);
                v3 Pp = bary(h.bb, h.bg, ld3(a), ld3(b), ld3(c));
                v3 Nr = bary(h.bb, h.bg, ld3(na), ld3(nb), ld3(nc));
                if (!GB_SPLIT_NEE) nee_at_hit(F, R, slot, Pp, Nr, P.mode != MODE_ADJOINT);
                F.hit_p.st_hit(slot, make_float4(Pp.x, Pp.y, Pp.z, a.w));
                F.hit_n.st_hit(slot, make_float4(Nr.x, Nr.y, Nr.z, __uint_as_float(h.best_id)));
            }
        }
        push(fin && hit, slot, qsh, cs + 2);
        end_paths(F, ended, slot, cn);
    };
    ray_loop<false, INSTR, MODE, STACK, BT>(count, cs + 1, P.refill, F.status, fetch, finish, &nvis, &ntri);
    if (INSTR) {
        add_stats(&F.stats[3], nvis);
        add_stats(&F.stats[4], ntri);
        add_stats(&F.stats[8], nhit);
    }
}

// Light samples of every hit of the iteration (shadow queue), when they are
// not taken inside k_extend (GB_SPLIT_NEE).
__global__ void __launch_bounds__(kBlock) k_nee(Frame F, int mode) {
    const uint32_t* cs = ctr_set(F, *F.iter);
    const uint32_t count = cs[2];
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
        const uint32_t slot = F.q[2][i];
        const SceneRec& R = scene_of(F, slot);
        nee_at_hit(F, R, slot, ld3(F.hit_p.ld(slot)), ld3(F.hit_n.ld(slot)), mode != MODE_ADJOINT);
    }
}

// Any-hit of the shadow queue; the result goes to sh_d.w (1 = occluded).
template <bool INSTR, int MODE, int STACK, int BT>
__global__ void __launch_bounds__(BT, GB_SHADOW_MIN_BLOCKS * 128 / BT) k_shadow(Frame F, RenderParams P) {
    const int it = *F.iter;
    uint32_t* cs = ctr_set(F, it);
    const uint32_t count = cs[2];
    const uint32_t* qsh = F.q[2];
    uint32_t nvis = 0, ntri = 0;
    // the handle finish gets back is the slot
    auto fetch = [&](uint32_t q, uint32_t* handle, v3* o, v3* d, float* tmax, const float4** nodes,
                     const float4** tris, const float4** shade) {
        const uint32_t slot = qsh[q];
        *handle = slot;
        float4 so = F.sh_o.ld(slot), sd = F.sh_d.ld(slot);
        const SceneRec& R = scene_of(F, slot);
        *nodes = R.S.nodes;
        *tris = R.S.tris;
        *shade = R.S.shade;
        *o = ld3(so); *d = ld3(sd); *tmax = so.w;
        const bool traced = so.w >= 0.0f;
        if (traced) add_stats_lane(&F.stats[2]);  // shadow rays traced
        return traced;
    };
    // smax: the shadow ray's max_t (negative: a dark sample, not traced)
    auto finish = [&](bool fin, uint32_t slot, const Trav& h, float smax) {
        if (fin) {
            bool occl = smax < 0.0f || h.best_id != 0xffffffffu;
            rec_st(reinterpret_cast<float*>(&F.sh_d[slot]) + 3, occl ? 1.0f : 0.0f);
        }
    };
    ray_loop<true, INSTR, MODE, STACK, BT>(count, cs + 3, GB_SHADOW_REFILL > 0 ? GB_SHADOW_REFILL : P.refill,
                                           F.status, fetch, finish, &nvis, &ntri);
    if (INSTR) { add_stats(&F.stats[5], nvis); add_stats(&F.stats[6], ntri); }
    if (GB_FUSED_RESTART && P.mode != MODE_ADJOINT) restart_misses(F, P);
}

// Material record of index mi; the texture fields (last float4) only when
// the scene has textures.
__device__ __forceinline__ MaterialRec load_material(const float* mats, uint32_t mi, bool textured = false) {
    float mf[kMaterialFloats];
    const float4* mp = (const float4*)(mats + (size_t)kMaterialFloats * mi);
#pragma unroll
    for (int k = 0; k < 7; ++k) {
        float4 q = __ldg(mp + k);
        mf[4 * k] = q.x; mf[4 * k + 1] = q.y; mf[4 * k + 2] = q.z; mf[4 * k + 3] = q.w;
    }
    float4 q = textured ? __ldg(mp + 7) : make_float4(0.0f, 0.0f, 0.0f, -1.0f);
    mf[28] = q.x; mf[29] = q.y; mf[30] = q.z; mf[31] = q.w;
    return unpack_material(mf);
}

// Light the NEE of a hit picked (arealight-sampler-cpu.cpp:32-39 on the
// light draw of k_extend).
__device__ __forceinline__ int nee_light(const Frame& F, const SceneRec& R, uint32_t slot, v3 rnd) {
    if (R.S.n_lights <= 0) return 0;
    float lz = rnd.z;
    if (R.rng_mode == 1) lz = halton((int)(F.pix.ld(slot) - R.pixel_base) + 1, 3);
    return pick_light(R.S.lights, R.S.n_lights, R.S.overall_power, lz);
}

// Hit of a path in a textured scene: the ray differentials move to the hit
// (computeRayDiffs, hybrid-pt.cpp:518-519) and a diffuse texture scales the
// material's base colour.  The hit's barycentrics are recomputed with the
// traversal's own triangle test (same operands, same bits).
__device__ __noinline__ void texture_hit(const Frame& F, const SceneRec& R, uint32_t slot, float4 hn,
                                         MaterialRec* m) {
    const uint32_t tid = __float_as_uint(hn.w);
    const float4* sh = R.S.shade + 6 * (size_t)tid;
    const v3 a = ld3(__ldg(sh)), b = ld3(__ldg(sh + 1)), c = ld3(__ldg(sh + 2));
    float t, bb = 0.0f, bg = 0.0f;
    intersect_tri(ld3(F.ray_o.ld(slot)), ld3(F.ray_d.ld(slot)), a, b - a, c - a, &t, &bb, &bg);
    const float* tcs = R.S.texcoord + 6 * (size_t)tid;
    float ts, tt;
    bary2(bb, bg, tcs, &ts, &tt);
    RayDiff df = ld_rdiff(F, slot);
    const float diff = ray_diff_hit(&df, a, b, c, tcs, ts, tt, normalize_div(ld3(hn)));
    st_rdiff(F, slot, df);
    if (m->dtex >= 0 && m->dtex < R.S.n_tex)
        *m = textured_material(*m, tex_sample_bilin_lod(R.S.tex[m->dtex], ts, tt, diff));
}

// BRDF sample/eval, NEE accumulation and next ray for every shadow-queue
// entry (compute_path_contribution_and_bounce for the hits); paths that end
// go to the free queue.  MODE_FROZEN evaluates the BRDF with the scene's
// eval records and carries the sampling throughput in tp0; MODE_ADJOINT
// writes the vertex record of the path-replay adjoint.  Every path leaves
// with pb's bounce field = the number of vertices it shaded.
template <int MODE, bool TEX>
__global__ void __launch_bounds__(kBlock, GB_SHADE_MIN_BLOCKS) k_shade(Frame F, RenderParams P) {
    const int it = *F.iter;
    uint32_t* cs = ctr_set(F, it);
    uint32_t* cn = ctr_set(F, it + 1);
    const uint32_t count = cs[2];
    const uint32_t* qsh = F.q[2];
    uint32_t* qout = F.q[(it + 1) & 1];
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t l0 = *F.path_ctr;
    const uint32_t avail = l0 < P.chunk_paths ? P.chunk_paths - l0 : 0u;
    for (uint32_t i0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); i0 < count; i0 += stride) {
        uint32_t qi = i0 + lane_id();
        bool valid = qi < count;
        uint32_t slot = 0;
        bool cont = false, ended = false;
        if (valid) {
            slot = qsh[qi];
            const SceneRec& R = scene_of(F, slot);
            float4 sd = F.sh_d.ld(slot);
            float4 hp = F.hit_p.ld(slot), hn = F.hit_n.ld(slot);
            uint32_t mi = __float_as_uint(hp.w);
            const bool textured = TEX && R.S.texcoord != nullptr;
            MaterialRec m = load_material(R.S.mats, mi, textured);
            if (textured) texture_hit(F, R, slot, hn, &m);
            uint32_t pbv = F.pb.ld(slot);
            int bounce = (int)(pbv & 1023u);
            uint32_t path = pbv >> 10;
            float4 rd = F.ray_d.ld(slot), tp4 = F.tp.ld(slot), rn = F.rnd.ld(slot),
                   ps = F.psc.ld(slot);
            float4 acc = F.accum.ld(slot);
            ShadeOut o;
            if (MODE == MODE_FROZEN) {
                MaterialRec me = load_material(R.S.mats_eval, mi);
                v3 t0 = ld3(F.tp0[slot]);
                o = shade_hit(m, ld3(hp), ld3(hn), ld3(rd), ld3(tp4), ld3(rn), sd.w == 0.0f, ld3(sd), ld3(ps), R.sp,
                              F.pix.ld(slot) - R.pixel_base, path, bounce, &me, &t0);
                F.tp0[slot] = make_float4(t0.x, t0.y, t0.z, 0.0f);
            } else if (MODE == MODE_ADJOINT) {
                ShadeTrace tr;
                o = shade_hit(m, ld3(hp), ld3(hn), ld3(rd), ld3(tp4), ld3(rn), sd.w == 0.0f, ld3(sd), ld3(ps), R.sp,
                              F.pix.ld(slot) - R.pixel_base, path, bounce, nullptr, nullptr, &tr);
                int light = nee_light(F, R, slot, ld3(rn));
                uint32_t info = (uint32_t)light | ((uint32_t)tr.lobe << 16) | (tr.clamp_mask << 20) |
                                (tr.nee ? (1u << 23) : 0u) | ((tr.flags & 7u) << 24);
                float4* rec = F.adj + (size_t)bounce * kAdjPlanes * F.nslots + slot;
                rec[0] = make_float4(tp4.x, tp4.y, tp4.z, tr.pdf);
                rec[(size_t)F.nslots] = make_float4(tr.wo.x, tr.wo.y, tr.wo.z, tr.q);
                rec[2 * (size_t)F.nslots] = make_float4(tr.wi.x, tr.wi.y, tr.wi.z, tr.nee ? ps.w : 0.0f);
                rec[3 * (size_t)F.nslots] = make_float4(tr.N.x, tr.N.y, tr.N.z, __uint_as_float(mi));
                rec[4 * (size_t)F.nslots] = make_float4(tr.ld.x, tr.ld.y, tr.ld.z, __uint_as_float(info));
            } else {
                o = shade_hit(m, ld3(hp), ld3(hn), ld3(rd), ld3(tp4), ld3(rn), sd.w == 0.0f, ld3(sd), ld3(ps), R.sp,
                              F.pix.ld(slot) - R.pixel_base, path, bounce);
            }
            acc = make_float4(acc.x + o.accum_add.x, acc.y + o.accum_add.y, acc.z + o.accum_add.z, 0.0f);
            cont = o.alive && bounce + 1 < R.L;
            ended = !cont;
            const float pbw = __uint_as_float(pbv + 1u);  // ray_d.w
            if (cont) {
                F.tp.st(slot, make_float4(o.tp.x, o.tp.y, o.tp.z, 0.0f));
                F.accum.st(slot, acc);
                F.ray_o.st(slot, make_float4(o.org.x, o.org.y, o.org.z, FLT_MAX));
                F.ray_d.st(slot, make_float4(o.dir.x, o.dir.y, o.dir.z, pbw));
            } else {
                store_sample(F, P, slot, pbv, acc);
                if (MODE == MODE_ADJOINT) F.ray_d.st(slot, make_float4(rd.x, rd.y, rd.z, pbw));  // bounces for k_adjoint
            }
        }
        if (GB_FUSED_RESTART && MODE != MODE_ADJOINT) {
            // a path that shading ends restarts on its slot at once: path
            // l0 + j, j counted on from k_shadow's restarts (cn[7])
            const uint32_t j = warp_inc(ended, &cn[7]);
            const bool restart = ended && j < avail;
            if (restart) start_path(F, P, slot, l0 + j);
            push(cont || restart, slot, qout, cn);
        } else {
            push(cont, slot, qout, cn);
            end_paths(F, ended, slot, cn);
        }
    }
}

// Path-replay adjoint of every path that ended this iteration (free queue,
// before k_regen reuses the slots).  The path's value is
//   C = sum_k T_k * bl_k * col_l(k) * s_k,  T_{k+1} = clamp1(T_k * brdf_k / pdf_k) / q_k
// with pdf, q, the clamp pattern and all directions held at their recorded
// values; the reverse sweep k = K-1 .. 0 carries a = dLoss/dT_{k+1} and adds
// the BRDF vector-Jacobian products and the emission gradient to this
// block's gradient replica.  g = dLoss/dI(pixel) / spp.
__global__ void __launch_bounds__(kBlock) k_adjoint(Frame F, RenderParams P) {
    const int it = *F.iter;
    uint32_t* cn = ctr_set(F, it + 1);
    const uint32_t count = cn[4];
    float* grad = F.grad + (size_t)(blockIdx.x % (uint32_t)F.grad_replicas) * (size_t)F.grad_stride;
    const size_t ns = (size_t)F.nslots;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t slot = F.q[3][i];
        const int K = (int)(F.pb.ld(slot) & 1023u);
        const float4 g4 = F.dimg[F.pix.ld(slot)];
        if (K == 0 || (g4.x == 0.0f && g4.y == 0.0f && g4.z == 0.0f)) continue;
        const SceneRec& R = scene_of(F, slot);
        const v3 g = ld3(g4);
        float* gm_base = grad + R.grad_base;
        float* gl_base = gm_base + (size_t)kMatGradFloats * (size_t)R.n_mats;
        v3 an = mk(0.0f, 0.0f, 0.0f);  // dLoss / dT_{k+1}
        // sampling terms: gsuf = g . (light-sample terms of the vertices
        // after k); each vertex's scores are kept for the path's final miss
        // term, known once every light-sample term has been seen
        const bool st = P.sampling_terms != 0;
        float gsuf = 0.0f;
        uint32_t smi[kMaxAdjBounces];
        float ssm[kMaxAdjBounces], ssr[kMaxAdjBounces];
        int nsc = 0;
        for (int k = K - 1; k >= 0; --k) {
            const float4* rec = F.adj + (size_t)k * kAdjPlanes * ns + slot;
            const float4 r0 = rec[0], r1 = rec[ns], r2 = rec[2 * ns], r3 = rec[3 * ns], r4 = rec[4 * ns];
            const v3 T = ld3(r0), wo = ld3(r1), wi = ld3(r2), N = ld3(r3), ld = ld3(r4);
            const float pdf = r0.w, q = r1.w, sc = r2.w;
            const uint32_t mi = __float_as_uint(r3.w), info = __float_as_uint(r4.w);
            const int light = (int)(info & 0xffffu), lobe = (int)((info >> 16) & 15u);
            const uint32_t cmask = (info >> 20) & 7u;
            const bool nee = (info >> 23) & 1u;
            const uint32_t sflags = (info >> 24) & 7u;
            const MaterialRec m = load_material(R.S.mats, mi);
            MatGrad mg;
            matgrad_zero(&mg);
            v3 ak = mk(0.0f, 0.0f, 0.0f);
            float gw = 0.0f;  // dLoss / d log w of this vertex's Walter weight (through T_{k+1})
            if (an.x != 0.0f || an.y != 0.0f || an.z != 0.0f) {
                const v3 brdf = material_eval(m, lobe, wo, wi, N);
                const float inv = 1.0f / (pdf * q);
                const v3 c = mk((cmask & 1u) ? 0.0f : 1.0f, (cmask & 2u) ? 0.0f : 1.0f, (cmask & 4u) ? 0.0f : 1.0f);
                const v3 db = (c * T * an) * inv;  // dLoss / d brdf
                material_eval_vjp(m, lobe, wo, wi, N, db, &mg);
                ak = (c * brdf * an) * inv;
                gw = -dot(db, brdf);
            }
            float gnee = 0.0f;  // g . this vertex's light-sample term
            if (nee) {
                const v3 col = R.S.lights[light].col;
                const v3 psc = col * sc;
                const v3 bl = material_eval(m, lobe, wo, ld, N);
                material_eval_vjp(m, lobe, wo, ld, N, g * T * psc, &mg);
                const v3 acol = (g * T * bl) * sc;
                float* gl = gl_base + 3 * light;
                if (acol.x != 0.0f) atomicAdd(gl + 0, acol.x);
                if (acol.y != 0.0f) atomicAdd(gl + 1, acol.y);
                if (acol.z != 0.0f) atomicAdd(gl + 2, acol.z);
                ak = ak + g * bl * psc;
                gnee = dot(g, T * (bl * psc));
            }
            if (st) {
                // the branch decision moves this vertex's light-sample term
                // and everything after it; the sampled direction moves what
                // comes after this vertex; the Walter weight divides T_{k+1}
                float sm, sr, wr, zlo = 0.0f, zhi = 1.0f;
                if (R.rng_mode == 0 && R.S.n_lights > 0)
                    light_pick_interval(R.S.lights, R.S.n_lights, R.S.overall_power, light, &zlo, &zhi);
                sampling_scores(m, lobe, sflags, wo, wi, N, pdf, zlo, zhi, &sm, &sr, &wr);
                mg.metallic += sm * (gnee + gsuf);
                mg.roughness += sr * gsuf + gw * wr;
                if (sm != 0.0f || sr != 0.0f) {
                    smi[nsc] = mi;
                    ssm[nsc] = sm;
                    ssr[nsc] = sr;
                    ++nsc;
                }
            }
            gsuf += gnee;
            float* gmat = gm_base + (size_t)kMatGradFloats * mi;
            const float* mv = &mg.cdlin[0];
#pragma unroll
            for (int f = 0; f < kMatGradFloats; ++f)
                if (mv[f] != 0.0f) atomicAdd(gmat + f, mv[f]);
            an = ak;
        }
        if (st && nsc > 0) {
            // the path's final miss (the white background a throughput of
            // (1, 1, 1) adds, hybrid-pt.cpp:567-572): its sample minus the
            // light-sample terms; below rounding of the sum it is none
            const uint32_t pbv = F.pb.ld(slot);
            const float4 sv = F.samples[P.round_start[(pbv >> 10) - (uint32_t)P.p0] + F.pix.ld(slot)];
            const float gtot = dot(g, ld3(sv));
            const float gmiss = gtot - gsuf;
            if (fabsf(gmiss) > 1e-4f * fabsf(gtot)) {
                for (int i = 0; i < nsc; ++i) {
                    float* gmat = gm_base + (size_t)kMatGradFloats * smi[i];
                    if (ssm[i] != 0.0f) atomicAdd(gmat + offsetof(MatGrad, metallic) / sizeof(float), ssm[i] * gmiss);
                    if (ssr[i] != 0.0f) atomicAdd(gmat + offsetof(MatGrad, roughness) / sizeof(float), ssr[i] * gmiss);
                }
            }
        }
    }
}

// Direct lighting as the reference's gpu_area_lights integrator
// (direct-lighting.cpp:29-104, arealight-sampler.cu:156-260, :340-364), one
// pixel per thread: the pixel-centre camera ray's first hit gives the
// material colour (material_t::diffuse_color; the background for a miss,
// evaluate_material), then `samples` area-light samples of the GPU sampler
// (shadow offset as given, 0.01 there) are averaged: each adds psc * colour
// when its shadow ray is unoccluded.  Sample k uses pool update max(0, k-1)
// of the pixel's MRG32k3a stream, as the reference's update order gives
// (the pool advances after the second sample is set up).  A missed pixel's
// psc is the scaled sky texel of the direction its ray buffer holds: the
// camera ray's for the first sample, (0, 0, 0) afterwards.
__global__ void __launch_bounds__(kBlock) k_direct(DevScene S, CameraRec cam, int w, int h, int samples,
                                                   uint32_t seed, float shadow_offset, v3 background, float* out,
                                                   uint32_t* status, const MrgSubseqTable T) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= w * h) return;
    v3 o, d;
    camera_ray(cam, g % w, g / w, 0.5f, 0.5f, 0.0f, 0.0f, &o, &d);
    TraceOut hit;
    const bool is_hit = traverse<false>(S, make_ray(o, d), FLT_MAX, &hit, status);
    v3 P = mk(0.0f, 0.0f, 0.0f), N = P, mcol = background;
    if (is_hit) {
        const float4* sh = S.shade + 6 * (size_t)hit.id;
        const float4 a = sh[0];
        P = bary(hit.beta, hit.gamma, ld3(a), ld3(sh[1]), ld3(sh[2]));
        N = bary(hit.beta, hit.gamma, ld3(sh[3]), ld3(sh[4]), ld3(sh[5]));
        const float* mf = S.mats + (size_t)kMaterialFloats * __float_as_uint(a.w);
        mcol = mk(mf[25], mf[26], mf[27]);
        const int dtex = (int)mf[31];
        if (S.texcoord && dtex >= 0 && dtex < S.n_tex) {
            // pixel_evaluate_material_bilin_lod_cpu (material-cpu.cpp:36-77)
            const float* tcs = S.texcoord + 6 * (size_t)hit.id;
            float ts, tt;
            bary2(hit.beta, hit.gamma, tcs, &ts, &tt);
            RayDiff df = camera_diff(cam, g % w, g / w);
            const float diff = ray_diff_hit(&df, ld3(a), ld3(sh[1]), ld3(sh[2]), tcs, ts, tt, N);
            mcol = mcol * tex_sample_bilin_lod(S.tex[dtex], ts, tt, diff);
        }
    }
    curandStateMRG32k3a st = mrg_expand(mrg_stream(T, seed, (uint32_t)g));
    v3 rnd = draw3(&st);
    v3 buf_dir = d;
    v3 acc = mk(0.0f, 0.0f, 0.0f);
    for (int k = 0; k < samples; ++k) {
        if (k >= 2) rnd = draw3(&st);
        v3 weight = mk(0.0f, 0.0f, 0.0f);
        bool occluded = false;
        if (is_hit && S.n_lights > 0) {
            const int l = pick_light(S.lights, S.n_lights, S.overall_power, rnd.z);
            const LightRec L = S.lights[l];
            v3 so, sd;
            float smax;
            if (L.type == 1)
                sky_light_sample_uniform(S.sky, L.power, S.overall_power, P, N, rnd.x, rnd.y, shadow_offset, &so,
                                         &sd, &smax, &weight);
            else
                rect_light_sample(L, L.col, S.overall_power, P, N, rnd.x, rnd.y, shadow_offset, &so, &sd, &smax,
                                  &weight, nullptr, false);
            buf_dir = sd;
            occluded = smax >= 0.0f && traverse<true>(S, make_ray(so, sd), smax, nullptr, status);
        } else {
            if (S.sky.light >= 0) weight = S.sky.scale * sky_eval(S.sky, buf_dir);
            buf_dir = mk(0.0f, 0.0f, 0.0f);
        }
        const v3 mat = occluded ? mk(0.0f, 0.0f, 0.0f) : mcol;
        acc = (float(k) * acc + weight * mat) / (float(k) + 1.0f);
    }
    out[3 * g] = acc.x;
    out[3 * g + 1] = acc.y;
    out[3 * g + 2] = acc.z;
}

// hybrid_area_lights (direct-lighting.cpp:203-316, direct-lighting.h:137-215):
// per pixel `cam_samples` jittered camera rays (jittered lens generator,
// jitter pool update c), the material colour of each camera hit
// (evaluate_material, material-cpu.cpp:20-80; footprint from the camera
// differentials), and `light_samples` samples of the CPU area-light sampler
// per camera sample (generate_arealight_sample, arealight-sampler-cpu.cpp:
// 25-143) folded into one moving average over sample c * L + j.  Sample j of
// a camera sample is set up before the pool's update of that step, so
// samples 0 and 1 share update c*L and sample j >= 2 takes c*L + j - 1; the
// L-th update of each camera sample goes unused.  All pools are seeded
// alike in the reference (curand_init(0, pixel, 0), util-kernels.cu:276-285),
// so the jitter and light draws are one stream read twice.
__global__ void __launch_bounds__(kBlock) k_direct_hybrid(DevScene S, CameraRec cam, int w, int h, int cam_samples,
                                                          int light_samples, uint32_t seed, float shadow_offset,
                                                          v3 background, float* out, uint32_t* status,
                                                          const MrgSubseqTable T) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= w * h) return;
    const int px = g % w, py = g / w;
    curandStateMRG32k3a js = mrg_expand(mrg_stream(T, seed, (uint32_t)g)), ls = js, lens;
    const bool aperture = cam.aperture != 0.0f;
    if (aperture) lens = mrg_expand(mrg_stream(T, seed, (uint32_t)((g + 17) % (w * h))));
    const int L = light_samples;
    v3 acc = mk(0.0f, 0.0f, 0.0f);
    for (int c = 0; c < cam_samples; ++c) {
        const v3 j = draw3(&js);
        float lx = 0.0f, ly = 0.0f;
        if (aperture) {
            const v3 lj = draw3(&lens);
            lx = lj.z - 0.5f;
            ly = lj.y - 0.5f;
        }
        v3 o, d;
        camera_ray(cam, px, py, j.x, j.y, lx, ly, &o, &d);
        TraceOut hit;
        const bool is_hit = traverse<false>(S, make_ray(o, d), FLT_MAX, &hit, status);
        v3 P = mk(0.0f, 0.0f, 0.0f), N = P, mcol = background;
        if (is_hit) {
            const float4* sh = S.shade + 6 * (size_t)hit.id;
            const float4 a = sh[0];
            P = bary(hit.beta, hit.gamma, ld3(a), ld3(sh[1]), ld3(sh[2]));
            N = bary(hit.beta, hit.gamma, ld3(sh[3]), ld3(sh[4]), ld3(sh[5]));
            const float* mf = S.mats + (size_t)kMaterialFloats * __float_as_uint(a.w);
            mcol = mk(mf[25], mf[26], mf[27]);
            const int dtex = (int)mf[31];
            if (S.texcoord && dtex >= 0 && dtex < S.n_tex) {
                const float* tcs = S.texcoord + 6 * (size_t)hit.id;
                float ts, tt;
                bary2(hit.beta, hit.gamma, tcs, &ts, &tt);
                RayDiff df = camera_diff(cam, px, py);
                const float diff = ray_diff_hit(&df, ld3(a), ld3(sh[1]), ld3(sh[2]), tcs, ts, tt, N);
                mcol = mcol * tex_sample_bilin_lod(S.tex[dtex], ts, tt, diff);
            }
        }
        v3 buf_dir = d;
        v3 rnd = draw3(&ls);
        for (int k = 0; k < L; ++k) {
            if (k >= 2) rnd = draw3(&ls);
            v3 weight = mk(0.0f, 0.0f, 0.0f);
            bool occluded = false;
            if (is_hit && S.n_lights > 0) {
                const int l = pick_light(S.lights, S.n_lights, S.overall_power, rnd.z);
                const LightRec Lr = S.lights[l];
                v3 so, sd;
                float smax;
                if (Lr.type == 1)
                    sky_light_sample(S.sky, Lr.power, S.overall_power, P, N, rnd.x, rnd.y, shadow_offset, &so, &sd,
                                     &smax, &weight);
                else
                    rect_light_sample(Lr, Lr.col, S.overall_power, P, N, rnd.x, rnd.y, shadow_offset, &so, &sd,
                                      &smax, &weight);
                buf_dir = sd;
                occluded = smax >= 0.0f && traverse<true>(S, make_ray(so, sd), smax, nullptr, status);
            } else {
                if (S.sky.light >= 0) weight = S.sky.scale * sky_eval(S.sky, buf_dir);
                buf_dir = mk(0.0f, 0.0f, 0.0f);
            }
            const v3 mat = occluded ? mk(0.0f, 0.0f, 0.0f) : mcol;
            const float s = float(c * L + k);
            acc = (s * acc + weight * mat) / (s + 1.0f);
        }
        if (L >= 2) draw3(&ls);
    }
    out[3 * g] = acc.x;
    out[3 * g + 1] = acc.y;
    out[3 * g + 2] = acc.z;
}

__global__ void k_dimg_pack(const float* __restrict__ src, int n, float scale, float4* dst) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dst[i] = make_float4(src[3 * i] * scale, src[3 * i + 1] * scale, src[3 * i + 2] * scale, 0.0f);
}

// L2 image loss of one scene of a fitting step: loss = sum (x - t)^2 over
// its n pixels (one block, double accumulation in a fixed order, so the sum
// is the same every launch) and the adjoint's image gradient
// dimg = 2 (x - t) * scale (scale = 1 / spp), the same float operations as
// k_dimg_pack applied to 2 (x - t).
__global__ void __launch_bounds__(1024) k_l2_loss(const float* __restrict__ img, const float* __restrict__ target,
                                                  int n, float scale, float4* dimg, double* loss) {
    __shared__ double part[1024];
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        float g[3];
        for (int c = 0; c < 3; ++c) {
            const float d = img[3 * (size_t)i + c] - target[3 * (size_t)i + c];
            acc += (double)d * (double)d;
            g[c] = (2.0f * d) * scale;
        }
        dimg[i] = make_float4(g[0], g[1], g[2], 0.0f);
    }
    part[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) part[threadIdx.x] += part[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *loss = part[0];
}

// Sum of the gradient replicas, in double.
__global__ void k_grad_reduce(const float* __restrict__ grad, int replicas, int stride, double* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= stride) return;
    double acc = 0.0;
    for (int r = 0; r < replicas; ++r) acc += (double)grad[(size_t)r * (size_t)stride + (size_t)i];
    out[i] = acc;
}

// new_path's moving average (util-kernels.cu:17-25) over the chunk's paths
// p0 .. min(p0 + rounds, spp)-1 of every pixel, in path order.
__global__ void k_combine(Frame F, RenderParams P) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= F.ntot) return;
    const int p0 = P.p0;
    const int pe = min(p0 + P.rounds, F.scenes[F.pscene[g]].spp);
    if (p0 >= pe) return;
    v3 o = mk(0.0f, 0.0f, 0.0f);
    if (p0 > 0) { float4 c = F.out[g]; o = mk(c.x, c.y, c.z); }
    for (int p = p0; p < pe; ++p) {
        float4 s = F.samples[P.round_start[p - p0] + (uint32_t)g];
        o = combine_sample(o, mk(s.x, s.y, s.z), p);
    }
    F.out[g] = make_float4(o.x, o.y, o.z, 0.0f);
}

__global__ void k_pack_rgb(const float4* __restrict__ src, int n, float* dst) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 v = src[i];
    dst[3 * i] = v.x; dst[3 * i + 1] = v.y; dst[3 * i + 2] = v.z;
}

__global__ void k_mrg_pool(int pixel0, int npix, uint32_t seed, int first_update, int num_updates, float* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npix) return;
    curandStateMRG32k3a s;
    curand_init((unsigned long long)seed, (unsigned long long)(uint32_t)(pixel0 + i), 0ull, &s);
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
        if (S.lights[l].type == 1)
            sky_light_sample(S.sky, S.lights[l].power, S.overall_power, Pp, Nr, r.x, r.y, shadow_offset, &so, &sd,
                             &sm, &ps);
        else
            rect_light_sample(S.lights[l], S.lights[l].col, S.overall_power, Pp, Nr, r.x, r.y, shadow_offset, &so,
                              &sd, &sm, &ps);
        ray_orig[3 * i] = so.x; ray_orig[3 * i + 1] = so.y; ray_orig[3 * i + 2] = so.z;
        ray_dir[3 * i] = sd.x; ray_dir[3 * i + 1] = sd.y; ray_dir[3 * i + 2] = sd.z;
        max_t[i] = sm;
        psc[3 * i] = ps.x; psc[3 * i + 1] = ps.y; psc[3 * i + 2] = ps.z;
    } else {
        // arealight-sampler-cpu.cpp:121-142: the ray is killed and psc is the
        // (scaled) sky texel of the direction the buffer held, 0 without a sky
        v3 d = mk(ray_dir[3 * i], ray_dir[3 * i + 1], ray_dir[3 * i + 2]);
        v3 le = S.sky.light >= 0 ? S.sky.scale * sky_eval(S.sky, d) : mk(0.0f, 0.0f, 0.0f);
        ray_orig[3 * i] = FLT_MAX; ray_orig[3 * i + 1] = FLT_MAX; ray_orig[3 * i + 2] = FLT_MAX;
        ray_dir[3 * i] = 0.0f; ray_dir[3 * i + 1] = 0.0f; ray_dir[3 * i + 2] = 0.0f;
        max_t[i] = -1.0f;
        psc[3 * i] = le.x; psc[3 * i + 1] = le.y; psc[3 * i + 2] = le.z;
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
        if (max_t[i] != -1.0f)
            ac = ac + miss_contribution(t, mk(ray_dir[3 * i], ray_dir[3 * i + 1], ray_dir[3 * i + 2]), sp, &S.sky);
        ray_orig[3 * i] = FLT_MAX; ray_orig[3 * i + 1] = FLT_MAX; ray_orig[3 * i + 2] = FLT_MAX;
        ray_dir[3 * i] = 0.0f; ray_dir[3 * i + 1] = 0.0f; ray_dir[3 * i + 2] = 0.0f;
        max_t[i] = -1.0f;
        t = mk(0.0f, 0.0f, 0.0f);
    }
    tp[3 * i] = t.x; tp[3 * i + 1] = t.y; tp[3 * i + 2] = t.z;
    accum[3 * i] = ac.x; accum[3 * i + 1] = ac.y; accum[3 * i + 2] = ac.z;
}

inline int blocks_for(int n) { return (n + kBlock - 1) / kBlock; }

// SMs and resident blocks per SM of a persistent kernel.
struct Grid {
    int sms, per;
};

template <typename K>
Grid persistent_grid(K kernel, int block = kBlock) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, block, 0);
    if (sms < 1) sms = 1;
    if (per < 1) per = 1;
    return Grid{sms, per};
}

template <typename K>
int persistent_blocks(K kernel) {
    Grid g = persistent_grid(kernel);
    return g.sms * g.per;
}

// Grid of a persistent traversal kernel: every SM holds min(occupancy
// limit, blocks_per_sm) blocks (all it can hold when blocks_per_sm is 0);
// blocks_per_sm counts 128-thread blocks, so blocks of bt threads scale it.
inline int traversal_grid(const Grid& g, int blocks_per_sm, int bt = kBlock) {
    const int want = blocks_per_sm > 0 ? std::max(1, blocks_per_sm * kBlock / bt) : g.per;
    return g.sms * std::min(g.per, want);
}

}  // namespace

cudaError_t k_launch_trace(const DevScene& S, int n, const float* orig, const float* dir, const float* tmax,
                           float4* hits, uint8_t* occluded, bool any, uint32_t* status, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_trace<<<blocks_for(n), kBlock, 0, st>>>(S, n, orig, dir, tmax, hits, occluded, any ? 1 : 0, status);
    return cudaGetLastError();
}

// The subsequence jumps, computed once per process.
const MrgSubseqTable& subseq_table() {
    static const MrgSubseqTable T = [] {
        MrgSubseqTable t;
        mrg_subsequence_table(&t);
        return t;
    }();
    return T;
}

cudaError_t k_launch_frame_init(const Frame& F, bool rng, cudaStream_t st) {
    k_fill_pscene<<<blocks_for(F.ntot), kBlock, 0, st>>>(F);
    if (rng) k_rng_init_frame<<<blocks_for(F.ntot), kBlock, 0, st>>>(F, subseq_table());
    return cudaGetLastError();
}

cudaError_t k_launch_start(const Frame& F, const RenderParams& P, int nstart, cudaStream_t st) {
    k_start<<<blocks_for(std::max(nstart, 1)), kBlock, 0, st>>>(F, P, nstart);
    return cudaGetLastError();
}

// Launch of a traversal kernel; with an L2 window in P (the scene's node
// array) the launch carries it as an access-policy attribute: node lines
// persist in the L2 set-aside, so that the per-iteration state streaming
// past does not evict them.
template <typename K>
void launch_traversal(K kernel, dim3 grid, int block, const Frame& F, const RenderParams& P, cudaStream_t st) {
    if (P.l2_nodes_bytes == 0) {
        kernel<<<grid, block, 0, st>>>(F, P);
        return;
    }
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeAccessPolicyWindow;
    at[0].val.accessPolicyWindow.base_ptr = const_cast<void*>(P.l2_nodes);
    at[0].val.accessPolicyWindow.num_bytes = (size_t)P.l2_nodes_bytes;
    at[0].val.accessPolicyWindow.hitRatio = P.l2_hit_ratio;
    at[0].val.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
    at[0].val.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, F, P);
}

template <bool INSTR, int MODE, int STACK, int BT>
void launch_extend_v(const Frame& F, const RenderParams& P, cudaStream_t st) {
    static Grid g = persistent_grid(k_extend<INSTR, MODE, STACK, BT>, BT);
    launch_traversal(k_extend<INSTR, MODE, STACK, BT>, traversal_grid(g, P.blocks_per_sm, BT), BT, F, P, st);
}

// The default triangle policy has variants for two stack depths and two
// block shapes (RenderParams::trav_variant), the other policies one each.
template <bool INSTR, int MODE>
void launch_extend_t(const Frame& F, const RenderParams& P, cudaStream_t st) {
    if (MODE == 0 && P.trav_variant == 1) launch_extend_v<INSTR, MODE, 24, 128>(F, P, st);
    else if (MODE == 0 && P.trav_variant == 2) launch_extend_v<INSTR, MODE, 32, 64>(F, P, st);
    else if (MODE == 0 && P.trav_variant == 3) launch_extend_v<INSTR, MODE, 24, 64>(F, P, st);
    else launch_extend_v<INSTR, MODE, kStack, kBlock>(F, P, st);
    if (GB_SPLIT_NEE) {
        static int gn = persistent_blocks(k_nee);
        k_nee<<<gn, kBlock, 0, st>>>(F, P.mode);
    }
}

template <bool INSTR, int MODE, int STACK, int BT>
void launch_shadow_v(const Frame& F, const RenderParams& P, cudaStream_t st) {
    static Grid g = persistent_grid(k_shadow<INSTR, MODE, STACK, BT>, BT);
    launch_traversal(k_shadow<INSTR, MODE, STACK, BT>, traversal_grid(g, P.blocks_per_sm, BT), BT, F, P, st);
}

template <bool INSTR, int MODE>
void launch_shadow_t(const Frame& F, const RenderParams& P, cudaStream_t st) {
    if (MODE == 0 && P.trav_variant == 1) launch_shadow_v<INSTR, MODE, 24, 128>(F, P, st);
    else if (MODE == 0 && P.trav_variant == 2) launch_shadow_v<INSTR, MODE, 32, 64>(F, P, st);
    else if (MODE == 0 && P.trav_variant == 3) launch_shadow_v<INSTR, MODE, 24, 64>(F, P, st);
    else launch_shadow_v<INSTR, MODE, kStack, kBlock>(F, P, st);
}

cudaError_t k_launch_extend(const Frame& F, const RenderParams& P, bool instrument, cudaStream_t st) {
    switch (P.tri_mode * 2 + (instrument ? 1 : 0)) {
        case 0: launch_extend_t<false, 0>(F, P, st); break;
        case 1: launch_extend_t<true, 0>(F, P, st); break;
        case 2: launch_extend_t<false, 1>(F, P, st); break;
        case 3: launch_extend_t<true, 1>(F, P, st); break;
        case 4: launch_extend_t<false, 2>(F, P, st); break;
        case 5: launch_extend_t<true, 2>(F, P, st); break;
        case 6: launch_extend_t<false, 3>(F, P, st); break;
        default: launch_extend_t<true, 3>(F, P, st); break;
    }
    return cudaGetLastError();
}

cudaError_t k_launch_shadow(const Frame& F, const RenderParams& P, bool instrument, cudaStream_t st) {
    switch (P.tri_mode * 2 + (instrument ? 1 : 0)) {
        case 0: launch_shadow_t<false, 0>(F, P, st); break;
        case 1: launch_shadow_t<true, 0>(F, P, st); break;
        case 2: launch_shadow_t<false, 1>(F, P, st); break;
        case 3: launch_shadow_t<true, 1>(F, P, st); break;
        case 4: launch_shadow_t<false, 2>(F, P, st); break;
        case 5: launch_shadow_t<true, 2>(F, P, st); break;
        case 6: launch_shadow_t<false, 3>(F, P, st); break;
        default: launch_shadow_t<true, 3>(F, P, st); break;
    }
    return cudaGetLastError();
}

// Grid of the streaming per-path kernels (k_shade, k_regen): persistent for
// pools of up to 2^20 slots, one thread per four slots above that (or
// always, with GB_WIDE_STREAM_GRIDS), each thread taking every
// (grid size)-th queue entry.  On the 1M-triangle frame with 2^21 slots a
// thread per slot shades in 7.0 ms against 8.0 for the persistent grid; with
// 2^24 slots a quarter of that grid (an iteration shades ~3 M hits) in
// 4.8 ms against 6.2 for a thread per slot (1071 against 1058 Mpaths/s); on
// the 256x256 16-spp Cornell frame (2^20 slots) the persistent grid in
// 0.39 ms against 0.47.
#ifndef GB_WIDE_GRID_DIV
#define GB_WIDE_GRID_DIV 4  // the wide grid has nslots / GB_WIDE_GRID_DIV threads
#endif
inline int stream_grid(int persistent, int nslots) {
    return (GB_WIDE_STREAM_GRIDS || nslots > (1 << 20)) ? std::max(1, blocks_for(nslots / GB_WIDE_GRID_DIV))
                                                          : persistent;
}

template <int MODE, bool TEX>
void launch_shade_t(const Frame& F, const RenderParams& P, cudaStream_t st) {
    static int g = persistent_blocks(k_shade<MODE, TEX>);
    k_shade<MODE, TEX><<<stream_grid(g, F.nslots), kBlock, 0, st>>>(F, P);
}

// The texture path is compiled into its own variant so that frames without
// textures run the kernel without it; replay and adjoint frames have none.
cudaError_t k_launch_shade(const Frame& F, const RenderParams& P, cudaStream_t st) {
    if (P.mode == MODE_FROZEN) launch_shade_t<MODE_FROZEN, false>(F, P, st);
    else if (P.mode == MODE_ADJOINT) launch_shade_t<MODE_ADJOINT, false>(F, P, st);
    else if (P.textured) launch_shade_t<MODE_FORWARD, true>(F, P, st);
    else launch_shade_t<MODE_FORWARD, false>(F, P, st);
    return cudaGetLastError();
}

int k_adjoint_grid() {
    static int g = persistent_blocks(k_adjoint);
    return g;
}

cudaError_t k_launch_adjoint(const Frame& F, const RenderParams& P, cudaStream_t st) {
    k_adjoint<<<k_adjoint_grid(), kBlock, 0, st>>>(F, P);
    return cudaGetLastError();
}

cudaError_t k_launch_direct(const DevScene& S, const CameraRec& cam, int w, int h, int samples, uint32_t seed,
                            float shadow_offset, v3 background, float* out, uint32_t* status, cudaStream_t st) {
    if (w * h <= 0) return cudaSuccess;
    k_direct<<<blocks_for(w * h), kBlock, 0, st>>>(S, cam, w, h, samples, seed, shadow_offset, background, out, status,
                                                   subseq_table());
    return cudaGetLastError();
}

cudaError_t k_launch_direct_hybrid(const DevScene& S, const CameraRec& cam, int w, int h, int cam_samples,
                                   int light_samples, uint32_t seed, float shadow_offset, v3 background, float* out,
                                   uint32_t* status, cudaStream_t st) {
    if (w * h <= 0) return cudaSuccess;
    k_direct_hybrid<<<blocks_for(w * h), kBlock, 0, st>>>(S, cam, w, h, cam_samples, light_samples, seed,
                                                          shadow_offset, background, out, status, subseq_table());
    return cudaGetLastError();
}

cudaError_t k_launch_dimg_pack(const float* src, int n, float scale, float4* dst, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_dimg_pack<<<blocks_for(n), kBlock, 0, st>>>(src, n, scale, dst);
    return cudaGetLastError();
}

cudaError_t k_launch_l2_loss(const float* img, const float* target, int n, float scale, float4* dimg, double* loss,
                             cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_l2_loss<<<1, 1024, 0, st>>>(img, target, n, scale, dimg, loss);
    return cudaGetLastError();
}

cudaError_t k_launch_grad_reduce(const float* grad, int replicas, int stride, double* out, cudaStream_t st) {
    if (stride <= 0) return cudaSuccess;
    k_grad_reduce<<<blocks_for(stride), kBlock, 0, st>>>(grad, replicas, stride, out);
    return cudaGetLastError();
}

int k_launches_per_iteration(int mode) {
    if (mode == MODE_ADJOINT) return 6;   // extend, shadow, shade, adjoint, regen, step
    return GB_FUSED_RESTART ? 4 : 5;      // restarts inside shadow and shade
}

cudaError_t k_launch_regen(const Frame& F, const RenderParams& P, cudaStream_t st) {
    if (GB_FUSED_RESTART && P.mode != MODE_ADJOINT) return cudaSuccess;  // restarted in k_shadow / k_shade
    static int g0 = persistent_blocks(k_regen);
    k_regen<<<stream_grid(g0, F.nslots), kBlock, 0, st>>>(F, P);
    return cudaGetLastError();
}

cudaError_t k_launch_step(const Frame& F, const RenderParams& P, unsigned long long cond, bool has_cond,
                          int max_iters, cudaStream_t st) {
    k_step<<<1, 1, 0, st>>>(F, P, cond, has_cond ? 1 : 0, max_iters);
    return cudaGetLastError();
}

cudaError_t k_launch_jitter_pool(const Frame& F, const RenderParams& P, cudaStream_t st) {
    k_jitter_pool<<<blocks_for(F.ntot), kBlock, 0, st>>>(F, P);
    return cudaGetLastError();
}

cudaError_t k_launch_combine(const Frame& F, const RenderParams& P, cudaStream_t st) {
    k_combine<<<blocks_for(F.ntot), kBlock, 0, st>>>(F, P);
    return cudaGetLastError();
}

cudaError_t k_launch_pack_rgb(const float4* src, int n, float* dst, cudaStream_t st) {
    k_pack_rgb<<<blocks_for(n), kBlock, 0, st>>>(src, n, dst);
    return cudaGetLastError();
}

cudaError_t k_launch_mrg_states(uint32_t seed, const uint32_t* sub, int n, int method, uint32_t* out,
                                cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_mrg_states<<<blocks_for(n), kBlock, 0, st>>>(subseq_table(), seed, sub, n, method, out);
    return cudaGetLastError();
}

cudaError_t k_launch_mrg_pool(int pixel0, int npix, uint32_t seed, int first_update, int num_updates, float* out,
                              cudaStream_t st) {
    k_mrg_pool<<<blocks_for(npix), kBlock, 0, st>>>(pixel0, npix, seed, first_update, num_updates, out);
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
