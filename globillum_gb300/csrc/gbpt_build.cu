// gbpt_build.cu -- device BVH construction: Morton order, PLOC clustering,
// bottom-up leaf decisions, level-by-level collapse to compressed 8-wide
// nodes, and refits.  Declarations and the method are in gbpt_build.h.
#include "gbpt_build.h"
#include "gbpt_bvh.h"

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cstring>
#include <vector>

namespace gb {

namespace {

const int kBuildBlock = 256;
const int kMaxRadius = 32;
const int kLeafMax = 3;  // triangles per leaf (the node meta holds 3 bits of them)

// Float order as unsigned order, for atomicMin / atomicMax of bounds.
__device__ __forceinline__ unsigned f2ord(float f) {
    unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// Box::area of gbpt_bvh.cpp.
__device__ __forceinline__ float box_area(float4 lo, float4 hi) {
    float dx = fmaxf(0.0f, hi.x - lo.x), dy = fmaxf(0.0f, hi.y - lo.y), dz = fmaxf(0.0f, hi.z - lo.z);
    return 2.0f * (dx * dy + dy * dz + dz * dx);
}
__device__ __forceinline__ float4 vmin(float4 a, float4 b) {
    return make_float4(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z), 0.0f);
}
__device__ __forceinline__ float4 vmax(float4 a, float4 b) {
    return make_float4(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z), 0.0f);
}
__device__ __forceinline__ float comp(float4 v, int a) { return a == 0 ? v.x : a == 1 ? v.y : v.z; }

__device__ __forceinline__ void tri_box(const float* pos, int t, float4* lo, float4* hi) {
    const float* p = pos + 9 * (size_t)t;
    float4 l = make_float4(p[0], p[1], p[2], 0.0f), h = l;
    for (int v = 1; v < 3; ++v) {
        float4 q = make_float4(p[3 * v], p[3 * v + 1], p[3 * v + 2], 0.0f);
        l = vmin(l, q);
        h = vmax(h, q);
    }
    *lo = l;
    *hi = h;
}

// Triangle boxes, centroid bounds (6 ordered uints: lo xyz, hi xyz) and a
// flag for non-finite vertices.
__global__ void k_tri_prep(const float* __restrict__ pos, int n, float4* tlo, float4* thi, unsigned* cb, int* bad) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    float4 c = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    bool ok = t < n;
    if (t < n) {
        const float* p = pos + 9 * (size_t)t;
        for (int k = 0; k < 9; ++k)
            if (!isfinite(p[k])) ok = false;
        if (!ok) atomicExch(bad, 1);
        float4 lo, hi;
        tri_box(pos, t, &lo, &hi);
        tlo[t] = lo;
        thi[t] = hi;
        c = make_float4(0.5f * (lo.x + hi.x), 0.5f * (lo.y + hi.y), 0.5f * (lo.z + hi.z), 0.0f);
    }
    unsigned v[6];
    v[0] = ok ? f2ord(c.x) : 0xffffffffu;
    v[1] = ok ? f2ord(c.y) : 0xffffffffu;
    v[2] = ok ? f2ord(c.z) : 0xffffffffu;
    v[3] = ok ? f2ord(c.x) : 0u;
    v[4] = ok ? f2ord(c.y) : 0u;
    v[5] = ok ? f2ord(c.z) : 0u;
    for (int o = 16; o > 0; o >>= 1)
        for (int k = 0; k < 6; ++k) {
            unsigned w = __shfl_xor_sync(0xffffffffu, v[k], o);
            v[k] = k < 3 ? min(v[k], w) : max(v[k], w);
        }
    if ((threadIdx.x & 31) == 0) {
        for (int k = 0; k < 3; ++k) atomicMin(&cb[k], v[k]);
        for (int k = 3; k < 6; ++k) atomicMax(&cb[k], v[k]);
    }
}

// 21 bits -> every third bit of 63.
__device__ __forceinline__ uint64_t spread3(uint64_t x) {
    x &= 0x1fffffull;
    x = (x | x << 32) & 0x1f00000000ffffull;
    x = (x | x << 16) & 0x1f0000ff0000ffull;
    x = (x | x << 8) & 0x100f00f00f00f00full;
    x = (x | x << 4) & 0x10c30c30c30c30c3ull;
    x = (x | x << 2) & 0x1249249249249249ull;
    return x;
}

__global__ void k_morton(const float4* __restrict__ tlo, const float4* __restrict__ thi, int n, const unsigned* cb,
                         uint64_t* keys, int* vals) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    float4 lo = tlo[t], hi = thi[t];
    float c[3] = {0.5f * (lo.x + hi.x), 0.5f * (lo.y + hi.y), 0.5f * (lo.z + hi.z)};
    uint64_t code = 0;
    for (int a = 0; a < 3; ++a) {
        float b0 = ord2f(cb[a]), b1 = ord2f(cb[3 + a]);
        float ext = b1 - b0;
        float q = ext > 0.0f ? (c[a] - b0) / ext * 2097152.0f : 0.0f;
        uint32_t qi = q <= 0.0f ? 0u : q >= 2097151.0f ? 2097151u : (uint32_t)q;
        code |= spread3(qi) << (2 - a);
    }
    keys[t] = code;
    vals[t] = t;
}

// Leaves of the binary tree in Morton order; they are also the first clusters.
__global__ void k_leaves(const int* __restrict__ order, const float4* __restrict__ tlo,
                         const float4* __restrict__ thi, int n, float4* blo, float4* bhi, int2* bchild,
                         int* bparent, float4* clo, float4* chi, int* cnode) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int t = order[i];
    float4 lo = tlo[t], hi = thi[t];
    blo[i] = lo;
    bhi[i] = hi;
    bchild[i] = make_int2(~t, -1);
    bparent[i] = -1;
    clo[i] = lo;
    chi[i] = hi;
    cnode[i] = i;
}

// ---------------------------------------------------------------- clustering
// Nearest neighbour of every cluster within `radius` positions of the
// Morton-ordered cluster list, by the surface area of the union box.  Pairs
// are ordered by (area, lower index, higher index), a strict total order on
// unordered pairs, so the smallest pair inside the window is always mutual
// and every pass merges at least one pair.
__global__ void __launch_bounds__(kBuildBlock) k_ploc_nn(const float4* __restrict__ clo,
                                                        const float4* __restrict__ chi, int n, int radius,
                                                        int* nn) {
    __shared__ float4 slo[kBuildBlock + 2 * kMaxRadius];
    __shared__ float4 shi[kBuildBlock + 2 * kMaxRadius];
    int base = blockIdx.x * kBuildBlock - radius;
    for (int k = threadIdx.x; k < kBuildBlock + 2 * radius; k += kBuildBlock) {
        int g = base + k;
        if (g >= 0 && g < n) {
            slo[k] = clo[g];
            shi[k] = chi[g];
        }
    }
    __syncthreads();
    int i = blockIdx.x * kBuildBlock + threadIdx.x;
    if (i >= n) return;
    int si = threadIdx.x + radius;
    float4 lo = slo[si], hi = shi[si];
    float best = 3.0e38f;
    int bj = -1;
    int j0 = max(0, i - radius), j1 = min(n - 1, i + radius);
    for (int j = j0; j <= j1; ++j) {
        if (j == i) continue;
        int sj = j - base;
        float a = box_area(vmin(lo, slo[sj]), vmax(hi, shi[sj]));
        // for a fixed i, the pair order at equal area is increasing j, the
        // order of this loop: the first of equal areas wins
        if (bj < 0 || a < best) {
            best = a;
            bj = j;
        }
    }
    nn[i] = bj;
}

// Keep / merge flags of a pass: cluster i survives when its neighbour does
// not choose it back, or when it is the lower index of a mutual pair (then
// it becomes the merged cluster).  Packed as keep << 32 | merge for one scan.
__global__ void k_ploc_flags(const int* __restrict__ nn, int n, unsigned long long* flags) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int j = nn[i];
    bool mutual = j >= 0 && j < n && nn[j] == i;
    unsigned long long keep = (!mutual || i < j) ? 1ull : 0ull;
    unsigned long long merge = (mutual && i < j) ? 1ull : 0ull;
    flags[i] = keep << 32 | merge;
}

// Writes the merged nodes and the next cluster list; the last thread
// stores (clusters left, nodes made) in totals.
__global__ void k_ploc_compact(const int* __restrict__ nn, int n, int inner_base,
                               const unsigned long long* __restrict__ offs, const float4* __restrict__ clo,
                               const float4* __restrict__ chi, const int* __restrict__ cnode, float4* olo,
                               float4* ohi, int* onode, float4* blo, float4* bhi, int2* bchild, int* bparent,
                               int2* totals) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int j = nn[i];
    bool mutual = j >= 0 && j < n && nn[j] == i;
    bool keep = !mutual || i < j;
    bool merge = mutual && i < j;
    unsigned long long o = offs[i];
    int pos = (int)(o >> 32), made = (int)(o & 0xffffffffull);
    if (merge) {
        int node = inner_base + made;
        int a = cnode[i], b = cnode[j];
        float4 lo = vmin(clo[i], clo[j]), hi = vmax(chi[i], chi[j]);
        blo[node] = lo;
        bhi[node] = hi;
        bchild[node] = make_int2(a, b);
        bparent[node] = -1;
        bparent[a] = node;
        bparent[b] = node;
        olo[pos] = lo;
        ohi[pos] = hi;
        onode[pos] = node;
    } else if (keep) {
        olo[pos] = clo[i];
        ohi[pos] = chi[i];
        onode[pos] = cnode[i];
    }
    if (i == n - 1) *totals = make_int2(pos + (keep ? 1 : 0), made + (merge ? 1 : 0));
}

// ------------------------------------------------------------ bottom-up pass
// One thread per leaf climbs towards the root; the second thread to reach a
// node combines its children (Karras, "Maximizing Parallelism in the
// Construction of BVHs, Octrees, and k-d Trees", HPG 2012).  Build mode:
// subtree triangle counts and the leaf rule of the host builder (a node of
// at most kLeafMax triangles is stored as one leaf when count <= 0.5 +
// (A_l c_l + A_r c_r) / A).  Refit mode: boxes from the moved vertices.
// bad = 2 if a parent chain is longer than the tree.
// SAH-optimal 8-wide grouping (WideDp of gbpt_bvh.cpp), when dcost is
// given: dcost[8v + i-1] = least cost of v's subtree as at most i slots of
// its wide parent, dhow[8v + i-1] = 0 (fewer slots) or the slots the left
// child gets (i = 1: 1 leaf, 2 wide node), dsplit[v] = the left child's share
// of the 8 slots of a wide node at v.  The leaf flag is then dhow[8v] == 1.
__device__ void wide_dp_node(int v, int l, int r, int cnt, float area, float prim_cost, float* dcost,
                             int8_t* dhow, int8_t* dsplit, uint8_t* bleaf) {
    float cl[8], cr[8];
    for (int k = 0; k < 8; ++k) {
        cl[k] = __ldcg(&dcost[8 * (size_t)l + k]);
        cr[k] = __ldcg(&dcost[8 * (size_t)r + k]);
    }
    float dist[9];
    int8_t dk[9];
    for (int j = 2; j <= 8; ++j) {
        dist[j] = 3.0e38f;
        dk[j] = 1;
        for (int k = 1; k < j; ++k) {
            const float c = cl[k - 1] + cr[j - k - 1];
            if (c < dist[j]) { dist[j] = c; dk[j] = (int8_t)k; }
        }
    }
    dsplit[v] = dk[8];
    const float wide = area + dist[8];
    const float leaf = cnt <= kLeafMax ? area * (float)cnt * prim_cost : 3.0e38f;
    float prev = leaf <= wide ? leaf : wide;
    dcost[8 * (size_t)v] = prev;
    dhow[8 * (size_t)v] = leaf <= wide ? 1 : 2;
    bleaf[v] = leaf <= wide ? 1 : 0;
    for (int i = 2; i <= 8; ++i) {
        if (dist[i] < prev) { prev = dist[i]; dhow[8 * (size_t)v + i - 1] = dk[i]; }
        else dhow[8 * (size_t)v + i - 1] = 0;
        dcost[8 * (size_t)v + i - 1] = prev;
    }
}

__global__ void k_bottom_up(int n, const int* __restrict__ bparent, const int2* __restrict__ bchild, float4* blo,
                            float4* bhi, int* bcount, uint8_t* bleaf, unsigned* visit, const float* __restrict__ pos,
                            int refit, int* bad, float* dcost, int8_t* dhow, int8_t* dsplit, float prim_cost) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (refit) {
        float4 lo, hi;
        tri_box(pos, ~bchild[i].x, &lo, &hi);
        blo[i] = lo;
        bhi[i] = hi;
    } else {
        bcount[i] = 1;
        bleaf[i] = 1;
        if (dcost) {
            const float c = box_area(blo[i], bhi[i]) * prim_cost;
            for (int k = 0; k < 8; ++k) {
                dcost[8 * (size_t)i + k] = c;
                dhow[8 * (size_t)i + k] = k == 0 ? 1 : 0;
            }
        }
    }
    int node = bparent[i];
    for (int guard = 0; node >= 0; ++guard) {
        if (guard >= n) {
            atomicExch(bad, 2);
            return;
        }
        __threadfence();
        if (atomicAdd(&visit[node], 1u) == 0u) return;  // the sibling's thread continues
        __threadfence();
        int2 c = bchild[node];
        float4 llo = __ldcg(&blo[c.x]), lhi = __ldcg(&bhi[c.x]);
        float4 rlo = __ldcg(&blo[c.y]), rhi = __ldcg(&bhi[c.y]);
        if (refit) {
            blo[node] = vmin(llo, rlo);
            bhi[node] = vmax(lhi, rhi);
        } else {
            int cl = __ldcg(&bcount[c.x]), cr = __ldcg(&bcount[c.y]);
            int cnt = cl + cr;
            bcount[node] = cnt;
            float pa = box_area(blo[node], bhi[node]);
            float best = box_area(llo, lhi) * (float)cl + box_area(rlo, rhi) * (float)cr;
            float split = 0.5f + (pa > 0.0f ? best / pa : 0.0f);
            bleaf[node] = (cnt <= kLeafMax && (float)cnt <= split) ? 1 : 0;
            if (dcost) wide_dp_node(node, c.x, c.y, cnt, pa, prim_cost, dcost, dhow, dsplit, bleaf);
            __threadfence();
        }
        node = bparent[node];
    }
}

// ------------------------------------------------------------------ collapse
// pad_box of gbpt_bvh.cpp: 2^-19 of the largest magnitude.
__device__ __forceinline__ void pad_box_d(float4* lo, float4* hi) {
    float m = 0.0f;
    m = fmaxf(m, fmaxf(fabsf(lo->x), fabsf(hi->x)));
    m = fmaxf(m, fmaxf(fabsf(lo->y), fabsf(hi->y)));
    m = fmaxf(m, fmaxf(fabsf(lo->z), fabsf(hi->z)));
    float d = m * (1.0f / 524288.0f) + 1e-30f;
    lo->x -= d; lo->y -= d; lo->z -= d;
    hi->x += d; hi->y += d; hi->z += d;
}

// Children of one 8-wide node (Collapser::fill of gbpt_bvh.cpp): the slots
// of the SAH-optimal grouping (dhow / dsplit from k_bottom_up), or, without
// it, the binary node's two children with the stored-inner child of largest
// area replaced by its two children while fewer than 8; then give each child
// the octant slot whose rays should visit it first (greedy on the centroid
// offset along the octant's diagonal).  plan gets the child of each slot
// (-1 = empty); flags = inner children << 32 | leaf triangles.
__global__ void k_collapse_plan(const int* __restrict__ q, int m, int node_base, const float4* __restrict__ blo,
                                const float4* __restrict__ bhi, const int2* __restrict__ bchild,
                                const uint8_t* __restrict__ bleaf, const int* __restrict__ bcount, int* plan,
                                unsigned long long* flags, const int8_t* __restrict__ dhow,
                                const int8_t* __restrict__ dsplit, int n) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    int b = q[k];
    int ch[8];
    int nc;
    if (bleaf[b]) {
        ch[0] = b;
        nc = 1;
    } else if (dhow) {
        // the slots of the SAH-optimal grouping, left to right
        int sv[8], si[8], sp = 0;
        const int2 c = bchild[b];
        sv[sp] = c.y; si[sp] = 8 - dsplit[b]; ++sp;
        sv[sp] = c.x; si[sp] = dsplit[b]; ++sp;
        nc = 0;
        while (sp > 0 && nc < 8) {
            const int v = sv[--sp];
            int i = si[sp];
            while (i > 1 && dhow[8 * (size_t)v + i - 1] == 0) --i;
            if (i <= 1 || v < n) { ch[nc++] = v; continue; }
            const int kk = dhow[8 * (size_t)v + i - 1];
            const int2 cc = bchild[v];
            if (sp + 2 > 8) { ch[nc++] = v; continue; }  // never taken: slot counts only shrink
            sv[sp] = cc.y; si[sp] = i - kk; ++sp;
            sv[sp] = cc.x; si[sp] = kk; ++sp;
        }
    } else {
        int2 c = bchild[b];
        ch[0] = c.x;
        ch[1] = c.y;
        nc = 2;
    }
    while (!dhow && nc < 8) {
        int best = -1;
        float ba = -1.0f;
        for (int i = 0; i < nc; ++i)
            if (!bleaf[ch[i]]) {
                float a = box_area(blo[ch[i]], bhi[ch[i]]);
                if (a > ba) { ba = a; best = i; }
            }
        if (best < 0) break;
        int2 c = bchild[ch[best]];
        ch[best] = c.x;
        ch[nc++] = c.y;
    }
    float4 clo[8], chi[8];
    float4 nlo = make_float4(3.0e38f, 3.0e38f, 3.0e38f, 0.0f), nhi = make_float4(-3.0e38f, -3.0e38f, -3.0e38f, 0.0f);
    for (int i = 0; i < nc; ++i) {
        clo[i] = blo[ch[i]];
        chi[i] = bhi[ch[i]];
        pad_box_d(&clo[i], &chi[i]);
        nlo = vmin(nlo, clo[i]);
        nhi = vmax(nhi, chi[i]);
    }
    float ncen[3] = {0.5f * (nlo.x + nhi.x), 0.5f * (nlo.y + nhi.y), 0.5f * (nlo.z + nhi.z)};
    float cost[8][8];
    for (int i = 0; i < nc; ++i)
        for (int s = 0; s < 8; ++s) {
            float c = 0.0f;
            for (int a = 0; a < 3; ++a) {
                float cc = 0.5f * (comp(clo[i], a) + comp(chi[i], a)) - ncen[a];
                c += ((s >> a) & 1) ? -cc : cc;
            }
            cost[i][s] = c;
        }
    int slot_child[8];
    for (int s = 0; s < 8; ++s) slot_child[s] = -1;
    unsigned used_ch = 0, used_slot = 0;
    for (int it = 0; it < nc; ++it) {
        float bc = 3.0e38f;
        int bi = -1, bs = -1;
        for (int i = 0; i < nc; ++i)
            if (!((used_ch >> i) & 1))
                for (int s = 0; s < 8; ++s)
                    if (!((used_slot >> s) & 1) && cost[i][s] < bc) { bc = cost[i][s]; bi = i; bs = s; }
        if (bi < 0) {  // non-finite costs: first free child into first free slot
            bi = __ffs(~used_ch) - 1;
            bs = __ffs(~used_slot) - 1;
        }
        used_ch |= 1u << bi;
        used_slot |= 1u << bs;
        slot_child[bs] = ch[bi];
    }
    unsigned long long n_inner = 0, n_tri = 0;
    for (int s = 0; s < 8; ++s) {
        int c = slot_child[s];
        plan[(size_t)(node_base + k) * 8 + s] = c;
        if (c < 0) continue;
        if (bleaf[c]) n_tri += (unsigned long long)bcount[c];
        else ++n_inner;
    }
    flags[k] = n_inner << 32 | n_tri;
}

// Smallest e >= -100 with 255 * 2^e >= ext (the exponent rule of the host
// collapse), from the binary exponent of ext / 255.
__device__ int plane_exponent(float ext) {
    if (!(ext > 0.0f)) return -100;
    int k;
    double mant = frexp((double)ext / 255.0, &k);
    int e = mant == 0.5 ? k - 1 : k;
    while (ldexp(255.0, e) < (double)ext) ++e;
    while (e > -100 && ldexp(255.0, e - 1) >= (double)ext) --e;
    return max(e, -100);
}

__device__ __forceinline__ uint32_t pack4(const uint8_t* b) {
    return (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) | ((uint32_t)b[3] << 24);
}

// Writes the 8-wide node of each planned item and the triangle records of
// its leaf children.  Build mode: child and triangle bases from the scan
// of the plan's counts, inner children queued for the next level, the last
// item writing (inner children, triangles) of the level to totals.  Refit
// mode (q unused, item = node index): bases from the node being rewritten.
// bad = 3 if an index would leave its buffer (nothing is written there).
__global__ void k_collapse_emit(const int* __restrict__ plan, int m, int node_base, int next_base, int tri_base,
                                const unsigned long long* __restrict__ offs,
                                const unsigned long long* __restrict__ flags, const float4* __restrict__ blo,
                                const float4* __restrict__ bhi, const int2* __restrict__ bchild,
                                const uint8_t* __restrict__ bleaf, int n, const float* __restrict__ pos,
                                uint4* nodes, float4* tris, int* q_next, int node_cap, int2* totals, int refit,
                                int* bad) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    int cw = node_base + k;
    if (cw >= node_cap) { atomicExch(bad, 3); return; }
    int base_child, base_tri;
    if (refit) {
        uint4 w4 = nodes[(size_t)cw * 5 + 1];
        base_child = (int)w4.x;
        base_tri = (int)w4.y;
    } else {
        base_child = next_base + (int)(offs[k] >> 32);
        base_tri = tri_base + (int)(offs[k] & 0xffffffffull);
    }
    int slot[8];
    float4 clo[8], chi[8];
    float4 nlo = make_float4(3.0e38f, 3.0e38f, 3.0e38f, 0.0f), nhi = make_float4(-3.0e38f, -3.0e38f, -3.0e38f, 0.0f);
    for (int s = 0; s < 8; ++s) {
        slot[s] = plan[(size_t)cw * 8 + s];
        if (slot[s] < 0) continue;
        clo[s] = blo[slot[s]];
        chi[s] = bhi[slot[s]];
        pad_box_d(&clo[s], &chi[s]);
        nlo = vmin(nlo, clo[s]);
        nhi = vmax(nhi, chi[s]);
    }
    int ex[3];
    float sc[3];
    for (int a = 0; a < 3; ++a) {
        ex[a] = plane_exponent(comp(nhi, a) - comp(nlo, a));
        sc[a] = ldexpf(1.0f, ex[a]);
    }
    uint8_t meta[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    uint8_t qv[6][8];
    uint32_t imask = 0;
    int k_inner = 0, tri_off = 0;
    for (int s = 0; s < 8; ++s) {
        for (int a = 0; a < 6; ++a) qv[a][s] = 0;
        int c = slot[s];
        if (c < 0) continue;
        for (int a = 0; a < 3; ++a) {
            float o = comp(nlo, a), l = comp(clo[s], a), h = comp(chi[s], a);
            double dl = ((double)l - (double)o) / (double)sc[a];
            double dh = ((double)h - (double)o) / (double)sc[a];
            int ql = (int)fmax(0.0, fmin(255.0, floor(dl)));
            int qh = (int)fmax(0.0, fmin(255.0, ceil(dh)));
            while (ql > 0 && o + (float)ql * sc[a] > l) --ql;
            while (qh < 255 && o + (float)qh * sc[a] < h) ++qh;
            qv[a][s] = (uint8_t)ql;
            qv[3 + a][s] = (uint8_t)qh;
        }
        if (!bleaf[c]) {
            imask |= 1u << s;
            meta[s] = 0x20;
            int child = base_child + k_inner;
            if (child >= node_cap) { atomicExch(bad, 3); return; }
            if (!refit) q_next[child - next_base] = c;
            ++k_inner;
            continue;
        }
        // leaf: its triangles, left to right, from the binary subtree
        int st[8], sp = 0, cnt = 0;
        st[sp++] = c;
        while (sp > 0) {
            int x = st[--sp];
            int2 xc = bchild[x];
            if (x < n) {
                int t = ~xc.x, dst = base_tri + tri_off + cnt;
                if (cnt >= kLeafMax || dst >= n || t < 0 || t >= n) { atomicExch(bad, 3); return; }
                const float* p = pos + 9 * (size_t)t;
                tris[(size_t)dst * 3] = make_float4(p[0], p[1], p[2], __uint_as_float((uint32_t)t));
                tris[(size_t)dst * 3 + 1] = make_float4(p[3] - p[0], p[4] - p[1], p[5] - p[2], 0.0f);
                tris[(size_t)dst * 3 + 2] = make_float4(p[6] - p[0], p[7] - p[1], p[8] - p[2], 0.0f);
                ++cnt;
            } else {
                if (sp + 2 > 8) { atomicExch(bad, 3); return; }
                st[sp++] = xc.y;
                st[sp++] = xc.x;
            }
        }
        meta[s] = (uint8_t)((((1u << cnt) - 1u) << 5) | (uint32_t)tri_off);
        tri_off += cnt;
    }
    uint32_t w[20];
    w[0] = __float_as_uint(nlo.x);
    w[1] = __float_as_uint(nlo.y);
    w[2] = __float_as_uint(nlo.z);
    w[3] = (uint32_t)(ex[0] + 127) | ((uint32_t)(ex[1] + 127) << 8) | ((uint32_t)(ex[2] + 127) << 16) | (imask << 24);
    w[4] = (uint32_t)base_child;
    w[5] = (uint32_t)base_tri;
    w[6] = pack4(meta);
    w[7] = pack4(meta + 4);
    for (int a = 0; a < 3; ++a) {
        w[8 + 2 * a] = pack4(qv[a]);
        w[9 + 2 * a] = pack4(qv[a] + 4);
        w[14 + 2 * a] = pack4(qv[3 + a]);
        w[15 + 2 * a] = pack4(qv[3 + a] + 4);
    }
    for (int j = 0; j < 5; ++j)
        nodes[(size_t)cw * 5 + j] = make_uint4(w[4 * j], w[4 * j + 1], w[4 * j + 2], w[4 * j + 3]);
    if (!refit && k == m - 1) {
        unsigned long long f = flags[k], o = offs[k];
        *totals = make_int2((int)(o >> 32) + (int)(f >> 32), (int)(o & 0xffffffffull) + (int)(f & 0xffffffffull));
    }
}

inline int blocks_of(long long n, int b) { return (int)std::max(1ll, (n + b - 1) / b); }

// Frees the temporary buffers however the build ends.
struct TempGuard {
    DevAllocator& A;
    explicit TempGuard(DevAllocator& a) : A(a) {}
    ~TempGuard() { A.release_temps(); }
};

}  // namespace

#define GB_TRY(call)                              \
    do {                                          \
        cudaError_t e_ = (call);                  \
        if (e_ != cudaSuccess) return e_;         \
    } while (0)

cudaError_t gpu_build_cwbvh(const float* d_pos, int n, int radius, DevAllocator& A, GpuBvh* out,
                            std::string* err, cudaStream_t st, bool sah_collapse, float prim_cost) {
    TempGuard guard(A);
    *out = GpuBvh();
    if (n <= 0) { *err = "empty triangle list"; return cudaErrorInvalidValue; }
    if (n > (1 << 28)) { *err = "too many triangles"; return cudaErrorInvalidValue; }
    if (radius < 1 || radius > kMaxRadius) { *err = "clustering radius must be 1 .. 32"; return cudaErrorInvalidValue; }
    const size_t N2 = 2 * (size_t)n - 1;
    const int cap = std::max(1, n);  // 8-wide nodes: every node but a single-leaf root has >= 2 children
    GpuBvh& B = *out;
    B.n = n;
    // kept
    GB_TRY(A.alloc((void**)&B.blo, sizeof(float4) * N2, true));
    GB_TRY(A.alloc((void**)&B.bhi, sizeof(float4) * N2, true));
    GB_TRY(A.alloc((void**)&B.bchild, sizeof(int2) * N2, true));
    GB_TRY(A.alloc((void**)&B.bparent, sizeof(int) * N2, true));
    GB_TRY(A.alloc((void**)&B.bleaf, N2, true));
    GB_TRY(A.alloc((void**)&B.tris, sizeof(float4) * 3 * (size_t)n, true));
    // temporaries
    float4 *tlo, *thi, *clo[2], *chi[2];
    int *vals[2], *cnode[2], *nn, *bcount, *q[2], *plan_tmp, *bad;
    uint64_t* keys[2];
    unsigned *cb, *visit;
    unsigned long long *flags, *offs;
    int2* totals;
    uint4* nodes_tmp;
    GB_TRY(A.alloc((void**)&tlo, sizeof(float4) * n, false));
    GB_TRY(A.alloc((void**)&thi, sizeof(float4) * n, false));
    for (int k = 0; k < 2; ++k) {
        GB_TRY(A.alloc((void**)&clo[k], sizeof(float4) * n, false));
        GB_TRY(A.alloc((void**)&chi[k], sizeof(float4) * n, false));
        GB_TRY(A.alloc((void**)&cnode[k], sizeof(int) * n, false));
        GB_TRY(A.alloc((void**)&vals[k], sizeof(int) * n, false));
        GB_TRY(A.alloc((void**)&keys[k], sizeof(uint64_t) * n, false));
        GB_TRY(A.alloc((void**)&q[k], sizeof(int) * cap, false));
    }
    GB_TRY(A.alloc((void**)&nn, sizeof(int) * n, false));
    GB_TRY(A.alloc((void**)&flags, sizeof(unsigned long long) * n, false));
    GB_TRY(A.alloc((void**)&offs, sizeof(unsigned long long) * n, false));
    GB_TRY(A.alloc((void**)&bcount, sizeof(int) * N2, false));
    GB_TRY(A.alloc((void**)&visit, sizeof(unsigned) * N2, false));
    GB_TRY(A.alloc((void**)&plan_tmp, sizeof(int) * 8 * (size_t)cap, false));
    GB_TRY(A.alloc((void**)&nodes_tmp, sizeof(uint4) * 5 * (size_t)cap, false));
    GB_TRY(A.alloc((void**)&cb, sizeof(unsigned) * 8, false));
    GB_TRY(A.alloc((void**)&bad, sizeof(int) * 2, false));
    GB_TRY(A.alloc((void**)&totals, sizeof(int2) * 2, false));
    size_t sort_bytes = 0, scan_bytes = 0;
    GB_TRY(cub::DeviceRadixSort::SortPairs(nullptr, sort_bytes, keys[0], keys[1], vals[0], vals[1], n, 0, 63, st));
    GB_TRY(cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, flags, offs, n, st));
    size_t cub_bytes = std::max(sort_bytes, scan_bytes);
    void* cub_tmp;
    GB_TRY(A.alloc(&cub_tmp, cub_bytes, false));

    const int T = kBuildBlock;
    GB_TRY(cudaMemsetAsync(cb, 0xff, sizeof(unsigned) * 3, st));
    GB_TRY(cudaMemsetAsync(cb + 3, 0, sizeof(unsigned) * 3, st));
    GB_TRY(cudaMemsetAsync(bad, 0, sizeof(int) * 2, st));
    k_tri_prep<<<blocks_of(n, T), T, 0, st>>>(d_pos, n, tlo, thi, cb, bad);
    GB_TRY(cudaGetLastError());
    int h_bad = 0;
    GB_TRY(cudaMemcpyAsync(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
    GB_TRY(cudaStreamSynchronize(st));
    if (h_bad) { *err = "non-finite vertex"; return cudaErrorInvalidValue; }
    k_morton<<<blocks_of(n, T), T, 0, st>>>(tlo, thi, n, cb, keys[0], vals[0]);
    GB_TRY(cudaGetLastError());
    GB_TRY(cub::DeviceRadixSort::SortPairs(cub_tmp, cub_bytes, keys[0], keys[1], vals[0], vals[1], n, 0, 63, st));
    k_leaves<<<blocks_of(n, T), T, 0, st>>>(vals[1], tlo, thi, n, B.blo, B.bhi, B.bchild, B.bparent, clo[0], chi[0],
                                           cnode[0]);
    GB_TRY(cudaGetLastError());

    // clustering passes: each merges at least one pair (see k_ploc_nn)
    int m = n, next_inner = n, cur = 0;
    int2 h_tot{0, 0};
    while (m > 1) {
        if (B.iterations > n) { *err = "clustering did not converge"; return cudaErrorInvalidValue; }
        k_ploc_nn<<<blocks_of(m, T), T, 0, st>>>(clo[cur], chi[cur], m, radius, nn);
        k_ploc_flags<<<blocks_of(m, T), T, 0, st>>>(nn, m, flags);
        GB_TRY(cudaGetLastError());
        GB_TRY(cub::DeviceScan::ExclusiveSum(cub_tmp, cub_bytes, flags, offs, m, st));
        k_ploc_compact<<<blocks_of(m, T), T, 0, st>>>(nn, m, next_inner, offs, clo[cur], chi[cur], cnode[cur],
                                                     clo[cur ^ 1], chi[cur ^ 1], cnode[cur ^ 1], B.blo, B.bhi,
                                                     B.bchild, B.bparent, totals);
        GB_TRY(cudaGetLastError());
        GB_TRY(cudaMemcpyAsync(&h_tot, totals, sizeof(int2), cudaMemcpyDeviceToHost, st));
        GB_TRY(cudaStreamSynchronize(st));
        if (h_tot.y <= 0 || h_tot.x != m - h_tot.y) { *err = "clustering made no progress"; return cudaErrorInvalidValue; }
        next_inner += h_tot.y;
        m = h_tot.x;
        cur ^= 1;
        ++B.iterations;
    }
    if ((size_t)next_inner != N2) { *err = "clustering left an incomplete tree"; return cudaErrorInvalidValue; }
    const int root = next_inner - 1;
    B.binary_nodes = (int)N2;

    GB_TRY(cudaMemsetAsync(visit, 0, sizeof(unsigned) * N2, st));
    float* dcost = nullptr;
    int8_t *dhow = nullptr, *dsplit = nullptr;
    if (sah_collapse) {
        GB_TRY(A.alloc((void**)&dcost, sizeof(float) * 8 * N2, false));
        GB_TRY(A.alloc((void**)&dhow, 8 * N2, false));
        GB_TRY(A.alloc((void**)&dsplit, N2, false));
    }
    k_bottom_up<<<blocks_of(n, T), T, 0, st>>>(n, B.bparent, B.bchild, B.blo, B.bhi, bcount, B.bleaf, visit, d_pos, 0,
                                               bad, dcost, dhow, dsplit, prim_cost);
    GB_TRY(cudaGetLastError());

    // collapse, one level of 8-wide nodes per pass
    int node_base = 0, tri_base = 0, level = 1;
    cur = 0;
    GB_TRY(cudaMemcpyAsync(q[0], &root, sizeof(int), cudaMemcpyHostToDevice, st));
    m = 1;
    while (m > 0) {
        int next_base = node_base + m;
        if (next_base > cap) { *err = "8-wide node count out of range"; return cudaErrorInvalidValue; }
        k_collapse_plan<<<blocks_of(m, T), T, 0, st>>>(q[cur], m, node_base, B.blo, B.bhi, B.bchild, B.bleaf, bcount,
                                                      plan_tmp, flags, dhow, dsplit, n);
        GB_TRY(cudaGetLastError());
        GB_TRY(cub::DeviceScan::ExclusiveSum(cub_tmp, cub_bytes, flags, offs, m, st));
        k_collapse_emit<<<blocks_of(m, T), T, 0, st>>>(plan_tmp, m, node_base, next_base, tri_base, offs, flags, B.blo,
                                                      B.bhi, B.bchild, B.bleaf, n, d_pos, nodes_tmp, B.tris,
                                                      q[cur ^ 1], cap, totals, 0, bad);
        GB_TRY(cudaGetLastError());
        int hb[2] = {0, 0};
        GB_TRY(cudaMemcpyAsync(&h_tot, totals, sizeof(int2), cudaMemcpyDeviceToHost, st));
        GB_TRY(cudaMemcpyAsync(hb, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
        GB_TRY(cudaStreamSynchronize(st));
        if (hb[0]) { *err = hb[0] == 2 ? "cycle in the binary tree" : "collapse index out of range"; return cudaErrorInvalidValue; }
        B.depth = level;
        node_base = next_base;
        tri_base += h_tot.y;
        m = h_tot.x;
        cur ^= 1;
        ++level;
        if (B.depth > kMaxStack) { *err = "8-wide tree deeper than the traversal stack"; return cudaErrorInvalidValue; }
    }
    if (tri_base != n) { *err = "collapse lost triangles"; return cudaErrorInvalidValue; }
    B.n_nodes = node_base;
    B.n_tris = n;
    GB_TRY(A.alloc((void**)&B.nodes, sizeof(uint4) * 5 * (size_t)B.n_nodes, true));
    GB_TRY(A.alloc((void**)&B.plan, sizeof(int) * 8 * (size_t)B.n_nodes, true));
    GB_TRY(cudaMemcpyAsync(B.nodes, nodes_tmp, sizeof(uint4) * 5 * (size_t)B.n_nodes, cudaMemcpyDeviceToDevice, st));
    GB_TRY(cudaMemcpyAsync(B.plan, plan_tmp, sizeof(int) * 8 * (size_t)B.n_nodes, cudaMemcpyDeviceToDevice, st));
    // the structure is checked on the host before any traversal reads it
    CwBvh chk;
    chk.n_nodes = B.n_nodes;
    chk.n_tris = n;
    chk.nodes.resize((size_t)B.n_nodes * kNodeWords);
    GB_TRY(cudaMemcpyAsync(chk.nodes.data(), B.nodes, sizeof(uint32_t) * chk.nodes.size(), cudaMemcpyDeviceToHost, st));
    GB_TRY(cudaStreamSynchronize(st));
    if (!validate_cwbvh(chk, err)) return cudaErrorInvalidValue;
    B.device_bytes = (sizeof(float4) * 2 + sizeof(int2) + sizeof(int) + 1) * N2 + sizeof(float4) * 3 * (size_t)n +
                     (sizeof(uint4) * 5 + sizeof(int) * 8) * (size_t)B.n_nodes;
    return cudaSuccess;
}

cudaError_t gpu_refit_cwbvh(const float* d_pos, DevAllocator& A, GpuBvh* bvh, std::string* err, cudaStream_t st) {
    TempGuard guard(A);
    GpuBvh& B = *bvh;
    const int n = B.n;
    if (n <= 0 || !B.nodes || !B.plan) { *err = "no device-built tree to refit"; return cudaErrorInvalidValue; }
    const size_t N2 = 2 * (size_t)n - 1;
    float4 *tlo, *thi;
    unsigned *cb, *visit;
    int* bad;
    GB_TRY(A.alloc((void**)&tlo, sizeof(float4) * n, false));
    GB_TRY(A.alloc((void**)&thi, sizeof(float4) * n, false));
    GB_TRY(A.alloc((void**)&cb, sizeof(unsigned) * 8, false));
    GB_TRY(A.alloc((void**)&visit, sizeof(unsigned) * N2, false));
    GB_TRY(A.alloc((void**)&bad, sizeof(int) * 2, false));
    const int T = kBuildBlock;
    GB_TRY(cudaMemsetAsync(cb, 0xff, sizeof(unsigned) * 3, st));
    GB_TRY(cudaMemsetAsync(cb + 3, 0, sizeof(unsigned) * 3, st));
    GB_TRY(cudaMemsetAsync(bad, 0, sizeof(int) * 2, st));
    k_tri_prep<<<blocks_of(n, T), T, 0, st>>>(d_pos, n, tlo, thi, cb, bad);
    GB_TRY(cudaGetLastError());
    int h_bad = 0;
    GB_TRY(cudaMemcpyAsync(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
    GB_TRY(cudaStreamSynchronize(st));
    if (h_bad) { *err = "non-finite vertex"; return cudaErrorInvalidValue; }
    GB_TRY(cudaMemsetAsync(visit, 0, sizeof(unsigned) * N2, st));
    k_bottom_up<<<blocks_of(n, T), T, 0, st>>>(n, B.bparent, B.bchild, B.blo, B.bhi, nullptr, nullptr, visit, d_pos, 1,
                                               bad, nullptr, nullptr, nullptr, 0.0f);
    GB_TRY(cudaGetLastError());
    k_collapse_emit<<<blocks_of(B.n_nodes, T), T, 0, st>>>(B.plan, B.n_nodes, 0, 0, 0, nullptr, nullptr, B.blo, B.bhi,
                                                          B.bchild, B.bleaf, n, d_pos, (uint4*)B.nodes, B.tris,
                                                          nullptr, B.n_nodes, nullptr, 1, bad);
    GB_TRY(cudaGetLastError());
    GB_TRY(cudaMemcpyAsync(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
    GB_TRY(cudaStreamSynchronize(st));
    if (h_bad) { *err = h_bad == 2 ? "cycle in the binary tree" : "refit index out of range"; return cudaErrorInvalidValue; }
    return cudaSuccess;
}

}  // namespace gb
