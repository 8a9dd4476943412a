// gbpt_bvh.cpp -- binned-SAH binary BVH + collapse to compressed 8-wide nodes.
#include "gbpt_bvh.h"

#include <algorithm>
#include <array>
#include <chrono>
#include <memory>
#include <cmath>
#include <cstring>

namespace gb {

namespace {

struct Box {
    float lo[3], hi[3];
    void empty() {
        for (int a = 0; a < 3; ++a) { lo[a] = 3.0e38f; hi[a] = -3.0e38f; }
    }
    void grow(const Box& b) {
        for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], b.lo[a]); hi[a] = std::max(hi[a], b.hi[a]); }
    }
    void grow(const float* p) {
        for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], p[a]); hi[a] = std::max(hi[a], p[a]); }
    }
    float area() const {
        float d[3];
        for (int a = 0; a < 3; ++a) d[a] = std::max(0.0f, hi[a] - lo[a]);
        return 2.0f * (d[0] * d[1] + d[1] * d[2] + d[2] * d[0]);
    }
};

struct BNode {
    Box box;
    int left = -1, right = -1;  // children (inner)
    int first = 0, count = 0;   // primitive range in `order` (leaf when count > 0)
};

struct Builder {
    const std::vector<Box>& tb;
    const std::vector<float>& cen;  // 3 per triangle
    std::vector<int>& order;
    std::vector<BNode> nodes;
    static const int kMaxBins = 64;
    int nbins = 32;  // SAH bins per axis and node
    static const int kMaxLeaf = 3;

    Builder(const std::vector<Box>& tb_, const std::vector<float>& cen_, std::vector<int>& order_)
        : tb(tb_), cen(cen_), order(order_) {}

    // Builds the subtree of order[b, e) into `out`; returns its root index.
    int build(std::vector<BNode>& out, int b, int e) {
        BNode node;
        node.box.empty();
        Box cb; cb.empty();
        for (int i = b; i < e; ++i) { node.box.grow(tb[order[i]]); cb.grow(&cen[3 * order[i]]); }
        int count = e - b;
        int me = (int)out.size();
        out.push_back(node);
        if (count == 1) { out[me].first = b; out[me].count = 1; return me; }

        // binned SAH over the centroid bounds
        float best_cost = 3.0e38f; int best_axis = -1, best_split = -1;
        for (int a = 0; a < 3; ++a) {
            float ext = cb.hi[a] - cb.lo[a];
            if (!(ext > 0.0f)) continue;
            Box bins[kMaxBins]; int cnt[kMaxBins];
            for (int k = 0; k < nbins; ++k) { bins[k].empty(); cnt[k] = 0; }
            float scale = (float)nbins * (1.0f - 1e-6f) / ext;
            for (int i = b; i < e; ++i) {
                int t = order[i];
                int k = std::min(nbins - 1, (int)((cen[3 * t + a] - cb.lo[a]) * scale));
                bins[k].grow(tb[t]); cnt[k]++;
            }
            float rarea[kMaxBins]; int rcnt[kMaxBins];
            Box acc; acc.empty(); int c = 0;
            for (int k = nbins - 1; k > 0; --k) { acc.grow(bins[k]); c += cnt[k]; rarea[k] = acc.area(); rcnt[k] = c; }
            acc.empty(); c = 0;
            for (int k = 0; k < nbins - 1; ++k) {
                acc.grow(bins[k]); c += cnt[k];
                if (c == 0 || rcnt[k + 1] == 0) continue;
                float cost = acc.area() * c + rarea[k + 1] * rcnt[k + 1];
                if (cost < best_cost) { best_cost = cost; best_axis = a; best_split = k; }
            }
        }
        float parea = node.box.area();
        float leaf_cost = (float)count;
        float split_cost = 0.5f + (parea > 0.0f ? best_cost / parea : 0.0f);
        if (count <= kMaxLeaf && (best_axis < 0 || leaf_cost <= split_cost)) {
            out[me].first = b; out[me].count = count; return me;
        }
        int mid;
        if (best_axis < 0) {
            mid = b + count / 2;  // all centroids coincide: split the range
        } else {
            float ext = cb.hi[best_axis] - cb.lo[best_axis];
            float scale = (float)nbins * (1.0f - 1e-6f) / ext;
            int* p = std::partition(order.data() + b, order.data() + e, [&](int t) {
                int k = std::min(nbins - 1, (int)((cen[3 * t + best_axis] - cb.lo[best_axis]) * scale));
                return k <= best_split;
            });
            mid = (int)(p - order.data());
            if (mid == b || mid == e) mid = b + count / 2;
        }
        int l = build(out, b, mid);
        int r = build(out, mid, e);
        out[me].left = l; out[me].right = r;
        return me;
    }
};

void pad_box(Box& b) {
    float m = 0.0f;
    for (int a = 0; a < 3; ++a) m = std::max(m, std::max(std::fabs(b.lo[a]), std::fabs(b.hi[a])));
    float d = m * (1.0f / 524288.0f) + 1e-30f;  // 2^-19 of the magnitude
    for (int a = 0; a < 3; ++a) { b.lo[a] -= d; b.hi[a] += d; }
}

inline uint32_t fbits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }

// SAH-optimal grouping of a binary tree into 8-wide nodes (Ylitie, Karras &
// Laine 2017, section 4.1): cost[n][i] is the least SAH cost of the subtree
// of binary node n as at most i slots of its wide parent; one slot is a leaf
// (at most kLeafTris triangles, cost A * p * prim_cost) or a wide node (cost
// A * node_cost + the best split of 8 slots between the two children).
struct WideDp {
    static const int kLeafTris = 3;
    const std::vector<BNode>& bn;
    double node_cost, prim_cost;
    std::vector<int> prims;                 // triangles under each binary node
    std::vector<std::array<double, 9>> cost;
    std::vector<std::array<int8_t, 9>> how;  // i: 0 fewer slots, k > 0 left gets k; i = 1: 1 leaf, 2 wide node
    std::vector<int8_t> split8;              // best split of 8 slots (wide node)
    WideDp(const std::vector<BNode>& bn_, double nc, double pc) : bn(bn_), node_cost(nc), prim_cost(pc) {
        const int n = (int)bn.size();
        prims.assign(n, 0);
        cost.assign(n, {});
        how.assign(n, {});
        split8.assign(n, 0);
        // children come after their parent in `bn`: a reverse sweep is post-order
        for (int v = n - 1; v >= 0; --v) {
            const BNode& b = bn[v];
            const double A = b.box.area();
            if (b.count > 0) {
                prims[v] = b.count;
                for (int i = 1; i <= 8; ++i) { cost[v][i] = A * b.count * prim_cost; how[v][i] = i == 1 ? 1 : 0; }
                continue;
            }
            const int l = b.left, r = b.right;
            prims[v] = prims[l] + prims[r];
            double dist[9];
            int8_t dk[9];
            for (int j = 2; j <= 8; ++j) {
                dist[j] = 1e300;
                dk[j] = 1;
                for (int k = 1; k < j; ++k) {
                    double c = cost[l][k] + cost[r][j - k];
                    if (c < dist[j]) { dist[j] = c; dk[j] = (int8_t)k; }
                }
            }
            split8[v] = dk[8];
            const double wide = A * node_cost + dist[8];
            const double leaf = prims[v] <= kLeafTris ? A * prims[v] * prim_cost : 1e300;
            cost[v][1] = leaf <= wide ? leaf : wide;
            how[v][1] = leaf <= wide ? 1 : 2;
            for (int i = 2; i <= 8; ++i) {
                if (dist[i] < cost[v][i - 1]) { cost[v][i] = dist[i]; how[v][i] = dk[i]; }
                else { cost[v][i] = cost[v][i - 1]; how[v][i] = 0; }
            }
        }
    }
    // Slots of the subtree of v given at most i of them: (binary node, leaf?).
    void collect(int v, int i, std::vector<std::pair<int, bool>>* out) const {
        while (i > 1 && how[v][i] == 0) --i;
        if (i == 1 || bn[v].count > 0) {
            out->push_back(std::make_pair(v, bn[v].count > 0 || how[v][1] == 1));
            return;
        }
        const int k = how[v][i];
        collect(bn[v].left, k, out);
        collect(bn[v].right, i - k, out);
    }
    // Children of the wide node made from binary node v.
    void children(int v, std::vector<std::pair<int, bool>>* out) const {
        if (bn[v].count > 0) { out->push_back(std::make_pair(v, true)); return; }
        collect(bn[v].left, split8[v], out);
        collect(bn[v].right, 8 - split8[v], out);
    }
};

struct Collapser {
    const std::vector<BNode>& bn;
    const std::vector<int>& order;
    const float* pos;
    CwBvh& out;
    int max_depth = 0;
    const WideDp* dp = nullptr;  // SAH-optimal grouping; greedy largest-area expansion without it
    Collapser(const std::vector<BNode>& bn_, const std::vector<int>& order_, const float* pos_, CwBvh& out_)
        : bn(bn_), order(order_), pos(pos_), out(out_) {}

    // Triangles under binary node v, left to right.
    void subtree_tris(int v, std::vector<int>* t) const {
        if (bn[v].count > 0) {
            for (int j = 0; j < bn[v].count; ++j) t->push_back(order[bn[v].first + j]);
            return;
        }
        subtree_tris(bn[v].left, t);
        subtree_tris(bn[v].right, t);
    }

    void emit_tri(int t) {
        const float* a = pos + 9 * t;
        float v0[3] = {a[0], a[1], a[2]};
        float e1[3] = {a[3] - a[0], a[4] - a[1], a[5] - a[2]};
        float e2[3] = {a[6] - a[0], a[7] - a[1], a[8] - a[2]};
        float w[12];
        w[0] = v0[0]; w[1] = v0[1]; w[2] = v0[2];
        uint32_t id = (uint32_t)t; std::memcpy(&w[3], &id, 4);
        w[4] = e1[0]; w[5] = e1[1]; w[6] = e1[2]; w[7] = 0.0f;
        w[8] = e2[0]; w[9] = e2[1]; w[10] = e2[2]; w[11] = 0.0f;
        out.tris.insert(out.tris.end(), w, w + 12);
    }

    // Fills 8-wide node `ci` from binary node `b`.
    void fill(int ci, int b, int depth) {
        max_depth = std::max(max_depth, depth);
        std::vector<int> ch;
        std::vector<bool> is_leaf;
        if (dp) {
            std::vector<std::pair<int, bool>> slots;
            dp->children(b, &slots);
            for (const auto& s : slots) { ch.push_back(s.first); is_leaf.push_back(s.second); }
        } else {
            if (bn[b].count > 0) ch.push_back(b);
            else { ch.push_back(bn[b].left); ch.push_back(bn[b].right); }
            while ((int)ch.size() < 8) {
                int best = -1; float ba = -1.0f;
                for (int i = 0; i < (int)ch.size(); ++i)
                    if (bn[ch[i]].count == 0 && bn[ch[i]].box.area() > ba) { ba = bn[ch[i]].box.area(); best = i; }
                if (best < 0) break;
                int x = ch[best];
                ch[best] = bn[x].left;
                ch.push_back(bn[x].right);
            }
            for (int c : ch) is_leaf.push_back(bn[c].count > 0);
        }
        int nc = (int)ch.size();
        // padded child boxes and their union
        Box cbx[8]; Box nb; nb.empty();
        for (int i = 0; i < nc; ++i) { cbx[i] = bn[ch[i]].box; pad_box(cbx[i]); nb.grow(cbx[i]); }
        float ncen[3];
        for (int a = 0; a < 3; ++a) ncen[a] = 0.5f * (nb.lo[a] + nb.hi[a]);
        // octant slot assignment: slot s is visited first by rays whose
        // direction signs equal the bits of s; put there the child that is
        // most "upstream" for that direction (greedy on dot(centroid, d_s)).
        int slot_of[8]; bool used_slot[8] = {false}, used_ch[8] = {false};
        float cost[8][8];
        for (int i = 0; i < nc; ++i)
            for (int s = 0; s < 8; ++s) {
                float c = 0.0f;
                for (int a = 0; a < 3; ++a) {
                    float cc = 0.5f * (cbx[i].lo[a] + cbx[i].hi[a]) - ncen[a];
                    c += ((s >> a) & 1) ? -cc : cc;
                }
                cost[i][s] = c;
            }
        for (int it = 0; it < nc; ++it) {
            float bc = 3.0e38f; int bi = -1, bs = -1;
            for (int i = 0; i < nc; ++i) if (!used_ch[i])
                for (int s = 0; s < 8; ++s) if (!used_slot[s] && cost[i][s] < bc) { bc = cost[i][s]; bi = i; bs = s; }
            used_ch[bi] = true; used_slot[bs] = true; slot_of[bi] = bs;
        }
        int child_at[8];
        for (int s = 0; s < 8; ++s) child_at[s] = -1;
        for (int i = 0; i < nc; ++i) child_at[slot_of[i]] = i;

        // quantisation grid
        int ex[3]; float sc[3];
        for (int a = 0; a < 3; ++a) {
            float ext = nb.hi[a] - nb.lo[a];
            int e = -100;
            if (ext > 0.0f) {
                e = (int)std::ceil(std::log2((double)ext / 255.0));
                while (std::ldexp(255.0, e) < (double)ext) ++e;
                if (e < -100) e = -100;
            }
            ex[a] = e; sc[a] = std::ldexp(1.0f, e);
        }
        uint32_t* w = &out.nodes[(size_t)ci * kNodeWords];
        std::memset(w, 0, sizeof(uint32_t) * kNodeWords);
        w[0] = fbits(nb.lo[0]); w[1] = fbits(nb.lo[1]); w[2] = fbits(nb.lo[2]);
        uint32_t imask = 0;
        for (int s = 0; s < 8; ++s)
            if (child_at[s] >= 0 && !is_leaf[child_at[s]]) imask |= 1u << s;
        w[3] = (uint32_t)(ex[0] + 127) | ((uint32_t)(ex[1] + 127) << 8) | ((uint32_t)(ex[2] + 127) << 16) | (imask << 24);
        uint8_t meta[8] = {0};
        uint8_t q[6][8] = {{0}};
        // inner children: contiguous block in slot order
        int n_inner = __builtin_popcount(imask);
        int base_child = out.n_nodes;
        out.n_nodes += n_inner;
        out.nodes.resize((size_t)out.n_nodes * kNodeWords);
        w = &out.nodes[(size_t)ci * kNodeWords];
        int base_tri = (int)(out.tris.size() / kTriWords);
        int tri_off = 0;
        std::vector<std::pair<int, int>> todo;  // (cw index, binary node)
        int k_inner = 0;
        for (int s = 0; s < 8; ++s) {
            int i = child_at[s];
            if (i < 0) continue;
            int c = ch[i];
            for (int a = 0; a < 3; ++a) {
                double lo = ((double)cbx[i].lo[a] - (double)nb.lo[a]) / (double)sc[a];
                double hi = ((double)cbx[i].hi[a] - (double)nb.lo[a]) / (double)sc[a];
                int ql = (int)std::floor(lo), qh = (int)std::ceil(hi);
                ql = std::max(0, std::min(255, ql)); qh = std::max(0, std::min(255, qh));
                while (ql > 0 && nb.lo[a] + (float)ql * sc[a] > cbx[i].lo[a]) --ql;
                while (qh < 255 && nb.lo[a] + (float)qh * sc[a] < cbx[i].hi[a]) ++qh;
                q[a][s] = (uint8_t)ql; q[3 + a][s] = (uint8_t)qh;
            }
            if (!is_leaf[i]) {
                meta[s] = 0x20;
                todo.push_back(std::make_pair(base_child + k_inner, c));
                ++k_inner;
            } else {
                std::vector<int> tl;
                subtree_tris(c, &tl);
                int cnt = (int)tl.size();
                meta[s] = (uint8_t)((((1u << cnt) - 1u) << 5) | (uint32_t)tri_off);
                for (int t : tl) emit_tri(t);
                tri_off += cnt;
            }
        }
        w = &out.nodes[(size_t)ci * kNodeWords];
        w[4] = (uint32_t)base_child;
        w[5] = (uint32_t)base_tri;
        std::memcpy(&w[6], meta, 8);
        for (int a = 0; a < 3; ++a) {
            std::memcpy(&w[8 + 2 * a], q[a], 8);
            std::memcpy(&w[14 + 2 * a], q[3 + a], 8);
        }
        for (auto& t : todo) fill(t.first, t.second, depth + 1);
    }
};

}  // namespace

bool build_cwbvh(const float* pos, int n, CwBvh* out, std::string* err, const WideCollapse* wide) {
    auto t0 = std::chrono::steady_clock::now();
    *out = CwBvh();
    if (n <= 0) { *err = "empty triangle list"; return false; }
    std::vector<Box> tb(n);
    std::vector<float> cen(3 * (size_t)n);
    for (int t = 0; t < n; ++t) {
        Box b; b.empty();
        for (int k = 0; k < 9; ++k)  // min/max would drop a NaN coordinate silently
            if (!std::isfinite(pos[9 * (size_t)t + k])) { *err = "non-finite vertex"; return false; }
        for (int v = 0; v < 3; ++v) b.grow(pos + 9 * (size_t)t + 3 * v);
        for (int a = 0; a < 3; ++a) cen[3 * (size_t)t + a] = 0.5f * (b.lo[a] + b.hi[a]);
        tb[t] = b;
    }
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    Builder B(tb, cen, order);
    if (wide && wide->bins > 0) B.nbins = std::min(wide->bins, (int)Builder::kMaxBins);
    std::vector<BNode> bn;
    bn.reserve(2 * (size_t)n);
    B.build(bn, 0, n);
    out->binary_nodes = (int)bn.size();
    out->n_nodes = 1;
    out->nodes.assign(kNodeWords, 0);
    out->tris.reserve((size_t)n * kTriWords);
    Collapser C(bn, order, pos, *out);
    std::unique_ptr<WideDp> dp;
    if (wide && wide->sah) {
        dp.reset(new WideDp(bn, 1.0, wide->prim_cost > 0.0 ? wide->prim_cost : 1.2));
        C.dp = dp.get();
    }
    C.fill(0, 0, 1);
    out->n_tris = (int)(out->tris.size() / kTriWords);
    out->depth = C.max_depth;
    auto t1 = std::chrono::steady_clock::now();
    out->build_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    if (out->depth > kMaxStack) { *err = "8-wide tree deeper than the traversal stack"; return false; }
    return validate_cwbvh(*out, err);
}

bool validate_cwbvh(const CwBvh& b, std::string* err) {
    if ((int)b.nodes.size() != b.n_nodes * kNodeWords) { *err = "node array size mismatch"; return false; }
    std::vector<uint8_t> seen(b.n_tris, 0);
    std::vector<uint8_t> node_ref(b.n_nodes, 0);
    node_ref[0] = 1;
    for (int i = 0; i < b.n_nodes; ++i) {
        const uint32_t* w = &b.nodes[(size_t)i * kNodeWords];
        uint32_t imask = w[3] >> 24;
        uint32_t base_child = w[4], base_tri = w[5];
        uint8_t meta[8]; std::memcpy(meta, &w[6], 8);
        int n_inner = __builtin_popcount(imask);
        if (n_inner > 0 && (uint64_t)base_child + n_inner > (uint64_t)b.n_nodes) { *err = "child index out of range"; return false; }
        for (int k = 0; k < n_inner; ++k) {
            if (base_child + k == 0 || node_ref[base_child + k]) { *err = "node referenced twice"; return false; }
            node_ref[base_child + k] = 1;
        }
        for (int s = 0; s < 8; ++s) {
            bool inner = (imask >> s) & 1;
            if (inner) { if (meta[s] == 0) { *err = "inner child without meta"; return false; } continue; }
            if (meta[s] == 0) continue;
            uint32_t bits = meta[s] >> 5, off = meta[s] & 31;
            int cnt = bits == 1 ? 1 : bits == 3 ? 2 : bits == 7 ? 3 : -1;
            if (cnt < 0 || off + cnt > 24) { *err = "bad leaf meta"; return false; }
            for (int j = 0; j < cnt; ++j) {
                uint64_t t = (uint64_t)base_tri + off + j;
                if (t >= (uint64_t)b.n_tris) { *err = "triangle index out of range"; return false; }
                if (seen[t]) { *err = "triangle referenced twice"; return false; }
                seen[t] = 1;
            }
        }
    }
    for (int t = 0; t < b.n_tris; ++t) if (!seen[t]) { *err = "unreferenced triangle"; return false; }
    for (int i = 0; i < b.n_nodes; ++i) if (!node_ref[i]) { *err = "unreferenced node"; return false; }
    return true;
}

}  // namespace gb
