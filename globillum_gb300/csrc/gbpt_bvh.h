// gbpt_bvh.h -- host BVH construction for the GB300 traversal kernels.
//
// The reference builds a binary BVH on the host with rta's binned-SAH
// builder (`-b bsah`, hl-main.cpp:375-385) and traverses 2 x float4 nodes
// (tracers.cu:26-36).  Here the binary binned-SAH tree is collapsed into
// compressed 8-wide nodes (5 x float4 = 80 B, child boxes quantised to 8
// bits per plane against a per-node origin and power-of-two scale, after
// Ylitie, Karras & Laine, "Efficient Incoherent Ray Traversal on GPUs
// Through Compressed Wide BVHs", HPG 2017).  Triangles are stored in leaf
// order as 3 x float4 (v0 | canonical id, e1, e2).
#pragma once
#include <stdint.h>
#include <string>
#include <vector>

namespace gb {

// Node layout (20 x 32-bit words):
//  w0-2  origin p (float)            w3  bytes: ex, ey, ez (biased exp), imask
//  w4    base child node index       w5  base triangle index
//  w6-7  meta[8] (0 = empty; leaf: unary(count)<<5 | tri offset; inner: 0x20)
//  w8-9  qlo_x[8]  w10-11 qlo_y[8]  w12-13 qlo_z[8]
//  w14-15 qhi_x[8] w16-17 qhi_y[8]  w18-19 qhi_z[8]
static const int kNodeWords = 20;
static const int kTriWords = 12;
static const int kMaxStack = 32;

struct CwBvh {
    std::vector<uint32_t> nodes;   // kNodeWords per node
    std::vector<float> tris;       // kTriWords per triangle, leaf order
    int n_nodes = 0;
    int n_tris = 0;
    int depth = 0;                 // levels of 8-wide nodes (<= kMaxStack required)
    int binary_nodes = 0;
    double build_ms = 0.0;
};

// How binary nodes are grouped into 8-wide nodes: greedily (the child of
// largest area is opened until 8) or by the SAH-optimal dynamic programme
// over slot counts, with a node visit costing 1 and a triangle test
// prim_cost (0 = 1.2).
struct WideCollapse {
    bool sah = false;
    double prim_cost = 0.0;
    int bins = 0;  // binned-SAH bins per axis of the binary build (0 = 32, at most 64)
};

// pos: 9 floats per triangle (a, b, c) in canonical order.  Returns false
// and fills err on failure (too deep, degenerate extents).
bool build_cwbvh(const float* pos, int n, CwBvh* out, std::string* err, const WideCollapse* wide = nullptr);

// Consistency check of a built tree (child / triangle ranges in bounds,
// every triangle referenced once).  Used before any upload.
bool validate_cwbvh(const CwBvh& b, std::string* err);

}  // namespace gb
