// gbpt_build.h -- BVH construction on the device.
//
// The reference builds its BVH on the host with rta's binned-SAH builder
// (`-b bsah`, hl-main.cpp:375-385); gbpt_bvh.cpp does the same.  This builder
// runs on the GPU: triangles are ordered along a 63-bit Morton curve of
// their centroids, a binary tree is formed by Parallel Locally-Ordered
// Clustering (Meister & Bittner, "Parallel Locally-Ordered Clustering for
// Bounding Volume Hierarchy Construction", IEEE TVCG 2018), and the tree is
// collapsed level by level into the compressed 8-wide nodes the traversal
// kernels read.  The collapse applies the host builder's rules (the
// SAH-optimal grouping of binary nodes into wide nodes, or the greedy one;
// octant slot order, box padding and 8-bit quantisation), so for a given
// binary tree it writes the nodes the host collapse would write; only the
// node numbering differs (level order).
//
// The binary tree and the 8-wide grouping are kept, so a scene whose
// vertices move can be refitted: boxes are recomputed bottom-up and the
// nodes re-quantised in place, with no change of topology.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

namespace gb {

// Device allocations of a build.  `keep` buffers belong to the scene and
// live as long as it does; the others are freed by release_temps(), which
// the builder calls before it returns.
struct DevAllocator {
    virtual cudaError_t alloc(void** p, size_t bytes, bool keep) = 0;
    virtual void release_temps() = 0;
    virtual ~DevAllocator() {}
};

struct GpuBvh {
    // the tree the traversal kernels read (kNodeWords / kTriWords layout of
    // gbpt_bvh.h), both allocated with keep = true
    float4* nodes = nullptr;
    float4* tris = nullptr;
    int n_nodes = 0, n_tris = 0, depth = 0, binary_nodes = 0;
    int iterations = 0;            // clustering passes
    // kept for refits
    int n = 0;                     // triangles
    float4* blo = nullptr;         // binary node boxes (2n - 1); leaves 0 .. n-1 in Morton order
    float4* bhi = nullptr;
    int2* bchild = nullptr;        // inner: (left, right); leaf: (~triangle, -1)
    int* bparent = nullptr;        // -1 at the root
    uint8_t* bleaf = nullptr;      // 1 where a binary node is stored as one leaf
    int* plan = nullptr;           // 8 binary nodes per 8-wide node, in slot order (-1 = empty)
    size_t device_bytes = 0;       // bytes of the kept buffers
};

// Builds the tree of the n triangles at d_pos (9 floats each, device
// memory) on stream st.  radius: clustering search radius (1 .. 32).
// sah_collapse: group binary nodes into 8-wide nodes by the SAH-optimal
// dynamic programme (node visit 1, triangle test prim_cost) instead of the
// host collapser's greedy rules.
// Returns cudaErrorInvalidValue with *err set for bad input (non-finite
// vertex, tree deeper than the traversal stack), any other error for CUDA
// failures.  The stream is synchronised on return.
cudaError_t gpu_build_cwbvh(const float* d_pos, int n, int radius, DevAllocator& A, GpuBvh* out,
                            std::string* err, cudaStream_t st, bool sah_collapse = false, float prim_cost = 1.2f);

// Recomputes the boxes of a built tree for moved vertices (same triangle
// count and order) and rewrites nodes and triangle records in place.
cudaError_t gpu_refit_cwbvh(const float* d_pos, DevAllocator& A, GpuBvh* bvh, std::string* err,
                            cudaStream_t st);

}  // namespace gb
