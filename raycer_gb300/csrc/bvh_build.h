// Host-side SAH flat BVH builder for triangle scenes.
//
// Produces the same preorder node array and primitive order as the
// reference's FlatBVH::build (src/Raytracing/Primitives/FlatBVH.cpp:89-343)
// with BVHBuildInfo { useSAH = true, regularSAHSplits = 0 } — the
// reference's defaults (FlatBVH.h:19-36). Same split candidates, same
// scores and tie-breaks, same in-place swap partition, same half-split
// fallback; so a traversal in the reference's order visits the same leaves
// in the same order and breaks distance ties the same way.
//
// What differs is only how the work is scheduled: the centroid median is
// found with a selection instead of a full sort (same value), and sibling
// subtrees below a size threshold are built in parallel and spliced into
// preorder afterwards.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace rcx
{

struct BuildNode
{
    double bmin[3];
    double bmax[3];
    int64_t rightOffset;  // 0 for a leaf, else (right child index - own index)
    uint64_t start;       // first primitive (into `order`)
    uint64_t count;       // primitive count of the subtree
};

struct BuildResult
{
    std::vector<BuildNode> nodes;  // preorder
    std::vector<uint32_t> order;   // order[i] = caller index of the i-th primitive
    uint32_t depth = 0;            // nodes on the longest root-to-leaf path
};

// vertices: n * 9 doubles (v0, v1, v2 per triangle).
// Returns false and sets `error` on invalid input.
bool buildFlatBVH(const double* vertices, int64_t n, uint32_t maxLeafSize, int threads, BuildResult& out,
                  std::string& error);

}  // namespace rcx
