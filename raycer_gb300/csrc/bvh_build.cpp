// Host-side SAH flat BVH builder (see bvh_build.h for the contract).
//
// The per-node decision procedure restates FlatBVH::build /
// calculateSAHSplit / calculateSAHScore / calculateMedianPoint
// (src/Raytracing/Primitives/FlatBVH.cpp:89-343) operation for operation in
// float64, because the node array and primitive order must come out
// identical to the reference's:
//   * node box   = union of the triangles' vertex boxes (AABB::expand).
//   * leaf       <=> count <= maxLeafSize.
//   * candidates = for axis 0, 1, 2: { node box centre, centroid median };
//                  the first strictly lowest score wins.
//   * score      = sum over non-empty sides of (SA(side) / SA(node)) * count.
//   * partition  = one forward pass that swaps every primitive whose centroid
//                  is <= split to the front (the reference's std::swap loop).
//   * fallback   = split the range in half (no sort) if one side is empty.
//   * numbering  = preorder, left child first.
// Subtrees are built into a pointer tree (sibling subtrees as OpenMP tasks)
// and flattened to preorder at the end.

#include "bvh_build.h"

#include <algorithm>
#include <cmath>
#include <limits>
#include <memory>

#include <omp.h>

namespace rcx
{
namespace
{

struct Box
{
    double mn[3] = { std::numeric_limits<double>::max(), std::numeric_limits<double>::max(),
                     std::numeric_limits<double>::max() };
    double mx[3] = { std::numeric_limits<double>::lowest(), std::numeric_limits<double>::lowest(),
                     std::numeric_limits<double>::lowest() };

    void expand(const double* omn, const double* omx)
    {
        for (int k = 0; k < 3; ++k)
        {
            mn[k] = std::min(mn[k], omn[k]);
            mx[k] = std::max(mx[k], omx[k]);
        }
    }

    // AABB::getSurfaceArea (AABB.cpp:139-143): same expression order.
    double area() const
    {
        double ex = mx[0] - mn[0];
        double ey = mx[1] - mn[1];
        double ez = mx[2] - mn[2];
        return 2.0 * (ex * ey + ez * ey + ex * ez);
    }

    double centre(int axis) const { return (mn[axis] + mx[axis]) * 0.5; }
};

struct TreeNode
{
    Box box;
    uint64_t start = 0;
    uint64_t count = 0;
    std::unique_ptr<TreeNode> left;
    std::unique_ptr<TreeNode> right;
};

class Builder
{
public:
    Builder(const double* v, int64_t n, uint32_t maxLeaf) : maxLeafSize(maxLeaf)
    {
        size_t N = size_t(n);
        pmin.resize(N * 3);
        pmax.resize(N * 3);
        pctr.resize(N * 3);
        order.resize(N);
        #pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i)
        {
            const double* t = v + i * 9;
            for (int k = 0; k < 3; ++k)
            {
                // AABB::createFromVertices (AABB.cpp:35-50).
                double lo = std::min(t[k], std::min(t[3 + k], t[6 + k]));
                double hi = std::max(t[k], std::max(t[3 + k], t[6 + k]));
                pmin[size_t(i) * 3 + k] = lo;
                pmax[size_t(i) * 3 + k] = hi;
                // AABB::getCenter (AABB.cpp:128-131): (min + max) * 0.5.
                pctr[size_t(i) * 3 + k] = (lo + hi) * 0.5;
            }
            order[size_t(i)] = uint32_t(i);
        }
    }

    std::unique_ptr<TreeNode> build(uint64_t start, uint64_t end)
    {
        auto node = std::make_unique<TreeNode>();
        node->start = start;
        node->count = end - start;

        for (uint64_t i = start; i < end; ++i)
        {
            uint32_t p = order[i];
            node->box.expand(&pmin[size_t(p) * 3], &pmax[size_t(p) * 3]);
        }

        if (node->count <= maxLeafSize)
            return node;

        int axis = 0;
        double split = node->box.centre(0);
        chooseSplit(node->box, start, end, axis, split);

        // In-place swap partition (FlatBVH.cpp:166-174).
        uint64_t middle = start;
        for (uint64_t i = start; i < end; ++i)
        {
            if (pctr[size_t(order[i]) * 3 + axis] <= split)
            {
                std::swap(order[i], order[middle]);
                middle++;
            }
        }

        // Fallback (FlatBVH.cpp:176-177).
        if (middle == start || middle == end)
            middle = start + (end - start) / 2;

        if (node->count >= kTaskThreshold)
        {
            #pragma omp task shared(node)
            node->left = build(start, middle);
            #pragma omp task shared(node)
            node->right = build(middle, end);
            #pragma omp taskwait
        }
        else
        {
            node->left = build(start, middle);
            node->right = build(middle, end);
        }
        return node;
    }

    std::vector<uint32_t> order;

private:
    static constexpr uint64_t kTaskThreshold = 16384;

    // calculateSAHScore (FlatBVH.cpp:288-321).
    double score(int axis, double split, const Box& nodeBox, uint64_t start, uint64_t end) const
    {
        Box lb, rb;
        uint64_t lc = 0, rc = 0;
        for (uint64_t i = start; i < end; ++i)
        {
            size_t p = size_t(order[i]);
            if (pctr[p * 3 + axis] <= split)
            {
                lb.expand(&pmin[p * 3], &pmax[p * 3]);
                lc++;
            }
            else
            {
                rb.expand(&pmin[p * 3], &pmax[p * 3]);
                rc++;
            }
        }
        double s = 0.0;
        if (lc > 0)
            s += (lb.area() / nodeBox.area()) * double(lc);
        if (rc > 0)
            s += (rb.area() / nodeBox.area()) * double(rc);
        return s;
    }

    // calculateMedianPoint (FlatBVH.cpp:323-342): the median of the sorted
    // centroids; for an even count the mean of the two middle values. A
    // selection gives the same order statistics as the reference's sort.
    double median(int axis, uint64_t start, uint64_t end) const
    {
        size_t n = size_t(end - start);
        std::vector<double> c(n);
        for (size_t i = 0; i < n; ++i)
            c[i] = pctr[size_t(order[start + i]) * 3 + axis];
        size_t h = n / 2;
        std::nth_element(c.begin(), c.begin() + std::ptrdiff_t(h), c.end());
        double upper = c[h];
        if (n % 2 == 0)
        {
            double lower = *std::max_element(c.begin(), c.begin() + std::ptrdiff_t(h));
            return (lower + upper) / 2.0;
        }
        return upper;
    }

    // calculateSAHSplit (FlatBVH.cpp:241-286) with regularSAHSplits = 0.
    // The reference leaves axis/split unset when every score is NaN (a node
    // of zero surface area); here the first candidate is kept, after which
    // the partition falls back to the half split like the reference's would.
    void chooseSplit(const Box& nodeBox, uint64_t start, uint64_t end, int& axis, double& split) const
    {
        double lowest = std::numeric_limits<double>::max();
        for (int a = 0; a <= 2; ++a)
        {
            double s = nodeBox.centre(a);
            double sc = score(a, s, nodeBox, start, end);
            if (sc < lowest)
            {
                axis = a;
                split = s;
                lowest = sc;
            }
            s = median(a, start, end);
            sc = score(a, s, nodeBox, start, end);
            if (sc < lowest)
            {
                axis = a;
                split = s;
                lowest = sc;
            }
        }
    }

    uint32_t maxLeafSize;
    std::vector<double> pmin, pmax, pctr;
};

uint32_t flatten(const TreeNode* t, std::vector<BuildNode>& out)
{
    size_t idx = out.size();
    BuildNode n;
    for (int k = 0; k < 3; ++k)
    {
        n.bmin[k] = t->box.mn[k];
        n.bmax[k] = t->box.mx[k];
    }
    n.start = t->start;
    n.count = t->count;
    n.rightOffset = 0;
    out.push_back(n);
    if (!t->left)
        return 1;
    uint32_t dl = flatten(t->left.get(), out);
    out[idx].rightOffset = int64_t(out.size() - idx);
    uint32_t dr = flatten(t->right.get(), out);
    return 1 + std::max(dl, dr);
}

}  // namespace

bool buildFlatBVH(const double* vertices, int64_t n, uint32_t maxLeafSize, int threads, BuildResult& out,
                  std::string& error)
{
    if (n <= 0 || vertices == nullptr)
    {
        error = "buildFlatBVH: no triangles";
        return false;
    }
    if (n > (int64_t(1) << 27))
    {
        error = "buildFlatBVH: more than 2^27 triangles";
        return false;
    }
    if (maxLeafSize < 1 || maxLeafSize > 15)
    {
        error = "buildFlatBVH: maxLeafSize must be in 1..15";
        return false;
    }
    for (int64_t i = 0; i < n * 9; ++i)
    {
        if (!std::isfinite(vertices[i]))
        {
            error = "buildFlatBVH: non-finite vertex coordinate";
            return false;
        }
    }

    int saved = omp_get_max_threads();
    if (threads > 0)
        omp_set_num_threads(threads);

    Builder b(vertices, n, maxLeafSize);
    std::unique_ptr<TreeNode> root;
    #pragma omp parallel
    {
        #pragma omp single
        root = b.build(0, uint64_t(n));
    }

    out.nodes.clear();
    out.nodes.reserve(size_t(n));
    out.depth = flatten(root.get(), out.nodes);
    out.order = std::move(b.order);

    if (threads > 0)
        omp_set_num_threads(saved);
    return true;
}

}  // namespace rcx
