// 4-wide BVH of a single-level scene, collapsed on the host from its binary
// device nodes at the scene's first PATH render, for the path tracer's
// extend kernel (bounce
// rays: 5 % less extend time than the binary tree on a 5M-triangle scene;
// for rc_cast's random rays it measured 3 % slower, so rc_cast keeps the
// binary tree).
//
// Each wide node starts from one binary node's two children and repeatedly
// replaces its inner child of largest surface area by that child's two
// children, up to four. Leaves stay as they are (the same leaf codes, the same
// triangle order), so a triangle test of the wide traversal is the binary
// traversal's. A child box of the binary tree lies inside its parent's box
// (also in float: both were rounded to nearest from nested boxes, or are
// float unions), and the slab test is monotone in the box, so every ray that
// reaches a grandchild through the binary tree reaches it through the wide
// node too: the nearest-first closest hit, which does not depend on the
// visiting order, is the same.
//
// The traversal pushes at most (children - 1) entries per node; a tree whose
// worst root-to-leaf sum exceeds the stack is left binary, and so is every
// scene when RC_WIDE_BVH=0 is set in the environment (read once).
//
// The same file writes the rope records of the stackless walk: every child
// box of the binary tree once, in the reference's preorder, with the index
// of the first record after its subtree (DevRope, traverse_stackless).

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <string>
#include <vector>

#include "host_internal.h"

namespace rcx
{
namespace
{

struct Child
{
    int32_t link;
    float lo[3];
    float hi[3];
};

void children_of(const DevNode& n, Child& a, Child& b)
{
    a.link = n.link.x;
    a.lo[0] = n.xy0.x;
    a.hi[0] = n.xy0.y;
    a.lo[1] = n.xy0.z;
    a.hi[1] = n.xy0.w;
    a.lo[2] = n.z01.x;
    a.hi[2] = n.z01.y;
    b.link = n.link.y;
    b.lo[0] = n.xy1.x;
    b.hi[0] = n.xy1.y;
    b.lo[1] = n.xy1.z;
    b.hi[1] = n.xy1.w;
    b.lo[2] = n.z01.z;
    b.hi[2] = n.z01.w;
}

double half_area(const Child& c)
{
    const double dx = std::max(0.0, double(c.hi[0]) - double(c.lo[0]));
    const double dy = std::max(0.0, double(c.hi[1]) - double(c.lo[1]));
    const double dz = std::max(0.0, double(c.hi[2]) - double(c.lo[2]));
    return dx * dy + dy * dz + dz * dx;
}

// Builds the wide nodes; returns the largest stack need (entries pushed on a
// root-to-leaf path), or -1 for a malformed binary tree.
int collapse(const std::vector<DevNode>& nodes, int32_t rootLink, std::vector<DevNode4>& out)
{
    struct Item
    {
        int32_t bin;   // binary inner node
        int32_t slot;  // its wide node
        int need;      // stack entries pushed above it
    };
    out.clear();
    out.reserve(nodes.size() / 2 + 1);
    out.push_back(DevNode4{});
    std::vector<Item> work{ { rootLink, 0, 0 } };
    int maxNeed = 0;
    const int32_t count = int32_t(nodes.size());
    while (!work.empty())
    {
        const Item it = work.back();
        work.pop_back();
        if (it.bin < 0 || it.bin >= count)
            return -1;
        Child c[4];
        int n = 2;
        children_of(nodes[size_t(it.bin)], c[0], c[1]);
        while (n < 4)
        {
            int best = -1;
            double bestA = -1.0;
            for (int k = 0; k < n; ++k)
                if (c[k].link >= 0 && half_area(c[k]) > bestA)
                {
                    best = k;
                    bestA = half_area(c[k]);
                }
            if (best < 0)
                break;
            if (c[best].link >= count)
                return -1;
            Child x, y;
            children_of(nodes[size_t(c[best].link)], x, y);
            c[best] = x;
            c[n++] = y;
        }
        DevNode4 w{};
        float* lox = &w.lox.x;
        float* hix = &w.hix.x;
        float* loy = &w.loy.x;
        float* hiy = &w.hiy.x;
        float* loz = &w.loz.x;
        float* hiz = &w.hiz.x;
        int* link = &w.link.x;
        const int need = it.need + (n - 1);
        maxNeed = std::max(maxNeed, need);
        for (int k = 0; k < n; ++k)
        {
            lox[k] = c[k].lo[0];
            hix[k] = c[k].hi[0];
            loy[k] = c[k].lo[1];
            hiy[k] = c[k].hi[1];
            loz[k] = c[k].lo[2];
            hiz[k] = c[k].hi[2];
            if (c[k].link >= 0)
            {
                link[k] = int32_t(out.size());
                out.push_back(DevNode4{});
                work.push_back({ c[k].link, link[k], need });
            }
            else
                link[k] = c[k].link;
        }
        w.meta.x = n;
        out[size_t(it.slot)] = w;
    }
    return maxNeed;
}

// Rope records of the binary tree in the reference's preorder (left child
// first; the root's own box is never tested, so its two children are the
// first subtrees). Returns false for malformed links.
bool build_ropes(const std::vector<DevNode>& nodes, int32_t rootLink, std::vector<DevRope>& out)
{
    out.clear();
    if (rootLink < 0)
        return true;  // a leaf root: the walk tests its triangles only
    const int32_t count = int32_t(nodes.size());
    if (rootLink >= count)
        return false;
    out.reserve(2 * nodes.size());
    // Explicit preorder: `work` holds the child boxes still to emit (next on
    // top). `open` holds the inner records whose subtrees are being emitted
    // (innermost last) and `pending` how many of their two child subtrees are
    // not complete yet; a record's miss link is set when its subtree is.
    std::vector<Child> work;
    std::vector<int32_t> open;
    std::vector<int> pending;
    Child x, y;
    children_of(nodes[size_t(rootLink)], x, y);
    work.push_back(y);
    work.push_back(x);
    while (!work.empty())
    {
        const Child c = work.back();
        work.pop_back();
        if (out.size() >= 2 * nodes.size() + 2)
            return false;  // a cycle in the links
        const int32_t r = int32_t(out.size());
        DevRope rec{};
        rec.a = make_float4(c.lo[0], c.lo[1], c.lo[2], c.hi[0]);
        rec.hi_y = c.hi[1];
        rec.hi_z = c.hi[2];
        rec.link = c.link;
        rec.miss = 0;
        out.push_back(rec);
        if (c.link >= 0)
        {
            if (c.link >= count)
                return false;
            children_of(nodes[size_t(c.link)], x, y);
            work.push_back(y);
            work.push_back(x);
            open.push_back(r);
            pending.push_back(2);
            continue;
        }
        out[size_t(r)].miss = r + 1;  // a leaf's subtree is itself
        // the leaf completes a child subtree of the innermost open record;
        // each record completed that way completes one of its parent's
        while (!open.empty() && --pending.back() == 0)
        {
            out[size_t(open.back())].miss = int32_t(out.size());
            open.pop_back();
            pending.pop_back();
        }
    }
    return open.empty();
}

}  // namespace

rc_status upload_wide(rc_tracer* h, const std::vector<DevNode>& nodes, int32_t rootLink)
{
    h->dWide = nullptr;
    h->wideCount = 0;
    h->wideRoot = rootLink;
    static const bool enabled = [] {
        const char* v = std::getenv("RC_WIDE_BVH");
        return !(v && v[0] == '0');
    }();
    if (rootLink < 0 || !enabled)
        return RC_OK;  // a leaf root (nothing to collapse) or switched off: binary traversal
    std::vector<DevNode4> wide;
    const int need = collapse(nodes, rootLink, wide);
    if (need < 0)
    {
        h->err = "wide BVH: malformed binary node links";
        return RC_DEVICE_ERROR;
    }
    if (need > kMaxStack)
        return RC_OK;  // stays binary
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&h->dWide), wide.size() * sizeof(DevNode4));
    if (e == cudaSuccess)
        e = cudaMemcpy(h->dWide, wide.data(), wide.size() * sizeof(DevNode4), cudaMemcpyHostToDevice);
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        cudaFree(h->dWide);
        h->dWide = nullptr;
        h->err = std::string("wide BVH: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? RC_OOM : RC_CUDA;
    }
    h->wideCount = wide.size();
    h->wideRoot = 0;
    h->deviceBytes += wide.size() * sizeof(DevNode4);
    return RC_OK;
}

rc_status ensure_wide(rc_tracer* h)
{
    if (h->wideTried || !h->sceneReady || h->nInstances > 0)
        return RC_OK;
    h->wideTried = true;
    std::vector<DevNode> nodes(h->rootLink >= 0 ? h->innerCount : 0);
    if (!nodes.empty())
    {
        cudaError_t e = cudaMemcpy(nodes.data(), h->dNodes, nodes.size() * sizeof(DevNode), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess)
        {
            cudaGetLastError();
            h->err = std::string("wide BVH: download nodes: ") + cudaGetErrorString(e);
            return RC_CUDA;
        }
    }
    return upload_wide(h, nodes, h->rootLink);
}

rc_status ensure_ropes(rc_tracer* h)
{
    if (h->ropesTried || !h->sceneReady || h->nInstances > 0)
        return RC_OK;
    h->ropesTried = true;
    if (h->rootLink < 0)
        return RC_OK;  // a leaf root: the stack walk tests it directly
    std::vector<DevNode> nodes(h->innerCount);
    cudaError_t e = cudaMemcpy(nodes.data(), h->dNodes, nodes.size() * sizeof(DevNode), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        h->err = std::string("rope records: download nodes: ") + cudaGetErrorString(e);
        return RC_CUDA;
    }
    std::vector<DevRope> ropes;
    if (!build_ropes(nodes, h->rootLink, ropes))
    {
        h->err = "rope records: malformed binary node links";
        return RC_DEVICE_ERROR;
    }
    e = cudaMalloc(reinterpret_cast<void**>(&h->dRopes), ropes.size() * sizeof(DevRope));
    if (e == cudaSuccess)
        e = cudaMemcpy(h->dRopes, ropes.data(), ropes.size() * sizeof(DevRope), cudaMemcpyHostToDevice);
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        cudaFree(h->dRopes);
        h->dRopes = nullptr;
        h->err = std::string("rope records: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? RC_OOM : RC_CUDA;
    }
    h->ropeCount = ropes.size();
    h->deviceBytes += ropes.size() * sizeof(DevRope);
    return RC_OK;
}

}  // namespace rcx
