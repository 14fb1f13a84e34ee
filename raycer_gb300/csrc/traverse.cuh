// BVH traversal of the flat SAH BVH (device side).
//
// The reference traverses with an explicit stack: pop a node; a leaf tests
// its triangles in order; an inner node tests the right child's box and
// pushes it, then the left child's box and pushes it, so the left subtree is
// finished first (FlatBVH::intersect FlatBVH.cpp:22-75, intersectBVH
// intersections.cl:98-148). The root's own box is never tested.
//
// Here the node is the 64-B two-child record of device_types.h, so one fetch
// tests both children:
//   ORDER_REF      descend left, push right (the reference's visit order;
//                  the same boxes are tested, the same triangles in the same
//                  order, the same closest hit — ties to the later triangle,
//                  Triangle.cpp:93 `t > distance` rejects only farther hits).
//   ORDER_NEAREST  descend into the nearer child, push the farther one with
//                  its entry distance, and skip boxes whose entry distance is
//                  beyond the current closest hit. The accepted hit is the
//                  same: minimum t, ties resolved to the larger BVH-order
//                  slot, which is what the reference's order yields.
// Any-hit (shadow rays: isShadowRay + fastOcclusion) always uses the
// reference order and stops at the first triangle found; triangles whose
// material is nonShadowing are skipped (Triangle.cpp:55).
//
// `skip` names the triangle a secondary ray leaves from (-1 for none). Its
// origin is the hit point moved by rayStartOffset along the ray direction, so
// in exact arithmetic the ray travels away from that triangle's plane and
// cannot hit it; in float32 the hit point's rounding (about 1e-6 at
// coordinates of 10) can exceed the 1e-5 offset at grazing angles and report
// the ray's own triangle. Skipping it gives the float64 reference's answer.
#pragma once

#include <cfloat>

#include "rc_math.cuh"

namespace rcx
{

enum TraversalOrder
{
    ORDER_REF = 0,
    ORDER_NEAREST = 1,
    ORDER_WIDE = 2  // kernels only: ORDER_NEAREST's closest hit through the 4-wide BVH (traverse_wide)
};

struct HitF
{
    int slot;  // BVH-order triangle slot, -1 = none
    float t;
    float u;
    float v;
    int inst;  // instance of the hit in a two-level scene, else -1
};

struct TravCount
{
    uint32_t nodes;  // inner nodes fetched (child-pair box tests)
    uint32_t tris;   // triangle tests
};

__device__ __forceinline__ void load_node(const DevNode* __restrict__ nodes, int i, float4& a, float4& b, float4& c,
                                          int4& l)
{
    const float4* p = reinterpret_cast<const float4*>(nodes + i);
    a = __ldg(p + 0);
    b = __ldg(p + 1);
    c = __ldg(p + 2);
    l = __ldg(reinterpret_cast<const int4*>(p + 3));
}

// The test of one leaf triangle in traverse(): nonShadowing triangles are
// skipped by any-hit rays (Triangle.cpp:55); returns true when an any-hit
// ray has found its occluder (the walk ends), else updates the closest hit
// (the reference order keeps the later of equal distances, nearest-first
// the larger slot).
template <bool ANY_HIT, int ORDER, bool COUNT>
__device__ __forceinline__ bool leaf_test(const RayF& ray, HitF& hit, bool& found, TravCount& cnt, int slot, int skip,
                                          const float4& ta, const float4& tb, const float4& tc)
{
    if (slot == skip)
        return false;
    if (ANY_HIT && (__float_as_uint(tc.y) & kMetaNonShadowing))
        return false;
    if (COUNT)
        cnt.tris++;
    float t, u, v;
    if (!tri_hit(ray, v3(ta.x, ta.y, ta.z), v3(ta.w, tb.x, tb.y), v3(tb.z, tb.w, tc.x), t, u, v))
        return false;
    if (ANY_HIT)
    {
        hit.slot = slot;
        hit.t = t;
        hit.u = u;
        hit.v = v;
        return true;
    }
    const bool take = ORDER == ORDER_REF ? !(t > hit.t) : (t < hit.t || (t == hit.t && slot > hit.slot));
    if (take)
    {
        hit.slot = slot;
        hit.t = t;
        hit.u = u;
        hit.v = v;
        found = true;
    }
    return false;
}

// Returns true if any triangle was accepted. `hit` must be initialised by
// the caller (slot -1, t = FLT_MAX for a fresh query). `err` is set to 1 on
// a stack overflow (the ray is then abandoned; the host reports it).
// OCT >= 0: the caller guarantees that the ray's inverse direction is finite
// with those signs (ray_octant), and the box tests take slab_oct<OCT>.
template <bool ANY_HIT, int ORDER, bool COUNT, int OCT = -1>
__device__ __forceinline__ bool traverse(const DevScene& sc, const RayF& ray, HitF& hit, TravCount& cnt, int& err,
                                         int skip = -1)
{
    int stack[kMaxStack];
    float sdist[ORDER == ORDER_NEAREST && !ANY_HIT ? kMaxStack : 1];
    int sp = 0;
    int cur = sc.rootLink;
    bool found = false;

    while (true)
    {
        if (cur >= 0)
        {
            float4 a, b, c;
            int4 l;
            load_node(sc.nodes, cur, a, b, c, l);
            if (COUNT)
                cnt.nodes++;
            float e0, e1;
            bool h0, h1;
            if (OCT >= 0)
            {
                h0 = slab_oct<OCT < 0 ? 0 : OCT>(ray, a.x, a.y, a.z, a.w, c.x, c.y, e0);
                h1 = slab_oct<OCT < 0 ? 0 : OCT>(ray, b.x, b.y, b.z, b.w, c.z, c.w, e1);
            }
#ifndef RC_EXACT_SLAB_ONLY
            else if (ray.finite)
#else
            else if (false)
#endif
            {
                h0 = slab_finite(ray, a.x, a.y, a.z, a.w, c.x, c.y, e0);
                h1 = slab_finite(ray, b.x, b.y, b.z, b.w, c.z, c.w, e1);
            }
            else
            {
                h0 = slab(ray, a.x, a.y, a.z, a.w, c.x, c.y, e0);
                h1 = slab(ray, b.x, b.y, b.z, b.w, c.z, c.w, e1);
            }
            if (ORDER == ORDER_NEAREST && !ANY_HIT)
            {
                h0 = h0 && !(e0 > hit.t);
                h1 = h1 && !(e1 > hit.t);
            }
            if (h0 && h1)
            {
                int nearC = l.x, farC = l.y;
                float farD = e1;
                if (ORDER == ORDER_NEAREST && !ANY_HIT && e1 < e0)
                {
                    nearC = l.y;
                    farC = l.x;
                    farD = e0;
                }
                if (sp >= kMaxStack)
                {
                    err = 1;
                    return found;
                }
                stack[sp] = farC;
                if (ORDER == ORDER_NEAREST && !ANY_HIT)
                    sdist[sp] = farD;
                sp++;
                cur = nearC;
                continue;
            }
            if (h0)
            {
                cur = l.x;
                continue;
            }
            if (h1)
            {
                cur = l.y;
                continue;
            }
        }
        else
        {
            int leaf = ~cur;
            int start = leaf >> kLeafCountBits;
            int count = leaf & ((1 << kLeafCountBits) - 1);
            if (!ANY_HIT && ORDER == ORDER_NEAREST)
            {
                // closest hit, nearest-first: two triangles fetched per step
                // (the accepted hit does not depend on the test order; 8 %
                // less time for rc_cast's random rays). Any-hit and
                // reference-order walks keep one triangle per step: in the
                // issue-bound RAY frame the pairs cost more than they hid.
                for (int i = 0; i < count; i += 2)
                {
                    const int s0 = start + i;
                    const int s1 = start + min(i + 1, count - 1);
                    const float4* p0 = reinterpret_cast<const float4*>(sc.tris + s0);
                    const float4* p1 = reinterpret_cast<const float4*>(sc.tris + s1);
                    const float4 a0 = __ldg(p0 + 0), b0 = __ldg(p0 + 1), c0 = __ldg(p0 + 2);
                    const float4 a1 = __ldg(p1 + 0), b1 = __ldg(p1 + 1), c1 = __ldg(p1 + 2);
                    leaf_test<ANY_HIT, ORDER, COUNT>(ray, hit, found, cnt, s0, skip, a0, b0, c0);
                    if (i + 1 < count)
                        leaf_test<ANY_HIT, ORDER, COUNT>(ray, hit, found, cnt, s1, skip, a1, b1, c1);
                }
            }
            else
            {
                for (int i = 0; i < count; ++i)
                {
                    const int slot = start + i;
                    const float4* tp = reinterpret_cast<const float4*>(sc.tris + slot);
                    if (slot != skip && leaf_test<ANY_HIT, ORDER, COUNT>(ray, hit, found, cnt, slot, skip,
                                                                         __ldg(tp + 0), __ldg(tp + 1), __ldg(tp + 2)))
                        return true;
                }
            }
        }

        // pop
        while (true)
        {
            if (sp == 0)
                return found;
            sp--;
            cur = stack[sp];
            if (ORDER == ORDER_NEAREST && !ANY_HIT && sdist[sp] > hit.t)
                continue;
            break;
        }
    }
}

// The reference's order without a stack, on the rope records (DevRope,
// every child box of the binary tree once, in the reference's preorder): a
// hit inner box continues at the next record (its left child), a hit leaf
// box's triangles are tested in order, and after a leaf or on a miss the
// walk jumps to the record after the box's subtree. Each ray meets the boxes
// and triangles of traverse<ANY_HIT, ORDER_REF> in the same order (the same
// slab test on the same float boxes), so it returns the same closest hit
// (ties to the later triangle) or the same first any-hit; one 32-byte record
// per tested box, no stack, and a descent reads the next record in memory.
// Needs sc.ropes (callers fall back to traverse() without them).
template <bool ANY_HIT>
__device__ __forceinline__ bool test_leaf(const DevScene& sc, const RayF& ray, HitF& hit, int leafCode, int skip,
                                          bool& found)
{
    const int leaf = ~leafCode;
    const int start = leaf >> kLeafCountBits;
    const int count = leaf & ((1 << kLeafCountBits) - 1);
    for (int i = 0; i < count; ++i)
    {
        const int slot = start + i;
        if (slot == skip)
            continue;
        const float4* tp = reinterpret_cast<const float4*>(sc.tris + slot);
        const float4 ta = __ldg(tp + 0);
        const float4 tb = __ldg(tp + 1);
        const float4 tc = __ldg(tp + 2);
        if (ANY_HIT && (__float_as_uint(tc.y) & kMetaNonShadowing))
            continue;
        float t, u, v;
        if (tri_hit(ray, v3(ta.x, ta.y, ta.z), v3(ta.w, tb.x, tb.y), v3(tb.z, tb.w, tc.x), t, u, v) &&
            (ANY_HIT || !(t > hit.t)))
        {
            hit.slot = slot;
            hit.t = t;
            hit.u = u;
            hit.v = v;
            found = true;
            if (ANY_HIT)
                return true;
        }
    }
    return false;
}

template <bool ANY_HIT>
__device__ __forceinline__ bool traverse_stackless(const DevScene& sc, const RayF& ray, HitF& hit, int skip)
{
    bool found = false;
    if (sc.rootLink < 0)
    {
        test_leaf<ANY_HIT>(sc, ray, hit, sc.rootLink, skip, found);  // a leaf root: its triangles only
        return found;
    }
    const int end = sc.ropeCount;
    int r = 0;
    while (r < end)
    {
        const float4* p = reinterpret_cast<const float4*>(sc.ropes + r);
        const float4 a = __ldg(p);
        const float4 b = __ldg(p + 1);  // hi.y, hi.z, link, miss
        float e;
        const bool h = ray.finite ? slab_finite(ray, a.x, a.w, a.y, b.x, a.z, b.y, e)
                                  : slab(ray, a.x, a.w, a.y, b.x, a.z, b.y, e);
        const int link = __float_as_int(b.z);
        if (h && link >= 0)
        {
            ++r;
            continue;
        }
        if (h && test_leaf<ANY_HIT>(sc, ray, hit, link, skip, found))
            return true;
        r = __float_as_int(b.w);
    }
    return found;
}

// Entry distance of one child box of a wide node, or +inf when the ray misses
// it or enters it beyond `limit` (the current closest hit).
__device__ __forceinline__ float wide_entry(const RayF& ray, float lox, float hix, float loy, float hiy, float loz,
                                            float hiz, float limit)
{
    float e;
    const bool h = ray.finite ? slab_finite(ray, lox, hix, loy, hiy, loz, hiz, e)
                              : slab(ray, lox, hix, loy, hiy, loz, hiz, e);
    return h && !(e > limit) ? e : __int_as_float(0x7f800000);
}

// Orders two (distance, link) pairs by distance.
__device__ __forceinline__ void wide_cswap(float& da, int& la, float& db, int& lb)
{
    const bool s = db < da;
    const float d = s ? db : da;
    const int l = s ? lb : la;
    db = s ? da : db;
    lb = s ? la : lb;
    da = d;
    la = l;
}

// Closest hit through the 4-wide BVH (sc.wide; wide_bvh.cpp): one 128-B
// node fetch tests up to four child boxes, the children hit within the
// current closest distance are sorted by entry distance (a five-exchange
// network), the nearest is entered and the others pushed farthest first with
// their entry distances, and pops skip entries beyond the current hit. The
// leaves and their triangle tests are the binary tree's, and the accepted
// hit (minimum t, ties to the larger slot) does not depend on the order, so
// it is traverse<false, ORDER_NEAREST>'s. No node or triangle counts: counted
// frames use the binary traversal.
// Where a 4-wide walk stands between steps: the node or leaf link to visit
// next and the stack depth (the stack arrays are the caller's).
struct WideWalk
{
    int cur;
    int sp;
    bool found;
};

// The closest-hit test of one leaf triangle in the 4-wide walk.
__device__ __forceinline__ void wide_leaf_test(const RayF& ray, HitF& hit, WideWalk& w, int slot, int skip,
                                               const float4& ta, const float4& tb, const float4& tc)
{
    if (slot == skip)
        return;
    float t, u, v;
    if (tri_hit(ray, v3(ta.x, ta.y, ta.z), v3(ta.w, tb.x, tb.y), v3(tb.z, tb.w, tc.x), t, u, v) &&
        (t < hit.t || (t == hit.t && slot > hit.slot)))
    {
        hit.slot = slot;
        hit.t = t;
        hit.u = u;
        hit.v = v;
        w.found = true;
    }
}

// One step of the 4-wide walk: a node fetch (entering its nearest child hit
// within the current closest distance, the others pushed) or a leaf's
// triangle tests; where no child is entered, the pop of the next stack entry
// still in range. Returns true when the walk is over (stack empty, or
// overflow: err = 1).
__device__ __forceinline__ bool wide_step(const DevNode4* __restrict__ wide, const DevTri* __restrict__ tris,
                                          const RayF& ray, HitF& hit, WideWalk& w, int* stack, float* sdist,
                                          int skip, int& err)
{
    const float kInf = __int_as_float(0x7f800000);
    if (w.cur >= 0)
    {
        const float4* p = reinterpret_cast<const float4*>(wide + w.cur);
        const float4 lox = __ldg(p + 0), hix = __ldg(p + 1), loy = __ldg(p + 2), hiy = __ldg(p + 3);
        const float4 loz = __ldg(p + 4), hiz = __ldg(p + 5);
        const int4 l = __ldg(reinterpret_cast<const int4*>(p + 6));
        const int nc = __ldg(reinterpret_cast<const int*>(p + 7));
        float d0 = wide_entry(ray, lox.x, hix.x, loy.x, hiy.x, loz.x, hiz.x, hit.t);
        float d1 = wide_entry(ray, lox.y, hix.y, loy.y, hiy.y, loz.y, hiz.y, hit.t);
        float d2 = nc > 2 ? wide_entry(ray, lox.z, hix.z, loy.z, hiy.z, loz.z, hiz.z, hit.t) : kInf;
        float d3 = nc > 3 ? wide_entry(ray, lox.w, hix.w, loy.w, hiy.w, loz.w, hiz.w, hit.t) : kInf;
        int l0 = l.x, l1 = l.y, l2 = l.z, l3 = l.w;
        const int hits = (d0 < kInf ? 1 : 0) + (d1 < kInf ? 1 : 0) + (d2 < kInf ? 1 : 0) + (d3 < kInf ? 1 : 0);
        if (hits == 1)
        {
            w.cur = d0 < kInf ? l0 : (d1 < kInf ? l1 : (d2 < kInf ? l2 : l3));
            return false;
        }
        if (hits > 1)
        {
            wide_cswap(d0, l0, d1, l1);
            wide_cswap(d2, l2, d3, l3);
            wide_cswap(d0, l0, d2, l2);
            wide_cswap(d1, l1, d3, l3);
            wide_cswap(d1, l1, d2, l2);
            if (w.sp + hits - 1 > kMaxStack)
            {
                err = 1;
                return true;
            }
            if (d3 < kInf)
            {
                stack[w.sp] = l3;
                sdist[w.sp] = d3;
                w.sp++;
            }
            if (d2 < kInf)
            {
                stack[w.sp] = l2;
                sdist[w.sp] = d2;
                w.sp++;
            }
            if (d1 < kInf)
            {
                stack[w.sp] = l1;
                sdist[w.sp] = d1;
                w.sp++;
            }
            w.cur = l0;
            return false;
        }
    }
    else
    {
        const int leaf = ~w.cur;
        const int start = leaf >> kLeafCountBits;
        const int count = leaf & ((1 << kLeafCountBits) - 1);
        // Two triangles per iteration, both fetched before either is tested
        // (the second index clamped to the leaf: an odd leaf fetches its last
        // triangle twice and tests it once), so a leaf's fetches overlap.
        // The accepted hit does not depend on the order of the tests.
        for (int i = 0; i < count; i += 2)
        {
            const int s0 = start + i;
            const int s1 = start + min(i + 1, count - 1);
            const float4* p0 = reinterpret_cast<const float4*>(tris + s0);
            const float4* p1 = reinterpret_cast<const float4*>(tris + s1);
            const float4 a0 = __ldg(p0 + 0), b0 = __ldg(p0 + 1), c0 = __ldg(p0 + 2);
            const float4 a1 = __ldg(p1 + 0), b1 = __ldg(p1 + 1), c1 = __ldg(p1 + 2);
            wide_leaf_test(ray, hit, w, s0, skip, a0, b0, c0);
            if (i + 1 < count)
                wide_leaf_test(ray, hit, w, s1, skip, a1, b1, c1);
        }
    }
    // pop
    while (true)
    {
        if (w.sp == 0)
            return true;
        w.sp--;
        w.cur = stack[w.sp];
        if (sdist[w.sp] > hit.t)
            continue;
        return false;
    }
}

__device__ __forceinline__ bool traverse_wide(const DevScene& sc, const RayF& ray, HitF& hit, int& err, int skip)
{
    int stack[kMaxStack];
    float sdist[kMaxStack];
    WideWalk w{ sc.wideRoot, 0, false };
    while (!wide_step(sc.wide, sc.tris, ray, hit, w, stack, sdist, skip, err))
    {
    }
    return w.found;
}

// One stack entry of the warp-wide traversal: a node link and the lanes
// whose rays take part in its subtree.
struct PacketEntry
{
    int link;
    unsigned lanes;
};

// Warp-wide (masked packet) closest-hit traversal: the 32 lanes of a warp,
// one ray each, walk one shared node sequence, so every node and triangle
// record is one broadcast load and the control flow stays converged. Must be
// called by all 32 lanes together; `active` marks the lanes with a ray;
// `wstack` is this warp's kMaxStack-entry stack in shared memory. Each lane
// makes the tests its own traverse() call would make, in the same order:
//   ORDER_REF      the shared sequence is the tree's preorder restricted to
//                  the boxes some lane hits (left subtree first); a lane takes
//                  part only in the subtrees whose box its ray hits, so it
//                  meets its triangles in its per-ray order and gets the same
//                  closest hit (ties to the later triangle).
//   ORDER_NEAREST  the warp descends first into the child that most of its
//                  lanes find nearer; each lane culls boxes whose entry
//                  distance lies beyond its own current hit. The accepted hit
//                  (minimum t, ties to the larger slot) does not depend on
//                  the order.
// It pays for coherent rays (the primary rays of a pixel tile); any-hit
// shadow rays, which stop at different depths, ran slower this way than one
// traversal per lane. Node and triangle counts are not kept: counted frames
// use traverse().
template <int ORDER>
__device__ __forceinline__ bool traverse_packet(const DevScene& sc, const RayF& ray, HitF& hit, int& err, int skip,
                                                bool active, PacketEntry* __restrict__ wstack)
{
    constexpr bool CULL = ORDER == ORDER_NEAREST;
    constexpr unsigned kAll = 0xffffffffu;
    float sdist[CULL ? kMaxStack : 1];  // this lane's entry distance of each stacked box
    const unsigned bit = 1u << (threadIdx.x & 31u);
    bool found = false;
    int sp = 0;
    int cur = sc.rootLink;
    unsigned curMask = __ballot_sync(kAll, active);
    if (curMask == 0)
        return false;

    while (true)
    {
        if (cur >= 0)
        {
            float4 a, b, c;
            int4 l;
            load_node(sc.nodes, cur, a, b, c, l);
            float e0 = 0.0f, e1 = 0.0f;
            bool h0 = false, h1 = false;
            if (curMask & bit)
            {
                if (ray.finite)
                {
                    h0 = slab_finite(ray, a.x, a.y, a.z, a.w, c.x, c.y, e0);
                    h1 = slab_finite(ray, b.x, b.y, b.z, b.w, c.z, c.w, e1);
                }
                else
                {
                    h0 = slab(ray, a.x, a.y, a.z, a.w, c.x, c.y, e0);
                    h1 = slab(ray, b.x, b.y, b.z, b.w, c.z, c.w, e1);
                }
                if (CULL)
                {
                    h0 = h0 && !(e0 > hit.t);
                    h1 = h1 && !(e1 > hit.t);
                }
            }
            const unsigned m0 = __ballot_sync(kAll, h0);
            const unsigned m1 = __ballot_sync(kAll, h1);
            if (m0 && m1)
            {
                bool rightFirst = false;
                if (CULL)
                {
                    const unsigned vote = __ballot_sync(kAll, h0 && h1 && e1 < e0);
                    rightFirst = 2 * __popc(vote) > __popc(m0 & m1);
                }
                if (sp >= kMaxStack)
                {
                    err = 1;
                    return found;
                }
                __syncwarp();  // every lane has read the entry this push may replace
                if ((threadIdx.x & 31u) == 0)
                    wstack[sp] = PacketEntry{ rightFirst ? l.x : l.y, rightFirst ? m0 : m1 };
                if (CULL)
                    sdist[sp] = rightFirst ? e0 : e1;
                sp++;
                cur = rightFirst ? l.y : l.x;
                curMask = rightFirst ? m1 : m0;
                continue;
            }
            if (m0 | m1)
            {
                cur = m0 ? l.x : l.y;
                curMask = m0 | m1;
                continue;
            }
        }
        else
        {
            const int leaf = ~cur;
            const int start = leaf >> kLeafCountBits;
            const int count = leaf & ((1 << kLeafCountBits) - 1);
            const bool in = (curMask & bit) != 0;
            TravCount none{ 0, 0 };
            for (int i = 0; i < count; ++i)
            {
                const int slot = start + i;
                const float4* tp = reinterpret_cast<const float4*>(sc.tris + slot);
                const float4 ta = __ldg(tp + 0);
                const float4 tb = __ldg(tp + 1);
                const float4 tc = __ldg(tp + 2);
                if (in)
                    leaf_test<false, ORDER, false>(ray, hit, found, none, slot, skip, ta, tb, tc);
            }
        }

        // pop the next subtree some lane still takes part in
        while (true)
        {
            if (sp == 0)
                return found;
            sp--;
            __syncwarp();
            const PacketEntry e = wstack[sp];
            bool in = (e.lanes & bit) != 0;
            if (CULL && in && sdist[sp] > hit.t)
                in = false;
            curMask = __ballot_sync(kAll, in);
            cur = e.link;
            if (curMask)
                break;
        }
    }
}

// Ray in an instance's object space: o' = A o + b, d' = A d. d' is not
// renormalised, so a hit's parameter t is the same in both spaces and the
// levels share one closest distance. (The reference's Instance normalises
// the direction and recomputes the world distance from the transformed hit
// point, Instance.cpp:65-100: the same t in exact arithmetic.)
__device__ __forceinline__ RayF instance_ray(const DevInstance& in, const RayF& r)
{
    if (in.identity)
        return r;
    V3 o = v3(__fmaf_rn(in.r0.x, r.o.x, __fmaf_rn(in.r0.y, r.o.y, __fmaf_rn(in.r0.z, r.o.z, in.r0.w))),
              __fmaf_rn(in.r1.x, r.o.x, __fmaf_rn(in.r1.y, r.o.y, __fmaf_rn(in.r1.z, r.o.z, in.r1.w))),
              __fmaf_rn(in.r2.x, r.o.x, __fmaf_rn(in.r2.y, r.o.y, __fmaf_rn(in.r2.z, r.o.z, in.r2.w))));
    V3 d = v3(__fmaf_rn(in.r0.x, r.d.x, __fmaf_rn(in.r0.y, r.d.y, __fmul_rn(in.r0.z, r.d.z))),
              __fmaf_rn(in.r1.x, r.d.x, __fmaf_rn(in.r1.y, r.d.y, __fmul_rn(in.r1.z, r.d.z))),
              __fmaf_rn(in.r2.x, r.d.x, __fmaf_rn(in.r2.y, r.d.y, __fmul_rn(in.r2.z, r.d.z))));
    return make_ray(o, d, r.tmin, r.tmax);
}

__device__ __forceinline__ DevInstance load_instance(const DevInstance* __restrict__ p, int k)
{
    const float4* q = reinterpret_cast<const float4*>(p + k);
    DevInstance in;
    in.r0 = __ldg(q + 0);
    in.r1 = __ldg(q + 1);
    in.r2 = __ldg(q + 2);
    const int4 m = __ldg(reinterpret_cast<const int4*>(q + 3));
    in.rootLink = m.x;
    in.material = m.y;
    in.primBase = m.z;
    in.identity = m.w;
    return in;
}

// Two-level traversal: the top-level BVH over instances (nearest child
// first, culled by the closest hit), and inside each instance its mesh's
// BVH with the object-space ray. `skip` / `skipInst` name the triangle (and
// its instance) a secondary ray leaves from. Instance materials that are
// nonShadowing are skipped by any-hit queries (Instance.cpp:25-26).
template <bool ANY_HIT, bool COUNT>
__device__ __noinline__ bool traverse_instanced(const DevScene& sc, const RayF& ray, HitF& hit, TravCount& cnt,
                                                int& err, int skip, int skipInst)
{
    constexpr int kTopStack = 32;
    int stack[kTopStack];
    float sdist[kTopStack];
    int sp = 0;
    int cur = sc.tlasRoot;
    bool found = false;
    DevScene mesh = sc;
    while (true)
    {
        if (cur >= 0)
        {
            float4 a, b, c;
            int4 l;
            load_node(sc.tlas, cur, a, b, c, l);
            float e0, e1;
            bool h0, h1;
            if (ray.finite)
            {
                h0 = slab_finite(ray, a.x, a.y, a.z, a.w, c.x, c.y, e0);
                h1 = slab_finite(ray, b.x, b.y, b.z, b.w, c.z, c.w, e1);
            }
            else
            {
                h0 = slab(ray, a.x, a.y, a.z, a.w, c.x, c.y, e0);
                h1 = slab(ray, b.x, b.y, b.z, b.w, c.z, c.w, e1);
            }
            if (!ANY_HIT)
            {
                h0 = h0 && !(e0 > hit.t);
                h1 = h1 && !(e1 > hit.t);
            }
            if (h0 && h1)
            {
                int nearC = l.x, farC = l.y;
                float farD = e1;
                if (!ANY_HIT && e1 < e0)
                {
                    nearC = l.y;
                    farC = l.x;
                    farD = e0;
                }
                if (sp >= kTopStack)
                {
                    err = 1;
                    return found;
                }
                stack[sp] = farC;
                sdist[sp] = farD;
                sp++;
                cur = nearC;
                continue;
            }
            if (h0)
            {
                cur = l.x;
                continue;
            }
            if (h1)
            {
                cur = l.y;
                continue;
            }
        }
        else
        {
            const int leaf = ~cur;
            const int start = leaf >> kLeafCountBits;
            const int count = leaf & ((1 << kLeafCountBits) - 1);
            for (int i = 0; i < count; ++i)
            {
                const int k = start + i;
                const DevInstance in = load_instance(sc.instances, k);
                if (ANY_HIT && in.material >= 0 &&
                    (__float_as_uint(__ldg(&sc.mats[in.material].emittance.w)) & kMatNonShadowing))
                    continue;
                const RayF r2 = instance_ray(in, ray);
                mesh.rootLink = in.rootLink;
                HitF h2 = hit;
                if (traverse<ANY_HIT, ORDER_NEAREST, COUNT>(mesh, r2, h2, cnt, err, k == skipInst ? skip : -1))
                {
                    hit = h2;
                    hit.inst = k;
                    found = true;
                    if (ANY_HIT)
                        return true;
                }
            }
        }
        while (true)
        {
            if (sp == 0)
                return found;
            sp--;
            cur = stack[sp];
            if (!ANY_HIT && sdist[sp] > hit.t)
                continue;
            break;
        }
    }
}

// Either traversal, by the scene's kind.
template <bool ANY_HIT, int ORDER, bool COUNT>
__device__ __forceinline__ bool traverse_scene(const DevScene& sc, const RayF& ray, HitF& hit, TravCount& cnt,
                                               int& err, int skip, int skipInst)
{
    if (sc.numInstances > 0)
        return traverse_instanced<ANY_HIT, COUNT>(sc, ray, hit, cnt, err, skip, skipInst);
    return traverse<ANY_HIT, ORDER, COUNT>(sc, ray, hit, cnt, err, skip);
}

}  // namespace rcx
