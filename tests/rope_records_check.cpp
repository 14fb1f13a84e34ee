// Host check of build_ropes: the rope walk visits the same leaves in the same
// order as the reference-order stack walk, for random trees and random box-hit
// predicates (keyed by the box's lo.x, unique per child).
#include "wide_bvh.cpp"
#include <cstdio>
#include <random>
using namespace rcx;
int main()
{
    std::mt19937 rng(7);
    for (int trial = 0; trial < 300; ++trial)
    {
        // random binary tree: inner node count n; children either inner (later index) or leaves
        int n = 1 + int(rng() % 200);
        std::vector<DevNode> nodes(n);
        std::vector<int> freeInner;  // indices 1..n-1 to be attached exactly once
        for (int i = 1; i < n; ++i) freeInner.push_back(i);
        std::shuffle(freeInner.begin(), freeInner.end(), rng);
        // BFS attach: each node gets two child slots
        int leafId = 0;
        float uniq = 0.0f;
        std::vector<int> queue{ 0 };
        size_t qi = 0, fi = 0;
        while (qi < queue.size())
        {
            int p = queue[qi++];
            int l[2];
            for (int k = 0; k < 2; ++k)
            {
                if (fi < freeInner.size() && (rng() % 3 != 0 || qi == queue.size()))
                {
                    l[k] = freeInner[fi++];
                    queue.push_back(l[k]);
                }
                else
                {
                    int start = leafId++, count = 1 + int(rng() % 4);
                    l[k] = ~((start << 4) | count);
                }
            }
            nodes[p].link = make_int4(l[0], l[1], 0, 0);
            nodes[p].xy0 = make_float4(uniq, uniq + 1, 0, 1); uniq += 2;
            nodes[p].xy1 = make_float4(uniq, uniq + 1, 0, 1); uniq += 2;
            nodes[p].z01 = make_float4(0, 1, 0, 1);
        }
        if (fi != freeInner.size()) { printf("tree gen incomplete\n"); return 1; }
        std::vector<DevRope> ropes;
        if (!build_ropes(nodes, 0, ropes)) { printf("build_ropes failed trial %d\n", trial); return 1; }
        if (ropes.size() != size_t(2 * n)) { printf("record count %zu vs %d\n", ropes.size(), 2 * n); return 1; }
        for (int pat = 0; pat < 20; ++pat)
        {
            uint32_t salt = rng();
            auto hitf = [&](float lox) { uint32_t hsh = uint32_t(lox * 7919.0f) * 2654435761u ^ salt; return (hsh >> 7) % 4 != 0; };
            // stack walk (reference order: left first)
            std::vector<int> a, b;
            std::vector<int> st;
            int cur = 0;
            while (true)
            {
                const DevNode& nd = nodes[cur];
                bool h0 = hitf(nd.xy0.x), h1 = hitf(nd.xy1.x);
                // traverse<ORDER_REF>: both hit -> left now, right later; a leaf child's triangles when reached
                std::vector<int> kids;
                if (h0) kids.push_back(nd.link.x);
                if (h1) kids.push_back(nd.link.y);
                for (int k = int(kids.size()) - 1; k >= 0; --k) st.push_back(kids[k]);
                bool moved = false;
                while (!st.empty())
                {
                    int c = st.back(); st.pop_back();
                    if (c < 0) { a.push_back(c); continue; }
                    cur = c; moved = true; break;
                }
                if (!moved) break;
            }
            // rope walk
            size_t r = 0;
            while (r < ropes.size())
            {
                const DevRope& q = ropes[r];
                bool h = hitf(q.a.x);
                if (h && q.link >= 0) { ++r; continue; }
                if (h) b.push_back(q.link);
                r = size_t(q.miss);
            }
            if (a != b) { printf("mismatch trial %d pattern %d: %zu vs %zu leaves\n", trial, pat, a.size(), b.size()); return 1; }
        }
    }
    printf("ropes ok\n");
    return 0;
}
