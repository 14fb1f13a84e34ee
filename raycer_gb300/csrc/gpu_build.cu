// GPU BVH builder: a linear BVH (Karras 2012, "Maximizing parallelism in
// the construction of BVHs, octrees, and k-d trees") built entirely on the
// device, as the fast alternative to the reference's SAH build
// (FlatBVH::build, FlatBVH.cpp:89-343, which stays the default and the
// parity mode).
//
//   1. k_prep        float vertices, triangle boxes and centroids; per-block
//                    centroid bounds (k_bounds_final reduces them)
//   2. k_morton      30-bit Morton code of each centroid in the centroid box
//                    (cubic cells: one scale, the box's largest extent)
//   3. radix sort    (code, triangle) pairs, 4 stable passes of 8 bits:
//                    per-tile digit histograms, one exclusive scan over
//                    (digit, tile), stable scatter ranked with __match_any_sync
//   4. k_hierarchy   the n - 1 internal nodes: each finds its key range and
//                    split from the sorted codes alone (ties in the code
//                    broken by index), so all nodes are built in parallel
//   5. k_boxes       bottom-up boxes and heights: one thread per leaf walks
//                    up; at each node the first thread to arrive stops and
//                    the second (which sees the sibling's box, published
//                    before the arrival counter) merges. No thread waits.
//   6. keep / scan / k_emit: internal nodes whose range holds more than
//                    `leafMax` triangles become device nodes (compact
//                    indices by a scan); smaller subtrees are contiguous
//                    ranges of the sorted order and become leaf links
//                    ~(start << 4 | count) directly.
//   7. k_tri_records triangle and shading records in sorted order, with the
//                    host builder's arithmetic (float32 edges; float64
//                    normal, tangent, bitangent with explicit rounding).

#include <cfloat>
#include <cstdint>
#include <utility>

#include "gpu_build.h"

namespace rcx
{
namespace
{

constexpr int kBlock = 256;
constexpr int kItems = 8;
constexpr int kTile = kBlock * kItems;  // keys per radix-sort tile / scan block

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

__global__ void k_prep(const double* __restrict__ v, int n, float4* __restrict__ lo, float4* __restrict__ hi,
                       float4* __restrict__ cen, float4* __restrict__ blockLo, float4* __restrict__ blockHi)
{
    __shared__ float sLo[3][kBlock];
    __shared__ float sHi[3][kBlock];
    const int i = blockIdx.x * kBlock + threadIdx.x;
    float c[3] = { FLT_MAX, FLT_MAX, FLT_MAX };
    float d[3] = { -FLT_MAX, -FLT_MAX, -FLT_MAX };
    if (i < n)
    {
        float f[9];
        for (int k = 0; k < 9; ++k)
            f[k] = float(v[size_t(i) * 9 + k]);  // round to nearest, as the host's float(t[k])
        float mn[3], mx[3], ce[3];
        for (int a = 0; a < 3; ++a)
        {
            mn[a] = fminf(f[a], fminf(f[3 + a], f[6 + a]));
            mx[a] = fmaxf(f[a], fmaxf(f[3 + a], f[6 + a]));
            ce[a] = 0.5f * (mn[a] + mx[a]);
            c[a] = ce[a];
            d[a] = ce[a];
        }
        lo[i] = make_float4(mn[0], mn[1], mn[2], 0.0f);
        hi[i] = make_float4(mx[0], mx[1], mx[2], 0.0f);
        cen[i] = make_float4(ce[0], ce[1], ce[2], 0.0f);
    }
    for (int a = 0; a < 3; ++a)
    {
        sLo[a][threadIdx.x] = c[a];
        sHi[a][threadIdx.x] = d[a];
    }
    __syncthreads();
    for (int s = kBlock / 2; s > 0; s >>= 1)
    {
        if (int(threadIdx.x) < s)
            for (int a = 0; a < 3; ++a)
            {
                sLo[a][threadIdx.x] = fminf(sLo[a][threadIdx.x], sLo[a][threadIdx.x + s]);
                sHi[a][threadIdx.x] = fmaxf(sHi[a][threadIdx.x], sHi[a][threadIdx.x + s]);
            }
        __syncthreads();
    }
    if (threadIdx.x == 0)
    {
        blockLo[blockIdx.x] = make_float4(sLo[0][0], sLo[1][0], sLo[2][0], 0.0f);
        blockHi[blockIdx.x] = make_float4(sHi[0][0], sHi[1][0], sHi[2][0], 0.0f);
    }
}

__global__ void k_bounds_final(const float4* __restrict__ blockLo, const float4* __restrict__ blockHi, int blocks,
                               float4* __restrict__ out)
{
    __shared__ float sLo[3][kBlock];
    __shared__ float sHi[3][kBlock];
    float c[3] = { FLT_MAX, FLT_MAX, FLT_MAX };
    float d[3] = { -FLT_MAX, -FLT_MAX, -FLT_MAX };
    for (int b = threadIdx.x; b < blocks; b += kBlock)
    {
        float4 l = blockLo[b], h = blockHi[b];
        c[0] = fminf(c[0], l.x);
        c[1] = fminf(c[1], l.y);
        c[2] = fminf(c[2], l.z);
        d[0] = fmaxf(d[0], h.x);
        d[1] = fmaxf(d[1], h.y);
        d[2] = fmaxf(d[2], h.z);
    }
    for (int a = 0; a < 3; ++a)
    {
        sLo[a][threadIdx.x] = c[a];
        sHi[a][threadIdx.x] = d[a];
    }
    __syncthreads();
    for (int s = kBlock / 2; s > 0; s >>= 1)
    {
        if (int(threadIdx.x) < s)
            for (int a = 0; a < 3; ++a)
            {
                sLo[a][threadIdx.x] = fminf(sLo[a][threadIdx.x], sLo[a][threadIdx.x + s]);
                sHi[a][threadIdx.x] = fmaxf(sHi[a][threadIdx.x], sHi[a][threadIdx.x + s]);
            }
        __syncthreads();
    }
    if (threadIdx.x == 0)
    {
        out[0] = make_float4(sLo[0][0], sLo[1][0], sLo[2][0], 0.0f);
        out[1] = make_float4(sHi[0][0], sHi[1][0], sHi[2][0], 0.0f);
    }
}

// 10 bits of x spread to every third bit.
__device__ __forceinline__ uint32_t spread3(uint32_t x)
{
    x = (x * 0x00010001u) & 0xFF0000FFu;
    x = (x * 0x00000101u) & 0x0F00F00Fu;
    x = (x * 0x00000011u) & 0xC30C30C3u;
    x = (x * 0x00000005u) & 0x49249249u;
    return x;
}

__global__ void k_morton(const float4* __restrict__ cen, int n, const float4* __restrict__ box,
                         uint32_t* __restrict__ keys, uint32_t* __restrict__ vals)
{
    const int i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= n)
        return;
    const float4 lo = box[0], hi = box[1], c = cen[i];
    // one scale for all axes (the largest extent): cells are cubes, so a flat
    // scene's thin axis only splits where the cells have become that small
    // (scaling each axis to its own extent would split a heightfield by
    // height at the second level, into boxes that overlap everywhere)
    const float ext = fmaxf(fmaxf(hi.x - lo.x, hi.y - lo.y), hi.z - lo.z);
    const float inv = ext > 0.0f ? 1024.0f / ext : 0.0f;
    const float p[3] = { c.x - lo.x, c.y - lo.y, c.z - lo.z };
    uint32_t q[3];
    for (int a = 0; a < 3; ++a)
        q[a] = uint32_t(fminf(fmaxf(p[a] * inv, 0.0f), 1023.0f));
    keys[i] = (spread3(q[0]) << 2) | (spread3(q[1]) << 1) | spread3(q[2]);
    vals[i] = uint32_t(i);
}

// ---- exclusive scan of uint32 (in place), kTile elements per block

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t x, uint32_t* sWarp, uint32_t& total)
{
    const int lane = int(lane_id()), warp = int(threadIdx.x >> 5);
    uint32_t incl = x;
    for (int o = 1; o < 32; o <<= 1)
    {
        uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o)
            incl += y;
    }
    if (lane == 31)
        sWarp[warp] = incl;
    __syncthreads();
    if (warp == 0)
    {
        uint32_t w = lane < kBlock / 32 ? sWarp[lane] : 0u;
        uint32_t wi = w;
        for (int o = 1; o < 32; o <<= 1)
        {
            uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o)
                wi += y;
        }
        if (lane < kBlock / 32)
            sWarp[lane] = wi - w;
        if (lane == kBlock / 32 - 1)
            sWarp[kBlock / 32] = wi;
    }
    __syncthreads();
    total = sWarp[kBlock / 32];
    const uint32_t r = sWarp[warp] + incl - x;
    __syncthreads();
    return r;
}

__global__ void k_scan_blocks(uint32_t* __restrict__ data, size_t m, uint32_t* __restrict__ sums)
{
    __shared__ uint32_t sWarp[kBlock / 32 + 1];
    const size_t base = size_t(blockIdx.x) * kTile + size_t(threadIdx.x) * kItems;
    uint32_t v[kItems];
    uint32_t s = 0;
    for (int k = 0; k < kItems; ++k)
    {
        v[k] = base + k < m ? data[base + k] : 0u;
        s += v[k];
    }
    uint32_t total;
    uint32_t run = block_exclusive_scan(s, sWarp, total);
    for (int k = 0; k < kItems; ++k)
    {
        if (base + k < m)
            data[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == 0 && sums)
        sums[blockIdx.x] = total;
}

__global__ void k_scan_add(uint32_t* __restrict__ data, size_t m, const uint32_t* __restrict__ sums)
{
    const uint32_t add = sums[blockIdx.x];
    const size_t base = size_t(blockIdx.x) * kTile + size_t(threadIdx.x) * kItems;
    for (int k = 0; k < kItems; ++k)
        if (base + k < m)
            data[base + k] += add;
}

// ---- radix sort pass (8-bit digit at `shift`)

__global__ void k_rs_hist(const uint32_t* __restrict__ keys, int n, int shift, int tiles, uint32_t* __restrict__ hist)
{
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const size_t base = size_t(blockIdx.x) * kTile;
    for (int j = 0; j < kItems; ++j)
    {
        const size_t i = base + size_t(j) * kBlock + threadIdx.x;
        if (i < size_t(n))
            atomicAdd(&h[(keys[i] >> shift) & 0xffu], 1u);
    }
    __syncthreads();
    hist[size_t(threadIdx.x) * size_t(tiles) + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter: items of a tile are taken in index order, 256 at a time;
// rank = items of the same digit earlier in the tile.
__global__ void k_rs_scatter(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ vals, int n, int shift,
                             int tiles, const uint32_t* __restrict__ offsets, uint32_t* __restrict__ keysOut,
                             uint32_t* __restrict__ valsOut)
{
    __shared__ uint32_t running[256];
    __shared__ uint32_t warpCount[kBlock / 32][256];
    const int warp = int(threadIdx.x >> 5), lane = int(lane_id());
    running[threadIdx.x] = 0;
    for (int w = 0; w < kBlock / 32; ++w)
        warpCount[w][threadIdx.x] = 0;
    __syncthreads();
    const uint32_t lanesBelow = (1u << lane) - 1u;
    const size_t base = size_t(blockIdx.x) * kTile;
    for (int j = 0; j < kItems; ++j)
    {
        const size_t i = base + size_t(j) * kBlock + threadIdx.x;
        const bool valid = i < size_t(n);
        uint32_t key = 0, val = 0, d = 0;
        if (valid)
        {
            key = keys[i];
            val = vals[i];
            d = (key >> shift) & 0xffu;
        }
        // invalid items get a value no valid digit has, unique per lane
        const uint32_t tag = valid ? d : 0x100u + uint32_t(lane);
        const uint32_t peers = __match_any_sync(0xffffffffu, tag);
        const uint32_t rankInWarp = __popc(peers & lanesBelow);
        if (valid && rankInWarp == 0)
            warpCount[warp][d] = __popc(peers);
        __syncthreads();
        if (valid)
        {
            uint32_t r = running[d] + rankInWarp;
            for (int w = 0; w < warp; ++w)
                r += warpCount[w][d];
            const size_t dst = size_t(offsets[size_t(d) * size_t(tiles) + blockIdx.x]) + r;
            keysOut[dst] = key;
            valsOut[dst] = val;
        }
        __syncthreads();
        uint32_t add = 0;
        for (int w = 0; w < kBlock / 32; ++w)
        {
            add += warpCount[w][threadIdx.x];
            warpCount[w][threadIdx.x] = 0;
        }
        running[threadIdx.x] += add;
        __syncthreads();
    }
}

// ---- hierarchy (Karras 2012, section 4)

__device__ __forceinline__ int common_prefix(const uint32_t* __restrict__ k, int n, int i, int j)
{
    if (j < 0 || j >= n)
        return -1;
    const uint32_t a = k[i], b = k[j];
    if (a == b)
        return 32 + __clz(uint32_t(i) ^ uint32_t(j));
    return __clz(a ^ b);
}

// child encoding: >= 0 internal node, < 0 ~leaf (sorted triangle index)
__global__ void k_hierarchy(const uint32_t* __restrict__ keys, int n, int2* __restrict__ child,
                            int2* __restrict__ range, int* __restrict__ parent, int* __restrict__ leafParent)
{
    const int i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= n - 1)
        return;
    const int d = common_prefix(keys, n, i, i + 1) - common_prefix(keys, n, i, i - 1) >= 0 ? 1 : -1;
    const int dMin = common_prefix(keys, n, i, i - d);
    int lMax = 2;
    while (common_prefix(keys, n, i, i + lMax * d) > dMin)
        lMax <<= 1;
    int l = 0;
    for (int t = lMax >> 1; t >= 1; t >>= 1)
        if (common_prefix(keys, n, i, i + (l + t) * d) > dMin)
            l += t;
    const int j = i + l * d;
    const int dNode = common_prefix(keys, n, i, j);
    int s = 0;
    int t = l;
    do
    {
        t = (t + 1) >> 1;
        if (common_prefix(keys, n, i, i + (s + t) * d) > dNode)
            s += t;
    } while (t > 1);
    const int gamma = i + s * d + (d < 0 ? -1 : 0);
    const int first = min(i, j), last = max(i, j);
    const int left = first == gamma ? ~gamma : gamma;
    const int right = last == gamma + 1 ? ~(gamma + 1) : gamma + 1;
    child[i] = make_int2(left, right);
    range[i] = make_int2(first, last);
    if (left >= 0)
        parent[left] = i;
    else
        leafParent[gamma] = i;
    if (right >= 0)
        parent[right] = i;
    else
        leafParent[gamma + 1] = i;
}

__device__ __forceinline__ float4 ld_cg(const float4* p) { return __ldcg(p); }

// Bottom-up boxes and heights. visits[] must be zero.
__global__ void k_boxes(int n, const uint32_t* __restrict__ sortedTri, const float4* __restrict__ triLo,
                        const float4* __restrict__ triHi, const int2* __restrict__ child,
                        const int* __restrict__ parent, const int* __restrict__ leafParent,
                        unsigned* __restrict__ visits, float4* __restrict__ nodeLo, float4* __restrict__ nodeHi,
                        int* __restrict__ height, float4* __restrict__ leafLo, float4* __restrict__ leafHi)
{
    const int i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= n)
        return;
    const uint32_t tri = sortedTri[i];
    leafLo[i] = triLo[tri];
    leafHi[i] = triHi[tri];
    int p = n > 1 ? leafParent[i] : -1;
    while (p >= 0)
    {
        __threadfence();
        if (atomicAdd(&visits[p], 1u) == 0u)
            return;  // the sibling subtree is not finished; its thread continues
        __threadfence();
        const int2 c = child[p];
        float4 l0, h0, l1, h1;
        int hl = 0, hr = 0;
        if (c.x < 0)
        {
            l0 = ld_cg(&leafLo[~c.x]);
            h0 = ld_cg(&leafHi[~c.x]);
        }
        else
        {
            l0 = ld_cg(&nodeLo[c.x]);
            h0 = ld_cg(&nodeHi[c.x]);
            hl = __ldcg(&height[c.x]);
        }
        if (c.y < 0)
        {
            l1 = ld_cg(&leafLo[~c.y]);
            h1 = ld_cg(&leafHi[~c.y]);
        }
        else
        {
            l1 = ld_cg(&nodeLo[c.y]);
            h1 = ld_cg(&nodeHi[c.y]);
            hr = __ldcg(&height[c.y]);
        }
        nodeLo[p] = make_float4(fminf(l0.x, l1.x), fminf(l0.y, l1.y), fminf(l0.z, l1.z), 0.0f);
        nodeHi[p] = make_float4(fmaxf(h0.x, h1.x), fmaxf(h0.y, h1.y), fmaxf(h0.z, h1.z), 0.0f);
        height[p] = 1 + max(hl, hr);
        p = p == 0 ? -1 : parent[p];
    }
}

__global__ void k_keep(const int2* __restrict__ range, int count, int leafMax, uint32_t* __restrict__ keep)
{
    const int i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= count)
        return;
    const int2 r = range[i];
    keep[i] = (r.y - r.x + 1) > leafMax ? 1u : 0u;
}

__device__ __forceinline__ int leaf_link(int first, int count) { return ~((first << kLeafCountBits) | count); }

// Device nodes of the kept internal nodes; index = exclusive scan of keep.
__global__ void k_emit(int count, int leafMax, const int2* __restrict__ child, const int2* __restrict__ range,
                       const uint32_t* __restrict__ keepScan, const float4* __restrict__ nodeLo,
                       const float4* __restrict__ nodeHi, const float4* __restrict__ leafLo,
                       const float4* __restrict__ leafHi, DevNode* __restrict__ out, int2* __restrict__ outRange)
{
    const int i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= count)
        return;
    const int2 r = range[i];
    if (r.y - r.x + 1 <= leafMax)
        return;
    const int2 c = child[i];
    float4 lo[2], hi[2];
    int link[2];
    const int cs[2] = { c.x, c.y };
    for (int k = 0; k < 2; ++k)
    {
        const int ch = cs[k];
        if (ch < 0)
        {
            lo[k] = leafLo[~ch];
            hi[k] = leafHi[~ch];
            link[k] = leaf_link(~ch, 1);
        }
        else
        {
            lo[k] = nodeLo[ch];
            hi[k] = nodeHi[ch];
            const int2 cr = range[ch];
            const int cnt = cr.y - cr.x + 1;
            link[k] = cnt > leafMax ? int(keepScan[ch]) : leaf_link(cr.x, cnt);
        }
    }
    DevNode d;
    d.xy0 = make_float4(lo[0].x, hi[0].x, lo[0].y, hi[0].y);
    d.xy1 = make_float4(lo[1].x, hi[1].x, lo[1].y, hi[1].y);
    d.z01 = make_float4(lo[0].z, hi[0].z, lo[1].z, hi[1].z);
    d.link = make_int4(link[0], link[1], 0, 0);
    out[keepScan[i]] = d;
    outRange[keepScan[i]] = make_int2(r.x, r.y - r.x + 1);
}

// Triangle and shading records in sorted order (tracer_host.cpp's host
// arithmetic: float32 vertices and edges, float64 frame with every
// operation rounded separately).
__global__ void k_tri_records(const double* __restrict__ v, const uint32_t* __restrict__ matIdx,
                              const DevMat* __restrict__ mats, const uint32_t* __restrict__ sortedTri, int n,
                              DevTri* __restrict__ tris, DevShade* __restrict__ shade)
{
    const int s = blockIdx.x * kBlock + threadIdx.x;
    if (s >= n)
        return;
    const uint32_t p = sortedTri[s];
    const double* t = v + size_t(p) * 9;
    float f[9];
    double dd[9];
    for (int k = 0; k < 9; ++k)
    {
        dd[k] = t[k];
        f[k] = float(dd[k]);
    }
    const float e1x = __fsub_rn(f[3], f[0]), e1y = __fsub_rn(f[4], f[1]), e1z = __fsub_rn(f[5], f[2]);
    const float e2x = __fsub_rn(f[6], f[0]), e2y = __fsub_rn(f[7], f[1]), e2z = __fsub_rn(f[8], f[2]);
    const uint32_t m = matIdx[p];
    const uint32_t matFlags = __float_as_uint(mats[m].emittance.w);
    const uint32_t meta = m | ((matFlags & kMatNonShadowing) ? kMetaNonShadowing : 0u);
    DevTri d;
    d.a = make_float4(f[0], f[1], f[2], e1x);
    d.b = make_float4(e1y, e1z, e2x, e2y);
    d.c = make_float4(e2z, __uint_as_float(meta), __int_as_float(int32_t(p)), 0.0f);
    tris[s] = d;

    // normal = normalize((b - a) x (c - a)); tangent = normalize(normal x
    // (0.0001, 1, 0.0001)); bitangent = normalize(tangent x normal)
    auto cross = [](double ax, double ay, double az, double bx, double by, double bz, double* o) {
        o[0] = __dsub_rn(__dmul_rn(ay, bz), __dmul_rn(az, by));
        o[1] = __dsub_rn(__dmul_rn(az, bx), __dmul_rn(ax, bz));
        o[2] = __dsub_rn(__dmul_rn(ax, by), __dmul_rn(ay, bx));
    };
    auto normalize = [](double* o) {
        const double len = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(o[0], o[0]), __dmul_rn(o[1], o[1])),
                                                __dmul_rn(o[2], o[2])));
        const double inv = __ddiv_rn(1.0, len);
        o[0] = __dmul_rn(o[0], inv);
        o[1] = __dmul_rn(o[1], inv);
        o[2] = __dmul_rn(o[2], inv);
    };
    double nrm[3], tan[3], bit[3];
    cross(__dsub_rn(dd[3], dd[0]), __dsub_rn(dd[4], dd[1]), __dsub_rn(dd[5], dd[2]), __dsub_rn(dd[6], dd[0]),
          __dsub_rn(dd[7], dd[1]), __dsub_rn(dd[8], dd[2]), nrm);
    normalize(nrm);
    cross(nrm[0], nrm[1], nrm[2], 0.0001, 1.0, 0.0001, tan);
    normalize(tan);
    cross(tan[0], tan[1], tan[2], nrm[0], nrm[1], nrm[2], bit);
    normalize(bit);
    DevShade sh;
    sh.n = make_float4(float(nrm[0]), float(nrm[1]), float(nrm[2]), 0.0f);
    sh.t = make_float4(float(tan[0]), float(tan[1]), float(tan[2]), 0.0f);
    sh.bt = make_float4(float(bit[0]), float(bit[1]), float(bit[2]), 0.0f);
    shade[s] = sh;
}

unsigned grid_of(size_t count, int per) { return unsigned((count + size_t(per) - 1) / size_t(per)); }

}  // namespace

namespace
{

struct Carver
{
    char* p;
    template <typename T>
    T* take(size_t count)
    {
        uintptr_t a = (reinterpret_cast<uintptr_t>(p) + 255) & ~uintptr_t(255);
        T* r = reinterpret_cast<T*>(a);
        p = reinterpret_cast<char*>(a + count * sizeof(T));
        return r;
    }
};

// The scratch arrays of a build of n triangles (the same layout every call).
struct Scratch
{
    float4 *triLo, *triHi, *cen, *blockLo, *blockHi, *box;
    uint32_t *keysA, *valsA, *keysB, *valsB, *hist, *scanTmp;
    int2 *child, *range;
    int *parent, *leafParent, *height;
    unsigned* visits;
    float4 *nodeLo, *nodeHi, *leafLo, *leafHi;
    uint32_t* keep;
    uint32_t* counts;  // [0] last keep flag, [1] its scan value, [2] root height
    char* end;
};

Scratch carve(void* base, size_t N)
{
    const size_t tiles = (N + kTile - 1) / kTile;
    const size_t prepBlocks = (N + kBlock - 1) / kBlock;
    Carver c{ static_cast<char*>(base) };
    Scratch s;
    s.triLo = c.take<float4>(N);
    s.triHi = c.take<float4>(N);
    s.cen = c.take<float4>(N);
    s.blockLo = c.take<float4>(prepBlocks);
    s.blockHi = c.take<float4>(prepBlocks);
    s.box = c.take<float4>(2);
    s.keysA = c.take<uint32_t>(N);
    s.valsA = c.take<uint32_t>(N);
    s.keysB = c.take<uint32_t>(N);
    s.valsB = c.take<uint32_t>(N);
    s.hist = c.take<uint32_t>(256 * tiles);
    s.scanTmp = c.take<uint32_t>(2 * tiles + 2 * kTile + 16);
    s.child = c.take<int2>(N);
    s.range = c.take<int2>(N);
    s.parent = c.take<int>(N);
    s.leafParent = c.take<int>(N);
    s.height = c.take<int>(N);
    s.visits = c.take<unsigned>(N);
    s.nodeLo = c.take<float4>(N);
    s.nodeHi = c.take<float4>(N);
    s.leafLo = c.take<float4>(N);
    s.leafHi = c.take<float4>(N);
    s.keep = c.take<uint32_t>(N);
    s.counts = c.take<uint32_t>(4);
    s.end = c.p;
    return s;
}

// Exclusive scan of m values in place (levels of kTile-element blocks);
// tmp needs ceil(m / kTile) + ceil(m / kTile^2) + ... entries.
cudaError_t scan_u32(uint32_t* data, size_t m, uint32_t* tmp, cudaStream_t stream)
{
    const unsigned blocks = grid_of(m, kTile);
    if (blocks <= 1)
    {
        k_scan_blocks<<<1, kBlock, 0, stream>>>(data, m, nullptr);
        return cudaGetLastError();
    }
    uint32_t* sums = tmp;
    k_scan_blocks<<<blocks, kBlock, 0, stream>>>(data, m, sums);
    cudaError_t e = scan_u32(sums, blocks, tmp + blocks, stream);
    if (e != cudaSuccess)
        return e;
    k_scan_add<<<blocks, kBlock, 0, stream>>>(data, m, sums);
    return cudaGetLastError();
}

}  // namespace

size_t gpu_build_scratch_bytes(int64_t n)
{
    Scratch s = carve(nullptr, size_t(n));
    return size_t(s.end - static_cast<char*>(nullptr)) + 256;
}

cudaError_t gpu_build_hierarchy(const GpuBuildInput& in, void* scratch, cudaStream_t stream)
{
    const int n = int(in.n);
    const size_t N = size_t(in.n);
    const size_t tiles = (N + kTile - 1) / kTile;
    Scratch s = carve(scratch, N);
    const unsigned prepBlocks = grid_of(N, kBlock);
    cudaError_t e;
    k_prep<<<prepBlocks, kBlock, 0, stream>>>(in.vertices, n, s.triLo, s.triHi, s.cen, s.blockLo, s.blockHi);
    k_bounds_final<<<1, kBlock, 0, stream>>>(s.blockLo, s.blockHi, int(prepBlocks), s.box);
    k_morton<<<grid_of(N, kBlock), kBlock, 0, stream>>>(s.cen, n, s.box, s.keysA, s.valsA);
    if ((e = cudaGetLastError()) != cudaSuccess)
        return e;
    uint32_t *ka = s.keysA, *va = s.valsA, *kb = s.keysB, *vb = s.valsB;
    for (int shift = 0; shift < 32; shift += 8)
    {
        k_rs_hist<<<unsigned(tiles), kBlock, 0, stream>>>(ka, n, shift, int(tiles), s.hist);
        if ((e = scan_u32(s.hist, 256 * tiles, s.scanTmp, stream)) != cudaSuccess)
            return e;
        k_rs_scatter<<<unsigned(tiles), kBlock, 0, stream>>>(ka, va, n, shift, int(tiles), s.hist, kb, vb);
        if ((e = cudaGetLastError()) != cudaSuccess)
            return e;
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    // four passes: the sorted pairs are back in keysA / valsA
    if ((e = cudaMemsetAsync(s.counts, 0, 4 * sizeof(uint32_t), stream)) != cudaSuccess)
        return e;
    if (n > 1)
    {
        k_hierarchy<<<grid_of(N - 1, kBlock), kBlock, 0, stream>>>(s.keysA, n, s.child, s.range, s.parent,
                                                                   s.leafParent);
        if ((e = cudaMemsetAsync(s.visits, 0, N * sizeof(unsigned), stream)) != cudaSuccess)
            return e;
    }
    k_boxes<<<grid_of(N, kBlock), kBlock, 0, stream>>>(n, s.valsA, s.triLo, s.triHi, s.child, s.parent,
                                                       s.leafParent, s.visits, s.nodeLo, s.nodeHi, s.height,
                                                       s.leafLo, s.leafHi);
    if (n > 1)
    {
        k_keep<<<grid_of(N - 1, kBlock), kBlock, 0, stream>>>(s.range, n - 1, in.leafMax, s.keep);
        if ((e = cudaMemcpyAsync(s.counts + 0, s.keep + (N - 2), sizeof(uint32_t), cudaMemcpyDeviceToDevice,
                                 stream)) != cudaSuccess)
            return e;
        if ((e = scan_u32(s.keep, N - 1, s.scanTmp, stream)) != cudaSuccess)
            return e;
        if ((e = cudaMemcpyAsync(s.counts + 1, s.keep + (N - 2), sizeof(uint32_t), cudaMemcpyDeviceToDevice,
                                 stream)) != cudaSuccess)
            return e;
        if ((e = cudaMemcpyAsync(s.counts + 2, s.height, sizeof(uint32_t), cudaMemcpyDeviceToDevice, stream)) !=
            cudaSuccess)
            return e;
    }
    return cudaGetLastError();
}

const uint32_t* gpu_build_counts(void* scratch, int64_t n) { return carve(scratch, size_t(n)).counts; }

cudaError_t gpu_build_emit(const GpuBuildInput& in, void* scratch, DevNode* nodes, int2* nodeRange, DevTri* tris,
                           DevShade* shade, uint32_t* order, cudaStream_t stream)
{
    const int n = int(in.n);
    const size_t N = size_t(in.n);
    Scratch s = carve(scratch, N);
    if (n > 1)
        k_emit<<<grid_of(N - 1, kBlock), kBlock, 0, stream>>>(n - 1, in.leafMax, s.child, s.range, s.keep, s.nodeLo,
                                                              s.nodeHi, s.leafLo, s.leafHi, nodes, nodeRange);
    k_tri_records<<<grid_of(N, kBlock), kBlock, 0, stream>>>(in.vertices, in.matIdx, in.mats, s.valsA, n, tris,
                                                             shade);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    return cudaMemcpyAsync(order, s.valsA, N * sizeof(uint32_t), cudaMemcpyDeviceToDevice, stream);
}

}  // namespace rcx
