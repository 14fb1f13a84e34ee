// Test infrastructure only: NOT part of the product (see oracle.h).
// C entry points of the oracle for the Python tests (oracle/__init__.py).

#include <omp.h>

#include <chrono>
#include <cstring>
#include <memory>

#include "oracle.h"
#include "oracle32.h"
#include "oracle64.h"

using namespace oracle;

namespace
{

struct Handle
{
    Scene64 s64;
    Scene32 s32;
};

Handle* H(void* h) { return static_cast<Handle*>(h); }

Camera64 cam64(const double* c)
{
    // position, right, up, image-plane centre (3 each), aspect, ipw, iph
    Camera64 k;
    k.pos = V3d{ c[0], c[1], c[2] };
    k.right = V3d{ c[3], c[4], c[5] };
    k.up = V3d{ c[6], c[7], c[8] };
    k.center = V3d{ c[9], c[10], c[11] };
    k.aspect = c[12];
    k.ipw = c[13];
    k.iph = c[14];
    return k;
}

Camera32 cam32(const float* c)
{
    // rc_camera layout: position, forward, right, up, centre, aspect, ipw, iph
    Camera32 k;
    for (int i = 0; i < 3; ++i)
    {
        k.pos[i] = c[i];
        k.fwd[i] = c[3 + i];
        k.right[i] = c[6 + i];
        k.up[i] = c[9 + i];
        k.center[i] = c[12 + i];
    }
    k.aspect = c[15];
    k.ipw = c[16];
    k.iph = c[17];
    return k;
}

}  // namespace

extern "C" {

// Scene: v n*9 doubles, mat n indices, materials (diffuse 3, emittance 3,
// flags) x m. prebuiltNodes/order: optional reference-form BVH (10 doubles
// per node: min xyz, max xyz, rightOffset, start, count as doubles... see
// or_scene_set_bvh); when absent the BVH is built (FlatBVH::build).
void or_scene_set_ior(void* hp, const float* ior, int32_t m)
{
    auto* h = static_cast<Handle*>(hp);
    for (int32_t i = 0; i < m && size_t(i) < h->s64.mats.size(); ++i)
        h->s64.mats[size_t(i)].ior = ior[i];
}

void* or_scene_new(const double* v, const uint32_t* mat, int64_t n, const float* diffuse, const float* emittance,
                   const int32_t* flags, int32_t m, uint32_t maxLeafSize, int build)
{
    auto h = std::make_unique<Handle>();
    h->s64.v.assign(v, v + n * 9);
    h->s64.mat.assign(mat, mat + n);
    h->s64.mats.resize(size_t(m));
    for (int32_t i = 0; i < m; ++i)
    {
        for (int k = 0; k < 3; ++k)
        {
            h->s64.mats[size_t(i)].diffuse[k] = diffuse[i * 3 + k];
            h->s64.mats[size_t(i)].emittance[k] = emittance[i * 3 + k];
        }
        h->s64.mats[size_t(i)].flags = flags[i];
    }
    h->s64.maxLeafSize = maxLeafSize;
    compute_frames(h->s64);
    if (build)
    {
        build_bvh(h->s64);
        make_scene32(h->s64, h->s32);
    }
    return h.release();
}

// Installs a prebuilt BVH (FlatBVH::restore, FlatBVH.cpp:206-214).
void or_scene_set_bvh(void* hp, int64_t nodeCount, const double* aabb6, const int64_t* right, const uint64_t* start,
                      const uint64_t* count, const uint64_t* order)
{
    Handle* h = H(hp);
    h->s64.nodes.resize(size_t(nodeCount));
    for (int64_t i = 0; i < nodeCount; ++i)
    {
        Node64& nd = h->s64.nodes[size_t(i)];
        for (int k = 0; k < 3; ++k)
        {
            nd.bmin[k] = aabb6[i * 6 + k];
            nd.bmax[k] = aabb6[i * 6 + 3 + k];
        }
        nd.rightOffset = right[i];
        nd.start = start[i];
        nd.count = count[i];
    }
    h->s64.order.assign(order, order + h->s64.mat.size());
    make_scene32(h->s64, h->s32);
}

void or_scene_free(void* h) { delete H(h); }

int64_t or_bvh_node_count(void* h) { return int64_t(H(h)->s64.nodes.size()); }

void or_bvh_nodes(void* hp, double* aabb6, int64_t* right, uint64_t* start, uint64_t* count, uint64_t* order)
{
    const Scene64& s = H(hp)->s64;
    for (size_t i = 0; i < s.nodes.size(); ++i)
    {
        for (int k = 0; k < 3; ++k)
        {
            aabb6[i * 6 + size_t(k)] = s.nodes[i].bmin[k];
            aabb6[i * 6 + 3 + size_t(k)] = s.nodes[i].bmax[k];
        }
        right[i] = s.nodes[i].rightOffset;
        start[i] = s.nodes[i].start;
        count[i] = s.nodes[i].count;
    }
    for (size_t i = 0; i < s.order.size(); ++i)
        order[i] = s.order[i];
}

void or_frames(void* hp, double* out)
{
    const Scene64& s = H(hp)->s64;
    std::memcpy(out, s.frame.data(), s.frame.size() * sizeof(double));
}

// ---- float64 restatement -------------------------------------------------

void or64_intersect(void* hp, int64_t n, const double* rays6, int shadow, int64_t* prim, double* t, double* u,
                    double* v, int threads)
{
    const Scene64& s = H(hp)->s64;
    if (threads > 0)
        omp_set_num_threads(threads);
    #pragma omp parallel for schedule(dynamic, 1000)
    for (int64_t i = 0; i < n; ++i)
    {
        Ray64 r = make_ray64(V3d{ rays6[i * 6], rays6[i * 6 + 1], rays6[i * 6 + 2] },
                             V3d{ rays6[i * 6 + 3], rays6[i * 6 + 4], rays6[i * 6 + 5] });
        if (shadow)
        {
            r.shadow = true;
            r.fastOcclusion = true;
        }
        Isect64 is;
        intersect64(s, r, is);
        prim[i] = is.found ? is.caller : -1;
        t[i] = is.found ? is.t : -1.0;
        u[i] = is.u;
        v[i] = is.v;
    }
}

// One triangle against one ray (float64, Triangle::intersect): returns 1 on a
// hit with t, u, v.
int or64_tri(void* hp, int64_t caller, const double* ray6, double* t, double* u, double* v)
{
    const Scene64& s = H(hp)->s64;
    Ray64 r = make_ray64(V3d{ ray6[0], ray6[1], ray6[2] }, V3d{ ray6[3], ray6[4], ray6[5] });
    Isect64 is;
    if (!tri_intersect64(s, uint64_t(caller), r, is))
        return 0;
    *t = is.t;
    *u = is.u;
    *v = is.v;
    return 1;
}

double or64_raycast(void* hp, const double* cam, uint64_t width, uint64_t pixelStart, uint64_t count,
                    const double* dirToLight, double rayStartOffset, int64_t* prim, double* t, int64_t* occluder,
                    int threads, uint64_t* rays)
{
    auto t0 = std::chrono::steady_clock::now();
    raycast64(H(hp)->s64, cam64(cam), width, pixelStart, count, dirToLight, rayStartOffset, prim, t, occluder, threads,
              rays);
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

double or64_render_path(void* hp, const double* cam, uint64_t width, uint64_t pixelStart, uint64_t count,
                        uint64_t maxPathLength, uint64_t pathSampleCount, uint64_t msSqrt, int samplerType, double rx,
                        double ry, double rayStartOffset, uint32_t seed, int threads, double* film, uint64_t* rays,
                        int filterType)
{
    PathSettings64 ps;
    ps.filterType = filterType;
    ps.maxPathLength = maxPathLength;
    ps.pathSampleCount = pathSampleCount;
    ps.multiSampleCountSqrt = msSqrt;
    ps.samplerType = samplerType;
    ps.filterRadius[0] = rx;
    ps.filterRadius[1] = ry;
    ps.rayStartOffset = rayStartOffset;
    auto t0 = std::chrono::steady_clock::now();
    render_path64(H(hp)->s64, cam64(cam), ps, width, pixelStart, count, film, threads, seed, rays);
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

void or64_tonemap(int64_t pixels, const float* linear, double key, double gamma, int shouldClamp, int applyGamma,
                  float* out)
{
    tonemap_reinhard64(pixels, linear, key, gamma, shouldClamp, applyGamma, out);
}

double or64_fastpow(double a, double b) { return fast_pow64(a, b); }

// ---- float32 twin of the device -----------------------------------------

void or32_cast(void* hp, int64_t n, const float* rays8, int anyHit, int order, int32_t* prim, float* t, float* u,
               float* v, uint64_t* counters, int threads)
{
    cast32(H(hp)->s32, n, rays8, anyHit, order, prim, t, u, v, counters, threads);
}

void or32_raycast(void* hp, const float* cam, uint64_t width, uint64_t pixelStart, uint64_t count, const float* L,
                  float rayStartOffset, int order, int32_t* out4, uint64_t* counters, int threads)
{
    raycast32(H(hp)->s32, cam32(cam), width, pixelStart, count, L, rayStartOffset, order, out4, counters, threads);
}

void or32_camera_rays(const float* cam, uint64_t width, uint64_t pixelStart, uint64_t count, float* rays8)
{
    Camera32 c = cam32(cam);
    for (uint64_t i = 0; i < count; ++i)
    {
        uint64_t px = pixelStart + i;
        V3f d = camera_dir32(c, float(px % width), float(px / width));
        float* r = rays8 + i * 8;
        r[0] = c.pos[0]; r[1] = c.pos[1]; r[2] = c.pos[2]; r[3] = 0.0f;
        r[4] = d.x; r[5] = d.y; r[6] = d.z; r[7] = FLT_MAX;
    }
}

void or32_render_path(void* hp, const float* cam, uint64_t width, uint64_t pixelStart, uint64_t count, int n, int P,
                      int samplerType, float rx, float ry, float rayStartOffset, int maxPathLength, int rrDepth,
                      int order, uint64_t seed, uint32_t frame, float* film, uint64_t* counters, int threads,
                      int filterType)
{
    PathSettings32 ps;
    ps.filterType = filterType;
    ps.n = n;
    ps.P = P;
    ps.samplerType = samplerType;
    ps.rx = rx;
    ps.ry = ry;
    ps.rayStartOffset = rayStartOffset;
    ps.maxPathLength = maxPathLength;
    ps.rrDepth = rrDepth;
    ps.order = order;
    ps.seed = seed;
    ps.frame = frame;
    render_path32(H(hp)->s32, cam32(cam), ps, width, pixelStart, count, film, counters, threads);
}

// CMJSampler::getSample2D restated (float64 port) for given jitter values.
void or64_cmj(uint64_t x, uint64_t y, uint64_t n, uint64_t permutation, double jx, double jy, double* out)
{
    out[0] = cmj_component(x, y, n, permutation, jx, jy, 0);
    out[1] = cmj_component(x, y, n, permutation, jx, jy, 1);
}

uint64_t or32_cmj_permute(uint64_t i, uint64_t l, uint64_t p) { return cmj_permute32(i, l, p); }

// Film filter weights of one axis at offsets x (BOX radius 0.5 for type 0):
// float32 twin of the device and float64 port of the reference.
void or32_filter_weight(int type, int64_t n, const float* x, float* out, float* radius)
{
    Filter32 f = filter32(type, 0.5f, 0.5f);
    for (int64_t i = 0; i < n; ++i)
        out[i] = filter_weight32(f, x[i], f.rx, f.ax, f.bx);
    *radius = f.rx;
}

void or64_filter_weight(int type, int64_t n, const double* x, double* out, double* radius)
{
    const double box[2] = { 0.5, 0.5 };
    double rad[2];
    filter_radius64(type, box, rad);
    for (int64_t i = 0; i < n; ++i)
        out[i] = filter_weight64(type, box, x[i]);
    *radius = rad[0];
}

void or32_filter_exp(int64_t n, const float* t, float* out)
{
    for (int64_t i = 0; i < n; ++i)
        out[i] = filter_exp32(t[i]);
}

void or32_sincos_turn(int64_t n, const float* x, float* s, float* c)
{
    for (int64_t i = 0; i < n; ++i)
        sincos_turn(x[i], s[i], c[i]);
}

}  // extern "C"
