// Test infrastructure only: NOT part of the product (see oracle.h).
//
// float32 twin of the device kernels. It restates the reference's OpenCL
// kernels — intersectAABB / intersectTriangle / intersectBVH
// (data/opencl/intersections.cl:1-148), getCameraRay (camera.cl:1-10),
// getHemisphereSample (sampler.cl:1-14), pathtrace (pathtrace.cl:1-80),
// calculateShadowAmount (lighting.cl:28-48) — over the reference's flat node
// array, with every float operation in the order the CUDA code performs it:
// dot and cross products fused as fma(a.z, b.z, fma(a.y, b.y, a.x * b.x)),
// everything else unfused (this file is compiled with -ffp-contract=off).
// Random numbers, CMJ permutation and sin/cos follow the device's own
// definitions (counter hash, Taylor polynomials), restated here.

#include <omp.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>

#include "oracle.h"
#include "oracle32.h"

namespace oracle
{

namespace
{

inline float bits_f(uint32_t u)
{
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

}  // namespace

void make_scene32(const Scene64& s, Scene32& o)
{
    o.src = &s;
    size_t nn = s.nodes.size();
    o.nodeBox.resize(nn * 6);
    for (size_t i = 0; i < nn; ++i)
        for (int k = 0; k < 3; ++k)
        {
            o.nodeBox[i * 6 + size_t(k)] = float(s.nodes[i].bmin[k]);
            o.nodeBox[i * 6 + 3 + size_t(k)] = float(s.nodes[i].bmax[k]);
        }
    size_t n = s.order.size();
    o.tri.resize(n * 9);
    o.meta.resize(n);
    o.caller.resize(n);
    o.shade.resize(n * 9);
    for (size_t slot = 0; slot < n; ++slot)
    {
        uint64_t p = s.order[slot];
        const double* t = &s.v[p * 9];
        float f[9];
        for (int k = 0; k < 9; ++k)
            f[k] = float(t[k]);
        float* d = &o.tri[slot * 9];
        d[0] = f[0]; d[1] = f[1]; d[2] = f[2];
        d[3] = f[3] - f[0]; d[4] = f[4] - f[1]; d[5] = f[5] - f[2];
        d[6] = f[6] - f[0]; d[7] = f[7] - f[1]; d[8] = f[8] - f[2];
        uint32_t m = s.mat[p];
        o.meta[slot] = m | ((s.mats[m].flags & 2) ? 0x80000000u : 0u);
        o.caller[slot] = int32_t(p);
        for (int k = 0; k < 9; ++k)
            o.shade[slot * 9 + size_t(k)] = float(s.frame[p * 9 + size_t(k)]);
    }
}

// ---------------------------------------------------------------------------

V3f cross3(V3f a, V3f b)
{
    return { std::fmaf(a.y, b.z, -(a.z * b.y)), std::fmaf(a.z, b.x, -(a.x * b.z)), std::fmaf(a.x, b.y, -(a.y * b.x)) };
}

float dot3(V3f a, V3f b) { return std::fmaf(a.z, b.z, std::fmaf(a.y, b.y, a.x * b.x)); }

Ray32 make_ray32(V3f o, V3f d, float tmin, float tmax)
{
    Ray32 r;
    r.o = o;
    r.d = d;
    r.inv = { 1.0f / d.x, 1.0f / d.y, 1.0f / d.z };
    r.tmin = tmin;
    r.tmax = tmax;
    return r;
}

namespace
{

// (b < a) ? b : a  and  (a < b) ? b : a — std::min / std::max.
inline float smin(float a, float b) { return (b < a) ? b : a; }
inline float smax(float a, float b) { return (a < b) ? b : a; }

// intersectAABB (intersections.cl:1-25); entry = max(tmin, 0).
bool aabb32(const float* bx, const Ray32& r, float& entry)
{
    float tx0 = (bx[0] - r.o.x) * r.inv.x;
    float tx1 = (bx[3] - r.o.x) * r.inv.x;
    float tmin = smin(tx0, tx1);
    float tmax = smax(tx0, tx1);
    float ty0 = (bx[1] - r.o.y) * r.inv.y;
    float ty1 = (bx[4] - r.o.y) * r.inv.y;
    tmin = smax(tmin, smin(ty0, ty1));
    tmax = smin(tmax, smax(ty0, ty1));
    float tz0 = (bx[2] - r.o.z) * r.inv.z;
    float tz1 = (bx[5] - r.o.z) * r.inv.z;
    tmin = smax(tmin, smin(tz0, tz1));
    tmax = smin(tmax, smax(tz0, tz1));
    entry = smax(tmin, 0.0f);
    return !(tmax < entry);
}

// intersectTriangle (intersections.cl:27-69) up to the distance window.
bool tri32(const float* tr, const Ray32& r, float& t, float& u, float& v)
{
    V3f v0{ tr[0], tr[1], tr[2] }, e1{ tr[3], tr[4], tr[5] }, e2{ tr[6], tr[7], tr[8] };
    V3f pvec = cross3(r.d, e2);
    float det = dot3(e1, pvec);
    if (std::fabs(det) < FLT_EPSILON)
        return false;
    float invDet = 1.0f / det;
    V3f tvec{ r.o.x - v0.x, r.o.y - v0.y, r.o.z - v0.z };
    u = dot3(tvec, pvec) * invDet;
    if (u < 0.0f || u > 1.0f)
        return false;
    V3f qvec = cross3(tvec, e1);
    v = dot3(r.d, qvec) * invDet;
    if (v < 0.0f || (u + v) > 1.0f)
        return false;
    t = dot3(e2, qvec) * invDet;
    if (t < 0.0f)
        return false;
    if (t < r.tmin || t > r.tmax)
        return false;
    return true;
}

}  // namespace

// intersectBVH (intersections.cl:98-148) over the reference's flat node
// array. order 0: the reference's visit order; order 1: nearer child first
// with distance culling (the device's alternative order).
bool traverse32(const Scene32& s, const Ray32& r, bool anyHit, int order, Hit32& h, uint64_t* nodes, uint64_t* tris,
                int64_t skip)
{
    const std::vector<Node64>& N = s.src->nodes;
    struct Entry
    {
        uint64_t idx;
        float dist;
    };
    Entry stack[128];
    int sp = 0;
    uint64_t cur = 0;
    bool found = false;
    bool nearest = (order == 1) && !anyHit;
    while (true)
    {
        const Node64& nd = N[cur];
        bool descended = false;
        if (nd.rightOffset == 0)
        {
            for (uint64_t i = 0; i < nd.count; ++i)
            {
                uint64_t slot = nd.start + i;
                if (int64_t(slot) == skip)
                    continue;
                if (anyHit && (s.meta[slot] & 0x80000000u))
                    continue;
                if (tris)
                    (*tris)++;
                float t, u, v;
                if (tri32(&s.tri[slot * 9], r, t, u, v))
                {
                    if (anyHit)
                    {
                        h.slot = int64_t(slot);
                        h.t = t;
                        h.u = u;
                        h.v = v;
                        return true;
                    }
                    bool take = nearest ? (t < h.t || (t == h.t && int64_t(slot) > h.slot)) : !(t > h.t);
                    if (take)
                    {
                        h.slot = int64_t(slot);
                        h.t = t;
                        h.u = u;
                        h.v = v;
                        found = true;
                    }
                }
            }
        }
        else
        {
            if (nodes)
                (*nodes)++;
            uint64_t l = cur + 1, rr = cur + uint64_t(nd.rightOffset);
            float el, er;
            bool hl = aabb32(&s.nodeBox[l * 6], r, el);
            bool hr = aabb32(&s.nodeBox[rr * 6], r, er);
            if (nearest)
            {
                hl = hl && !(el > h.t);
                hr = hr && !(er > h.t);
            }
            if (hl && hr)
            {
                uint64_t nearC = l, farC = rr;
                float farD = er;
                if (nearest && er < el)
                {
                    nearC = rr;
                    farC = l;
                    farD = el;
                }
                if (sp >= 64)
                    return found;  // the device's stack holds 64 entries
                stack[sp++] = { farC, farD };
                cur = nearC;
                descended = true;
            }
            else if (hl)
            {
                cur = l;
                descended = true;
            }
            else if (hr)
            {
                cur = rr;
                descended = true;
            }
        }
        if (descended)
            continue;
        while (true)
        {
            if (sp == 0)
                return found;
            Entry e = stack[--sp];
            if (nearest && e.dist > h.t)
                continue;
            cur = e.idx;
            break;
        }
    }
}

V3f camera_dir32(const Camera32& c, float px, float py)
{
    float dx = (px / c.ipw) - 0.5f;
    float dy = (py / c.iph) - 0.5f;
    float dya = dy * c.aspect;
    V3f p{ std::fmaf(c.up[0], dya, std::fmaf(c.right[0], dx, c.center[0])),
           std::fmaf(c.up[1], dya, std::fmaf(c.right[1], dx, c.center[1])),
           std::fmaf(c.up[2], dya, std::fmaf(c.right[2], dx, c.center[2])) };
    V3f v{ p.x - c.pos[0], p.y - c.pos[1], p.z - c.pos[2] };
    float len = std::sqrt(dot3(v, v));
    float inv = 1.0f / len;
    return { v.x * inv, v.y * inv, v.z * inv };
}

// ---------------------------------------------------------------------------
// Device sampling restated: lowbias32 hash stream, Taylor sin/cos of 2*pi*x,
// cosine hemisphere, CMJ.

uint32_t mix32(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

uint32_t stream_key(uint64_t seed, uint32_t frame, uint64_t pixel, uint32_t sample)
{
    uint32_t k = mix32(uint32_t(seed) ^ 0x68bc21ebu);
    k = mix32(k ^ uint32_t(seed >> 32));
    k = mix32(k ^ frame);
    k = mix32(k ^ uint32_t(pixel));
    k = mix32(k ^ uint32_t(pixel >> 32));
    k = mix32(k ^ sample);
    return k;
}

uint32_t stream_u32(uint32_t key, uint32_t counter) { return mix32(key ^ mix32(counter + 0x9e3779b9u)); }

float stream_float(uint32_t key, uint32_t counter)
{
    return float(stream_u32(key, counter) >> 8) * 5.9604644775390625e-8f;
}

void sincos_turn(float x, float& s, float& c)
{
    float t = x * 4.0f;
    int q = int(t);
    if (q > 3)
        q = 3;
    float r = t - float(q);
    bool swap = r > 0.5f;
    float a = swap ? (1.0f - r) : r;
    float al = a * 1.57079632679489662f;
    float a2 = al * al;
    float ps = std::fmaf(a2, 2.7557319e-6f, -1.9841270e-4f);
    ps = std::fmaf(a2, ps, 8.3333333e-3f);
    ps = std::fmaf(a2, ps, -1.6666667e-1f);
    ps = std::fmaf(a2, ps, 1.0f);
    float sa = al * ps;
    float pc = std::fmaf(a2, -2.7557319e-7f, 2.4801587e-5f);
    pc = std::fmaf(a2, pc, -1.3888889e-3f);
    pc = std::fmaf(a2, pc, 4.1666667e-2f);
    pc = std::fmaf(a2, pc, -0.5f);
    float ca = std::fmaf(a2, pc, 1.0f);
    float sr = swap ? ca : sa;
    float cr = swap ? sa : ca;
    switch (q)
    {
    case 0: s = sr; c = cr; break;
    case 1: s = cr; c = -sr; break;
    case 2: s = -sr; c = -cr; break;
    default: s = -cr; c = sr; break;
    }
}

// The device's dielectric_bounce (pathtrace.cu): Schlick Fresnel choice,
// mirror reflection or refraction, same operations.
static V3f dielectric32(V3f d, V3f n, float ior, float xi)
{
    const float c = dot3(d, n);
    const bool outside = c < 0.0f;
    const float n1 = outside ? 1.0f : ior;
    const float n2 = outside ? ior : 1.0f;
    const V3f N = outside ? n : V3f{ -n.x, -n.y, -n.z };
    const float ci = std::fabs(c);
    float r0 = (n2 - n1) / (n2 + n1);
    r0 = r0 * r0;
    const float m = 1.0f - ci;
    const float m2 = m * m;
    const float m5 = (m2 * m2) * m;
    const float R = r0 + (1.0f - r0) * m5;
    const float eta = n1 / n2;
    const float k = 1.0f - (eta * eta) * (1.0f - ci * ci);
    if (k <= 0.0f || xi < R)
    {
        const float s2 = 2.0f * ci;
        return V3f{ std::fmaf(N.x, s2, d.x), std::fmaf(N.y, s2, d.y), std::fmaf(N.z, s2, d.z) };
    }
    const float a = eta * ci - std::sqrt(k);
    V3f r{ std::fmaf(N.x, a, d.x * eta), std::fmaf(N.y, a, d.y * eta), std::fmaf(N.z, a, d.z * eta) };
    const float len = std::sqrt(dot3(r, r));
    return V3f{ r.x / len, r.y / len, r.z / len };
}

V3f hemisphere32(V3f U, V3f V, V3f W, float x, float y)
{
    float sp, cp;
    sincos_turn(x, sp, cp);
    float ct = std::sqrt(1.0f - y);
    float st = std::sqrt(1.0f - ct * ct);
    float u = st * cp;
    float v = st * sp;
    return { std::fmaf(W.x, ct, std::fmaf(V.x, v, U.x * u)), std::fmaf(W.y, ct, std::fmaf(V.y, v, U.y * u)),
             std::fmaf(W.z, ct, std::fmaf(V.z, v, U.z * u)) };
}

uint64_t cmj_permute32(uint64_t i, uint64_t l, uint64_t p)
{
    uint64_t w = l - 1;
    w |= w >> 1;
    w |= w >> 2;
    w |= w >> 4;
    w |= w >> 8;
    w |= w >> 16;
    uint64_t i0 = i;
    int rounds = 0;
    do
    {
        i ^= p;
        i *= 0xe170893dull;
        i ^= p >> 16;
        i ^= (i & w) >> 4;
        i ^= p >> 8;
        i *= 0x0929eb3full;
        i ^= p >> 23;
        i ^= (i & w) >> 1;
        i *= 1 | p >> 27;
        i *= 0x6935fa69ull;
        i ^= (i & w) >> 11;
        i *= 0x74dcb303ull;
        i ^= (i & w) >> 2;
        i *= 0x9e501cc3ull;
        i ^= (i & w) >> 2;
        i *= 0xc860a3dfull;
        i &= w;
        i ^= i >> 5;
        if (++rounds >= 64 && i >= l)
        {
            i = i0 % l;
            break;
        }
    } while (i >= l);
    return (i + p) % l;
}

// ---------------------------------------------------------------------------
// Frame-level twins.

void raycast32(const Scene32& s, const Camera32& cam, uint64_t width, uint64_t pixelStart, uint64_t count,
               const float* L, float rayStartOffset, int order, int32_t* out4, uint64_t* counters, int threads)
{
    if (threads > 0)
        omp_set_num_threads(threads);
    uint64_t totalNodes = 0, totalTris = 0, totalRays = 0;
    #pragma omp parallel for schedule(dynamic, 256) reduction(+ : totalNodes, totalTris, totalRays)
    for (int64_t i = 0; i < int64_t(count); ++i)
    {
        uint64_t px = pixelStart + uint64_t(i);
        V3f d = camera_dir32(cam, float(px % width), float(px / width));
        V3f o{ cam.pos[0], cam.pos[1], cam.pos[2] };
        Ray32 r = make_ray32(o, d, 0.0f, FLT_MAX);
        Hit32 h;
        uint64_t nn = 0, nt = 0;
        bool found = traverse32(s, r, false, order, h, &nn, &nt, -1);
        totalRays++;
        int32_t* w = out4 + i * 4;
        w[0] = found ? s.caller[size_t(h.slot)] : -1;
        float tt = found ? h.t : -1.0f;
        std::memcpy(&w[1], &tt, 4);
        w[2] = -1;
        w[3] = found ? 1 : 0;
        if (found && L)
        {
            V3f ip{ std::fmaf(d.x, h.t, o.x), std::fmaf(d.y, h.t, o.y), std::fmaf(d.z, h.t, o.z) };
            V3f dl{ L[0], L[1], L[2] };
            V3f so{ std::fmaf(dl.x, rayStartOffset, ip.x), std::fmaf(dl.y, rayStartOffset, ip.y),
                    std::fmaf(dl.z, rayStartOffset, ip.z) };
            Ray32 sr = make_ray32(so, dl, 0.0f, FLT_MAX);
            Hit32 sh;
            // the shadow ray skips the triangle it leaves from (exact-arithmetic
            // semantics of the offset origin; same as the device)
            bool occ = traverse32(s, sr, true, 0, sh, &nn, &nt, h.slot);
            totalRays++;
            w[2] = occ ? s.caller[size_t(sh.slot)] : -1;
            w[3] = 1 | 2 | (occ ? 4 : 0);
        }
        totalNodes += nn;
        totalTris += nt;
    }
    if (counters)
    {
        counters[0] = totalRays;
        counters[1] = totalNodes;
        counters[2] = totalTris;
    }
}

void cast32(const Scene32& s, int64_t n, const float* rays8, int anyHit, int order, int32_t* prim, float* t, float* u,
            float* v, uint64_t* counters, int threads)
{
    if (threads > 0)
        omp_set_num_threads(threads);
    uint64_t totalNodes = 0, totalTris = 0;
    #pragma omp parallel for schedule(dynamic, 256) reduction(+ : totalNodes, totalTris)
    for (int64_t i = 0; i < n; ++i)
    {
        const float* q = rays8 + i * 8;
        Ray32 r = make_ray32(V3f{ q[0], q[1], q[2] }, V3f{ q[4], q[5], q[6] }, q[3], q[7]);
        Hit32 h;
        uint64_t nn = 0, nt = 0;
        bool found = traverse32(s, r, anyHit != 0, order, h, &nn, &nt, -1);
        prim[i] = found ? s.caller[size_t(h.slot)] : -1;
        t[i] = found ? h.t : -1.0f;
        u[i] = found ? h.u : 0.0f;
        v[i] = found ? h.v : 0.0f;
        totalNodes += nn;
        totalTris += nt;
    }
    if (counters)
    {
        counters[0] = uint64_t(n);
        counters[1] = totalNodes;
        counters[2] = totalTris;
    }
}

// Film filters (the device's filters.cuh restated: same constants, same
// operation order, std::fma where the device fuses).
Filter32 filter32(int type, float boxRx, float boxRy)
{
    Filter32 f{};
    f.type = type;
    switch (type)
    {
    case 0:
        f.rx = boxRx;
        f.ry = boxRy;
        f.ax = 1.0f / (2.0f * f.rx);
        f.ay = 1.0f / (2.0f * f.ry);
        break;
    case 1:
        f.rx = f.ry = 1.0f;
        f.ax = f.ay = 1.0f;
        break;
    case 2:
        f.rx = f.ry = 1.5f;
        break;
    case 3:
        f.ax = f.ay = float(1.0 / std::sqrt(2.0 * 3.14159265358979323846));
        f.bx = f.by = -0.5f;
        f.rx = f.ry = float(7.43384 / 2.0);
        break;
    case 4:
    {
        const double B = 1.0 / 3.0, C = 1.0 / 3.0;
        const double k[8] = { (12.0 - 9.0 * B - 6.0 * C) / 6.0, (-18.0 + 12.0 * B + 6.0 * C) / 6.0, 0.0,
                              (6.0 - 2.0 * B) / 6.0, (-B - 6.0 * C) / 6.0, (6.0 * B + 30.0 * C) / 6.0,
                              (-12.0 * B - 48.0 * C) / 6.0, (8.0 * B + 24.0 * C) / 6.0 };
        for (int i = 0; i < 8; ++i)
            f.cubic[i] = float(k[i]);
        f.rx = f.ry = 2.0f;
        break;
    }
    default:
        f.rx = f.ry = 2.0f;
        break;
    }
    return f;
}

float filter_exp32(float t)
{
    const float y = t * 1.44269504088896341f;
    const float n = std::floor(y + 0.5f);
    float f = std::fma(-n, 0.693145751953125f, t);
    f = std::fma(-n, 1.42860682030941723e-6f, f);
    float p = std::fma(f, 1.98412698412698413e-4f, 1.38888888888888889e-3f);
    p = std::fma(f, p, 8.33333333333333333e-3f);
    p = std::fma(f, p, 4.16666666666666667e-2f);
    p = std::fma(f, p, 1.66666666666666667e-1f);
    p = std::fma(f, p, 0.5f);
    p = std::fma(f, p, 1.0f);
    p = std::fma(f, p, 1.0f);
    const int e = int(n);
    if (e < -126)
        return 0.0f;
    uint32_t bits = uint32_t(e + 127) << 23;
    float scale;
    std::memcpy(&scale, &bits, 4);
    return p * scale;
}

static float filter_sinc32(float s)
{
    float sv, cv;
    sincos_turn(s * 0.5f, sv, cv);
    return sv / (3.14159265358979324f * s);
}

float filter_weight32(const Filter32& f, float x, float r, float a, float b)
{
    switch (f.type)
    {
    case 0:
        return (x >= -r && x < r) ? a : 0.0f;
    case 1:
    {
        const float s = std::fabs(x * a);
        return s < 1.0f ? (1.0f - s) * a : 0.0f;
    }
    case 2:
    {
        const float s = std::fabs(x);
        if (s < 0.5f)
            return 0.75f - s * s;
        if (s <= 1.5f)
        {
            const float t = s - 1.5f;
            return 0.5f * (t * t);
        }
        return 0.0f;
    }
    case 3:
        return a * filter_exp32((x * x) * b);
    case 4:
    {
        const float s = std::fabs(x);
        const float* c = s <= 1.0f ? f.cubic : f.cubic + 4;
        if (s > 2.0f)
            return 0.0f;
        return std::fma(std::fma(std::fma(c[0], s, c[1]), s, c[2]), s, c[3]);
    }
    default:
    {
        const float s = std::fabs(x);
        if (s == 0.0f)
            return 1.0f;
        if (s > r)
            return 0.0f;
        return filter_sinc32(s) * filter_sinc32(s / r);
    }
    }
}

// The device's PATH render (pathtrace.cu) path by path: generate, then
// extend/shade per segment, then accumulate per pixel in sample order.
void render_path32(const Scene32& s, const Camera32& cam, const PathSettings32& ps, uint64_t width,
                   uint64_t pixelStart, uint64_t count, float* film, uint64_t* counters, int threads)
{
    if (threads > 0)
        omp_set_num_threads(threads);
    const int n = ps.n, P = ps.P;
    const int nn = n * n;
    const Filter32 flt = filter32(ps.filterType, ps.rx, ps.ry);
    uint64_t totalRays = 0;
    #pragma omp parallel for schedule(dynamic, 64) reduction(+ : totalRays)
    for (int64_t pl = 0; pl < int64_t(count); ++pl)
    {
        uint64_t pg = pixelStart + uint64_t(pl);
        float* f = film + pl * 4;
        for (int j = 0; j < nn; ++j)
        {
            // generate (camera sample j)
            float px = float(pg % width);
            float py = float(pg / width);
            float w = 1.0f;
            if (n > 1)
            {
                uint32_t gx = uint32_t(j) % uint32_t(n), gy = uint32_t(j) / uint32_t(n);
                uint32_t jkey = stream_key(ps.seed, ps.frame, pg, 0x80000000u | uint32_t(j));
                float jx = stream_float(jkey, 8192u + 0u);
                float jy = stream_float(jkey, 8192u + 1u);
                float sx, sy;
                if (ps.samplerType == 4)
                {
                    uint32_t pkey = stream_key(ps.seed, ps.frame, pg, 0xffffffffu);
                    uint64_t perm = (uint64_t(stream_u32(pkey, 1)) << 32) | stream_u32(pkey, 2);
                    uint64_t sxp = cmj_permute32(gx, uint64_t(n), perm * 0x68bc21ebull);
                    uint64_t syp = cmj_permute32(gy, uint64_t(n), perm * 0x02e5be93ull);
                    float fn = float(n);
                    sx = (float(gx) + (float(syp) + jx) / fn) / fn;
                    sy = (float(gy) + (float(sxp) + jy) / fn) / fn;
                }
                else if (ps.samplerType == 1)
                {
                    sx = jx;
                    sy = jy;
                }
                else
                {
                    sx = 0.5f;
                    sy = 0.5f;
                }
                float ox = ((sx - 0.5f) * 2.0f) * flt.rx;
                float oy = ((sy - 0.5f) * 2.0f) * flt.ry;
                w = filter_weight32(flt, ox, flt.rx, flt.ax, flt.bx) * filter_weight32(flt, oy, flt.ry, flt.ay, flt.by);
                px = px + ox;
                py = py + oy;
            }
            V3f d0 = camera_dir32(cam, px, py);
            float sr = 0.0f, sg = 0.0f, sb = 0.0f;
            for (int k = 0; k < P; ++k)
            {
                uint32_t sample = uint32_t(j) * uint32_t(P) + uint32_t(k);
                uint32_t key = stream_key(ps.seed, ps.frame, pg, sample);
                V3f o{ cam.pos[0], cam.pos[1], cam.pos[2] };
                V3f d = d0;
                int64_t from = -1;
                float thr[3] = { 1.0f, 1.0f, 1.0f };
                float res[3] = { 0.0f, 0.0f, 0.0f };
                for (int seg = 0; seg < ps.maxPathLength; ++seg)
                {
                    Ray32 r = make_ray32(o, d, 0.0f, FLT_MAX);
                    Hit32 h;
                    totalRays++;
                    if (!traverse32(s, r, false, ps.order, h, nullptr, nullptr, from))
                        break;
                    const Material& m = s.src->mats[s.meta[size_t(h.slot)] & 0x00ffffffu];
                    if (m.flags & 1)
                    {
                        res[0] = thr[0] * m.emittance[0];
                        res[1] = thr[1] * m.emittance[1];
                        res[2] = thr[2] * m.emittance[2];
                        break;
                    }
                    if (seg + 1 >= ps.maxPathLength)
                        break;
                    if (ps.rrDepth > 0 && seg + 1 >= ps.rrDepth)
                    {
                        float mx = std::fmax(thr[0], std::fmax(thr[1], thr[2]));
                        float qs = std::fmin(mx, 1.0f);
                        float xi = stream_float(key, 4096u + uint32_t(seg));
                        if (!(xi < qs))
                            break;
                        thr[0] = thr[0] / qs;
                        thr[1] = thr[1] / qs;
                        thr[2] = thr[2] / qs;
                    }
                    const float* sh = &s.shade[size_t(h.slot) * 9];
                    V3f nrm{ sh[0], sh[1], sh[2] };
                    if (m.flags & 4)
                        nrm = V3f{ -nrm.x, -nrm.y, -nrm.z };
                    float xr = stream_float(key, 2u * uint32_t(seg));
                    float yr = stream_float(key, 2u * uint32_t(seg) + 1u);
                    const bool dielectric = (m.flags & 8) != 0;
                    V3f dir = dielectric ? dielectric32(d, nrm, m.ior, xr)
                                         : hemisphere32(V3f{ sh[3], sh[4], sh[5] }, V3f{ sh[6], sh[7], sh[8] }, nrm, xr, yr);
                    V3f ip{ std::fmaf(d.x, h.t, o.x), std::fmaf(d.y, h.t, o.y), std::fmaf(d.z, h.t, o.z) };
                    o = V3f{ std::fmaf(dir.x, ps.rayStartOffset, ip.x), std::fmaf(dir.y, ps.rayStartOffset, ip.y),
                             std::fmaf(dir.z, ps.rayStartOffset, ip.z) };
                    d = dir;
                    from = h.slot;
                    if (dielectric)
                        continue;
                    float alpha = std::fabs(dot3(dir, nrm));
                    thr[0] = thr[0] * ((2.0f * m.diffuse[0]) * alpha);
                    thr[1] = thr[1] * ((2.0f * m.diffuse[1]) * alpha);
                    thr[2] = thr[2] * ((2.0f * m.diffuse[2]) * alpha);
                }
                sr = sr + res[0];
                sg = sg + res[1];
                sb = sb + res[2];
            }
            float fP = float(P);
            f[0] = f[0] + (sr / fP) * w;
            f[1] = f[1] + (sg / fP) * w;
            f[2] = f[2] + (sb / fP) * w;
            f[3] = f[3] + w;
        }
    }
    if (counters)
        counters[0] = totalRays;
}

}  // namespace oracle
