// Test infrastructure only: NOT part of the product (see oracle.h).
//
// float64 restatement of the reference's CPU hot path. Each function cites
// the reference code it follows; arithmetic is in the same order as there.

#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <random>

#include "oracle.h"
#include "oracle64.h"

namespace oracle
{

// ---------------------------------------------------------------------------
// BVH build: FlatBVH::build (FlatBVH.cpp:89-204), calculateSAHSplit (:241),
// calculateSAHScore (:288), calculateMedianPoint (:323), BVHBuildInfo
// defaults (useSAH, regularSAHSplits = 0).

namespace
{

struct Box64
{
    double mn[3] = { std::numeric_limits<double>::max(), std::numeric_limits<double>::max(),
                     std::numeric_limits<double>::max() };
    double mx[3] = { std::numeric_limits<double>::lowest(), std::numeric_limits<double>::lowest(),
                     std::numeric_limits<double>::lowest() };
    void expand(const Box64& o)
    {
        for (int k = 0; k < 3; ++k)
        {
            mn[k] = std::min(mn[k], o.mn[k]);
            mx[k] = std::max(mx[k], o.mx[k]);
        }
    }
    double centre(int a) const { return (mn[a] + mx[a]) * 0.5; }
    double area() const
    {
        double ex = mx[0] - mn[0], ey = mx[1] - mn[1], ez = mx[2] - mn[2];
        return 2.0 * (ex * ey + ez * ey + ex * ez);
    }
};

struct Builder
{
    const Scene64& s;
    std::vector<Box64> box;  // per caller triangle
    std::vector<uint64_t> prims;

    explicit Builder(const Scene64& sc) : s(sc)
    {
        size_t n = sc.mat.size();
        box.resize(n);
        prims.resize(n);
        for (size_t i = 0; i < n; ++i)
        {
            const double* t = &sc.v[i * 9];
            for (int k = 0; k < 3; ++k)
            {
                box[i].mn[k] = std::min(t[k], std::min(t[3 + k], t[6 + k]));
                box[i].mx[k] = std::max(t[k], std::max(t[3 + k], t[6 + k]));
            }
            prims[i] = i;
        }
    }

    double score(int axis, double split, const Box64& nodeBox, uint64_t start, uint64_t end) const
    {
        Box64 lb, rb;
        uint64_t lc = 0, rc = 0;
        for (uint64_t i = start; i < end; ++i)
        {
            const Box64& b = box[prims[i]];
            if (b.centre(axis) <= split)
            {
                lb.expand(b);
                lc++;
            }
            else
            {
                rb.expand(b);
                rc++;
            }
        }
        double sc = 0.0;
        if (lc > 0)
            sc += (lb.area() / nodeBox.area()) * double(lc);
        if (rc > 0)
            sc += (rb.area() / nodeBox.area()) * double(rc);
        return sc;
    }

    double median(int axis, uint64_t start, uint64_t end) const
    {
        std::vector<double> c;
        c.reserve(end - start);
        for (uint64_t i = start; i < end; ++i)
            c.push_back(box[prims[i]].centre(axis));
        std::sort(c.begin(), c.end());
        size_t n = c.size();
        if (n % 2 == 0)
            return (c[n / 2 - 1] + c[n / 2]) / 2.0;
        return c[n / 2];
    }
};

}  // namespace

void build_bvh(Scene64& s)
{
    Builder b(s);
    struct Entry
    {
        uint64_t start, end;
        int64_t parent;
    };
    enum { ROOT = -4, UNVISITED = -3, VISITED_TWICE = -1 };
    std::vector<Entry> stack;
    stack.push_back({ 0, uint64_t(s.mat.size()), ROOT });
    s.nodes.clear();
    uint64_t nodeCount = 0;
    while (!stack.empty())
    {
        Entry e = stack.back();
        stack.pop_back();
        nodeCount++;
        Node64 node;
        Box64 nb;
        for (uint64_t i = e.start; i < e.end; ++i)
            nb.expand(b.box[b.prims[i]]);
        for (int k = 0; k < 3; ++k)
        {
            node.bmin[k] = nb.mn[k];
            node.bmax[k] = nb.mx[k];
        }
        node.rightOffset = UNVISITED;
        node.start = e.start;
        node.count = e.end - e.start;
        if (node.count <= s.maxLeafSize)
            node.rightOffset = 0;
        s.nodes.push_back(node);
        if (e.parent != ROOT)
        {
            s.nodes[uint64_t(e.parent)].rightOffset++;
            if (s.nodes[uint64_t(e.parent)].rightOffset == VISITED_TWICE)
                s.nodes[uint64_t(e.parent)].rightOffset = int64_t(nodeCount) - 1 - e.parent;
        }
        if (node.rightOffset == 0)
            continue;

        int axis = 0;
        double split = nb.centre(0);
        double lowest = std::numeric_limits<double>::max();
        for (int a = 0; a <= 2; ++a)
        {
            double sp = nb.centre(a);
            double sc = b.score(a, sp, nb, e.start, e.end);
            if (sc < lowest)
            {
                axis = a;
                split = sp;
                lowest = sc;
            }
            sp = b.median(a, e.start, e.end);
            sc = b.score(a, sp, nb, e.start, e.end);
            if (sc < lowest)
            {
                axis = a;
                split = sp;
                lowest = sc;
            }
        }
        uint64_t middle = e.start;
        for (uint64_t i = e.start; i < e.end; ++i)
        {
            if (b.box[b.prims[i]].centre(axis) <= split)
            {
                std::swap(b.prims[i], b.prims[middle]);
                middle++;
            }
        }
        if (middle == e.start || middle == e.end)
            middle = e.start + (e.end - e.start) / 2;
        stack.push_back({ middle, e.end, int64_t(nodeCount) - 1 });
        stack.push_back({ e.start, middle, int64_t(nodeCount) - 1 });
    }
    s.order = b.prims;
}

// Triangle::initialize (Triangle.cpp:18-47), zero texcoords.
void compute_frames(Scene64& s)
{
    size_t n = s.mat.size();
    s.frame.resize(n * 9);
    for (size_t i = 0; i < n; ++i)
    {
        const double* t = &s.v[i * 9];
        V3d a{ t[0], t[1], t[2] }, b{ t[3], t[4], t[5] }, c{ t[6], t[7], t[8] };
        V3d nrm = normalized(cross(sub(b, a), sub(c, a)));
        V3d tan = normalized(cross(nrm, V3d{ 0.0001, 1.0, 0.0001 }));
        V3d bit = normalized(cross(tan, nrm));
        double* f = &s.frame[i * 9];
        f[0] = nrm.x; f[1] = nrm.y; f[2] = nrm.z;
        f[3] = tan.x; f[4] = tan.y; f[5] = tan.z;
        f[6] = bit.x; f[7] = bit.y; f[8] = bit.z;
    }
}

// ---------------------------------------------------------------------------
// Queries: FlatBVH::intersect (FlatBVH.cpp:22-75), AABB::intersects
// (AABB.cpp:56-80), Triangle::intersect (Triangle.cpp:51-121).

namespace
{

bool aabb_hit(const Node64& nd, const Ray64& r)
{
    double tx0 = (nd.bmin[0] - r.o.x) * r.inv.x;
    double tx1 = (nd.bmax[0] - r.o.x) * r.inv.x;
    double tmin = std::min(tx0, tx1);
    double tmax = std::max(tx0, tx1);
    double ty0 = (nd.bmin[1] - r.o.y) * r.inv.y;
    double ty1 = (nd.bmax[1] - r.o.y) * r.inv.y;
    tmin = std::max(tmin, std::min(ty0, ty1));
    tmax = std::min(tmax, std::max(ty0, ty1));
    double tz0 = (nd.bmin[2] - r.o.z) * r.inv.z;
    double tz1 = (nd.bmax[2] - r.o.z) * r.inv.z;
    tmin = std::max(tmin, std::min(tz0, tz1));
    tmax = std::min(tmax, std::max(tz0, tz1));
    if (tmax < std::max(tmin, 0.0))
        return false;
    return true;
}

}  // namespace

bool tri_intersect64(const Scene64& s, uint64_t caller, const Ray64& r, Isect64& is)
{
    const Material& m = s.mats[s.mat[caller]];
    if (r.shadow && (m.flags & 2))
        return false;
    if (r.fastOcclusion && is.found)
        return true;
    const double* t = &s.v[caller * 9];
    V3d v0{ t[0], t[1], t[2] };
    V3d v0v1 = sub(V3d{ t[3], t[4], t[5] }, v0);
    V3d v0v2 = sub(V3d{ t[6], t[7], t[8] }, v0);
    V3d pvec = cross(r.d, v0v2);
    double det = dot(v0v1, pvec);
    if (std::abs(det) < std::numeric_limits<double>::epsilon())
        return false;
    double invDet = 1.0 / det;
    V3d tvec = sub(r.o, v0);
    double u = dot(tvec, pvec) * invDet;
    if (u < 0.0 || u > 1.0)
        return false;
    V3d qvec = cross(tvec, v0v1);
    double v = dot(r.d, qvec) * invDet;
    if (v < 0.0 || (u + v) > 1.0)
        return false;
    double d = dot(v0v2, qvec) * invDet;
    if (d < 0.0)
        return false;
    if (d < r.tmin || d > r.tmax)
        return false;
    if (d > is.t)
        return false;
    is.found = true;
    is.t = d;
    is.caller = int64_t(caller);
    is.u = u;
    is.v = v;
    return true;
}

bool intersect64(const Scene64& s, const Ray64& r, Isect64& is)
{
    if (r.fastOcclusion && is.found)
        return true;
    uint64_t stack[128];
    uint64_t sp = 0;
    bool found = false;
    stack[sp++] = 0;
    while (sp > 0)
    {
        uint64_t idx = stack[--sp];
        const Node64& nd = s.nodes[idx];
        if (nd.rightOffset == 0)
        {
            for (uint64_t i = 0; i < nd.count; ++i)
            {
                if (tri_intersect64(s, s.order[nd.start + i], r, is))
                {
                    if (r.fastOcclusion)
                        return true;
                    found = true;
                }
            }
        }
        else
        {
            if (aabb_hit(s.nodes[idx + uint64_t(nd.rightOffset)], r))
                stack[sp++] = idx + uint64_t(nd.rightOffset);
            if (aabb_hit(s.nodes[idx + 1], r))
                stack[sp++] = idx + 1;
            if (sp > 126)
                return found;  // the reference's stack holds 128 entries
        }
    }
    return found;
}

Ray64 make_ray64(V3d o, V3d d)
{
    Ray64 r;
    r.o = o;
    r.d = d;
    r.inv = V3d{ 1.0 / d.x, 1.0 / d.y, 1.0 / d.z };  // Ray::precalculate
    return r;
}

// Camera::getRay, perspective (Camera.cpp:321-331), from the camera state.
Ray64 camera_ray64(const Camera64& c, double px, double py)
{
    double dx = (px / c.ipw) - 0.5;
    double dy = (py / c.iph) - 0.5;
    V3d p = add(add(c.center, scale(c.right, dx)), scale(c.up, dy * c.aspect));
    return make_ray64(c.pos, normalized(sub(p, c.pos)));
}

// ---------------------------------------------------------------------------
// Samplers: mapToHemisphere (Sampler.cpp:50-64), CMJSampler (CMJSampler.cpp:
// 13-76), RandomSampler (RandomSampler.cpp:23-36).

namespace
{

uint64_t permute(uint64_t i, uint64_t l, uint64_t p)
{
    uint64_t w = l - 1;
    w |= w >> 1;
    w |= w >> 2;
    w |= w >> 4;
    w |= w >> 8;
    w |= w >> 16;
    do
    {
        i ^= p;
        i *= 0xe170893d;
        i ^= p >> 16;
        i ^= (i & w) >> 4;
        i ^= p >> 8;
        i *= 0x0929eb3f;
        i ^= p >> 23;
        i ^= (i & w) >> 1;
        i *= 1 | p >> 27;
        i *= 0x6935fa69;
        i ^= (i & w) >> 11;
        i *= 0x74dcb303;
        i ^= (i & w) >> 2;
        i *= 0x9e501cc3;
        i ^= (i & w) >> 2;
        i *= 0xc860a3df;
        i &= w;
        i ^= i >> 5;
    } while (i >= l);
    return (i + p) % l;
}

V3d hemisphere64(const V3d& u_, const V3d& v_, const V3d& w_, double x, double y)
{
    double phi = 2.0 * M_PI * x;
    double cos_phi = std::cos(phi);
    double sin_phi = std::sin(phi);
    double cos_theta = std::pow(1.0 - y, 1.0 / (1.0 + 1.0));
    double sin_theta = std::sqrt(1.0 - cos_theta * cos_theta);
    double u = sin_theta * cos_phi;
    double v = sin_theta * sin_phi;
    double w = cos_theta;
    return add(add(scale(u_, u), scale(v_, v)), scale(w_, w));
}

struct RGB
{
    double r = 0.0, g = 0.0, b = 0.0;
};

RGB trace_recursive(const Scene64& s, const PathSettings64& ps, const Ray64& ray, uint64_t iteration,
                    std::mt19937& gen, uint64_t& rays)
{
    if (iteration >= ps.maxPathLength)
        return RGB{};
    Isect64 is;
    rays++;
    intersect64(s, ray, is);
    if (!is.found)
        return RGB{};
    const Material& m = s.mats[s.mat[uint64_t(is.caller)]];
    if (m.flags & 1)
        return RGB{ m.emittance[0], m.emittance[1], m.emittance[2] };
    const double* f = &s.frame[uint64_t(is.caller) * 9];
    V3d n{ f[0], f[1], f[2] };
    if (m.flags & 4)
        n = V3d{ -n.x, -n.y, -n.z };
    std::uniform_real_distribution<double> uni(0.0, 1.0);
    double sx = uni(gen);
    double sy = uni(gen);
    V3d dir = hemisphere64(V3d{ f[3], f[4], f[5] }, V3d{ f[6], f[7], f[8] }, n, sx, sy);
    V3d pos = add(ray.o, scale(ray.d, is.t));
    Ray64 nr = make_ray64(add(pos, scale(dir, ps.rayStartOffset)), dir);
    double alpha = std::abs(dot(dir, n));
    RGB brdf{ 2.0 * double(m.diffuse[0]) * alpha, 2.0 * double(m.diffuse[1]) * alpha,
              2.0 * double(m.diffuse[2]) * alpha };
    RGB refl = trace_recursive(s, ps, nr, iteration + 1, gen, rays);
    return RGB{ brdf.r * refl.r, brdf.g * refl.g, brdf.b * refl.b };
}

}  // namespace

double cmj_component(uint64_t x, uint64_t y, uint64_t n, uint64_t permutation, double jx, double jy, int which)
{
    uint64_t sx = permute(x, n, permutation * 0x68bc21eb);
    uint64_t sy = permute(y, n, permutation * 0x02e5be93);
    if (which == 0)
        return (double(x) + (double(sy) + jx) / double(n)) / double(n);
    return (double(y) + (double(sx) + jy) / double(n)) / double(n);
}

// Tracer::run (Tracer.cpp:58-113) + generateMultiSamples (:115-144) +
// PathTracer::trace / traceRecursive (PathTracer.cpp:13-75) + Film::addSample.
void filter_radius64(int type, const double* boxRadius, double* radius)
{
    switch (type)
    {
    case 0: radius[0] = boxRadius[0]; radius[1] = boxRadius[1]; break;   // BoxFilter(0.5, 0.5) or as set
    case 1: radius[0] = radius[1] = 1.0; break;                          // TentFilter(1, 1)
    case 2: radius[0] = radius[1] = 1.5; break;                          // BellFilter
    case 3: radius[0] = radius[1] = (7.43384 * 1.0) / 2.0; break;        // GaussianFilter(1, 1)
    default: radius[0] = radius[1] = 2.0; break;                         // Mitchell, LanczosSinc(2, 2)
    }
}

// One axis of the filter at offset x; boxRadius points at that axis's BOX radius.
double filter_weight64(int type, const double* boxRadius, double x)
{
    const double pi = 3.14159265358979323846;
    switch (type)
    {
    case 0:
    {
        const double r = boxRadius[0];
        return (x >= -r && x < r) ? 1.0 / (2.0 * r) : 0.0;
    }
    case 1:
    {
        const double inv = 1.0 / 1.0;
        const double s = std::abs(x * inv);
        return (s < 1.0 ? 1.0 - s : 0.0) * inv;
    }
    case 2:
    {
        const double s = std::abs(x);
        if (s < 0.5)
            return 0.75 - s * s;
        if (s <= 1.5)
            return 0.5 * std::pow(s - 1.5, 2.0);
        return 0.0;
    }
    case 3:
    {
        const double sd = 1.0;
        const double alpha = 1.0 / (std::sqrt(2.0 * pi) * sd);
        const double beta = -1.0 / (2.0 * sd * sd);
        return alpha * std::exp(x * x * beta);
    }
    case 4:
    {
        const double B = 1.0 / 3.0, C = 1.0 / 3.0;
        const double s = std::abs(x);
        if (s <= 1.0)
            return ((12.0 - 9.0 * B - 6.0 * C) * (s * s * s) + (-18.0 + 12.0 * B + 6.0 * C) * (s * s) +
                    (6.0 - 2.0 * B)) *
                   (1.0 / 6.0);
        if (s <= 2.0)
            return ((-B - 6.0 * C) * (s * s * s) + (6.0 * B + 30.0 * C) * (s * s) + (-12.0 * B - 48.0 * C) * s +
                    (8.0 * B + 24.0 * C)) *
                   (1.0 / 6.0);
        return 0.0;
    }
    default:
    {
        const double size = 2.0;
        const double s = std::abs(x);
        if (s == 0.0)
            return 1.0;
        if (s > size)
            return 0.0;
        auto sinc = [pi](double v) { return std::sin(pi * v) / (pi * v); };
        return sinc(s) * sinc(s / size);
    }
    }
}

void render_path64(const Scene64& s, const Camera64& cam, const PathSettings64& ps, uint64_t width, uint64_t pixelStart,
                   uint64_t pixelCount, double* film, int threads, uint32_t seed, uint64_t* raysOut)
{
    if (threads > 0)
        omp_set_num_threads(threads);
    int maxThreads = std::max(1, omp_get_max_threads());
    std::vector<std::mt19937> gens(static_cast<size_t>(maxThreads));
    for (int t = 0; t < maxThreads; ++t)
        gens[size_t(t)].seed(seed + uint32_t(t) * 7919u);
    std::vector<uint64_t> rayCount(size_t(maxThreads) * 8, 0);

    #pragma omp parallel for schedule(dynamic, 1000)
    for (int64_t pi = 0; pi < int64_t(pixelCount); ++pi)
    {
        int tid = omp_get_thread_num();
        std::mt19937& gen = gens[size_t(tid)];
        uint64_t& rays = rayCount[size_t(tid) * 8];
        uint64_t off = uint64_t(pi) + pixelStart;
        double x = double(off % width);
        double y = double(off / width);
        double* fp = film + size_t(pi) * 4;
        auto trace = [&](double px, double py) {
            Ray64 r = camera_ray64(cam, px, py);
            RGB sum;
            for (uint64_t i = 0; i < ps.pathSampleCount; ++i)
            {
                RGB c = trace_recursive(s, ps, r, 0, gen, rays);
                sum.r += c.r;
                sum.g += c.g;
                sum.b += c.b;
            }
            double P = double(ps.pathSampleCount);
            return RGB{ sum.r / P, sum.g / P, sum.b / P };
        };
        if (ps.multiSampleCountSqrt == 1)
        {
            RGB c = trace(x, y);
            fp[0] += c.r;
            fp[1] += c.g;
            fp[2] += c.b;
            fp[3] += 1.0;
            continue;
        }
        std::uniform_int_distribution<uint64_t> randomPermutation;
        uint64_t permutation = randomPermutation(gen);
        uint64_t n = ps.multiSampleCountSqrt;
        std::uniform_real_distribution<double> uni(0.0, 1.0);
        double rad[2];
        filter_radius64(ps.filterType, ps.filterRadius, rad);
        for (uint64_t sy = 0; sy < n; ++sy)
        {
            for (uint64_t sx = 0; sx < n; ++sx)
            {
                double smx, smy;
                if (ps.samplerType == 4)
                {
                    double jx = uni(gen);
                    double jy = uni(gen);
                    smx = cmj_component(sx, sy, n, permutation, jx, jy, 0);
                    smy = cmj_component(sx, sy, n, permutation, jx, jy, 1);
                }
                else if (ps.samplerType == 1)
                {
                    smx = uni(gen);
                    smy = uni(gen);
                }
                else
                {
                    smx = 0.5;
                    smy = 0.5;
                }
                double ox = (smx - 0.5) * 2.0 * rad[0];
                double oy = (smy - 0.5) * 2.0 * rad[1];
                RGB c = trace(x + ox, y + oy);
                double w = filter_weight64(ps.filterType, ps.filterRadius, ox) *
                           filter_weight64(ps.filterType, ps.filterRadius + 1, oy);
                fp[0] += c.r * w;
                fp[1] += c.g * w;
                fp[2] += c.b * w;
                fp[3] += w;
            }
        }
    }
    uint64_t total = 0;
    for (int t = 0; t < maxThreads; ++t)
        total += rayCount[size_t(t) * 8];
    if (raysOut)
        *raysOut = total;
}

// The RAY tracer's ray set (Raytracer::traceRecursive, Raytracer.cpp:27-97,
// with one directional light): a closest-hit primary ray per pixel and, for
// each hit, the shadow ray of calculateShadowAmount (Raytracer.cpp:497-522).
void raycast64(const Scene64& s, const Camera64& cam, uint64_t width, uint64_t pixelStart, uint64_t pixelCount,
               const double* dirToLight, double rayStartOffset, int64_t* prim, double* tOut, int64_t* occluder,
               int threads, uint64_t* raysOut)
{
    if (threads > 0)
        omp_set_num_threads(threads);
    int maxThreads = std::max(1, omp_get_max_threads());
    std::vector<uint64_t> rayCount(size_t(maxThreads) * 8, 0);
    V3d L{ dirToLight[0], dirToLight[1], dirToLight[2] };

    #pragma omp parallel for schedule(dynamic, 1000)
    for (int64_t pi = 0; pi < int64_t(pixelCount); ++pi)
    {
        uint64_t& rays = rayCount[size_t(omp_get_thread_num()) * 8];
        uint64_t off = uint64_t(pi) + pixelStart;
        Ray64 r = camera_ray64(cam, double(off % width), double(off / width));
        Isect64 is;
        rays++;
        intersect64(s, r, is);
        prim[pi] = is.found ? is.caller : -1;
        tOut[pi] = is.found ? is.t : -1.0;
        occluder[pi] = -1;
        if (!is.found || !dirToLight)
            continue;
        V3d pos = add(r.o, scale(r.d, is.t));
        Ray64 sr = make_ray64(add(pos, scale(L, rayStartOffset)), L);
        sr.shadow = true;
        sr.fastOcclusion = true;
        Isect64 si;
        rays++;
        if (intersect64(s, sr, si))
            occluder[pi] = si.caller;
    }
    uint64_t total = 0;
    for (int t = 0; t < maxThreads; ++t)
        total += rayCount[size_t(t) * 8];
    if (raysOut)
        *raysOut = total;
}

// ---------------------------------------------------------------------------
// ReinhardToneMapper::apply (ReinhardToneMapper.cpp:18-86) with
// MathUtils::fastPow (MathUtils.cpp:56-68).

double fast_pow64(double a, double b)
{
    uint64_t bits;
    std::memcpy(&bits, &a, 8);
    int32_t hi = int32_t(uint32_t(bits >> 32));
    int32_t nh = static_cast<int32_t>(b * double(hi - 1072632447) + 1072632447);
    uint64_t out = uint64_t(uint32_t(nh)) << 32;
    double r;
    std::memcpy(&r, &out, 8);
    return r;
}

void tonemap_reinhard64(int64_t pixels, const float* linear, double key, double gamma, int shouldClamp, int applyGamma,
                        float* out)
{
    const double epsilon = 0.01;
    double logSum = 0.0;
    double maxL = 1.0;
    for (int64_t i = 0; i < pixels; ++i)
    {
        double L = 0.2126 * double(linear[i * 4]) + 0.7152 * double(linear[i * 4 + 1]) +
                   0.0722 * double(linear[i * 4 + 2]);
        logSum += std::log(epsilon + L);
        if (L > maxL)
            maxL = L;
    }
    const double avg = std::exp(logSum / double(pixels));
    const double scaleL = key / avg;
    const double maxL2Inv = 1.0 / (maxL * maxL);
    const double invGamma = 1.0 / gamma;
    for (int64_t i = 0; i < pixels; ++i)
    {
        double c[3] = { double(linear[i * 4]), double(linear[i * 4 + 1]), double(linear[i * 4 + 2]) };
        double L = 0.2126 * c[0] + 0.7152 * c[1] + 0.0722 * c[2];
        double sL = scaleL * L;
        double mapped = (sL * (1.0 + (sL * maxL2Inv))) / (1.0 + sL);
        double cs = mapped / L;
        // A black pixel gives 0/0. The reference's build (x86-64) produces the
        // default NaN with the sign bit set, which MathUtils::fastPow maps to
        // a tiny value (0 in float) when clamping is off; other hosts' default
        // NaN is positive and would map to +inf. Use the reference's NaN.
        if (std::isnan(cs))
            cs = -std::numeric_limits<double>::quiet_NaN();
        for (int k = 0; k < 3; ++k)
        {
            double x = c[k] * cs;
            if (shouldClamp)
                x = std::max(0.0, std::min(x, 1.0));
            if (applyGamma)
                x = fast_pow64(x, invGamma);
            out[i * 4 + k] = float(x);
        }
        out[i * 4 + 3] = 1.0f;
    }
}

}  // namespace oracle
