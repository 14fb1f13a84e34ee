// Float32 ray/box/triangle arithmetic of the hot path (device side).
//
// Every operation is written with an explicitly rounded intrinsic
// (__fadd_rn, __fmul_rn, __fmaf_rn, __fdiv_rn, __fsqrt_rn, __frcp_rn) so
// nvcc cannot contract or reorder it. The CPU float32 oracle performs the
// same operations in the same order, which makes hit ids, distances and
// barycentrics bit-identical between the two. The formulas are those of the
// reference's float32 kernels (data/opencl/intersections.cl:1-96,
// camera.cl:1-10, sampler.cl:1-14), with products-and-sums of dot and cross
// products fused (the reference builds them with -cl-mad-enable,
// misc/settings.ini).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "device_types.h"

namespace rcx
{

struct V3
{
    float x, y, z;
};

__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{ x, y, z }; }
__device__ __forceinline__ V3 vsub(V3 a, V3 b) { return v3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)); }
__device__ __forceinline__ V3 vscale(V3 a, float s) { return v3(__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s)); }
// a * s + b, per component, fused.
__device__ __forceinline__ V3 vfma(V3 a, float s, V3 b) { return v3(__fmaf_rn(a.x, s, b.x), __fmaf_rn(a.y, s, b.y), __fmaf_rn(a.z, s, b.z)); }
// dot(a, b) = fma(a.z, b.z, fma(a.y, b.y, a.x * b.x))
__device__ __forceinline__ float vdot(V3 a, V3 b) { return __fmaf_rn(a.z, b.z, __fmaf_rn(a.y, b.y, __fmul_rn(a.x, b.x))); }
// cross(a, b).x = fma(a.y, b.z, -(a.z * b.y)), cyclic.
__device__ __forceinline__ V3 vcross(V3 a, V3 b)
{
    return v3(__fmaf_rn(a.y, b.z, -__fmul_rn(a.z, b.y)),
              __fmaf_rn(a.z, b.x, -__fmul_rn(a.x, b.z)),
              __fmaf_rn(a.x, b.y, -__fmul_rn(a.y, b.x)));
}
// normalize(v) = v * (1 / sqrt(dot(v, v))) (Vector3::normalized, Vector3.cpp:162).
__device__ __forceinline__ V3 vnormalize(V3 v)
{
    float len = __fsqrt_rn(vdot(v, v));
    float inv = __frcp_rn(len);
    return vscale(v, inv);
}

// std::min / std::max semantics (the OpenCL min/max of intersectAABB):
// min(a, b) = (b < a) ? b : a ; max(a, b) = (a < b) ? b : a.
__device__ __forceinline__ float smin(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float smax(float a, float b) { return (a < b) ? b : a; }

struct RayF
{
    V3 o;
    V3 d;
    V3 inv;  // 1 / d per component (Ray::precalculate, Ray.cpp:10)
    float tmin;
    float tmax;
    bool finite;  // all of inv finite: no slab product can be NaN
};

__device__ __forceinline__ RayF make_ray(V3 o, V3 d, float tmin, float tmax)
{
    RayF r;
    r.o = o;
    r.d = d;
    r.inv = v3(__frcp_rn(d.x), __frcp_rn(d.y), __frcp_rn(d.z));
    r.tmin = tmin;
    r.tmax = tmax;
    r.finite = isfinite(r.inv.x) && isfinite(r.inv.y) && isfinite(r.inv.z);
    return r;
}

// Slab test of intersectAABB (intersections.cl:1-25): hit iff
// tmax >= max(tmin, 0). `entry` receives max(tmin, 0) for ordering/culling.
__device__ __forceinline__ bool slab(const RayF& r, float lox, float hix, float loy, float hiy, float loz, float hiz,
                                     float& entry)
{
    float tx0 = __fmul_rn(__fsub_rn(lox, r.o.x), r.inv.x);
    float tx1 = __fmul_rn(__fsub_rn(hix, r.o.x), r.inv.x);
    float tmin = smin(tx0, tx1);
    float tmax = smax(tx0, tx1);
    float ty0 = __fmul_rn(__fsub_rn(loy, r.o.y), r.inv.y);
    float ty1 = __fmul_rn(__fsub_rn(hiy, r.o.y), r.inv.y);
    tmin = smax(tmin, smin(ty0, ty1));
    tmax = smin(tmax, smax(ty0, ty1));
    float tz0 = __fmul_rn(__fsub_rn(loz, r.o.z), r.inv.z);
    float tz1 = __fmul_rn(__fsub_rn(hiz, r.o.z), r.inv.z);
    tmin = smax(tmin, smin(tz0, tz1));
    tmax = smin(tmax, smax(tz0, tz1));
    entry = smax(tmin, 0.0f);
    return !(tmax < entry);
}

// The same test for a ray whose inverse direction is finite. Then every
// product (lo - o) * inv is a number (finite or an overflowed infinity, never
// NaN), and for non-NaN operands fminf/fmaxf pick the same value as the
// compare-and-select of std::min/std::max up to the sign of a zero, which no
// comparison below can see. So the decision and the entry distance's order
// relations are identical, at one FMNMX instruction per min/max.
__device__ __forceinline__ bool slab_finite(const RayF& r, float lox, float hix, float loy, float hiy, float loz,
                                            float hiz, float& entry)
{
    float tx0 = __fmul_rn(__fsub_rn(lox, r.o.x), r.inv.x);
    float tx1 = __fmul_rn(__fsub_rn(hix, r.o.x), r.inv.x);
    float ty0 = __fmul_rn(__fsub_rn(loy, r.o.y), r.inv.y);
    float ty1 = __fmul_rn(__fsub_rn(hiy, r.o.y), r.inv.y);
    float tz0 = __fmul_rn(__fsub_rn(loz, r.o.z), r.inv.z);
    float tz1 = __fmul_rn(__fsub_rn(hiz, r.o.z), r.inv.z);
    float tmin = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fminf(tz0, tz1));
    float tmax = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1));
    entry = fmaxf(tmin, 0.0f);
    return !(tmax < entry);
}

// The same test for a ray whose inverse direction is finite with the signs
// of octant OCT (bit k set: component k negative). (lo - o) and (hi - o)
// are ordered like lo and hi (rounding is monotone), and multiplying by a
// positive inverse keeps that order and by a negative one reverses it, so
// the near and far plane distances of each axis are known without a
// min/max: the values slab_finite's min/max pick, up to the sign of a zero
// (which no comparison sees). Six FMNMX fewer per box.
template <int OCT>
__device__ __forceinline__ bool slab_oct(const RayF& r, float lox, float hix, float loy, float hiy, float loz,
                                         float hiz, float& entry)
{
    const float nx = __fmul_rn(__fsub_rn((OCT & 1) ? hix : lox, r.o.x), r.inv.x);
    const float fx = __fmul_rn(__fsub_rn((OCT & 1) ? lox : hix, r.o.x), r.inv.x);
    const float ny = __fmul_rn(__fsub_rn((OCT & 2) ? hiy : loy, r.o.y), r.inv.y);
    const float fy = __fmul_rn(__fsub_rn((OCT & 2) ? loy : hiy, r.o.y), r.inv.y);
    const float nz = __fmul_rn(__fsub_rn((OCT & 4) ? hiz : loz, r.o.z), r.inv.z);
    const float fz = __fmul_rn(__fsub_rn((OCT & 4) ? loz : hiz, r.o.z), r.inv.z);
    const float tmin = fmaxf(fmaxf(nx, ny), nz);
    const float tmax = fminf(fminf(fx, fy), fz);
    entry = fmaxf(tmin, 0.0f);
    return !(tmax < entry);
}

// Sign octant of a ray's inverse direction (slab_oct's OCT), or -1 when a
// component is not finite (slab_oct does not apply).
__device__ __forceinline__ int ray_octant(const RayF& r)
{
    if (!r.finite)
        return -1;
    return (r.inv.x < 0.0f ? 1 : 0) | (r.inv.y < 0.0f ? 2 : 0) | (r.inv.z < 0.0f ? 4 : 0);
}

// Möller–Trumbore of intersectTriangle (intersections.cl:27-69 /
// Triangle.cpp:51-93) up to the distance window; the caller applies the
// closest-hit comparison. Returns true with t, u, v on a hit.
__device__ __forceinline__ bool tri_hit(const RayF& r, V3 v0, V3 e1, V3 e2, float& t, float& u, float& v)
{
    V3 pvec = vcross(r.d, e2);
    float det = vdot(e1, pvec);
    if (fabsf(det) < 1.1920928955078125e-7f)  // FLT_EPSILON
        return false;
    float invDet = __frcp_rn(det);
    V3 tvec = vsub(r.o, v0);
    u = __fmul_rn(vdot(tvec, pvec), invDet);
    if (u < 0.0f || u > 1.0f)
        return false;
    V3 qvec = vcross(tvec, e1);
    v = __fmul_rn(vdot(r.d, qvec), invDet);
    if (v < 0.0f || __fadd_rn(u, v) > 1.0f)
        return false;
    t = __fmul_rn(vdot(e2, qvec), invDet);
    if (t < 0.0f)
        return false;
    if (t < r.tmin || t > r.tmax)
        return false;
    return true;
}

// Perspective camera ray for a (sub)pixel coordinate (camera.cl:1-10,
// Camera::getRay Camera.cpp:321-331):
//   dx = px / (W - 1) - 0.5, dy = py / (H - 1) - 0.5
//   p  = centre + dx * right + (dy * aspect) * up
//   d  = normalize(p - position)
__device__ __forceinline__ V3 camera_dir(const DevCamera& c, float px, float py)
{
    float dx = __fsub_rn(__fdiv_rn(px, c.ipw), 0.5f);
    float dy = __fsub_rn(__fdiv_rn(py, c.iph), 0.5f);
    float dya = __fmul_rn(dy, c.aspect);
    V3 p = vfma(v3(c.up[0], c.up[1], c.up[2]), dya,
                vfma(v3(c.right[0], c.right[1], c.right[2]), dx, v3(c.center[0], c.center[1], c.center[2])));
    return vnormalize(vsub(p, v3(c.pos[0], c.pos[1], c.pos[2])));
}

}  // namespace rcx
