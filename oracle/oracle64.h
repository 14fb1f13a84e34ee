// Test infrastructure only: NOT part of the product (see oracle.h).
// float64 vector helpers and query types of the float64 restatement.
#pragma once

#include <cmath>
#include <cstdint>
#include <limits>

#include "oracle.h"

namespace oracle
{

struct V3d
{
    double x, y, z;
};

inline V3d add(V3d a, V3d b) { return { a.x + b.x, a.y + b.y, a.z + b.z }; }
inline V3d sub(V3d a, V3d b) { return { a.x - b.x, a.y - b.y, a.z - b.z }; }
inline V3d scale(V3d a, double s) { return { a.x * s, a.y * s, a.z * s }; }
// Vector3::dot / cross (Vector3.cpp:200-214)
inline double dot(V3d a, V3d b) { return (a.x * b.x) + (a.y * b.y) + (a.z * b.z); }
inline V3d cross(V3d a, V3d b) { return { a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x }; }
// Vector3::normalized = v / length, and operator/ multiplies by 1 / s (Vector3.cpp:57-61, 162-165)
inline V3d normalized(V3d v)
{
    double inv = 1.0 / std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
    return { v.x * inv, v.y * inv, v.z * inv };
}

struct Ray64
{
    V3d o{}, d{}, inv{};
    double tmin = std::numeric_limits<double>::lowest();
    double tmax = std::numeric_limits<double>::max();
    bool shadow = false;
    bool fastOcclusion = false;
};

struct Isect64
{
    bool found = false;
    double t = std::numeric_limits<double>::max();
    int64_t caller = -1;
    double u = 0.0, v = 0.0;
};

// Camera state of Camera::update (position, right, up, image-plane centre,
// aspect ratio, image-plane width/height).
struct Camera64
{
    V3d pos, right, up, center;
    double aspect, ipw, iph;
};

struct PathSettings64
{
    uint64_t maxPathLength = 4;
    uint64_t pathSampleCount = 1;
    uint64_t multiSampleCountSqrt = 1;
    int samplerType = 4;
    int filterType = 0;                     // FilterType (Filter.h:10)
    double filterRadius[2] = { 0.5, 0.5 };  // BOX only; the others use their defaults
    double rayStartOffset = 0.00001;
};

// The reference's film filters in float64 (Rendering/Filters/*.cpp, default
// constructors as Tracer.cpp:50-55 makes them): radius and per-axis weight.
void filter_radius64(int type, const double* boxRadius, double* radius);
double filter_weight64(int type, const double* boxRadius, double x);

Ray64 make_ray64(V3d o, V3d d);
Ray64 camera_ray64(const Camera64& c, double px, double py);
bool intersect64(const Scene64& s, const Ray64& r, Isect64& is);
bool tri_intersect64(const Scene64& s, uint64_t caller, const Ray64& r, Isect64& is);
double cmj_component(uint64_t x, uint64_t y, uint64_t n, uint64_t permutation, double jx, double jy, int which);
void render_path64(const Scene64& s, const Camera64& cam, const PathSettings64& ps, uint64_t width, uint64_t pixelStart,
                   uint64_t pixelCount, double* film, int threads, uint32_t seed, uint64_t* raysOut);
void raycast64(const Scene64& s, const Camera64& cam, uint64_t width, uint64_t pixelStart, uint64_t pixelCount,
               const double* dirToLight, double rayStartOffset, int64_t* prim, double* tOut, int64_t* occluder,
               int threads, uint64_t* raysOut);
double fast_pow64(double a, double b);
void tonemap_reinhard64(int64_t pixels, const float* linear, double key, double gamma, int shouldClamp, int applyGamma,
                        float* out);

}  // namespace oracle
