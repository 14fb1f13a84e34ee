// Test infrastructure only: NOT part of the product (see oracle.h).
// Types of the float32 twin of the device kernels.
#pragma once

#include <cfloat>
#include <cstdint>

#include "oracle.h"

namespace oracle
{

struct V3f
{
    float x, y, z;
};

struct Ray32
{
    V3f o, d, inv;
    float tmin, tmax;
};

struct Hit32
{
    int64_t slot = -1;
    float t = FLT_MAX;
    float u = 0.0f, v = 0.0f;
};

// Same fields as rc_camera.
struct Camera32
{
    float pos[3], fwd[3], right[3], up[3], center[3];
    float aspect, ipw, iph;
};

struct PathSettings32
{
    int n = 1;          // multiSampleCountSqrt
    int P = 1;          // pathSampleCount
    int samplerType = 4;
    int filterType = 0;  // rc_filter_type; rx, ry = BOX radius
    float rx = 0.5f, ry = 0.5f;
    float rayStartOffset = 0.00001f;
    int maxPathLength = 4;
    int rrDepth = 0;
    int order = 1;
    uint64_t seed = 1;
    uint32_t frame = 0;
};

Ray32 make_ray32(V3f o, V3f d, float tmin, float tmax);
bool traverse32(const Scene32& s, const Ray32& r, bool anyHit, int order, Hit32& h, uint64_t* nodes, uint64_t* tris,
                int64_t skip);
V3f camera_dir32(const Camera32& c, float px, float py);
void raycast32(const Scene32& s, const Camera32& cam, uint64_t width, uint64_t pixelStart, uint64_t count,
               const float* L, float rayStartOffset, int order, int32_t* out4, uint64_t* counters, int threads);
void cast32(const Scene32& s, int64_t n, const float* rays8, int anyHit, int order, int32_t* prim, float* t, float* u,
            float* v, uint64_t* counters, int threads);
void render_path32(const Scene32& s, const Camera32& cam, const PathSettings32& ps, uint64_t width,
                   uint64_t pixelStart, uint64_t count, float* film, uint64_t* counters, int threads);
void sincos_turn(float x, float& s, float& c);
// Film filter of the device (filters.cuh): radius and per-axis weight.
struct Filter32
{
    int type;
    float rx, ry, ax, ay, bx, by;
    float cubic[8];
};
Filter32 filter32(int type, float boxRx, float boxRy);
float filter_weight32(const Filter32& f, float x, float r, float a, float b);
float filter_exp32(float t);
uint32_t stream_key(uint64_t seed, uint32_t frame, uint64_t pixel, uint32_t sample);
float stream_float(uint32_t key, uint32_t counter);
uint64_t cmj_permute32(uint64_t i, uint64_t l, uint64_t p);

}  // namespace oracle
