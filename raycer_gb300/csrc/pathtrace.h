// Parameters of one wavefront path-tracing pass (see pathtrace.cu) and the
// tone-mapping launchers (tonemap.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.h"


namespace rcx
{

struct PathParams
{
    DevScene sc;
    DevCamera cam;
    float4* o;
    float4* d;
    float4* thr;
    float4* res;
    int4* hit;
    int* qa;
    int* qb;
    unsigned* counts;   // per segment: [queue count, extend head, shade head, unused]
    float4* film;       // r, g, b, weight sum per film pixel
    DevControl* ctl;
    uint64_t pixelStart;  // global pixel index of render-local pixel 0
    uint64_t passPixel;   // render-local index of the pass's first pixel
    int64_t width;        // film width (pixel coordinates)
    int n;                // multiSampleCountSqrt
    int P;                // pathSampleCount
    int spp;              // n * n * P slots per pixel
    int nslots;           // slots in this pass
    int samplerType;
    float rx, ry;         // box filter radius
    float wx, wy;         // box filter weight per axis: 1 / (2 r)
    float rayStartOffset;
    int maxPathLength;
    int rrDepth;          // 0 = no Russian roulette
    uint64_t seed;
    uint32_t frame;
};

// Bytes of path state per slot (o, d, thr, res, hit, two queue entries).
constexpr size_t kPathBytesPerSlot = 5 * 16 + 2 * 4;

// extendEvents: 2 * maxPathLength events recorded around each extend launch
// (or nullptr).
cudaError_t launch_path_pass(const PathParams& p, int pixelsInPass, int order, int counting, cudaStream_t stream,
                             int numSMs, const cudaEvent_t* extendEvents);

// Reinhard / passthrough resolve of the film into out (float4 per pixel).
// partials needs tone_partials_bytes(pixels) bytes.
size_t tone_partials_bytes(uint64_t pixels);
cudaError_t launch_tonemap(const float4* film, uint64_t pixels, int type, int applyGamma, int shouldClamp,
                           double gamma, double key, void* partials, float4* out, cudaStream_t stream, int numSMs);
cudaError_t launch_linear(const float4* film, uint64_t pixels, float4* out, cudaStream_t stream);

}  // namespace rcx
