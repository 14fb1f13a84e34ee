// Parameters of the wavefront path tracer (pathtrace.cu) and the
// tone-mapping launchers (tonemap.cu).
//
// A render is a list of passes. A pass holds up to `nslots` path slots, cut
// into chunks; a chunk is a run of whole pixels of one scene, and its pixels'
// paths occupy consecutive slots (spp slots per pixel: n*n camera samples x P
// paths). A single-scene render is a one-scene table with one chunk per pass;
// the batched renderer packs chunks of many scenes into the same passes. Both
// run the same kernels, so a scene renders identically either way.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.h"

namespace rcx
{

// Everything a slot of one scene needs (device memory, one per scene).
struct PathScene
{
    DevScene sc;
    DevCamera cam;
    float4* film;         // r, g, b, weight sum per film pixel
    uint64_t pixelStart;  // global pixel index of render-local pixel 0
    int64_t width;        // film width (pixel coordinates)
    int n;                // multiSampleCountSqrt
    int P;                // pathSampleCount
    int spp;              // n * n * P slots per pixel
    int samplerType;
    float rx, ry;         // box filter radius
    float wx, wy;         // box filter weight per axis: 1 / (2 r)
    float rayStartOffset;
    int maxPathLength;
    int rrDepth;          // 0 = no Russian roulette
    uint32_t frame;
    uint64_t seed;
};

struct PathChunk
{
    int scene;
    uint32_t slotBegin;         // first slot of the chunk in its pass
    uint32_t pixelPassBegin;    // index of the chunk's first pixel among the pass's pixels
    uint32_t pixels;            // whole pixels in the chunk
    uint64_t pixelLocalBegin;   // render-local index of the chunk's first pixel
};

struct PassParams
{
    const PathScene* scenes;
    const PathChunk* chunks;
    int numChunks;
    int nslots;      // slots used by this pass
    int npixels;     // pixels in this pass
    int segments;    // extend/shade rounds (max maxPathLength over the pass's scenes)
    float4* o;
    float4* d;
    float4* thr;
    float4* res;
    int4* hit;
    int* qa;
    int* qb;
    int* chunkOf;    // slot -> chunk (written by generate)
    unsigned* counts;  // per segment: [queue count, extend head, shade head, unused]
    DevControl* ctl;
};

// Bytes of path state per slot (o, d, thr, res, hit, two queue entries, chunk id).
constexpr size_t kPathBytesPerSlot = 5 * 16 + 3 * 4;

// Kernel shapes the autotuner chooses among (threads per block of the
// persistent extend / shade kernels).
constexpr int kNumBlockShapes = 3;
constexpr int kBlockShapes[kNumBlockShapes] = { 64, 128, 256 };

struct PassShape
{
    int extendBlock = 128;  // one of kBlockShapes
    int shadeBlock = 128;
};

// Launch the kernels of one pass (generate, segments x (extend, shade),
// accumulate) on `stream`. extendEvents: 2 * segments events recorded around
// each extend launch, or nullptr. Graph-capturable (no host reads).
cudaError_t launch_path_pass(const PassParams& p, int order, int counting, const PassShape& shape,
                             cudaStream_t stream, int numSMs, const cudaEvent_t* extendEvents);

// Reinhard / passthrough resolve of the film into out (float4 per pixel).
// partials needs tone_partials_bytes(pixels) bytes.
size_t tone_partials_bytes(uint64_t pixels);
cudaError_t launch_tonemap(const float4* film, uint64_t pixels, int type, int applyGamma, int shouldClamp,
                           double gamma, double key, void* partials, float4* out, cudaStream_t stream, int numSMs);
cudaError_t launch_linear(const float4* film, uint64_t pixels, float4* out, cudaStream_t stream);

}  // namespace rcx
