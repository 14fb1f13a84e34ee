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
#include "nrc_kernels.h"

namespace rcx
{

// Film reconstruction filter (filters.cuh) with its per-axis constants.
struct FilterSpec
{
    int type;        // rc_filter_type
    float rx, ry;    // radius: camera samples are offset within [-r, r)
    float ax, ay;    // BOX 1/(2r), TENT 1/r, GAUSSIAN alpha
    float bx, by;    // GAUSSIAN beta
    float cubic[8];  // MITCHELL: |x| <= 1 and 1 < |x| <= 2 cubics, highest power first
};

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
    FilterSpec filter;
    float rayStartOffset;
    int maxPathLength;
    int rrDepth;          // 0 = no Russian roulette
    uint32_t frame;
    int skyOn;            // misses return `sky` (GPU extension; the reference returns black)
    float sky[3];
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

// Neural-radiance-cache state of one pass (all pointers null: plain paths).
// Slot s is a training path when s % trainStride == pick(s / trainStride)
// (one random slot per run of trainStride slots); every other path ends at
// the hit of segment termSegment with a cache lookup.
struct NrcPass
{
    NrcRecord* query;     // cache lookups, [nslots]; tag = slot
    NrcRecord* vtx;       // training vertices [segments][groups]; radiance = bounce factor
    float4* term;         // per training path: terminal radiance; w = flags (below)
    int* index;           // training samples (vertex record indices), [segments * groups]
    unsigned* counters;   // [0] lookups, [1] training samples
    int termSegment;
    int trainStride;      // 0: no training paths
    int groups;           // ceil(nslots / trainStride)
    int minSuffix;        // vertices a suffix cut by the depth limit needs to be a sample
    uint32_t trainKey;    // per-pass key of the training-slot choice
    int lookupVertexOnly; // 1: the vertex at termSegment is a path's only sample
};
// NrcPass::term flags: vertex count | truncated << 8 | active << 9.
constexpr uint32_t kNrcTermTruncated = 1u << 8;
constexpr uint32_t kNrcTermActive = 1u << 9;

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
    NrcPass nrc;
    int instanced;   // 1: the pass has two-level scenes (k_extend_instanced)
    int wide;        // 1: every scene of the pass has its 4-wide BVH (uncounted nearest-first extend uses it)
    int singleScene = 0;  // 1: every slot of the pass is scene0's (a one-scene render), so the
                          // extend kernels read the scene record from the parameters, not the table
    DevScene scene0;
    RenderMonitor* monitor = nullptr;         // monitored render (rc_render): cancel word and progress, else null
    unsigned long long budgetNs = kNoBudget;  // the render's time budget (kNoBudget: none)
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
// The same pass in two halves, for work between the last shade and the film
// update (cache lookups): generate + segments, then accumulate.
cudaError_t launch_path_segments(const PassParams& p, int order, int counting, const PassShape& shape,
                                 cudaStream_t stream, int numSMs, const cudaEvent_t* extendEvents);
cudaError_t launch_path_accumulate(const PassParams& p, cudaStream_t stream);
// Training targets of the pass's training paths (radiance of each vertex's
// suffix, written over the bounce factors) and the sample index list.
cudaError_t launch_nrc_targets(const PassParams& p, cudaStream_t stream);

// Reinhard / passthrough resolve of the film into out (float4 per pixel).
// partials needs tone_partials_bytes(pixels) bytes.
size_t tone_partials_bytes(uint64_t pixels);
// The filter record of a General record (the reference's filter constructors'
// defaults; BOX takes filter_radius).
FilterSpec filter_spec(const rc_general& g);
cudaError_t launch_tonemap(const float4* film, uint64_t pixels, int type, int applyGamma, int shouldClamp,
                           double gamma, double key, void* partials, float4* out, cudaStream_t stream, int numSMs);
cudaError_t launch_linear(const float4* film, uint64_t pixels, float4* out, cudaStream_t stream);
// acc += film (float64); clear != 0 zeroes the film afterwards.
cudaError_t launch_film_accumulate_f64(float4* film, uint64_t pixels, double4_32a* acc, int clear, cudaStream_t stream);
// Display-space RMSE of film vs truth (float64), result in device memory.
size_t rmse_scratch_bytes();
cudaError_t launch_rmse_f64(const float4* film, const double4_32a* truth, uint64_t pixels, int applyGamma, int shouldClamp,
                            double gamma, double key, void* scratch, double* result, cudaStream_t stream, int numSMs);

}  // namespace rcx
