// Batched path tracing (rc_batch_*): many independent scenes in one CUDA-graph
// launch.
//
// Each scene lives in its own rc_tracer (scene buffers, film, records). The
// batch plans passes per scene-size bucket: a pass is filled with whole-pixel
// chunks of the bucket's scenes up to the bucket's slot count, so scenes of
// very different sizes share passes and no pass runs half empty. All passes
// of a frame are captured once into a CUDA graph (memsets, the pass kernels,
// an event-record node after every pass); a frame is then one graph launch.
// The scene table (including each scene's frame counter) lives in device
// memory and is refreshed before each launch, so the captured graph stays
// valid across frames. The autotuner times candidate pass sizes and block
// shapes per bucket on the bucket's first paths and keeps the fastest.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "host_internal.h"
#include "pathtrace.h"

using namespace rcx;

namespace
{

constexpr int kBuckets = 4;
constexpr uint32_t kBucketMin[kBuckets] = { 0, 16384, 131072, 1048576 };
constexpr uint32_t kSlotChoices[3] = { 1u << 20, 1u << 21, 1u << 22 };

struct Pass
{
    int bucket;
    uint32_t firstChunk;
    int numChunks;
    uint64_t nslots;
    uint64_t npixels;
    int segments;
};

}  // namespace

struct rc_batch
{
    int device = 0;
    int numSMs = 1;
    cudaStream_t stream = nullptr;
    std::string err;

    std::vector<rc_tracer*> scenes;
    std::vector<int> bucketOf;
    rc_batch_tuning tuning{};

    void* dPath = nullptr;
    size_t capPath = 0;
    uint64_t pathSlots = 0;
    void* dCounts = nullptr;
    size_t capCounts = 0;
    void* dScenes = nullptr;
    size_t capScenes = 0;
    void* dChunks = nullptr;
    size_t capChunks = 0;
    DevControl* dCtl = nullptr;

    std::vector<Pass> passes;
    std::vector<PathChunk> chunks;
    std::vector<int> sceneLastPass;

    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool graphValid = false;
    std::vector<cudaEvent_t> passEvents;
    cudaEvent_t evStart = nullptr;
    cudaEvent_t evEnd = nullptr;

    rc_batch_stats stats{};
};

namespace
{

rc_status fail(rc_batch* b, rc_status s, const std::string& msg)
{
    b->err = msg;
    return s;
}

rc_status cuda_fail(rc_batch* b, cudaError_t e, const char* what)
{
    return fail(b, e == cudaErrorMemoryAllocation ? RC_OOM : RC_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define RB_TRY(b, expr, what)                  \
    do                                         \
    {                                          \
        cudaError_t e_ = (expr);               \
        if (e_ != cudaSuccess)                 \
            return cuda_fail((b), e_, (what)); \
    } while (0)

rc_status grow(rc_batch* b, void** ptr, size_t* cap, size_t bytes, const char* what)
{
    if (*ptr && *cap >= bytes)
        return RC_OK;
    if (*ptr)
    {
        cudaFree(*ptr);
        *ptr = nullptr;
        *cap = 0;
    }
    cudaError_t e = cudaMalloc(ptr, bytes);
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        return cuda_fail(b, e, what);
    }
    *cap = bytes;
    return RC_OK;
}

void drop_graph(rc_batch* b)
{
    if (b->exec)
        cudaGraphExecDestroy(b->exec);
    if (b->graph)
        cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->graphValid = false;
}

uint64_t scene_spp(const rc_tracer* h)
{
    const rc_general& g = h->general;
    return uint64_t(g.multi_sample_count_sqrt) * uint64_t(g.multi_sample_count_sqrt) * uint64_t(g.path_sample_count);
}

// Packs whole-pixel chunks of the scenes into passes, bucket by bucket.
// onlyBucket >= 0 restricts the plan to one bucket; maxPaths > 0 stops once
// that many paths are planned (the autotuner's sample).
void plan(rc_batch* b, int onlyBucket, uint64_t maxPaths, const uint32_t* slotsPerBucket)
{
    b->passes.clear();
    b->chunks.clear();
    b->sceneLastPass.assign(b->scenes.size(), -1);
    uint64_t planned = 0;
    for (int bucket = 0; bucket < kBuckets; ++bucket)
    {
        if (onlyBucket >= 0 && bucket != onlyBucket)
            continue;
        const uint64_t slots = slotsPerBucket[bucket];
        bool open = false;
        uint64_t remaining = 0;
        for (size_t i = 0; i < b->scenes.size(); ++i)
        {
            if (b->bucketOf[i] != bucket)
                continue;
            const rc_tracer* h = b->scenes[i];
            const uint64_t spp = scene_spp(h);
            const uint64_t pixels = h->filmPixels;
            uint64_t done = 0;
            while (done < pixels)
            {
                if (maxPaths && planned >= maxPaths)
                    return;
                if (!open || remaining < spp)
                {
                    b->passes.push_back(Pass{ bucket, uint32_t(b->chunks.size()), 0, 0, 0, 0 });
                    remaining = slots;
                    open = true;
                }
                Pass& p = b->passes.back();
                uint64_t take = std::min(pixels - done, remaining / spp);
                PathChunk c;
                c.scene = int(i);
                c.slotBegin = uint32_t(p.nslots);
                c.pixelPassBegin = uint32_t(p.npixels);
                c.pixels = uint32_t(take);
                c.pixelLocalBegin = done;
                b->chunks.push_back(c);
                p.numChunks++;
                p.nslots += take * spp;
                p.npixels += take;
                p.segments = std::max(p.segments, h->general.max_path_length);
                remaining -= take * spp;
                done += take;
                planned += take * spp;
                b->sceneLastPass[i] = int(b->passes.size()) - 1;
            }
        }
    }
}

rc_status upload_plan(rc_batch* b)
{
    uint64_t maxSlots = 0;
    int maxSeg = 0;
    for (const Pass& p : b->passes)
    {
        maxSlots = std::max(maxSlots, p.nslots);
        maxSeg = std::max(maxSeg, p.segments);
    }
    rc_status s;
    if (b->pathSlots < maxSlots)
    {
        if ((s = grow(b, &b->dPath, &b->capPath, size_t(maxSlots) * kPathBytesPerSlot, "allocate path state")) !=
            RC_OK)
            return s;
        b->pathSlots = maxSlots;
    }
    if ((s = grow(b, &b->dCounts, &b->capCounts, size_t(maxSeg + 1) * 4 * sizeof(unsigned), "allocate counters")) !=
            RC_OK ||
        (s = grow(b, &b->dScenes, &b->capScenes, std::max<size_t>(1, b->scenes.size()) * sizeof(PathScene),
                  "allocate scene table")) != RC_OK ||
        (s = grow(b, &b->dChunks, &b->capChunks, std::max<size_t>(1, b->chunks.size()) * sizeof(PathChunk),
                  "allocate chunk table")) != RC_OK)
        return s;
    if (!b->chunks.empty())
        RB_TRY(b, cudaMemcpy(b->dChunks, b->chunks.data(), b->chunks.size() * sizeof(PathChunk),
                             cudaMemcpyHostToDevice),
               "upload chunk table");
    return RC_OK;
}

rc_status upload_scene_table(rc_batch* b)
{
    rc_status s = grow(b, &b->dScenes, &b->capScenes, std::max<size_t>(1, b->scenes.size()) * sizeof(PathScene),
                       "allocate scene table");
    if (s != RC_OK)
        return s;
    std::vector<PathScene> table(b->scenes.size());
    for (size_t i = 0; i < b->scenes.size(); ++i)
    {
        if ((s = ensure_wide(b->scenes[i])) != RC_OK)
            return fail(b, s, "batch: scene " + std::to_string(i) + ": " + b->scenes[i]->err);
        table[i] = path_scene(b->scenes[i], 0);
    }
    RB_TRY(b, cudaMemcpyAsync(b->dScenes, table.data(), table.size() * sizeof(PathScene), cudaMemcpyHostToDevice,
                              b->stream),
           "upload scene table");
    // the table's host copy must outlive the copy
    RB_TRY(b, cudaStreamSynchronize(b->stream), "upload scene table");
    return RC_OK;
}

PassShape shape_of(const rc_batch* b, int bucket)
{
    PassShape sh;
    sh.extendBlock = b->tuning.extend_block[bucket];
    sh.shadeBlock = b->tuning.shade_block[bucket];
    return sh;
}

// Enqueues every pass of the current plan on the batch's stream.
rc_status enqueue_passes(rc_batch* b, bool recordPassEvents)
{
    for (size_t k = 0; k < b->passes.size(); ++k)
    {
        const Pass& ps = b->passes[k];
        RB_TRY(b, cudaMemsetAsync(b->dCounts, 0, size_t(ps.segments + 1) * 4 * sizeof(unsigned), b->stream),
               "reset queue counters");
        PassParams pp = pass_params(b->dPath, b->pathSlots, static_cast<unsigned*>(b->dCounts), b->dCtl);
        pp.scenes = static_cast<const PathScene*>(b->dScenes);
        pp.chunks = static_cast<const PathChunk*>(b->dChunks) + ps.firstChunk;
        pp.numChunks = ps.numChunks;
        pp.nslots = int(ps.nslots);
        pp.npixels = int(ps.npixels);
        pp.segments = ps.segments;
        pp.wide = 1;
        for (const rc_tracer* h : b->scenes)
            if (!h->dWide || h->nInstances > 0)
                pp.wide = 0;
        RB_TRY(b, launch_path_pass(pp, RC_ORDER_NEAREST, 0, shape_of(b, ps.bucket), b->stream, b->numSMs, nullptr),
               "launch pass");
        if (recordPassEvents)
            RB_TRY(b, cudaEventRecordWithFlags(b->passEvents[k], b->stream, cudaEventRecordExternal),
                   "record pass event");
    }
    return RC_OK;
}

rc_status capture(rc_batch* b)
{
    drop_graph(b);
    uint32_t slots[kBuckets];
    for (int k = 0; k < kBuckets; ++k)
        slots[k] = b->tuning.slots[k];
    plan(b, -1, 0, slots);
    rc_status s = upload_plan(b);
    if (s != RC_OK)
        return s;
    while (b->passEvents.size() < b->passes.size())
    {
        cudaEvent_t e;
        RB_TRY(b, cudaEventCreate(&e), "create event");
        b->passEvents.push_back(e);
    }
    RB_TRY(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "begin graph capture");
    rc_status st = RC_OK;
    cudaError_t e = cudaMemsetAsync(b->dCtl, 0, sizeof(DevControl), b->stream);
    if (e == cudaSuccess)
        e = cudaEventRecordWithFlags(b->evStart, b->stream, cudaEventRecordExternal);
    if (e == cudaSuccess)
        st = enqueue_passes(b, true);
    if (e == cudaSuccess && st == RC_OK)
        e = cudaEventRecordWithFlags(b->evEnd, b->stream, cudaEventRecordExternal);
    cudaGraph_t g = nullptr;
    cudaError_t ee = cudaStreamEndCapture(b->stream, &g);
    if (e != cudaSuccess || st != RC_OK || ee != cudaSuccess)
    {
        if (g)
            cudaGraphDestroy(g);
        cudaGetLastError();
        if (st != RC_OK)
            return st;
        return cuda_fail(b, e != cudaSuccess ? e : ee, "capture batch graph");
    }
    b->graph = g;
    RB_TRY(b, cudaGraphInstantiate(&b->exec, b->graph, 0), "instantiate batch graph");
    size_t nodes = 0;
    cudaGraphGetNodes(b->graph, nullptr, &nodes);
    b->stats.graph_nodes = int32_t(nodes);
    b->stats.passes = int32_t(b->passes.size());
    b->graphValid = true;
    return RC_OK;
}

}  // namespace

extern "C" {

rc_status rc_batch_create(rc_batch** out, int device)
{
    if (!out)
        return RC_INVALID_ARG;
    *out = nullptr;
    rc_batch* b = new (std::nothrow) rc_batch();
    if (!b)
        return RC_OOM;
    b->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&b->numSMs, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess)
        e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaEventCreate(&b->evStart);
    if (e == cudaSuccess)
        e = cudaEventCreate(&b->evEnd);
    if (e == cudaSuccess)
        e = cudaMalloc(reinterpret_cast<void**>(&b->dCtl), sizeof(DevControl));
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        rc_batch_destroy(b);
        return e == cudaErrorMemoryAllocation ? RC_OOM : RC_CUDA;
    }
    for (int k = 0; k < kBuckets; ++k)
    {
        b->tuning.bucket_min_triangles[k] = kBucketMin[k];
        b->tuning.slots[k] = 1u << 22;
        b->tuning.extend_block[k] = 128;
        b->tuning.shade_block[k] = 128;
        b->tuning.measured_paths_per_ms[k] = 0.0;
    }
    *out = b;
    return RC_OK;
}

void rc_batch_destroy(rc_batch* b)
{
    if (!b)
        return;
    cudaSetDevice(b->device);
    if (b->stream)
        cudaStreamSynchronize(b->stream);
    drop_graph(b);
    for (rc_tracer* h : b->scenes)
        rc_destroy(h);
    void* bufs[] = { b->dPath, b->dCounts, b->dScenes, b->dChunks, b->dCtl };
    for (void* p : bufs)
        if (p)
            cudaFree(p);
    for (cudaEvent_t e : b->passEvents)
        cudaEventDestroy(e);
    if (b->evStart)
        cudaEventDestroy(b->evStart);
    if (b->evEnd)
        cudaEventDestroy(b->evEnd);
    if (b->stream)
        cudaStreamDestroy(b->stream);
    delete b;
}

const char* rc_batch_last_error(const rc_batch* b) { return b ? b->err.c_str() : "null batch"; }

rc_status rc_batch_add_scene(rc_batch* b, const double* vertices, const uint32_t* material_index, int64_t n,
                             const rc_material* materials, int32_t material_count, uint32_t max_leaf_size,
                             const rc_camera* camera, const rc_general* general, uint64_t width, uint64_t height,
                             int32_t* index)
{
    if (!b)
        return RC_INVALID_ARG;
    if (!camera || !general)
        return fail(b, RC_INVALID_ARG, "batch_add_scene: null camera or general record");
    if (general->tracer_type != RC_TRACER_PATH)
        return fail(b, RC_UNSUPPORTED, "batch_add_scene: only PATH scenes are batched");
    rc_tracer* h = nullptr;
    rc_status s = rc_create(&h, b->device);
    if (s != RC_OK)
        return fail(b, s, "batch_add_scene: could not create the scene's tracer");
    if ((s = rc_upload_scene(h, vertices, material_index, n, materials, material_count, max_leaf_size)) != RC_OK ||
        (s = rc_set_camera(h, camera)) != RC_OK || (s = rc_set_general(h, general)) != RC_OK ||
        (s = rc_resize(h, width, height)) != RC_OK)
    {
        b->err = std::string("batch_add_scene: ") + rc_last_error(h);
        rc_destroy(h);
        return s;
    }
    if (scene_spp(h) > (1u << 20))
    {
        rc_destroy(h);
        return fail(b, RC_UNSUPPORTED, "batch_add_scene: samples per pixel exceed the smallest pass");
    }
    int bucket = 0;
    for (int k = 0; k < kBuckets; ++k)
        if (uint64_t(n) >= kBucketMin[k])
            bucket = k;
    b->scenes.push_back(h);
    b->bucketOf.push_back(bucket);
    b->stats.scenes = int32_t(b->scenes.size());
    drop_graph(b);
    if (index)
        *index = int32_t(b->scenes.size()) - 1;
    return RC_OK;
}

rc_status rc_batch_autotune(rc_batch* b, double budget_ms)
{
    if (!b)
        return RC_INVALID_ARG;
    cudaSetDevice(b->device);
    const int blocks[3] = { 64, 128, 256 };
    double spent = 0.0;
    rc_status s = upload_scene_table(b);
    if (s != RC_OK)
        return s;
    for (int bucket = 0; bucket < kBuckets; ++bucket)
    {
        if (std::find(b->bucketOf.begin(), b->bucketOf.end(), bucket) == b->bucketOf.end())
            continue;
        double best = -1.0;
        for (uint32_t slots : kSlotChoices)
        {
            for (int blk : blocks)
            {
                if (spent > budget_ms && best > 0.0)
                    break;
                uint32_t perBucket[kBuckets];
                for (int k = 0; k < kBuckets; ++k)
                    perBucket[k] = slots;
                plan(b, bucket, uint64_t(1) << 22, perBucket);
                if ((s = upload_plan(b)) != RC_OK)
                    return s;
                int32_t savedE = b->tuning.extend_block[bucket], savedS = b->tuning.shade_block[bucket];
                b->tuning.extend_block[bucket] = blk;
                b->tuning.shade_block[bucket] = blk;
                uint64_t paths = 0;
                for (const Pass& p : b->passes)
                    paths += p.nslots;
                RB_TRY(b, cudaEventRecord(b->evStart, b->stream), "record event");
                if ((s = enqueue_passes(b, false)) != RC_OK)
                    return s;
                RB_TRY(b, cudaEventRecord(b->evEnd, b->stream), "record event");
                RB_TRY(b, cudaStreamSynchronize(b->stream), "autotune run");
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, b->evStart, b->evEnd);
                spent += double(ms);
                double rate = double(paths) / std::max(1e-6, double(ms));
                if (rate > best)
                {
                    best = rate;
                    b->tuning.slots[bucket] = slots;
                    b->tuning.measured_paths_per_ms[bucket] = rate;
                }
                else
                {
                    b->tuning.extend_block[bucket] = savedE;
                    b->tuning.shade_block[bucket] = savedS;
                }
            }
        }
    }
    drop_graph(b);
    return rc_batch_clear(b);
}

rc_status rc_batch_get_tuning(const rc_batch* b, rc_batch_tuning* out)
{
    if (!b || !out)
        return RC_INVALID_ARG;
    *out = b->tuning;
    return RC_OK;
}

rc_status rc_batch_render(rc_batch* b, double* scene_done_ms)
{
    if (!b)
        return RC_INVALID_ARG;
    if (b->scenes.empty())
        return fail(b, RC_NOT_READY, "batch_render: no scenes");
    cudaSetDevice(b->device);
    rc_status s;
    if (!b->graphValid && (s = capture(b)) != RC_OK)
        return s;
    if ((s = upload_scene_table(b)) != RC_OK)
        return s;
    RB_TRY(b, cudaGraphLaunch(b->exec, b->stream), "launch batch graph");
    DevControl ctl;
    RB_TRY(b, cudaMemcpyAsync(&ctl, b->dCtl, sizeof(ctl), cudaMemcpyDeviceToHost, b->stream), "read control block");
    RB_TRY(b, cudaStreamSynchronize(b->stream), "batch render");
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, b->evStart, b->evEnd);
    b->stats.last_ms = double(ms);
    b->stats.rays_traced = ctl.stats[0];
    uint64_t paths = 0;
    for (const Pass& p : b->passes)
        paths += p.nslots;
    b->stats.paths = paths;
    if (scene_done_ms)
    {
        for (size_t i = 0; i < b->scenes.size(); ++i)
        {
            float t = 0.0f;
            int last = b->sceneLastPass[i];
            if (last >= 0)
                cudaEventElapsedTime(&t, b->evStart, b->passEvents[size_t(last)]);
            scene_done_ms[i] = double(t);
        }
    }
    for (rc_tracer* h : b->scenes)
        h->frameIndex++;
    if (ctl.error & 1)
        return fail(b, RC_DEVICE_ERROR, "batch_render: traversal stack overflow");
    return RC_OK;
}

rc_status rc_batch_clear(rc_batch* b)
{
    if (!b)
        return RC_INVALID_ARG;
    for (rc_tracer* h : b->scenes)
    {
        rc_status s = rc_clear(h);
        if (s != RC_OK)
            return fail(b, s, std::string("batch_clear: ") + rc_last_error(h));
    }
    return RC_OK;
}

rc_status rc_batch_read_film(rc_batch* b, int32_t index, float* out_rgbw)
{
    if (!b)
        return RC_INVALID_ARG;
    if (index < 0 || size_t(index) >= b->scenes.size())
        return fail(b, RC_INVALID_ARG, "batch_read_film: bad scene index");
    rc_status s = rc_read_film(b->scenes[size_t(index)], out_rgbw);
    if (s != RC_OK)
        b->err = rc_last_error(b->scenes[size_t(index)]);
    return s;
}

rc_status rc_batch_resolve(rc_batch* b, int32_t index, const rc_tonemapper* tonemapper, float* out_rgba)
{
    if (!b)
        return RC_INVALID_ARG;
    if (index < 0 || size_t(index) >= b->scenes.size())
        return fail(b, RC_INVALID_ARG, "batch_resolve: bad scene index");
    rc_tracer* h = b->scenes[size_t(index)];
    rc_status s = RC_OK;
    if (tonemapper)
        s = rc_set_tonemapper(h, tonemapper);
    if (s == RC_OK)
        s = rc_resolve(h, out_rgba);
    if (s != RC_OK)
        b->err = rc_last_error(h);
    return s;
}

rc_status rc_batch_get_stats(const rc_batch* b, rc_batch_stats* out)
{
    if (!b || !out)
        return RC_INVALID_ARG;
    *out = b->stats;
    return RC_OK;
}

}  // extern "C"
