// Host orchestration of the PATH tracer and of the film read-back / tone
// mapping entry points (rc_render for PATH, rc_resolve, rc_read_linear,
// rc_read_film).

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "host_internal.h"
#include "pathtrace.h"

using namespace rcx;

namespace
{

// Target slots per pass: 4M paths x 88 B of state = 352 MB.
constexpr uint64_t kTargetSlots = uint64_t(1) << 22;

rc_status fail(rc_tracer* h, rc_status s, const std::string& msg)
{
    h->err = msg;
    return s;
}

rc_status cuda_fail(rc_tracer* h, cudaError_t e, const char* what)
{
    std::string msg = std::string(what) + ": " + cudaGetErrorString(e);
    return fail(h, e == cudaErrorMemoryAllocation ? RC_OOM : RC_CUDA, msg);
}

#define RC_CUDA_TRY(h, expr, what)             \
    do                                         \
    {                                          \
        cudaError_t e_ = (expr);               \
        if (e_ != cudaSuccess)                 \
            return cuda_fail((h), e_, (what)); \
    } while (0)

rc_status grow(rc_tracer* h, void** ptr, size_t* cap, size_t bytes, const char* what)
{
    if (*ptr && *cap >= bytes)
        return RC_OK;
    if (*ptr)
    {
        cudaFree(*ptr);
        h->deviceBytes -= *cap;
        *ptr = nullptr;
        *cap = 0;
    }
    cudaError_t e = cudaMalloc(ptr, bytes);
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        return cuda_fail(h, e, what);
    }
    *cap = bytes;
    h->deviceBytes += bytes;
    return RC_OK;
}

}  // namespace

namespace rcx
{

rc_status device_grow(rc_tracer* h, void** ptr, size_t* cap, size_t bytes, const char* what)
{
    return grow(h, ptr, cap, bytes, what);
}

void release_render_buffers(rc_tracer* h)
{
    void** ptrs[] = { &h->dPath, reinterpret_cast<void**>(&h->dCounts), &h->dTone, &h->dImage, &h->dTables };
    size_t* caps[] = { &h->capPath, &h->capCounts, &h->capTone, &h->capImage, &h->capTables };
    for (int i = 0; i < 5; ++i)
    {
        if (*ptrs[i])
        {
            cudaFree(*ptrs[i]);
            h->deviceBytes -= *caps[i];
            *ptrs[i] = nullptr;
            *caps[i] = 0;
        }
    }
    h->pathSlots = 0;
}

FilterSpec filter_spec(const rc_general& g)
{
    FilterSpec f{};
    f.type = g.filter_type;
    switch (g.filter_type)
    {
    case RC_FILTER_BOX:
        // BoxFilter::setRadius (BoxFilter.cpp:15-21): weight = 1 / (2 r)
        f.rx = g.filter_radius[0];
        f.ry = g.filter_radius[1];
        f.ax = 1.0f / (2.0f * f.rx);
        f.ay = 1.0f / (2.0f * f.ry);
        break;
    case RC_FILTER_TENT:
        // TentFilter() radius 1 (TentFilter.h:16)
        f.rx = f.ry = 1.0f;
        f.ax = f.ay = 1.0f;
        break;
    case RC_FILTER_BELL:
        f.rx = f.ry = 1.5f;  // BellFilter.cpp:23-27
        break;
    case RC_FILTER_GAUSSIAN:
    {
        // GaussianFilter(1, 1): alpha = 1 / (sqrt(2 pi) sd), beta = -1 / (2 sd^2),
        // radius = 7.43384 sd / 2 (GaussianFilter.cpp:12-21)
        const double sd = 1.0;
        f.ax = f.ay = float(1.0 / (std::sqrt(2.0 * 3.14159265358979323846) * sd));
        f.bx = f.by = float(-1.0 / (2.0 * sd * sd));
        f.rx = f.ry = float((7.43384 * sd) / 2.0);
        break;
    }
    case RC_FILTER_MITCHELL:
    {
        // MitchellFilter(1/3, 1/3), radius 2 (MitchellFilter.h:16, .cpp:8-36):
        // the two cubics with the 1/6 folded in
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
        f.rx = f.ry = 2.0f;  // LanczosSincFilter(2, 2)
        break;
    }
    return f;
}

// Fills the per-scene record the pass kernels read (pathtrace.h).
PathScene path_scene(const rc_tracer* h, uint64_t pixelStart)
{
    const rc_general& g = h->general;
    PathScene ps{};
    ps.sc.nodes = h->dNodes;
    ps.sc.tris = h->dTris;
    ps.sc.shade = h->dShade;
    ps.sc.mats = h->dMats;
    ps.sc.rootLink = h->rootLink;
    ps.sc.numTris = int(h->nTris);
    ps.sc.numMats = int(h->nMats);
    ps.sc.tlas = h->dTlas;
    ps.sc.instances = h->dInstances;
    ps.sc.tlasRoot = h->tlasRoot;
    ps.sc.numInstances = int(h->nInstances);
    ps.sc.wide = h->dWide;
    ps.sc.wideRoot = h->wideRoot;
    for (int k = 0; k < 3; ++k)
    {
        ps.cam.pos[k] = h->camera.position[k];
        ps.cam.fwd[k] = h->camera.forward[k];
        ps.cam.right[k] = h->camera.right[k];
        ps.cam.up[k] = h->camera.up[k];
        ps.cam.center[k] = h->camera.image_plane_center[k];
    }
    ps.cam.aspect = h->camera.aspect_ratio;
    ps.cam.ipw = h->camera.image_plane_width;
    ps.cam.iph = h->camera.image_plane_height;
    ps.film = h->dFilm;
    ps.pixelStart = pixelStart;
    ps.width = int64_t(h->width);
    ps.n = g.multi_sample_count_sqrt;
    ps.P = g.path_sample_count;
    ps.spp = g.multi_sample_count_sqrt * g.multi_sample_count_sqrt * g.path_sample_count;
    ps.samplerType = g.multi_sampler_type;
    ps.filter = filter_spec(g);
    ps.rayStartOffset = g.ray_start_offset;
    ps.maxPathLength = g.max_path_length;
    ps.rrDepth = g.russian_roulette_depth;
    ps.frame = h->frameIndex;
    ps.skyOn = (g.flags & RC_GENERAL_SKY) ? 1 : 0;
    for (int k = 0; k < 3; ++k)
        ps.sky[k] = g.background[k];
    ps.seed = g.seed;
    return ps;
}

PassParams pass_params(void* state, uint64_t slots, unsigned* counts, DevControl* ctl)
{
    char* base = static_cast<char*>(state);
    const size_t S = size_t(slots);
    PassParams p{};
    p.o = reinterpret_cast<float4*>(base);
    p.d = reinterpret_cast<float4*>(base + S * 16);
    p.thr = reinterpret_cast<float4*>(base + S * 32);
    p.res = reinterpret_cast<float4*>(base + S * 48);
    p.hit = reinterpret_cast<int4*>(base + S * 64);
    p.qa = reinterpret_cast<int*>(base + S * 80);
    p.qb = reinterpret_cast<int*>(base + S * 84);
    p.chunkOf = reinterpret_cast<int*>(base + S * 88);
    p.counts = counts;
    p.ctl = ctl;
    return p;
}

rc_status render_path(rc_tracer* h, uint64_t pixelStart, uint64_t count, RenderWatch* watch)
{
    const volatile int32_t* cancel = watch ? watch->cancel : nullptr;
    const rc_general& g = h->general;
    {
        rc_status ws = ensure_wide(h);
        if (ws != RC_OK)
            return ws;
    }
    const uint64_t spp = uint64_t(g.multi_sample_count_sqrt) * uint64_t(g.multi_sample_count_sqrt) *
                         uint64_t(g.path_sample_count);
    if (spp > kTargetSlots)
        return fail(h, RC_UNSUPPORTED, "render: samples per pixel exceed one pass");
    const uint64_t pixelsPerPass = std::max<uint64_t>(1, kTargetSlots / spp);
    const uint64_t slots = std::min<uint64_t>(pixelsPerPass, count) * spp;
    const uint64_t passes = (count + pixelsPerPass - 1) / pixelsPerPass;

    if (h->pathSlots < slots)
    {
        rc_status s = grow(h, &h->dPath, &h->capPath, size_t(slots) * kPathBytesPerSlot, "allocate path state");
        if (s != RC_OK)
            return s;
        h->pathSlots = slots;
    }
    size_t countsBytes = size_t(g.max_path_length + 1) * 4 * sizeof(unsigned);
    {
        void* p = h->dCounts;
        size_t cap = h->capCounts;
        rc_status s = grow(h, &p, &cap, countsBytes, "allocate queue counters");
        h->dCounts = static_cast<unsigned*>(p);
        h->capCounts = cap;
        if (s != RC_OK)
            return s;
    }

    // Scene record + one chunk per pass.
    std::vector<unsigned char> table(sizeof(PathScene) + size_t(passes) * sizeof(PathChunk));
    PathScene ps = path_scene(h, pixelStart);
    std::memcpy(table.data(), &ps, sizeof(ps));
    PathChunk* chunks = reinterpret_cast<PathChunk*>(table.data() + sizeof(PathScene));
    for (uint64_t i = 0; i < passes; ++i)
    {
        uint64_t done = i * pixelsPerPass;
        chunks[i] = PathChunk{ 0, 0, 0, uint32_t(std::min(pixelsPerPass, count - done)), done };
    }
    {
        rc_status s = grow(h, &h->dTables, &h->capTables, table.size(), "allocate pass tables");
        if (s != RC_OK)
            return s;
    }
    RC_CUDA_TRY(h, cudaMemcpyAsync(h->dTables, table.data(), table.size(), cudaMemcpyHostToDevice, h->stream),
                "upload pass tables");
    const PathScene* dScene = static_cast<const PathScene*>(h->dTables);
    const PathChunk* dChunks = reinterpret_cast<const PathChunk*>(static_cast<char*>(h->dTables) + sizeof(PathScene));

    // Events around every extend launch of every pass (stage 0 timing).
    const size_t needEvents = size_t(passes) * size_t(2 * std::max(g.max_path_length, 0));
    const bool timeStages = needEvents <= 4096;
    while (timeStages && h->evPool.size() < needEvents)
    {
        cudaEvent_t e;
        RC_CUDA_TRY(h, cudaEventCreate(&e), "create event");
        h->evPool.push_back(e);
    }

    PassParams pp = pass_params(h->dPath, h->pathSlots, h->dCounts, h->dCtl);
    pp.scenes = dScene;
    pp.numChunks = 1;
    pp.segments = g.max_path_length;
    pp.instanced = h->nInstances > 0 ? 1 : 0;
    pp.wide = h->dWide != nullptr && h->nInstances == 0 ? 1 : 0;
    pp.singleScene = 1;
    pp.scene0 = ps.sc;
    if (watch)
    {
        pp.monitor = watch->dev;
        pp.budgetNs = watch->budgetNs;
    }
    PassShape shape;
    const bool nrc = nrc_active(h);
    if (nrc)
    {
        rc_status s = nrc_prepare(h, slots, g.max_path_length);
        if (s != RC_OK)
            return s;
    }

    RC_CUDA_TRY(h, cudaMemsetAsync(h->dCtl, 0, sizeof(DevControl), h->stream), "reset control block");
    RC_CUDA_TRY(h, cudaEventRecord(h->ev0, h->stream), "record start event");
    for (uint64_t pass = 0; pass < passes; ++pass)
    {
        if (pass > 0 && cancel && *cancel)
        {
            // raised while the passes were being queued: the device stops the
            // passes already queued at their next work-queue check
            if (watch && watch->dev)
                h->monHost->cancel = 1;
            cudaStreamSynchronize(h->stream);
            h->frameIndex++;
            DevControl ctl;
            if (cudaMemcpy(&ctl, h->dCtl, sizeof(ctl), cudaMemcpyDeviceToHost) == cudaSuccess && watch &&
                watch->pixels)
                __atomic_store_n(watch->pixels, uint64_t(ctl.progress), __ATOMIC_RELAXED);
            return fail(h, RC_CANCELLED, "render: cancelled");
        }
        pp.chunks = dChunks + pass;
        pp.npixels = int(chunks[pass].pixels);
        pp.nslots = int(uint64_t(chunks[pass].pixels) * spp);
        RC_CUDA_TRY(h, cudaMemsetAsync(h->dCounts, 0, countsBytes, h->stream), "reset queue counters");
        const cudaEvent_t* ev = timeStages ? h->evPool.data() + pass * size_t(2 * g.max_path_length) : nullptr;
        if (!nrc)
        {
            RC_CUDA_TRY(h, launch_path_pass(pp, h->order, h->counting, shape, h->stream, h->numSMs, ev),
                        "launch path-tracing pass");
            continue;
        }
        nrc_pass_state(h, pp, uint32_t(pass));
        RC_CUDA_TRY(h, launch_path_segments(pp, h->order, h->counting, shape, h->stream, h->numSMs, ev),
                    "launch path-tracing pass");
        rc_status s = nrc_lookups(h, pp);
        if (s == RC_OK)
        {
            RC_CUDA_TRY(h, launch_path_accumulate(pp, h->stream), "launch film update");
            s = nrc_train_pass(h, pp);
        }
        if (s != RC_OK)
            return s;
    }
    RC_CUDA_TRY(h, cudaEventRecord(h->ev1, h->stream), "record end event");
    {
        // before the read-back below: a copy into pageable memory returns
        // only once the kernels are done
        rc_status ws = wait_render(h, watch, h->ev1);
        if (ws != RC_OK)
            return ws;
    }
    DevControl ctl;
    RC_CUDA_TRY(h, cudaMemcpyAsync(&ctl, h->dCtl, sizeof(ctl), cudaMemcpyDeviceToHost, h->stream),
                "read control block");
    RC_CUDA_TRY(h, cudaStreamSynchronize(h->stream), "path tracing");
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    double extendMs = 0.0;
    if (timeStages)
    {
        for (size_t i = 0; i + 1 < needEvents; i += 2)
        {
            float m = 0.0f;
            cudaEventElapsedTime(&m, h->evPool[i], h->evPool[i + 1]);
            extendMs += double(m);
        }
    }
    if (nrc)
    {
        float tm = 0.0f;
        cudaEventElapsedTime(&tm, h->nrc.evTrain0, h->nrc.evTrain1);
        h->nrc.trainMs = double(tm);
    }
    h->stats.last_ms = double(ms);
    h->stats.stage_ms[0] = extendMs;
    h->stats.stage_ms[1] = double(ms) - extendMs;
    h->stats.rays_traced = ctl.stats[0];
    h->stats.node_visits = ctl.stats[1];
    h->stats.tri_tests = ctl.stats[2];
    h->stats.stage_rays[0] = ctl.stats[0];
    h->stats.stage_nodes[0] = ctl.stats[1];
    h->stats.stage_tris[0] = ctl.stats[2];
    h->stats.stage_rays[1] = h->stats.stage_nodes[1] = h->stats.stage_tris[1] = 0;
    h->frameIndex++;
    if (watch && watch->pixels)
        __atomic_store_n(watch->pixels, uint64_t(ctl.progress), __ATOMIC_RELAXED);
    if ((ctl.error & kNrcTcTimeout) && !(ctl.error & kErrStack))
        return fail(h, RC_DEVICE_ERROR, "path tracing: a radiance-cache tensor-core wait timed out");
    return render_outcome(h, ctl.error, "path tracing");
}

}  // namespace rcx

extern "C" {

rc_status rc_resolve(rc_tracer* h, float* out_rgba)
{
    if (!h)
        return RC_INVALID_ARG;
    if (!h->dFilm || !out_rgba)
        return fail(h, RC_NOT_READY, "resolve: no film or null output");
    cudaSetDevice(h->device);
    rc_status s = grow(h, &h->dTone, &h->capTone, tone_partials_bytes(h->filmPixels), "allocate tone scratch");
    if (s != RC_OK)
        return s;
    const rc_tonemapper& t = h->tonemapper;
    // Where the device reaches the caller's buffer (page-locked memory, or
    // resident pageable memory on a Grace host) and it is 16-byte aligned,
    // the mapping kernel writes the image there over the host link; else it
    // writes a device image that one copy brings back (RC_RESOLVE_COPY=1 in
    // the environment forces the copy).
    static const bool forceCopy = [] {
        const char* v = std::getenv("RC_RESOLVE_COPY");
        return v && v[0] == '1';
    }();
    float4* direct = nullptr;
    if (!forceCopy && (reinterpret_cast<uintptr_t>(out_rgba) & 15u) == 0)
        direct = static_cast<float4*>(device_view(h, out_rgba, size_t(h->filmPixels) * sizeof(float4)));
    if (direct)
    {
        RC_CUDA_TRY(h,
                    launch_tonemap(h->dFilm, h->filmPixels, t.type, t.apply_gamma, t.should_clamp, t.gamma, t.key,
                                   h->dTone, direct, h->stream, h->numSMs),
                    "launch tone mapping");
        RC_CUDA_TRY(h, cudaStreamSynchronize(h->stream), "resolve");
        return RC_OK;
    }
    if ((s = grow(h, &h->dImage, &h->capImage, size_t(h->filmPixels) * sizeof(float4), "allocate image")) != RC_OK)
        return s;
    RC_CUDA_TRY(h,
                launch_tonemap(h->dFilm, h->filmPixels, t.type, t.apply_gamma, t.should_clamp, t.gamma, t.key,
                               h->dTone, static_cast<float4*>(h->dImage), h->stream, h->numSMs),
                "launch tone mapping");
    RC_CUDA_TRY(h,
                cudaMemcpyAsync(out_rgba, h->dImage, size_t(h->filmPixels) * sizeof(float4), cudaMemcpyDeviceToHost,
                                h->stream),
                "download image");
    RC_CUDA_TRY(h, cudaStreamSynchronize(h->stream), "resolve");
    return RC_OK;
}

rc_status rc_tonemap_film(rc_tracer* h, const float* film_rgbw, uint64_t pixels, float* out_rgba)
{
    if (!h)
        return RC_INVALID_ARG;
    if (!film_rgbw || !out_rgba || pixels == 0 || pixels > (uint64_t(1) << 31))
        return fail(h, RC_INVALID_ARG, "tonemap_film: null buffer or bad pixel count");
    cudaSetDevice(h->device);
    size_t bytes = size_t(pixels) * sizeof(float4);
    rc_status s = grow(h, &h->dTone, &h->capTone, tone_partials_bytes(pixels), "allocate tone scratch");
    if (s != RC_OK)
        return s;
    if ((s = grow(h, &h->dImage, &h->capImage, 2 * bytes, "allocate image")) != RC_OK)
        return s;
    float4* dIn = static_cast<float4*>(h->dImage);
    float4* dOut = dIn + pixels;
    const rc_tonemapper& t = h->tonemapper;
    RC_CUDA_TRY(h, cudaMemcpyAsync(dIn, film_rgbw, bytes, cudaMemcpyHostToDevice, h->stream), "upload film");
    RC_CUDA_TRY(h,
                launch_tonemap(dIn, pixels, t.type, t.apply_gamma, t.should_clamp, t.gamma, t.key, h->dTone, dOut,
                               h->stream, h->numSMs),
                "launch tone mapping");
    RC_CUDA_TRY(h, cudaMemcpyAsync(out_rgba, dOut, bytes, cudaMemcpyDeviceToHost, h->stream), "download image");
    RC_CUDA_TRY(h, cudaStreamSynchronize(h->stream), "tonemap_film");
    return RC_OK;
}

rc_status rc_read_linear(rc_tracer* h, float* out_rgba)
{
    if (!h)
        return RC_INVALID_ARG;
    if (!h->dFilm || !out_rgba)
        return fail(h, RC_NOT_READY, "read_linear: no film or null output");
    cudaSetDevice(h->device);
    rc_status s = grow(h, &h->dImage, &h->capImage, size_t(h->filmPixels) * sizeof(float4), "allocate image");
    if (s != RC_OK)
        return s;
    RC_CUDA_TRY(h, launch_linear(h->dFilm, h->filmPixels, static_cast<float4*>(h->dImage), h->stream),
                "launch linear resolve");
    RC_CUDA_TRY(h,
                cudaMemcpyAsync(out_rgba, h->dImage, size_t(h->filmPixels) * sizeof(float4), cudaMemcpyDeviceToHost,
                                h->stream),
                "download linear image");
    RC_CUDA_TRY(h, cudaStreamSynchronize(h->stream), "read_linear");
    return RC_OK;
}

rc_status rc_film_accumulate_f64(rc_tracer* h, double* d_acc, int32_t clear_film)
{
    if (!h)
        return RC_INVALID_ARG;
    if (!h->dFilm || !d_acc)
        return fail(h, RC_NOT_READY, "film_accumulate_f64: no film or null accumulator");
    if (reinterpret_cast<uintptr_t>(d_acc) & 31u)
        return fail(h, RC_INVALID_ARG, "film_accumulate_f64: accumulator must be 32-byte aligned");
    cudaSetDevice(h->device);
    RC_CUDA_TRY(h,
                launch_film_accumulate_f64(h->dFilm, h->filmPixels, reinterpret_cast<double4_32a*>(d_acc), clear_film,
                                           h->stream),
                "launch float64 accumulation");
    RC_CUDA_TRY(h, cudaStreamSynchronize(h->stream), "film_accumulate_f64");
    return RC_OK;
}

rc_status rc_film_rmse_f64(rc_tracer* h, const double* d_truth, double* rmse)
{
    if (!h)
        return RC_INVALID_ARG;
    if (!h->dFilm || !d_truth || !rmse)
        return fail(h, RC_NOT_READY, "film_rmse_f64: no film or null buffer");
    if (reinterpret_cast<uintptr_t>(d_truth) & 31u)
        return fail(h, RC_INVALID_ARG, "film_rmse_f64: truth must be 32-byte aligned");
    cudaSetDevice(h->device);
    rc_status s = grow(h, &h->dRmse, &h->capRmse, rmse_scratch_bytes() + 64, "allocate rmse scratch");
    if (s != RC_OK)
        return s;
    // rmse_scratch_bytes() is a multiple of 8
    double* dResult = reinterpret_cast<double*>(static_cast<char*>(h->dRmse) + rmse_scratch_bytes());
    const rc_tonemapper& t = h->tonemapper;
    RC_CUDA_TRY(h,
                launch_rmse_f64(h->dFilm, reinterpret_cast<const double4_32a*>(d_truth), h->filmPixels, t.apply_gamma,
                                t.should_clamp, t.gamma, t.key, h->dRmse, dResult, h->stream, h->numSMs),
                "launch rmse");
    RC_CUDA_TRY(h, cudaMemcpyAsync(rmse, dResult, sizeof(double), cudaMemcpyDeviceToHost, h->stream), "read rmse");
    RC_CUDA_TRY(h, cudaStreamSynchronize(h->stream), "film_rmse_f64");
    return RC_OK;
}

rc_status rc_read_film(rc_tracer* h, float* out_rgbw)
{
    if (!h)
        return RC_INVALID_ARG;
    if (!h->dFilm || !out_rgbw)
        return fail(h, RC_NOT_READY, "read_film: no film or null output");
    cudaSetDevice(h->device);
    RC_CUDA_TRY(h,
                cudaMemcpyAsync(out_rgbw, h->dFilm, size_t(h->filmPixels) * sizeof(float4), cudaMemcpyDeviceToHost,
                                h->stream),
                "download film");
    RC_CUDA_TRY(h, cudaStreamSynchronize(h->stream), "read_film");
    return RC_OK;
}

}  // extern "C"
