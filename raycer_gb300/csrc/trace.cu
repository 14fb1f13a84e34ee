// Ray-casting kernels: generic closest/any-hit queries and the RAY tracer's
// frame (one primary ray per pixel + one shadow ray per hit).
//
// Work distribution: persistent blocks (occupancy x SM count) whose warps
// take 32 rays (an 8x4-pixel tile of a whole frame) at a time from a global
// atomic work counter. An uncounted RAY frame is one kernel: each lane whose
// primary ray hit traces its shadow ray right after its tile. Counted frames
// (and RC_TRACE_FUSED=0) keep two stages: the shadow stage is fed by a queue
// that the primary stage fills with one atomicAdd per warp after a ballot
// over the lanes that hit (warp-aggregated compaction), so shadow warps
// carry no missed pixels.

#include <cfloat>
#include <cmath>

#include "kernels.h"
#include <cstdlib>

#include "monitor.cuh"

#include "traverse.cuh"

namespace rcx
{
namespace
{

constexpr int kBlock = 128;

// Minimum resident blocks per SM the ray kernels are compiled for (register
// budget: 10 blocks x 128 threads -> at most 48 registers, no spills).
#ifndef RC_TRACE_MIN_BLOCKS
#define RC_TRACE_MIN_BLOCKS 10
#endif
// The one-kernel RAY frame (primary + shadow walks) at 9 blocks: 56
// registers, no spills; 0.405 ms per 1080p heightfield frame against 0.417
// at 10 blocks (48 registers, spills) and 0.420 at 8.
#ifndef RC_FUSED_MIN_BLOCKS
#define RC_FUSED_MIN_BLOCKS 9
#endif
#ifndef RC_TRACE_TILES
#define RC_TRACE_TILES 1
#endif
constexpr int kWarpsPerBlock = kBlock / 32;

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

__device__ __forceinline__ unsigned warp_fetch(unsigned* head, unsigned amount)
{
    unsigned base = 0;
    if (lane_id() == 0)
        base = atomicAdd(head, amount);
    return __shfl_sync(0xffffffffu, base, 0);
}

__device__ __forceinline__ void flush_counts(DevControl* ctl, int stage, unsigned long long rays, const TravCount& c,
                                             int err)
{
    unsigned long long n = c.nodes, t = c.tris;
    for (int o = 16; o > 0; o >>= 1)
    {
        rays += __shfl_down_sync(0xffffffffu, rays, o);
        n += __shfl_down_sync(0xffffffffu, n, o);
        t += __shfl_down_sync(0xffffffffu, t, o);
    }
    if (lane_id() == 0)
    {
        atomicAdd(&ctl->stats[3 * stage + 0], rays);
        if (n)
            atomicAdd(&ctl->stats[3 * stage + 1], n);
        if (t)
            atomicAdd(&ctl->stats[3 * stage + 2], t);
    }
    if (err)
        atomicOr(&ctl->error, 1);
}

__device__ __forceinline__ int caller_index(const DevScene& sc, int slot)
{
    return __float_as_int(__ldg(&sc.tris[slot].c.z));
}

template <bool ANY, int ORDER, bool COUNT, bool SL>
__global__ void __launch_bounds__(kBlock, RC_TRACE_MIN_BLOCKS) k_cast(DevScene sc, const rc_ray* __restrict__ rays, int n,
                                                 rc_hit* __restrict__ hits, DevControl* ctl)
{
    TravCount cnt{ 0, 0 };
    int err = 0;
    unsigned long long done = 0;
    while (true)
    {
        unsigned base = warp_fetch(&ctl->head[0], 32u);
        if (base >= unsigned(n))
            break;
        int i = int(base + lane_id());
        if (i < n)
        {
            const float4* rp = reinterpret_cast<const float4*>(rays + i);
            float4 r0 = __ldg(rp);
            float4 r1 = __ldg(rp + 1);
            RayF ray = make_ray(v3(r0.x, r0.y, r0.z), v3(r1.x, r1.y, r1.z), r0.w, r1.w);
            HitF h{ -1, FLT_MAX, 0.0f, 0.0f, -1 };
            // SL: the reference order of a single-level scene on the rope records
            bool found = SL ? traverse_stackless<ANY>(sc, ray, h, -1)
                            : traverse_scene<ANY, ORDER, COUNT>(sc, ray, h, cnt, err, -1, -1);
            int4 out;
            // two-level scenes: the flattened index (instance's first + mesh-local)
            out.x = found ? caller_index(sc, h.slot) + (h.inst >= 0 ? __ldg(&sc.instances[h.inst].primBase) : 0) : -1;
            out.y = __float_as_int(found ? h.t : -1.0f);
            out.z = __float_as_int(found ? h.u : 0.0f);
            out.w = __float_as_int(found ? h.v : 0.0f);
            reinterpret_cast<int4*>(hits)[i] = out;
            done++;
        }
    }
    flush_counts(ctl, 0, done, cnt, err);
}

__device__ __forceinline__ RayF primary_ray(const DevCamera& cam, const rc_ray* __restrict__ rays, uint64_t pixel,
                                            int64_t local, int64_t width)
{
    if (rays)
    {
        const float4* rp = reinterpret_cast<const float4*>(rays + local);
        float4 r0 = __ldg(rp);
        float4 r1 = __ldg(rp + 1);
        return make_ray(v3(r0.x, r0.y, r0.z), v3(r1.x, r1.y, r1.z), r0.w, r1.w);
    }
    float px = float(pixel % uint64_t(width));
    float py = float(pixel / uint64_t(width));
    V3 d = camera_dir(cam, px, py);
    return make_ray(v3(cam.pos[0], cam.pos[1], cam.pos[2]), d, 0.0f, FLT_MAX);
}

// The shadow ray of a primary hit, traced where the hit was found: the
// arithmetic of stage 2 below (origin = o + t d, then + L * rayStartOffset;
// the hit's own triangle, of its instance, skipped). Completes the record:
// occluder and flags.
// SOCT >= 0: the light's direction has the signs of octant SOCT (the host
// checked that its inverse is finite), and the walk's box tests use them
// (slab_oct: the same decisions, six FMNMX fewer per box).
template <bool INST, bool SL, int SOCT = -1>
__device__ __forceinline__ void shadow_of(const DevScene& sc, const RayF& ray, const HitF& h, float3 L,
                                          float rayStartOffset, int4& o, TravCount& cnt, int& err)
{
    const V3 dl = v3(L.x, L.y, L.z);
    const RayF sr = make_ray(vfma(dl, rayStartOffset, vfma(ray.d, h.t, ray.o)), dl, 0.0f, FLT_MAX);
    HitF s{ -1, FLT_MAX, 0.0f, 0.0f, -1 };
    bool occ;
    if (INST)
        occ = traverse_instanced<true, false>(sc, sr, s, cnt, err, h.slot, h.inst);
    else if (SL)
        occ = traverse_stackless<true>(sc, sr, s, h.slot);
    else
        occ = traverse<true, ORDER_REF, false, SOCT>(sc, sr, s, cnt, err, h.slot);
    o.z = occ ? caller_index(sc, s.slot) + (INST ? __ldg(&sc.instances[s.inst].primBase) : 0) : -1;
    o.w = 1 | 2 | (occ ? 4 : 0);
}

// Stage 1 of the RAY frame: closest hit of every pixel's primary ray.
// Whole frames (tilesX > 0: camera rays, or caller rays one per pixel) are
// walked in 8x4-pixel tiles, one tile per warp fetch, so a warp's rays are
// spatially coherent; pixel ranges are walked in order.
// PACKET: the warp traverses its 32 rays together (traverse_packet); the
// counted frame keeps one traversal per lane, whose node and triangle counts
// are the algorithm's. INST: a two-level scene (traverse_instanced; the
// record's prim is the flattened index, instance's first + mesh-local, and
// while a shadow ray is to follow its occluder field holds the hit's
// instance, for the shadow ray to skip the hit triangle of that instance).
// FUSED (uncounted frames with a light): each lane whose ray hit traces its
// shadow ray right after the tile's primary rays, with the shadow kernel's
// arithmetic (stage 2 below; SL: the stackless walk), and the pixel's record
// is written once, complete; no queue. The shadow rays of a tile whose
// pixels all hit (or all miss) keep the warp full (or cost nothing); only
// tiles on a silhouette leave lanes idle. With the caller's rays in host
// memory the shadow work then overlaps the ray reads over the host link.
template <int ORDER, bool COUNT, bool PACKET, bool INST, bool FUSED = false, bool SL = false, int SOCT = -1>
__global__ void __launch_bounds__(kBlock, FUSED ? RC_FUSED_MIN_BLOCKS : RC_TRACE_MIN_BLOCKS) k_raycast_primary(DevScene sc, DevCamera cam, const rc_ray* __restrict__ rays,
                                                            uint64_t pixelStart, int64_t count, int64_t width,
                                                            int64_t height, int64_t tilesX, int castShadow,
                                                            rc_cast_pixel* __restrict__ out, int* __restrict__ queue,
                                                            DevControl* ctl, float3 L, float rayStartOffset,
                                                            float4* __restrict__ origins)
{
    static_assert(!(FUSED && COUNT), "counted frames keep the two stages");
    TravCount cnt1{ 0, 0 };  // FUSED: the shadow rays' counts
    unsigned long long done1 = 0;
    __shared__ PacketEntry wstack[PACKET ? kWarpsPerBlock : 1][PACKET ? kMaxStack : 1];
    TravCount cnt{ 0, 0 };
    int err = 0;
    unsigned long long done = 0;
    const int64_t items = tilesX > 0 ? tilesX * ((height + 3) / 4) * 32 : count;
    if (is_watch_warp(sc.monitor, sc.budgetNs))
    {
        watch_queue(sc.monitor, sc.budgetNs, ctl, &ctl->head[0], static_cast<unsigned long long>(items),
                    FUSED ? kPublishEstimate : kPublishNone, static_cast<unsigned long long>(count));
        return;
    }
    while (true)
    {
        unsigned base = warp_fetch(&ctl->head[0], 32u);
        if (int64_t(base) >= items)
            break;
        int64_t i = int64_t(base) + lane_id();
        bool valid = i < items;
        if (tilesX > 0 && valid)
        {
            int64_t tile = i >> 5;
            int64_t px = (tile % tilesX) * 8 + (i & 7);
            int64_t py = (tile / tilesX) * 4 + ((i >> 3) & 3);
            valid = px < width && py < height;
            i = py * width + px;
        }
        bool hitAny = false;
        int hitSlot = -1;
        float4 sorg = make_float4(0.0f, 0.0f, 0.0f, 0.0f);  // shadow-ray origin (+ instance) for `origins`
        if (PACKET)
        {
            // all lanes together, the ray of an invalid lane unused
            RayF ray = primary_ray(cam, rays, valid ? pixelStart + uint64_t(i) : pixelStart, valid ? i : 0, width);
            HitF h{ -1, FLT_MAX, 0.0f, 0.0f, -1 };
            bool found = traverse_packet<ORDER>(sc, ray, h, err, -1, valid, wstack[threadIdx.x >> 5]);
            // the one-kernel and two-stage records are built apart: one shared
            // branch measured 1 % slower on the one-kernel frame
            if (FUSED)
            {
                int4 o;
                o.x = found ? caller_index(sc, h.slot) : -1;
                o.y = __float_as_int(found ? h.t : -1.0f);
                o.z = -1;
                o.w = found ? 1 : 0;
                if (valid && found)
                    shadow_of<false, SL, SOCT>(sc, ray, h, L, rayStartOffset, o, cnt1, err);
                if (valid)
                {
                    reinterpret_cast<int4*>(out)[i] = o;
                    done++;
                    done1 += found ? 1 : 0;
                }
            }
            else if (valid)
            {
                int4 o;
                o.x = found ? caller_index(sc, h.slot) : -1;
                o.y = __float_as_int(found ? h.t : -1.0f);
                o.z = -1;
                o.w = found ? 1 : 0;
                reinterpret_cast<int4*>(out)[i] = o;
                hitAny = found && castShadow;
                hitSlot = h.slot;
                if (origins && hitAny)
                {
                    // the shadow kernel's own arithmetic (ip = o + t d, then + L * offset)
                    const V3 dl = v3(L.x, L.y, L.z);
                    const V3 so = vfma(dl, rayStartOffset, vfma(ray.d, h.t, ray.o));
                    sorg = make_float4(so.x, so.y, so.z, __int_as_float(-1));
                }
                done++;
            }
        }
        else if (valid)
        {
            RayF ray = primary_ray(cam, rays, pixelStart + uint64_t(i), i, width);
            HitF h{ -1, FLT_MAX, 0.0f, 0.0f, -1 };
            bool found;
            if (INST)
                found = traverse_instanced<false, COUNT>(sc, ray, h, cnt, err, -1, -1);
            else
                found = traverse<false, ORDER, COUNT>(sc, ray, h, cnt, err);
            int4 o;
            o.x = found ? caller_index(sc, h.slot) + (INST ? __ldg(&sc.instances[h.inst].primBase) : 0) : -1;
            o.y = __float_as_int(found ? h.t : -1.0f);
            o.z = INST && found && castShadow && !FUSED ? h.inst : -1;
            o.w = found ? 1 : 0;
            if (FUSED)
            {
                if (found)
                {
                    shadow_of<INST, SL, INST ? -1 : SOCT>(sc, ray, h, L, rayStartOffset, o, cnt1, err);
                    done1++;
                }
            }
            else if (origins && found && castShadow)
            {
                const V3 dl = v3(L.x, L.y, L.z);
                const V3 so = vfma(dl, rayStartOffset, vfma(ray.d, h.t, ray.o));
                sorg = make_float4(so.x, so.y, so.z, __int_as_float(INST ? h.inst : -1));
            }
            reinterpret_cast<int4*>(out)[i] = o;
            hitAny = found && castShadow && !FUSED;
            hitSlot = h.slot;
            done++;
        }
        // Warp-aggregated compaction of the hit pixels into the shadow queue.
        unsigned mask = FUSED ? 0u : __ballot_sync(0xffffffffu, hitAny);
        if (mask)
        {
            unsigned qbase = 0;
            if (lane_id() == 0)
                qbase = atomicAdd(&ctl->head[1], unsigned(__popc(mask)));
            qbase = __shfl_sync(0xffffffffu, qbase, 0);
            if (hitAny)
            {
                const unsigned qi = qbase + __popc(mask & ((1u << lane_id()) - 1u));
                reinterpret_cast<int2*>(queue)[qi] = make_int2(int(i), hitSlot);
                if (origins)
                    origins[qi] = sorg;
            }
        }
    }
    flush_counts(ctl, 0, done, cnt, err);
    if (FUSED)
        flush_counts(ctl, 1, done1, cnt1, 0);
}

// Stage 2: one any-hit shadow ray toward the light per queued pixel
// (Raytracer::calculateShadowAmount, Raytracer.cpp:497-522 /
// lighting.cl:28-48): origin = hit position + dirToLight * rayStartOffset;
// the primary hit's own triangle is skipped (see traverse.cuh).
template <bool COUNT, bool INST, bool SL>
__global__ void __launch_bounds__(kBlock, RC_TRACE_MIN_BLOCKS) k_raycast_shadow(DevScene sc, DevCamera cam, const rc_ray* __restrict__ rays,
                                                           uint64_t pixelStart, int64_t width, float3 L,
                                                           float rayStartOffset, rc_cast_pixel* __restrict__ out,
                                                           const int* __restrict__ queue, DevControl* ctl,
                                                           const float4* __restrict__ origins)
{
    TravCount cnt{ 0, 0 };
    int err = 0;
    unsigned long long done = 0;
    const unsigned total = *reinterpret_cast<volatile unsigned*>(&ctl->head[1]);
    while (true)
    {
        unsigned base = warp_fetch(&ctl->head[2], 32u);
        if (base >= total)
            break;
        unsigned q = base + lane_id();
        if (q < total)
        {
            int2 e = reinterpret_cast<const int2*>(queue)[q];
            int i = e.x;
            V3 dl = v3(L.x, L.y, L.z);
            RayF sr;
            int skipInst = -1;
            if (origins)
            {
                // stored by the primary kernel with the arithmetic below
                const float4 so = origins[q];
                sr = make_ray(v3(so.x, so.y, so.z), dl, 0.0f, FLT_MAX);
                skipInst = __float_as_int(so.w);
            }
            else
            {
                RayF pr = primary_ray(cam, rays, pixelStart + uint64_t(i), i, width);
                float t = out[i].t;
                // ip = origin + t * direction (intersections.cl:85)
                V3 ip = vfma(pr.d, t, pr.o);
                sr = make_ray(vfma(dl, rayStartOffset, ip), dl, 0.0f, FLT_MAX);
                if (INST)
                    skipInst = out[i].occluder;  // the primary stage left the hit's instance there
            }
            HitF h{ -1, FLT_MAX, 0.0f, 0.0f, -1 };
            bool occ;
            if (INST)
                occ = traverse_instanced<true, COUNT>(sc, sr, h, cnt, err, e.y, skipInst);
            else if (SL)
                occ = traverse_stackless<true>(sc, sr, h, e.y);  // the same first occluder, no stack
            else
                occ = traverse<true, ORDER_REF, COUNT>(sc, sr, h, cnt, err, e.y);
            out[i].occluder = occ ? caller_index(sc, h.slot) + (INST ? __ldg(&sc.instances[h.inst].primBase) : 0) : -1;
            out[i].flags = 1 | 2 | (occ ? 4 : 0);
            done++;
        }
    }
    flush_counts(ctl, 1, done, cnt, err);
}

// Persistent grid of a ray kernel: resident blocks per SM (cached per
// device) x the launching handle's SMs.
template <typename K>
int persistent_blocks(K kernel, int numSMs, OccupancyCache& cache)
{
    return blocks_per_sm(kernel, kBlock, 0, cache) * numSMs;
}

template <bool ANY, int ORDER, bool COUNT, bool SL = false>
cudaError_t cast_t(const LaunchInfo& li, const DevScene& sc, const rc_ray* rays, int64_t n, rc_hit* hits,
                   DevControl* ctl)
{
    auto k = k_cast<ANY, ORDER, COUNT, SL>;
    static OccupancyCache occ;
    k<<<persistent_blocks(k, li.numSMs, occ), kBlock, 0, li.stream>>>(sc, rays, int(n), hits, ctl);
    return cudaGetLastError();
}

// Warp-wide traversal of the primary rays of uncounted RAY frames walked in
// pixel tiles: RC_TRACE_PACKETS = 2 (default) for camera frames and caller
// ray frames, 1 for camera frames only, 0 never (read once). On the 1080p
// heightfield the primary rays of an 8x4-pixel tile take 0.302 ms this way
// against 0.327 ms per lane, and the caller-ray frame through host memory
// gains 3 %. A caller frame whose neighbouring rays are not coherent would
// lose instead (mode 1). Shadow rays stay per lane: each stops at its first
// occluder, and the warp-wide walk of the union of their paths measured 1.8x
// slower (0.306 vs 0.172 ms).
int trace_packets()
{
    static const int mode = [] {
        const char* v = std::getenv("RC_TRACE_PACKETS");
        return v && v[0] >= '0' && v[0] <= '2' ? int(v[0] - '0') : 2;
    }();
    return mode;
}

// A whole image of at least one 8x4 tile (pixel ranges, and ray lists passed
// as one row, are walked in order).
bool whole_frame(uint64_t pixelStart, int64_t count, int64_t width)
{
    return RC_TRACE_TILES && pixelStart == 0 && width >= 8 && count / width >= 4 && (count / width) * width == count;
}


// Sign octant of the shadow rays' direction L for slab_oct (bit k: component
// k negative), or -1 where a component is zero, not finite or too small for
// its reciprocal to be finite (the general box test then applies).
int light_octant(float3 L)
{
    const float c[3] = { L.x, L.y, L.z };
    int oct = 0;
    for (int k = 0; k < 3; ++k)
    {
        if (!std::isfinite(c[k]) || !(std::fabs(c[k]) > 1e-30f))
            return -1;
        if (c[k] < 0.0f)
            oct |= 1 << k;
    }
    return oct;
}

#define RC_FUSED_ARGS li, sc, cam, rays, pixelStart, count, width, height, tilesX, castShadow, L, off, out, queue, ctl

// The one-kernel RAY frame, its shadow walk specialised to the light's
// octant SOCT (or general, -1).
template <int ORDER, bool PACKET, bool INST, bool SL, int SOCT>
cudaError_t launch_fused(const LaunchInfo& li, const DevScene& sc, const DevCamera& cam, const rc_ray* rays,
                         uint64_t pixelStart, int64_t count, int64_t width, int64_t height, int64_t tilesX,
                         int castShadow, float3 L, float off, rc_cast_pixel* out, int* queue, DevControl* ctl)
{
    auto kf = k_raycast_primary<ORDER, false, PACKET, INST, true, SL, SOCT>;
    static OccupancyCache occF;
    kf<<<persistent_blocks(kf, li.numSMs, occF), kBlock, 0, li.stream>>>(sc, cam, rays, pixelStart, count, width,
                                                                         height, tilesX, castShadow, out, queue, ctl,
                                                                         L, off, nullptr);
    return cudaGetLastError();
}

template <int ORDER, bool COUNT, bool PACKET, bool INST, bool SL = false, bool FUSED = false>
cudaError_t raycast_t(const LaunchInfo& li, const DevScene& sc, const DevCamera& cam, const rc_ray* rays,
                      uint64_t pixelStart, int64_t count, int64_t width, int castShadow, float3 L, float off,
                      rc_cast_pixel* out, int* queue, DevControl* ctl, cudaEvent_t between, float4* origins,
                      int& kernels)
{
    // Tile a whole frame (pixel range = the full image; camera rays or one
    // caller ray per pixel): only the order the warps take the pixels in.
    const int64_t height = width > 0 ? count / width : 0;
    const int64_t tilesX = whole_frame(pixelStart, count, width) ? (width + 7) / 8 : 0;
    if (FUSED && castShadow)
    {
        kernels = 1;
        if constexpr (!INST && !SL)
        {
            switch (light_octant(L))
            {
            case 0: return launch_fused<ORDER, PACKET, INST, SL, 0>(RC_FUSED_ARGS);
            case 1: return launch_fused<ORDER, PACKET, INST, SL, 1>(RC_FUSED_ARGS);
            case 2: return launch_fused<ORDER, PACKET, INST, SL, 2>(RC_FUSED_ARGS);
            case 3: return launch_fused<ORDER, PACKET, INST, SL, 3>(RC_FUSED_ARGS);
            case 4: return launch_fused<ORDER, PACKET, INST, SL, 4>(RC_FUSED_ARGS);
            case 5: return launch_fused<ORDER, PACKET, INST, SL, 5>(RC_FUSED_ARGS);
            case 6: return launch_fused<ORDER, PACKET, INST, SL, 6>(RC_FUSED_ARGS);
            case 7: return launch_fused<ORDER, PACKET, INST, SL, 7>(RC_FUSED_ARGS);
            default: break;
            }
        }
        return launch_fused<ORDER, PACKET, INST, SL, -1>(RC_FUSED_ARGS);
    }
    auto kp = k_raycast_primary<ORDER, COUNT, PACKET, INST>;
    auto ks = k_raycast_shadow<COUNT, INST, SL>;
    static OccupancyCache occP, occS;
    kp<<<persistent_blocks(kp, li.numSMs, occP), kBlock, 0, li.stream>>>(sc, cam, rays, pixelStart, count, width, height, tilesX, castShadow, out, queue,
                                     ctl, L, off, castShadow ? origins : nullptr);
    kernels = 1;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !castShadow)
        return e;
    if (between)
        e = cudaEventRecord(between, li.stream);
    if (e != cudaSuccess)
        return e;
    ks<<<persistent_blocks(ks, li.numSMs, occS), kBlock, 0, li.stream>>>(sc, cam, rays, pixelStart, width, L, off, out, queue, ctl, origins);
    kernels = 2;
    return cudaGetLastError();
}

// Whether uncounted RAY frames trace each shadow ray in the primary kernel
// (k_raycast_primary FUSED); RC_TRACE_FUSED=0 keeps the two kernels with the
// compacted shadow queue (read once).
bool fused_frames()
{
    static const bool on = [] {
        const char* v = std::getenv("RC_TRACE_FUSED");
        return !(v && v[0] == '0');
    }();
    return on;
}

// Uncounted frames: the fused or the two-kernel form.
template <int ORDER, bool PACKET, bool INST, bool SL = false>
cudaError_t raycast_u(const LaunchInfo& li, const DevScene& sc, const DevCamera& cam, const rc_ray* rays,
                      uint64_t pixelStart, int64_t count, int64_t width, int castShadow, float3 L, float off,
                      rc_cast_pixel* out, int* queue, DevControl* ctl, cudaEvent_t between, float4* origins,
                      int& kernels)
{
    return fused_frames() ? raycast_t<ORDER, false, PACKET, INST, SL, true>(li, sc, cam, rays, pixelStart, count,
                                                                             width, castShadow, L, off, out, queue,
                                                                             ctl, between, origins, kernels)
                          : raycast_t<ORDER, false, PACKET, INST, SL, false>(li, sc, cam, rays, pixelStart, count,
                                                                              width, castShadow, L, off, out, queue,
                                                                              ctl, between, origins, kernels);
}

}  // namespace

// Whether the reference-order queries of uncounted frames (the RAY frame's
// shadow rays, rc_cast in RC_ORDER_REFERENCE) take the stackless walk over
// the rope records (RC_STACKLESS=1; read once). The same hits.
bool stackless_walk()
{
    static const bool on = [] {
        const char* v = std::getenv("RC_STACKLESS");
        return v && v[0] == '1';
    }();
    return on;
}

cudaError_t launch_cast(const LaunchInfo& li, const DevScene& sc, const rc_ray* rays, int64_t n, int anyHit,
                        int order, rc_hit* hits, DevControl* ctl)
{
    if (n <= 0)
        return cudaSuccess;
    const bool sl = !li.counting && sc.numInstances == 0 && sc.ropes && stackless_walk();
    if (anyHit)
        return li.counting ? cast_t<true, ORDER_REF, true>(li, sc, rays, n, hits, ctl)
               : sl        ? cast_t<true, ORDER_REF, false, true>(li, sc, rays, n, hits, ctl)
                           : cast_t<true, ORDER_REF, false>(li, sc, rays, n, hits, ctl);
    if (order == ORDER_NEAREST)
        return li.counting ? cast_t<false, ORDER_NEAREST, true>(li, sc, rays, n, hits, ctl)
                           : cast_t<false, ORDER_NEAREST, false>(li, sc, rays, n, hits, ctl);
    return li.counting ? cast_t<false, ORDER_REF, true>(li, sc, rays, n, hits, ctl)
           : sl        ? cast_t<false, ORDER_REF, false, true>(li, sc, rays, n, hits, ctl)
                       : cast_t<false, ORDER_REF, false>(li, sc, rays, n, hits, ctl);
}

cudaError_t launch_raycast(const LaunchInfo& li, const DevScene& sc, const DevCamera& cam, const rc_ray* rays,
                           uint64_t pixelStart, int64_t count, int64_t width, int order, int castShadow,
                           float3 dirToLight, float rayStartOffset, rc_cast_pixel* out, int* shadowQueue,
                           DevControl* ctl, cudaEvent_t between, float4* shadowOrigins, int* kernels)
{
    int launched = 0;
    if (!kernels)
        kernels = &launched;
    *kernels = 0;
    if (count <= 0)
        return cudaSuccess;
#define RC_RAYCAST_ARGS li, sc, cam, rays, pixelStart, count, width, castShadow, dirToLight, rayStartOffset, out, \
                        shadowQueue, ctl, between, shadowOrigins, *kernels
    // two-level scenes: the top level nearest-first, like rc_cast's
    if (sc.numInstances > 0)
        return li.counting ? raycast_t<ORDER_NEAREST, true, false, true>(RC_RAYCAST_ARGS)
                           : raycast_u<ORDER_NEAREST, false, true>(RC_RAYCAST_ARGS);
    if (li.counting)
        return order == ORDER_NEAREST ? raycast_t<ORDER_NEAREST, true, false, false>(RC_RAYCAST_ARGS)
                                      : raycast_t<ORDER_REF, true, false, false>(RC_RAYCAST_ARGS);
    const int packets = trace_packets();
    const bool packet = whole_frame(pixelStart, count, width) && (packets == 2 || (packets == 1 && !rays));
    if (stackless_walk() && sc.ropes)
    {
        if (packet)
            return order == ORDER_NEAREST ? raycast_u<ORDER_NEAREST, true, false, true>(RC_RAYCAST_ARGS)
                                          : raycast_u<ORDER_REF, true, false, true>(RC_RAYCAST_ARGS);
        return order == ORDER_NEAREST ? raycast_u<ORDER_NEAREST, false, false, true>(RC_RAYCAST_ARGS)
                                      : raycast_u<ORDER_REF, false, false, true>(RC_RAYCAST_ARGS);
    }
    if (packet)
        return order == ORDER_NEAREST ? raycast_u<ORDER_NEAREST, true, false>(RC_RAYCAST_ARGS)
                                      : raycast_u<ORDER_REF, true, false>(RC_RAYCAST_ARGS);
    return order == ORDER_NEAREST ? raycast_u<ORDER_NEAREST, false, false>(RC_RAYCAST_ARGS)
                                  : raycast_u<ORDER_REF, false, false>(RC_RAYCAST_ARGS);
#undef RC_RAYCAST_ARGS
}

}  // namespace rcx
