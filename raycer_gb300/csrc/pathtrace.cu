// Wavefront path tracer (PathTracer, src/Raytracing/Tracers/PathTracer.cpp:13-75;
// pathtrace.cl:1-80): the kernels of one pass (see pathtrace.h for passes,
// chunks and the scene table).
//
// Slot s of a pass belongs to chunk c = chunkOf[s], pixel (s - slotBegin) / spp
// of the chunk and sample (s - slotBegin) % spp of that pixel, where
// spp = n*n camera samples (Tracer.cpp:115-144, CMJ + box filter) x
// pathSampleCount paths per camera sample (PathTracer.cpp:19). Path state
// lives in SoA arrays indexed by slot:
//   o, d       ray (float4 each); o.w = the triangle the ray leaves from
//              (skipped by its closest-hit query, see traverse.cuh)
//   thr        path throughput (rgb)
//   res        radiance result (rgb) + the camera sample's filter weight (w)
//   hit        closest hit of the last extend (slot, t, u, v)
// Stages (one launch each, per segment):
//   generate   camera rays for every slot; queue 0 = all slots
//   extend     closest hit for every queued slot              (persistent)
//   shade      miss -> 0; emissive -> res = thr * emittance; the scene's last
//              segment -> 0; else optional Russian roulette, cosine bounce,
//              thr *= 2*rho*|w.n| (PathTracer.cpp:58-72), and the slot is
//              appended to the next queue (warp-ballot compaction) (persistent)
//   accumulate per pixel, in sample order: c_j = (sum_k L_jk) / P,
//              film.rgb += w_j * c_j, film.w += w_j (Film::addSample,
//              Film.cpp:54-59). One thread owns one pixel: deterministic.
// Uncounted nearest-first passes over the 4-wide BVH run extend and shade of
// a segment as one kernel (k_extend_shade); the hit record is then never
// written.
// Queue counts live on the device, so a pass is a fixed launch sequence the
// host never waits on (and can be captured in a CUDA graph).

#include <cfloat>
#include <cstdlib>

#include "filters.cuh"
#include "monitor.cuh"
#include "pathtrace.h"
#include "sampling.cuh"
#include "traverse.cuh"

namespace rcx
{
namespace
{

#ifndef RC_TRACE_MIN_BLOCKS
#define RC_TRACE_MIN_BLOCKS 10
#endif
// Resident 128-thread blocks per SM the extend kernel is compiled for (its
// register budget: 65,536 / (128 x this)).
#ifndef RC_EXTEND_MIN_BLOCKS
#define RC_EXTEND_MIN_BLOCKS 10
#endif
// The same for the two-level extend kernel.
#ifndef RC_EXTEND_INST_MIN_BLOCKS
#define RC_EXTEND_INST_MIN_BLOCKS 8
#endif
// The same for the 4-wide traversal (four boxes per node in registers).
#ifndef RC_EXTEND_WIDE_MIN_BLOCKS
#define RC_EXTEND_WIDE_MIN_BLOCKS 9
#endif
// The same for the extend + shade kernel of radiance-cache passes, whose
// shading also writes training vertices and lookups: at 9 blocks it spilled
// 96 bytes, at 8 (64 registers) 52, and cache frames ran 1 % faster.
#ifndef RC_EXTEND_SHADE_NRC_MIN_BLOCKS
#define RC_EXTEND_SHADE_NRC_MIN_BLOCKS 8
#endif

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

__device__ __forceinline__ unsigned warp_fetch(unsigned* head, unsigned amount)
{
    unsigned base = 0;
    if (lane_id() == 0)
        base = atomicAdd(head, amount);
    return __shfl_sync(0xffffffffu, base, 0);
}

// A monitored render whose earlier kernel stopped it (cancel or time
// budget): the pass's remaining kernels do nothing, so the film keeps whole
// passes only.
__device__ __forceinline__ bool pass_stopped(const PassParams& p)
{
    return monitored(p.monitor, p.budgetNs) && render_stopped(p.ctl);
}

// Largest chunk whose first slot (pixel) is <= s.
__device__ __forceinline__ int chunk_of_slot(const PassParams& p, uint32_t s)
{
    int lo = 0, hi = p.numChunks - 1;
    while (lo < hi)
    {
        int mid = (lo + hi + 1) >> 1;
        if (p.chunks[mid].slotBegin <= s)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ int chunk_of_pixel(const PassParams& p, uint32_t pix)
{
    int lo = 0, hi = p.numChunks - 1;
    while (lo < hi)
    {
        int mid = (lo + hi + 1) >> 1;
        if (p.chunks[mid].pixelPassBegin <= pix)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

struct SlotInfo
{
    uint64_t pixelGlobal;
    uint32_t sample;  // j * P + k
    uint32_t j;
};

__device__ __forceinline__ SlotInfo slot_info(const PathChunk& ch, const PathScene& sc, uint32_t s)
{
    SlotInfo si;
    uint32_t rel = s - ch.slotBegin;
    uint32_t pix = rel / uint32_t(sc.spp);
    si.sample = rel - pix * uint32_t(sc.spp);
    si.j = si.sample / uint32_t(sc.P);
    si.pixelGlobal = sc.pixelStart + ch.pixelLocalBegin + pix;
    return si;
}

__global__ void __launch_bounds__(256) k_generate(PassParams p)
{
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    const bool stopped = pass_stopped(p);
    if (s == 0)
    {
        // a stopped render's pass: an empty queue, no lookups or samples
        p.counts[0] = stopped ? 0u : uint32_t(p.nslots);
        if (p.nrc.counters)
        {
            p.nrc.counters[0] = 0;
            p.nrc.counters[1] = 0;
        }
    }
    if (stopped || s >= uint32_t(p.nslots))
        return;
    // Training-path records start inactive; the path's end marks them.
    if (p.nrc.term && s % uint32_t(p.nrc.trainStride) == 0)
        p.nrc.term[s / uint32_t(p.nrc.trainStride)] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const int c = chunk_of_slot(p, s);
    p.chunkOf[s] = c;
    const PathChunk ch = p.chunks[c];
    const PathScene& sc = p.scenes[ch.scene];
    SlotInfo si = slot_info(ch, sc, s);
    float px = float(si.pixelGlobal % uint64_t(sc.width));
    float py = float(si.pixelGlobal / uint64_t(sc.width));
    float w = 1.0f;
    if (sc.n > 1)
    {
        uint32_t gx = si.j % uint32_t(sc.n);
        uint32_t gy = si.j / uint32_t(sc.n);
        uint32_t jkey = stream_key(sc.seed, sc.frame, si.pixelGlobal, 0x80000000u | si.j);
        float jx = stream_float(jkey, kCounterJitter + 0);
        float jy = stream_float(jkey, kCounterJitter + 1);
        float sx, sy;
        if (sc.samplerType == RC_SAMPLER_CMJ)
        {
            // CMJSampler::getSample2D (CMJSampler.cpp:61-76), permutation per pixel.
            uint32_t pkey = stream_key(sc.seed, sc.frame, si.pixelGlobal, 0xffffffffu);
            uint64_t perm = (uint64_t(stream_u32(pkey, 1)) << 32) | stream_u32(pkey, 2);
            uint64_t n = uint64_t(sc.n);
            uint64_t sxp = cmj_permute(gx, n, perm * 0x68bc21ebull);
            uint64_t syp = cmj_permute(gy, n, perm * 0x02e5be93ull);
            float fn = float(sc.n);
            sx = __fdiv_rn(__fadd_rn(float(gx), __fdiv_rn(__fadd_rn(float(syp), jx), fn)), fn);
            sy = __fdiv_rn(__fadd_rn(float(gy), __fdiv_rn(__fadd_rn(float(sxp), jy), fn)), fn);
        }
        else if (sc.samplerType == RC_SAMPLER_RANDOM)
        {
            sx = jx;
            sy = jy;
        }
        else
        {
            sx = 0.5f;
            sy = 0.5f;
        }
        // sampleOffset = (sample - 0.5) * 2 * radius (Tracer.cpp:138)
        float ox = __fmul_rn(__fmul_rn(__fsub_rn(sx, 0.5f), 2.0f), sc.filter.rx);
        float oy = __fmul_rn(__fmul_rn(__fsub_rn(sy, 0.5f), 2.0f), sc.filter.ry);
        w = filter_weight(sc.filter, ox, oy);
        px = __fadd_rn(px, ox);
        py = __fadd_rn(py, oy);
    }
    V3 d = camera_dir(sc.cam, px, py);
    p.o[s] = make_float4(sc.cam.pos[0], sc.cam.pos[1], sc.cam.pos[2], __int_as_float(-1));
    p.d[s] = make_float4(d.x, d.y, d.z, __int_as_float(-1));  // w: instance the ray leaves from
    p.thr[s] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
    p.res[s] = make_float4(0.0f, 0.0f, 0.0f, w);
    p.qa[s] = int(s);
}

__device__ __forceinline__ DevScene scene_of_slot(const PassParams& p, int s)
{
    // one-scene renders: no dependent loads through the slot's chunk
    return p.singleScene ? p.scene0 : p.scenes[p.chunks[p.chunkOf[s]].scene].sc;
}

__device__ __forceinline__ void flush_extend_counts(const PassParams& p, unsigned long long done, const TravCount& cnt,
                                                    int err)
{
    unsigned long long n = cnt.nodes, t = cnt.tris;
    for (int o = 16; o > 0; o >>= 1)
    {
        done += __shfl_down_sync(0xffffffffu, done, o);
        n += __shfl_down_sync(0xffffffffu, n, o);
        t += __shfl_down_sync(0xffffffffu, t, o);
    }
    if (lane_id() == 0)
    {
        atomicAdd(&p.ctl->stats[0], done);
        atomicAdd(&p.ctl->stats[1], n);
        atomicAdd(&p.ctl->stats[2], t);
    }
    if (err)
        atomicOr(&p.ctl->error, 1);
}

template <int ORDER, bool COUNT, int BLOCK>
__global__ void __launch_bounds__(BLOCK, ((ORDER == ORDER_WIDE ? RC_EXTEND_WIDE_MIN_BLOCKS : RC_EXTEND_MIN_BLOCKS) * 128) /
                                             BLOCK) k_extend(PassParams p, int segment)
{
    const unsigned total = *reinterpret_cast<volatile unsigned*>(&p.counts[segment * 4 + 0]);
    const int* __restrict__ queue = (segment & 1) ? p.qb : p.qa;
    TravCount cnt{ 0, 0 };
    int err = 0;
    unsigned long long done = 0;
    if (pass_stopped(p))
        return;
    if (is_watch_warp(p.monitor, p.budgetNs))
    {
        watch_queue(p.monitor, p.budgetNs, p.ctl, &p.counts[segment * 4 + 1], total, kPublishProgress, 0);
        return;
    }
    while (true)
    {
        unsigned base = warp_fetch(&p.counts[segment * 4 + 1], 32u);
        if (base >= total)
            break;
        unsigned q = base + lane_id();
        if (q < total)
        {
            int s = queue[q];
            const DevScene sc = scene_of_slot(p, s);
            float4 o = p.o[s];
            float4 d = p.d[s];
            RayF ray = make_ray(v3(o.x, o.y, o.z), v3(d.x, d.y, d.z), 0.0f, FLT_MAX);
            HitF h{ -1, FLT_MAX, 0.0f, 0.0f, -1 };
            bool found = ORDER == ORDER_WIDE ? traverse_wide(sc, ray, h, err, __float_as_int(o.w))
                                             : traverse<false, ORDER, COUNT>(sc, ray, h, cnt, err, __float_as_int(o.w));
            p.hit[s] = make_int4(found ? h.slot : -1, __float_as_int(h.t), __float_as_int(h.u), __float_as_int(h.v));
            done++;
        }
    }
    flush_extend_counts(p, done, cnt, err);
}

// Extend through the 4-wide BVH with lane refill (Aila & Laine 2009's
// dynamic fetch): bounce rays are incoherent and their walks differ in
// length, so a warp that takes 32 rays and walks them to the end spends most
// of its issue slots on a few long walks (about 7.6 of 32 lanes active per
// instruction). Here a lane whose ray is done takes a new one: whenever at
// least kRefillLanes lanes are idle the warp takes that many queue entries
// with one atomic and hands them to its idle lanes, which start their walks
// while the others continue theirs (wide_step keeps each walk's position
// between steps). Each ray's walk, hence its hit, is traverse_wide's.
#ifndef RC_EXTEND_REFILL_LANES
#define RC_EXTEND_REFILL_LANES 8
#endif
#ifndef RC_EXTEND_REFILL_MIN_BLOCKS
#define RC_EXTEND_REFILL_MIN_BLOCKS 8
#endif

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK, (RC_EXTEND_REFILL_MIN_BLOCKS * 128) / BLOCK)
    k_extend_refill(PassParams p, int segment)
{
    const unsigned total = *reinterpret_cast<volatile unsigned*>(&p.counts[segment * 4 + 0]);
    const int* __restrict__ queue = (segment & 1) ? p.qb : p.qa;
    unsigned* head = &p.counts[segment * 4 + 1];
    if (pass_stopped(p))
        return;
    int err = 0;
    unsigned long long done = 0;
    int stack[kMaxStack];
    float sdist[kMaxStack];
    int s = -1;  // this lane's path slot, -1 = idle
    RayF ray;
    HitF h{ -1, FLT_MAX, 0.0f, 0.0f, -1 };
    WideWalk w{ 0, 0, false };
    int skip = -1;
    const DevNode4* wide = nullptr;
    const DevTri* tris = nullptr;
    bool drained = false;  // warp-uniform
    const unsigned below = (1u << lane_id()) - 1u;
    if (is_watch_warp(p.monitor, p.budgetNs))
    {
        watch_queue(p.monitor, p.budgetNs, p.ctl, head, total, kPublishProgress, 0);
        return;
    }
    while (true)
    {
        const unsigned idle = __ballot_sync(0xffffffffu, s < 0);
        if (!drained && __popc(idle) >= RC_EXTEND_REFILL_LANES)
        {
            const unsigned n = unsigned(__popc(idle));
            unsigned base = 0;
            if (lane_id() == 0)
                base = atomicAdd(head, n);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= total)
                drained = true;
            else if (s < 0)
            {
                const unsigned q = base + unsigned(__popc(idle & below));
                if (q < total)
                {
                    s = queue[q];
                    const DevScene sc = scene_of_slot(p, s);
                    const float4 o = p.o[s];
                    const float4 d = p.d[s];
                    ray = make_ray(v3(o.x, o.y, o.z), v3(d.x, d.y, d.z), 0.0f, FLT_MAX);
                    h = HitF{ -1, FLT_MAX, 0.0f, 0.0f, -1 };
                    w = WideWalk{ sc.wideRoot, 0, false };
                    skip = __float_as_int(o.w);
                    wide = sc.wide;
                    tris = sc.tris;
                }
            }
        }
        if (__ballot_sync(0xffffffffu, s >= 0) == 0u)
        {
            if (drained)
                break;
            continue;
        }
        if (s >= 0 && wide_step(wide, tris, ray, h, w, stack, sdist, skip, err))
        {
            p.hit[s] = make_int4(w.found ? h.slot : -1, __float_as_int(h.t), __float_as_int(h.u), __float_as_int(h.v));
            done++;
            s = -1;
        }
    }
    flush_extend_counts(p, done, TravCount{ 0, 0 }, err);
}

// Extend for passes with two-level scenes: 32 queue entries per warp fetch,
// each ray traced in one go.
template <bool COUNT>
__global__ void __launch_bounds__(128, RC_EXTEND_INST_MIN_BLOCKS) k_extend_instanced(PassParams p, int segment)
{
    const unsigned total = *reinterpret_cast<volatile unsigned*>(&p.counts[segment * 4 + 0]);
    const int* __restrict__ queue = (segment & 1) ? p.qb : p.qa;
    TravCount cnt{ 0, 0 };
    int err = 0;
    unsigned long long done = 0;
    if (pass_stopped(p))
        return;
    if (is_watch_warp(p.monitor, p.budgetNs))
    {
        watch_queue(p.monitor, p.budgetNs, p.ctl, &p.counts[segment * 4 + 1], total, kPublishProgress, 0);
        return;
    }
    while (true)
    {
        unsigned base = warp_fetch(&p.counts[segment * 4 + 1], 32u);
        if (base >= total)
            break;
        unsigned q = base + lane_id();
        if (q < total)
        {
            int s = queue[q];
            const DevScene sc = scene_of_slot(p, s);
            float4 o = p.o[s];
            float4 d = p.d[s];
            RayF ray = make_ray(v3(o.x, o.y, o.z), v3(d.x, d.y, d.z), 0.0f, FLT_MAX);
            HitF h{ -1, FLT_MAX, 0.0f, 0.0f, -1 };
            bool found = traverse_scene<false, ORDER_NEAREST, COUNT>(sc, ray, h, cnt, err, __float_as_int(o.w),
                                                                     __float_as_int(d.w));
            // w: v, or the instance of a two-level scene's hit (shading uses neither u nor v)
            p.hit[s] = make_int4(found ? h.slot : -1, __float_as_int(h.t), __float_as_int(h.u),
                                 sc.numInstances > 0 ? h.inst : __float_as_int(h.v));
            done++;
        }
    }
    flush_extend_counts(p, done, cnt, err);
}

// Shading frame of a hit: the triangle's normal, tangent and bitangent
// (Triangle::initialize), the normal inverted for invertNormal materials;
// in an instance, each transformed by A^T (the inverse transpose of the
// instance transform) and normalised, as Instance transforms its ONB
// (Instance.cpp:98-99, ONB.cpp:21-30).
struct ShadeFrame
{
    V3 n, t, b;
};

__device__ __forceinline__ V3 inst_normal(const DevInstance& in, V3 v)
{
    V3 w = v3(__fmaf_rn(in.r0.x, v.x, __fmaf_rn(in.r1.x, v.y, __fmul_rn(in.r2.x, v.z))),
              __fmaf_rn(in.r0.y, v.x, __fmaf_rn(in.r1.y, v.y, __fmul_rn(in.r2.y, v.z))),
              __fmaf_rn(in.r0.z, v.x, __fmaf_rn(in.r1.z, v.y, __fmul_rn(in.r2.z, v.z))));
    const float len = __fsqrt_rn(vdot(w, w));
    return v3(__fdiv_rn(w.x, len), __fdiv_rn(w.y, len), __fdiv_rn(w.z, len));
}

__device__ __forceinline__ ShadeFrame shade_frame(const DevScene& sc, int slot, const DevInstance* in, uint32_t mflags)
{
    const float4* sp = reinterpret_cast<const float4*>(sc.shade + slot);
    const float4 sn = __ldg(sp + 0), st = __ldg(sp + 1), sb = __ldg(sp + 2);
    ShadeFrame f{ v3(sn.x, sn.y, sn.z), v3(st.x, st.y, st.z), v3(sb.x, sb.y, sb.z) };
    if (in && !in->identity)
    {
        f.n = inst_normal(*in, f.n);
        f.t = inst_normal(*in, f.t);
        f.b = inst_normal(*in, f.b);
    }
    if (mflags & kMatInvertNormal)
        f.n = v3(-f.n.x, -f.n.y, -f.n.z);
    return f;
}

// Specular bounce off a dielectric (GPU extension: the reference's path
// tracer is diffuse only). Fresnel reflectance by Schlick's approximation
// as the reference's Whitted tracer computes it (Raytracer.cpp:126-143);
// reflect with that probability (or on total internal reflection), else
// refract (Raytracer.cpp:230-246 with the normal facing the ray). The
// throughput is unchanged: the choice probability equals its weight.
__device__ __forceinline__ V3 dielectric_bounce(V3 d, V3 n, float ior, float xi)
{
    const float c = vdot(d, n);
    const bool outside = c < 0.0f;
    const float n1 = outside ? 1.0f : ior;
    const float n2 = outside ? ior : 1.0f;
    const V3 N = outside ? n : v3(-n.x, -n.y, -n.z);
    const float ci = fabsf(c);
    float r0 = __fdiv_rn(__fsub_rn(n2, n1), __fadd_rn(n2, n1));
    r0 = __fmul_rn(r0, r0);
    const float m = __fsub_rn(1.0f, ci);
    const float m2 = __fmul_rn(m, m);
    const float m5 = __fmul_rn(__fmul_rn(m2, m2), m);
    const float R = __fadd_rn(r0, __fmul_rn(__fsub_rn(1.0f, r0), m5));
    const float eta = __fdiv_rn(n1, n2);
    const float k = __fsub_rn(1.0f, __fmul_rn(__fmul_rn(eta, eta), __fsub_rn(1.0f, __fmul_rn(ci, ci))));
    if (k <= 0.0f || xi < R)
        return vfma(N, __fmul_rn(2.0f, ci), d);  // d - 2 (d.N) N, d.N = -ci
    const V3 r = vfma(N, __fsub_rn(__fmul_rn(eta, ci), __fsqrt_rn(k)), vscale(d, eta));
    const float len = __fsqrt_rn(vdot(r, r));
    return v3(__fdiv_rn(r.x, len), __fdiv_rn(r.y, len), __fdiv_rn(r.z, len));
}

// Training-path choice of slot s: one random slot per run of trainStride.
__device__ __forceinline__ uint32_t nrc_pick(const NrcPass& n, uint32_t g)
{
    return mix32(n.trainKey ^ mix32(g + 0x9e3779b9u)) % uint32_t(n.trainStride);
}

__device__ __forceinline__ bool nrc_training(const NrcPass& n, uint32_t s)
{
    if (n.trainStride <= 0)
        return false;
    uint32_t g = s / uint32_t(n.trainStride);
    return s - g * uint32_t(n.trainStride) == nrc_pick(n, g);
}

__device__ __forceinline__ NrcRecord nrc_record(V3 x, float4 d, V3 nrm, float4 rho, float r, float g, float b,
                                                float tag)
{
    NrcRecord rec;
    rec.a = make_float4(x.x, x.y, x.z, -d.x);
    rec.b = make_float4(-d.y, -d.z, nrm.x, nrm.y);
    rec.c = make_float4(nrm.z, rho.x, rho.y, rho.z);
    rec.d = make_float4(r, g, b, tag);
    return rec;
}

__device__ __forceinline__ void nrc_end(const NrcPass& n, uint32_t g, float r, float gg, float b, uint32_t flags)
{
    n.term[g] = make_float4(r, gg, b, __uint_as_float(flags | kNrcTermActive));
}

// The shade stage for one queued slot whose extend found hit h (slot, t as
// bits, u, v; x < 0: a miss): a miss sees the sky (or black), an emitter
// ends the path with thr * emittance, the scene's last segment ends it, and
// otherwise optional Russian roulette, the cosine bounce and
// thr *= 2 * rho * |w.n| (PathTracer.cpp:58-72). With the radiance cache,
// training paths record every vertex (query + bounce factor) and their
// terminal radiance, and other paths end at the hit of segment termSegment
// with a cache lookup (res gets thr * cache after the last segment).
// Returns whether the path goes on (the slot joins the next segment's
// queue); a cache lookup sets `lookup` and `lrec`. With OD the caller passes
// the slot's ray (o, d) it already holds, else they are read from the path
// state.
template <bool NRC, bool OD>
__device__ __forceinline__ bool shade_slot(const PassParams& p, int segment, int s, int4 h, float4 o, float4 d,
                                           bool& lookup, NrcRecord& lrec)
{
    bool cont = false;
    // a one-scene pass has one chunk: no dependent load of the slot's chunk
    const PathChunk& ch = p.chunks[p.singleScene && p.numChunks == 1 ? 0 : p.chunkOf[s]];
    const PathScene& scn = p.scenes[ch.scene];
    const bool train = NRC && nrc_training(p.nrc, uint32_t(s));
    const uint32_t g = NRC ? uint32_t(s) / uint32_t(max(p.nrc.trainStride, 1)) : 0u;
    if (h.x < 0)
    {
        if (scn.skyOn)
        {
            // GPU extension: misses see a constant sky radiance.
            float4 thr = p.thr[s];
            float4 r = p.res[s];
            r.x = __fmul_rn(thr.x, scn.sky[0]);
            r.y = __fmul_rn(thr.y, scn.sky[1]);
            r.z = __fmul_rn(thr.z, scn.sky[2]);
            p.res[s] = r;
        }
        if (train)
        {
            const float on = scn.skyOn ? 1.0f : 0.0f;
            nrc_end(p.nrc, g, on * scn.sky[0], on * scn.sky[1], on * scn.sky[2], uint32_t(segment));
        }
    }
    else
    {
        const DevScene sc = scn.sc;
        const float4* tp = reinterpret_cast<const float4*>(sc.tris + h.x);
        float4 tc = __ldg(tp + 2);
        uint32_t mi = __float_as_uint(tc.y) & kMetaMaterialMask;
        const int inst = sc.numInstances > 0 ? h.w : -1;
        DevInstance in{};
        if (inst >= 0)
        {
            in = load_instance(sc.instances, inst);
            if (in.material >= 0)
                mi = uint32_t(in.material);  // Instance::changePrimitive (Instance.cpp:93)
        }
        float4 md = __ldg(&sc.mats[mi].diffuse);
        float4 me = __ldg(&sc.mats[mi].emittance);
        uint32_t mflags = __float_as_uint(me.w);
        const bool dielectric = (mflags & kMatDielectric) != 0;
        float4 thr = p.thr[s];
        if (mflags & kMatEmissive)
        {
            // sampleColor *= emittance (pathtrace.cl:44-51)
            float4 r = p.res[s];
            r.x = __fmul_rn(thr.x, me.x);
            r.y = __fmul_rn(thr.y, me.y);
            r.z = __fmul_rn(thr.z, me.z);
            p.res[s] = r;
            if (train)
                nrc_end(p.nrc, g, me.x, me.y, me.z, uint32_t(segment));
        }
        else if (NRC && !train && !dielectric && segment >= p.nrc.termSegment)
        {
            const ShadeFrame fr = shade_frame(sc, h.x, inst >= 0 ? &in : nullptr, mflags);
            o = OD ? o : p.o[s];
            d = OD ? d : p.d[s];
            V3 ip = vfma(v3(d.x, d.y, d.z), __int_as_float(h.y), v3(o.x, o.y, o.z));
            lrec = nrc_record(ip, d, fr.n, md, 0.0f, 0.0f, 0.0f, __int_as_float(s));
            lookup = true;
        }
        else if (segment + 1 < scn.maxPathLength)
        {
            SlotInfo si = slot_info(ch, scn, uint32_t(s));
            uint32_t key = stream_key(scn.seed, scn.frame, si.pixelGlobal, si.sample);
            bool alive = true;
            float qs = 1.0f;
            if (scn.rrDepth > 0 && segment + 1 >= scn.rrDepth)
            {
                float m = fmaxf(thr.x, fmaxf(thr.y, thr.z));
                qs = fminf(m, 1.0f);
                float xi = stream_float(key, kCounterRoulette + uint32_t(segment));
                if (!(xi < qs))
                    alive = false;
                else
                {
                    thr.x = __fdiv_rn(thr.x, qs);
                    thr.y = __fdiv_rn(thr.y, qs);
                    thr.z = __fdiv_rn(thr.z, qs);
                }
            }
            const ShadeFrame frm = shade_frame(sc, h.x, inst >= 0 ? &in : nullptr, mflags);
            const V3 nrm = frm.n;
            o = OD ? o : p.o[s];
            d = OD ? d : p.d[s];
            float t = __int_as_float(h.y);
            V3 ip = vfma(v3(d.x, d.y, d.z), t, v3(o.x, o.y, o.z));
            if (alive)
            {
                float xr = stream_float(key, kCounterBounce + 2u * uint32_t(segment));
                float yr = stream_float(key, kCounterBounce + 2u * uint32_t(segment) + 1u);
                V3 dir;
                float fr, fg, fb;
                if (dielectric)
                {
                    dir = dielectric_bounce(v3(d.x, d.y, d.z), nrm, md.w, xr);
                    fr = fg = fb = 1.0f;
                }
                else
                {
                    dir = hemisphere_cosine(frm.t, frm.b, nrm, xr, yr);
                    float alpha = fabsf(vdot(dir, nrm));
                    // brdf = 2 * reflectance * alpha (PathTracer.cpp:70-71)
                    fr = __fmul_rn(__fmul_rn(2.0f, md.x), alpha);
                    fg = __fmul_rn(__fmul_rn(2.0f, md.y), alpha);
                    fb = __fmul_rn(__fmul_rn(2.0f, md.z), alpha);
                    thr.x = __fmul_rn(thr.x, fr);
                    thr.y = __fmul_rn(thr.y, fg);
                    thr.z = __fmul_rn(thr.z, fb);
                }
                V3 no = vfma(dir, scn.rayStartOffset, ip);
                p.o[s] = make_float4(no.x, no.y, no.z, __int_as_float(h.x));
                p.d[s] = make_float4(dir.x, dir.y, dir.z, __int_as_float(inst));
                p.thr[s] = thr;
                cont = true;
                if (train)
                {
                    // specular vertices pass radiance on but are not training samples
                    NrcRecord rec = nrc_record(ip, d, nrm, md, fr / qs, fg / qs, fb / qs, 0.0f);
                    if (dielectric)
                        rec.c.y = -1.0f;
                    p.nrc.vtx[size_t(segment) * size_t(p.nrc.groups) + g] = rec;
                }
            }
            else if (train)
            {
                NrcRecord rec = nrc_record(ip, d, nrm, md, 0.0f, 0.0f, 0.0f, 0.0f);
                if (dielectric)
                    rec.c.y = -1.0f;
                p.nrc.vtx[size_t(segment) * size_t(p.nrc.groups) + g] = rec;
                nrc_end(p.nrc, g, 0.0f, 0.0f, 0.0f, uint32_t(segment + 1));
            }
        }
        else if (train)
        {
            // The depth limit cuts the path: its radiance from here on is 0.
            const ShadeFrame fr = shade_frame(sc, h.x, inst >= 0 ? &in : nullptr, mflags);
            o = OD ? o : p.o[s];
            d = OD ? d : p.d[s];
            V3 ip = vfma(v3(d.x, d.y, d.z), __int_as_float(h.y), v3(o.x, o.y, o.z));
            NrcRecord rec = nrc_record(ip, d, fr.n, md, 0.0f, 0.0f, 0.0f, 0.0f);
            if (dielectric)
                rec.c.y = -1.0f;
            p.nrc.vtx[size_t(segment) * size_t(p.nrc.groups) + g] = rec;
            nrc_end(p.nrc, g, 0.0f, 0.0f, 0.0f, uint32_t(segment + 1) | kNrcTermTruncated);
        }
    }
    return cont;
}

// Appends the cache lookups of the warp's slots to the lookup queue (one
// atomic per warp).
__device__ __forceinline__ void enqueue_lookup(bool lookup, const NrcRecord& lrec, const PassParams& p)
{
    unsigned lmask = __ballot_sync(0xffffffffu, lookup);
    if (lmask)
    {
        unsigned lbase = 0;
        if (lane_id() == 0)
            lbase = atomicAdd(&p.nrc.counters[0], unsigned(__popc(lmask)));
        lbase = __shfl_sync(0xffffffffu, lbase, 0);
        if (lookup)
            p.nrc.query[lbase + __popc(lmask & ((1u << lane_id()) - 1u))] = lrec;
    }
}

// Appends the slots whose paths go on to the next segment's queue: one
// atomic per warp (warp-ballot compaction).
__device__ __forceinline__ void enqueue_continuing(bool cont, int s, unsigned* outCount, int* __restrict__ qout)
{
    unsigned mask = __ballot_sync(0xffffffffu, cont);
    if (mask)
    {
        unsigned qbase = 0;
        if (lane_id() == 0)
            qbase = atomicAdd(outCount, unsigned(__popc(mask)));
        qbase = __shfl_sync(0xffffffffu, qbase, 0);
        if (cont)
            qout[qbase + __popc(mask & ((1u << lane_id()) - 1u))] = s;
    }
}

// The shade stage as its own kernel (passes that keep extend and shade
// apart): shade_slot for each queued slot, from the extend's hit records.
template <int BLOCK, bool NRC>
__global__ void __launch_bounds__(BLOCK) k_shade(PassParams p, int segment)
{
    const unsigned total = *reinterpret_cast<volatile unsigned*>(&p.counts[segment * 4 + 0]);
    const int* __restrict__ qin = (segment & 1) ? p.qb : p.qa;
    int* __restrict__ qout = (segment & 1) ? p.qa : p.qb;
    unsigned* outCount = &p.counts[(segment + 1) * 4 + 0];
    if (pass_stopped(p))
        return;
    while (true)
    {
        unsigned base = warp_fetch(&p.counts[segment * 4 + 2], 32u);
        if (base >= total)
            break;
        unsigned q = base + lane_id();
        bool cont = false;
        bool lookup = false;
        int s = -1;
        NrcRecord lrec;
        if (q < total)
        {
            s = qin[q];
            cont = shade_slot<NRC, false>(p, segment, s, p.hit[s], make_float4(0.0f, 0.0f, 0.0f, 0.0f),
                                          make_float4(0.0f, 0.0f, 0.0f, 0.0f), lookup, lrec);
        }
        enqueue_continuing(cont, s, outCount, qout);
        if (NRC)
            enqueue_lookup(lookup, lrec, p);
    }
}

// Extend and shade in one kernel (uncounted nearest-first passes over the
// 4-wide BVH of a single-level scene, plain or with the radiance cache):
// each lane walks its slot's ray as k_extend does, then shades the slot at
// once with the ray still in registers (shade_slot), and the warp appends
// the slots that go on to the next queue (and the cache lookups to the
// lookup queue). The hit record never goes through memory and a segment is
// one launch instead of two; the arithmetic, and so the film, is that of the
// two kernels. (Two-level scenes keep the two kernels: the fused form of
// their walk spilled and measured no faster.)
template <int BLOCK, bool NRC>
__global__ void __launch_bounds__(BLOCK,
                                  ((NRC ? RC_EXTEND_SHADE_NRC_MIN_BLOCKS : RC_EXTEND_WIDE_MIN_BLOCKS) * 128) / BLOCK)
    k_extend_shade(PassParams p, int segment)
{
    const unsigned total = *reinterpret_cast<volatile unsigned*>(&p.counts[segment * 4 + 0]);
    const int* __restrict__ queue = (segment & 1) ? p.qb : p.qa;
    int* __restrict__ qout = (segment & 1) ? p.qa : p.qb;
    unsigned* outCount = &p.counts[(segment + 1) * 4 + 0];
    int err = 0;
    unsigned long long done = 0;
    if (pass_stopped(p))
        return;
    if (is_watch_warp(p.monitor, p.budgetNs))
    {
        watch_queue(p.monitor, p.budgetNs, p.ctl, &p.counts[segment * 4 + 1], total, kPublishProgress, 0);
        return;
    }
    while (true)
    {
        unsigned base = warp_fetch(&p.counts[segment * 4 + 1], 32u);
        if (base >= total)
            break;
        unsigned q = base + lane_id();
        bool cont = false;
        bool lookup = false;
        int s = -1;
        NrcRecord lrec;
        if (q < total)
        {
            s = queue[q];
            const DevScene sc = scene_of_slot(p, s);
            const float4 o = p.o[s];
            const float4 d = p.d[s];
            RayF ray = make_ray(v3(o.x, o.y, o.z), v3(d.x, d.y, d.z), 0.0f, FLT_MAX);
            HitF h{ -1, FLT_MAX, 0.0f, 0.0f, -1 };
            const bool found = traverse_wide(sc, ray, h, err, __float_as_int(o.w));
            done++;
            cont = shade_slot<NRC, true>(p, segment, s, make_int4(found ? h.slot : -1, __float_as_int(h.t), 0, -1),
                                         o, d, lookup, lrec);
        }
        enqueue_continuing(cont, s, outCount, qout);
        if (NRC)
            enqueue_lookup(lookup, lrec, p);
    }
    flush_extend_counts(p, done, TravCount{ 0, 0 }, err);
}

__global__ void __launch_bounds__(256) k_accumulate(PassParams p)
{
    int pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= p.npixels || pass_stopped(p))
        return;
    if (p.monitor && threadIdx.x == 0)
        atomicAdd(&p.ctl->progress, static_cast<unsigned long long>(min(256, p.npixels - pix)));
    const PathChunk ch = p.chunks[chunk_of_pixel(p, uint32_t(pix))];
    const PathScene& sc = p.scenes[ch.scene];
    const uint32_t inChunk = uint32_t(pix) - ch.pixelPassBegin;
    const int nn = sc.n * sc.n;
    const float fP = float(sc.P);
    float4* fp = sc.film + ch.pixelLocalBegin + inChunk;
    float4 f = *fp;
    size_t base = size_t(ch.slotBegin) + size_t(inChunk) * size_t(sc.spp);
    for (int j = 0; j < nn; ++j)
    {
        float sr = 0.0f, sg = 0.0f, sb = 0.0f, w = 0.0f;
        for (int k = 0; k < sc.P; ++k)
        {
            float4 r = p.res[base + size_t(j) * size_t(sc.P) + size_t(k)];
            sr = __fadd_rn(sr, r.x);
            sg = __fadd_rn(sg, r.y);
            sb = __fadd_rn(sb, r.z);
            w = r.w;
        }
        // PathTracer::trace divides by pathSampleCount (PathTracer.cpp:22);
        // Film::addSample adds color * weight and weight (Film.cpp:57-58).
        f.x = __fadd_rn(f.x, __fmul_rn(__fdiv_rn(sr, fP), w));
        f.y = __fadd_rn(f.y, __fmul_rn(__fdiv_rn(sg, fP), w));
        f.z = __fadd_rn(f.z, __fmul_rn(__fdiv_rn(sb, fP), w));
        f.w = __fadd_rn(f.w, w);
    }
    *fp = f;
}

// Persistent grid: resident blocks per SM (cached per device) x the
// launching handle's SMs.
template <typename K>
int persistent_blocks(K kernel, int block, int numSMs, OccupancyCache& cache)
{
    return blocks_per_sm(kernel, block, 0, cache) * numSMs;
}

template <int ORDER, bool COUNT, int BLOCK>
cudaError_t extend_b(const PassParams& p, int segment, cudaStream_t stream, int numSMs)
{
    auto k = k_extend<ORDER, COUNT, BLOCK>;
    static OccupancyCache occ;
    k<<<persistent_blocks(k, BLOCK, numSMs, occ), BLOCK, 0, stream>>>(p, segment);
    return cudaGetLastError();
}

template <int BLOCK>
cudaError_t extend_refill_b(const PassParams& p, int segment, cudaStream_t stream, int numSMs)
{
    auto k = k_extend_refill<BLOCK>;
    static OccupancyCache occ;
    k<<<persistent_blocks(k, BLOCK, numSMs, occ), BLOCK, 0, stream>>>(p, segment);
    return cudaGetLastError();
}

// Whether the uncounted 4-wide extend refills idle lanes (k_extend_refill,
// RC_EXTEND_REFILL=1; read once). Off by default: on the 1080p workloads it
// measured 3-6 % slower than one batch of 32 rays per warp at every refill
// threshold (4-24 idle lanes) and register budget (6-9 blocks per SM) tried.
bool extend_refill()
{
    static const bool on = [] {
        const char* v = std::getenv("RC_EXTEND_REFILL");
        return v && v[0] == '1';
    }();
    return on;
}

template <int ORDER, bool COUNT>
cudaError_t extend_t(const PassParams& p, int segment, int block, cudaStream_t stream, int numSMs)
{
    if (ORDER == ORDER_WIDE && !COUNT && extend_refill())
    {
        if (block == 64)
            return extend_refill_b<64>(p, segment, stream, numSMs);
        if (block == 256)
            return extend_refill_b<256>(p, segment, stream, numSMs);
        return extend_refill_b<128>(p, segment, stream, numSMs);
    }
    if (block == 64)
        return extend_b<ORDER, COUNT, 64>(p, segment, stream, numSMs);
    if (block == 256)
        return extend_b<ORDER, COUNT, 256>(p, segment, stream, numSMs);
    return extend_b<ORDER, COUNT, 128>(p, segment, stream, numSMs);
}

// RC_EXTEND_SHADE=0 in the environment (read once) keeps extend and shade
// as two kernels per segment.
bool extend_shade_fused()
{
    static const bool on = [] {
        const char* v = std::getenv("RC_EXTEND_SHADE");
        return !(v && v[0] == '0');
    }();
    return on;
}

template <int BLOCK, bool NRC>
cudaError_t extend_shade_b(const PassParams& p, int segment, cudaStream_t stream, int numSMs)
{
    auto k = k_extend_shade<BLOCK, NRC>;
    static OccupancyCache occ;
    k<<<persistent_blocks(k, BLOCK, numSMs, occ), BLOCK, 0, stream>>>(p, segment);
    return cudaGetLastError();
}

// The block sizes of the kernels it replaces: the autotuned extend block for
// plain passes, 128 threads for cache passes.
cudaError_t extend_shade_t(const PassParams& p, int segment, int block, cudaStream_t stream, int numSMs)
{
    if (p.nrc.query)
        return extend_shade_b<128, true>(p, segment, stream, numSMs);
    if (block == 64)
        return extend_shade_b<64, false>(p, segment, stream, numSMs);
    if (block == 256)
        return extend_shade_b<256, false>(p, segment, stream, numSMs);
    return extend_shade_b<128, false>(p, segment, stream, numSMs);
}

template <bool COUNT>
cudaError_t extend_inst(const PassParams& p, int segment, cudaStream_t stream, int numSMs)
{
    auto k = k_extend_instanced<COUNT>;
    static OccupancyCache occ;
    k<<<persistent_blocks(k, 128, numSMs, occ), 128, 0, stream>>>(p, segment);
    return cudaGetLastError();
}

template <int BLOCK, bool NRC>
cudaError_t shade_b(const PassParams& p, int segment, cudaStream_t stream, int numSMs)
{
    auto k = k_shade<BLOCK, NRC>;
    static OccupancyCache occ;
    k<<<persistent_blocks(k, BLOCK, numSMs, occ), BLOCK, 0, stream>>>(p, segment);
    return cudaGetLastError();
}

cudaError_t shade_t(const PassParams& p, int segment, int block, cudaStream_t stream, int numSMs)
{
    if (p.nrc.query)
        return shade_b<128, true>(p, segment, stream, numSMs);
    if (block == 64)
        return shade_b<64, false>(p, segment, stream, numSMs);
    if (block == 256)
        return shade_b<256, false>(p, segment, stream, numSMs);
    return shade_b<128, false>(p, segment, stream, numSMs);
}

// One thread per training path: walks its vertices backwards, replacing
// each bounce factor f_i by the suffix radiance L_i = f_i * L_{i+1}
// (L_V = the terminal radiance), and lists the vertices that are samples:
// all of them when the path ended by leaving the scene, on an emitter or
// by Russian roulette; when the depth limit cut it, those with at least
// minSuffix vertices from themselves to the cut.
__global__ void __launch_bounds__(256) k_nrc_targets(PassParams p)
{
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= uint32_t(p.nrc.groups) || pass_stopped(p))
        return;
    const float4 t = p.nrc.term[g];
    const uint32_t flags = __float_as_uint(t.w);
    if (!(flags & kNrcTermActive))
        return;
    const int V = int(flags & 255u);
    const bool truncated = (flags & kNrcTermTruncated) != 0;
    // a suffix cut by the depth limit counts only with minSuffix vertices
    const int last = truncated ? V - p.nrc.minSuffix : V - 1;
    float r = t.x, gg = t.y, b = t.z;
    int count = 0;
    for (int i = V - 1; i >= 0; --i)
    {
        const size_t idx = size_t(i) * size_t(p.nrc.groups) + g;
        float4 d = p.nrc.vtx[idx].d;
        r = __fmul_rn(d.x, r);
        gg = __fmul_rn(d.y, gg);
        b = __fmul_rn(d.z, b);
        // tag: vertex index << 24 | training path (group) index
        p.nrc.vtx[idx].d = make_float4(r, gg, b, __uint_as_float((uint32_t(i) << 24) | g));
        // specular (dielectric) vertices carry albedo -1: not samples
        if (i <= last && !(p.nrc.vtx[idx].c.y < 0.0f) && (!p.nrc.lookupVertexOnly || i == p.nrc.termSegment))
            count++;
    }
    if (count == 0)
        return;
    unsigned k = atomicAdd(&p.nrc.counters[1], unsigned(count));
    for (int i = last; i >= 0; --i)
    {
        const size_t idx = size_t(i) * size_t(p.nrc.groups) + g;
        if (!(p.nrc.vtx[idx].c.y < 0.0f) && (!p.nrc.lookupVertexOnly || i == p.nrc.termSegment))
            p.nrc.index[k++] = int(idx);
    }
}

}  // namespace

cudaError_t launch_path_segments(const PassParams& p, int order, int counting, const PassShape& shape,
                                 cudaStream_t stream, int numSMs, const cudaEvent_t* extendEvents)
{
    k_generate<<<unsigned((p.nslots + 255) / 256), 256, 0, stream>>>(p);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    // uncounted nearest-first passes over a 4-wide tree: one kernel per segment
    const bool fused = !p.instanced && order == ORDER_NEAREST && !counting && p.wide && !extend_refill() &&
                       extend_shade_fused();
    for (int seg = 0; seg < p.segments; ++seg)
    {
        if (extendEvents && (e = cudaEventRecord(extendEvents[2 * seg], stream)) != cudaSuccess)
            return e;
        if (fused)
        {
            if ((e = extend_shade_t(p, seg, shape.extendBlock, stream, numSMs)) != cudaSuccess)
                return e;
            if (extendEvents && (e = cudaEventRecord(extendEvents[2 * seg + 1], stream)) != cudaSuccess)
                return e;
            continue;
        }
        if (p.instanced)
            e = counting ? extend_inst<true>(p, seg, stream, numSMs) : extend_inst<false>(p, seg, stream, numSMs);
        else if (order == ORDER_NEAREST)
            e = counting ? extend_t<ORDER_NEAREST, true>(p, seg, shape.extendBlock, stream, numSMs)
                : p.wide ? extend_t<ORDER_WIDE, false>(p, seg, shape.extendBlock, stream, numSMs)
                         : extend_t<ORDER_NEAREST, false>(p, seg, shape.extendBlock, stream, numSMs);
        else
            e = counting ? extend_t<ORDER_REF, true>(p, seg, shape.extendBlock, stream, numSMs)
                         : extend_t<ORDER_REF, false>(p, seg, shape.extendBlock, stream, numSMs);
        if (e != cudaSuccess)
            return e;
        if (extendEvents && (e = cudaEventRecord(extendEvents[2 * seg + 1], stream)) != cudaSuccess)
            return e;
        if ((e = shade_t(p, seg, shape.shadeBlock, stream, numSMs)) != cudaSuccess)
            return e;
    }
    return cudaSuccess;
}

cudaError_t launch_path_accumulate(const PassParams& p, cudaStream_t stream)
{
    k_accumulate<<<unsigned((p.npixels + 255) / 256), 256, 0, stream>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_path_pass(const PassParams& p, int order, int counting, const PassShape& shape,
                             cudaStream_t stream, int numSMs, const cudaEvent_t* extendEvents)
{
    cudaError_t e = launch_path_segments(p, order, counting, shape, stream, numSMs, extendEvents);
    if (e != cudaSuccess)
        return e;
    return launch_path_accumulate(p, stream);
}

cudaError_t launch_nrc_targets(const PassParams& p, cudaStream_t stream)
{
    if (p.nrc.groups <= 0)
        return cudaSuccess;
    k_nrc_targets<<<unsigned((p.nrc.groups + 255) / 256), 256, 0, stream>>>(p);
    return cudaGetLastError();
}

}  // namespace rcx
