// Wavefront path tracer (PathTracer, src/Raytracing/Tracers/PathTracer.cpp:13-75;
// pathtrace.cl:1-80) for one pass of paths.
//
// A pass holds whole pixels: slot s belongs to pixel s / spp of the pass and
// to sample (s % spp) of it, where spp = n*n camera samples (Tracer.cpp:
// 115-144, CMJ + box filter) x pathSampleCount paths per camera sample
// (PathTracer.cpp:19). Path state lives in SoA arrays indexed by slot:
//   o, d       ray (float4 each); o.w = the triangle the ray leaves from
//              (skipped by its closest-hit query, see traverse.cuh)
//   thr        path throughput (rgb)
//   res        radiance result (rgb) + the camera sample's filter weight (w)
//   hit        closest hit of the last extend (slot, t, u, v)
// Stages (one launch each, per segment):
//   generate   camera rays for every slot; queue 0 = all slots
//   extend     closest hit for every queued slot              (persistent)
//   shade      miss -> 0; emissive -> res = thr * emittance; last segment
//              -> 0; else cosine bounce, thr *= 2*rho*|w.n| (PathTracer.cpp:
//              58-72), optional Russian roulette, and the slot is appended
//              to the next queue (warp-ballot compaction)      (persistent)
//   accumulate per pixel, in sample order: c_j = (sum_k L_jk) / P,
//              film.rgb += w_j * c_j, film.w += w_j (Film::addSample,
//              Film.cpp:54-59). One thread owns one pixel: deterministic.
// Queue counts live on the device, so the host launches a fixed sequence
// without reading them back.

#include <cfloat>

#include "pathtrace.h"
#include "sampling.cuh"
#include "traverse.cuh"

namespace rcx
{
namespace
{

constexpr int kBlock = 128;

#ifndef RC_TRACE_MIN_BLOCKS
#define RC_TRACE_MIN_BLOCKS 10
#endif

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

__device__ __forceinline__ unsigned warp_fetch(unsigned* head, unsigned amount)
{
    unsigned base = 0;
    if (lane_id() == 0)
        base = atomicAdd(head, amount);
    return __shfl_sync(0xffffffffu, base, 0);
}

struct SlotInfo
{
    uint64_t pixelGlobal;
    uint64_t pixelLocal;
    uint32_t sample;  // j * P + k
    uint32_t j;
};

__device__ __forceinline__ SlotInfo slot_info(const PathParams& p, uint32_t s)
{
    SlotInfo si;
    uint32_t pix = s / uint32_t(p.spp);
    si.sample = s - pix * uint32_t(p.spp);
    si.j = si.sample / uint32_t(p.P);
    si.pixelLocal = p.passPixel + pix;
    si.pixelGlobal = p.pixelStart + si.pixelLocal;
    return si;
}

__device__ __forceinline__ float box_weight(float x, float r, float w)
{
    // BoxFilter::getWeightX (BoxFilter.cpp:23-29)
    return (x >= -r && x < r) ? w : 0.0f;
}

__global__ void __launch_bounds__(256) k_generate(PathParams p)
{
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s == 0)
        p.counts[0] = uint32_t(p.nslots);
    if (s >= uint32_t(p.nslots))
        return;
    SlotInfo si = slot_info(p, s);
    float px = float(si.pixelGlobal % uint64_t(p.width));
    float py = float(si.pixelGlobal / uint64_t(p.width));
    float w = 1.0f;
    if (p.n > 1)
    {
        uint32_t gx = si.j % uint32_t(p.n);
        uint32_t gy = si.j / uint32_t(p.n);
        uint32_t jkey = stream_key(p.seed, p.frame, si.pixelGlobal, 0x80000000u | si.j);
        float jx = stream_float(jkey, kCounterJitter + 0);
        float jy = stream_float(jkey, kCounterJitter + 1);
        float sx, sy;
        if (p.samplerType == RC_SAMPLER_CMJ)
        {
            // CMJSampler::getSample2D (CMJSampler.cpp:61-76), permutation per pixel.
            uint32_t pkey = stream_key(p.seed, p.frame, si.pixelGlobal, 0xffffffffu);
            uint64_t perm = (uint64_t(stream_u32(pkey, 1)) << 32) | stream_u32(pkey, 2);
            uint64_t n = uint64_t(p.n);
            uint64_t sxp = cmj_permute(gx, n, perm * 0x68bc21ebull);
            uint64_t syp = cmj_permute(gy, n, perm * 0x02e5be93ull);
            float fn = float(p.n);
            sx = __fdiv_rn(__fadd_rn(float(gx), __fdiv_rn(__fadd_rn(float(syp), jx), fn)), fn);
            sy = __fdiv_rn(__fadd_rn(float(gy), __fdiv_rn(__fadd_rn(float(sxp), jy), fn)), fn);
        }
        else if (p.samplerType == RC_SAMPLER_RANDOM)
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
        float ox = __fmul_rn(__fmul_rn(__fsub_rn(sx, 0.5f), 2.0f), p.rx);
        float oy = __fmul_rn(__fmul_rn(__fsub_rn(sy, 0.5f), 2.0f), p.ry);
        w = __fmul_rn(box_weight(ox, p.rx, p.wx), box_weight(oy, p.ry, p.wy));
        px = __fadd_rn(px, ox);
        py = __fadd_rn(py, oy);
    }
    V3 d = camera_dir(p.cam, px, py);
    p.o[s] = make_float4(p.cam.pos[0], p.cam.pos[1], p.cam.pos[2], __int_as_float(-1));
    p.d[s] = make_float4(d.x, d.y, d.z, 0.0f);
    p.thr[s] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
    p.res[s] = make_float4(0.0f, 0.0f, 0.0f, w);
    p.qa[s] = int(s);
}

template <int ORDER, bool COUNT>
__global__ void __launch_bounds__(kBlock, RC_TRACE_MIN_BLOCKS) k_extend(PathParams p, int segment)
{
    const unsigned total = *reinterpret_cast<volatile unsigned*>(&p.counts[segment * 4 + 0]);
    const int* __restrict__ queue = (segment & 1) ? p.qb : p.qa;
    TravCount cnt{ 0, 0 };
    int err = 0;
    unsigned long long done = 0;
    while (true)
    {
        unsigned base = warp_fetch(&p.counts[segment * 4 + 1], 32u);
        if (base >= total)
            break;
        unsigned q = base + lane_id();
        if (q < total)
        {
            int s = queue[q];
            float4 o = p.o[s];
            float4 d = p.d[s];
            RayF ray = make_ray(v3(o.x, o.y, o.z), v3(d.x, d.y, d.z), 0.0f, FLT_MAX);
            HitF h{ -1, FLT_MAX, 0.0f, 0.0f };
            bool found = traverse<false, ORDER, COUNT>(p.sc, ray, h, cnt, err, __float_as_int(o.w));
            p.hit[s] = make_int4(found ? h.slot : -1, __float_as_int(h.t), __float_as_int(h.u), __float_as_int(h.v));
            done++;
        }
    }
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
        if (COUNT)
        {
            atomicAdd(&p.ctl->stats[1], n);
            atomicAdd(&p.ctl->stats[2], t);
        }
    }
    if (err)
        atomicOr(&p.ctl->error, 1);
}

__global__ void __launch_bounds__(kBlock) k_shade(PathParams p, int segment)
{
    const unsigned total = *reinterpret_cast<volatile unsigned*>(&p.counts[segment * 4 + 0]);
    const int* __restrict__ qin = (segment & 1) ? p.qb : p.qa;
    int* __restrict__ qout = (segment & 1) ? p.qa : p.qb;
    unsigned* outCount = &p.counts[(segment + 1) * 4 + 0];
    const bool lastSegment = segment + 1 >= p.maxPathLength;
    while (true)
    {
        unsigned base = warp_fetch(&p.counts[segment * 4 + 2], 32u);
        if (base >= total)
            break;
        unsigned q = base + lane_id();
        bool cont = false;
        int s = -1;
        if (q < total)
        {
            s = qin[q];
            int4 h = p.hit[s];
            if (h.x >= 0)
            {
                const float4* tp = reinterpret_cast<const float4*>(p.sc.tris + h.x);
                float4 tc = __ldg(tp + 2);
                uint32_t mi = __float_as_uint(tc.y) & kMetaMaterialMask;
                float4 md = __ldg(&p.sc.mats[mi].diffuse);
                float4 me = __ldg(&p.sc.mats[mi].emittance);
                uint32_t mflags = __float_as_uint(me.w);
                float4 thr = p.thr[s];
                if (mflags & kMatEmissive)
                {
                    // sampleColor *= emittance (pathtrace.cl:44-51)
                    float4 r = p.res[s];
                    r.x = __fmul_rn(thr.x, me.x);
                    r.y = __fmul_rn(thr.y, me.y);
                    r.z = __fmul_rn(thr.z, me.z);
                    p.res[s] = r;
                }
                else if (!lastSegment)
                {
                    SlotInfo si = slot_info(p, uint32_t(s));
                    uint32_t key = stream_key(p.seed, p.frame, si.pixelGlobal, si.sample);
                    bool alive = true;
                    if (p.rrDepth > 0 && segment + 1 >= p.rrDepth)
                    {
                        float m = fmaxf(thr.x, fmaxf(thr.y, thr.z));
                        float qs = fminf(m, 1.0f);
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
                    if (alive)
                    {
                        const float4* sp = reinterpret_cast<const float4*>(p.sc.shade + h.x);
                        float4 sn = __ldg(sp + 0);
                        float4 st = __ldg(sp + 1);
                        float4 sb = __ldg(sp + 2);
                        V3 nrm = v3(sn.x, sn.y, sn.z);
                        if (mflags & kMatInvertNormal)
                            nrm = v3(-nrm.x, -nrm.y, -nrm.z);
                        float xr = stream_float(key, kCounterBounce + 2u * uint32_t(segment));
                        float yr = stream_float(key, kCounterBounce + 2u * uint32_t(segment) + 1u);
                        V3 dir = hemisphere_cosine(v3(st.x, st.y, st.z), v3(sb.x, sb.y, sb.z), nrm, xr, yr);
                        float4 o = p.o[s];
                        float4 d = p.d[s];
                        float t = __int_as_float(h.y);
                        V3 ip = vfma(v3(d.x, d.y, d.z), t, v3(o.x, o.y, o.z));
                        V3 no = vfma(dir, p.rayStartOffset, ip);
                        float alpha = fabsf(vdot(dir, nrm));
                        // brdf = 2 * reflectance * alpha (PathTracer.cpp:70-71)
                        thr.x = __fmul_rn(thr.x, __fmul_rn(__fmul_rn(2.0f, md.x), alpha));
                        thr.y = __fmul_rn(thr.y, __fmul_rn(__fmul_rn(2.0f, md.y), alpha));
                        thr.z = __fmul_rn(thr.z, __fmul_rn(__fmul_rn(2.0f, md.z), alpha));
                        p.o[s] = make_float4(no.x, no.y, no.z, __int_as_float(h.x));
                        p.d[s] = make_float4(dir.x, dir.y, dir.z, 0.0f);
                        p.thr[s] = thr;
                        cont = true;
                    }
                }
            }
        }
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
}

__global__ void __launch_bounds__(256) k_accumulate(PathParams p, int pixelsInPass)
{
    int pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= pixelsInPass)
        return;
    const int nn = p.n * p.n;
    const float fP = float(p.P);
    float4 f = p.film[p.passPixel + uint64_t(pix)];
    size_t base = size_t(pix) * size_t(p.spp);
    for (int j = 0; j < nn; ++j)
    {
        float sr = 0.0f, sg = 0.0f, sb = 0.0f, w = 0.0f;
        for (int k = 0; k < p.P; ++k)
        {
            float4 r = p.res[base + size_t(j) * size_t(p.P) + size_t(k)];
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
    p.film[p.passPixel + uint64_t(pix)] = f;
}

template <typename K>
int persistent_blocks(K kernel, int numSMs)
{
    int perSM = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kernel, kBlock, 0) != cudaSuccess || perSM < 1)
        perSM = 1;
    return perSM * numSMs;
}

template <int ORDER, bool COUNT>
cudaError_t extend_t(const PathParams& p, int segment, cudaStream_t stream, int numSMs)
{
    auto k = k_extend<ORDER, COUNT>;
    static int grid = 0;
    if (grid == 0)
        grid = persistent_blocks(k, numSMs);
    k<<<grid, kBlock, 0, stream>>>(p, segment);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_path_pass(const PathParams& p, int pixelsInPass, int order, int counting, cudaStream_t stream,
                             int numSMs, const cudaEvent_t* extendEvents)
{
    k_generate<<<unsigned((p.nslots + 255) / 256), 256, 0, stream>>>(p);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    static int shadeGrid = 0;
    if (shadeGrid == 0)
        shadeGrid = persistent_blocks(k_shade, numSMs);
    for (int seg = 0; seg < p.maxPathLength; ++seg)
    {
        if (extendEvents && (e = cudaEventRecord(extendEvents[2 * seg], stream)) != cudaSuccess)
            return e;
        if (order == ORDER_NEAREST)
            e = counting ? extend_t<ORDER_NEAREST, true>(p, seg, stream, numSMs)
                         : extend_t<ORDER_NEAREST, false>(p, seg, stream, numSMs);
        else
            e = counting ? extend_t<ORDER_REF, true>(p, seg, stream, numSMs)
                         : extend_t<ORDER_REF, false>(p, seg, stream, numSMs);
        if (e != cudaSuccess)
            return e;
        if (extendEvents && (e = cudaEventRecord(extendEvents[2 * seg + 1], stream)) != cudaSuccess)
            return e;
        k_shade<<<shadeGrid, kBlock, 0, stream>>>(p, seg);
        if ((e = cudaGetLastError()) != cudaSuccess)
            return e;
    }
    k_accumulate<<<unsigned((pixelsInPass + 255) / 256), 256, 0, stream>>>(p, pixelsInPass);
    return cudaGetLastError();
}

}  // namespace rcx
