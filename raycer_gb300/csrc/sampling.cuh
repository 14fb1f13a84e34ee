// Sampling for the path tracer (device side).
//
//  * Random numbers: a counter-based stream. Every path owns a 32-bit key
//    (seed, frame, pixel, sample within the pixel); the n-th number of the
//    path is a hash of (key, n). The hash is "lowbias32" (C. Wellons,
//    hash-prospector, 2018). Numbers are 24-bit uniforms in [0, 1). The
//    reference draws from per-thread std::mt19937 (Tracer.cpp:65-72) and
//    MWC64X on the GPU (random.cl); only the distribution matters for
//    parity, which is statistical.
//  * sin/cos of 2*pi*x for x in [0, 1): quarter-turn reduction, octant swap
//    and Taylor polynomials of degree 9 (sin) and 10 (cos) on [0, pi/4],
//    evaluated with fused multiply-adds (absolute error < 2e-7). The CPU
//    float32 oracle evaluates the same polynomial, so directions match bit
//    for bit.
//  * Cosine-weighted hemisphere (mapToHemisphere, Sampler.cpp:50-64 /
//    sampler.cl:1-14 with distribution 1): phi = 2*pi*x,
//    cos(theta) = (1 - y)^(1/2), sin(theta) = sqrt(1 - cos^2),
//    direction = u*onb.u + v*onb.v + w*onb.w.
//  * Correlated multi-jittered pixel samples (CMJSampler.cpp:13-76: Kensler's
//    permute() in 64-bit arithmetic, as the reference writes it).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "rc_math.cuh"

namespace rcx
{

__host__ __device__ __forceinline__ uint32_t mix32(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

__host__ __device__ __forceinline__ uint32_t stream_key(uint64_t seed, uint32_t frame, uint64_t pixel, uint32_t sample)
{
    uint32_t k = mix32(uint32_t(seed) ^ 0x68bc21ebu);
    k = mix32(k ^ uint32_t(seed >> 32));
    k = mix32(k ^ frame);
    k = mix32(k ^ uint32_t(pixel));
    k = mix32(k ^ uint32_t(pixel >> 32));
    k = mix32(k ^ sample);
    return k;
}

__host__ __device__ __forceinline__ uint32_t stream_u32(uint32_t key, uint32_t counter)
{
    return mix32(key ^ mix32(counter + 0x9e3779b9u));
}

__device__ __forceinline__ float stream_float(uint32_t key, uint32_t counter)
{
    return __uint2float_rn(stream_u32(key, counter) >> 8) * 5.9604644775390625e-8f;  // 2^-24
}

// Counter layout of a path's stream.
constexpr uint32_t kCounterBounce = 0;      // + 2 * segment + {0, 1}
constexpr uint32_t kCounterRoulette = 4096;  // + segment
constexpr uint32_t kCounterJitter = 8192;    // + {0, 1}

// sin and cos of 2*pi*x, x in [0, 1).
__device__ __forceinline__ void sincos_turn(float x, float& s, float& c)
{
    float t = __fmul_rn(x, 4.0f);
    int q = int(t);
    if (q > 3)
        q = 3;
    float r = __fsub_rn(t, float(q));
    bool swap = r > 0.5f;
    float a = swap ? __fsub_rn(1.0f, r) : r;
    float al = __fmul_rn(a, 1.57079632679489662f);
    float a2 = __fmul_rn(al, al);
    // sin(al) = al * (1 - a2/6 + a2^2/120 - a2^3/5040 + a2^4/362880)
    float ps = __fmaf_rn(a2, 2.7557319e-6f, -1.9841270e-4f);
    ps = __fmaf_rn(a2, ps, 8.3333333e-3f);
    ps = __fmaf_rn(a2, ps, -1.6666667e-1f);
    ps = __fmaf_rn(a2, ps, 1.0f);
    float sa = __fmul_rn(al, ps);
    // cos(al) = 1 - a2/2 + a2^2/24 - a2^3/720 + a2^4/40320 - a2^5/3628800
    float pc = __fmaf_rn(a2, -2.7557319e-7f, 2.4801587e-5f);
    pc = __fmaf_rn(a2, pc, -1.3888889e-3f);
    pc = __fmaf_rn(a2, pc, 4.1666667e-2f);
    pc = __fmaf_rn(a2, pc, -0.5f);
    float ca = __fmaf_rn(a2, pc, 1.0f);
    float sr = swap ? ca : sa;
    float cr = swap ? sa : ca;
    switch (q)
    {
    case 0: s = sr; c = cr; break;
    case 1: s = cr; c = -sr; break;
    case 2: s = -sr; c = -cr; break;
    default: s = -cr; c = sr; break;
    }
}

// Cosine-weighted direction about the frame (U, V, W).
__device__ __forceinline__ V3 hemisphere_cosine(V3 U, V3 V, V3 W, float x, float y)
{
    float sp, cp;
    sincos_turn(x, sp, cp);
    float ct = __fsqrt_rn(__fsub_rn(1.0f, y));
    float st = __fsqrt_rn(__fsub_rn(1.0f, __fmul_rn(ct, ct)));
    float u = __fmul_rn(st, cp);
    float v = __fmul_rn(st, sp);
    // u*U + v*V + w*W
    return vfma(W, ct, vfma(V, v, vscale(U, u)));
}

// Kensler's permute(), 64-bit arithmetic as in CMJSampler.cpp:13-45, with a
// cycle-walk bound (the walk ends after a couple of rounds in practice; past
// 64 rounds i % l is used, identically in the CPU oracle).
__host__ __device__ __forceinline__ uint64_t cmj_permute(uint64_t i, uint64_t l, uint64_t p)
{
    uint64_t w = l - 1;
    w |= w >> 1;
    w |= w >> 2;
    w |= w >> 4;
    w |= w >> 8;
    w |= w >> 16;
    uint64_t i0 = i;
    int rounds = 0;
    do
    {
        i ^= p;
        i *= 0xe170893dull;
        i ^= p >> 16;
        i ^= (i & w) >> 4;
        i ^= p >> 8;
        i *= 0x0929eb3full;
        i ^= p >> 23;
        i ^= (i & w) >> 1;
        i *= 1 | p >> 27;
        i *= 0x6935fa69ull;
        i ^= (i & w) >> 11;
        i *= 0x74dcb303ull;
        i ^= (i & w) >> 2;
        i *= 0x9e501cc3ull;
        i ^= (i & w) >> 2;
        i *= 0xc860a3dfull;
        i &= w;
        i ^= i >> 5;
        if (++rounds >= 64 && i >= l)
        {
            i = i0 % l;
            break;
        }
    } while (i >= l);
    return (i + p) % l;
}

}  // namespace rcx
