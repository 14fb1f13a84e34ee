// Reconstruction filters of the film (Rendering/Filters/*.cpp), float32,
// with explicitly rounded operations so the CPU float32 oracle reproduces
// every weight bit for bit. The filter is separable: the weight of a sample
// at offset (x, y) from the pixel centre is w(x) * w(y) (Filter.cpp:26-29),
// and offsets span [-radius, radius) per axis (Tracer.cpp:135-139).
//
//   BOX       x in [-r, r) ? 1 / (2 r) : 0                       (BoxFilter.cpp:23-29)
//   TENT      s = |x / r|: s < 1 ? (1 - s) / r : 0, r = 1        (TentFilter.cpp:8-40)
//   BELL      s = |x|: s < 1/2 ? 3/4 - s^2 : s <= 3/2 ? (s - 3/2)^2 / 2 : 0, r = 3/2
//   GAUSSIAN  alpha exp(beta x^2), alpha = 1 / sqrt(2 pi), beta = -1/2,
//             r = 7.43384 / 2 (full width at a thousandth)       (GaussianFilter.cpp:12-31)
//   MITCHELL  B = C = 1/3 cubic on |x| <= 1 and 1 < |x| <= 2, r = 2  (MitchellFilter.cpp:8-45)
//   LANCZOS   s = |x|: s = 0 ? 1 : s > r ? 0 : sinc(s) sinc(s / r), r = 2
//
// exp(t) for the Gaussian (t in [-7, 0]): t = n ln2 + f with n the nearest
// integer to t / ln2 (Cody-Waite split of ln2 into a 16-bit head and a
// tail), e^f by its Taylor series to degree 7 (|f| <= 0.35: truncation
// error < 1e-8), times 2^n built in the exponent field. sin(pi s) for the
// Lanczos sinc: sincos_turn (sampling.cuh) of s / 2.
#pragma once

#include <cuda_runtime.h>

#include "pathtrace.h"
#include "sampling.cuh"

namespace rcx
{

__device__ __forceinline__ float filter_exp(float t)
{
    const float y = __fmul_rn(t, 1.44269504088896341f);
    const float n = floorf(__fadd_rn(y, 0.5f));
    float f = __fmaf_rn(-n, 0.693145751953125f, t);
    f = __fmaf_rn(-n, 1.42860682030941723e-6f, f);
    float p = __fmaf_rn(f, 1.98412698412698413e-4f, 1.38888888888888889e-3f);
    p = __fmaf_rn(f, p, 8.33333333333333333e-3f);
    p = __fmaf_rn(f, p, 4.16666666666666667e-2f);
    p = __fmaf_rn(f, p, 1.66666666666666667e-1f);
    p = __fmaf_rn(f, p, 0.5f);
    p = __fmaf_rn(f, p, 1.0f);
    p = __fmaf_rn(f, p, 1.0f);
    const int e = int(n);
    if (e < -126)
        return 0.0f;
    return __fmul_rn(p, __int_as_float((e + 127) << 23));
}

// sin(pi s) / (pi s), s in (0, 2].
__device__ __forceinline__ float filter_sinc(float s)
{
    float sv, cv;
    sincos_turn(__fmul_rn(s, 0.5f), sv, cv);
    return __fdiv_rn(sv, __fmul_rn(3.14159265358979324f, s));
}

// Weight of one axis: x the sample's offset, r the radius, a and b the
// per-axis constants of FilterSpec.
__device__ __forceinline__ float filter_weight_1d(const FilterSpec& f, float x, float r, float a, float b)
{
    switch (f.type)
    {
    case RC_FILTER_BOX:
        return (x >= -r && x < r) ? a : 0.0f;
    case RC_FILTER_TENT:
    {
        const float s = fabsf(__fmul_rn(x, a));
        return s < 1.0f ? __fmul_rn(__fsub_rn(1.0f, s), a) : 0.0f;
    }
    case RC_FILTER_BELL:
    {
        const float s = fabsf(x);
        if (s < 0.5f)
            return __fsub_rn(0.75f, __fmul_rn(s, s));
        if (s <= 1.5f)
        {
            const float t = __fsub_rn(s, 1.5f);
            return __fmul_rn(0.5f, __fmul_rn(t, t));
        }
        return 0.0f;
    }
    case RC_FILTER_GAUSSIAN:
        return __fmul_rn(a, filter_exp(__fmul_rn(__fmul_rn(x, x), b)));
    case RC_FILTER_MITCHELL:
    {
        const float s = fabsf(x);
        const float* c = s <= 1.0f ? f.cubic : f.cubic + 4;
        if (s > 2.0f)
            return 0.0f;
        return __fmaf_rn(__fmaf_rn(__fmaf_rn(c[0], s, c[1]), s, c[2]), s, c[3]);
    }
    default:  // RC_FILTER_LANCZOS_SINC
    {
        const float s = fabsf(x);
        if (s == 0.0f)
            return 1.0f;
        if (s > r)
            return 0.0f;
        return __fmul_rn(filter_sinc(s), filter_sinc(__fdiv_rn(s, r)));
    }
    }
}

__device__ __forceinline__ float filter_weight(const FilterSpec& f, float ox, float oy)
{
    return __fmul_rn(filter_weight_1d(f, ox, f.rx, f.ax, f.bx), filter_weight_1d(f, oy, f.ry, f.ay, f.by));
}

}  // namespace rcx
