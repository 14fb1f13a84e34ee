// Neural radiance cache: input encoding and network layout (device side).
//
// Query record (12 floats): position x, direction w (unit, pointing from the
// surface back toward where the path came from), geometric normal n, diffuse
// albedo rho.
//
// Input features (128, BF16):
//   [  0,  72)  position: for each axis a (x, y, z) and frequency k = 0..11:
//               sin(2^k pi u_a), cos(2^k pi u_a), u = (x - box_min) / box_size
//   [ 72,  96)  direction: for each axis and k = 0..3: sin / cos(2^k pi (w_a+1)/2)
//               (sin / cos(pi x) by nrc_sincospi below, float accurate)
//   [ 96,  99)  normal, [99, 102) albedo, [102] = 1 (the layers have no bias)
//   [103, 128)  0
// Network: 128 -> 64 -> 64 -> 64 -> 64 -> 3, ReLU between, exp on the output
// (4 hidden layers of width 64). Weights W_l are stored [out][in] in BF16 with
// FP32 master copies; the output layer is padded to 8 rows (rows 3..7 zero).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "nrc_kernels.h"

namespace rcx
{

constexpr int kNrcHidden = 64;
constexpr int kNrcOutPad = 8;
constexpr int kNrcOut = 3;
// Offsets (in elements) of each layer's [out][in] matrix in the packed weights.
constexpr int kNrcW1 = 0;
constexpr int kNrcW2 = kNrcW1 + kNrcHidden * kNrcIn;      // 8192
constexpr int kNrcW3 = kNrcW2 + kNrcHidden * kNrcHidden;  // 12288
constexpr int kNrcW4 = kNrcW3 + kNrcHidden * kNrcHidden;  // 16384
constexpr int kNrcW5 = kNrcW4 + kNrcHidden * kNrcHidden;  // 20480
constexpr int kNrcParams = kNrcW5 + kNrcOutPad * kNrcHidden;  // 20992 (20,672 used)
static_assert(kNrcParams == kNrcParamCount, "parameter count mismatch");

// q[base + i] for a run-time i in [0, n) without dynamic register indexing.
template <int N>
__device__ __forceinline__ float pick(const float* q, int base, int i)
{
    float v = q[base];
#pragma unroll
    for (int k = 1; k < N; ++k)
        v = i == k ? q[base + k] : v;
    return v;
}

// sin(pi x) and cos(pi x) in float. x = j + r with j = rint(x) and |r| <= 1/2
// (both exact); sin(pi r) and cos(pi r) from their Taylor series through r^11
// and r^12 (truncation error below 5.7e-8 and 6.4e-9 at |r| = 1/2), in Horner
// form; then sin(pi x) = (-1)^j sin(pi r), cos(pi x) = (-1)^j cos(pi r). The
// parity of j is read in float (j / 2 is exact), so it holds for every |x|.
__device__ __forceinline__ void nrc_sincospi(float x, float& s, float& c)
{
    const float j = rintf(x);
    const float r = x - j;
    const float r2 = r * r;
    // (-1)^n pi^(2n+1) / (2n+1)!  and  (-1)^n pi^(2n) / (2n)!
    float ps = -0.007370430945714348f;
    ps = fmaf(ps, r2, 0.08214588661112819f);
    ps = fmaf(ps, r2, -0.5992645293207919f);
    ps = fmaf(ps, r2, 2.550164039877345f);
    ps = fmaf(ps, r2, -5.167712780049969f);
    ps = fmaf(ps, r2, 3.141592653589793f);
    float pc = 0.001929574309403922f;
    pc = fmaf(pc, r2, -0.02580689139001405f);
    pc = fmaf(pc, r2, 0.23533063035889312f);
    pc = fmaf(pc, r2, -1.3352627688545893f);
    pc = fmaf(pc, r2, 4.058712126416768f);
    pc = fmaf(pc, r2, -4.934802200544679f);
    pc = fmaf(pc, r2, 1.0f);
    ps = ps * r;
    const float h = 0.5f * j;
    const bool odd = rintf(h) != h;
    s = odd ? -ps : ps;
    c = odd ? -pc : pc;
}

// Features c and c + 1 of a query, c even (see the table above), in float:
// one sin / cos pair of the frequency encoding, or two plain values.
__device__ __forceinline__ void nrc_feature_pair(int c, const float* q, const NrcBox& box, float& f0, float& f1)
{
    if (c < 96)
    {
        float u;
        int k;
        if (c < 72)
        {
            const int a = c / 24;
            k = (c - a * 24) >> 1;
            const float lo = a == 0 ? box.lo[0] : (a == 1 ? box.lo[1] : box.lo[2]);
            const float inv = a == 0 ? box.inv[0] : (a == 1 ? box.inv[1] : box.inv[2]);
            u = (pick<3>(q, 0, a) - lo) * inv;
        }
        else
        {
            const int r = c - 72;
            const int a = r / 8;
            k = (r - a * 8) >> 1;
            u = 0.5f * (pick<3>(q, 3, a) + 1.0f);
        }
        // u * 2^k: exact, like ldexp
        nrc_sincospi(u * __int_as_float((127 + k) << 23), f0, f1);
        return;
    }
    if (c < 102)
    {
        f0 = pick<6>(q, 6, c - 96);
        f1 = pick<6>(q, 6, c - 95);
        return;
    }
    f0 = c == 102 ? 1.0f : 0.0f;
    f1 = 0.0f;
}

// Feature c of a query, in float.
__device__ __forceinline__ float nrc_feature(int c, const float* q, const NrcBox& box)
{
    float f0, f1;
    nrc_feature_pair(c & ~1, q, box, f0, f1);
    return (c & 1) ? f1 : f0;
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

// Two features as packed BF16 (c even).
__device__ __forceinline__ uint32_t nrc_feature_bf16x2(int c, const float* q, const NrcBox& box)
{
    float f0, f1;
    nrc_feature_pair(c, q, box, f0, f1);
    return pack_bf16(f0, f1);
}

// D = A * B + D for one m16n8k16 tile (BF16 inputs, FP32 accumulate).
__device__ __forceinline__ void mma_bf16(float* d, const uint32_t* a, const uint32_t* b)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

}  // namespace rcx
