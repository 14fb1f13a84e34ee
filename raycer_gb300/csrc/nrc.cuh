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

// Feature c of a query (see the table above), in float.
__device__ __forceinline__ float nrc_feature(int c, const float* q, const NrcBox& box)
{
    if (c < 72)
    {
        int a = c / 24;
        int r = c - a * 24;
        int k = r >> 1;
        float lo = a == 0 ? box.lo[0] : (a == 1 ? box.lo[1] : box.lo[2]);
        float inv = a == 0 ? box.inv[0] : (a == 1 ? box.inv[1] : box.inv[2]);
        float u = (pick<3>(q, 0, a) - lo) * inv;
        float s, co;
        sincospif(ldexpf(u, k), &s, &co);
        return (r & 1) ? co : s;
    }
    if (c < 96)
    {
        int r = c - 72;
        int a = r / 8;
        int k = (r - a * 8) >> 1;
        float u = 0.5f * (pick<3>(q, 3, a) + 1.0f);
        float s, co;
        sincospif(ldexpf(u, k), &s, &co);
        return (r & 1) ? co : s;
    }
    if (c < 102)
        return pick<6>(q, 6, c - 96);
    return c == 102 ? 1.0f : 0.0f;
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
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
