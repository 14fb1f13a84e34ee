// Neural radiance cache: fused BF16 MLP kernels on the tensor cores
// (mma.sync m16n8k16, FP32 accumulation) and FP32 Adam.
//
// Inference (k_nrc_infer): one warp evaluates 16 queries at a time. The
// encoded inputs are computed straight into the A fragments; each layer's
// accumulator fragments (16 rows x 8 columns per n-tile) are, after ReLU and
// BF16 packing, exactly the next layer's A fragments, so activations never
// leave registers. Weights sit in shared memory with rows padded by 8
// elements (no bank conflicts on the B-fragment loads).
//
// Training (k_nrc_train): per warp, a 16-sample tile runs forward with the
// activations stored to its shared-memory scratch (BF16), then backward:
// relative-L2 loss gradient, dH = dZ W (mma), dZ = dH * relu', and
// dW = dZ^T H (mma over the 16 samples) added into a per-block FP32 gradient
// array in shared memory. Each block writes its gradient sum to its own
// partial buffer; k_nrc_adam sums the partials in a fixed order, so the
// step is independent of block scheduling, and applies Adam to the FP32
// master weights, refreshing the BF16 copy.

#include <cuda_bf16.h>

#include <algorithm>

#include "nrc.cuh"
#include "sampling.cuh"
#include "nrc_kernels.h"

namespace rcx
{
namespace
{

constexpr int kWarps = 4;
constexpr int kThreads = kWarps * 32;
// padded row strides (elements) of the shared-memory weight copies
constexpr int kLd1 = kNrcIn + 8;       // 136
constexpr int kLdH = kNrcHidden + 8;   // 72
constexpr int kS1 = 0;
constexpr int kS2 = kS1 + kNrcHidden * kLd1;   // 8704
constexpr int kS3 = kS2 + kNrcHidden * kLdH;   // 13312
constexpr int kS4 = kS3 + kNrcHidden * kLdH;   // 17920
constexpr int kS5 = kS4 + kNrcHidden * kLdH;   // 22528
constexpr int kSmemW = kS5 + kNrcOutPad * kLdH;  // 23104 elements = 46,208 B

// per-warp training scratch (elements of BF16)
constexpr int kLdT = 16 + 8;  // dZ5: 16 columns
constexpr int kScH0 = 0;
constexpr int kScH1 = kScH0 + 16 * kLd1;
constexpr int kScH2 = kScH1 + 16 * kLdH;
constexpr int kScH3 = kScH2 + 16 * kLdH;
constexpr int kScH4 = kScH3 + 16 * kLdH;
constexpr int kScZa = kScH4 + 16 * kLdH;
constexpr int kScZb = kScZa + 16 * kLdH;
constexpr int kScZ5 = kScZb + 16 * kLdH;
constexpr int kScratch = kScZ5 + 16 * kLdT;  // per warp

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// Copies the packed [out][in] weights into the padded shared-memory layout.
__device__ void load_weights(__nv_bfloat16* s, const __nv_bfloat16* __restrict__ w)
{
    for (int i = threadIdx.x; i < kNrcParams; i += blockDim.x)
    {
        int dst;
        if (i < kNrcW2)
            dst = kS1 + (i / kNrcIn) * kLd1 + (i % kNrcIn);
        else if (i < kNrcW5)
        {
            int l = (i - kNrcW2) / (kNrcHidden * kNrcHidden);
            int r = (i - kNrcW2) % (kNrcHidden * kNrcHidden);
            dst = kS2 + l * kNrcHidden * kLdH + (r / kNrcHidden) * kLdH + (r % kNrcHidden);
        }
        else
            dst = kS5 + ((i - kNrcW5) / kNrcHidden) * kLdH + ((i - kNrcW5) % kNrcHidden);
        s[dst] = w[i];
    }
}

__device__ __forceinline__ uint32_t ld32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

__device__ __forceinline__ uint32_t pack_raw(__nv_bfloat16 lo, __nv_bfloat16 hi)
{
    return uint32_t(__bfloat16_as_ushort(lo)) | (uint32_t(__bfloat16_as_ushort(hi)) << 16);
}

// Encoded inputs of rows r0 (= gid) and r1 (= gid + 8) as A fragments.
__device__ __forceinline__ void encode_fragments(const float* q0, const float* q1, const NrcBox& box,
                                                 uint32_t (&A)[8][4])
{
    const int tig = int(lane_id() & 3u);
#pragma unroll
    for (int t = 0; t < 8; ++t)
    {
        int c0 = 16 * t + tig * 2;
        int c1 = c0 + 8;
        A[t][0] = pack_bf16(nrc_feature(c0, q0, box), nrc_feature(c0 + 1, q0, box));
        A[t][1] = pack_bf16(nrc_feature(c0, q1, box), nrc_feature(c0 + 1, q1, box));
        A[t][2] = pack_bf16(nrc_feature(c1, q0, box), nrc_feature(c1 + 1, q0, box));
        A[t][3] = pack_bf16(nrc_feature(c1, q1, box), nrc_feature(c1 + 1, q1, box));
    }
}

// C[8 n-tiles] = A[KT k-tiles] x W^T, W = [64][ld] in shared memory.
template <int KT>
__device__ __forceinline__ void layer_mma(const uint32_t (&A)[KT][4], const __nv_bfloat16* W, int ld, float (&C)[8][4])
{
    const int gid = int(lane_id() >> 2), tig = int(lane_id() & 3u);
#pragma unroll
    for (int j = 0; j < 8; ++j)
    {
        C[j][0] = C[j][1] = C[j][2] = C[j][3] = 0.0f;
        const __nv_bfloat16* row = W + (8 * j + gid) * ld + tig * 2;
#pragma unroll
        for (int t = 0; t < KT; ++t)
        {
            uint32_t b[2] = { ld32(row + 16 * t), ld32(row + 16 * t + 8) };
            mma_bf16(C[j], A[t], b);
        }
    }
}

__device__ __forceinline__ void relu_pack(const float (&C)[8][4], uint32_t (&A)[4][4])
{
#pragma unroll
    for (int t = 0; t < 4; ++t)
    {
        A[t][0] = pack_bf16(fmaxf(C[2 * t][0], 0.0f), fmaxf(C[2 * t][1], 0.0f));
        A[t][1] = pack_bf16(fmaxf(C[2 * t][2], 0.0f), fmaxf(C[2 * t][3], 0.0f));
        A[t][2] = pack_bf16(fmaxf(C[2 * t + 1][0], 0.0f), fmaxf(C[2 * t + 1][1], 0.0f));
        A[t][3] = pack_bf16(fmaxf(C[2 * t + 1][2], 0.0f), fmaxf(C[2 * t + 1][3], 0.0f));
    }
}

// Output layer: out[8] fragment (columns 0..2 used) from the last hidden A fragments.
__device__ __forceinline__ void output_mma(const uint32_t (&A)[4][4], const __nv_bfloat16* W5, float (&C)[4])
{
    const int gid = int(lane_id() >> 2), tig = int(lane_id() & 3u);
    C[0] = C[1] = C[2] = C[3] = 0.0f;
    const __nv_bfloat16* row = W5 + gid * kLdH + tig * 2;
#pragma unroll
    for (int t = 0; t < 4; ++t)
    {
        uint32_t b[2] = { ld32(row + 16 * t), ld32(row + 16 * t + 8) };
        mma_bf16(C, A[t], b);
    }
}

// Full forward pass of the 16-row tile; returns the output fragment.
__device__ __forceinline__ void forward(const uint32_t (&A0)[8][4], const __nv_bfloat16* sW, float (&out)[4])
{
    float C[8][4];
    uint32_t A[4][4];
    layer_mma<8>(A0, sW + kS1, kLd1, C);
    relu_pack(C, A);
    layer_mma<4>(A, sW + kS2, kLdH, C);
    relu_pack(C, A);
    layer_mma<4>(A, sW + kS3, kLdH, C);
    relu_pack(C, A);
    layer_mma<4>(A, sW + kS4, kLdH, C);
    relu_pack(C, A);
    output_mma(A, sW + kS5, out);
}

__device__ __forceinline__ void load_query(const NrcRecord* rec, int r, float (&q)[kNrcQueryFloats])
{
    const float4* p = reinterpret_cast<const float4*>(rec + r);
    float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
    q[0] = a.x; q[1] = a.y; q[2] = a.z; q[3] = a.w;
    q[4] = b.x; q[5] = b.y; q[6] = b.z; q[7] = b.w;
    q[8] = c.x; q[9] = c.y; q[10] = c.z; q[11] = c.w;
}

__device__ __forceinline__ void zero_query(float (&q)[kNrcQueryFloats])
{
#pragma unroll
    for (int k = 0; k < kNrcQueryFloats; ++k)
        q[k] = 0.0f;
}

// Writes exp(o0), exp(o1) for output columns col, col + 1 of record r.
__device__ __forceinline__ void emit(const NrcInferParams& p, int r, int col, float o0, float o1)
{
    if (p.out)
    {
        p.out[size_t(r) * 3 + col] = __expf(o0);
        if (col + 1 < 3)
            p.out[size_t(r) * 3 + col + 1] = __expf(o1);
        return;
    }
    const int s = __float_as_int(__ldg(&p.rec[r].d.w));
    const float* th = reinterpret_cast<const float*>(p.thr + s);
    float* re = reinterpret_cast<float*>(p.res + s);
    re[col] = __fadd_rn(re[col], __fmul_rn(th[col], __expf(o0)));
    if (col + 1 < 3)
        re[col + 1] = __fadd_rn(re[col + 1], __fmul_rn(th[col + 1], __expf(o1)));
}

__global__ void __launch_bounds__(kThreads) k_nrc_infer(NrcInferParams p)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __nv_bfloat16* sW = reinterpret_cast<__nv_bfloat16*>(smem);
    const int n = int(*p.count);
    if (n == 0)
        return;
    load_weights(sW, p.weights);
    __syncthreads();
    const int tiles = (n + 15) / 16;
    const int warp = int(threadIdx.x >> 5);
    const int gid = int(lane_id() >> 2), tig = int(lane_id() & 3u);
    for (int tile = blockIdx.x * kWarps + warp; tile < tiles; tile += gridDim.x * kWarps)
    {
        const int r0 = tile * 16 + gid, r1 = r0 + 8;
        float q0[kNrcQueryFloats], q1[kNrcQueryFloats];
        if (r0 < n)
            load_query(p.rec, r0, q0);
        else
            zero_query(q0);
        if (r1 < n)
            load_query(p.rec, r1, q1);
        else
            zero_query(q1);
        uint32_t A0[8][4];
        encode_fragments(q0, q1, p.box, A0);
        float o[4];
        forward(A0, sW, o);
        // accumulator columns: lanes with tig 0 hold outputs 0, 1; tig 1 holds 2 (and padding 3)
        if (tig < 2)
        {
            if (r0 < n)
                emit(p, r0, tig * 2, o[0], o[1]);
            if (r1 < n)
                emit(p, r1, tig * 2, o[2], o[3]);
        }
    }
}

// ---------------------------------------------------------------------------
// Training

// A fragment of a row-major [16][ld] matrix at columns col0..col0+15.
__device__ __forceinline__ void frag_a(const __nv_bfloat16* M, int ld, int col0, uint32_t (&a)[4])
{
    const int gid = int(lane_id() >> 2), tig = int(lane_id() & 3u);
    a[0] = ld32(M + gid * ld + col0 + tig * 2);
    a[1] = ld32(M + (gid + 8) * ld + col0 + tig * 2);
    a[2] = ld32(M + gid * ld + col0 + 8 + tig * 2);
    a[3] = ld32(M + (gid + 8) * ld + col0 + 8 + tig * 2);
}

// A fragment of M^T (A[m][k] = M[k][m]) for m in m0.., k in 0..15; M = [16][ld].
__device__ __forceinline__ void frag_a_t(const __nv_bfloat16* M, int ld, int m0, uint32_t (&a)[4])
{
    const int gid = int(lane_id() >> 2), tig = int(lane_id() & 3u);
    const int k = tig * 2;
    a[0] = pack_raw(M[k * ld + m0 + gid], M[(k + 1) * ld + m0 + gid]);
    a[1] = pack_raw(M[k * ld + m0 + gid + 8], M[(k + 1) * ld + m0 + gid + 8]);
    a[2] = pack_raw(M[(k + 8) * ld + m0 + gid], M[(k + 9) * ld + m0 + gid]);
    a[3] = pack_raw(M[(k + 8) * ld + m0 + gid + 8], M[(k + 9) * ld + m0 + gid + 8]);
}

// B fragment with B[k][n] = M[k][n] (M row-major [rows][ld]) for k in k0..k0+15
// (rows >= kRows read as 0), n in n0..n0+7.
__device__ __forceinline__ void frag_b_kn(const __nv_bfloat16* M, int ld, int kRows, int k0, int n0, uint32_t (&b)[2])
{
    const int gid = int(lane_id() >> 2), tig = int(lane_id() & 3u);
    const __nv_bfloat16 z = __float2bfloat16(0.0f);
    int k = k0 + tig * 2;
    b[0] = pack_raw(k < kRows ? M[k * ld + n0 + gid] : z, k + 1 < kRows ? M[(k + 1) * ld + n0 + gid] : z);
    k += 8;
    b[1] = pack_raw(k < kRows ? M[k * ld + n0 + gid] : z, k + 1 < kRows ? M[(k + 1) * ld + n0 + gid] : z);
}

// Stores a [16 x 64] accumulator (8 n-tiles) as BF16 rows into M[16][ld], with ReLU.
__device__ __forceinline__ void store_relu(const float (&C)[8][4], __nv_bfloat16* M, int ld)
{
    const int gid = int(lane_id() >> 2), tig = int(lane_id() & 3u);
#pragma unroll
    for (int j = 0; j < 8; ++j)
    {
        *reinterpret_cast<uint32_t*>(M + gid * ld + 8 * j + tig * 2) =
            pack_bf16(fmaxf(C[j][0], 0.0f), fmaxf(C[j][1], 0.0f));
        *reinterpret_cast<uint32_t*>(M + (gid + 8) * ld + 8 * j + tig * 2) =
            pack_bf16(fmaxf(C[j][2], 0.0f), fmaxf(C[j][3], 0.0f));
    }
}

// dW[o][i] += sum over the 16 samples of dZ[s][o] * H[s][i]: outputs o in
// [0, outRows), inputs i in [0, inCols); added into the FP32 gradient g
// ([out][in], row stride inCols).
__device__ __forceinline__ void weight_grad(const __nv_bfloat16* dZ, int ldZ, int outRows, const __nv_bfloat16* H,
                                            int ldHh, int inCols, float* g)
{
    const int gid = int(lane_id() >> 2), tig = int(lane_id() & 3u);
    for (int m0 = 0; m0 < outRows; m0 += 16)
    {
        uint32_t a[4];
        frag_a_t(dZ, ldZ, m0, a);
        for (int n0 = 0; n0 < inCols; n0 += 8)
        {
            uint32_t b[2];
            frag_b_kn(H, ldHh, 16, 0, n0, b);
            float c[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
            mma_bf16(c, a, b);
            const int o0 = m0 + gid, o1 = o0 + 8, i = n0 + tig * 2;
            if (o0 < outRows)
            {
                atomicAdd(g + o0 * inCols + i, c[0]);
                atomicAdd(g + o0 * inCols + i + 1, c[1]);
            }
            if (o1 < outRows)
            {
                atomicAdd(g + o1 * inCols + i, c[2]);
                atomicAdd(g + o1 * inCols + i + 1, c[3]);
            }
        }
    }
}

// dZ_prev = (dZ x W) * (H_prev > 0), W = [out][ldW] padded shared weights with
// `outRows` rows; dZ = [16][ldZ] with K = 16 * kTiles columns; result written
// as BF16 into D[16][ldD] (64 columns).
__device__ __forceinline__ void input_grad(const __nv_bfloat16* dZ, int ldZ, int kTiles, const __nv_bfloat16* W,
                                           int ldW, int outRows, const __nv_bfloat16* Hprev, int ldHp,
                                           __nv_bfloat16* D, int ldD)
{
    const int gid = int(lane_id() >> 2), tig = int(lane_id() & 3u);
    for (int j = 0; j < 8; ++j)
    {
        float c[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
        for (int t = 0; t < kTiles; ++t)
        {
            uint32_t a[4], b[2];
            frag_a(dZ, ldZ, 16 * t, a);
            frag_b_kn(W, ldW, outRows, 16 * t, 8 * j, b);
            mma_bf16(c, a, b);
        }
        const int col = 8 * j + tig * 2;
        float m0 = __bfloat162float(Hprev[gid * ldHp + col]) > 0.0f ? 1.0f : 0.0f;
        float m1 = __bfloat162float(Hprev[gid * ldHp + col + 1]) > 0.0f ? 1.0f : 0.0f;
        float m2 = __bfloat162float(Hprev[(gid + 8) * ldHp + col]) > 0.0f ? 1.0f : 0.0f;
        float m3 = __bfloat162float(Hprev[(gid + 8) * ldHp + col + 1]) > 0.0f ? 1.0f : 0.0f;
        *reinterpret_cast<uint32_t*>(D + gid * ldD + col) = pack_bf16(c[0] * m0, c[1] * m1);
        *reinterpret_cast<uint32_t*>(D + (gid + 8) * ldD + col) = pack_bf16(c[2] * m2, c[3] * m3);
    }
}

// Record index of sample r of a training step.
__device__ __forceinline__ int sample_index(const NrcTrainParams& p, unsigned total, int r)
{
    if (!p.index)
        return p.first + r;
    uint32_t h = mix32(p.key ^ mix32(uint32_t(r) + 0x9e3779b9u));
    return p.index[h % total];
}

__global__ void __launch_bounds__(kThreads) k_nrc_train(NrcTrainParams p)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __nv_bfloat16* sW = reinterpret_cast<__nv_bfloat16*>(smem);
    float* sG = reinterpret_cast<float*>(smem + kSmemW * 2);
    __nv_bfloat16* scratchAll = reinterpret_cast<__nv_bfloat16*>(smem + kSmemW * 2 + kNrcParams * 4);
    load_weights(sW, p.weights);
    for (int i = threadIdx.x; i < kNrcParams; i += blockDim.x)
        sG[i] = 0.0f;
    __syncthreads();

    const int warp = int(threadIdx.x >> 5);
    const int gid = int(lane_id() >> 2), tig = int(lane_id() & 3u);
    __nv_bfloat16* sc = scratchAll + warp * kScratch;
    __nv_bfloat16* H0 = sc + kScH0;
    __nv_bfloat16* H1 = sc + kScH1;
    __nv_bfloat16* H2 = sc + kScH2;
    __nv_bfloat16* H3 = sc + kScH3;
    __nv_bfloat16* H4 = sc + kScH4;
    __nv_bfloat16* Za = sc + kScZa;
    __nv_bfloat16* Zb = sc + kScZb;
    __nv_bfloat16* Z5 = sc + kScZ5;
    float lossSum = 0.0f;
    const unsigned total = p.index ? *p.total : unsigned(p.batch);
    const int n = total == 0 ? 0 : p.batch;
    const int tiles = (n + 15) / 16;

    for (int tile = blockIdx.x * kWarps + warp; tile < tiles; tile += gridDim.x * kWarps)
    {
        const int r0 = tile * 16 + gid, r1 = r0 + 8;
        const bool v0 = r0 < n, v1 = r1 < n;
        const int i0 = v0 ? sample_index(p, total, r0) : 0;
        const int i1 = v1 ? sample_index(p, total, r1) : 0;
        float q0[kNrcQueryFloats], q1[kNrcQueryFloats];
        if (v0)
            load_query(p.rec, i0, q0);
        else
            zero_query(q0);
        if (v1)
            load_query(p.rec, i1, q1);
        else
            zero_query(q1);
        uint32_t A0[8][4];
        encode_fragments(q0, q1, p.box, A0);
        // H0: the encoded inputs
#pragma unroll
        for (int t = 0; t < 8; ++t)
        {
            *reinterpret_cast<uint32_t*>(H0 + gid * kLd1 + 16 * t + tig * 2) = A0[t][0];
            *reinterpret_cast<uint32_t*>(H0 + (gid + 8) * kLd1 + 16 * t + tig * 2) = A0[t][1];
            *reinterpret_cast<uint32_t*>(H0 + gid * kLd1 + 16 * t + 8 + tig * 2) = A0[t][2];
            *reinterpret_cast<uint32_t*>(H0 + (gid + 8) * kLd1 + 16 * t + 8 + tig * 2) = A0[t][3];
        }
        float C[8][4];
        uint32_t A[4][4];
        layer_mma<8>(A0, sW + kS1, kLd1, C);
        store_relu(C, H1, kLdH);
        relu_pack(C, A);
        layer_mma<4>(A, sW + kS2, kLdH, C);
        store_relu(C, H2, kLdH);
        relu_pack(C, A);
        layer_mma<4>(A, sW + kS3, kLdH, C);
        store_relu(C, H3, kLdH);
        relu_pack(C, A);
        layer_mma<4>(A, sW + kS4, kLdH, C);
        store_relu(C, H4, kLdH);
        relu_pack(C, A);
        float o[4];
        output_mma(A, sW + kS5, o);

        // Relative L2 loss (p - y)^2 / (p^2 + 0.01), mean over batch x 3;
        // the denominator is held constant for the gradient.
        for (int k = lane_id(); k < 16 * kLdT; k += 32)
            Z5[k] = __float2bfloat16(0.0f);
        __syncwarp();
        if (tig < 2)
        {
            const int col = tig * 2;
            const float scale = 1.0f / (float(n) * 3.0f);
            for (int h = 0; h < 2; ++h)
            {
                const bool valid = h == 0 ? v0 : v1;
                const int idx = h == 0 ? i0 : i1;
                const int row = h == 0 ? gid : gid + 8;
                for (int e = 0; e < 2; ++e)
                {
                    const int c = col + e;
                    if (!valid || c >= 3)
                        continue;
                    float pr = __expf(o[2 * h + e]);
                    float y = reinterpret_cast<const float*>(&p.rec[idx].d)[c];
                    float den = pr * pr + 0.01f;
                    float diff = pr - y;
                    lossSum += diff * diff / den * scale;
                    float g = 2.0f * diff / den * scale * pr;  // d/dz of exp(z)
                    Z5[row * kLdT + c] = __float2bfloat16(g);
                }
            }
        }
        __syncwarp();

        // layer 5: dW5, dZ4
        weight_grad(Z5, kLdT, kNrcOut, H4, kLdH, kNrcHidden, sG + kNrcW5);
        input_grad(Z5, kLdT, 1, sW + kS5, kLdH, kNrcOutPad, H4, kLdH, Za, kLdH);
        __syncwarp();
        // layer 4
        weight_grad(Za, kLdH, kNrcHidden, H3, kLdH, kNrcHidden, sG + kNrcW4);
        input_grad(Za, kLdH, 4, sW + kS4, kLdH, kNrcHidden, H3, kLdH, Zb, kLdH);
        __syncwarp();
        // layer 3
        weight_grad(Zb, kLdH, kNrcHidden, H2, kLdH, kNrcHidden, sG + kNrcW3);
        input_grad(Zb, kLdH, 4, sW + kS3, kLdH, kNrcHidden, H2, kLdH, Za, kLdH);
        __syncwarp();
        // layer 2
        weight_grad(Za, kLdH, kNrcHidden, H1, kLdH, kNrcHidden, sG + kNrcW2);
        input_grad(Za, kLdH, 4, sW + kS2, kLdH, kNrcHidden, H1, kLdH, Zb, kLdH);
        __syncwarp();
        // layer 1
        weight_grad(Zb, kLdH, kNrcHidden, H0, kLd1, kNrcIn, sG + kNrcW1);
        __syncwarp();
    }
    for (int off = 16; off > 0; off >>= 1)
        lossSum += __shfl_down_sync(0xffffffffu, lossSum, off);
    __shared__ float sLoss[kWarps];
    if (lane_id() == 0)
        sLoss[warp] = lossSum;
    __syncthreads();
    float* part = p.partials + size_t(blockIdx.x) * kNrcParams;
    for (int i = threadIdx.x; i < kNrcParams; i += blockDim.x)
        part[i] = sG[i];
    if (threadIdx.x == 0)
    {
        float l = 0.0f;
        for (int w = 0; w < kWarps; ++w)
            l += sLoss[w];
        p.lossPartials[blockIdx.x] = l;
    }
}

// Sums the per-block gradients (fixed order) and applies Adam, or only
// writes the summed gradient (adam == 0).
__global__ void k_nrc_adam(NrcAdamParams p)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0)
    {
        float l = 0.0f;
        for (int b = 0; b < p.numPartials; ++b)
            l += p.lossPartials[b];
        *p.loss = l;
    }
    if (i >= kNrcParams)
        return;
    float g = 0.0f;
    for (int b = 0; b < p.numPartials; ++b)
        g += p.partials[size_t(b) * kNrcParams + i];
    if (p.gradOut)
        p.gradOut[i] = g;
    if (!p.adam || (p.total && *p.total == 0))
        return;
    float m = p.beta1 * p.m[i] + (1.0f - p.beta1) * g;
    float v = p.beta2 * p.v[i] + (1.0f - p.beta2) * g * g;
    p.m[i] = m;
    p.v[i] = v;
    float mh = m / (1.0f - p.beta1Pow);
    float vh = v / (1.0f - p.beta2Pow);
    float w = p.master[i] - p.lr * mh / (sqrtf(vh) + p.eps);
    p.master[i] = w;
    p.weights[i] = __float2bfloat16(w);
}

__global__ void k_nrc_encode(const NrcRecord* __restrict__ rec, int n, NrcBox box, __nv_bfloat16* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * kNrcIn)
        return;
    const int r = i / kNrcIn, c = i - r * kNrcIn;
    float q[kNrcQueryFloats];
    load_query(rec, r, q);
    out[i] = __float2bfloat16(nrc_feature(c, q, box));
}

__global__ void k_nrc_to_bf16(const float* __restrict__ master, __nv_bfloat16* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kNrcParams)
        out[i] = __float2bfloat16(master[i]);
}

size_t nrc_infer_smem() { return size_t(kSmemW) * 2; }

}  // namespace

size_t nrc_train_smem() { return size_t(kSmemW) * 2 + size_t(kNrcParams) * 4 + size_t(kWarps * kScratch) * 2; }

int nrc_train_blocks(int numSMs) { return numSMs; }

cudaError_t launch_nrc_infer(const NrcInferParams& p, int maxRecords, cudaStream_t stream, int numSMs)
{
    static bool configured = false;
    if (!configured)
    {
        cudaError_t e =
            cudaFuncSetAttribute(k_nrc_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, int(nrc_infer_smem()));
        if (e != cudaSuccess)
            return e;
        configured = true;
    }
    int tiles = (maxRecords + 15) / 16;
    int grid = std::max(1, std::min((tiles + kWarps - 1) / kWarps, numSMs * 4));
    k_nrc_infer<<<grid, kThreads, nrc_infer_smem(), stream>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_nrc_train(const NrcTrainParams& p, int blocks, cudaStream_t stream)
{
    static bool configured = false;
    if (!configured)
    {
        cudaError_t e =
            cudaFuncSetAttribute(k_nrc_train, cudaFuncAttributeMaxDynamicSharedMemorySize, int(nrc_train_smem()));
        if (e != cudaSuccess)
            return e;
        configured = true;
    }
    k_nrc_train<<<blocks, kThreads, nrc_train_smem(), stream>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_nrc_adam(const NrcAdamParams& p, cudaStream_t stream)
{
    k_nrc_adam<<<(kNrcParams + 255) / 256, 256, 0, stream>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_nrc_encode(const NrcRecord* rec, int n, const NrcBox& box, __nv_bfloat16* out, cudaStream_t stream)
{
    if (n <= 0)
        return cudaSuccess;
    int total = n * kNrcIn;
    k_nrc_encode<<<(total + 255) / 256, 256, 0, stream>>>(rec, n, box, out);
    return cudaGetLastError();
}

cudaError_t launch_nrc_to_bf16(const float* master, __nv_bfloat16* out, cudaStream_t stream)
{
    k_nrc_to_bf16<<<(kNrcParams + 255) / 256, 256, 0, stream>>>(master, out);
    return cudaGetLastError();
}

}  // namespace rcx
