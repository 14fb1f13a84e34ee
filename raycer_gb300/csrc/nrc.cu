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
// Training (k_nrc_train): a block of 8 warps takes 128 samples at a time;
// forward and the backward chain dZ_{l-1} = (dZ_l W_l) * relu' run per warp
// on its 16 rows (register chains, activations and gradients also stored to
// shared memory as BF16), and dW_l = dZ_l^T H_{l-1} is a block-wide product
// over the 128 samples with every warp owning fixed dW tiles in registers
// (see the comment at k_nrc_train). Each block writes its gradient sum once
// to its own partial buffer; k_nrc_adam sums the partials in a fixed order
// and applies Adam to the FP32 master weights, refreshing the BF16 copy.

#include <cuda_bf16.h>

#include <algorithm>

#include "nrc.cuh"
#include "sampling.cuh"
#include "kernels.h"
#include "nrc_kernels.h"

namespace rcx
{
namespace
{

constexpr int kWarps = 8;  // inference block
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

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// Copies the packed [out][in] weights into the padded shared-memory layout,
// 8 elements (16 bytes) per load: every row length is a multiple of 8.
__device__ void load_weights(__nv_bfloat16* s, const __nv_bfloat16* __restrict__ w)
{
    constexpr int kVec = kNrcParams / 8;
    const uint4* __restrict__ src = reinterpret_cast<const uint4*>(w);
#pragma unroll 4
    for (int v = threadIdx.x; v < kVec; v += blockDim.x)
    {
        const int i = v * 8;
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
        *reinterpret_cast<uint4*>(s + dst) = __ldg(src + v);
    }
}

__device__ __forceinline__ uint32_t ld32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

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
        A[t][0] = nrc_feature_bf16x2(c0, q0, box);
        A[t][1] = nrc_feature_bf16x2(c0, q1, box);
        A[t][2] = nrc_feature_bf16x2(c1, q0, box);
        A[t][3] = nrc_feature_bf16x2(c1, q1, box);
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
//
// One block = 8 warps; it takes 128 samples at a time (16 rows per warp).
//   F   each warp: forward of its rows (register chain), H0..H4 and the
//       output-layer gradient dZ5 stored to shared memory (BF16)
//   P5  block: dW5 += dZ5^T H4;  each warp: dZ4 = (dZ5 W5) * [H4 > 0] (own rows)
//   P4  block: dW4 += dZ4^T H3;  each warp: dZ3 = (dZ4 W4) * [H3 > 0]
//   P3, P2 likewise; P1 block: dW1 += dZ1^T H0
// with a block barrier between phases (dZ alternates between two buffers).
// The weight gradient is a sum over samples, K = 128 per chunk: every warp
// owns a fixed set of 16x8 output tiles of dW (21 tiles, 84 FP32
// accumulators per lane) that stay in registers across all the block's
// chunks; the transposed operands come from shared memory through
// ldmatrix.trans. Each block writes its dW once (no atomics), so a block's
// sum has a fixed order.

constexpr int kTWarps = 8;
constexpr int kTThreads = kTWarps * 32;
constexpr int kChunk = 16 * kTWarps;            // 128 samples
constexpr int kLdT = 16 + 8;                     // dZ5 row stride: 16 columns used
constexpr int kTW = 0;                           // weights (W5 padded to 16 rows)
constexpr int kTH0 = kSmemW + 8 * kLdH;          // 23,680
constexpr int kTH1 = kTH0 + kChunk * kLd1;
constexpr int kTH2 = kTH1 + kChunk * kLdH;
constexpr int kTH3 = kTH2 + kChunk * kLdH;
constexpr int kTH4 = kTH3 + kChunk * kLdH;
constexpr int kTZA = kTH4 + kChunk * kLdH;
constexpr int kTZB = kTZA + kChunk * kLdH;
constexpr int kTZ5 = kTZB + kChunk * kLdH;
constexpr int kTEnd = kTZ5 + kChunk * kLdT;      // 99,456 elements = 198,912 B
static_assert(kTH0 % 8 == 0 && kTH1 % 8 == 0 && kTZ5 % 8 == 0, "ldmatrix rows need 16-byte alignment");

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Four 8x8 BF16 matrices, transposed; lane l gives the row address of
// matrix l / 8, row l % 8.
__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], const __nv_bfloat16* p)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_addr(p)));
}

__device__ __forceinline__ void ldsm_x2_t(uint32_t (&r)[2], const __nv_bfloat16* p)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n"
                 : "=r"(r[0]), "=r"(r[1])
                 : "r"(smem_addr(p)));
}

// Row address for an A fragment of M^T (A[m][k] = M[k][m], M row-major):
// matrices (k0-7, m0-7), (k0-7, m8-15), (k8-15, m0-7), (k8-15, m8-15).
__device__ __forceinline__ const __nv_bfloat16* a_trans_row(const __nv_bfloat16* M, int ld, int k0, int m0)
{
    const int l = int(lane_id());
    return M + (k0 + (l & 7) + ((l >> 4) & 1) * 8) * ld + m0 + ((l >> 3) & 1) * 8;
}

// Row address for the B fragments of two n-tiles of a row-major [k][n]
// matrix: (k0-7, n0-7), (k8-15, n0-7), (k0-7, n8-15), (k8-15, n8-15) ->
// {b0, b1} of tile n0 and of tile n0 + 8.
__device__ __forceinline__ const __nv_bfloat16* b_pair_row(const __nv_bfloat16* M, int ld, int k0, int n0)
{
    const int l = int(lane_id());
    return M + (k0 + (l & 7) + ((l >> 3) & 1) * 8) * ld + n0 + ((l >> 4) & 1) * 8;
}

// Stores a 16 x 64 accumulator of the warp's rows with ReLU, as BF16.
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

// 1 where a stored BF16 activation is > 0 (ReLU outputs are >= 0).
__device__ __forceinline__ float active(uint32_t bits16) { return (bits16 & 0x7fffu) ? 1.0f : 0.0f; }

// One backward step for the warp's 16 rows: D = (A x W) * [Hprev > 0], W a
// row-major [16 KT][64] shared-memory matrix (rows = this layer's outputs),
// D stored as BF16 rows and returned as the next step's A fragments.
template <int KT>
__device__ __forceinline__ void chain_step(const uint32_t (&A)[KT][4], const __nv_bfloat16* W, const __nv_bfloat16* Hprev,
                                           __nv_bfloat16* D, uint32_t (&An)[4][4])
{
    const int gid = int(lane_id() >> 2), tig = int(lane_id() & 3u);
    float C[8][4];
#pragma unroll
    for (int j = 0; j < 8; ++j)
        C[j][0] = C[j][1] = C[j][2] = C[j][3] = 0.0f;
#pragma unroll
    for (int t = 0; t < KT; ++t)
    {
#pragma unroll
        for (int jp = 0; jp < 4; ++jp)
        {
            uint32_t b[4];
            ldsm_x4_t(b, b_pair_row(W, kLdH, 16 * t, 16 * jp));
            uint32_t b0[2] = { b[0], b[1] }, b1[2] = { b[2], b[3] };
            mma_bf16(C[2 * jp], A[t], b0);
            mma_bf16(C[2 * jp + 1], A[t], b1);
        }
    }
#pragma unroll
    for (int j = 0; j < 8; ++j)
    {
        const int col = 8 * j + tig * 2;
        const uint32_t h01 = ld32(Hprev + gid * kLdH + col);
        const uint32_t h23 = ld32(Hprev + (gid + 8) * kLdH + col);
        const uint32_t p01 = pack_bf16(C[j][0] * active(h01), C[j][1] * active(h01 >> 16));
        const uint32_t p23 = pack_bf16(C[j][2] * active(h23), C[j][3] * active(h23 >> 16));
        *reinterpret_cast<uint32_t*>(D + gid * kLdH + col) = p01;
        *reinterpret_cast<uint32_t*>(D + (gid + 8) * kLdH + col) = p23;
        An[j >> 1][(j & 1) * 2 + 0] = p01;
        An[j >> 1][(j & 1) * 2 + 1] = p23;
    }
}

// acc[NT] (16 x 8 tiles of dW at rows m0.., columns n0 + 8 j) += Z^T H over
// the chunk's 128 samples; Z = [128][ldZ] gradients, H = [128][ldH] inputs.
template <int NT>
__device__ __forceinline__ void dw_tiles(float (&acc)[NT][4], const __nv_bfloat16* Z, int ldZ, int m0,
                                         const __nv_bfloat16* H, int ldH, int n0)
{
#pragma unroll 2
    for (int ks = 0; ks < kChunk / 16; ++ks)
    {
        uint32_t a[4];
        ldsm_x4_t(a, a_trans_row(Z, ldZ, 16 * ks, m0));
#pragma unroll
        for (int jp = 0; jp < NT / 2; ++jp)
        {
            uint32_t b[4];
            ldsm_x4_t(b, b_pair_row(H, ldH, 16 * ks, n0 + 16 * jp));
            uint32_t b0[2] = { b[0], b[1] }, b1[2] = { b[2], b[3] };
            mma_bf16(acc[2 * jp], a, b0);
            mma_bf16(acc[2 * jp + 1], a, b1);
        }
    }
}

// The output layer's single tile per warp (rows 0-15 of dW5, columns n0..n0+7).
__device__ __forceinline__ void dw_tile5(float (&acc)[4], const __nv_bfloat16* Z5, const __nv_bfloat16* H4, int n0)
{
    const int l = int(lane_id());
#pragma unroll 2
    for (int ks = 0; ks < kChunk / 16; ++ks)
    {
        uint32_t a[4], b[2];
        ldsm_x4_t(a, a_trans_row(Z5, kLdT, 16 * ks, 0));
        ldsm_x2_t(b, H4 + (16 * ks + (l & 7) + ((l >> 3) & 1) * 8) * kLdH + n0);
        mma_bf16(acc, a, b);
    }
}

// Writes a warp's dW tiles (rows m0 + gid, + 8; columns n0 + 8 j + 2 tig, + 1)
// into the [out][in] gradient g.
template <int NT>
__device__ __forceinline__ void write_tiles(const float (&acc)[NT][4], float* g, int in, int m0, int n0)
{
    const int gid = int(lane_id() >> 2), tig = int(lane_id() & 3u);
#pragma unroll
    for (int j = 0; j < NT; ++j)
    {
        const int c = n0 + 8 * j + tig * 2;
        *reinterpret_cast<float2*>(g + (m0 + gid) * in + c) = make_float2(acc[j][0], acc[j][1]);
        *reinterpret_cast<float2*>(g + (m0 + gid + 8) * in + c) = make_float2(acc[j][2], acc[j][3]);
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

__global__ void __launch_bounds__(kTThreads, 1) k_nrc_train(NrcTrainParams p)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __nv_bfloat16* S = reinterpret_cast<__nv_bfloat16*>(smem);
    __nv_bfloat16* sW = S + kTW;
    load_weights(sW, p.weights);
    // rows 8..15 of the output layer (read by the 16-row B fragments) are zero
    for (int i = threadIdx.x; i < 8 * kLdH; i += blockDim.x)
        sW[kS5 + 8 * kLdH + i] = __float2bfloat16(0.0f);
    __syncthreads();

    const int warp = int(threadIdx.x >> 5);
    const int gid = int(lane_id() >> 2), tig = int(lane_id() & 3u);
    const unsigned total = p.index ? *p.total : unsigned(p.batch);
    const int n = total == 0 ? 0 : p.batch;
    const int chunks = (n + kChunk - 1) / kChunk;
    const float scale = 1.0f / (float(n > 0 ? n : 1) * 3.0f);

    // this warp's dW tiles
    const int mt = warp >> 1;                   // 16-row block of the 64 hidden outputs
    float acc1[8][4], acc2[4][4], acc3[4][4], acc4[4][4], acc5[4];
#pragma unroll
    for (int j = 0; j < 8; ++j)
        acc1[j][0] = acc1[j][1] = acc1[j][2] = acc1[j][3] = 0.0f;
#pragma unroll
    for (int j = 0; j < 4; ++j)
    {
        acc2[j][0] = acc2[j][1] = acc2[j][2] = acc2[j][3] = 0.0f;
        acc3[j][0] = acc3[j][1] = acc3[j][2] = acc3[j][3] = 0.0f;
        acc4[j][0] = acc4[j][1] = acc4[j][2] = acc4[j][3] = 0.0f;
    }
    acc5[0] = acc5[1] = acc5[2] = acc5[3] = 0.0f;
    float lossSum = 0.0f;

    __nv_bfloat16* H0 = S + kTH0;
    __nv_bfloat16* H1 = S + kTH1;
    __nv_bfloat16* H2 = S + kTH2;
    __nv_bfloat16* H3 = S + kTH3;
    __nv_bfloat16* H4 = S + kTH4;
    __nv_bfloat16* ZA = S + kTZA;
    __nv_bfloat16* ZB = S + kTZB;
    __nv_bfloat16* Z5 = S + kTZ5;
    const int rowBase = 16 * warp;  // this warp's rows in the chunk

    for (int chunk = blockIdx.x; chunk < chunks; chunk += gridDim.x)
    {
        // ---- F: forward of the warp's rows
        const int r0 = chunk * kChunk + rowBase + gid, r1 = r0 + 8;
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
        {
            __nv_bfloat16* h0 = H0 + rowBase * kLd1;
#pragma unroll
            for (int t = 0; t < 8; ++t)
            {
                *reinterpret_cast<uint32_t*>(h0 + gid * kLd1 + 16 * t + tig * 2) = A0[t][0];
                *reinterpret_cast<uint32_t*>(h0 + (gid + 8) * kLd1 + 16 * t + tig * 2) = A0[t][1];
                *reinterpret_cast<uint32_t*>(h0 + gid * kLd1 + 16 * t + 8 + tig * 2) = A0[t][2];
                *reinterpret_cast<uint32_t*>(h0 + (gid + 8) * kLd1 + 16 * t + 8 + tig * 2) = A0[t][3];
            }
        }
        uint32_t A[4][4];
        {
            float C[8][4];
            layer_mma<8>(A0, sW + kS1, kLd1, C);
            store_relu(C, H1 + rowBase * kLdH, kLdH);
            relu_pack(C, A);
            layer_mma<4>(A, sW + kS2, kLdH, C);
            store_relu(C, H2 + rowBase * kLdH, kLdH);
            relu_pack(C, A);
            layer_mma<4>(A, sW + kS3, kLdH, C);
            store_relu(C, H3 + rowBase * kLdH, kLdH);
            relu_pack(C, A);
            layer_mma<4>(A, sW + kS4, kLdH, C);
            store_relu(C, H4 + rowBase * kLdH, kLdH);
            relu_pack(C, A);
        }
        float o[4];
        output_mma(A, sW + kS5, o);

        // Relative L2 loss (p - y)^2 / (p^2 + 0.01), mean over batch x 3;
        // the denominator is held constant for the gradient. Output columns
        // (2 tig, 2 tig + 1) of rows gid and gid + 8; only columns 0..2 exist.
        float d[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
#pragma unroll
        for (int e = 0; e < 4; ++e)
        {
            const int c = tig * 2 + (e & 1);
            const bool valid = (e < 2 ? v0 : v1) && c < 3;
            if (!valid)
                continue;
            const int idx = e < 2 ? i0 : i1;
            const float pr = __expf(o[e]);
            const float y = reinterpret_cast<const float*>(&p.rec[idx].d)[c];
            const float den = pr * pr + 0.01f;
            const float diff = pr - y;
            lossSum += diff * diff / den * scale;
            d[e] = 2.0f * diff / den * scale * pr;  // d/dz of exp(z)
        }
        uint32_t A5[1][4];
        A5[0][0] = pack_bf16(d[0], d[1]);
        A5[0][1] = pack_bf16(d[2], d[3]);
        A5[0][2] = 0u;  // columns 8..15
        A5[0][3] = 0u;
        {
            __nv_bfloat16* z5 = Z5 + rowBase * kLdT;
            *reinterpret_cast<uint32_t*>(z5 + gid * kLdT + tig * 2) = A5[0][0];
            *reinterpret_cast<uint32_t*>(z5 + (gid + 8) * kLdT + tig * 2) = A5[0][1];
            *reinterpret_cast<uint32_t*>(z5 + gid * kLdT + 8 + tig * 2) = 0u;
            *reinterpret_cast<uint32_t*>(z5 + (gid + 8) * kLdT + 8 + tig * 2) = 0u;
        }
        __syncthreads();

        // ---- P5
        dw_tile5(acc5, Z5, H4, 8 * warp);
        chain_step<1>(A5, sW + kS5, H4 + rowBase * kLdH, ZA + rowBase * kLdH, A);
        __syncthreads();
        // ---- P4
        dw_tiles<4>(acc4, ZA, kLdH, 16 * mt, H3, kLdH, (warp & 1) * 32);
        chain_step<4>(A, sW + kS4, H3 + rowBase * kLdH, ZB + rowBase * kLdH, A);
        __syncthreads();
        // ---- P3
        dw_tiles<4>(acc3, ZB, kLdH, 16 * mt, H2, kLdH, (warp & 1) * 32);
        chain_step<4>(A, sW + kS3, H2 + rowBase * kLdH, ZA + rowBase * kLdH, A);
        __syncthreads();
        // ---- P2
        dw_tiles<4>(acc2, ZA, kLdH, 16 * mt, H1, kLdH, (warp & 1) * 32);
        chain_step<4>(A, sW + kS2, H1 + rowBase * kLdH, ZB + rowBase * kLdH, A);
        __syncthreads();
        // ---- P1
        dw_tiles<8>(acc1, ZB, kLdH, 16 * mt, H0, kLd1, (warp & 1) * 64);
        __syncthreads();
    }

    float* part = p.partials + size_t(blockIdx.x) * kNrcParams;
    write_tiles<8>(acc1, part + kNrcW1, kNrcIn, 16 * mt, (warp & 1) * 64);
    write_tiles<4>(acc2, part + kNrcW2, kNrcHidden, 16 * mt, (warp & 1) * 32);
    write_tiles<4>(acc3, part + kNrcW3, kNrcHidden, 16 * mt, (warp & 1) * 32);
    write_tiles<4>(acc4, part + kNrcW4, kNrcHidden, 16 * mt, (warp & 1) * 32);
    // dW5: rows 0..7 of the padded output layer (rows 3..7 are zero)
    *reinterpret_cast<float2*>(part + kNrcW5 + gid * kNrcHidden + 8 * warp + tig * 2) = make_float2(acc5[0], acc5[1]);

    for (int off = 16; off > 0; off >>= 1)
        lossSum += __shfl_down_sync(0xffffffffu, lossSum, off);
    __shared__ float sLoss[kTWarps];
    if (lane_id() == 0)
        sLoss[warp] = lossSum;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        float l = 0.0f;
        for (int w = 0; w < kTWarps; ++w)
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
    // eight independent running sums (more loads in flight), combined in a fixed order
    float acc[8] = { 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f };
    int b = 0;
    for (; b + 8 <= p.numPartials; b += 8)
    {
#pragma unroll
        for (int k = 0; k < 8; ++k)
            acc[k] += __ldg(p.partials + size_t(b + k) * kNrcParams + i);
    }
    for (; b < p.numPartials; ++b)
        acc[0] += __ldg(p.partials + size_t(b) * kNrcParams + i);
    const float g = ((acc[0] + acc[1]) + (acc[2] + acc[3])) + ((acc[4] + acc[5]) + (acc[6] + acc[7]));
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

size_t nrc_train_smem() { return size_t(kTEnd) * 2; }

int nrc_train_blocks(int numSMs) { return numSMs; }

cudaError_t launch_nrc_infer(const NrcInferParams& p, int maxRecords, cudaStream_t stream, int numSMs)
{
    static DeviceOnce once;
    static OccupancyCache occ;
    cudaError_t e = once_per_device(once, [] {
        return cudaFuncSetAttribute(k_nrc_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, int(nrc_infer_smem()));
    });
    if (e != cudaSuccess)
        return e;
    const int perSM = blocks_per_sm(k_nrc_infer, kThreads, nrc_infer_smem(), occ);
    int tiles = (maxRecords + 15) / 16;
    int grid = std::max(1, std::min((tiles + kWarps - 1) / kWarps, numSMs * perSM));
    k_nrc_infer<<<grid, kThreads, nrc_infer_smem(), stream>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_nrc_train(const NrcTrainParams& p, int blocks, cudaStream_t stream)
{
    static DeviceOnce once;
    cudaError_t e = once_per_device(once, [] {
        return cudaFuncSetAttribute(k_nrc_train, cudaFuncAttributeMaxDynamicSharedMemorySize, int(nrc_train_smem()));
    });
    if (e != cudaSuccess)
        return e;
    k_nrc_train<<<blocks, kTThreads, nrc_train_smem(), stream>>>(p);
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
