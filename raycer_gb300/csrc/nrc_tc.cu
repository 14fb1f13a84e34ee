// Radiance-cache inference on the 5th-generation tensor cores: tcgen05.mma
// with the accumulators in tensor memory (TMEM).
//
// One CTA = 4 warps = 128 threads works on tiles of 128 queries, one query
// per thread, which is exactly one M = 128 tcgen05.mma per 16-wide K step:
//   features   thread r encodes query r into A0 (128 x 128 BF16, shared)
//   layer l    thread 0 issues the K/16 MMAs D(TMEM, 128 lanes x 64 FP32
//              columns) = A x W_l^T and commits them to an mbarrier; every
//              warp then loads its 32 lanes of D (tcgen05.ld), applies ReLU,
//              converts to BF16 and stores row r into H (128 x 64, shared),
//              the next layer's A
//   output     W5 padded to 16 rows: D = 128 x 16, columns 0..2 -> exp
// Operands live in shared memory in the canonical K-major layout without
// swizzle: 8 x 8 BF16 core matrices of 128 contiguous bytes (row i at
// 16 i), the core matrices of an 8-row group contiguous along K
// (leading-dimension offset 128 B), 8-row groups 16 K bytes apart
// (stride-dimension offset K * 16 B). Weights are staged once per CTA.
//
// Every wait on the mbarrier is bounded: past the bound the CTA sets
// kNrcTcTimeout in the error word (the caller returns RC_DEVICE_ERROR), waits
// once more (bounded) for its MMAs, frees its TMEM and returns.

#include <cuda_bf16.h>

#include <algorithm>

#include "nrc.cuh"
#include "nrc_kernels.h"

namespace rcx
{
namespace
{

constexpr int kRows = 128;
constexpr int kTcThreads = 128;
// shared memory (bytes)
constexpr int kW1Bytes = 64 * 128 * 2;   // N 64 x K 128
constexpr int kWhBytes = 64 * 64 * 2;    // N 64 x K 64
constexpr int kW5Bytes = 16 * 64 * 2;    // N 16 x K 64
constexpr int kA0Bytes = kRows * 128 * 2;
constexpr int kHBytes = kRows * 64 * 2;
constexpr int kOffW1 = 0;
constexpr int kOffW2 = kOffW1 + kW1Bytes;
constexpr int kOffW3 = kOffW2 + kWhBytes;
constexpr int kOffW4 = kOffW3 + kWhBytes;
constexpr int kOffW5 = kOffW4 + kWhBytes;
constexpr int kOffA0 = kOffW5 + kW5Bytes;
constexpr int kOffH = kOffA0 + kA0Bytes;
constexpr int kOffBar = kOffH + kHBytes;   // mbarrier (8 B) + TMEM address (4 B)
// The operands are laid out so that even descriptors read with the leading
// and stride offsets exchanged stay inside this allocation (the largest
// such span, H read as a 128 x 64 operand, ends 895 B past H): 4 KB slack.
constexpr int kTcSmem = kOffBar + 16 + 4096;
constexpr int kTmemCols = 64;
constexpr unsigned kWaitLimit = 1u << 22;  // mbarrier polls before giving up

__device__ __forceinline__ uint32_t sm_addr(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

// Byte offset of element (row, k) in a canonical K-major operand with K columns.
__device__ __forceinline__ int canon(int row, int k, int K)
{
    return (row >> 3) * (K * 16) + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

// Shared-memory matrix descriptor: start address, leading-dimension offset
// 128 B (between core matrices along K), stride-dimension offset K * 16 B
// (between 8-row groups), the fixed 0b001 at bits 46-48, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, int K)
{
    return uint64_t((addr & 0x3FFFFu) >> 4) | (uint64_t(128 >> 4) << 16) | (uint64_t((K * 16) >> 4) << 32) |
           (uint64_t(1) << 46);
}

// Instruction descriptor, kind::f16: FP32 D, BF16 A and B, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}

__device__ __forceinline__ void mma_issue(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, int acc)
{
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "setp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
        "}\n" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar));
}

// Bounded wait for the mbarrier phase `parity` to complete.
__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity)
{
    for (unsigned i = 0; i < kWaitLimit; ++i)
    {
        uint32_t done;
        asm volatile(
            "{\n"
            ".reg .pred p;\n"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.u32 %0, 1, 0, p;\n"
            "}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity));
        if (done)
            return true;
    }
    return false;
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
__device__ __forceinline__ void tc_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i)
        v[i] = __uint_as_float(r[i]);
}

// Packed [out][in] weights (global) -> canonical K-major tiles (shared);
// W5 padded to 16 rows with zeros.
__device__ void stage_weights(unsigned char* smem, const __nv_bfloat16* __restrict__ w)
{
    const uint4* src = reinterpret_cast<const uint4*>(w);
    // 8-element chunks: W1 1024, W2..W4 512 each, W5 rows 0..7 -> 64
    for (int c = threadIdx.x; c < kNrcParamCount / 8; c += blockDim.x)
    {
        const int i = c * 8;
        int off;
        if (i < kNrcW2)
            off = kOffW1 + canon(i / kNrcIn, i % kNrcIn, kNrcIn);
        else if (i < kNrcW5)
        {
            const int l = (i - kNrcW2) / (kNrcHidden * kNrcHidden);
            const int r = (i - kNrcW2) % (kNrcHidden * kNrcHidden);
            off = kOffW2 + l * kWhBytes + canon(r / kNrcHidden, r % kNrcHidden, kNrcHidden);
        }
        else
            off = kOffW5 + canon((i - kNrcW5) / kNrcHidden, (i - kNrcW5) % kNrcHidden, kNrcHidden);
        *reinterpret_cast<uint4*>(smem + off) = __ldg(src + c);
    }
    // rows 8..15 of W5
    for (int c = threadIdx.x; c < 8 * kNrcHidden / 8; c += blockDim.x)
        *reinterpret_cast<uint4*>(smem + kOffW5 + canon(8 + c / 8, (c % 8) * 8, kNrcHidden)) = make_uint4(0, 0, 0, 0);
}

__global__ void __launch_bounds__(kTcThreads) k_nrc_infer_tc(NrcInferParams p, int* errorFlag)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    const int tid = int(threadIdx.x);
    const int warp = tid >> 5;
    const uint32_t bar = sm_addr(smem + kOffBar);
    uint32_t* tmemSlot = reinterpret_cast<uint32_t*>(smem + kOffBar + 8);
    const int n = int(*p.count);
    if (n == 0)
        return;

    stage_weights(smem, p.weights);
    if (tid == 0)
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar));
    if (warp == 0)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(sm_addr(tmemSlot)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    fence_async_smem();
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    const uint32_t tmem = *tmemSlot;
    const uint32_t lane0 = uint32_t(warp * 32) << 16;  // this warp's TMEM lanes

    const uint32_t a0 = sm_addr(smem + kOffA0);
    const uint32_t hb = sm_addr(smem + kOffH);
    const uint32_t w1 = sm_addr(smem + kOffW1);
    const uint32_t w5 = sm_addr(smem + kOffW5);
    uint32_t phase = 0;
    bool ok = true;
    const int tiles = (n + kRows - 1) / kRows;
    for (int tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x)
    {
        const int r = tile * kRows + tid;
        float q[kNrcQueryFloats];
        if (r < n)
        {
            const float4* rp = reinterpret_cast<const float4*>(p.rec + r);
            const float4 a = __ldg(rp), b = __ldg(rp + 1), c = __ldg(rp + 2);
            q[0] = a.x; q[1] = a.y; q[2] = a.z; q[3] = a.w;
            q[4] = b.x; q[5] = b.y; q[6] = b.z; q[7] = b.w;
            q[8] = c.x; q[9] = c.y; q[10] = c.z; q[11] = c.w;
        }
        else
        {
#pragma unroll
            for (int k = 0; k < kNrcQueryFloats; ++k)
                q[k] = 0.0f;
        }
        for (int k = 0; k < kNrcIn; k += 8)
        {
            uint4 v;
            v.x = pack_bf16(nrc_feature(k + 0, q, p.box), nrc_feature(k + 1, q, p.box));
            v.y = pack_bf16(nrc_feature(k + 2, q, p.box), nrc_feature(k + 3, q, p.box));
            v.z = pack_bf16(nrc_feature(k + 4, q, p.box), nrc_feature(k + 5, q, p.box));
            v.w = pack_bf16(nrc_feature(k + 6, q, p.box), nrc_feature(k + 7, q, p.box));
            *reinterpret_cast<uint4*>(smem + kOffA0 + canon(tid, k, kNrcIn)) = v;
        }
        for (int layer = 0; layer < 5 && ok; ++layer)
        {
            // operands written by the threads -> visible to the tensor core
            fence_async_smem();
            tc_before_sync();
            __syncthreads();
            tc_after_sync();
            const int K = layer == 0 ? kNrcIn : kNrcHidden;
            const int N = layer == 4 ? 16 : kNrcHidden;
            if (tid == 0)
            {
                const uint32_t abase = layer == 0 ? a0 : hb;
                const uint32_t bbase = layer == 0 ? w1 : (layer == 4 ? w5 : w1 + uint32_t(kOffW2 + (layer - 1) * kWhBytes));
                const uint32_t idesc = idesc_bf16(kRows, N);
                for (int ks = 0; ks < K / 16; ++ks)
                    mma_issue(tmem, smem_desc(abase + uint32_t(ks * 256), K), smem_desc(bbase + uint32_t(ks * 256), K),
                              idesc, ks > 0 ? 1 : 0);
                mma_commit(bar);
            }
            // one decision for the whole CTA (the loop has barriers)
            ok = __syncthreads_and(bar_wait(bar, phase) ? 1 : 0) != 0;
            phase ^= 1u;
            tc_after_sync();
            if (!ok)
                break;
            if (layer < 4)
            {
#pragma unroll
                for (int cb = 0; cb < kNrcHidden; cb += 16)
                {
                    float v[16];
                    tmem_ld16(tmem + lane0 + uint32_t(cb), v);
                    uint4 lo, hi;
                    lo.x = pack_bf16(fmaxf(v[0], 0.0f), fmaxf(v[1], 0.0f));
                    lo.y = pack_bf16(fmaxf(v[2], 0.0f), fmaxf(v[3], 0.0f));
                    lo.z = pack_bf16(fmaxf(v[4], 0.0f), fmaxf(v[5], 0.0f));
                    lo.w = pack_bf16(fmaxf(v[6], 0.0f), fmaxf(v[7], 0.0f));
                    hi.x = pack_bf16(fmaxf(v[8], 0.0f), fmaxf(v[9], 0.0f));
                    hi.y = pack_bf16(fmaxf(v[10], 0.0f), fmaxf(v[11], 0.0f));
                    hi.z = pack_bf16(fmaxf(v[12], 0.0f), fmaxf(v[13], 0.0f));
                    hi.w = pack_bf16(fmaxf(v[14], 0.0f), fmaxf(v[15], 0.0f));
                    *reinterpret_cast<uint4*>(smem + kOffH + canon(tid, cb, kNrcHidden)) = lo;
                    *reinterpret_cast<uint4*>(smem + kOffH + canon(tid, cb + 8, kNrcHidden)) = hi;
                }
            }
            else
            {
                float v[16];
                tmem_ld16(tmem + lane0, v);  // every lane of the warp (a .sync.aligned load)
                if (r < n && p.out)
                {
                    p.out[size_t(r) * 3 + 0] = __expf(v[0]);
                    p.out[size_t(r) * 3 + 1] = __expf(v[1]);
                    p.out[size_t(r) * 3 + 2] = __expf(v[2]);
                }
                else if (r < n)
                {
                    const int s = __float_as_int(__ldg(&p.rec[r].d.w));
                    const float4 th = p.thr[s];
                    float4 re = p.res[s];
                    re.x = __fadd_rn(re.x, __fmul_rn(th.x, __expf(v[0])));
                    re.y = __fadd_rn(re.y, __fmul_rn(th.y, __expf(v[1])));
                    re.z = __fadd_rn(re.z, __fmul_rn(th.z, __expf(v[2])));
                    p.res[s] = re;
                }
            }
        }
        // every thread agrees on ok (the same mbarrier), so the loop ends together
    }
    if (!ok)
    {
        if (tid == 0)
            atomicOr(errorFlag, kNrcTcTimeout);
        // let any MMA still in flight finish before the TMEM is released
        bar_wait(bar, phase);
    }
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemCols));
}

}  // namespace

size_t nrc_infer_tc_smem() { return size_t(kTcSmem); }

cudaError_t launch_nrc_infer_tc(const NrcInferParams& p, int maxRecords, int* errorFlag, cudaStream_t stream,
                                int numSMs)
{
    static int perSM = 0;
    if (perSM == 0)
    {
        cudaError_t e = cudaFuncSetAttribute(k_nrc_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
        if (e != cudaSuccess)
            return e;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_nrc_infer_tc, kTcThreads, kTcSmem) !=
                cudaSuccess ||
            perSM < 1)
            perSM = 1;
    }
    const int tiles = (maxRecords + kRows - 1) / kRows;
    const int grid = std::max(1, std::min(tiles, numSMs * perSM));
    k_nrc_infer_tc<<<grid, kTcThreads, kTcSmem, stream>>>(p, errorFlag);
    return cudaGetLastError();
}

}  // namespace rcx
