// Radiance-cache inference on the 5th-generation tensor cores: tcgen05.mma
// with the accumulators in tensor memory (TMEM).
//
// One CTA per SM = 32 warps in 8 independent groups of 4 warps. A group
// works on tiles of 128 queries, one query per thread, which is exactly one
// M = 128 tcgen05.mma per 16-wide K step, with its own 16 KB operand buffer,
// 64 TMEM columns, mbarrier and named barrier, so that while some groups
// wait for the tensor core the others encode or run their epilogues:
//   features   thread r encodes features 0..63 of query r into A (128 x 64
//              BF16); the group's first thread issues D = A x W1[:, 0:64]^T
//              and commits it to the group's mbarrier; after the wait the
//              threads encode features 64..127 into A and D += A x
//              W1[:, 64:128]^T (the buffer holds half of the input row, so
//              that eight groups fit in shared memory)
//   layer l    D(TMEM, 128 lanes x 64 FP32 columns) = H x W_l^T; every warp
//              loads its 32 lanes of the previous D (tcgen05.ld), applies
//              ReLU while converting to BF16 and stores row r of H (128 x 64)
//              into A
//   output     W5 padded to 16 rows: D = 128 x 16, columns 0..2 -> exp
// Operands live in shared memory in the canonical K-major layout without
// swizzle: 8 x 8 BF16 core matrices of 128 contiguous bytes (row i at
// 16 i), the core matrices of an 8-row group contiguous along K
// (leading-dimension offset 128 B), 8-row groups 16 K bytes apart
// (stride-dimension offset K * 16 B). The weights are copied once per CTA
// (cp.async) while the first tile is encoded.
//
// Every wait on an mbarrier is bounded: past the bound the group sets
// kNrcTcTimeout in the error word (the caller returns RC_DEVICE_ERROR), waits
// once more (bounded) for its MMAs and leaves its tile loop; the CTA frees
// its TMEM and returns.

#include <cuda_bf16.h>

#include <algorithm>

#include "nrc.cuh"
#include "kernels.h"
#include "nrc_kernels.h"

namespace rcx
{
namespace
{

constexpr int kRows = 128;
constexpr int kGroups = 8;  // independent 4-warp groups per CTA
constexpr int kGroupThreads = 128;
constexpr int kTcThreads = kGroups * kGroupThreads;
constexpr int kHalf = 64;  // input features per layer-0 pass
// shared memory (bytes)
constexpr int kW1Bytes = 64 * 128 * 2;  // N 64 x K 128
constexpr int kWhBytes = 64 * 64 * 2;   // N 64 x K 64
constexpr int kW5Bytes = 16 * 64 * 2;   // N 16 x K 64
constexpr int kABytes = kRows * 64 * 2; // one group's operand: 128 x 64 (half the features, or hidden)
constexpr int kOffW1 = 0;
constexpr int kOffW2 = kOffW1 + kW1Bytes;
constexpr int kOffW5 = kOffW2 + 3 * kWhBytes;
constexpr int kOffA = kOffW5 + kW5Bytes;
constexpr int kOffBar = kOffA + kGroups * kABytes;  // one mbarrier (8 B) per group + the TMEM address (4 B)
// The operands are laid out so that even descriptors read with the leading
// and stride offsets exchanged stay inside this allocation (the largest
// such span, a 128 x 64 operand, ends 895 B past its buffer): 4 KB slack.
constexpr int kTcSmem = kOffBar + 8 * kGroups + 16 + 4096;
constexpr int kTmemCols = kGroups * 64;
static_assert(kTcSmem <= 227 * 1024, "shared memory");
static_assert(kTmemCols <= 512, "tensor memory");
constexpr unsigned kWaitLimit = 1u << 22;  // mbarrier polls before giving up

__device__ __forceinline__ uint32_t sm_addr(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

// Byte offset of element (row, k) in a canonical K-major operand with K columns.
__host__ __device__ constexpr int canon(int row, int k, int K)
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

// Bounded wait for the mbarrier phase `parity` to complete: at most `polls`
// polls (the MMA waits take NrcInferParams::waitPolls; the drain after a wait
// ran out always takes kWaitLimit).
__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity, unsigned polls)
{
    for (unsigned i = 0; i < polls; ++i)
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

// 16 consecutive FP32 columns of this thread's TMEM lane (no wait).
__device__ __forceinline__ void tmem_ld16_nowait(uint32_t taddr, uint32_t* r)
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

// max(a, 0), max(b, 0) rounded to BF16 and packed (a in the low half): the
// ReLU is part of the conversion (cvt.rn.relu).
__device__ __forceinline__ uint32_t relu_pack_bf16(uint32_t a, uint32_t b)
{
    uint32_t d;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;\n" : "=r"(d) : "f"(__uint_as_float(b)), "f"(__uint_as_float(a)));
    return d;
}

// ReLU of 8 FP32 accumulators (as bits) -> 8 BF16.
__device__ __forceinline__ uint4 relu_bf16x8(const uint32_t* r)
{
    uint4 o;
    o.x = relu_pack_bf16(r[0], r[1]);
    o.y = relu_pack_bf16(r[2], r[3]);
    o.z = relu_pack_bf16(r[4], r[5]);
    o.w = relu_pack_bf16(r[6], r[7]);
    return o;
}

// 16-byte asynchronous copy global -> shared (completed by cp.async.wait_all).
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// One [rows][K] matrix of the packed weights (global, BF16) -> its canonical
// K-major tile (shared), by asynchronous copies. Consecutive threads take
// consecutive rows of one 8-column chunk, so that eight of them fill one
// 128-byte core matrix (no bank conflicts).
__device__ __forceinline__ void stage_matrix(unsigned char* dst, const __nv_bfloat16* __restrict__ src, int rows, int K)
{
    const int chunks = rows * K / 8;
    for (int c = int(threadIdx.x); c < chunks; c += int(blockDim.x))
    {
        const int row = c % rows, kc = c / rows;
        cp_async16(sm_addr(dst + canon(row, kc * 8, K)), src + size_t(row) * size_t(K) + size_t(kc) * 8);
    }
}

// Packed [out][in] weights -> canonical tiles; W5 padded to 16 rows with
// zeros. The copies are in flight until cp_async_wait_all.
__device__ void stage_weights(unsigned char* smem, const __nv_bfloat16* __restrict__ w)
{
    stage_matrix(smem + kOffW1, w + kNrcW1, kNrcHidden, kNrcIn);
    for (int l = 0; l < 3; ++l)
        stage_matrix(smem + kOffW2 + l * kWhBytes, w + kNrcW2 + l * kNrcHidden * kNrcHidden, kNrcHidden, kNrcHidden);
    stage_matrix(smem + kOffW5, w + kNrcW5, kNrcOutPad, kNrcHidden);
    for (int c = int(threadIdx.x); c < 8 * kNrcHidden / 8; c += int(blockDim.x))
        *reinterpret_cast<uint4*>(smem + kOffW5 + canon(8 + c % 8, (c / 8) * 8, kNrcHidden)) = make_uint4(0, 0, 0, 0);
}

// Features [64 h, 64 h + 64) of one query, encoded at compile-time feature
// indices (every branch of nrc_feature_pair folds), into row `row` of a
// canonical K = 64 operand.
template <int H>
__device__ __forceinline__ void encode_half(unsigned char* a, int row, const float* q, const NrcBox& box)
{
#pragma unroll
    for (int k = 0; k < kHalf; k += 8)
    {
        uint4 v;
        v.x = nrc_feature_bf16x2(H * kHalf + k + 0, q, box);
        v.y = nrc_feature_bf16x2(H * kHalf + k + 2, q, box);
        v.z = nrc_feature_bf16x2(H * kHalf + k + 4, q, box);
        v.w = nrc_feature_bf16x2(H * kHalf + k + 6, q, box);
        *reinterpret_cast<uint4*>(a + canon(row, k, kHalf)) = v;
    }
}

// The 12 query floats of record r (zeros past the end).
__device__ __forceinline__ void load_query(const NrcInferParams& p, int r, int n, float (&q)[kNrcQueryFloats])
{
    float4 a = make_float4(0.0f, 0.0f, 0.0f, 0.0f), b = a, c = a;
    if (r < n)
    {
        const float4* rp = reinterpret_cast<const float4*>(p.rec + r);
        a = __ldg(rp);
        b = __ldg(rp + 1);
        c = __ldg(rp + 2);
    }
    q[0] = a.x; q[1] = a.y; q[2] = a.z; q[3] = a.w;
    q[4] = b.x; q[5] = b.y; q[6] = b.z; q[7] = b.w;
    q[8] = c.x; q[9] = c.y; q[10] = c.z; q[11] = c.w;
}

// Named barrier over the 128 threads of group g (ids 1..8; 0 is __syncthreads).
__device__ __forceinline__ void group_sync(int g)
{
    asm volatile("bar.sync %0, %1;\n" ::"r"(g + 1), "r"(kGroupThreads) : "memory");
}

// Named barrier that also ANDs a predicate over the group: one decision for
// all of its threads.
__device__ __forceinline__ bool group_all(bool v, int g)
{
    uint32_t r;
    asm volatile(
        "{\n"
        ".reg .pred p, q;\n"
        "setp.ne.u32 p, %1, 0;\n"
        "bar.red.and.pred q, %2, %3, p;\n"
        "selp.u32 %0, 1, 0, q;\n"
        "}\n"
        : "=r"(r)
        : "r"(uint32_t(v)), "r"(g + 1), "r"(kGroupThreads)
        : "memory");
    return r != 0;
}

// Per-group state of the tile loop.
struct Group
{
    int g;            // group index
    int gt;           // thread within the group: row of the tile, TMEM lane
    uint32_t tmem;    // the group's first TMEM column, lane 0
    uint32_t lane0;   // this warp's TMEM lane offset
    uint32_t bar;     // the group's mbarrier
    uint32_t aaddr;   // the group's operand buffer (shared address)
    uint32_t phase;   // parity of the mbarrier phase the next wait is for
    unsigned polls;   // polls per MMA wait
};

// Operands written -> visible to the tensor core, then the group's first
// thread issues K/16 MMAs (accumulating from the first if acc) with B a
// K-chunk range of a canonical tile of bK columns, and commits; returns
// whether the MMAs completed within the bound (the same for the group).
__device__ __forceinline__ bool run_mma(Group& G, uint32_t bbase, int K, int bK, int N, bool acc)
{
    fence_async_smem();
    tc_before_sync();
    group_sync(G.g);
    tc_after_sync();
    if (G.gt == 0)
    {
        const uint32_t idesc = idesc_bf16(kRows, N);
        for (int ks = 0; ks < K / 16; ++ks)
            mma_issue(G.tmem, smem_desc(G.aaddr + uint32_t(ks * 256), K), smem_desc(bbase + uint32_t(ks * 256), bK),
                      idesc, (acc || ks > 0) ? 1 : 0);
        mma_commit(G.bar);
    }
    const bool ok = group_all(bar_wait(G.bar, G.phase, G.polls), G.g);
    G.phase ^= 1u;
    tc_after_sync();
    return ok;
}

// D (64 columns) -> ReLU -> BF16 rows of H in the operand buffer (whose
// previous contents the completed MMAs no longer read).
__device__ __forceinline__ void hidden_epilogue(const Group& G, unsigned char* abuf)
{
#pragma unroll
    for (int cb = 0; cb < kNrcHidden; cb += 32)
    {
        uint32_t v[32];
        tmem_ld16_nowait(G.tmem + G.lane0 + uint32_t(cb), v);
        tmem_ld16_nowait(G.tmem + G.lane0 + uint32_t(cb + 16), v + 16);
        tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < 32; j += 8)
            *reinterpret_cast<uint4*>(abuf + canon(G.gt, cb + j, kNrcHidden)) = relu_bf16x8(v + j);
    }
}

__global__ void __launch_bounds__(kTcThreads, 1) k_nrc_infer_tc(NrcInferParams p, int* errorFlag)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    const int tid = int(threadIdx.x);
    Group G;
    G.g = tid / kGroupThreads;
    G.gt = tid % kGroupThreads;
    G.bar = sm_addr(smem + kOffBar + 8 * G.g);
    G.phase = 0;
    G.polls = p.waitPolls;
    uint32_t* tmemSlot = reinterpret_cast<uint32_t*>(smem + kOffBar + 8 * kGroups);
    stage_weights(smem, p.weights);
    const int n = int(*p.count);
    if (n == 0)
    {
        cp_async_wait_all();
        return;
    }
    if (G.gt == 0)
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(G.bar));
    if (tid < 32)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(sm_addr(tmemSlot)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    unsigned char* abuf = smem + kOffA + G.g * kABytes;
    G.aaddr = sm_addr(abuf);
    const int tiles = (n + kRows - 1) / kRows;
    const int stride = int(gridDim.x) * kGroups;
    int tile = int(blockIdx.x) * kGroups + G.g;
    // the first tile's features 0..63 are encoded while the weights arrive
    float q[kNrcQueryFloats];
    if (tile < tiles)
    {
        load_query(p, tile * kRows + G.gt, n, q);
        encode_half<0>(abuf, G.gt, q, p.box);
    }
    cp_async_wait_all();
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    fence_async_smem();
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    const uint32_t tmemBase = *tmemSlot;
    G.tmem = tmemBase + uint32_t(G.g * kNrcHidden);   // this group's 64 columns
    G.lane0 = uint32_t(((tid >> 5) & 3) * 32) << 16;  // warp w of the group: lanes 32 w .. 32 w + 31

    const uint32_t w1 = sm_addr(smem + kOffW1);
    const uint32_t w2 = sm_addr(smem + kOffW2);
    const uint32_t w5 = sm_addr(smem + kOffW5);
    bool ok = true;
    while (tile < tiles && ok)
    {
        const int r = tile * kRows + G.gt;
        // W1 columns 0..63: K-chunks 0..3 of its K = 128 tile
        ok = run_mma(G, w1, kHalf, kNrcIn, kNrcHidden, false);
        if (!ok)
            break;
        encode_half<1>(abuf, G.gt, q, p.box);
        // W1 columns 64..127: K-chunks 4..7
        ok = run_mma(G, w1 + 4u * 256u, kHalf, kNrcIn, kNrcHidden, true);
        for (int l = 0; l < 3 && ok; ++l)
        {
            hidden_epilogue(G, abuf);
            ok = run_mma(G, w2 + uint32_t(l * kWhBytes), kNrcHidden, kNrcHidden, kNrcHidden, false);
        }
        if (!ok)
            break;
        hidden_epilogue(G, abuf);
        ok = run_mma(G, w5, kNrcHidden, kNrcHidden, 16, false);
        if (!ok)
            break;
        uint32_t v[16];
        tmem_ld16_nowait(G.tmem + G.lane0, v);  // every lane of the warp (a .sync.aligned load)
        tmem_wait_ld();
        if (r < n && p.out)
        {
            p.out[size_t(r) * 3 + 0] = __expf(__uint_as_float(v[0]));
            p.out[size_t(r) * 3 + 1] = __expf(__uint_as_float(v[1]));
            p.out[size_t(r) * 3 + 2] = __expf(__uint_as_float(v[2]));
        }
        else if (r < n)
        {
            const int s = __float_as_int(__ldg(&p.rec[r].d.w));
            const float4 th = p.thr[s];
            float4 re = p.res[s];
            re.x = __fadd_rn(re.x, __fmul_rn(th.x, __expf(__uint_as_float(v[0]))));
            re.y = __fadd_rn(re.y, __fmul_rn(th.y, __expf(__uint_as_float(v[1]))));
            re.z = __fadd_rn(re.z, __fmul_rn(th.z, __expf(__uint_as_float(v[2]))));
            p.res[s] = re;
        }
        // the next tile's encoding overwrites A: every MMA of this tile is complete
        tile += stride;
        if (tile < tiles)
        {
            load_query(p, tile * kRows + G.gt, n, q);
            encode_half<0>(abuf, G.gt, q, p.box);
        }
    }
    if (!ok)
    {
        if (G.gt == 0)
            atomicOr(errorFlag, kNrcTcTimeout);
        // let this group's MMAs still in flight finish before the TMEM is
        // released (run_mma flipped the parity past the phase that ran out)
        bar_wait(G.bar, G.phase ^ 1u, kWaitLimit);
    }
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    if (tid < 32)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmemBase), "r"(kTmemCols));
}

}  // namespace

size_t nrc_infer_tc_smem() { return size_t(kTcSmem); }

cudaError_t launch_nrc_infer_tc(const NrcInferParams& p, int maxRecords, int* errorFlag, cudaStream_t stream,
                                int numSMs)
{
    static DeviceOnce once;
    cudaError_t e = once_per_device(
        once, [] { return cudaFuncSetAttribute(k_nrc_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem); });
    if (e != cudaSuccess)
        return e;
    // one CTA per SM: it allocates all of the SM's TMEM columns
    const int tiles = (maxRecords + kRows - 1) / kRows;
    const int grid = std::max(1, std::min((tiles + kGroups - 1) / kGroups, numSMs));
    k_nrc_infer_tc<<<grid, kTcThreads, kTcSmem, stream>>>(p, errorFlag);
    return cudaGetLastError();
}

}  // namespace rcx
