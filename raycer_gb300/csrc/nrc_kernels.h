// Launchers and parameter blocks of the neural radiance cache kernels
// (nrc.cu). Host-includable: no device code.
//
// Records: every query, training sample and cache lookup is one 16-float
// record (NrcRecord): floats 0..11 are the query of nrc.cuh (position,
// direction, normal, albedo), floats 12..14 the radiance (training target,
// or the bounce factor while a training path is in flight), float 15 a
// 32-bit tag (the path slot of a cache lookup).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace rcx
{

struct NrcBox
{
    float lo[3];
    float inv[3];  // 1 / size
};

struct NrcRecord
{
    float4 a;  // x, y, z, wx
    float4 b;  // wy, wz, nx, ny
    float4 c;  // nz, rho r, rho g, rho b
    float4 d;  // radiance r, g, b, tag
};

constexpr int kNrcParamCount = 20992;  // packed [out][in] weights of the five layers (nrc.cuh)
constexpr int kNrcIn = 128;            // encoded inputs
constexpr int kNrcQueryFloats = 12;    // floats of a query

struct NrcInferParams
{
    const __nv_bfloat16* weights;
    const NrcRecord* rec;
    const unsigned* count;   // device: number of records
    float* out;              // rgb per record (out != nullptr), or:
    const float4* thr;       // res[tag] += thr[tag] * cache (out == nullptr)
    float4* res;
    NrcBox box;
    unsigned waitPolls;      // tcgen05 kernel: polls per bounded MMA wait (0: give up at once)
};

// Polls per bounded mbarrier wait of a configuration's tc_wait_polls.
inline unsigned nrc_wait_polls(int32_t configured)
{
    return configured == 0 ? (1u << 22) : configured < 0 ? 0u : unsigned(configured);
}

struct NrcTrainParams
{
    const __nv_bfloat16* weights;
    const NrcRecord* rec;
    const int* index;        // sample r of the step is rec[index[hash(key, r) % *total]]
    const unsigned* total;   //   (index != nullptr), else rec[first + r] for r < batch
    uint32_t key;
    int first;
    int batch;
    NrcBox box;
    float* partials;         // [blocks][kNrcParamCount] weight-gradient sums
    float* lossPartials;     // [blocks]
};

struct NrcAdamParams
{
    const float* partials;
    const float* lossPartials;
    int numPartials;
    const unsigned* total;   // skip the update when *total == 0 (total != nullptr)
    float* gradOut;          // summed gradient (optional)
    float* loss;             // summed loss (device scalar)
    int adam;                // 0: only sum
    float lr, beta1, beta2, eps;
    float beta1Pow, beta2Pow;  // beta^t of this step (t >= 1)
    float* master;
    float* m;
    float* v;
    __nv_bfloat16* weights;
};

// Error-word bit set by the tcgen05 kernel when an mbarrier wait ran out.
constexpr int kNrcTcTimeout = 2;

size_t nrc_train_smem();
int nrc_train_blocks(int numSMs);
cudaError_t launch_nrc_infer(const NrcInferParams& p, int maxRecords, cudaStream_t stream, int numSMs);
// The same lookups with tcgen05.mma / TMEM (nrc_tc.cu), 128 queries per tile.
cudaError_t launch_nrc_infer_tc(const NrcInferParams& p, int maxRecords, int* errorWord, cudaStream_t stream,
                                int numSMs);
cudaError_t launch_nrc_train(const NrcTrainParams& p, int blocks, cudaStream_t stream);
cudaError_t launch_nrc_adam(const NrcAdamParams& p, cudaStream_t stream);
// BF16 input features of n records ([n][128]), for tests of the encoding.
cudaError_t launch_nrc_encode(const NrcRecord* rec, int n, const NrcBox& box, __nv_bfloat16* out,
                              cudaStream_t stream);
// FP32 master weights -> BF16 copy.
cudaError_t launch_nrc_to_bf16(const float* master, __nv_bfloat16* out, cudaStream_t stream);

}  // namespace rcx
