// Host side of the neural radiance cache: the rc_nrc_* entry points and the
// per-pass cache work of a PATH render (see nrc_kernels.h / nrc.cu for the
// network and pathtrace.cu for the lookups and training paths).
//
// Per render pass, in stream order:
//   generate, extend/shade segments   training paths record their vertices,
//                                     other paths queue a lookup at the hit
//                                     of segment terminate_segment
//   k_nrc_infer                       res[slot] += thr[slot] * cache(query)
//   accumulate                        film update
//   k_nrc_targets                     suffix radiance per training vertex
//   train_steps x (k_nrc_train, k_nrc_adam)
// The lookups use the weights trained up to the previous pass.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "host_internal.h"
#include "pathtrace.h"

using namespace rcx;

namespace
{

constexpr int64_t kApiMax = int64_t(1) << 20;

rc_status fail(rc_tracer* h, rc_status s, const std::string& msg)
{
    h->err = msg;
    return s;
}

rc_status cuda_fail(rc_tracer* h, cudaError_t e, const char* what)
{
    std::string msg = std::string("nrc: ") + what + ": " + cudaGetErrorString(e);
    return fail(h, e == cudaErrorMemoryAllocation ? RC_OOM : RC_CUDA, msg);
}

#define NRC_TRY(h, expr, what)                 \
    do                                         \
    {                                          \
        cudaError_t e_ = (expr);               \
        if (e_ != cudaSuccess)                 \
            return cuda_fail((h), e_, (what)); \
    } while (0)

#define NRC_STATUS(expr)           \
    do                             \
    {                              \
        rc_status s_ = (expr);     \
        if (s_ != RC_OK)           \
            return s_;             \
    } while (0)

// lowbias32 (C. Wellons), for the per-pass and per-step keys.
uint32_t mix32(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

uint64_t splitmix64(uint64_t& state)
{
    uint64_t z = (state += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

// He-uniform weights: U(-sqrt(6 / fan_in), +sqrt(6 / fan_in)); the output
// layer's padding rows 3..7 are zero.
std::vector<float> init_weights(uint64_t seed)
{
    std::vector<float> w(kNrcParamCount, 0.0f);
    uint64_t st = seed ^ 0x2545f4914f6cdd1dull;
    auto fill = [&](int offset, int rows, int cols) {
        const double lim = std::sqrt(6.0 / double(cols));
        for (int i = 0; i < rows * cols; ++i)
        {
            double u = double(splitmix64(st) >> 11) * (1.0 / 9007199254740992.0);
            w[size_t(offset + i)] = float((2.0 * u - 1.0) * lim);
        }
    };
    fill(0, 64, 128);
    fill(8192, 64, 64);
    fill(12288, 64, 64);
    fill(16384, 64, 64);
    fill(20480, 3, 64);
    return w;
}

rc_status alloc_state(rc_tracer* h)
{
    NrcState& n = h->nrc;
    if (n.dMaster)
        return RC_OK;
    const size_t P = kNrcParamCount;
    n.blocks = nrc_train_blocks(h->numSMs);
    void* p = nullptr;
    size_t cap = 0;
    NRC_STATUS(device_grow(h, &p, &cap, P * 4 * 3 + P * 2, "allocate weights"));
    n.dMaster = static_cast<float*>(p);
    n.dM = n.dMaster + P;
    n.dV = n.dM + P;
    n.dW = reinterpret_cast<__nv_bfloat16*>(n.dV + P);
    p = nullptr;
    cap = 0;
    NRC_STATUS(device_grow(h, &p, &cap, size_t(n.blocks) * P * 4 + size_t(n.blocks) * 4 + P * 4 + 64,
                           "allocate gradient partials"));
    n.dPartials = static_cast<float*>(p);
    n.dLossPartials = n.dPartials + size_t(n.blocks) * P;
    n.dGrad = n.dLossPartials + n.blocks;
    n.dCounters = reinterpret_cast<unsigned*>(n.dGrad + P);
    NRC_TRY(h, cudaEventCreate(&n.evTrain0), "create event");
    NRC_TRY(h, cudaEventCreate(&n.evTrain1), "create event");
    return RC_OK;
}

rc_status upload_weights(rc_tracer* h, const float* w)
{
    NrcState& n = h->nrc;
    const size_t bytes = size_t(kNrcParamCount) * 4;
    NRC_TRY(h, cudaMemcpyAsync(n.dMaster, w, bytes, cudaMemcpyHostToDevice, h->stream), "upload weights");
    NRC_TRY(h, cudaMemsetAsync(n.dM, 0, 2 * bytes, h->stream), "reset optimizer");
    NRC_TRY(h, launch_nrc_to_bf16(n.dMaster, n.dW, h->stream), "convert weights");
    NRC_TRY(h, cudaStreamSynchronize(h->stream), "upload weights");
    n.steps = 0;
    return RC_OK;
}

rc_status loss_buffer(rc_tracer* h, int steps)
{
    void* p = h->nrc.dLoss;
    size_t cap = h->nrc.capLoss;
    rc_status s = device_grow(h, &p, &cap, size_t(std::max(steps, 1)) * 4, "allocate loss buffer");
    h->nrc.dLoss = static_cast<float*>(p);
    h->nrc.capLoss = cap;
    return s;
}

bool valid_box(const rc_nrc_config& c)
{
    for (int k = 0; k < 3; ++k)
        if (!(c.box_max[k] > c.box_min[k]))
            return false;
    return true;
}

// Encoding box: the configured one, else the scene's root bounds.
rc_status encoding_box(rc_tracer* h, NrcBox& box)
{
    const rc_nrc_config& c = h->nrc.cfg;
    double lo[3], hi[3];
    if (valid_box(c))
    {
        for (int k = 0; k < 3; ++k)
        {
            lo[k] = c.box_min[k];
            hi[k] = c.box_max[k];
        }
    }
    else
    {
        if (!h->sceneReady)
            return fail(h, RC_NOT_READY, "nrc: no encoding box configured and no scene bounds");
        for (int k = 0; k < 3; ++k)
        {
            lo[k] = h->bounds[k];
            hi[k] = h->bounds[3 + k];
            if (!(hi[k] > lo[k]))
                hi[k] = lo[k] + 1.0;
        }
    }
    for (int k = 0; k < 3; ++k)
    {
        box.lo[k] = float(lo[k]);
        box.inv[k] = float(1.0 / (hi[k] - lo[k]));
    }
    return RC_OK;
}

rc_status check_ready(rc_tracer* h, const char* what)
{
    if (!h->nrc.configured)
        return fail(h, RC_NOT_READY, std::string(what) + ": rc_nrc_configure has not been called");
    return RC_OK;
}

// Host queries (+ targets) -> device records.
rc_status upload_records(rc_tracer* h, const float* queries, const float* targets, int64_t n)
{
    NrcState& st = h->nrc;
    NRC_STATUS(device_grow(h, &st.dApi, &st.capApi, size_t(n) * sizeof(NrcRecord), "allocate records"));
    std::vector<float> rec(size_t(n) * 16, 0.0f);
    for (int64_t i = 0; i < n; ++i)
    {
        std::memcpy(&rec[size_t(i) * 16], queries + i * kNrcQueryFloats, kNrcQueryFloats * sizeof(float));
        if (targets)
            std::memcpy(&rec[size_t(i) * 16 + 12], targets + i * 3, 3 * sizeof(float));
    }
    NRC_TRY(h, cudaMemcpyAsync(st.dApi, rec.data(), rec.size() * sizeof(float), cudaMemcpyHostToDevice, h->stream),
            "upload records");
    // the host copy must outlive the copy
    NRC_TRY(h, cudaStreamSynchronize(h->stream), "upload records");
    return RC_OK;
}

NrcAdamParams adam_params(rc_tracer* h, int adam, const unsigned* total, float* lossOut)
{
    NrcState& n = h->nrc;
    NrcAdamParams a{};
    a.partials = n.dPartials;
    a.lossPartials = n.dLossPartials;
    a.numPartials = n.blocks;
    a.total = total;
    a.gradOut = adam ? nullptr : n.dGrad;
    a.loss = lossOut;
    a.adam = adam;
    a.lr = n.cfg.learning_rate;
    a.beta1 = n.cfg.beta1;
    a.beta2 = n.cfg.beta2;
    a.eps = n.cfg.epsilon;
    if (adam)
    {
        n.steps++;
        a.beta1Pow = float(std::pow(double(n.cfg.beta1), double(n.steps)));
        a.beta2Pow = float(std::pow(double(n.cfg.beta2), double(n.steps)));
    }
    a.master = n.dMaster;
    a.m = n.dM;
    a.v = n.dV;
    a.weights = n.dW;
    return a;
}

}  // namespace

namespace rcx
{

bool nrc_active(const rc_tracer* h) { return h->nrc.configured && h->nrc.cfg.enabled != 0; }

rc_status nrc_prepare(rc_tracer* h, uint64_t slots, int segments)
{
    NrcState& n = h->nrc;
    const uint64_t stride = uint64_t(std::max(n.cfg.train_stride, 1));
    const uint64_t groups = (slots + stride - 1) / stride;
    const uint64_t segs = uint64_t(std::max(segments, 1));
    NRC_STATUS(device_grow(h, &n.dQuery, &n.capQuery, size_t(slots) * sizeof(NrcRecord), "allocate lookups"));
    NRC_STATUS(device_grow(h, &n.dVtx, &n.capVtx, size_t(segs * groups) * sizeof(NrcRecord),
                           "allocate training vertices"));
    NRC_STATUS(device_grow(h, &n.dTerm, &n.capTerm, size_t(groups) * sizeof(float4), "allocate training ends"));
    NRC_STATUS(device_grow(h, &n.dIndex, &n.capIndex, size_t(segs * groups) * sizeof(int),
                           "allocate sample index"));
    NRC_STATUS(loss_buffer(h, n.cfg.train_steps));
    n.trainMs = 0.0;
    return RC_OK;
}

void nrc_pass_state(rc_tracer* h, PassParams& pp, uint32_t passIndex)
{
    NrcState& n = h->nrc;
    NrcPass& q = pp.nrc;
    q.query = static_cast<NrcRecord*>(n.dQuery);
    q.vtx = static_cast<NrcRecord*>(n.dVtx);
    q.term = static_cast<float4*>(n.dTerm);
    q.index = static_cast<int*>(n.dIndex);
    q.counters = n.dCounters;
    q.termSegment = n.cfg.terminate_segment;
    q.trainStride = std::max(n.cfg.train_stride, 1);
    q.groups = int((uint64_t(pp.nslots) + uint64_t(q.trainStride) - 1) / uint64_t(q.trainStride));
    q.minSuffix = n.cfg.min_suffix;
    q.lookupVertexOnly = n.cfg.sample_vertices == RC_NRC_LOOKUP_VERTEX ? 1 : 0;
    q.trainKey = mix32(mix32(mix32(uint32_t(n.cfg.seed) ^ 0x4e524331u) ^ uint32_t(n.cfg.seed >> 32) ^ h->frameIndex) ^
                       passIndex);
}

rc_status nrc_lookups(rc_tracer* h, const PassParams& pp)
{
    NrcState& n = h->nrc;
    NrcInferParams ip{};
    ip.weights = n.dW;
    ip.rec = pp.nrc.query;
    ip.count = n.dCounters;
    ip.waitPolls = nrc_wait_polls(n.cfg.tc_wait_polls);
    ip.out = nullptr;
    ip.thr = pp.thr;
    ip.res = pp.res;
    NRC_STATUS(encoding_box(h, ip.box));
    if (n.cfg.lookup_kernel == RC_NRC_TCGEN05)
        NRC_TRY(h, launch_nrc_infer_tc(ip, pp.nslots, &pp.ctl->error, h->stream, h->numSMs), "launch cache lookups");
    else
        NRC_TRY(h, launch_nrc_infer(ip, pp.nslots, h->stream, h->numSMs), "launch cache lookups");
    return RC_OK;
}

rc_status nrc_train_pass(rc_tracer* h, const PassParams& pp)
{
    NrcState& n = h->nrc;
    NRC_TRY(h, cudaEventRecord(n.evTrain0, h->stream), "record event");
    NRC_TRY(h, launch_nrc_targets(pp, h->stream), "launch training targets");
    NrcTrainParams tp{};
    tp.weights = n.dW;
    tp.rec = pp.nrc.vtx;
    tp.index = pp.nrc.index;
    tp.total = n.dCounters + 1;
    tp.batch = n.cfg.train_batch;
    tp.partials = n.dPartials;
    tp.lossPartials = n.dLossPartials;
    NRC_STATUS(encoding_box(h, tp.box));
    for (int step = 0; step < n.cfg.train_steps; ++step)
    {
        tp.key = mix32(pp.nrc.trainKey ^ mix32(uint32_t(step) * 0x85ebca6bu + 1u));
        NRC_TRY(h, launch_nrc_train(tp, n.blocks, h->stream), "launch training step");
        NrcAdamParams a = adam_params(h, 1, n.dCounters + 1, n.dLoss + step);
        NRC_TRY(h, launch_nrc_adam(a, h->stream), "launch optimizer step");
    }
    NRC_TRY(h, cudaEventRecord(n.evTrain1, h->stream), "record event");
    n.lastSteps = n.cfg.train_steps;
    n.passes++;
    return RC_OK;
}

void nrc_release(rc_tracer* h)
{
    NrcState& n = h->nrc;
    void* ptrs[] = { n.dMaster, n.dPartials, n.dLoss, n.dQuery, n.dVtx, n.dTerm, n.dIndex, n.dApi, n.dApiOut };
    for (void* p : ptrs)
        if (p)
            cudaFree(p);
    if (n.evTrain0)
        cudaEventDestroy(n.evTrain0);
    if (n.evTrain1)
        cudaEventDestroy(n.evTrain1);
    n = NrcState{};
}

}  // namespace rcx

extern "C" {

rc_status rc_nrc_defaults(rc_nrc_config* c)
{
    if (!c)
        return RC_INVALID_ARG;
    std::memset(c, 0, sizeof(*c));
    c->enabled = 1;
    c->terminate_segment = 2;
    c->train_stride = 16;
    c->train_steps = 4;
    c->train_batch = 16384;
    c->min_suffix = 3;
    c->learning_rate = 1e-2f;
    c->beta1 = 0.9f;
    c->beta2 = 0.99f;
    c->epsilon = 1e-8f;
    c->seed = 1;
    c->lookup_kernel = RC_NRC_TCGEN05;
    c->sample_vertices = RC_NRC_LOOKUP_VERTEX;
    return RC_OK;
}

rc_status rc_nrc_configure(rc_tracer* h, const rc_nrc_config* c)
{
    if (!h)
        return RC_INVALID_ARG;
    if (!c)
        return fail(h, RC_INVALID_ARG, "nrc_configure: null config");
    if (c->terminate_segment < 0 || c->train_stride < 1 || c->train_steps < 0 || c->train_batch < 1 ||
        c->train_batch > kApiMax || c->min_suffix < 1)
        return fail(h, RC_INVALID_ARG, "nrc_configure: terminate_segment / train_* / min_suffix out of range");
    if (!(c->learning_rate > 0.0f) || !(c->beta1 >= 0.0f && c->beta1 < 1.0f) || !(c->beta2 >= 0.0f && c->beta2 < 1.0f) ||
        !(c->epsilon > 0.0f))
        return fail(h, RC_INVALID_ARG, "nrc_configure: invalid optimizer settings");
    if (c->lookup_kernel != RC_NRC_MMA_SYNC && c->lookup_kernel != RC_NRC_TCGEN05)
        return fail(h, RC_INVALID_ARG, "nrc_configure: unknown lookup kernel");
    if ((c->sample_vertices != RC_NRC_ALL_VERTICES && c->sample_vertices != RC_NRC_LOOKUP_VERTEX) || c->reserved != 0)
        return fail(h, RC_INVALID_ARG, "nrc_configure: unknown sample_vertices / reserved not 0");
    cudaSetDevice(h->device);
    h->nrc.cfg = *c;
    NRC_STATUS(alloc_state(h));
    std::vector<float> w = init_weights(c->seed);
    NRC_STATUS(upload_weights(h, w.data()));
    h->nrc.configured = true;
    h->nrc.passes = 0;
    return RC_OK;
}

rc_status rc_nrc_set_enabled(rc_tracer* h, int32_t enabled)
{
    if (!h)
        return RC_INVALID_ARG;
    NRC_STATUS(check_ready(h, "nrc_set_enabled"));
    h->nrc.cfg.enabled = enabled ? 1 : 0;
    return RC_OK;
}

rc_status rc_nrc_get_params(rc_tracer* h, float* params, int64_t count)
{
    if (!h)
        return RC_INVALID_ARG;
    NRC_STATUS(check_ready(h, "nrc_get_params"));
    if (!params || count != kNrcParamCount)
        return fail(h, RC_INVALID_ARG, "nrc_get_params: need RC_NRC_PARAMS floats");
    cudaSetDevice(h->device);
    NRC_TRY(h, cudaMemcpyAsync(params, h->nrc.dMaster, size_t(count) * 4, cudaMemcpyDeviceToHost, h->stream),
            "download weights");
    NRC_TRY(h, cudaStreamSynchronize(h->stream), "download weights");
    return RC_OK;
}

rc_status rc_nrc_set_params(rc_tracer* h, const float* params, int64_t count)
{
    if (!h)
        return RC_INVALID_ARG;
    NRC_STATUS(check_ready(h, "nrc_set_params"));
    if (!params || count != kNrcParamCount)
        return fail(h, RC_INVALID_ARG, "nrc_set_params: need RC_NRC_PARAMS floats");
    for (int i = 20480 + 3 * 64; i < kNrcParamCount; ++i)
        if (params[i] != 0.0f)
            return fail(h, RC_INVALID_ARG, "nrc_set_params: output padding rows 3..7 must be zero");
    cudaSetDevice(h->device);
    return upload_weights(h, params);
}

rc_status rc_nrc_infer(rc_tracer* h, const float* queries, int64_t n, float* rgb)
{
    if (!h)
        return RC_INVALID_ARG;
    NRC_STATUS(check_ready(h, "nrc_infer"));
    if (!queries || !rgb || n <= 0 || n > kApiMax)
        return fail(h, RC_INVALID_ARG, "nrc_infer: null buffer or n outside [1, 2^20]");
    cudaSetDevice(h->device);
    NrcState& st = h->nrc;
    NRC_STATUS(upload_records(h, queries, nullptr, n));
    NRC_STATUS(device_grow(h, &st.dApiOut, &st.capApiOut, size_t(n) * 3 * 4, "allocate outputs"));
    unsigned cnt = unsigned(n);
    NRC_TRY(h, cudaMemcpyAsync(st.dCounters + 2, &cnt, 4, cudaMemcpyHostToDevice, h->stream), "upload count");
    NrcInferParams ip{};
    ip.weights = st.dW;
    ip.rec = static_cast<const NrcRecord*>(st.dApi);
    ip.count = st.dCounters + 2;
    ip.waitPolls = nrc_wait_polls(st.cfg.tc_wait_polls);
    ip.out = static_cast<float*>(st.dApiOut);
    NRC_STATUS(encoding_box(h, ip.box));
    int errWord = 0;
    if (st.cfg.lookup_kernel == RC_NRC_TCGEN05)
    {
        NRC_TRY(h, cudaMemsetAsync(st.dCounters + 3, 0, sizeof(unsigned), h->stream), "reset error word");
        NRC_TRY(h, launch_nrc_infer_tc(ip, int(n), reinterpret_cast<int*>(st.dCounters + 3), h->stream, h->numSMs),
                "launch inference");
        NRC_TRY(h, cudaMemcpyAsync(&errWord, st.dCounters + 3, sizeof(int), cudaMemcpyDeviceToHost, h->stream),
                "read error word");
    }
    else
        NRC_TRY(h, launch_nrc_infer(ip, int(n), h->stream, h->numSMs), "launch inference");
    NRC_TRY(h, cudaMemcpyAsync(rgb, st.dApiOut, size_t(n) * 3 * 4, cudaMemcpyDeviceToHost, h->stream),
            "download outputs");
    NRC_TRY(h, cudaStreamSynchronize(h->stream), "inference");
    if (errWord & kNrcTcTimeout)
        return fail(h, RC_DEVICE_ERROR, "nrc_infer: a tensor-core wait timed out");
    return RC_OK;
}

rc_status rc_nrc_encode(rc_tracer* h, const float* queries, int64_t n, float* features)
{
    if (!h)
        return RC_INVALID_ARG;
    NRC_STATUS(check_ready(h, "nrc_encode"));
    if (!queries || !features || n <= 0 || n > kApiMax)
        return fail(h, RC_INVALID_ARG, "nrc_encode: null buffer or n outside [1, 2^20]");
    cudaSetDevice(h->device);
    NrcState& st = h->nrc;
    NRC_STATUS(upload_records(h, queries, nullptr, n));
    NRC_STATUS(device_grow(h, &st.dApiOut, &st.capApiOut, size_t(n) * kNrcIn * 2, "allocate features"));
    NrcBox box;
    NRC_STATUS(encoding_box(h, box));
    NRC_TRY(h,
            launch_nrc_encode(static_cast<const NrcRecord*>(st.dApi), int(n), box,
                              static_cast<__nv_bfloat16*>(st.dApiOut), h->stream),
            "launch encoding");
    std::vector<uint16_t> raw(size_t(n) * kNrcIn);
    NRC_TRY(h, cudaMemcpyAsync(raw.data(), st.dApiOut, raw.size() * 2, cudaMemcpyDeviceToHost, h->stream),
            "download features");
    NRC_TRY(h, cudaStreamSynchronize(h->stream), "encoding");
    for (size_t i = 0; i < raw.size(); ++i)
    {
        uint32_t bits = uint32_t(raw[i]) << 16;
        std::memcpy(&features[i], &bits, 4);
    }
    return RC_OK;
}

rc_status rc_nrc_gradient(rc_tracer* h, const float* queries, const float* targets, int64_t n, float* grad,
                          float* loss)
{
    if (!h)
        return RC_INVALID_ARG;
    NRC_STATUS(check_ready(h, "nrc_gradient"));
    if (!queries || !targets || n <= 0 || n > kApiMax)
        return fail(h, RC_INVALID_ARG, "nrc_gradient: null buffer or n outside [1, 2^20]");
    cudaSetDevice(h->device);
    NrcState& st = h->nrc;
    NRC_STATUS(upload_records(h, queries, targets, n));
    NRC_STATUS(loss_buffer(h, 1));
    NrcTrainParams tp{};
    tp.weights = st.dW;
    tp.rec = static_cast<const NrcRecord*>(st.dApi);
    tp.batch = int(n);
    tp.partials = st.dPartials;
    tp.lossPartials = st.dLossPartials;
    NRC_STATUS(encoding_box(h, tp.box));
    NRC_TRY(h, launch_nrc_train(tp, st.blocks, h->stream), "launch gradient");
    NrcAdamParams a = adam_params(h, 0, nullptr, st.dLoss);
    NRC_TRY(h, launch_nrc_adam(a, h->stream), "launch gradient sum");
    if (grad)
        NRC_TRY(h, cudaMemcpyAsync(grad, st.dGrad, size_t(kNrcParamCount) * 4, cudaMemcpyDeviceToHost, h->stream),
                "download gradient");
    if (loss)
        NRC_TRY(h, cudaMemcpyAsync(loss, st.dLoss, 4, cudaMemcpyDeviceToHost, h->stream), "download loss");
    NRC_TRY(h, cudaStreamSynchronize(h->stream), "gradient");
    return RC_OK;
}

rc_status rc_nrc_train(rc_tracer* h, const float* queries, const float* targets, int64_t n, int32_t steps,
                       float* losses)
{
    if (!h)
        return RC_INVALID_ARG;
    NRC_STATUS(check_ready(h, "nrc_train"));
    if (!queries || !targets || n <= 0 || n > kApiMax || steps < 1 || steps > 1000000)
        return fail(h, RC_INVALID_ARG, "nrc_train: null buffer, n outside [1, 2^20] or steps < 1");
    cudaSetDevice(h->device);
    NrcState& st = h->nrc;
    NRC_STATUS(upload_records(h, queries, targets, n));
    NRC_STATUS(loss_buffer(h, steps));
    NrcTrainParams tp{};
    tp.weights = st.dW;
    tp.rec = static_cast<const NrcRecord*>(st.dApi);
    tp.batch = int(n);
    tp.partials = st.dPartials;
    tp.lossPartials = st.dLossPartials;
    NRC_STATUS(encoding_box(h, tp.box));
    for (int s = 0; s < steps; ++s)
    {
        NRC_TRY(h, launch_nrc_train(tp, st.blocks, h->stream), "launch training step");
        NrcAdamParams a = adam_params(h, 1, nullptr, st.dLoss + s);
        NRC_TRY(h, launch_nrc_adam(a, h->stream), "launch optimizer step");
    }
    if (losses)
        NRC_TRY(h, cudaMemcpyAsync(losses, st.dLoss, size_t(steps) * 4, cudaMemcpyDeviceToHost, h->stream),
                "download losses");
    NRC_TRY(h, cudaStreamSynchronize(h->stream), "training");
    st.lastSteps = steps;
    return RC_OK;
}

rc_status rc_nrc_read_samples(rc_tracer* h, float* records, int64_t capacity, int64_t* count)
{
    if (!h)
        return RC_INVALID_ARG;
    NRC_STATUS(check_ready(h, "nrc_read_samples"));
    if (!count || (capacity > 0 && !records))
        return fail(h, RC_INVALID_ARG, "nrc_read_samples: null buffer");
    cudaSetDevice(h->device);
    NrcState& st = h->nrc;
    *count = 0;
    if (!st.dVtx || !st.dIndex)
        return RC_OK;
    unsigned c[2] = { 0, 0 };
    NRC_TRY(h, cudaMemcpyAsync(c, st.dCounters, sizeof(c), cudaMemcpyDeviceToHost, h->stream), "read counters");
    NRC_TRY(h, cudaStreamSynchronize(h->stream), "read counters");
    *count = int64_t(c[1]);
    const int64_t take = std::min<int64_t>(capacity, int64_t(c[1]));
    if (take <= 0)
        return RC_OK;
    std::vector<int> index(static_cast<size_t>(c[1]));
    NRC_TRY(h, cudaMemcpyAsync(index.data(), st.dIndex, index.size() * 4, cudaMemcpyDeviceToHost, h->stream),
            "read sample index");
    NRC_TRY(h, cudaStreamSynchronize(h->stream), "read sample index");
    int maxIdx = 0;
    for (int v : index)
        maxIdx = std::max(maxIdx, v);
    std::vector<NrcRecord> vtx(size_t(maxIdx) + 1);
    NRC_TRY(h, cudaMemcpyAsync(vtx.data(), st.dVtx, vtx.size() * sizeof(NrcRecord), cudaMemcpyDeviceToHost, h->stream),
            "read training vertices");
    NRC_TRY(h, cudaStreamSynchronize(h->stream), "read training vertices");
    // samples in vertex-record order, so the result does not depend on scheduling
    std::sort(index.begin(), index.end());
    for (int64_t i = 0; i < take; ++i)
    {
        NrcRecord r = vtx[size_t(index[size_t(i)])];
        std::memcpy(records + i * 16, &r, sizeof(r));
    }
    return RC_OK;
}

rc_status rc_nrc_get_stats(rc_tracer* h, rc_nrc_stats* out)
{
    if (!h)
        return RC_INVALID_ARG;
    if (!out)
        return fail(h, RC_INVALID_ARG, "nrc_get_stats: null output");
    std::memset(out, 0, sizeof(*out));
    if (!h->nrc.configured)
        return RC_OK;
    cudaSetDevice(h->device);
    NrcState& st = h->nrc;
    unsigned c[2] = { 0, 0 };
    float loss = 0.0f;
    NRC_TRY(h, cudaMemcpyAsync(c, st.dCounters, sizeof(c), cudaMemcpyDeviceToHost, h->stream), "read counters");
    if (st.lastSteps > 0 && st.dLoss)
        NRC_TRY(h, cudaMemcpyAsync(&loss, st.dLoss + (st.lastSteps - 1), 4, cudaMemcpyDeviceToHost, h->stream),
                "read loss");
    NRC_TRY(h, cudaStreamSynchronize(h->stream), "read stats");
    out->lookups = c[0];
    out->training_samples = c[1];
    out->steps = st.steps;
    out->last_loss = loss;
    out->train_ms = st.trainMs;
    return RC_OK;
}

}  // extern "C"
