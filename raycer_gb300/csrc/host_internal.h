// Internal definition of the rc_tracer handle and the render helpers shared
// by the host translation units.
#pragma once

#include <cuda_runtime.h>

#include <chrono>
#include <string>
#include <vector>

#include "../../include/raycer_gb300.h"
#include "bvh_build.h"
#include "device_types.h"
#include "kernels.h"
#include "nrc_kernels.h"

namespace rcx
{

// Device-layout records of one scene built on the host: the reference-form
// flat BVH and primitive order, triangles and shading records in BVH order,
// materials. The device nodes are derived from `flat` at upload.
struct HostScene
{
    std::vector<BuildNode> flat;
    std::vector<uint32_t> order;
    std::vector<DevTri> tris;
    std::vector<DevShade> shade;
    std::vector<DevMat> mats;
    uint32_t depth = 0;
};

// One mesh of an uploaded two-level scene, kept on the host for scene
// files: its flat BVH and primitive order, and its range in the pooled
// triangle arrays.
struct InstancedMesh
{
    std::vector<BuildNode> flat;
    std::vector<uint32_t> order;
    uint32_t depth = 0;
    int64_t firstTri = 0;
    int64_t triangles = 0;
};

// Neural radiance cache state of a handle (nrc_host.cpp).
struct NrcState
{
    rc_nrc_config cfg{};
    bool configured = false;
    uint64_t steps = 0;        // Adam steps taken (t)
    uint64_t passes = 0;       // render passes that trained
    float* dMaster = nullptr;  // FP32 weights, Adam m, v: kNrcParamCount each
    float* dM = nullptr;
    float* dV = nullptr;
    __nv_bfloat16* dW = nullptr;
    float* dPartials = nullptr;      // [blocks][params]
    float* dLossPartials = nullptr;  // [blocks]
    float* dLoss = nullptr;          // per step of the last training call
    size_t capLoss = 0;
    float* dGrad = nullptr;
    unsigned* dCounters = nullptr;   // [0] lookups, [1] training samples, [2] api count
    void* dQuery = nullptr;          // lookups, one record per slot
    size_t capQuery = 0;
    void* dVtx = nullptr;            // training vertices
    size_t capVtx = 0;
    void* dTerm = nullptr;
    size_t capTerm = 0;
    void* dIndex = nullptr;
    size_t capIndex = 0;
    void* dApi = nullptr;            // host-batch records
    size_t capApi = 0;
    void* dApiOut = nullptr;
    size_t capApiOut = 0;
    int blocks = 0;
    int lastSteps = 0;
    double trainMs = 0.0;
    cudaEvent_t evTrain0 = nullptr;
    cudaEvent_t evTrain1 = nullptr;
};

}  // namespace rcx

struct rc_tracer
{
    int device = 0;
    int numSMs = 1;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr;
    cudaEvent_t ev1 = nullptr;
    cudaEvent_t evMid = nullptr;           // between the RAY frame's two kernels
    std::vector<cudaEvent_t> evPool;       // around each PATH extend launch
    std::string err;

    // Scene (device layout of device_types.h) and its host flat-BVH copy.
    rcx::DevNode* dNodes = nullptr;
    rcx::DevTri* dTris = nullptr;
    rcx::DevShade* dShade = nullptr;
    rcx::DevMat* dMats = nullptr;
    size_t innerCount = 0;
    int64_t nTris = 0;
    int32_t nMats = 0;
    int32_t rootLink = 0;
    uint64_t bvhInner = 0;
    uint64_t bvhDepth = 0;
    bool sceneReady = false;
    std::vector<rcx::BuildNode> hostNodes;
    std::vector<uint32_t> hostOrder;
    double bounds[6] = { 0, 0, 0, 0, 0, 0 };  // scene box: min xyz, max xyz
    // Two-level scenes (rc_upload_instanced): top-level BVH over instances.
    rcx::DevNode* dTlas = nullptr;
    size_t tlasCount = 0;
    rcx::DevInstance* dInstances = nullptr;
    int64_t nInstances = 0;
    int32_t tlasRoot = 0;
    std::vector<rcx::InstancedMesh> instMeshes;  // two-level scene: its meshes
    std::vector<rc_instance> instDescs;          //   and instances, for rc_save_scene
    // 4-wide BVH of a single-level scene (wide_bvh.cpp), or none.
    rcx::DevNode4* dWide = nullptr;
    size_t wideCount = 0;
    int32_t wideRoot = 0;
    bool wideTried = false;  // ensure_wide ran for the current scene
    // Rope records of a single-level scene for the stackless walk (wide_bvh.cpp), or none.
    rcx::DevRope* dRopes = nullptr;
    size_t ropeCount = 0;
    bool ropesTried = false;  // ensure_ropes ran for the current scene

    // Per-frame records.
    rc_camera camera{};
    bool cameraSet = false;
    rc_general general{};
    rc_tonemapper tonemapper{};
    std::vector<rc_directional_light> lights;
    int order = RC_ORDER_NEAREST;
    int counting = 0;
    int builder = RC_BUILDER_REFERENCE_SAH;
    uint32_t frameIndex = 0;  // advances per PATH render, reset by rc_clear

    // Film: r, g, b, filter-weight sum per pixel (float32), and the RAY
    // tracer's per-pixel cast records.
    uint64_t width = 0;
    uint64_t height = 0;
    uint64_t filmPixels = 0;
    float4* dFilm = nullptr;
    rc_cast_pixel* dCast = nullptr;
    int* dQueue = nullptr;

    // Path-tracer wavefront state (grow-only; see pathtrace.cu).
    void* dPath = nullptr;
    size_t capPath = 0;
    uint64_t pathSlots = 0;
    unsigned* dCounts = nullptr;
    size_t capCounts = 0;
    void* dTables = nullptr;   // scene record + per-pass chunk records
    size_t capTables = 0;

    // Tone-mapping scratch (partial sums) and output staging.
    void* dTone = nullptr;
    size_t capTone = 0;
    void* dImage = nullptr;
    size_t capImage = 0;

    // Scratch for the host-buffer entry points.
    void* dTmpA = nullptr;
    size_t capTmpA = 0;
    void* dTmpB = nullptr;
    size_t capTmpB = 0;

    rcx::DevControl* dCtl = nullptr;
    // Host-buffer ray casts: copies on their own streams, overlapped with
    // the kernels chunk by chunk.
    cudaStream_t copyIn = nullptr;
    cudaStream_t copyOut = nullptr;
    std::vector<cudaEvent_t> evChunk;
    void* dCtlChunks = nullptr;
    size_t capCtlChunks = 0;
    rc_stats stats{};
    size_t deviceBytes = 0;

    rcx::NrcState nrc;
    // FP64 RMSE scratch (rc_film_rmse_f64)
    void* dRmse = nullptr;
    size_t capRmse = 0;

    // rc_render's progress / cancel word: pinned host memory mapped into the
    // device (monHost, and monDev as the kernels address it), and the time
    // budget of rc_set_time_budget.
    rcx::RenderMonitor* monHost = nullptr;
    rcx::RenderMonitor* monDev = nullptr;
    unsigned long long budgetNs = rcx::kNoBudget;
};

namespace rcx
{

// One rc_render call's monitoring. `dev` (the kernels' monitor pointer) is
// set when the caller passed a cancel flag or a progress counter; budgetNs
// when the handle has a time budget. wait_render forwards the caller's flag
// to the device and the device's progress to the caller while the render's
// kernels run.
struct RenderWatch
{
    RenderMonitor* dev = nullptr;
    unsigned long long budgetNs = kNoBudget;
    const volatile int32_t* cancel = nullptr;
    uint64_t* pixels = nullptr;
    uint64_t seen = 0;
};
// The device address through which kernels on h's GPU can read or write
// the host buffer [p, p + bytes) in place (page-locked memory, or pageable
// memory whose pages are resident where the device uses the host page
// tables), or null where they should not.
void* device_view(rc_tracer* h, const void* p, size_t bytes);

// Blocks until `done` has completed; while it waits, raises the device's
// cancel word once the caller's flag is set and stores every larger
// progress value it reads into the caller's counter (relaxed atomic stores).
rc_status wait_render(rc_tracer* h, RenderWatch* w, cudaEvent_t done);
// Status of a render whose control block reads `error` (stack overflow,
// cancel, time budget; RC_OK for none of them). Sets the message.
rc_status render_outcome(rc_tracer* h, int error, const char* what);

// dOrigins (optional): per shadow-queue entry, the shadow ray's origin
// (launch_raycast's shadowOrigins). watch: rc_render's monitoring, or null.
rc_status raycast_into(rc_tracer* h, const rc_ray* dRays, uint64_t pixelStart, uint64_t count, int order,
                       rc_cast_pixel* dOut, int* dQueue, float4* dOrigins = nullptr, RenderWatch* watch = nullptr);
rc_status render_raycast(rc_tracer* h, uint64_t pixelStart, uint64_t count, const rc_ray* dRays,
                         RenderWatch* watch = nullptr);
rc_status render_path(rc_tracer* h, uint64_t pixelStart, uint64_t count, RenderWatch* watch);
void release_render_buffers(rc_tracer* h);
// Scene construction (tracer_host.cpp), shared with the scene files (scene_file.cpp).
void build_host_scene(const double* v, const uint32_t* matIdx, int64_t n, const rc_material* mats, int32_t matCount,
                      std::vector<BuildNode>&& nodes, std::vector<uint32_t>&& order, uint32_t depth, HostScene& hs);
rc_status upload_host_scene(rc_tracer* h, HostScene&& hs);
void release_scene_data(rc_tracer* h);
// Collapses the binary device nodes (root `rootLink`) into the 4-wide BVH and
// uploads it (h->dWide); leaves it out where its stack need exceeds the
// traversal stack. Failure to allocate is an error.
rc_status upload_wide(rc_tracer* h, const std::vector<DevNode>& nodes, int32_t rootLink);
// Builds the 4-wide BVH of the handle's single-level scene on first use (the
// first PATH or batch render of a scene): downloads the binary nodes once,
// collapses and uploads them. Uploads and RAY frames do not pay for it.
rc_status ensure_wide(rc_tracer* h);
// Builds the rope records of the handle's single-level scene on first use
// (the first RAY frame or rc_cast while the stackless walk is on): one
// download of the binary nodes, one upload of the records.
rc_status ensure_ropes(rc_tracer* h);
// Two-level scenes (instancing.cpp): argument checks, one SAH build per mesh
// (host scenes in BVH order), and the pooled upload with instance transforms
// and the top-level BVH (which also keeps the meshes and instances on the
// handle for scene files). err gets the reason of a failure.
rc_status check_instanced_args(const rc_mesh* meshes, int32_t mesh_count, const rc_instance* instances,
                               int64_t instance_count, const rc_material* materials, int32_t material_count,
                               uint32_t max_leaf_size, std::string& err);
rc_status build_mesh_scenes(const rc_mesh* meshes, int32_t mesh_count, const rc_material* materials,
                            int32_t material_count, uint32_t max_leaf_size, std::vector<HostScene>& out,
                            std::string& err);
// The scene box of instances of these meshes (the union of their world boxes).
void instanced_scene_box(const std::vector<HostScene>& meshes, const rc_instance* instances, int64_t ni, double box[6]);
rc_status upload_instanced_scenes(rc_tracer* h, std::vector<HostScene>&& meshScenes, const rc_instance* instances,
                                  int64_t instance_count, int32_t material_count,
                                  std::chrono::steady_clock::time_point t0);
void device_nodes(const std::vector<BuildNode>& nodes, std::vector<DevNode>& dn, int32_t& rootLink, uint64_t& inner);
// Upload through the GPU BVH builder (gpu_build_host.cpp).
rc_status upload_gpu_built(rc_tracer* h, const double* v, const uint32_t* matIdx, int64_t n, const rc_material* mats,
                           int32_t matCount, uint32_t maxLeafSize);
bool validate_flat_bvh(const std::vector<BuildNode>& nodes, uint64_t n, uint32_t& depth, std::string& err);
// Grow-only device buffer (frees the old one); counts into deviceBytes.
rc_status device_grow(rc_tracer* h, void** ptr, size_t* cap, size_t bytes, const char* what);

struct PassParams;
// NRC work of a PATH render (nrc_host.cpp): buffers and per-pass state,
// the lookups before the film update, the training after it.
rc_status nrc_prepare(rc_tracer* h, uint64_t slots, int segments);
void nrc_pass_state(rc_tracer* h, PassParams& pp, uint32_t passIndex);
rc_status nrc_lookups(rc_tracer* h, const PassParams& pp);
rc_status nrc_train_pass(rc_tracer* h, const PassParams& pp);
bool nrc_active(const rc_tracer* h);
void nrc_release(rc_tracer* h);

struct PathScene;
// The pass kernels' record of a handle's scene, camera, PATH settings and film.
PathScene path_scene(const rc_tracer* h, uint64_t pixelStart);
// Slot arrays of a path-state buffer of `slots` slots (pathtrace.h layout).
PassParams pass_params(void* state, uint64_t slots, unsigned* counts, DevControl* ctl);

}  // namespace rcx
