/*
 * raycer_gb300 — C ABI of the GB300 (sm_103a) path-tracing / ray-casting hot path.
 *
 * This is the drop-in boundary for raycer's GPU tracer. Every entry point
 * replaces one piece of the reference's OpenCL tracer host side
 * (src/OpenCL/CLTracer.{h,cpp}, src/OpenCL/CLScene.cpp) or of the CPU
 * Tracer API (src/Raytracing/Tracers/Tracer.h), as cited beside it.
 *
 * Conventions
 *   - Plain C: pointers + sizes, no C++ or torch types. Nothing throws.
 *   - Every function returns an rc_status (0 = RC_OK). On failure the
 *     handle's message is available from rc_last_error(). The C++ wrapper
 *     (raycer_gb300/cpp/CudaTracer.hpp) turns status + message into
 *     std::runtime_error, which is how CLManager::checkError reports errors
 *     (src/OpenCL/CLManager.cpp:73-101).
 *   - A handle owns all device memory it allocates (like CLTracer owns its
 *     cl_mem objects, CLTracer.cpp:38-43, 165-170, 240-260). Caller-owned
 *     host arrays are only read during the call; no pointer is retained.
 *   - One handle per host thread / stream. Calls on one handle are serialised
 *     by the caller, as the reference's render thread does
 *     (src/Runners/ConsoleRunner.cpp:94-142).
 *   - Pixel (0,0) is the bottom-left pixel and y grows upwards
 *     (src/Rendering/Image.h:10-14); images are row-major RGBA float32.
 */
#ifndef RAYCER_GB300_H
#define RAYCER_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* Status codes                                                              */

typedef enum rc_status
{
    RC_OK = 0,
    RC_INVALID_ARG = 1,  /* bad pointer, size or record field              */
    RC_OOM = 2,          /* device or host allocation refused              */
    RC_CUDA = 3,         /* a CUDA runtime call failed (message has it)    */
    RC_CANCELLED = 4,    /* the caller's cancel flag was raised            */
    RC_TIMEOUT = 5,      /* the render's time budget ran out (rc_set_time_budget) */
    RC_NOT_READY = 6,    /* call order: e.g. render before upload/resize   */
    RC_UNSUPPORTED = 7,  /* valid in the reference, not in this build      */
    RC_DEVICE_ERROR = 8, /* a kernel reported an error status (e.g. stack) */
    RC_IO = 9            /* a file could not be read / written or is invalid */
} rc_status;

typedef struct rc_tracer rc_tracer; /* opaque handle: one tracer on one GPU */

/* ------------------------------------------------------------------------ */
/* Plain records (host side)                                                 */

/* Material fields the hot path reads: src/Raytracing/Material.h:23-44,
 * flattened like OpenCL::Material (src/OpenCL/CLStructs.h, CLScene.cpp:110-147).
 * Textures are not supported (texture indices of the reference = -1). */
typedef struct rc_material
{
    float diffuse[3];     /* diffuseReflectance                          */
    float emittance[3];   /* emittance                                   */
    int32_t is_emissive;  /* isEmissive                                  */
    int32_t non_shadowing;/* nonShadowing: skipped by shadow rays        */
    int32_t invert_normal;/* invertNormal                                */
    int32_t dielectric;   /* GPU extension: 1 = smooth dielectric (PATH   */
                          /* tracer: Fresnel reflection / refraction)    */
    float ior;            /* its index of refraction (> 0); 0 otherwise  */
} rc_material;

/* Float32 camera record, the fields CLScene::readSceneCamera copies
 * (src/OpenCL/CLScene.cpp:242-262) for a perspective camera. Fill it with
 * rc_camera_from_euler() or from the reference's Camera::cameraState. */
typedef struct rc_camera
{
    float position[3];
    float forward[3];
    float right[3];
    float up[3];
    float image_plane_center[3];
    float aspect_ratio;        /* height / width        (Camera.cpp:33) */
    float image_plane_width;   /* width - 1             (Camera.cpp:31) */
    float image_plane_height;  /* height - 1            (Camera.cpp:32) */
} rc_camera;

typedef enum rc_tracer_type { RC_TRACER_RAY = 0, RC_TRACER_PATH = 1 } rc_tracer_type;
/* Values follow the reference's enums (Rendering/Samplers/Sampler.h:24,
 * Rendering/Filters/Filter.h:10, Rendering/ToneMappers/ToneMapper.h:15). */
typedef enum rc_sampler_type { RC_SAMPLER_CENTER = 0, RC_SAMPLER_RANDOM = 1, RC_SAMPLER_CMJ = 4 } rc_sampler_type;
typedef enum rc_filter_type
{
    RC_FILTER_BOX = 0,
    RC_FILTER_TENT = 1,
    RC_FILTER_BELL = 2,
    RC_FILTER_GAUSSIAN = 3,
    RC_FILTER_MITCHELL = 4,
    RC_FILTER_LANCZOS_SINC = 5
} rc_filter_type;
typedef enum rc_tonemapper_type { RC_TONEMAP_PASSTHROUGH = 0, RC_TONEMAP_REINHARD = 3 } rc_tonemapper_type;

/* Scene::General fields on the hot path (src/Raytracing/Scene.h:89-131)
 * plus the GPU-only knobs. */
typedef struct rc_general
{
    int32_t tracer_type;             /* rc_tracer_type (tracerType)                 */
    int32_t max_path_length;         /* maxPathLength: segments per path            */
    int32_t path_sample_count;       /* pathSampleCount: paths per camera ray       */
    int32_t multi_sample_count_sqrt; /* multiSampleCountSqrt: n x n film samples    */
    int32_t multi_sampler_type;      /* rc_sampler_type (multiSamplerType)          */
    int32_t filter_type;             /* rc_filter_type (multiSamplerFilterType)     */
    float filter_radius[2];          /* BOX radius (BoxFilter.h:16: 0.5, 0.5); the  */
                                     /* others use their constructors' defaults as  */
                                     /* the reference's Tracer does (Tracer.cpp:50) */
    float ray_start_offset;          /* rayStartOffset (Scene.h:95: 1e-5)           */
    float background[3];             /* backgroundColor (RAY tracer, miss)          */
    int32_t russian_roulette_depth;  /* 0 = off (reference); else first RR segment  */
    int32_t flags;                   /* rc_general_flags (0 = reference behaviour)  */
    uint64_t seed;                   /* random stream seed (paths, CMJ permutation) */
} rc_general;

/* GPU-only extensions of the PATH tracer (no counterpart in the reference).
 * RC_GENERAL_SKY: a path that leaves the scene receives `background` as
 * radiance, times its throughput (PathTracer::traceRecursive returns black,
 * PathTracer.cpp:43-44). */
typedef enum rc_general_flags { RC_GENERAL_SKY = 1 } rc_general_flags;

/* Scene::ToneMapper fields (src/Raytracing/Scene.h:135-159). */
typedef struct rc_tonemapper
{
    int32_t type;          /* rc_tonemapper_type */
    int32_t apply_gamma;
    int32_t should_clamp;
    int32_t reserved;      /* must be 0 */
    double gamma;
    double key;
} rc_tonemapper;

/* DirectionalLight (src/Raytracing/Lights.h:47-57): direction the light
 * travels; shadow rays go toward -direction (Raytracer.cpp:499). */
typedef struct rc_directional_light
{
    float direction[3];
    float color[3];
    float intensity;
} rc_directional_light;

/* One node of the reference's flat BVH (FlatBVHNode, FlatBVH.h:38-53):
 * preorder array; left child = i + 1, right child = i + right_offset,
 * leaf <=> right_offset == 0. */
typedef struct rc_bvh_node
{
    double aabb_min[3];
    double aabb_max[3];
    int64_t right_offset;
    uint64_t start_offset;
    uint64_t primitive_count;
} rc_bvh_node;

/* Ray for the generic cast entry points: origin, direction (need not be
 * normalised), and the [t_min, t_max] window of Ray::minDistance /
 * maxDistance (src/Raytracing/Ray.h:16-17). */
typedef struct rc_ray
{
    float origin[3];
    float t_min;
    float direction[3];
    float t_max;
} rc_ray;

/* Hit record: prim = caller's triangle index (the reference's primitive id
 * minus the first id) or -1 for a miss; t = hit distance; u, v =
 * barycentrics of the reported hit. */
typedef struct rc_hit
{
    int32_t prim;
    float t;
    float u;
    float v;
} rc_hit;

/* Per-pixel ray-cast result (RAY tracer): primary hit and the directional
 * light's shadow query (Raytracer::calculateShadowAmount, Raytracer.cpp:497). */
typedef struct rc_cast_pixel
{
    int32_t prim;      /* primary hit triangle (caller index) or -1          */
    float t;           /* primary hit distance                               */
    int32_t occluder;  /* first triangle the shadow ray found, -1 = lit       */
    int32_t flags;     /* bit0: primary hit; bit1: shadow ray cast; bit2: occluded */
} rc_cast_pixel;

/* Traversal order of the closest-hit query.
 * RC_ORDER_REFERENCE: the reference's preorder DFS (left subtree first, no
 *   distance culling; FlatBVH::intersect FlatBVH.cpp:22-75).
 * RC_ORDER_NEAREST: nearer child first + distance culling; reports the same
 *   hit (minimum t, ties to the later triangle in BVH order, Triangle.cpp:93). */
typedef enum rc_traversal_order { RC_ORDER_REFERENCE = 0, RC_ORDER_NEAREST = 1 } rc_traversal_order;

typedef struct rc_stats
{
    uint64_t rays_traced;      /* BVH queries in the last render / cast call   */
    uint64_t node_visits;      /* inner-node pair tests (when counting is on)  */
    uint64_t tri_tests;        /* triangle tests (when counting is on)         */
    double last_ms;            /* device time of the last render / cast call   */
    uint64_t bvh_inner_nodes;  /* inner nodes of the device BVH                */
    uint64_t bvh_depth;        /* depth of the uploaded BVH                    */
    uint64_t device_bytes;     /* device memory held by the handle             */
    /* Per stage of the last call. RAY render / cast_with_shadow: rays, nodes
     * and triangles 0 = primary closest hit, 1 = shadow any hit; times 0 =
     * the primary kernel, 1 = the shadow kernel where the frame runs as two
     * kernels (counted frames, RC_TRACE_FUSED=0), else 0 = the one kernel
     * that traces both and 1 = 0.0. (The in-place rc_cast_with_shadow
     * leaves both times 0.0.) PATH render: 0 = the extend (closest-hit)
     * kernels of all segments, 1 = everything else (generate, shade,
     * accumulate); where a segment's extend and shade run as one kernel
     * (plain passes over the 4-wide tree), 0 includes the shading. cast:
     * 0 = the cast kernel. */
    uint64_t stage_rays[2];
    uint64_t stage_nodes[2];   /* when counting is on */
    uint64_t stage_tris[2];    /* when counting is on */
    double stage_ms[2];        /* device time from CUDA events around the stage's launches */
    double build_ms;           /* host wall time of the last scene build + upload */
} rc_stats;

/* ------------------------------------------------------------------------ */
/* Lifetime — CLTracer::CLTracer / ~CLTracer (CLTracer.cpp:32-43) and
 * CLTracer::initializeKernels / releaseKernels (CLTracer.cpp:45-98).        */

rc_status rc_create(rc_tracer** out, int device);
void rc_destroy(rc_tracer* h);
const char* rc_last_error(const rc_tracer* h);
const char* rc_version(void);

/* ------------------------------------------------------------------------ */
/* Scene — CLTracer::initializeBuffers + CLScene::readSceneFull
 * (CLTracer.cpp:173-238, CLScene.cpp:72-240).                               */

/* Upload triangles (vertices: n*9 doubles, v0 v1 v2, caller order) with a
 * material index per triangle into `materials`, and build the SAH flat BVH
 * on the host exactly as FlatBVH::build does (FlatBVH.cpp:89-343: SAH over
 * {AABB centre, centroid median} per axis, in-place partition, half split
 * fallback) with BVHBuildInfo.maxLeafSize = max_leaf_size (1..15). */
rc_status rc_upload_scene(rc_tracer* h, const double* vertices, const uint32_t* material_index, int64_t n,
                          const rc_material* materials, int32_t material_count, uint32_t max_leaf_size);

/* Same, but with a BVH the caller already built (the reference's
 * scene.rootBVH.bvh.flatNodes and the order of its orderedPrimitives, as
 * caller triangle indices) — the verbatim node copy of
 * CLScene.cpp:224-237. The node array is validated before use. */
rc_status rc_upload_scene_prebuilt(rc_tracer* h, const double* vertices, const uint32_t* material_index, int64_t n,
                                   const rc_material* materials, int32_t material_count,
                                   const rc_bvh_node* nodes, int64_t node_count, const uint64_t* ordered_index);

/* The flat BVH of the last upload in the reference's FlatBVHNode form (for
 * checks and for caching; nodes: node_count entries, ordered_index: n). */
rc_status rc_get_bvh(const rc_tracer* h, rc_bvh_node* nodes, int64_t node_capacity, int64_t* node_count,
                     uint64_t* ordered_index, int64_t index_capacity);

/* BVH builder of the next rc_upload_scene (no counterpart in the reference;
 * GPU-only extension). RC_BUILDER_REFERENCE_SAH (default): FlatBVH::build's
 * SAH tree on the host, identical to the reference's. RC_BUILDER_GPU_LBVH:
 * a linear BVH built on the device (Morton order, Karras 2012), leaves of up
 * to max_leaf_size triangles; much faster to build, not the reference's
 * tree (closest hits equal except at equal-distance ties). */
typedef enum rc_bvh_builder { RC_BUILDER_REFERENCE_SAH = 0, RC_BUILDER_GPU_LBVH = 1 } rc_bvh_builder;
rc_status rc_set_bvh_builder(rc_tracer* h, int32_t builder);

/* Host-only SAH build (no device memory, no GPU needed): the BVH
 * rc_upload_scene would build, returned in the reference's FlatBVHNode form
 * (FlatBVH::build, FlatBVH.cpp:89-204). Call with nodes == NULL to get the
 * node count. ordered_index receives n entries. */
rc_status rc_build_bvh(const double* vertices, int64_t n, uint32_t max_leaf_size, rc_bvh_node* nodes,
                       int64_t node_capacity, int64_t* node_count, uint64_t* ordered_index, uint32_t* depth);

/* Release the scene buffers — CLTracer::releaseBuffers (CLTracer.cpp:240). */
rc_status rc_release_scene(rc_tracer* h);

/* Per-frame records — CLTracer::uploadMinimalData (CLTracer.cpp:441-451)
 * and the General / ToneMapper / light uploads of uploadFullData (:389). */
rc_status rc_set_camera(rc_tracer* h, const rc_camera* camera);
rc_status rc_set_general(rc_tracer* h, const rc_general* general);
rc_status rc_set_tonemapper(rc_tracer* h, const rc_tonemapper* tonemapper);
rc_status rc_set_directional_lights(rc_tracer* h, const rc_directional_light* lights, int32_t count);

/* Camera::update's perspective basis (Camera.cpp:157-160, 277-283:
 * ONB::fromNormal(EulerAngle::getDirection()), imagePlaneDistance =
 * 0.5 / tan(fov / 2), fov horizontal, degrees) in float64, cast to the
 * float32 record, for a width x height film (Camera::setImagePlaneSize). */
rc_status rc_camera_from_euler(const double position[3], double pitch, double yaw, double roll, double fov,
                               uint64_t width, uint64_t height, rc_camera* out);

/* Default General / ToneMapper records (the reference's defaults,
 * Scene.h:89-159 — MITCHELL film filter, CMJ sampler — with the given
 * tracer type). */
void rc_general_defaults(rc_general* out, int32_t tracer_type);
void rc_tonemapper_defaults(rc_tonemapper* out);

/* ------------------------------------------------------------------------ */
/* Film — CLTracer::initializeImageBuffers / releaseImageBuffers / clear
 * (CLTracer.cpp:100-171, 325-333).                                          */

rc_status rc_resize(rc_tracer* h, uint64_t width, uint64_t height);
rc_status rc_clear(rc_tracer* h);

/* ------------------------------------------------------------------------ */
/* Render — Tracer::run / CLTracer::run (Tracer.cpp:58-113, CLTracer.cpp:262).
 * Renders pixel_count pixels starting at pixel_start of a film_width x
 * film_height image into film pixels [0, pixel_count) — the TracerState
 * contract (TracerState.h:13-26) the network runner uses
 * (NetworkRunner.cpp:398-417). PATH: adds filter-weighted samples to the
 * film. RAY: casts the primary ray of every pixel and, for each hit, one
 * shadow ray per directional light, into the cast buffer (rc_read_cast).
 * Blocks until the device is done.
 *
 * Progress and cancellation, as Tracer::run's `interrupted` check and
 * pixelsProcessed updates (Tracer.cpp:76-112) read by a second thread
 * (ConsoleRunner.cpp:126-142):
 *   cancel (optional): a flag another host thread may raise at any time
 *     during the call. The calling thread forwards it to a word in pinned,
 *     device-mapped host memory that one watching warp of the kernels checks
 *     about every 2 microseconds; the working warps then take no more work
 *     (items of 32 rays or paths already taken finish). The call returns
 *     RC_CANCELLED. A RAY frame keeps the records of the pixels it traced
 *     (the others are untouched); a PATH film keeps whole passes only.
 *   pixels_processed (optional): set to 0 at entry; while the kernels run
 *     the calling thread stores into it (relaxed atomic stores of a
 *     uint64_t, so another thread may read it with an atomic load, e.g.
 *     through a std::atomic<uint64_t> of the same object) the pixels the
 *     device reports finished, never decreasing: PATH renders per pass as
 *     each pass's film update lands; RAY frames a lower bound (the pixels
 *     of the 32-pixel work items taken before those still in flight). At
 *     the end it holds the exact number of pixels finished: pixel_count on
 *     success.
 * A cancel flag or progress counter makes the calling thread wait by
 * polling (it yields between polls) instead of sleeping in the driver. */
rc_status rc_render(rc_tracer* h, uint64_t pixel_start, uint64_t pixel_count,
                    const volatile int32_t* cancel, uint64_t* pixels_processed);

/* Time budget of every later rc_render on this handle (GPU-only extension;
 * the reference has no counterpart): the kernels stop taking work once
 * `milliseconds` of device time have passed since the render's first work
 * (checked about every 2 microseconds), and the call returns RC_TIMEOUT with
 * the results of rc_render's cancel case. 0 stops at the first check (the
 * items taken by then still finish); a negative value removes the budget
 * (the default). */
rc_status rc_set_time_budget(rc_tracer* h, double milliseconds);

/* Film::generateToneMappedImage (Film.cpp:61-69) with the handle's tone
 * mapper (ReinhardToneMapper::apply, ReinhardToneMapper.cpp:18-86), and the
 * download of CLTracer::downloadImage (CLTracer.cpp:307): out_rgba =
 * film pixels x 4 floats on the host (or in device memory). The mapping
 * kernel writes the buffer in place when the device can reach it and it is
 * 16-byte aligned (device memory, page-locked memory, or pageable memory
 * whose pages are all resident on a host whose GPU uses its page tables);
 * otherwise through one copy. Per pixel in float32 (the reference: double),
 * within 4e-6 of the reference's image. */
rc_status rc_resolve(rc_tracer* h, float* out_rgba);

/* Linear film resolve (cumulativeColor / filterWeightSum) to the host, and
 * the raw accumulators (r, g, b, weight per pixel). */
rc_status rc_read_linear(rc_tracer* h, float* out_rgba);
rc_status rc_read_film(rc_tracer* h, float* out_rgbw);

/* Tone-map a caller film (pixels x {r, g, b, weight sum}, host floats) with
 * the handle's tone mapper: Film::generateToneMappedImage on any film
 * (Film.cpp:61-69), e.g. one the CPU-compatible adapter accumulated.
 * Copies in and out are included. */
rc_status rc_tonemap_film(rc_tracer* h, const float* film_rgbw, uint64_t pixels, float* out_rgba);

/* Per-pixel results of the last RAY render (film pixels entries). */
rc_status rc_read_cast(rc_tracer* h, rc_cast_pixel* out);

/* ------------------------------------------------------------------------ */
/* Ray queries through the root BVH — the intersect calls of
 * PathTracer::traceRecursive (PathTracer.cpp:36-40) and
 * Raytracer::calculateShadowAmount (Raytracer.cpp:497-522), batched.
 * any_hit != 0: shadow-ray semantics (isShadowRay + fastOcclusion:
 * nonShadowing triangles skipped, first hit found is reported).
 * n = 0 is an empty batch in every form: RC_OK, nothing read or written.  */

/* Host buffers: rays -> hits, copies included. */
rc_status rc_cast(rc_tracer* h, const rc_ray* rays, int64_t n, int32_t any_hit, int32_t order, rc_hit* hits);

/* Device buffers (device pointers, on the handle's stream); no copies. */
rc_status rc_cast_device(rc_tracer* h, const rc_ray* d_rays, int64_t n, int32_t any_hit, int32_t order,
                         rc_hit* d_hits);

/* Primary + shadow cast of whole frames from host-side primary rays: the
 * RAY render's ray set fed from the host (n rays in, n rc_cast_pixel out,
 * host buffers, copies included). Uses the first directional light. */
rc_status rc_cast_with_shadow(rc_tracer* h, const rc_ray* rays, int64_t n, int32_t order, rc_cast_pixel* out);

/* Allocation-free form of rc_cast_with_shadow on device buffers. No
 * counterpart in the reference: it is for callers that cannot allocate device
 * memory when they trace — an application whose GPU memory belongs to its own
 * pool allocator, or a per-frame callback that cannot take cudaMalloc's
 * implicit synchronisation. d_rays / d_out: n device records (16-byte
 * aligned), on the handle's stream; blocks until done. The work counters and
 * the shadow-ray queue live in a static device array of the library (8 MiB per
 * GPU, held while the process runs): at most 1,048,576 rays per call, larger n
 * returns RC_INVALID_ARG. Every call on every handle shares that array, so
 * calls that overlap on the GPU race. The first call on a device looks up the
 * array's address (once per device); make that first call before any stream
 * capture begins. The rays are a list, walked one ray per lane: even a whole
 * camera frame in pixel order does not get the warp-wide tile walk of RAY
 * renders, so this form is slower than rc_cast_with_shadow on such frames.
 * With rc_set_counting on it runs the counted two-kernel form (same scratch)
 * and reports node and triangle counts; rc_get_stats then describes this
 * call alone, with times of 0. */
rc_status rc_cast_with_shadow_device_noalloc(rc_tracer* h, const rc_ray* d_rays, int64_t n, int32_t order,
                                             rc_cast_pixel* d_out);

/* ------------------------------------------------------------------------ */
/* Batched path tracing: many independent scenes of uneven size rendered as
 * one CUDA-graph launch. No counterpart in the reference (its Tracer::run
 * renders one scene per call); each scene's film equals what a handle of its
 * own would render for the same records (same kernels, same random streams). */

typedef struct rc_batch rc_batch;

typedef struct rc_batch_stats
{
    uint64_t rays_traced;    /* BVH queries of the last rc_batch_render              */
    uint64_t paths;          /* paths started (pixels x samples over all scenes)     */
    double last_ms;          /* device time of the last rc_batch_render              */
    int32_t passes;          /* passes in the graph                                  */
    int32_t scenes;
    int32_t graph_nodes;     /* nodes of the captured graph                          */
    int32_t reserved;
} rc_batch_stats;

/* Per scene-size bucket (by triangle count: < 16k, < 128k, < 1M, >= 1M) the
 * autotuner's choice: path slots per pass (queue size) and threads per block
 * of the extend / shade kernels. */
typedef struct rc_batch_tuning
{
    uint32_t bucket_min_triangles[4];
    uint32_t slots[4];
    int32_t extend_block[4];
    int32_t shade_block[4];
    double measured_paths_per_ms[4];  /* of the chosen configuration (0 = not tuned) */
} rc_batch_tuning;

rc_status rc_batch_create(rc_batch** out, int device);
void rc_batch_destroy(rc_batch* b);
const char* rc_batch_last_error(const rc_batch* b);

/* Adds one scene (triangles and materials as rc_upload_scene; the SAH BVH is
 * built on the host), its camera, its PATH settings and its film size.
 * index receives the scene's index. Invalidates a captured graph. */
rc_status rc_batch_add_scene(rc_batch* b, const double* vertices, const uint32_t* material_index, int64_t n,
                             const rc_material* materials, int32_t material_count, uint32_t max_leaf_size,
                             const rc_camera* camera, const rc_general* general, uint64_t width, uint64_t height,
                             int32_t* index);

/* Times candidate configurations (pass sizes 1M/2M/4M slots x 64/128/256
 * threads per block) on each bucket's first paths and keeps the fastest per
 * bucket; spends at most about budget_ms of device time. Clears the films. */
rc_status rc_batch_autotune(rc_batch* b, double budget_ms);
rc_status rc_batch_get_tuning(const rc_batch* b, rc_batch_tuning* out);

/* One frame of every scene (adds filter-weighted samples to each film) as
 * one graph launch; the graph is captured on the first call after a change.
 * scene_done_ms (optional, `scenes` entries): device time from the launch's
 * start until each scene's last pass finished. Blocks until done. */
rc_status rc_batch_render(rc_batch* b, double* scene_done_ms);
rc_status rc_batch_clear(rc_batch* b);
rc_status rc_batch_read_film(rc_batch* b, int32_t index, float* out_rgbw);
rc_status rc_batch_resolve(rc_batch* b, int32_t index, const rc_tonemapper* tonemapper, float* out_rgba);
rc_status rc_batch_get_stats(const rc_batch* b, rc_batch_stats* out);

/* ------------------------------------------------------------------------ */
/* Options, statistics, synchronisation.                                     */

/* Closest-hit traversal order for renders (rc_traversal_order). */
rc_status rc_set_traversal_order(rc_tracer* h, int32_t order);
/* Count node / triangle tests in kernels (slower; off by default). */
rc_status rc_set_counting(rc_tracer* h, int32_t enable);
rc_status rc_get_stats(const rc_tracer* h, rc_stats* out);
/* The handle's CUDA stream (cudaStream_t) as an opaque pointer. */
void* rc_stream(rc_tracer* h);
rc_status rc_sync(rc_tracer* h);

/* ------------------------------------------------------------------------ */
/* Instanced (two-level) scenes — Instance (Instance.cpp:17-116) placing a  */
/* PrimitiveGroup with its own BVH (PrimitiveGroup.cpp:13-62). Each mesh    */
/* gets the reference's SAH BVH; each instance the reference's transform   */
/* T(c + translate) * R_x(pitch) R_y(yaw) R_z(roll) * S(scale) * T(-c), c  */
/* the mesh's box centre; a BVH over the instances' world boxes finds them. */
/* Geometry that is not instanced is a mesh with an identity instance.     */
/* Traced by rc_cast / rc_cast_device (hit prim = the flattened index:     */
/* the triangles of instance 0, then of instance 1, ...), RAY frames and   */
/* rc_cast_with_shadow (prim and occluder flattened the same way) and PATH */
/* renders, and stored by scene files (version 2); rc_get_bvh and the      */
/* allocation-free entry point take single-level scenes only.              */

typedef struct rc_mesh
{
    const double* vertices;          /* triangle_count * 9 */
    const uint32_t* material_index;  /* triangle_count */
    int64_t triangle_count;
} rc_mesh;

typedef struct rc_instance
{
    int32_t mesh;         /* index into the mesh array                           */
    int32_t material;     /* material for all its triangles (changePrimitive), or -1 */
    double scale[3];      /* Instance::scale                                      */
    double rotate[3];     /* Instance::rotate: pitch, yaw, roll (degrees)          */
    double translate[3];  /* Instance::translate                                  */
} rc_instance;

rc_status rc_upload_instanced(rc_tracer* h, const rc_mesh* meshes, int32_t mesh_count, const rc_instance* instances,
                              int64_t instance_count, const rc_material* materials, int32_t material_count,
                              uint32_t max_leaf_size);

/* ------------------------------------------------------------------------ */
/* Binary scene + BVH cache files (replace Scene::saveToFile / loadFromFile, */
/* Scene.cpp:67-183, and FlatBVH's serialised nodes restored by              */
/* FlatBVH::restore, FlatBVH.h:98-105, for this path; the format is this     */
/* build's own, not cereal's). A file holds the flat BVH in the reference's */
/* form, the primitive order and the device triangle / shading / material   */
/* records: loading builds nothing. A two-level scene's file holds each     */
/* mesh's BVH and records and the instance descriptions; loading rebuilds   */
/* only the BVH over the instances. Every load validates the file (magic,   */
/* version, sizes, a 64-bit checksum, each BVH's structure and depth, the   */
/* triangle records, the instances) before it allocates device memory;      */
/* RC_IO + message on failure.                                               */

typedef struct rc_scene_file_info
{
    uint64_t triangles;
    uint64_t materials;
    uint64_t bvh_nodes;   /* flat (reference-form) nodes (two-level: of all meshes) */
    uint64_t bvh_depth;   /* (two-level: of the deepest mesh BVH) */
    double bounds[6];     /* root box / scene box: min xyz, max xyz */
    uint64_t meshes;      /* 0 for a single-level scene, else the mesh count */
    uint64_t instances;   /* 0 for a single-level scene, else the instance count */
} rc_scene_file_info;

/* Writes the uploaded scene of a handle. */
rc_status rc_save_scene(rc_tracer* h, const char* path);
/* Replaces the handle's scene with the file's (as rc_upload_scene would). */
rc_status rc_load_scene(rc_tracer* h, const char* path);
/* Host only (no GPU): builds the scene rc_upload_scene would upload and
 * writes it. error (optional) receives a message on failure. */
rc_status rc_write_scene_file(const double* vertices, const uint32_t* material_index, int64_t n,
                              const rc_material* materials, int32_t material_count, uint32_t max_leaf_size,
                              const char* path, char* error, int64_t error_capacity);
/* Host only (no GPU): builds the two-level scene rc_upload_instanced would
 * upload (one SAH BVH per mesh) and writes it; rc_load_scene restores it
 * (rebuilding only the top-level BVH over the instances). */
rc_status rc_write_instanced_scene_file(const rc_mesh* meshes, int32_t mesh_count, const rc_instance* instances,
                                        int64_t instance_count, const rc_material* materials, int32_t material_count,
                                        uint32_t max_leaf_size, const char* path, char* error,
                                        int64_t error_capacity);
/* Host only: validates a file and reports its contents. */
rc_status rc_inspect_scene_file(const char* path, rc_scene_file_info* out, char* error, int64_t error_capacity);

/* ------------------------------------------------------------------------ */
/* Neural radiance cache (GPU-only extension; no counterpart in the          */
/* reference, whose PathTracer::traceRecursive always recurses to           */
/* maxPathLength, PathTracer.cpp:30-75).                                     */
/*                                                                           */
/* A small MLP (128 encoded inputs -> 4 x 64 ReLU -> 3, exp output; BF16     */
/* weights and activations, FP32 accumulation on the tensor cores) predicts */
/* the radiance a path would carry from a surface point. When enabled, a    */
/* PATH render ends every path at the hit of `terminate_segment` with a     */
/* cache lookup, except one random slot in each run of `train_stride`,      */
/* which traces the full plain path (and contributes it to the film) and    */
/* records its vertices; after the pass the suffix radiance of each vertex  */
/* becomes a training sample and `train_steps` Adam steps of `train_batch`  */
/* random samples update the cache.                                          */
/*                                                                           */
/* A query is 12 floats: position[3], direction[3] (unit, from the surface  */
/* toward where the path came from), normal[3], diffuse albedo[3].          */

#define RC_NRC_PARAMS 20992       /* packed [out][in] weights: 64x128, 3 x 64x64, 8x64 (rows 3-7 zero) */
#define RC_NRC_QUERY_FLOATS 12
#define RC_NRC_INPUTS 128

typedef struct rc_nrc_config
{
    int32_t enabled;            /* PATH renders use the cache                        */
    int32_t terminate_segment;  /* paths end at the hit of this segment (2)          */
    int32_t train_stride;       /* one training path per this many slots (16)        */
    int32_t train_steps;        /* optimizer steps per render pass (4)               */
    int32_t train_batch;        /* samples per step (16384)                          */
    int32_t min_suffix;         /* vertices a depth-limited suffix needs (3)         */
    float learning_rate;        /* Adam step size (1e-2)                             */
    float beta1;                /* 0.9                                               */
    float beta2;                /* 0.99                                              */
    float epsilon;              /* 1e-8                                              */
    float box_min[3];           /* position-encoding box; box_max <= box_min on any */
    float box_max[3];           /*   axis = the scene's bounds at render time        */
    uint64_t seed;              /* weight initialisation and training-slot choice    */
    int32_t lookup_kernel;      /* RC_NRC_TCGEN05 (tcgen05.mma, TMEM accumulators;   */
                                /* default) or RC_NRC_MMA_SYNC (warp-level mma.sync) */
    int32_t tc_wait_polls;      /* RC_NRC_TCGEN05: polls of each bounded mbarrier    */
                                /* wait for an MMA before the kernel gives up and    */
                                /* the call reports RC_DEVICE_ERROR; 0 = default     */
                                /* (4,194,304); < 0 = none, so every wait gives up   */
                                /* at once (exercises that error path; the kernel    */
                                /* still lets its MMAs finish before it frees TMEM)  */
    int32_t sample_vertices;    /* training samples of a training path:             */
                                /* RC_NRC_LOOKUP_VERTEX (default): only the vertex  */
                                /* at terminate_segment, whose suffix has exactly   */
                                /* the depth budget (max_path_length minus the      */
                                /* segments before it) that a lookup stands for;    */
                                /* RC_NRC_ALL_VERTICES: every diffuse vertex with a */
                                /* long enough suffix (deeper vertices have smaller */
                                /* budgets, so a depth-limited render is biased low */
                                /* where paths reach the limit)                     */
    int32_t reserved;           /* 0                                                 */
} rc_nrc_config;

typedef enum rc_nrc_sample_vertices { RC_NRC_ALL_VERTICES = 0, RC_NRC_LOOKUP_VERTEX = 1 } rc_nrc_sample_vertices;

typedef enum rc_nrc_lookup_kernel { RC_NRC_MMA_SYNC = 0, RC_NRC_TCGEN05 = 1 } rc_nrc_lookup_kernel;

typedef struct rc_nrc_stats
{
    uint64_t lookups;           /* cache lookups of the last render pass            */
    uint64_t training_samples;  /* training samples it produced                     */
    uint64_t steps;             /* optimizer steps taken since configure            */
    float last_loss;            /* loss of the last step (relative L2, mean)        */
    float reserved;
    double train_ms;            /* time of the last render's training work          */
} rc_nrc_stats;

rc_status rc_nrc_defaults(rc_nrc_config* out);
/* (Re)initialises the weights (seeded He-uniform) and the optimizer. */
rc_status rc_nrc_configure(rc_tracer* h, const rc_nrc_config* cfg);
rc_status rc_nrc_set_enabled(rc_tracer* h, int32_t enabled);
/* FP32 master weights, RC_NRC_PARAMS floats; set also resets the optimizer. */
rc_status rc_nrc_get_params(rc_tracer* h, float* params, int64_t count);
rc_status rc_nrc_set_params(rc_tracer* h, const float* params, int64_t count);
/* Cache output (rgb) of n host queries. */
rc_status rc_nrc_infer(rc_tracer* h, const float* queries, int64_t n, float* rgb);
/* The encoded BF16 inputs of n queries, widened to float (n x 128). */
rc_status rc_nrc_encode(rc_tracer* h, const float* queries, int64_t n, float* features);
/* Gradient (RC_NRC_PARAMS floats, [out][in] per layer) and value of the mean
 * relative L2 loss sum((p - y)^2 / (p^2 + 0.01)) / (3 n), the denominator
 * held constant, at the current weights; no update. */
rc_status rc_nrc_gradient(rc_tracer* h, const float* queries, const float* targets, int64_t n, float* grad,
                          float* loss);
/* `steps` Adam steps on one host batch (n <= 1<<20); losses[steps] optional. */
rc_status rc_nrc_train(rc_tracer* h, const float* queries, const float* targets, int64_t n, int32_t steps,
                       float* losses);
/* Training samples of the last render pass: 16 floats each (query[12],
 * target rgb[3], tag), the tag's 32 bits = vertex index << 24 | training
 * path index (slot / train_stride). Ordered by (vertex, path); *count =
 * samples available, at most `capacity` copied. */
rc_status rc_nrc_read_samples(rc_tracer* h, float* records, int64_t capacity, int64_t* count);
rc_status rc_nrc_get_stats(rc_tracer* h, rc_nrc_stats* out);

/* ------------------------------------------------------------------------ */
/* High-spp ground truth and its error (GPU-only extension).                */

/* d_acc (device, 4 doubles per film pixel) += the film's r, g, b, weight
 * sums in float64; clear_film != 0 then zeroes the film (the frame counter
 * keeps running, unlike rc_clear). */
rc_status rc_film_accumulate_f64(rc_tracer* h, double* d_acc, int32_t clear_film);
/* RMSE over all pixels and channels between the display images of the film
 * and of d_truth (4 doubles per pixel): both resolved (rgb / weight) and
 * Reinhard-mapped with the tonemapper record's key, the log-average and
 * maximum luminance taken from d_truth, then gamma and clamp as configured;
 * computed in float64. */
rc_status rc_film_rmse_f64(rc_tracer* h, const double* d_truth, double* rmse);

#ifdef __cplusplus
}
#endif

#endif /* RAYCER_GB300_H */
