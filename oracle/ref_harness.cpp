// Test infrastructure only: NOT part of the product.
//
// C harness around the reference's own CPU hot path (mikoro/raycer, compiled
// unmodified from its sources by oracle/Makefile.ref). It lets the tests and
// the fixture generator drive the reference's Scene / FlatBVH / Triangle /
// Camera / Tracer / Film / ReinhardToneMapper code with plain arrays:
//
//   * Scene set-up + Scene::initialize (src/Raytracing/Scene.cpp:203-500),
//     which builds the root FlatBVH (src/Raytracing/Primitives/FlatBVH.cpp:89).
//   * Read back the flat node array and orderedPrimitiveIds (FlatBVH.h:84-85).
//   * Camera::setImagePlaneSize + Camera::update (Camera.cpp:29, :48) and the
//     float32 camera record CLScene::readSceneCamera builds (CLScene.cpp:242).
//   * Closest-hit / any-hit queries through the root BVH
//     (FlatBVH::intersect FlatBVH.cpp:22, Triangle::intersect Triangle.cpp:51).
//   * Tracer::run (Tracer.cpp:58) for the PATH and RAY tracers, with a
//     counting wrapper as primitives.visible[0] to count BVH queries, and
//     Film::generateToneMappedImage (Film.cpp:61).
//   * ValueNoise (Utils/ValueNoise.cpp:26-97), MathUtils::fastPow
//     (MathUtils.cpp:56), CMJ / hemisphere sampling.
//
// It also provides the few App/ModelLoader symbols the compiled subset of the
// reference refers to (the GUI/OpenCL/network parts are not compiled).

#include "stdafx.h"

#include "App.h"
#include "Settings.h"
#include "Utils/Log.h"
#include "Utils/ModelLoader.h"
#include "Utils/ValueNoise.h"
#include "Runners/WindowRunner.h"
#include "Raytracing/Scene.h"
#include "Raytracing/Ray.h"
#include "Raytracing/Intersection.h"
#include "Raytracing/Primitives/FlatBVH.h"
#include "Raytracing/Primitives/Triangle.h"
#include "Raytracing/Primitives/PrimitiveGroup.h"
#include "Raytracing/Primitives/Instance.h"
#include "Raytracing/Tracers/Tracer.h"
#include "Raytracing/Tracers/TracerState.h"
#include "Rendering/Film.h"
#include "Rendering/Image.h"
#include "Rendering/Samplers/CMJSampler.h"
#include "Rendering/Filters/Filter.h"
#include "Rendering/ToneMappers/ReinhardToneMapper.h"
#include "Math/MathUtils.h"
#include "Math/Vector2.h"
#include "Math/ONB.h"

using namespace Raycer;

// ---------------------------------------------------------------------------
// App / loader symbols needed by the compiled subset.

namespace
{
    Log& harnessLog()
    {
        static Log log;
        static bool init = false;
        if (!init)
        {
            log.setMinimumMessageLevel(LogMessageLevel::ERROR);
            init = true;
        }
        return log;
    }

    Settings& harnessSettings()
    {
        static Settings settings{};
        return settings;
    }

    WindowRunner& harnessWindowRunner()
    {
        static WindowRunner runner;
        return runner;
    }
}

Log& App::getLog() { return harnessLog(); }
Settings& App::getSettings() { return harnessSettings(); }
WindowRunner& App::getWindowRunner() { return harnessWindowRunner(); }

ModelLoaderResult ModelLoader::readObjFile(const ModelLoaderInfo& info)
{
    (void)info;
    throw std::runtime_error("OBJ loading is not part of the oracle build");
}

// Friend of Camera (Camera.h declares `friend class CLScene`): the OpenCL
// directory is not compiled here, so this harness-only class can read the
// camera state the same way CLScene::readSceneCamera does.
namespace Raycer
{
    class CLScene
    {
    public:
        static void readCamera(const Camera& c, double* out)
        {
            const CameraState& s = c.cameraState;
            const Vector3* v[5] = { &s.position, &s.forward, &s.right, &s.up, &s.imagePlaneCenter };
            for (int i = 0; i < 5; ++i)
            {
                out[i * 3 + 0] = v[i]->x;
                out[i * 3 + 1] = v[i]->y;
                out[i * 3 + 2] = v[i]->z;
            }
            out[15] = c.aspectRatio;
            out[16] = c.imagePlaneWidth;
            out[17] = c.imagePlaneHeight;
            out[18] = c.imagePlaneDistance;
        }
    };
}

// ---------------------------------------------------------------------------
// Counting wrapper: forwards to the root BVH and counts queries per thread.

namespace
{
    struct alignas(64) PaddedCounter
    {
        uint64_t value = 0;
    };

    class CountingPrimitive : public Primitive
    {
    public:
        void initialize(const Scene&) override {}
        bool intersect(const Ray& ray, Intersection& intersection, std::vector<Intersection>& intersections) override
        {
            counters[size_t(omp_get_thread_num()) % counters.size()].value++;
            return target->intersect(ray, intersection, intersections);
        }
        AABB getAABB() const override { return target->getAABB(); }
        void transform(const Vector3&, const EulerAngle&, const Vector3&) override {}

        Primitive* target = nullptr;
        std::vector<PaddedCounter> counters = std::vector<PaddedCounter>(512);

        uint64_t total() const
        {
            uint64_t sum = 0;
            for (const auto& c : counters)
                sum += c.value;
            return sum;
        }
        void reset()
        {
            for (auto& c : counters)
                c.value = 0;
        }
    };

    struct RefScene
    {
        Scene scene;
        CountingPrimitive counter;
        bool initialized = false;
        std::string error;
    };

    RefScene* S(void* h) { return static_cast<RefScene*>(h); }
}

extern "C" {

void* ref_scene_new()
{
    return new RefScene();
}

void ref_scene_free(void* h)
{
    delete S(h);
}

// Triangles: v = n*9 doubles (v0, v1, v2); materialIds[n]. Primitive ids are
// firstId + i (ids must be non-zero and unique, Scene.cpp:327-336).
void ref_scene_add_triangles(void* h, int64_t n, const double* v, const uint64_t* materialIds, uint64_t firstId)
{
    Scene& scene = S(h)->scene;
    scene.primitives.triangles.reserve(scene.primitives.triangles.size() + size_t(n));
    for (int64_t i = 0; i < n; ++i)
    {
        Triangle t;
        t.id = firstId + uint64_t(i);
        t.materialId = materialIds[i];
        for (int k = 0; k < 3; ++k)
        {
            t.vertices[k] = Vector3(v[i * 9 + k * 3 + 0], v[i * 9 + k * 3 + 1], v[i * 9 + k * 3 + 2]);
            t.normals[k] = Vector3(0.0, 0.0, 0.0);
        }
        scene.primitives.triangles.push_back(t);
    }
}

// A mesh placed by instances: its triangles (ids firstTriId + i) are
// invisible and grouped in a PrimitiveGroup with its own BVH (id groupId);
// each instance k (id firstInstanceId + k) references the group with
// srt[k] = scale xyz, rotate pitch/yaw/roll (degrees), translate xyz. With
// changePrimitive off, hits report the mesh triangle (Instance.cpp:93).
void ref_scene_add_instanced_mesh(void* h, int64_t n, const double* v, const uint64_t* materialIds,
                                  uint64_t firstTriId, uint64_t groupId, int64_t instances, const double* srt,
                                  uint64_t firstInstanceId)
{
    Scene& scene = S(h)->scene;
    PrimitiveGroup group;
    group.id = groupId;
    group.invisible = true;
    group.enableBVH = true;
    for (int64_t i = 0; i < n; ++i)
    {
        Triangle t;
        t.id = firstTriId + uint64_t(i);
        t.materialId = materialIds[i];
        t.invisible = true;
        for (int k = 0; k < 3; ++k)
        {
            t.vertices[k] = Vector3(v[i * 9 + k * 3 + 0], v[i * 9 + k * 3 + 1], v[i * 9 + k * 3 + 2]);
            t.normals[k] = Vector3(0.0, 0.0, 0.0);
        }
        scene.primitives.triangles.push_back(t);
        group.primitiveIds.push_back(t.id);
    }
    scene.primitives.primitiveGroups.push_back(group);
    for (int64_t k = 0; k < instances; ++k)
    {
        const double* p = srt + k * 9;
        Instance in;
        in.id = firstInstanceId + uint64_t(k);
        in.primitiveId = groupId;
        in.materialId = materialIds[0];
        in.scale = Vector3(p[0], p[1], p[2]);
        in.rotate = EulerAngle(p[3], p[4], p[5]);
        in.translate = Vector3(p[6], p[7], p[8]);
        in.changePrimitive = false;
        scene.primitives.instances.push_back(in);
    }
}

void ref_scene_add_material(void* h, uint64_t id, const double* diffuse, const double* emittance, int isEmissive, int nonShadowing)
{
    Material m;
    m.id = id;
    m.diffuseReflectance = Color(diffuse[0], diffuse[1], diffuse[2]);
    m.emittance = Color(emittance[0], emittance[1], emittance[2]);
    m.isEmissive = isEmissive != 0;
    m.nonShadowing = nonShadowing != 0;
    S(h)->scene.materials.push_back(m);
}

void ref_scene_add_directional_light(void* h, const double* direction, const double* color, double intensity)
{
    DirectionalLight l;
    l.direction = Vector3(direction[0], direction[1], direction[2]);
    l.color = Color(color[0], color[1], color[2]);
    l.intensity = intensity;
    S(h)->scene.lights.directionalLights.push_back(l);
}

void ref_scene_set_ambient(void* h, const double* color, double intensity)
{
    S(h)->scene.lights.ambientLight.color = Color(color[0], color[1], color[2]);
    S(h)->scene.lights.ambientLight.intensity = intensity;
}

void ref_scene_set_camera(void* h, const double* position, double pitch, double yaw, double roll, double fov)
{
    Camera& c = S(h)->scene.camera;
    c.position = Vector3(position[0], position[1], position[2]);
    c.orientation = EulerAngle(pitch, yaw, roll);
    c.fov = fov;
    c.projectionType = CameraProjectionType::PERSPECTIVE;
}

// tracerType: 0 RAY, 1 PATH. samplerType / filterType are the reference's
// enum values (SamplerType, FilterType).
void ref_scene_set_general(void* h, int tracerType, uint64_t maxPathLength, uint64_t pathSampleCount,
                           uint64_t multiSampleCountSqrt, int samplerType, int filterType, double rayStartOffset)
{
    Scene::General& g = S(h)->scene.general;
    g.tracerType = tracerType == 0 ? TracerType::RAY : TracerType::PATH;
    g.maxPathLength = maxPathLength;
    g.pathSampleCount = pathSampleCount;
    g.multiSampleCountSqrt = multiSampleCountSqrt;
    g.multiSamplerType = SamplerType(samplerType);
    g.multiSamplerFilterType = FilterType(filterType);
    g.rayStartOffset = rayStartOffset;
}

// type: reference ToneMapperType value (REINHARD = 3).
void ref_scene_set_tonemapper(void* h, int type, int applyGamma, int shouldClamp, double gamma, double key)
{
    Scene::ToneMapper& t = S(h)->scene.toneMapper;
    t.type = ToneMapperType(type);
    t.applyGamma = applyGamma != 0;
    t.shouldClamp = shouldClamp != 0;
    t.gamma = gamma;
    t.key = key;
}

// Scene::initialize with the root BVH enabled (SAH, MEDIAN, regularSAHSplits
// 0 - the BVHBuildInfo defaults - and the given maxLeafSize). Returns 0 or -1
// (message via ref_last_error).
int ref_scene_initialize(void* h, uint64_t maxLeafSize)
{
    RefScene* rs = S(h);
    try
    {
        rs->scene.rootBVH.enabled = true;
        rs->scene.rootBVH.buildInfo.maxLeafSize = maxLeafSize;
        rs->scene.initialize();
        rs->counter.target = rs->scene.primitives.visible.at(0);
        rs->initialized = true;
        return 0;
    }
    catch (const std::exception& e)
    {
        rs->error = e.what();
        return -1;
    }
}

const char* ref_last_error(void* h)
{
    return S(h)->error.c_str();
}

int64_t ref_bvh_node_count(void* h)
{
    return int64_t(S(h)->scene.rootBVH.bvh.flatNodes.size());
}

void ref_bvh_nodes(void* h, double* aabb6, int64_t* rightOffset, uint64_t* startOffset, uint64_t* primitiveCount)
{
    const auto& nodes = S(h)->scene.rootBVH.bvh.flatNodes;
    for (size_t i = 0; i < nodes.size(); ++i)
    {
        Vector3 mn = nodes[i].aabb.getMin();
        Vector3 mx = nodes[i].aabb.getMax();
        aabb6[i * 6 + 0] = mn.x; aabb6[i * 6 + 1] = mn.y; aabb6[i * 6 + 2] = mn.z;
        aabb6[i * 6 + 3] = mx.x; aabb6[i * 6 + 4] = mx.y; aabb6[i * 6 + 5] = mx.z;
        rightOffset[i] = nodes[i].rightOffset;
        startOffset[i] = nodes[i].startOffset;
        primitiveCount[i] = nodes[i].primitiveCount;
    }
}

void ref_bvh_ordered_ids(void* h, uint64_t* ids)
{
    const auto& v = S(h)->scene.rootBVH.bvh.orderedPrimitiveIds;
    for (size_t i = 0; i < v.size(); ++i)
        ids[i] = v[i];
}

// Triangle::initialize results (normal, tangent, bitangent) for triangle i
// (in the caller's order): out = 9 doubles.
void ref_triangle_frame(void* h, int64_t i, double* out)
{
    const Triangle& t = S(h)->scene.primitives.triangles.at(size_t(i));
    const Vector3* v[3] = { &t.normal, &t.tangent, &t.bitangent };
    for (int k = 0; k < 3; ++k)
    {
        out[k * 3 + 0] = v[k]->x;
        out[k * 3 + 1] = v[k]->y;
        out[k * 3 + 2] = v[k]->z;
    }
}

// Camera::setImagePlaneSize(w, h) + Camera::update(scene, 0). out[19]:
// position, forward, right, up, imagePlaneCenter (3 each), aspectRatio,
// imagePlaneWidth, imagePlaneHeight, imagePlaneDistance.
void ref_camera_state(void* h, uint64_t width, uint64_t height, double* out)
{
    Scene& scene = S(h)->scene;
    scene.camera.setImagePlaneSize(width, height);
    scene.camera.update(scene, 0.0);
    CLScene::readCamera(scene.camera, out);
}

// Camera::getRay for n pixel coordinates (xy pairs, doubles); rays6 out.
void ref_camera_rays(void* h, int64_t n, const double* xy, double* rays6)
{
    const Scene& scene = S(h)->scene;
    for (int64_t i = 0; i < n; ++i)
    {
        Ray ray;
        scene.camera.getRay(Vector2(xy[i * 2], xy[i * 2 + 1]), ray, 0.0);
        rays6[i * 6 + 0] = ray.origin.x; rays6[i * 6 + 1] = ray.origin.y; rays6[i * 6 + 2] = ray.origin.z;
        rays6[i * 6 + 3] = ray.direction.x; rays6[i * 6 + 4] = ray.direction.y; rays6[i * 6 + 5] = ray.direction.z;
    }
}

// Root-BVH queries for n rays (origin, direction as 6 doubles). shadow != 0
// sets isShadowRay + fastOcclusion (the shadow-ray set-up of
// Raytracer::calculateShadowAmount, Raytracer.cpp:497-522). Outputs: prim =
// (primitive id - idBase) of the reported hit or -1, t (hit distance or -1).
void ref_intersect(void* h, int64_t n, const double* rays6, int shadow, uint64_t idBase, int64_t* prim, double* t, int threads)
{
    Scene& scene = S(h)->scene;
    Primitive* root = scene.primitives.visible.at(0);
    if (threads > 0)
        omp_set_num_threads(threads);

    #pragma omp parallel for schedule(dynamic, 1000)
    for (int64_t i = 0; i < n; ++i)
    {
        Ray ray;
        ray.origin = Vector3(rays6[i * 6 + 0], rays6[i * 6 + 1], rays6[i * 6 + 2]);
        ray.direction = Vector3(rays6[i * 6 + 3], rays6[i * 6 + 4], rays6[i * 6 + 5]);
        if (shadow)
        {
            ray.isShadowRay = true;
            ray.fastOcclusion = true;
            ray.maxDistance = std::numeric_limits<double>::max();
        }
        ray.precalculate();

        Intersection isect;
        std::vector<Intersection> tmp;
        root->intersect(ray, isect, tmp);

        if (isect.wasFound)
        {
            prim[i] = int64_t(isect.primitive->id - idBase);
            t[i] = isect.distance;
        }
        else
        {
            prim[i] = -1;
            t[i] = -1.0;
        }
    }
}

// Tracer::run over the whole film (pixelStartOffset 0, pixelCount w*h), then
// Film::generateToneMappedImage. The counting wrapper replaces
// primitives.visible[0] for the run so every root-BVH query is counted.
// linearRgba / toneMappedRgba: w*h*4 floats (either may be null).
// Returns 0 or -1.
int ref_render(void* h, uint64_t width, uint64_t height, int threads,
               float* linearRgba, float* toneMappedRgba, uint64_t* rayCount, double* seconds)
{
    RefScene* rs = S(h);
    Scene& scene = rs->scene;
    try
    {
        App::getSettings().general.maxThreadCount = threads > 0 ? threads : omp_get_num_procs();
        scene.camera.setImagePlaneSize(width, height);
        scene.camera.update(scene, 0.0);

        Film film;
        film.resize(width, height);

        TracerState state;
        state.scene = &scene;
        state.film = &film;
        state.filmWidth = width;
        state.filmHeight = height;
        state.pixelStartOffset = 0;
        state.pixelCount = width * height;

        Primitive* original = scene.primitives.visible.at(0);
        rs->counter.target = original;
        rs->counter.reset();
        scene.primitives.visible[0] = &rs->counter;

        std::unique_ptr<Tracer> tracer = Tracer::getTracer(scene.general.tracerType);
        std::atomic<bool> interrupted(false);

        auto t0 = std::chrono::high_resolution_clock::now();
        tracer->run(state, interrupted);
        auto t1 = std::chrono::high_resolution_clock::now();

        scene.primitives.visible[0] = original;

        if (seconds)
            *seconds = std::chrono::duration<double>(t1 - t0).count();
        if (rayCount)
            *rayCount = rs->counter.total();

        if (linearRgba || toneMappedRgba)
        {
            film.generateToneMappedImage(scene);
        }
        if (toneMappedRgba)
        {
            const auto& px = film.getToneMappedImage().getPixelDataConst();
            for (size_t i = 0; i < px.size(); ++i)
            {
                toneMappedRgba[i * 4 + 0] = px[i].r;
                toneMappedRgba[i * 4 + 1] = px[i].g;
                toneMappedRgba[i * 4 + 2] = px[i].b;
                toneMappedRgba[i * 4 + 3] = px[i].a;
            }
        }
        if (linearRgba)
        {
            // Film keeps its linear image (cumulativeColor / filterWeightSum,
            // Film.cpp:63-64) private; the PASSTHROUGH tone mapper copies it
            // out unchanged.
            Scene::ToneMapper saved = scene.toneMapper;
            scene.toneMapper.type = ToneMapperType::PASSTHROUGH;
            film.generateToneMappedImage(scene);
            const auto& px = film.getToneMappedImage().getPixelDataConst();
            for (size_t i = 0; i < px.size(); ++i)
            {
                linearRgba[i * 4 + 0] = px[i].r;
                linearRgba[i * 4 + 1] = px[i].g;
                linearRgba[i * 4 + 2] = px[i].b;
                linearRgba[i * 4 + 3] = px[i].a;
            }
            scene.toneMapper = saved;
        }
        return 0;
    }
    catch (const std::exception& e)
    {
        rs->error = e.what();
        return -1;
    }
}

// ReinhardToneMapper::apply on a caller-supplied linear image (w*h*4 floats).
void ref_tonemap_reinhard(int64_t pixelCount, const float* linearRgba, double key, double gamma,
                          int shouldClamp, int applyGamma, float* outRgba)
{
    Scene scene;
    scene.toneMapper.type = ToneMapperType::REINHARD;
    scene.toneMapper.key = key;
    scene.toneMapper.gamma = gamma;
    scene.toneMapper.shouldClamp = shouldClamp != 0;
    scene.toneMapper.applyGamma = applyGamma != 0;
    scene.toneMapper.enableAveraging = false;

    Image in(uint64_t(pixelCount), 1);
    Image out(uint64_t(pixelCount), 1);
    for (int64_t i = 0; i < pixelCount; ++i)
        in.setPixel(uint64_t(i), Colorf(linearRgba[i * 4 + 0], linearRgba[i * 4 + 1], linearRgba[i * 4 + 2], linearRgba[i * 4 + 3]).toColor());

    ReinhardToneMapper tm;
    tm.apply(scene, in, out);

    const auto& px = out.getPixelDataConst();
    for (int64_t i = 0; i < pixelCount; ++i)
    {
        outRgba[i * 4 + 0] = px[size_t(i)].r;
        outRgba[i * 4 + 1] = px[size_t(i)].g;
        outRgba[i * 4 + 2] = px[size_t(i)].b;
        outRgba[i * 4 + 3] = px[size_t(i)].a;
    }
}

double ref_fastpow(double a, double b)
{
    return MathUtils::fastPow(a, b);
}

// ValueNoise(seed).getFbmNoise(octaves, lacunarity, persistence, x, y, z)
// for n points (xyz triples); octaves == 0 -> plain getNoise.
void ref_value_noise(uint32_t seed, int64_t n, const double* xyz, uint64_t octaves, double lacunarity,
                     double persistence, double* out)
{
    ValueNoise noise(seed);
    for (int64_t i = 0; i < n; ++i)
    {
        if (octaves == 0)
            out[i] = noise.getNoise(xyz[i * 3], xyz[i * 3 + 1], xyz[i * 3 + 2]);
        else
            out[i] = noise.getFbmNoise(octaves, lacunarity, persistence, xyz[i * 3], xyz[i * 3 + 1], xyz[i * 3 + 2]);
    }
}

// CMJSampler::getSample2D for every (x, y) of an n x n pattern with the given
// permutation; the random jitter comes from std::mt19937(seed). out: n*n*2.
// jitter (optional, n*n*2): the uniform draws the sampler consumed, in order
// (taken from a second generator with the same seed).
void ref_cmj_pattern(uint64_t n, uint64_t permutation, uint32_t seed, double* out, double* jitter)
{
    if (jitter)
    {
        std::mt19937 twin(seed);
        std::uniform_real_distribution<double> u(0.0, 1.0);
        for (uint64_t i = 0; i < n * n * 2; ++i)
            jitter[i] = u(twin);
    }
    CMJSampler sampler;
    std::mt19937 gen(seed);
    for (uint64_t y = 0; y < n; ++y)
        for (uint64_t x = 0; x < n; ++x)
        {
            Vector2 s = sampler.getSample2D(x, y, n, n, permutation, gen);
            out[(y * n + x) * 2 + 0] = s.x;
            out[(y * n + x) * 2 + 1] = s.y;
        }
}

// The reference's film filter (Filter::getFilter, default constructors as
// the Tracer makes them, Tracer.cpp:50-55): weight of one axis at offsets x.
void ref_filter_weight(int type, int64_t n, const double* x, double* out, double* radius)
{
    std::unique_ptr<Filter> f = Filter::getFilter(FilterType(type));
    for (int64_t i = 0; i < n; ++i)
        out[i] = f->getWeightX(x[i]);
    *radius = f->getRadiusX();
}

}
