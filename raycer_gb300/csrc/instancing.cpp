// Two-level scenes: rc_upload_instanced. Meshes (PrimitiveGroup with its
// BVH, PrimitiveGroup.cpp:13-62) are built with the reference's SAH builder
// into pooled device arrays; instances (Instance, Instance.cpp:17-116) get
// the reference's transform
//   M = T(c + translate) * R_x(pitch) R_y(yaw) R_z(roll) * S(scale) * T(-c),
// c = the mesh's box centre (Instance::initialize), and the reference's
// world box: the mesh box's 8 corners through M (AABB::transformed,
// AABB.cpp:151-186). A top-level SAH BVH over the instance boxes (leaves of
// up to 2 instances) indexes the instance records, which are stored in
// its order. Non-instanced geometry is a mesh with an identity instance.

#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "host_internal.h"

using namespace rcx;

namespace
{

rc_status fail(rc_tracer* h, rc_status s, const std::string& msg)
{
    h->err = msg;
    return s;
}

struct M4
{
    double m[4][4];
};

M4 identity()
{
    M4 r{};
    for (int i = 0; i < 4; ++i)
        r.m[i][i] = 1.0;
    return r;
}

M4 mul(const M4& a, const M4& b)
{
    M4 r{};
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
        {
            double s = 0.0;
            for (int k = 0; k < 4; ++k)
                s += a.m[i][k] * b.m[k][j];
            r.m[i][j] = s;
        }
    return r;
}

M4 translate(double x, double y, double z)
{
    M4 r = identity();
    r.m[0][3] = x;
    r.m[1][3] = y;
    r.m[2][3] = z;
    return r;
}

M4 scale(double x, double y, double z)
{
    M4 r = identity();
    r.m[0][0] = x;
    r.m[1][1] = y;
    r.m[2][2] = z;
    return r;
}

// Matrix4x4::rotateX/Y/Z (Matrix4x4.cpp): angles in degrees.
M4 rotate_axis(int axis, double deg)
{
    const double a = deg * (3.14159265358979323846 / 180.0);
    const double s = std::sin(a), c = std::cos(a);
    M4 r = identity();
    if (axis == 0)
    {
        r.m[1][1] = c;
        r.m[1][2] = -s;
        r.m[2][1] = s;
        r.m[2][2] = c;
    }
    else if (axis == 1)
    {
        r.m[0][0] = c;
        r.m[0][2] = s;
        r.m[2][0] = -s;
        r.m[2][2] = c;
    }
    else
    {
        r.m[0][0] = c;
        r.m[0][1] = -s;
        r.m[1][0] = s;
        r.m[1][1] = c;
    }
    return r;
}

// General 4x4 inverse by cofactors (Matrix4x4::inverted's method).
bool invert(const M4& a, M4& out)
{
    const double* n = &a.m[0][0];
    double inv[16];
    inv[0] = n[5] * n[10] * n[15] - n[5] * n[11] * n[14] - n[9] * n[6] * n[15] + n[9] * n[7] * n[14] +
             n[13] * n[6] * n[11] - n[13] * n[7] * n[10];
    inv[4] = -n[4] * n[10] * n[15] + n[4] * n[11] * n[14] + n[8] * n[6] * n[15] - n[8] * n[7] * n[14] -
             n[12] * n[6] * n[11] + n[12] * n[7] * n[10];
    inv[8] = n[4] * n[9] * n[15] - n[4] * n[11] * n[13] - n[8] * n[5] * n[15] + n[8] * n[7] * n[13] +
             n[12] * n[5] * n[11] - n[12] * n[7] * n[9];
    inv[12] = -n[4] * n[9] * n[14] + n[4] * n[10] * n[13] + n[8] * n[5] * n[14] - n[8] * n[6] * n[13] -
              n[12] * n[5] * n[10] + n[12] * n[6] * n[9];
    inv[1] = -n[1] * n[10] * n[15] + n[1] * n[11] * n[14] + n[9] * n[2] * n[15] - n[9] * n[3] * n[14] -
             n[13] * n[2] * n[11] + n[13] * n[3] * n[10];
    inv[5] = n[0] * n[10] * n[15] - n[0] * n[11] * n[14] - n[8] * n[2] * n[15] + n[8] * n[3] * n[14] +
             n[12] * n[2] * n[11] - n[12] * n[3] * n[10];
    inv[9] = -n[0] * n[9] * n[15] + n[0] * n[11] * n[13] + n[8] * n[1] * n[15] - n[8] * n[3] * n[13] -
             n[12] * n[1] * n[11] + n[12] * n[3] * n[9];
    inv[13] = n[0] * n[9] * n[14] - n[0] * n[10] * n[13] - n[8] * n[1] * n[14] + n[8] * n[2] * n[13] +
              n[12] * n[1] * n[10] - n[12] * n[2] * n[9];
    inv[2] = n[1] * n[6] * n[15] - n[1] * n[7] * n[14] - n[5] * n[2] * n[15] + n[5] * n[3] * n[14] +
             n[13] * n[2] * n[7] - n[13] * n[3] * n[6];
    inv[6] = -n[0] * n[6] * n[15] + n[0] * n[7] * n[14] + n[4] * n[2] * n[15] - n[4] * n[3] * n[14] -
             n[12] * n[2] * n[7] + n[12] * n[3] * n[6];
    inv[10] = n[0] * n[5] * n[15] - n[0] * n[7] * n[13] - n[4] * n[1] * n[15] + n[4] * n[3] * n[13] +
              n[12] * n[1] * n[7] - n[12] * n[3] * n[5];
    inv[14] = -n[0] * n[5] * n[14] + n[0] * n[6] * n[13] + n[4] * n[1] * n[14] - n[4] * n[2] * n[13] -
              n[12] * n[1] * n[6] + n[12] * n[2] * n[5];
    inv[3] = -n[1] * n[6] * n[11] + n[1] * n[7] * n[10] + n[5] * n[2] * n[11] - n[5] * n[3] * n[10] -
             n[9] * n[2] * n[7] + n[9] * n[3] * n[6];
    inv[7] = n[0] * n[6] * n[11] - n[0] * n[7] * n[10] - n[4] * n[2] * n[11] + n[4] * n[3] * n[10] +
             n[8] * n[2] * n[7] - n[8] * n[3] * n[6];
    inv[11] = -n[0] * n[5] * n[11] + n[0] * n[7] * n[9] + n[4] * n[1] * n[11] - n[4] * n[3] * n[9] -
              n[8] * n[1] * n[7] + n[8] * n[3] * n[5];
    inv[15] = n[0] * n[5] * n[10] - n[0] * n[6] * n[9] - n[4] * n[1] * n[10] + n[4] * n[2] * n[9] +
              n[8] * n[1] * n[6] - n[8] * n[2] * n[5];
    const double det = n[0] * inv[0] + n[1] * inv[4] + n[2] * inv[8] + n[3] * inv[12];
    if (det == 0.0 || !std::isfinite(det))
        return false;
    const double rd = 1.0 / det;
    for (int i = 0; i < 16; ++i)
        (&out.m[0][0])[i] = inv[i] * rd;
    return true;
}

// The reference's instance transform about the mesh box's centre c:
// T(c + translate) * R_x(pitch) R_y(yaw) R_z(roll) * S(scale) * T(-c).
M4 instance_transform(const double* meshBox, const rc_instance& r)
{
    double c[3];
    for (int a = 0; a < 3; ++a)
        c[a] = (meshBox[a] + meshBox[3 + a]) * 0.5;  // AABB::getCenter
    return mul(mul(mul(translate(c[0] + r.translate[0], c[1] + r.translate[1], c[2] + r.translate[2]),
                       mul(mul(rotate_axis(0, r.rotate[0]), rotate_axis(1, r.rotate[1])), rotate_axis(2, r.rotate[2]))),
                   scale(r.scale[0], r.scale[1], r.scale[2])),
               translate(-c[0], -c[1], -c[2]));
}

// World box of a mesh box under M: its 8 corners through M (AABB::transformed).
void world_box(const double* mb, const M4& M, double* lo, double* hi)
{
    for (int a = 0; a < 3; ++a)
    {
        lo[a] = 1e300;
        hi[a] = -1e300;
    }
    for (int corner = 0; corner < 8; ++corner)
    {
        const double p[3] = { (corner & 1) ? mb[3] : mb[0], (corner & 2) ? mb[4] : mb[1], (corner & 4) ? mb[5] : mb[2] };
        for (int a = 0; a < 3; ++a)
        {
            const double w = M.m[a][0] * p[0] + M.m[a][1] * p[1] + M.m[a][2] * p[2] + M.m[a][3];
            lo[a] = std::min(lo[a], w);
            hi[a] = std::max(hi[a], w);
        }
    }
}

}  // namespace

namespace rcx
{

void instanced_scene_box(const std::vector<HostScene>& meshes, const rc_instance* instances, int64_t ni, double box[6])
{
    for (int a = 0; a < 3; ++a)
    {
        box[a] = 1e300;
        box[3 + a] = -1e300;
    }
    for (int64_t k = 0; k < ni; ++k)
    {
        const rc_instance& r = instances[k];
        if (r.mesh < 0 || size_t(r.mesh) >= meshes.size())
            continue;
        const HostScene& hs = meshes[size_t(r.mesh)];
        double mb[6];
        for (int a = 0; a < 3; ++a)
        {
            mb[a] = hs.flat[0].bmin[a];
            mb[3 + a] = hs.flat[0].bmax[a];
        }
        double lo[3], hi[3];
        world_box(mb, instance_transform(mb, r), lo, hi);
        for (int a = 0; a < 3; ++a)
        {
            box[a] = std::min(box[a], lo[a]);
            box[3 + a] = std::max(box[3 + a], hi[a]);
        }
    }
}

rc_status check_instanced_args(const rc_mesh* meshes, int32_t mesh_count, const rc_instance* instances,
                               int64_t instance_count, const rc_material* materials, int32_t material_count,
                               uint32_t max_leaf_size, std::string& err)
{
    if (!meshes || mesh_count <= 0 || !instances || instance_count <= 0 || !materials || material_count <= 0)
    {
        err = "null array or empty scene";
        return RC_INVALID_ARG;
    }
    if (max_leaf_size < 1 || max_leaf_size > 15)
    {
        err = "max_leaf_size must be in 1..15";
        return RC_UNSUPPORTED;
    }
    if (instance_count > (int64_t(1) << 24) || material_count > int32_t(kMetaMaterialMask))
    {
        err = "too many instances or materials";
        return RC_UNSUPPORTED;
    }
    for (int32_t i = 0; i < material_count; ++i)
        if ((materials[i].dielectric != 0 && materials[i].dielectric != 1) ||
            (materials[i].dielectric && !(materials[i].ior > 0.0f && std::isfinite(materials[i].ior))))
        {
            err = "rc_material.dielectric must be 0 or 1 with ior > 0";
            return RC_INVALID_ARG;
        }
    return RC_OK;
}

rc_status build_mesh_scenes(const rc_mesh* meshes, int32_t mesh_count, const rc_material* materials,
                            int32_t material_count, uint32_t max_leaf_size, std::vector<HostScene>& out,
                            std::string& err)
{
    out.clear();
    out.resize(static_cast<size_t>(mesh_count));
    int64_t total = 0;
    for (int32_t m = 0; m < mesh_count; ++m)
    {
        const rc_mesh& me = meshes[m];
        const int64_t n = me.triangle_count;
        if (!me.vertices || !me.material_index || n <= 0)
        {
            err = "mesh " + std::to_string(m) + " is empty";
            return RC_INVALID_ARG;
        }
        for (int64_t i = 0; i < n; ++i)
            if (me.material_index[i] >= uint32_t(material_count))
            {
                err = "material index out of range in mesh " + std::to_string(m);
                return RC_INVALID_ARG;
            }
        for (int64_t i = 0; i < n * 9; ++i)
            if (!std::isfinite(me.vertices[i]))
            {
                err = "non-finite vertex in mesh " + std::to_string(m);
                return RC_INVALID_ARG;
            }
        total += n;
        if (total > (int64_t(1) << 27))
        {
            err = "more than 2^27 mesh triangles in total";
            return RC_UNSUPPORTED;
        }
        BuildResult br;
        if (!buildFlatBVH(me.vertices, n, max_leaf_size, 0, br, err))
        {
            err = "mesh " + std::to_string(m) + ": " + err;
            return RC_INVALID_ARG;
        }
        if (br.depth > uint32_t(kMaxStack))
        {
            err = "a mesh BVH is deeper than the traversal stack";
            return RC_UNSUPPORTED;
        }
        build_host_scene(me.vertices, me.material_index, n, materials, material_count, std::move(br.nodes),
                         std::move(br.order), br.depth, out[size_t(m)]);
    }
    return RC_OK;
}

rc_status upload_instanced_scenes(rc_tracer* h, std::vector<HostScene>&& meshScenes, const rc_instance* instances,
                                  int64_t instance_count, int32_t material_count,
                                  std::chrono::steady_clock::time_point t0)
{
    const int32_t mesh_count = int32_t(meshScenes.size());
    cudaSetDevice(h->device);
    // Meshes, pooled (node links and leaf starts offset).
    std::vector<DevNode> nodes;
    std::vector<DevTri> tris;
    std::vector<DevShade> shade;
    std::vector<int32_t> meshRoot(static_cast<size_t>(mesh_count));
    std::vector<double> meshBox(static_cast<size_t>(mesh_count) * 6);
    std::vector<uint32_t> meshDepth(static_cast<size_t>(mesh_count));
    std::vector<int64_t> meshTris(static_cast<size_t>(mesh_count));
    std::vector<int64_t> meshFirst(static_cast<size_t>(mesh_count));
    std::vector<DevMat> mats;
    for (int32_t m = 0; m < mesh_count; ++m)
    {
        HostScene& hs = meshScenes[size_t(m)];
        const int64_t n = int64_t(hs.tris.size());
        for (int k = 0; k < 3; ++k)
        {
            meshBox[size_t(m) * 6 + k] = hs.flat[0].bmin[k];
            meshBox[size_t(m) * 6 + 3 + k] = hs.flat[0].bmax[k];
        }
        std::vector<DevNode> dn;
        int32_t root = 0;
        uint64_t inner = 0;
        device_nodes(hs.flat, dn, root, inner);
        const int32_t nodeBase = int32_t(nodes.size());
        const int32_t triBase = int32_t(tris.size());
        auto relink = [&](int32_t l) -> int32_t {
            if (l >= 0)
                return l + nodeBase;
            const uint32_t code = uint32_t(~l);
            const uint32_t start = (code >> kLeafCountBits) + uint32_t(triBase);
            return ~int32_t((start << kLeafCountBits) | (code & ((1u << kLeafCountBits) - 1u)));
        };
        if (inner > 0)
            for (DevNode& d : dn)
            {
                d.link.x = relink(d.link.x);
                d.link.y = relink(d.link.y);
                nodes.push_back(d);
            }
        meshRoot[size_t(m)] = relink(root);
        meshDepth[size_t(m)] = hs.depth;
        meshTris[size_t(m)] = n;
        meshFirst[size_t(m)] = int64_t(triBase);
        tris.insert(tris.end(), hs.tris.begin(), hs.tris.end());
        shade.insert(shade.end(), hs.shade.begin(), hs.shade.end());
        if (m == 0)
            mats = hs.mats;
    }
    // Instances: transforms, world boxes, flattened primitive numbering.
    const int64_t ni = instance_count;
    std::vector<DevInstance> inst(static_cast<size_t>(ni));
    std::vector<double> boxTris(static_cast<size_t>(ni) * 9);
    int64_t primBase = 0;
    for (int64_t k = 0; k < ni; ++k)
    {
        const rc_instance& r = instances[k];
        if (r.mesh < 0 || r.mesh >= mesh_count)
            return fail(h, RC_INVALID_ARG, "upload_instanced: instance " + std::to_string(k) + " names no mesh");
        if (r.material < -1 || r.material >= material_count)
            return fail(h, RC_INVALID_ARG, "upload_instanced: instance material out of range");
        for (int a = 0; a < 3; ++a)
            if (!std::isfinite(r.scale[a]) || !std::isfinite(r.rotate[a]) || !std::isfinite(r.translate[a]) ||
                r.scale[a] == 0.0)
                return fail(h, RC_INVALID_ARG, "upload_instanced: non-finite or zero transform component");
        const double* mb = &meshBox[size_t(r.mesh) * 6];
        const M4 M = instance_transform(mb, r);
        M4 Mi;
        if (!invert(M, Mi))
            return fail(h, RC_INVALID_ARG, "upload_instanced: singular instance transform");
        const bool ident = r.scale[0] == 1.0 && r.scale[1] == 1.0 && r.scale[2] == 1.0 && r.rotate[0] == 0.0 &&
                           r.rotate[1] == 0.0 && r.rotate[2] == 0.0 && r.translate[0] == 0.0 &&
                           r.translate[1] == 0.0 && r.translate[2] == 0.0;
        DevInstance& d = inst[size_t(k)];
        d.r0 = make_float4(float(Mi.m[0][0]), float(Mi.m[0][1]), float(Mi.m[0][2]), float(Mi.m[0][3]));
        d.r1 = make_float4(float(Mi.m[1][0]), float(Mi.m[1][1]), float(Mi.m[1][2]), float(Mi.m[1][3]));
        d.r2 = make_float4(float(Mi.m[2][0]), float(Mi.m[2][1]), float(Mi.m[2][2]), float(Mi.m[2][3]));
        d.rootLink = meshRoot[size_t(r.mesh)];
        d.material = r.material;
        d.primBase = int32_t(primBase);
        d.identity = ident ? 1 : 0;
        primBase += meshTris[size_t(r.mesh)];
        // world box: the mesh box's corners through M
        double lo[3], hi[3];
        world_box(mb, M, lo, hi);
        // the SAH builder takes triangles: (lo, hi, hi) has this box and centre
        for (int a = 0; a < 3; ++a)
        {
            boxTris[size_t(k) * 9 + a] = lo[a];
            boxTris[size_t(k) * 9 + 3 + a] = hi[a];
            boxTris[size_t(k) * 9 + 6 + a] = hi[a];
        }
    }
    if (primBase > (int64_t(1) << 31) - 1)
        return fail(h, RC_UNSUPPORTED, "upload_instanced: more than 2^31 flattened primitives");

    BuildResult tb;
    std::string err;
    double sceneBox[6] = { 1e300, 1e300, 1e300, -1e300, -1e300, -1e300 };
    for (int64_t k = 0; k < ni; ++k)
        for (int a = 0; a < 3; ++a)
        {
            sceneBox[a] = std::min(sceneBox[a], boxTris[size_t(k) * 9 + a]);
            sceneBox[3 + a] = std::max(sceneBox[3 + a], boxTris[size_t(k) * 9 + 3 + a]);
        }
    if (!buildFlatBVH(boxTris.data(), ni, 2, 0, tb, err))
        return fail(h, RC_INVALID_ARG, "upload_instanced: top-level build: " + err);
    if (tb.depth > 32)
        return fail(h, RC_UNSUPPORTED, "upload_instanced: top-level BVH deeper than 32");
    std::vector<DevNode> tn;
    int32_t troot = 0;
    uint64_t tinner = 0;
    device_nodes(tb.nodes, tn, troot, tinner);
    std::vector<DevInstance> ordered(static_cast<size_t>(ni));
    for (int64_t s = 0; s < ni; ++s)
        ordered[size_t(s)] = inst[tb.order[size_t(s)]];
    if (nodes.empty())
        nodes.push_back(DevNode{});

    release_scene_data(h);
    void* pN = nullptr;
    void* pT = nullptr;
    void* pS = nullptr;
    void* pM = nullptr;
    void* pTl = nullptr;
    void* pI = nullptr;
    cudaError_t e = cudaMalloc(&pN, nodes.size() * sizeof(DevNode));
    if (e == cudaSuccess)
        e = cudaMalloc(&pT, tris.size() * sizeof(DevTri));
    if (e == cudaSuccess)
        e = cudaMalloc(&pS, shade.size() * sizeof(DevShade));
    if (e == cudaSuccess)
        e = cudaMalloc(&pM, mats.size() * sizeof(DevMat));
    if (e == cudaSuccess)
        e = cudaMalloc(&pTl, tn.size() * sizeof(DevNode));
    if (e == cudaSuccess)
        e = cudaMalloc(&pI, ordered.size() * sizeof(DevInstance));
    if (e == cudaSuccess)
        e = cudaMemcpy(pN, nodes.data(), nodes.size() * sizeof(DevNode), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(pT, tris.data(), tris.size() * sizeof(DevTri), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(pS, shade.data(), shade.size() * sizeof(DevShade), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(pM, mats.data(), mats.size() * sizeof(DevMat), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(pTl, tn.data(), tn.size() * sizeof(DevNode), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(pI, ordered.data(), ordered.size() * sizeof(DevInstance), cudaMemcpyHostToDevice);
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        cudaFree(pN);
        cudaFree(pT);
        cudaFree(pS);
        cudaFree(pM);
        cudaFree(pTl);
        cudaFree(pI);
        return fail(h, e == cudaErrorMemoryAllocation ? RC_OOM : RC_CUDA,
                    std::string("upload_instanced: ") + cudaGetErrorString(e));
    }
    h->dNodes = static_cast<DevNode*>(pN);
    h->dTris = static_cast<DevTri*>(pT);
    h->dShade = static_cast<DevShade*>(pS);
    h->dMats = static_cast<DevMat*>(pM);
    h->dTlas = static_cast<DevNode*>(pTl);
    h->dInstances = static_cast<DevInstance*>(pI);
    h->innerCount = nodes.size();
    h->nTris = int64_t(tris.size());
    h->nMats = material_count;
    h->tlasCount = tn.size();
    h->nInstances = ni;
    h->tlasRoot = troot;
    h->rootLink = meshRoot[0];
    uint32_t depth = 0;
    for (uint32_t d : meshDepth)
        depth = std::max(depth, d);
    h->bvhDepth = depth + tb.depth;
    h->bvhInner = nodes.size() + tn.size();
    h->deviceBytes += nodes.size() * sizeof(DevNode) + tris.size() * (sizeof(DevTri) + sizeof(DevShade)) +
                      mats.size() * sizeof(DevMat) + tn.size() * sizeof(DevNode) + ordered.size() * sizeof(DevInstance);
    h->hostNodes.clear();
    h->hostOrder.clear();
    // kept for rc_save_scene: each mesh's flat BVH, order and place in the
    // pooled triangle arrays, and the instance descriptions
    h->instMeshes.clear();
    h->instMeshes.resize(static_cast<size_t>(mesh_count));
    for (int32_t m = 0; m < mesh_count; ++m)
    {
        InstancedMesh& im = h->instMeshes[size_t(m)];
        im.flat = std::move(meshScenes[size_t(m)].flat);
        im.order = std::move(meshScenes[size_t(m)].order);
        im.depth = meshDepth[size_t(m)];
        im.firstTri = meshFirst[size_t(m)];
        im.triangles = meshTris[size_t(m)];
    }
    h->instDescs.assign(instances, instances + ni);
    for (int k = 0; k < 6; ++k)
        h->bounds[k] = sceneBox[k];
    h->sceneReady = true;
    h->stats.build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return RC_OK;
}

}  // namespace rcx

extern "C" rc_status rc_upload_instanced(rc_tracer* h, const rc_mesh* meshes, int32_t mesh_count,
                                         const rc_instance* instances, int64_t instance_count,
                                         const rc_material* materials, int32_t material_count,
                                         uint32_t max_leaf_size)
{
    if (!h)
        return RC_INVALID_ARG;
    std::string err;
    rc_status s = check_instanced_args(meshes, mesh_count, instances, instance_count, materials, material_count,
                                       max_leaf_size, err);
    if (s != RC_OK)
        return fail(h, s, "upload_instanced: " + err);
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<HostScene> meshScenes;
    if ((s = build_mesh_scenes(meshes, mesh_count, materials, material_count, max_leaf_size, meshScenes, err)) !=
        RC_OK)
        return fail(h, s, "upload_instanced: " + err);
    return upload_instanced_scenes(h, std::move(meshScenes), instances, instance_count, material_count, t0);
}
