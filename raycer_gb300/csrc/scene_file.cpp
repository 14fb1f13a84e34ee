// Binary scene + BVH cache files: the GPU path's replacement for the
// reference's scene serialisation (Scene::saveToFile / loadFromFile with
// cereal archives, Scene.cpp:67-183, and FlatBVH's serialised nodes +
// orderedPrimitiveIds restored by FlatBVH::restore, FlatBVH.h:98-105). A
// file holds what a render needs and nothing is rebuilt on load: the
// reference-form flat BVH, the primitive order, the triangle and shading
// records in BVH order and the materials. The device nodes are derived from
// the flat BVH after it has been validated.
//
// Layout (little-endian, both hosts of this build are):
//   header, 128 bytes:
//     char     magic[8]      "RCGBSCN1"
//     uint32   version       1
//     uint32   headerBytes   128
//     uint64   triangles, materials, flatNodes
//     uint32   depth, reserved
//     uint64   payloadBytes
//     uint64   checksum      of the payload (below)
//     double   bounds[6]     root box min xyz, max xyz
//   payload:
//     rc_bvh_node[flatNodes]  72 B each (FlatBVHNode fields)
//     uint32[triangles]       primitive order (caller index of BVH slot i)
//     DevTri[triangles]       48 B, DevShade[triangles] 48 B, DevMat[materials] 32 B
// Checksum: 64-bit words w of the payload (zero-padded tail), h = (h ^ w) *
// 0x100000001b3 from 0xcbf29ce484222325, then a final avalanche (the
// FNV-1a constants applied per word; a corruption check, not a
// cryptographic one).
//
// Loading validates, before any device allocation: magic, version, sizes,
// checksum, the flat BVH's structure (validate_flat_bvh), the traversal
// depth, and each triangle record against the order and the material count.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "host_internal.h"

using namespace rcx;

namespace
{

constexpr char kMagic[8] = { 'R', 'C', 'G', 'B', 'S', 'C', 'N', '1' };
constexpr uint32_t kVersion = 1;

struct FileHeader
{
    char magic[8];
    uint32_t version;
    uint32_t headerBytes;
    uint64_t triangles;
    uint64_t materials;
    uint64_t flatNodes;
    uint32_t depth;
    uint32_t reserved;
    uint64_t payloadBytes;
    uint64_t checksum;
    double bounds[6];
    unsigned char pad[128 - 8 - 4 - 4 - 8 * 3 - 4 - 4 - 8 - 8 - 48];
};
static_assert(sizeof(FileHeader) == 128, "scene file header is 128 bytes");
static_assert(sizeof(rc_bvh_node) == 72 && sizeof(DevTri) == 48 && sizeof(DevShade) == 48 && sizeof(DevMat) == 32,
              "scene file record sizes");

struct Checksum
{
    uint64_t h = 0xcbf29ce484222325ull;
    unsigned char tail[8];
    size_t tailLen = 0;

    void word(uint64_t w) { h = (h ^ w) * 0x100000001b3ull; }
    void add(const void* data, size_t bytes)
    {
        const unsigned char* p = static_cast<const unsigned char*>(data);
        while (tailLen > 0 && bytes > 0)
        {
            tail[tailLen++] = *p++;
            --bytes;
            if (tailLen == 8)
            {
                uint64_t w;
                std::memcpy(&w, tail, 8);
                word(w);
                tailLen = 0;
            }
        }
        for (; bytes >= 8; bytes -= 8, p += 8)
        {
            uint64_t w;
            std::memcpy(&w, p, 8);
            word(w);
        }
        for (; bytes > 0; --bytes)
            tail[tailLen++] = *p++;
    }
    uint64_t finish()
    {
        if (tailLen > 0)
        {
            std::memset(tail + tailLen, 0, 8 - tailLen);
            uint64_t w;
            std::memcpy(&w, tail, 8);
            word(w);
            tailLen = 0;
        }
        uint64_t z = h;
        z = (z ^ (z >> 33)) * 0xff51afd7ed558ccdull;
        z = (z ^ (z >> 33)) * 0xc4ceb9fe1a85ec53ull;
        return z ^ (z >> 33);
    }
};

rc_bvh_node to_record(const BuildNode& b)
{
    rc_bvh_node r;
    for (int k = 0; k < 3; ++k)
    {
        r.aabb_min[k] = b.bmin[k];
        r.aabb_max[k] = b.bmax[k];
    }
    r.right_offset = b.rightOffset;
    r.start_offset = b.start;
    r.primitive_count = b.count;
    return r;
}

BuildNode from_record(const rc_bvh_node& r)
{
    BuildNode b;
    for (int k = 0; k < 3; ++k)
    {
        b.bmin[k] = r.aabb_min[k];
        b.bmax[k] = r.aabb_max[k];
    }
    b.rightOffset = r.right_offset;
    b.start = r.start_offset;
    b.count = r.primitive_count;
    return b;
}

struct FileCloser
{
    FILE* f;
    ~FileCloser()
    {
        if (f)
            std::fclose(f);
    }
};

bool write_all(FILE* f, const void* p, size_t bytes, Checksum* sum)
{
    if (sum)
        sum->add(p, bytes);
    return bytes == 0 || std::fwrite(p, 1, bytes, f) == bytes;
}

// Writes a host scene; err gets the reason on failure.
bool write_scene(const HostScene& hs, const char* path, std::string& err)
{
    FileHeader hd{};
    std::memcpy(hd.magic, kMagic, 8);
    hd.version = kVersion;
    hd.headerBytes = sizeof(FileHeader);
    hd.triangles = hs.tris.size();
    hd.materials = hs.mats.size();
    hd.flatNodes = hs.flat.size();
    hd.depth = hs.depth;
    for (int k = 0; k < 3; ++k)
    {
        hd.bounds[k] = hs.flat.empty() ? 0.0 : hs.flat[0].bmin[k];
        hd.bounds[3 + k] = hs.flat.empty() ? 0.0 : hs.flat[0].bmax[k];
    }
    std::vector<rc_bvh_node> recs(hs.flat.size());
    for (size_t i = 0; i < hs.flat.size(); ++i)
        recs[i] = to_record(hs.flat[i]);
    Checksum sum;
    sum.add(recs.data(), recs.size() * sizeof(rc_bvh_node));
    sum.add(hs.order.data(), hs.order.size() * 4);
    sum.add(hs.tris.data(), hs.tris.size() * sizeof(DevTri));
    sum.add(hs.shade.data(), hs.shade.size() * sizeof(DevShade));
    sum.add(hs.mats.data(), hs.mats.size() * sizeof(DevMat));
    hd.payloadBytes = recs.size() * sizeof(rc_bvh_node) + hs.order.size() * 4 + hs.tris.size() * sizeof(DevTri) +
                      hs.shade.size() * sizeof(DevShade) + hs.mats.size() * sizeof(DevMat);
    hd.checksum = sum.finish();

    FileCloser fc{ std::fopen(path, "wb") };
    if (!fc.f)
    {
        err = std::string("cannot open ") + path + " for writing";
        return false;
    }
    bool ok = write_all(fc.f, &hd, sizeof(hd), nullptr) &&
              write_all(fc.f, recs.data(), recs.size() * sizeof(rc_bvh_node), nullptr) &&
              write_all(fc.f, hs.order.data(), hs.order.size() * 4, nullptr) &&
              write_all(fc.f, hs.tris.data(), hs.tris.size() * sizeof(DevTri), nullptr) &&
              write_all(fc.f, hs.shade.data(), hs.shade.size() * sizeof(DevShade), nullptr) &&
              write_all(fc.f, hs.mats.data(), hs.mats.size() * sizeof(DevMat), nullptr);
    if (std::fclose(fc.f) != 0)
        ok = false;
    fc.f = nullptr;
    if (!ok)
        err = std::string("write to ") + path + " failed";
    return ok;
}

template <typename T>
bool read_array(FILE* f, std::vector<T>& v, uint64_t count, Checksum& sum)
{
    v.resize(size_t(count));
    size_t bytes = size_t(count) * sizeof(T);
    if (bytes > 0 && std::fread(v.data(), 1, bytes, f) != bytes)
        return false;
    sum.add(v.data(), bytes);
    return true;
}

// Reads and validates a scene file into hs.
bool read_scene(const char* path, HostScene& hs, FileHeader& hd, std::string& err)
{
    FileCloser fc{ std::fopen(path, "rb") };
    if (!fc.f)
    {
        err = std::string("cannot open ") + path;
        return false;
    }
    if (std::fread(&hd, 1, sizeof(hd), fc.f) != sizeof(hd))
    {
        err = "scene file: truncated header";
        return false;
    }
    if (std::memcmp(hd.magic, kMagic, 8) != 0)
    {
        err = "scene file: not a raycer_gb300 scene file (bad magic)";
        return false;
    }
    if (hd.version != kVersion || hd.headerBytes != sizeof(FileHeader))
    {
        err = "scene file: unsupported version " + std::to_string(hd.version);
        return false;
    }
    if (hd.triangles == 0 || hd.triangles > (uint64_t(1) << 27) || hd.materials == 0 ||
        hd.materials > uint64_t(kMetaMaterialMask) || hd.flatNodes == 0 || hd.flatNodes > 2 * hd.triangles)
    {
        err = "scene file: counts out of range";
        return false;
    }
    const uint64_t expect = hd.flatNodes * sizeof(rc_bvh_node) + hd.triangles * 4 +
                            hd.triangles * (sizeof(DevTri) + sizeof(DevShade)) + hd.materials * sizeof(DevMat);
    if (hd.payloadBytes != expect)
    {
        err = "scene file: payload size does not match the counts";
        return false;
    }
    Checksum sum;
    std::vector<rc_bvh_node> recs;
    if (!read_array(fc.f, recs, hd.flatNodes, sum) || !read_array(fc.f, hs.order, hd.triangles, sum) ||
        !read_array(fc.f, hs.tris, hd.triangles, sum) || !read_array(fc.f, hs.shade, hd.triangles, sum) ||
        !read_array(fc.f, hs.mats, hd.materials, sum))
    {
        err = "scene file: truncated payload";
        return false;
    }
    if (std::fgetc(fc.f) != EOF)
    {
        err = "scene file: trailing bytes after the payload";
        return false;
    }
    if (sum.finish() != hd.checksum)
    {
        err = "scene file: checksum mismatch (corrupted file)";
        return false;
    }
    hs.flat.resize(recs.size());
    for (size_t i = 0; i < recs.size(); ++i)
        hs.flat[i] = from_record(recs[i]);
    uint32_t depth = 0;
    if (!validate_flat_bvh(hs.flat, hd.triangles, depth, err))
    {
        err = "scene file: " + err;
        return false;
    }
    if (depth != hd.depth)
    {
        err = "scene file: BVH depth does not match the header";
        return false;
    }
    hs.depth = depth;
    // every BVH slot holds a distinct caller triangle with a valid material
    std::vector<unsigned char> seen(size_t(hd.triangles), 0);
    for (uint64_t s = 0; s < hd.triangles; ++s)
    {
        uint32_t p = hs.order[size_t(s)];
        uint32_t meta, idx;
        std::memcpy(&meta, &hs.tris[size_t(s)].c.y, 4);
        std::memcpy(&idx, &hs.tris[size_t(s)].c.z, 4);
        if (p >= hd.triangles || seen[p] || idx != p || (meta & kMetaMaterialMask) >= hd.materials)
        {
            err = "scene file: triangle records do not match the primitive order / materials";
            return false;
        }
        seen[p] = 1;
    }
    return true;
}

void copy_error(const std::string& msg, char* error, int64_t capacity)
{
    if (!error || capacity <= 0)
        return;
    size_t n = std::min<size_t>(msg.size(), size_t(capacity - 1));
    std::memcpy(error, msg.data(), n);
    error[n] = '\0';
}

rc_status fail(rc_tracer* h, rc_status s, const std::string& msg)
{
    h->err = msg;
    return s;
}

}  // namespace

extern "C" {

rc_status rc_write_scene_file(const double* vertices, const uint32_t* material_index, int64_t n,
                              const rc_material* materials, int32_t material_count, uint32_t max_leaf_size,
                              const char* path, char* error, int64_t error_capacity)
{
    if (!vertices || !material_index || !materials || !path || n <= 0 || material_count <= 0)
    {
        copy_error("write_scene_file: null array or empty scene", error, error_capacity);
        return RC_INVALID_ARG;
    }
    if (n > (int64_t(1) << 27) || material_count > int32_t(kMetaMaterialMask))
    {
        copy_error("write_scene_file: more than 2^27 triangles or too many materials", error, error_capacity);
        return RC_UNSUPPORTED;
    }
    for (int64_t i = 0; i < n; ++i)
        if (material_index[i] >= uint32_t(material_count))
        {
            copy_error("write_scene_file: material index out of range", error, error_capacity);
            return RC_INVALID_ARG;
        }
    for (int32_t i = 0; i < material_count; ++i)
        if ((materials[i].dielectric != 0 && materials[i].dielectric != 1) ||
            (materials[i].dielectric && !(materials[i].ior > 0.0f && std::isfinite(materials[i].ior))))
        {
            copy_error("write_scene_file: rc_material.dielectric must be 0 or 1 with ior > 0", error, error_capacity);
            return RC_INVALID_ARG;
        }
    for (int64_t i = 0; i < n * 9; ++i)
        if (!std::isfinite(vertices[i]))
        {
            copy_error("write_scene_file: non-finite vertex coordinate", error, error_capacity);
            return RC_INVALID_ARG;
        }
    BuildResult br;
    std::string err;
    if (!buildFlatBVH(vertices, n, max_leaf_size, 0, br, err))
    {
        copy_error("write_scene_file: " + err, error, error_capacity);
        return RC_INVALID_ARG;
    }
    if (br.depth > uint32_t(kMaxStack))
    {
        copy_error("write_scene_file: BVH deeper than the traversal stack", error, error_capacity);
        return RC_UNSUPPORTED;
    }
    HostScene hs;
    build_host_scene(vertices, material_index, n, materials, material_count, std::move(br.nodes),
                     std::move(br.order), br.depth, hs);
    if (!write_scene(hs, path, err))
    {
        copy_error("write_scene_file: " + err, error, error_capacity);
        return RC_IO;
    }
    return RC_OK;
}

rc_status rc_inspect_scene_file(const char* path, rc_scene_file_info* out, char* error, int64_t error_capacity)
{
    if (!path || !out)
    {
        copy_error("inspect_scene_file: null argument", error, error_capacity);
        return RC_INVALID_ARG;
    }
    HostScene hs;
    FileHeader hd;
    std::string err;
    if (!read_scene(path, hs, hd, err))
    {
        copy_error(err, error, error_capacity);
        return RC_IO;
    }
    out->triangles = hd.triangles;
    out->materials = hd.materials;
    out->bvh_nodes = hd.flatNodes;
    out->bvh_depth = hd.depth;
    for (int k = 0; k < 6; ++k)
        out->bounds[k] = hd.bounds[k];
    return RC_OK;
}

rc_status rc_save_scene(rc_tracer* h, const char* path)
{
    if (!h)
        return RC_INVALID_ARG;
    if (!path)
        return fail(h, RC_INVALID_ARG, "save_scene: null path");
    if (!h->sceneReady)
        return fail(h, RC_NOT_READY, "save_scene: no scene uploaded");
    if (h->nInstances > 0)
        return fail(h, RC_UNSUPPORTED, "save_scene: instanced scenes are not stored in scene files");
    cudaSetDevice(h->device);
    HostScene hs;
    hs.flat = h->hostNodes;
    hs.order = h->hostOrder;
    hs.depth = uint32_t(h->bvhDepth);
    hs.tris.resize(size_t(h->nTris));
    hs.shade.resize(size_t(h->nTris));
    hs.mats.resize(size_t(h->nMats));
    cudaError_t e = cudaMemcpy(hs.tris.data(), h->dTris, hs.tris.size() * sizeof(DevTri), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
        e = cudaMemcpy(hs.shade.data(), h->dShade, hs.shade.size() * sizeof(DevShade), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
        e = cudaMemcpy(hs.mats.data(), h->dMats, hs.mats.size() * sizeof(DevMat), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
        return fail(h, RC_CUDA, std::string("save_scene: download: ") + cudaGetErrorString(e));
    std::string err;
    if (!write_scene(hs, path, err))
        return fail(h, RC_IO, "save_scene: " + err);
    return RC_OK;
}

rc_status rc_load_scene(rc_tracer* h, const char* path)
{
    if (!h)
        return RC_INVALID_ARG;
    if (!path)
        return fail(h, RC_INVALID_ARG, "load_scene: null path");
    HostScene hs;
    FileHeader hd;
    std::string err;
    if (!read_scene(path, hs, hd, err))
        return fail(h, RC_IO, "load_scene: " + err);
    cudaSetDevice(h->device);
    return upload_host_scene(h, std::move(hs));
}

}  // extern "C"
