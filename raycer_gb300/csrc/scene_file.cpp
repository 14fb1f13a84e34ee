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
//     uint32   version       1 (single-level scene) or 2 (two-level scene)
//     uint32   headerBytes   128
//     uint64   triangles, materials, flatNodes   (version 2: of all meshes)
//     uint32   depth         (version 2: the deepest mesh BVH)
//     uint32   meshes        0 (version 1) or the mesh count
//     uint64   payloadBytes
//     uint64   checksum      of the payload (below)
//     double   bounds[6]     root box / scene box min xyz, max xyz
//     uint64   instances     0 (version 1) or the instance count
//   payload, version 1:
//     rc_bvh_node[flatNodes]  72 B each (FlatBVHNode fields)
//     uint32[triangles]       primitive order (caller index of BVH slot i)
//     DevTri[triangles]       48 B, DevShade[triangles] 48 B, DevMat[materials] 32 B
//   payload, version 2:
//     per mesh {uint64 triangles, uint64 flatNodes, uint32 depth, uint32 0}
//     per mesh: rc_bvh_node[], uint32 order[], DevTri[], DevShade[] as above
//       (caller indices mesh-local)
//     DevMat[materials], rc_instance[instances] (80 B each: mesh, material,
//       scale, rotate, translate)
//   A two-level scene's top-level BVH over the instances is rebuilt on load
//   (a few hundred boxes); every mesh BVH is read.
// Checksum: 64-bit words w of the payload (zero-padded tail), h = (h ^ w) *
// 0x100000001b3 from 0xcbf29ce484222325, then a final avalanche (the
// FNV-1a constants applied per word; a corruption check, not a
// cryptographic one).
//
// Loading validates, before any device allocation: magic, version, sizes,
// checksum, each flat BVH's structure (validate_flat_bvh), the traversal
// depth, and each triangle record against the order and the material count;
// instances are checked like rc_upload_instanced's.

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
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
constexpr uint32_t kVersion = 1;          // single-level scene
constexpr uint32_t kVersionInstanced = 2; // two-level scene

struct FileHeader
{
    char magic[8];
    uint32_t version;
    uint32_t headerBytes;
    uint64_t triangles;
    uint64_t materials;
    uint64_t flatNodes;
    uint32_t depth;
    uint32_t meshes;
    uint64_t payloadBytes;
    uint64_t checksum;
    double bounds[6];
    uint64_t instances;
    unsigned char pad[128 - 8 - 4 - 4 - 8 * 3 - 4 - 4 - 8 - 8 - 48 - 8];
};
static_assert(sizeof(FileHeader) == 128, "scene file header is 128 bytes");

struct MeshEntry
{
    uint64_t triangles;
    uint64_t flatNodes;
    uint32_t depth;
    uint32_t zero;
};
static_assert(sizeof(MeshEntry) == 24 && sizeof(rc_instance) == 80, "scene file record sizes");
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

bool read_instanced_payload(FILE* f, const FileHeader& hd, std::vector<HostScene>& meshes,
                            std::vector<rc_instance>& inst, std::string& err);

// Reads and validates a scene file: a single-level scene into hs, a
// two-level one (hd.version == kVersionInstanced) into meshes and inst.
bool read_scene(const char* path, HostScene& hs, FileHeader& hd, std::string& err,
                std::vector<HostScene>* meshes = nullptr, std::vector<rc_instance>* inst = nullptr)
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
    if ((hd.version != kVersion && hd.version != kVersionInstanced) || hd.headerBytes != sizeof(FileHeader))
    {
        err = "scene file: unsupported version " + std::to_string(hd.version);
        return false;
    }
    if (hd.version == kVersionInstanced)
    {
        std::vector<HostScene> localMeshes;
        std::vector<rc_instance> localInst;
        return read_instanced_payload(fc.f, hd, meshes ? *meshes : localMeshes, inst ? *inst : localInst, err);
    }
    if (hd.meshes != 0 || hd.instances != 0)
    {
        err = "scene file: counts out of range";
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

// Writes a two-level scene (meshes in BVH order, shared materials, instances).
bool write_instanced(const std::vector<HostScene>& meshes, const std::vector<DevMat>& mats,
                     const std::vector<rc_instance>& inst, const double* bounds, const char* path, std::string& err)
{
    FileHeader hd{};
    std::memcpy(hd.magic, kMagic, 8);
    hd.version = kVersionInstanced;
    hd.headerBytes = sizeof(FileHeader);
    hd.materials = mats.size();
    hd.meshes = uint32_t(meshes.size());
    hd.instances = inst.size();
    for (int k = 0; k < 6; ++k)
        hd.bounds[k] = bounds[k];
    std::vector<MeshEntry> table(meshes.size());
    std::vector<std::vector<rc_bvh_node>> recs(meshes.size());
    Checksum sum;
    for (size_t m = 0; m < meshes.size(); ++m)
    {
        const HostScene& hs = meshes[m];
        table[m] = MeshEntry{ hs.tris.size(), hs.flat.size(), hs.depth, 0 };
        hd.triangles += hs.tris.size();
        hd.flatNodes += hs.flat.size();
        hd.depth = std::max(hd.depth, hs.depth);
        recs[m].resize(hs.flat.size());
        for (size_t i = 0; i < hs.flat.size(); ++i)
            recs[m][i] = to_record(hs.flat[i]);
    }
    sum.add(table.data(), table.size() * sizeof(MeshEntry));
    hd.payloadBytes = table.size() * sizeof(MeshEntry);
    for (size_t m = 0; m < meshes.size(); ++m)
    {
        const HostScene& hs = meshes[m];
        sum.add(recs[m].data(), recs[m].size() * sizeof(rc_bvh_node));
        sum.add(hs.order.data(), hs.order.size() * 4);
        sum.add(hs.tris.data(), hs.tris.size() * sizeof(DevTri));
        sum.add(hs.shade.data(), hs.shade.size() * sizeof(DevShade));
        hd.payloadBytes += recs[m].size() * sizeof(rc_bvh_node) + hs.order.size() * 4 +
                           hs.tris.size() * (sizeof(DevTri) + sizeof(DevShade));
    }
    sum.add(mats.data(), mats.size() * sizeof(DevMat));
    sum.add(inst.data(), inst.size() * sizeof(rc_instance));
    hd.payloadBytes += mats.size() * sizeof(DevMat) + inst.size() * sizeof(rc_instance);
    hd.checksum = sum.finish();

    FileCloser fc{ std::fopen(path, "wb") };
    if (!fc.f)
    {
        err = std::string("cannot open ") + path + " for writing";
        return false;
    }
    bool ok = write_all(fc.f, &hd, sizeof(hd), nullptr) &&
              write_all(fc.f, table.data(), table.size() * sizeof(MeshEntry), nullptr);
    for (size_t m = 0; ok && m < meshes.size(); ++m)
    {
        const HostScene& hs = meshes[m];
        ok = write_all(fc.f, recs[m].data(), recs[m].size() * sizeof(rc_bvh_node), nullptr) &&
             write_all(fc.f, hs.order.data(), hs.order.size() * 4, nullptr) &&
             write_all(fc.f, hs.tris.data(), hs.tris.size() * sizeof(DevTri), nullptr) &&
             write_all(fc.f, hs.shade.data(), hs.shade.size() * sizeof(DevShade), nullptr);
    }
    ok = ok && write_all(fc.f, mats.data(), mats.size() * sizeof(DevMat), nullptr) &&
         write_all(fc.f, inst.data(), inst.size() * sizeof(rc_instance), nullptr);
    if (std::fclose(fc.f) != 0)
        ok = false;
    fc.f = nullptr;
    if (!ok)
        err = std::string("write to ") + path + " failed";
    return ok;
}

// The flat BVH and records of one scene (or mesh) against each other: the
// BVH's structure and depth, and every slot holding a distinct caller
// triangle with a valid material.
bool check_records(const std::vector<rc_bvh_node>& recs, HostScene& hs, uint64_t triangles, uint32_t depthIn,
                   uint64_t materials, std::string& err)
{
    hs.flat.resize(recs.size());
    for (size_t i = 0; i < recs.size(); ++i)
        hs.flat[i] = from_record(recs[i]);
    uint32_t depth = 0;
    if (!validate_flat_bvh(hs.flat, triangles, depth, err))
        return false;
    if (depth != depthIn)
    {
        err = "BVH depth does not match the header";
        return false;
    }
    if (depth > uint32_t(kMaxStack))
    {
        err = "BVH deeper than the traversal stack";
        return false;
    }
    hs.depth = depth;
    std::vector<unsigned char> seen(size_t(triangles), 0);
    for (uint64_t s = 0; s < triangles; ++s)
    {
        uint32_t p = hs.order[size_t(s)];
        uint32_t meta, idx;
        std::memcpy(&meta, &hs.tris[size_t(s)].c.y, 4);
        std::memcpy(&idx, &hs.tris[size_t(s)].c.z, 4);
        if (p >= triangles || seen[p] || idx != p || (meta & kMetaMaterialMask) >= materials)
        {
            err = "triangle records do not match the primitive order / materials";
            return false;
        }
        seen[p] = 1;
    }
    return true;
}

// Reads the payload of a version-2 file (header already read and checked).
bool read_instanced_payload(FILE* f, const FileHeader& hd, std::vector<HostScene>& meshes,
                            std::vector<rc_instance>& inst, std::string& err)
{
    if (hd.meshes == 0 || hd.instances == 0 || hd.instances > (uint64_t(1) << 24) || hd.triangles == 0 ||
        hd.triangles > (uint64_t(1) << 27) || hd.materials == 0 || hd.materials > uint64_t(kMetaMaterialMask) ||
        hd.meshes > hd.triangles)
    {
        err = "scene file: counts out of range";
        return false;
    }
    Checksum sum;
    std::vector<MeshEntry> table;
    if (!read_array(f, table, hd.meshes, sum))
    {
        err = "scene file: truncated payload";
        return false;
    }
    uint64_t tris = 0, nodes = 0, bytes = uint64_t(hd.meshes) * sizeof(MeshEntry);
    for (const MeshEntry& e : table)
    {
        if (e.triangles == 0 || e.flatNodes == 0 || e.flatNodes > 2 * e.triangles || e.zero != 0)
        {
            err = "scene file: mesh table out of range";
            return false;
        }
        tris += e.triangles;
        nodes += e.flatNodes;
        bytes += e.flatNodes * sizeof(rc_bvh_node) + e.triangles * (4 + sizeof(DevTri) + sizeof(DevShade));
    }
    bytes += hd.materials * sizeof(DevMat) + hd.instances * sizeof(rc_instance);
    if (tris != hd.triangles || nodes != hd.flatNodes || bytes != hd.payloadBytes)
    {
        err = "scene file: payload size does not match the counts";
        return false;
    }
    meshes.assign(hd.meshes, HostScene{});
    std::vector<std::vector<rc_bvh_node>> recs(hd.meshes);
    for (uint32_t m = 0; m < hd.meshes; ++m)
    {
        HostScene& hs = meshes[m];
        if (!read_array(f, recs[m], table[m].flatNodes, sum) || !read_array(f, hs.order, table[m].triangles, sum) ||
            !read_array(f, hs.tris, table[m].triangles, sum) || !read_array(f, hs.shade, table[m].triangles, sum))
        {
            err = "scene file: truncated payload";
            return false;
        }
    }
    std::vector<DevMat> mats;
    if (!read_array(f, mats, hd.materials, sum) || !read_array(f, inst, hd.instances, sum))
    {
        err = "scene file: truncated payload";
        return false;
    }
    if (std::fgetc(f) != EOF)
    {
        err = "scene file: trailing bytes after the payload";
        return false;
    }
    if (sum.finish() != hd.checksum)
    {
        err = "scene file: checksum mismatch (corrupted file)";
        return false;
    }
    uint32_t deepest = 0;
    for (uint32_t m = 0; m < hd.meshes; ++m)
    {
        if (!check_records(recs[m], meshes[m], table[m].triangles, table[m].depth, hd.materials, err))
        {
            err = "scene file: mesh " + std::to_string(m) + ": " + err;
            return false;
        }
        deepest = std::max(deepest, meshes[m].depth);
        meshes[m].mats = mats;
    }
    if (deepest != hd.depth)
    {
        err = "scene file: BVH depth does not match the header";
        return false;
    }
    for (const rc_instance& r : inst)
    {
        bool ok = r.mesh >= 0 && uint32_t(r.mesh) < hd.meshes && r.material >= -1 &&
                  (r.material < 0 || uint64_t(r.material) < hd.materials);
        for (int a = 0; a < 3 && ok; ++a)
            ok = std::isfinite(r.scale[a]) && std::isfinite(r.rotate[a]) && std::isfinite(r.translate[a]) &&
                 r.scale[a] != 0.0;
        if (!ok)
        {
            err = "scene file: instance out of range";
            return false;
        }
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
    out->meshes = hd.meshes;
    out->instances = hd.instances;
    return RC_OK;
}

rc_status rc_write_instanced_scene_file(const rc_mesh* meshes, int32_t mesh_count, const rc_instance* instances,
                                        int64_t instance_count, const rc_material* materials, int32_t material_count,
                                        uint32_t max_leaf_size, const char* path, char* error, int64_t error_capacity)
{
    std::string err;
    rc_status s = path ? check_instanced_args(meshes, mesh_count, instances, instance_count, materials,
                                              material_count, max_leaf_size, err)
                       : RC_INVALID_ARG;
    if (!path)
        err = "null path";
    if (s != RC_OK)
    {
        copy_error("write_instanced_scene_file: " + err, error, error_capacity);
        return s;
    }
    for (int64_t k = 0; k < instance_count; ++k)
    {
        const rc_instance& r = instances[k];
        bool ok = r.mesh >= 0 && r.mesh < mesh_count && r.material >= -1 && r.material < material_count;
        for (int a = 0; a < 3 && ok; ++a)
            ok = std::isfinite(r.scale[a]) && std::isfinite(r.rotate[a]) && std::isfinite(r.translate[a]) &&
                 r.scale[a] != 0.0;
        if (!ok)
        {
            copy_error("write_instanced_scene_file: instance " + std::to_string(k) + " out of range", error,
                       error_capacity);
            return RC_INVALID_ARG;
        }
    }
    std::vector<HostScene> scenes;
    if ((s = build_mesh_scenes(meshes, mesh_count, materials, material_count, max_leaf_size, scenes, err)) != RC_OK)
    {
        copy_error("write_instanced_scene_file: " + err, error, error_capacity);
        return s;
    }
    double box[6];
    instanced_scene_box(scenes, instances, instance_count, box);
    const std::vector<DevMat> mats = scenes[0].mats;
    if (!write_instanced(scenes, mats, std::vector<rc_instance>(instances, instances + instance_count), box, path,
                         err))
    {
        copy_error("write_instanced_scene_file: " + err, error, error_capacity);
        return RC_IO;
    }
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
    cudaSetDevice(h->device);
    if (h->nInstances > 0)
    {
        // two-level scene: each mesh's records from its range of the pooled arrays
        std::vector<HostScene> meshes(h->instMeshes.size());
        std::vector<DevMat> mats(size_t(h->nMats));
        cudaError_t e = cudaMemcpy(mats.data(), h->dMats, mats.size() * sizeof(DevMat), cudaMemcpyDeviceToHost);
        for (size_t m = 0; m < meshes.size() && e == cudaSuccess; ++m)
        {
            const InstancedMesh& im = h->instMeshes[m];
            HostScene& hs = meshes[m];
            hs.flat = im.flat;
            hs.order = im.order;
            hs.depth = im.depth;
            hs.tris.resize(size_t(im.triangles));
            hs.shade.resize(size_t(im.triangles));
            e = cudaMemcpy(hs.tris.data(), h->dTris + im.firstTri, hs.tris.size() * sizeof(DevTri),
                           cudaMemcpyDeviceToHost);
            if (e == cudaSuccess)
                e = cudaMemcpy(hs.shade.data(), h->dShade + im.firstTri, hs.shade.size() * sizeof(DevShade),
                               cudaMemcpyDeviceToHost);
        }
        if (e != cudaSuccess)
            return fail(h, RC_CUDA, std::string("save_scene: download: ") + cudaGetErrorString(e));
        std::string err;
        if (!write_instanced(meshes, mats, h->instDescs, h->bounds, path, err))
            return fail(h, RC_IO, "save_scene: " + err);
        return RC_OK;
    }
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
    std::vector<HostScene> meshes;
    std::vector<rc_instance> inst;
    const auto t0 = std::chrono::steady_clock::now();
    if (!read_scene(path, hs, hd, err, &meshes, &inst))
        return fail(h, RC_IO, "load_scene: " + err);
    cudaSetDevice(h->device);
    if (hd.version == kVersionInstanced)
        return upload_instanced_scenes(h, std::move(meshes), inst.data(), int64_t(inst.size()), int32_t(hd.materials),
                                       t0);
    return upload_host_scene(h, std::move(hs));
}

}  // extern "C"
