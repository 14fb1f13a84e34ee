// GPU linear-BVH builder (gpu_build.cu). Host-includable.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "device_types.h"

namespace rcx
{

struct GpuBuildInput
{
    const double* vertices;  // device: n * 9 (v0, v1, v2 per triangle, caller order)
    const uint32_t* matIdx;  // device: n material indices
    const DevMat* mats;      // device: material records
    int64_t n;
    int leafMax;             // 1..15 triangles per leaf
};

// Device scratch a build of n triangles needs.
size_t gpu_build_scratch_bytes(int64_t n);

// Phase 1: sort, hierarchy, boxes, node selection. Afterwards the device
// array gpu_build_counts() holds [0] the last keep flag, [1] its exclusive
// scan value (kept nodes = [0] + [1]) and [2] the root's height in internal
// levels; read it before phase 2.
cudaError_t gpu_build_hierarchy(const GpuBuildInput& in, void* scratch, cudaStream_t stream);
const uint32_t* gpu_build_counts(void* scratch, int64_t n);

// Phase 2: device nodes (kept-node count entries) with their triangle
// ranges (start, count), triangle and shading records in sorted order, and
// the sorted order (caller index of each slot).
cudaError_t gpu_build_emit(const GpuBuildInput& in, void* scratch, DevNode* nodes, int2* nodeRange, DevTri* tris,
                           DevShade* shade, uint32_t* order, cudaStream_t stream);

}  // namespace rcx
