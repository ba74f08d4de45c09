// Host-side PatchMap quadtree (built from patch params) and its device mirror.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "../../include/osd_gb300.h"
#include "patchmap_walk.cuh"

namespace gb300 {

struct PatchMapHost {
    int triangular = 0, minFace = 0, maxFace = -1, maxDepth = 0;
    std::vector<uint32_t> nodes;  // 4 packed children per node; roots first (one per face)
    std::vector<int> handles;     // 4 ints per patch: array, patch, vert, pad
};

struct PatchMapDevice {
    void *nodes = nullptr;
    void *handles = nullptr;
    int triangular = 0, minFace = 0, maxFace = -1, maxDepth = 0, numPatches = 0;
};

// Builds the quadtree of far/patchMap.cpp:89-202 from host arrays (6 ints per patch array,
// 3 x 32-bit per patch param).
int build_patch_map(int numArrays, const int *arrays, int numPatches, const int *params,
                    int triangular, PatchMapHost &out);

// Kernel-argument view of a device map.
PatchMapView view_of(const PatchMapDevice &m);

// The device map of a patch table (GB300PatchTableCreate), for kernels that locate points.
const PatchMapDevice *patch_map_of(const GB300PatchTable *table);

int find_patches(const PatchMapDevice &m, int n, const int *faces, const float *u,
                 const float *v, void *coordsOut, cudaStream_t s);

int eval_stencils(const float *src, float *const *dst, const int *strides,
                  const float *const *w, int length, int srcStride, const int *sizes,
                  const int *offsets, const int *indices, int start, int end, cudaStream_t s,
                  const char *who);

// quadFamily: every patch array holds only REGULAR / GREGORY_BASIS / QUADS patches, which
// selects the element-lane kernel (known for device tables; raw-pointer calls pass 0).
// grouped: consecutive coords mostly share a patch (a tessellation's coords), which selects
// the one-thread-per-point kernel for every table.
int eval_patches(const float *src, float *const *dst, const int *strides, int length,
                 int srcStride, int numCoords, const void *coords, const void *arrays,
                 const int *indices, const void *params, cudaStream_t s, const char *who,
                 int quadFamily, int grouped = 0);

// Draw-time tessellation factors of every patch of a table (tess_factors.cu).
int tess_factors(const void *arrays, int numArrays, const int *indices, const void *params,
                 int numPatches, const float *src, int srcStride,
                 const GB300PatchTessOptions *o, float *outer, float *inner, float *outerLo,
                 float *outerHi, cudaStream_t s);

// Limit stencils at device PatchCoords of a table, composed over the stencils of its points
// (stencil_factory.cu).
GB300StencilTable *tess_stencils(const void *arrays, const int *indices, const void *params,
                                 int numPoints, const void *patchCoords, int baseNumStencils,
                                 int64_t baseNumIndices, const int *baseSizes,
                                 const int *baseOffsets, const int *baseIndices,
                                 const float *baseWeights, int numChannels, int sortEntries,
                                 cudaStream_t s, const char *who);

}  // namespace gb300
