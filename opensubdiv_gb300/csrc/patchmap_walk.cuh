// Device walk of the PatchMap quadtree (far/patchMap.h:192-231), shared by the FindPatches
// kernel and kernels that locate the points they generate.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace gb300 {

// Child slot encoding of a packed quadtree node: set, leaf (a patch handle index) or inner
// node index.
static constexpr uint32_t kSet = 0x80000000u, kLeaf = 0x40000000u, kIndex = 0x3fffffffu;

struct PatchMapView {
    const uint4 *nodes;
    const int4 *handles;
    int minFace, maxFace, maxDepth, triangular, numPatches;
};

__device__ __forceinline__ uint32_t child_of(const uint4 &n, int q) {
    return q == 0 ? n.x : q == 1 ? n.y : q == 2 ? n.z : n.w;
}

// Handle {array, patch, vert} of the patch holding (f, fu, fv), or {-1, -1, -1} for a miss.
__device__ __forceinline__ int4 patch_map_find(const PatchMapView &m, int f, float fu,
                                               float fv) {
    int4 h = make_int4(-1, -1, -1, 0);
    const bool in_range = m.numPatches > 0 && f >= m.minFace && f <= m.maxFace && fu >= 0.0f &&
                          fu <= 1.0f && fv >= 0.0f && fv <= 1.0f;
    if (!in_range) return h;
    uint4 node = __ldg(m.nodes + (f - m.minFace));
    if (!(node.x & kSet)) return h;
    if (!m.triangular) {
        float u = fu, v = fv, median = 0.5f;
        for (int d = 0; d <= m.maxDepth; ++d, median *= 0.5f) {
            int q = 0;
            if (u >= median) { u -= median; q |= 1; }
            if (v >= median) { v -= median; q |= 2; }
            const uint32_t c = child_of(node, q);
            if (!(c & kSet)) break;
            if (c & kLeaf) { h = __ldg(m.handles + (c & kIndex)); break; }
            node = __ldg(m.nodes + (c & kIndex));
        }
    } else {
        // every subtraction takes the power-of-two median from a value in [median, 2 * median]
        // (exact in float, Sterbenz), so u and v hold the reference's double values exactly;
        // only the sums u + v, which the reference rounds in double, are formed in double
        float u = fu, v = fv, median = 0.5f;
        bool rot = false;
        for (int d = 0; d <= m.maxDepth; ++d, median *= 0.5f) {
            int q;
            if (!rot) {
                if (u >= median) { u -= median; q = 1; }
                else if (v >= median) { v -= median; q = 2; }
                else if (((double)u + (double)v) >= (double)median) { rot = true; q = 3; }
                else q = 0;
            } else {
                if (u < median) { v -= median; q = 1; }
                else if (v < median) { u -= median; q = 2; }
                else {
                    u -= median;
                    v -= median;
                    if (((double)u + (double)v) < (double)median) { rot = false; q = 3; }
                    else q = 0;
                }
            }
            const uint32_t c = child_of(node, q);
            if (!(c & kSet)) break;
            if (c & kLeaf) { h = __ldg(m.handles + (c & kIndex)); break; }
            node = __ldg(m.nodes + (c & kIndex));
        }
    }
    return h;
}

}  // namespace gb300
