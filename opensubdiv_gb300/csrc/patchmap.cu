// Device PatchMap: (ptex face, u, v) -> patch handle, bit-exact with Far::PatchMap::FindPatch
// (far/patchMap.h:192-231) for float (u, v) in [0, 1].
//
// The quadtree is built on the host from the patch params (the construction of
// far/patchMap.cpp:134-194) and uploaded once per patch table.  Node = 4 packed children
// (bit 31 set, bit 30 leaf, bits 0..29 node or handle index).  Quad tables walk in float:
// every step subtracts a power of two `median` from a value in [median, 2*median], which is
// exact (Sterbenz), so the float walk takes the reference's double-precision decisions.
// Triangle tables walk the same way and form only their u + v tests in double, as the
// reference rounds them.
#include "common.cuh"
#include "patchmap.h"
#include "patchmap_walk.cuh"

#include <algorithm>
#include <cstring>

namespace gb300 {


struct HostNode {
    uint32_t c[4];
};

static int tri_quadrant(double median, double &u, double &v, bool &rot) {
    if (!rot) {
        if (u >= median) { u -= median; return 1; }
        if (v >= median) { v -= median; return 2; }
        if ((u + v) >= median) { rot = true; return 3; }
        return 0;
    }
    if (u < median) { v -= median; return 1; }
    if (v < median) { u -= median; return 2; }
    u -= median;
    v -= median;
    if ((u + v) < median) { rot = false; return 3; }
    return 0;
}

int build_patch_map(int numArrays, const int *arrays, int numPatches, const int *params,
                    int triangular, PatchMapHost &out) {
    out = PatchMapHost();
    out.triangular = triangular;
    if (numPatches <= 0) return ok();
    int total = 0;
    for (int a = 0; a < numArrays; ++a) total += arrays[6 * a + 2];
    if (total != numPatches)
        return fail(GB300_ERR_INVALID_ARGUMENT,
                    "patch map: arrays hold %d patches but %d params were given", total,
                    numPatches);
    out.handles.resize((size_t)numPatches * 4);
    int minF = params[0] & 0xfffffff, maxF = minF;
    // handles: (array, global patch index, j * patch size) as far/patchMap.cpp:100-132
    for (int a = 0, h = 0; a < numArrays; ++a) {
        const int np = arrays[6 * a + 2], stride = arrays[6 * a + 4];
        for (int j = 0; j < np; ++j, ++h) {
            out.handles[4 * (size_t)h + 0] = a;
            out.handles[4 * (size_t)h + 1] = h;
            out.handles[4 * (size_t)h + 2] = j * stride;
            out.handles[4 * (size_t)h + 3] = 0;
            const int f = params[3 * (size_t)h] & 0xfffffff;
            minF = std::min(minF, f);
            maxF = std::max(maxF, f);
        }
    }
    out.minFace = minF;
    out.maxFace = maxF;
    std::vector<HostNode> nodes((size_t)(maxF - minF + 1));
    std::memset(nodes.data(), 0, nodes.size() * sizeof(HostNode));
    auto descend = [&](int node, bool leaf, int q, int handle) -> int {
        if (leaf) {
            nodes[node].c[q] = kSet | kLeaf | (uint32_t)handle;
            return node;
        }
        if (nodes[node].c[q] & kSet) return (int)(nodes[node].c[q] & kIndex);
        const int nn = (int)nodes.size();
        nodes.push_back(HostNode{{0, 0, 0, 0}});
        nodes[node].c[q] = kSet | (uint32_t)nn;
        return nn;
    };
    int maxDepth = 0;
    for (int h = 0; h < numPatches; ++h) {
        const int f1 = params[3 * (size_t)h + 1];
        const int depth = f1 & 0xf, root = (f1 >> 4) & 1;
        const int pu = (f1 >> 22) & 0x3ff, pv = (f1 >> 12) & 0x3ff;
        maxDepth = std::max(maxDepth, depth);
        int node = (params[3 * (size_t)h] & 0xfffffff) - minF;
        if (depth == root) {
            for (int q = 0; q < 4; ++q) nodes[node].c[q] = kSet | kLeaf | (uint32_t)h;
            continue;
        }
        if (!triangular) {
            for (int j = root + 1; j <= depth; ++j) {
                const int q = (((pv >> (depth - j)) & 1) << 1) | ((pu >> (depth - j)) & 1);
                node = descend(node, j == depth, q, h);
            }
        } else {
            // an interior point of the patch locates its quadrants (far/patchMap.cpp:176-189)
            double u = 0.25, v = 0.25;
            const float frac = 1.0f / (float)(1 << (depth - root));
            if (pu + pv >= (1 << depth)) {
                const int df = 1 << depth;
                u = ((double)(df - pu) - u) * frac;
                v = ((double)(df - pv) - v) * frac;
            } else {
                u = (u + (double)pu) * (double)frac;
                v = (v + (double)pv) * (double)frac;
            }
            double median = 0.5;
            bool rot = false;
            for (int j = root + 1; j <= depth; ++j, median *= 0.5) {
                const int q = tri_quadrant(median, u, v, rot);
                node = descend(node, j == depth, q, h);
            }
        }
    }
    out.maxDepth = maxDepth;
    out.nodes.resize(nodes.size() * 4);
    std::memcpy(out.nodes.data(), nodes.data(), nodes.size() * sizeof(HostNode));
    return ok();
}

struct FindArgs {
    PatchMapView map;
    int n;
    const int *faces;
    const float *u;
    const float *v;
    int *out;  // 5 x 32 bit per query (OsdPatchCoord)
};

__global__ void __launch_bounds__(256) k_find_patches(const FindArgs a) {
    const int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
        const float fu = a.u[i], fv = a.v[i];
        const int4 h = patch_map_find(a.map, a.faces[i], fu, fv);
        int *o = a.out + 5 * (size_t)i;
        o[0] = h.x;
        o[1] = h.y;
        o[2] = h.z;
        o[3] = __float_as_int(fu);
        o[4] = __float_as_int(fv);
    }
}

PatchMapView view_of(const PatchMapDevice &m) {
    PatchMapView v;
    v.nodes = (const uint4 *)m.nodes;
    v.handles = (const int4 *)m.handles;
    v.minFace = m.minFace;
    v.maxFace = m.maxFace;
    v.maxDepth = m.maxDepth;
    v.triangular = m.triangular;
    v.numPatches = m.numPatches;
    return v;
}

int find_patches(const PatchMapDevice &m, int n, const int *faces, const float *u,
                 const float *v, void *coordsOut, cudaStream_t s) {
    if (n <= 0) return ok();
    if (!faces || !u || !v || !coordsOut)
        return fail(GB300_ERR_INVALID_ARGUMENT, "FindPatches: null pointer");
    FindArgs a;
    a.map = view_of(m);
    a.n = n;
    a.faces = faces;
    a.u = u;
    a.v = v;
    a.out = (int *)coordsOut;
    const int threads = 256;
    long long blocks = ((long long)n + threads - 1) / threads;
    long long cap = (long long)num_sms() * 16;
    k_find_patches<<<(int)(blocks < cap ? blocks : cap), threads, 0, s>>>(a);
    count_launch();
    return check_launch("FindPatches");
}

}  // namespace gb300
