// Bfr::Tessellation over every face of a mesh at once (bfr/tessellation.h:142-262), with the
// points located on a device patch table for evaluation.
//
// Launches on one stream:
//   count    one thread per face: the face's coord, facet and ptex-face counts, then device
//            exclusive scans into the caller's offset arrays (the only host sync is the read
//            of the three totals, which the caller needs to size its buffers);
//   patterns with a single uniform rate every face of the same size has the same pattern: one
//            thread builds it per face size (3..10), once per device and request (cached);
//   generate one thread per face without a shared pattern (per-face rates, polygons above 10
//            sides) writes its coords and facets straight into its slice of the output, facet
//            indices offset to the mesh-wide coord numbering
//            (Tessellation::TransformFacetCoordIndices, tessellation.cpp:2429-2447);
//   finish   one warp per face, lanes over the face's coords and facets (coalesced): copies
//            the shared pattern out with offset indices, and turns each coord into a
//            PatchCoord: Parameterization::ConvertCoordToNormalizedSubFace
//            (bfr/parameterization.cpp:135-162) picks the ptex sub-face of an N-gon and the
//            PatchMap walk finds the patch -- the lookup the reference's Bfr regression does
//            for every tessellation coord (regression/bfr_evaluate/farPatchEvaluator.cpp:
//            190-207).
//   share    (GB300TessellationShare, optional) shared vertex and edge points as the
//            reference's tutorial 2.2 makes them: claims by 64-bit atomicMin, counts, a scan
//            that numbers the points, per-corner records, then one warp per face moves the
//            PatchCoords of the points it makes and rewrites its facets to point indices.
// A staged variant (faces generated into a shared-memory arena, copied out coalesced) was
// slower: about 900 bytes of arena per face left too few warps resident to hide latency.
#include "common.cuh"
#include "patchmap.h"
#include "patchmap_walk.cuh"
#include "tess_pattern.cuh"

#include <cub/device/device_scan.cuh>

#include <atomic>
#include <climits>
#include <cstring>
#include <mutex>
#include <vector>

namespace gb300 {
namespace {

using tess::Face;
using tess::Sink;

constexpr int kFirstShared = 3;  // face sizes with a shared uniform pattern: 3 .. 10
constexpr int kNumShared = 8;

// The rates of face f: p == null means the single rate `one` (the uniform rate).
struct FaceRates {
    const int *p;
    int n, one;
};

__device__ __forceinline__ void rates_of(const int *rateOffsets, const int *rates,
                                         int uniformRate, int f, FaceRates &r) {
    r.one = uniformRate;
    if (!rates) {
        r.p = nullptr;
        r.n = 1;
    } else if (!rateOffsets) {
        r.p = rates + f;
        r.n = 1;
    } else {
        const int a = rateOffsets[f];
        r.p = rates + a;
        r.n = rateOffsets[f + 1] - a;
    }
}

struct CountArgs {
    int reg, numFaces, uniformRate, fs, pq;
    const int *faceSizes, *rateOffsets, *rates;
    int64_t *cc, *fc, *pc;  // per-face counts, [numFaces] = 0
};

__global__ void __launch_bounds__(256) k_tess_count(const CountArgs a) {
    const int stride = gridDim.x * blockDim.x;
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f <= a.numFaces; f += stride) {
        if (f == a.numFaces) {
            a.cc[f] = a.fc[f] = a.pc[f] = 0;
            continue;
        }
        const int N = a.faceSizes[f];
        FaceRates r;
        rates_of(a.rateOffsets, a.rates, a.uniformRate, f, r);
        Face face;
        const bool ok = face.init(a.reg, N, r.n, r.p, a.fs, a.pq, r.one);
        a.cc[f] = ok ? face.num_coords() : 0;
        a.fc[f] = ok ? face.nFacets : 0;
        a.pc[f] = N > 0 ? tess::ptex_count(a.reg, N) : 0;
    }
}

struct GenArgs {
    int reg, numFaces, uniformRate, fs, pq, coordStride, facetStride;
    const int *faceSizes, *rateOffsets, *rates;
    const int64_t *co, *fo, *po;
    float *coords;
    int *facets;
    int offsetIndices;
    int coordPairs;  // coordStride 2 and 8-byte aligned coords: (u,v) stored as one float2
    // shared uniform patterns for face sizes kFirstShared + k (packed: stride 2 / fs, local
    // facet indices)
    int shared;
    int patC[kNumShared + 1], patF[kNumShared + 1];
    const float *patCoords;
    const int *patFacets;
    // location on a patch table (optional)
    int locate;
    PatchMapView map;
    int *patchCoords;  // 5 x 32 bit per coord
    // per-face rates: faces with the same size and rates share one pattern, generated by the
    // lowest-numbered of them (the owner) and copied from its output slice by the others;
    // faceSlot[f] is the face's hash slot (-1: generated on its own), owners[slot] the owner
    int dedupe;
    unsigned long long *keys;
    int *owners;
    int *faceSlot;
    unsigned int slotMask;
};

__device__ __forceinline__ bool uses_shared(const GenArgs &a, int N) {
    return a.shared && N >= kFirstShared && N < kFirstShared + kNumShared;
}

// One thread per shared pattern (a face size 3..10 at the uniform rate).
__global__ void __launch_bounds__(32) k_tess_patterns(int reg, int rate, int fs, int pq,
                                                      const int *patC, const int *patF,
                                                      float *patCoords, int *patFacets) {
    const int t = threadIdx.x;
    if (t >= kNumShared) return;
    Face face;
    if (!face.init(reg, kFirstShared + t, 1, nullptr, fs, pq, rate)) return;
    Sink o{patCoords + 2 * (int64_t)patC[t], 2, patFacets + (int64_t)fs * patF[t], fs, fs};
    face.coords(o);
    face.facets(o);
}

// PatchCoord of a coord of face (size N, first ptex face ptex0): the ptex sub-face and
// normalized (s, t) of Parameterization::ConvertCoordToNormalizedSubFace
// (bfr/parameterization.cpp:135-162), then the PatchMap walk.
__device__ __forceinline__ void locate_coord(const GenArgs &a, int N, int ptex0, float u, float v,
                                             int *o) {
    int sub = 0;
    float s = u, t = v;
    if (N != a.reg) {
        const int udim = (N < 10) ? 2 + (N > 4) : 1 + (int)sqrtf((float)(N - 1));
        int ut = (int)u, vt = (int)v;
        float uf = __fsub_rn(u, (float)ut), vf = __fsub_rn(v, (float)vt);
        if (uf > 0.75f) { ut++; uf = __fsub_rn(uf, 1.0f); }
        if (vf > 0.75f) { vt++; vf = __fsub_rn(vf, 1.0f); }
        s = __fmul_rn(uf, 2.0f);
        t = __fmul_rn(vf, 2.0f);
        sub = udim * vt + ut;
    }
    const int4 h = patch_map_find(a.map, ptex0 + sub, s, t);
    o[0] = h.x;
    o[1] = h.y;
    o[2] = h.z;
    o[3] = __float_as_int(s);
    o[4] = __float_as_int(t);
}

constexpr unsigned long long kEmptyKey = ~0ull;

// The face's (size, rates) as one 64-bit key: triangles and quads with at most 6 rates below
// 1024 (1 bit size, 3 bits rate count, 10 bits per rate; a count of 7 never occurs, so the
// all-ones empty key cannot either).  Other faces are not shared.
__device__ __forceinline__ bool pattern_key(int N, const FaceRates &r, unsigned long long &key) {
    if (N < 3 || N > 4 || r.n < 1 || r.n > 6) return false;
    unsigned long long k = (unsigned long long)(N - 3) | ((unsigned long long)r.n << 1);
    for (int i = 0; i < r.n; ++i) {
        const int v = r.p ? r.p[i] : r.one;
        if (v < 0 || v > 1023) return false;
        k |= (unsigned long long)v << (4 + 10 * i);
    }
    key = k;
    return true;
}

__device__ __forceinline__ unsigned int key_hash(unsigned long long k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return (unsigned int)k;
}

// One thread per face: the face's slot in an open-addressing table of keys (capacity at least
// twice the faces, so a free slot is always found), and the lowest face index per key.
// Neighbouring faces often share a key, so the lanes of a warp with the same key insert once,
// through their lowest lane (the lowest face of the group).
__global__ void __launch_bounds__(256) k_tess_dedupe(const GenArgs a) {
    const int stride = gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    // every lane runs the same number of iterations, so the warp stays converged
    const int rounds = (a.numFaces + stride - 1) / stride;
    for (int it = 0; it < rounds; ++it) {
        const int f = it * stride + blockIdx.x * blockDim.x + threadIdx.x;
        unsigned long long key = kEmptyKey;
        bool keyed = false;
        if (f < a.numFaces) {
            FaceRates r;
            rates_of(a.rateOffsets, a.rates, a.uniformRate, f, r);
            keyed = pattern_key(a.faceSizes[f], r, key);
        }
        const unsigned keyedMask = __ballot_sync(0xffffffffu, keyed);
        const unsigned same = __match_any_sync(0xffffffffu, key) & keyedMask;
        const int leader = same ? __ffs(same) - 1 : lane;
        int slot = -1;
        if (keyed && leader == lane) {
            unsigned int h = key_hash(key) & a.slotMask;
            for (unsigned int probe = 0; probe <= a.slotMask; ++probe) {
                const unsigned long long prev = atomicCAS(a.keys + h, kEmptyKey, key);
                if (prev == kEmptyKey || prev == key) {
                    atomicMin(a.owners + h, f);
                    slot = (int)h;
                    break;
                }
                h = (h + 1) & a.slotMask;
            }
        }
        slot = __shfl_sync(0xffffffffu, slot, leader);
        if (f < a.numFaces) a.faceSlot[f] = keyed ? slot : -1;
    }
}

// The face whose output slice holds face f's pattern (f itself unless a lower face shares it).
__device__ __forceinline__ int owner_of(const GenArgs &a, int f) {
    if (!a.dedupe) return f;
    const int slot = a.faceSlot[f];
    return slot < 0 ? f : a.owners[slot];
}

// One thread per face without a shared pattern: the face's coords and facets (indices already
// offset to the mesh numbering) straight into its slice of the output.  One launch per
// parameterization kind K present in the scheme, each generating only that kind's faces.
template <int K>
__global__ void __launch_bounds__(128, 8) k_tess_generate(const GenArgs a) {
    const int stride = gridDim.x * blockDim.x;
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < a.numFaces; f += stride) {
        const int N = a.faceSizes[f];
        const int kind = N == a.reg ? (a.reg == 4 ? tess::kQuad : tess::kTri) : tess::kQsub;
        if (kind != K || uses_shared(a, N) || owner_of(a, f) != f) continue;
        FaceRates r;
        rates_of(a.rateOffsets, a.rates, a.uniformRate, f, r);
        Face face;
        if (!face.init(a.reg, N, r.n, r.p, a.fs, a.pq, r.one)) continue;
        const int64_t c0 = a.co[f];
        Sink o{a.coords + c0 * a.coordStride, a.coordStride, a.facets + a.fo[f] * a.facetStride,
               a.fs, a.facetStride, a.offsetIndices ? (int)c0 : 0, a.coordPairs != 0};
        face.coords_k<K>(o);
        face.facets_k<K>(o);
    }
}

// One warp per face: copies a shared pattern out (coords as float2 pairs, one lane per facet
// with its indices offset), and locates every coord of the face on the patch table.
template <int FS>
__global__ void __launch_bounds__(256) k_tess_finish(const GenArgs a) {
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int f = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; f < a.numFaces; f += warps) {
        const int64_t c0 = a.co[f];
        const int nc = (int)(a.co[f + 1] - c0);
        if (nc == 0) continue;
        const int N = a.faceSizes[f];
        const bool sh = uses_shared(a, N);
        const int own = sh ? f : owner_of(a, f);
        if (!sh && own == f && !a.locate) continue;
        const int k = N - kFirstShared;
        const int ptex0 = a.locate ? (int)a.po[f] : 0;
        if (!sh && own != f) {
            // a copy of the owner's slice: same coords, facet indices moved by the difference
            // of the two faces' first coords
            const int64_t s0 = a.co[own];
            for (int i = lane; i < nc; i += 32) {
                const float *c = a.coords + (s0 + i) * a.coordStride;
                float *d = a.coords + (c0 + i) * a.coordStride;
                float u, v;
                if (a.coordPairs) {
                    const float2 uv = *reinterpret_cast<const float2 *>(c);
                    *reinterpret_cast<float2 *>(d) = uv;
                    u = uv.x;
                    v = uv.y;
                } else {
                    u = c[0];
                    v = c[1];
                    d[0] = u;
                    d[1] = v;
                }
                if (a.locate) locate_coord(a, N, ptex0, u, v, a.patchCoords + 5 * (c0 + i));
            }
            const int64_t f0 = a.fo[f], g0 = a.fo[own];
            const int nf = (int)(a.fo[f + 1] - f0);
            const int delta = a.offsetIndices ? (int)(c0 - s0) : 0;
            for (int q = lane; q < nf; q += 32) {
                const int *src = a.facets + (g0 + q) * a.facetStride;
                int *d = a.facets + (f0 + q) * a.facetStride;
#pragma unroll
                for (int c = 0; c < FS; ++c) {
                    const int v = src[c];
                    d[c] = v >= 0 ? v + delta : v;
                }
            }
        } else if (sh) {
            const float2 *pc = reinterpret_cast<const float2 *>(a.patCoords) + a.patC[k];
            for (int i = lane; i < nc; i += 32) {
                const float2 uv = pc[i];
                float *d = a.coords + (c0 + i) * a.coordStride;
                if (a.coordPairs) {
                    *reinterpret_cast<float2 *>(d) = uv;
                } else {
                    d[0] = uv.x;
                    d[1] = uv.y;
                }
                if (a.locate) locate_coord(a, N, ptex0, uv.x, uv.y, a.patchCoords + 5 * (c0 + i));
            }
            const int64_t f0 = a.fo[f];
            const int nf = (int)(a.fo[f + 1] - f0);
            const int off = a.offsetIndices ? (int)c0 : 0;
            const int *pf = a.patFacets + FS * a.patF[k];
            for (int q = lane; q < nf; q += 32) {
                int *d = a.facets + (f0 + q) * a.facetStride;
#pragma unroll
                for (int c = 0; c < FS; ++c) {
                    const int v = pf[FS * q + c];
                    d[c] = v >= 0 ? v + off : v;
                }
            }
        } else {
            for (int i = lane; i < nc; i += 32) {
                const float *c = a.coords + (c0 + i) * a.coordStride;
                float u, v;
                if (a.coordPairs) {
                    const float2 uv = *reinterpret_cast<const float2 *>(c);
                    u = uv.x;
                    v = uv.y;
                } else {
                    u = c[0];
                    v = c[1];
                }
                locate_coord(a, N, ptex0, u, v, a.patchCoords + 5 * (c0 + i));
            }
        }
    }
}

// ---- shared (watertight) points --------------------------------------------------------------
// The bookkeeping of the reference's tessellation with shared vertex and edge points
// (tutorials/bfr/tutorial_2_2/bfr_tutorial_2_2.cpp:244-430) for every face at once.  The point
// of a mesh vertex, and the points inside a mesh edge, are made by the lowest face that reaches
// them (its lowest corner that does): the face the tutorial's in-order loop reaches them with
// first.  Each face makes its points in boundary order (vertex, then the points inside the
// edge that follows it), then its interior coords; a prefix sum over the faces numbers them as
// the tutorial does.  Faces without coords take no part.
struct ShareArgs {
    int reg, numFaces, uniformRate, fs, pq, coordStride, facetStride, meshIndices;
    int numVertices, numEdges;
    int64_t numCorners;  // entries of faceVerts and faceEdges
    const int *faceSizes, *faceVerts, *faceEdges, *rateOffsets, *rates;
    const int64_t *co, *fo;
    int64_t *cornerOff;                     // first corner of each face (scan of faceSizes)
    int4 *cornerInfo;                       // per corner: share_corner's record
    unsigned long long *vertKey, *edgeKey;  // min over faces of (face << 32 | corner)
    int *edgeN;                             // points inside each edge, set by its maker
    int64_t *counts;                        // points each face makes; [numFaces] = 0
    const int64_t *po;                      // their exclusive scan: first point of each face
    int *vertPoint, *edgePoint;             // point of each vertex, first point of each edge
    int *facets;
    const int *coordPC;  // 5 x 32 bit per coord (PatchCoord), optional
    const float *coords;
    int *pointPC;
    float *pointCoords;
    int *pointFaces;
    int *err;  // {index errors, first such face, rate mismatches, first such face}, then the
               // point and corner totals (two 64-bit words), read back in one copy
};

constexpr int kCornerEdgeMask = 0x7fff;  // points inside the edge (rate - 1 <= 32766)
constexpr int kCornerVertNew = 1 << 15;
constexpr int kCornerEdgeNew = 1 << 16;
constexpr int kCornerReversed = 1 << 17;
constexpr int kCornerBad = 1 << 18;

__device__ __forceinline__ void share_error(int *err, int kind, int f) {
    atomicAdd(err + 2 * kind, 1);
    atomicMin(err + 2 * kind + 1, f);
}

__device__ __forceinline__ unsigned long long corner_key(int f, int i) {
    return ((unsigned long long)(unsigned)f << 32) | (unsigned)i;
}

__device__ __forceinline__ bool share_face(const ShareArgs &a, int f, Face &face) {
    FaceRates r;
    rates_of(a.rateOffsets, a.rates, a.uniformRate, f, r);
    return face.init(a.reg, a.faceSizes[f], r.n, r.p, a.fs, a.pq, r.one);
}

// Face sizes (scanned into corner offsets after), unclaimed vertices and edges without
// points, and the error words.
__global__ void __launch_bounds__(256) k_share_init(const ShareArgs a) {
    const int stride = gridDim.x * blockDim.x;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0) a.err[0] = 0, a.err[1] = INT_MAX, a.err[2] = 0, a.err[3] = INT_MAX;
    for (int f = t; f <= a.numFaces; f += stride)
        a.counts[f] = f < a.numFaces ? a.faceSizes[f] : 0;
    for (int v = t; v < a.numVertices; v += stride) {
        a.vertKey[v] = ~0ull;
        a.vertPoint[v] = -1;
    }
    for (int e = t; e < a.numEdges; e += stride) {
        a.edgeKey[e] = ~0ull;
        a.edgePoint[e] = -1;
    }
}

// One thread per face: claim the face's vertices and edges (lowest face and corner wins).
__global__ void __launch_bounds__(256) k_share_own(const ShareArgs a) {
    const int stride = gridDim.x * blockDim.x;
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < a.numFaces; f += stride) {
        Face face;
        if (a.co[f + 1] == a.co[f] || !share_face(a, f, face)) continue;
        const int N = face.N;
        const int64_t c0 = a.cornerOff[f];
        if (c0 + N > a.numCorners) {
            share_error(a.err, 0, f);
            continue;
        }
        for (int i = 0; i < N; ++i) {
            const int v = a.faceVerts[c0 + i], e = a.faceEdges[c0 + i];
            if ((unsigned)v >= (unsigned)a.numVertices || (unsigned)e >= (unsigned)a.numEdges) {
                share_error(a.err, 0, f);
                continue;
            }
            atomicMin(a.vertKey + v, corner_key(f, i));
            atomicMin(a.edgeKey + e, corner_key(f, i));
        }
    }
}

// One thread per face: the points the face makes (its claimed vertices, the points inside its
// claimed edges, its interior coords); a claimed edge records its number of inside points.
__global__ void __launch_bounds__(256) k_share_count(const ShareArgs a) {
    const int stride = gridDim.x * blockDim.x;
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f <= a.numFaces; f += stride) {
        int64_t n = 0;
        const int64_t nc = f < a.numFaces ? a.co[f + 1] - a.co[f] : 0;
        Face face;
        const bool valid = nc > 0 && share_face(a, f, face);
        if (nc > 0 && !valid) share_error(a.err, 0, f);  // coords the tessellation cannot have
        const int64_t c0 = valid ? a.cornerOff[f] : 0;
        if (valid && c0 + face.N <= a.numCorners) {
            n = nc - face.nBoundary;
            for (int i = 0; i < face.N; ++i) {
                const int v = a.faceVerts[c0 + i], e = a.faceEdges[c0 + i];
                if ((unsigned)v >= (unsigned)a.numVertices ||
                    (unsigned)e >= (unsigned)a.numEdges)
                    continue;
                const unsigned long long key = corner_key(f, i);
                if (a.vertKey[v] == key) ++n;
                if (a.edgeKey[e] == key) {
                    const int k = face.outer(i) - 1;
                    a.edgeN[e] = k;
                    n += k;
                }
            }
        }
        a.counts[f] = n;
    }
}

// One thread per face: number the points of the vertices and edges the face claimed.
__global__ void __launch_bounds__(256) k_share_assign(const ShareArgs a) {
    const int stride = gridDim.x * blockDim.x;
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < a.numFaces; f += stride) {
        if (a.co[f + 1] == a.co[f]) continue;
        Face face;
        if (!share_face(a, f, face)) continue;
        const int64_t c0 = a.cornerOff[f];
        if (c0 + face.N > a.numCorners) continue;
        int p = (int)a.po[f];
        for (int i = 0; i < face.N; ++i) {
            const int v = a.faceVerts[c0 + i], e = a.faceEdges[c0 + i];
            if ((unsigned)v >= (unsigned)a.numVertices || (unsigned)e >= (unsigned)a.numEdges)
                continue;
            const unsigned long long key = corner_key(f, i);
            if (a.vertKey[v] == key) a.vertPoint[v] = p++;
            if (a.edgeKey[e] == key) {
                a.edgePoint[e] = p;
                p += face.outer(i) - 1;
            }
        }
    }
}

// Corner i of face f, whose vertex coord is boundary coord P: {P, the vertex's point, the
// first point inside the edge that follows, flags | points inside the edge}.  An edge run
// from the other end than its maker ran it takes its points in reverse.
__device__ __forceinline__ int4 share_corner(const ShareArgs &a, const Face &face, int f,
                                             int64_t c0, int i, int P) {
    const int v = a.faceVerts[c0 + i], e = a.faceEdges[c0 + i];
    const int n = face.outer(i) - 1;
    if ((unsigned)v >= (unsigned)a.numVertices || (unsigned)e >= (unsigned)a.numEdges)
        return make_int4(P, -1, -1, n | kCornerBad);
    const unsigned long long key = corner_key(f, i);
    int meta = n;
    if (a.vertKey[v] == key) meta |= kCornerVertNew;
    const unsigned long long ek = a.edgeKey[e];
    if (ek == key) {
        meta |= kCornerEdgeNew;
    } else if (a.edgeN[e] != n) {
        meta |= kCornerBad;
    } else {
        const int g = (int)(ek >> 32), j = (int)(ek & 0xffffffffu);
        if (a.faceVerts[a.cornerOff[g] + j] != v) meta |= kCornerReversed;
    }
    return make_int4(P, a.vertPoint[v], a.edgePoint[e], meta);
}

// The point of boundary coord idx in corner c (its vertex coord or inside its edge); `made`
// when this face made the point.
__device__ __forceinline__ int share_boundary_point(int4 c, int idx, bool &made) {
    const int j = idx - c.x;
    if (j == 0) {
        made = (c.w & kCornerVertNew) != 0;
        return c.y;
    }
    made = (c.w & kCornerEdgeNew) != 0;
    if (c.w & kCornerBad) return -1;
    const int n = c.w & kCornerEdgeMask;
    return (c.w & kCornerReversed) ? c.z + n - j : c.z + j - 1;
}

// The point of coord idx of a face with N corner records `cs` (shared or global memory),
// nb boundary coords and interior coord idx at point idx + interior; `made` when the face
// made the point.
__device__ __forceinline__ int share_point(const int4 *cs, int N, int nb, int interior,
                                           int idx, bool &made) {
    if (idx >= nb) {
        made = true;
        return idx + interior;
    }
    int lo = 0, hi = N - 1;  // the last corner whose vertex coord is at or before idx
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (cs[mid].x <= idx) lo = mid; else hi = mid - 1;
    }
    return share_boundary_point(cs[lo], idx, made);
}

// The point and corner totals beside the error words, so one copy reads all of them.
__global__ void k_share_totals(const ShareArgs a) {
    if (threadIdx.x == 0) {
        long long *t = reinterpret_cast<long long *>(a.err + 4);
        t[0] = a.po[a.numFaces];
        t[1] = a.cornerOff[a.numFaces];
    }
}

// One thread per face: the record of each of its corners, for the emit pass.
__global__ void __launch_bounds__(256) k_share_corners(const ShareArgs a) {
    const int stride = gridDim.x * blockDim.x;
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < a.numFaces; f += stride) {
        if (a.co[f + 1] == a.co[f]) continue;
        Face face;
        if (!share_face(a, f, face)) continue;
        const int64_t c0 = a.cornerOff[f];
        if (c0 + face.N > a.numCorners) continue;
        int P = 0;
        for (int i = 0; i < face.N; ++i) {
            const int4 c = share_corner(a, face, f, c0, i, P);
            if (c.w & kCornerBad) share_error(a.err, c.y < 0 ? 0 : 1, f);
            a.cornerInfo[c0 + i] = c;
            P += face.outer(i);
        }
    }
}

// One warp per face.  Every load of a face is issued before its first store -- its corner
// records, PatchCoord words and facet index words, kShareWords of each per lane per round --
// so a face costs about one memory latency, and the next face's offsets (eight words, one per
// lane) are fetched while this one is processed.  The point of each boundary coord goes into
// a per-warp table in shared memory (faces up to kShareTable boundary coords and 32 sides;
// larger faces search their corner records per index), interior coords map to points by an
// offset.  Then each PatchCoord word of a coord that makes a point goes to the point's slot,
// and each facet index becomes its point (Tessellation::TransformFacetCoordIndices with
// boundary indices and an interior offset, tessellation.cpp:2449-2464).
constexpr int kShareWords = 6;
constexpr int kShareTable = 128;
constexpr int kShareMade = int(0x80000000u);

template <int FS>
__global__ void __launch_bounds__(256, 4) k_share_emit(const ShareArgs a) {
    __shared__ int4 corners[8][32];
    __shared__ int table[8][kShareTable];  // point | kShareMade of each boundary coord
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    // lane j < 8 holds offset j of face f: co[f], co[f+1], cornerOff[f], cornerOff[f+1],
    // fo[f], fo[f+1], po[f], po[f+1]
    auto offsets_of = [&](int f) -> long long {
        if (f >= a.numFaces || lane >= 8) return 0;
        const int64_t *src = lane < 2 ? a.co : lane < 4 ? a.cornerOff : lane < 6 ? a.fo : a.po;
        return __ldg((const long long *)src + f + (lane & 1));
    };
    int f = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    long long next = offsets_of(f);
    for (; f < a.numFaces; f += warps) {
        const long long mine = next;
        next = offsets_of(f + warps);
        const int64_t c0 = __shfl_sync(0xffffffffu, mine, 0);
        const int64_t c1 = __shfl_sync(0xffffffffu, mine, 1);
        const int64_t k0 = __shfl_sync(0xffffffffu, mine, 2);
        const int64_t k1 = __shfl_sync(0xffffffffu, mine, 3);
        const int64_t f0 = __shfl_sync(0xffffffffu, mine, 4);
        const int64_t f1 = __shfl_sync(0xffffffffu, mine, 5);
        const int base = (int)__shfl_sync(0xffffffffu, mine, 6);
        const int end = (int)__shfl_sync(0xffffffffu, mine, 7);
        const int nc = (int)(c1 - c0), N = (int)(k1 - k0);
        if (nc == 0 || k1 > a.numCorners || N < 3) continue;
        const int4 *cg = a.cornerInfo + k0;
        const bool small = N <= 32;
        const int pcWords = a.pointPC ? 5 * nc : 0;
        const int nf = (int)(f1 - f0), fWords = nf * FS;
        const int *pcSrc = a.coordPC + 5 * c0;
        int *d0 = a.facets + f0 * a.facetStride;
        const int off = a.meshIndices ? (int)c0 : 0;
        int nb = 0, interior = 0;
        bool tabled = false;
        // the point of coord idx, with kShareMade when this face made it
        auto point_of = [&](int idx) -> int {
            if (idx >= nb) return (idx + interior) | kShareMade;
            if (tabled) return table[w][idx];
            bool made;
            const int p = small ? share_point(corners[w], N, nb, interior, idx, made)
                                : share_point(cg, N, nb, interior, idx, made);
            return made ? (p | kShareMade) : p;
        };
        const int rounds = max(pcWords, fWords);
        for (int r0 = 0; r0 < rounds; r0 += 32 * kShareWords) {
            int pw[kShareWords], fw[kShareWords];
            int4 mine4 = make_int4(0, 0, 0, 0);
            if (r0 == 0 && small && lane < N) mine4 = __ldg(cg + lane);
#pragma unroll
            for (int u = 0; u < kShareWords; ++u) {
                const int k = r0 + lane + 32 * u;
                pw[u] = k < pcWords ? __ldg(pcSrc + k) : 0;
                fw[u] = k < fWords ? d0[(int64_t)(k / FS) * a.facetStride + (k % FS)] : -1;
            }
            if (r0 == 0) {
                if (small) {
                    if (lane < N) corners[w][lane] = mine4;
                    __syncwarp();
                }
                const int4 last = small ? corners[w][N - 1] : cg[N - 1];
                nb = last.x + (last.w & kCornerEdgeMask) + 1;
                interior = end - nc;
                if (small && nb <= kShareTable) {
                    for (int i = lane; i < nb; i += 32) {
                        bool made;
                        const int p = share_point(corners[w], N, nb, interior, i, made);
                        table[w][i] = made ? (p | kShareMade) : p;
                    }
                    __syncwarp();
                    tabled = true;
                }
            }
#pragma unroll
            for (int u = 0; u < kShareWords; ++u) {
                const int k = r0 + lane + 32 * u;
                if (k < pcWords) {
                    const int i = k / 5;
                    const int t = point_of(i);
                    const int p = t & ~kShareMade;
                    if ((t & kShareMade) && p >= base && p < end)
                        a.pointPC[5 * (int64_t)p + (k - 5 * i)] = pw[u];
                }
                if (k < fWords && fw[u] >= 0) {
                    const int local = fw[u] - off;
                    int p = -1;
                    if (local < nc && local >= 0) {
                        const int t = point_of(local);
                        p = (t == -1) ? -1 : (t & ~kShareMade);
                    } else {
                        share_error(a.err, 0, f);
                    }
                    d0[(int64_t)(k / FS) * a.facetStride + (k % FS)] = p;
                }
            }
        }
        if (a.pointCoords || a.pointFaces) {
            for (int i = lane; i < nc; i += 32) {
                const int t = point_of(i);
                const int p = t & ~kShareMade;
                if (!(t & kShareMade) || p < base || p >= end) continue;
                if (a.pointCoords) {
                    const float *s = a.coords + (c0 + i) * a.coordStride;
                    a.pointCoords[2 * (int64_t)p] = s[0];
                    a.pointCoords[2 * (int64_t)p + 1] = s[1];
                }
                if (a.pointFaces) a.pointFaces[p] = f;
            }
        }
        __syncwarp();
    }
}

// ---- edge rates from edge lengths (tutorial 2.1) ---------------------------------------------
// Thread per face corner: the length of the edge from the corner to the next corner of its
// face, from the corners' points (mesh vertices, or one point per corner), and the rate
// 1 + (int)(length / interval) capped at maxRate (tutorials/bfr/tutorial_2_1/
// bfr_tutorial_2_1.cpp:121-166).  Every float step is explicitly rounded, so a shared edge
// gets the same rate from both of its faces.
struct RateArgs {
    int numFaces, perCorner, stride, maxRate, numPoints;
    int64_t numCorners;
    float interval;
    const int *faceSizes, *faceVerts;
    const int64_t *cornerOff;
    const float *points;
    int *rates, *rateOffsets;
    int *err;
};

__global__ void __launch_bounds__(256) k_edge_rates(const RateArgs a) {
    const int stride = gridDim.x * blockDim.x;
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f <= a.numFaces; f += stride) {
        const int64_t c0 = a.cornerOff[f];
        if (a.rateOffsets) a.rateOffsets[f] = (int)c0;
        if (f == a.numFaces) continue;
        const int N = a.faceSizes[f];
        if (c0 + N > a.numCorners) {
            atomicAdd(a.err, 1);
            continue;
        }
        for (int i = 0; i < N; ++i) {
            const int64_t ci = c0 + i, cj = c0 + (i + 1 == N ? 0 : i + 1);
            int64_t pi = ci, pj = cj;
            if (!a.perCorner) {
                pi = a.faceVerts[ci];
                pj = a.faceVerts[cj];
                if ((uint64_t)pi >= (uint64_t)a.numPoints || (uint64_t)pj >= (uint64_t)a.numPoints) {
                    atomicAdd(a.err, 1);
                    a.rates[ci] = 1;
                    continue;
                }
            }
            const float *x0 = a.points + pi * a.stride, *x1 = a.points + pj * a.stride;
            const float d0 = fabsf(__fsub_rn(x0[0], x1[0]));
            const float d1 = fabsf(__fsub_rn(x0[1], x1[1]));
            const float d2 = fabsf(__fsub_rn(x0[2], x1[2]));
            const float len = __fsqrt_rn(
                __fadd_rn(__fadd_rn(__fmul_rn(d0, d0), __fmul_rn(d1, d1)), __fmul_rn(d2, d2)));
            const float q = __fdiv_rn(len, a.interval);
            // (int) of the quotient, saturated before the cap
            const int r = q < (float)a.maxRate ? 1 + (int)q : a.maxRate;
            a.rates[ci] = r < a.maxRate ? r : a.maxRate;
        }
    }
}

// Shared uniform patterns, cached per device and request (they depend only on the scheme's
// face size, the rate and the facet options) up to kPatternCacheBytes; beyond that a call
// builds them in per-call scratch.
struct PatternKey {
    int dev, reg, rate, fs, pq;
    bool operator==(const PatternKey &o) const {
        return dev == o.dev && reg == o.reg && rate == o.rate && fs == o.fs && pq == o.pq;
    }
};
struct Patterns {
    int patC[kNumShared + 1], patF[kNumShared + 1];
    void *mem = nullptr;
    size_t bytes = 0;
};
constexpr size_t kPatternCacheBytes = size_t(64) << 20;
std::mutex g_patMutex;
std::vector<std::pair<PatternKey, Patterns>> g_patterns;
size_t g_patBytes = 0;

void pattern_sizes(int reg, int rate, int fs, int pq, Patterns &p) {
    p.patC[0] = p.patF[0] = 0;
    for (int k = 0; k < kNumShared; ++k) {
        Face face;
        const bool v = face.init(reg, kFirstShared + k, 1, nullptr, fs, pq, rate);
        p.patC[k + 1] = p.patC[k] + (v ? face.num_coords() : 0);
        p.patF[k + 1] = p.patF[k] + (v ? face.nFacets : 0);
    }
    const size_t cb = sizeof(float) * 2 * (size_t)p.patC[kNumShared];
    p.bytes = ((cb + 15) & ~size_t(15)) + sizeof(int) * (size_t)fs * p.patF[kNumShared] +
              sizeof(int) * 2 * (kNumShared + 1);
}

// Builds the patterns of `p` into p.mem: the offset tables go after the coords and facets.
int build_patterns(int reg, int rate, int fs, int pq, Patterns &p, cudaStream_t s,
                   const char *who) {
    const size_t cb = sizeof(float) * 2 * (size_t)p.patC[kNumShared];
    float *pc = (float *)p.mem;
    int *pf = (int *)((char *)p.mem + ((cb + 15) & ~size_t(15)));
    int *tables = pf + (size_t)fs * p.patF[kNumShared];
    int host[2 * (kNumShared + 1)];
    for (int k = 0; k <= kNumShared; ++k) host[k] = p.patC[k], host[kNumShared + 1 + k] = p.patF[k];
    int st = check_cuda(cudaMemcpyAsync(tables, host, sizeof(host), cudaMemcpyHostToDevice, s), who);
    if (st != GB300_OK) return st;
    k_tess_patterns<<<1, 32, 0, s>>>(reg, rate, fs, pq, tables, tables + kNumShared + 1, pc, pf);
    count_launch();
    st = check_launch(who);
    // the host array is read by the copy above
    if (st == GB300_OK) st = check_cuda(cudaStreamSynchronize(s), who);
    return st;
}

int grid_for(long long items, int threads, int perSm) {
    long long blocks = (items + threads - 1) / threads;
    const long long cap = (long long)num_sms() * perSm;
    if (blocks > cap) blocks = cap;
    return (int)(blocks < 1 ? 1 : blocks);
}

struct Opts {
    int fs, pq, coordStride, facetStride;
};

int read_options(const GB300TessellationOptions *o, Opts &out, const char *who) {
    out.fs = (o && o->facetSize == 4) ? 4 : 3;
    out.pq = o ? (o->preserveQuads != 0) : 0;
    out.coordStride = (o && o->coordStride) ? o->coordStride : 2;
    out.facetStride = (o && o->facetStride) ? o->facetStride : out.fs;
    if (out.coordStride < 2)
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: coordStride %d < 2", who, out.coordStride);
    if (out.facetStride < out.fs)
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: facetStride %d < facet size %d", who,
                    out.facetStride, out.fs);
    return ok();
}

int check_faces(int reg, int numFaces, const int *faceSizes, const char *who) {
    if (reg != 3 && reg != 4)
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: regularFaceSize must be 3 or 4", who);
    if (numFaces < 0 || (numFaces > 0 && !faceSizes))
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: bad face list", who);
    return ok();
}

}  // namespace
}  // namespace gb300

using namespace gb300;

extern "C" int GB300TessellationCount(int regularFaceSize, int numFaces, const int *faceSizes,
                                      const int *rateOffsets, const int *rates, int uniformRate,
                                      const GB300TessellationOptions *options,
                                      int64_t *coordOffsets, int64_t *facetOffsets,
                                      int64_t *ptexOffsets, int64_t *totals, void *stream) {
    const char *who = "GB300TessellationCount";
    int st = check_faces(regularFaceSize, numFaces, faceSizes, who);
    if (st != GB300_OK) return st;
    Opts o;
    if ((st = read_options(options, o, who)) != GB300_OK) return st;
    if (!coordOffsets || !facetOffsets || !ptexOffsets || !totals)
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: null offsets or totals", who);
    cudaStream_t s = as_stream(stream);
    const int n1 = numFaces + 1;
    int64_t *counts = nullptr;
    if ((st = scratch_alloc((void **)&counts, sizeof(int64_t) * 3 * (size_t)n1, s, who)) !=
        GB300_OK)
        return st;
    CountArgs a;
    a.reg = regularFaceSize;
    a.numFaces = numFaces;
    a.uniformRate = uniformRate;
    a.fs = o.fs;
    a.pq = o.pq;
    a.faceSizes = faceSizes;
    a.rateOffsets = rateOffsets;
    a.rates = rates;
    a.cc = counts;
    a.fc = counts + n1;
    a.pc = counts + 2 * (size_t)n1;
    k_tess_count<<<grid_for(n1, 256, 16), 256, 0, s>>>(a);
    count_launch();
    st = check_launch(who);
    size_t bytes = 0;
    void *tmp = nullptr;
    if (st == GB300_OK)
        st = check_cuda(cub::DeviceScan::ExclusiveSum(nullptr, bytes, a.cc, coordOffsets, n1, s),
                        who);
    if (st == GB300_OK) st = scratch_alloc(&tmp, bytes, s, who);
    int64_t *outs[3] = {coordOffsets, facetOffsets, ptexOffsets};
    for (int k = 0; k < 3 && st == GB300_OK; ++k)
        st = check_cuda(cub::DeviceScan::ExclusiveSum(tmp, bytes, counts + k * (size_t)n1,
                                                      outs[k], n1, s),
                        who);
    int64_t host[3] = {0, 0, 0};
    for (int k = 0; k < 3 && st == GB300_OK; ++k)
        st = check_cuda(cudaMemcpyAsync(host + k, outs[k] + numFaces, sizeof(int64_t),
                                        cudaMemcpyDeviceToHost, s),
                        who);
    if (tmp) scratch_free(tmp, s);
    scratch_free(counts, s);
    if (st == GB300_OK) st = check_cuda(cudaStreamSynchronize(s), who);
    if (st != GB300_OK) return st;
    for (int k = 0; k < 3; ++k) totals[k] = host[k];
    if (host[0] > INT_MAX)
        return fail(GB300_ERR_INVALID_ARGUMENT,
                    "%s: %lld coords exceed the int range of facet indices", who,
                    (long long)host[0]);
    return ok();
}

extern "C" int GB300TessellationGenerate(
    int regularFaceSize, int numFaces, const int *faceSizes, const int *rateOffsets,
    const int *rates, int uniformRate, const GB300TessellationOptions *options,
    const int64_t *coordOffsets, const int64_t *facetOffsets, const int64_t *ptexOffsets,
    float *coords, int *facets, int offsetFacetIndices, const GB300PatchTable *table,
    void *patchCoords, void *stream) {
    const char *who = "GB300TessellationGenerate";
    int st = check_faces(regularFaceSize, numFaces, faceSizes, who);
    if (st != GB300_OK) return st;
    Opts o;
    if ((st = read_options(options, o, who)) != GB300_OK) return st;
    if (!coordOffsets || !facetOffsets || !coords || !facets)
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: null offsets or outputs", who);
    if ((table != nullptr) != (patchCoords != nullptr) || (table && !ptexOffsets))
        return fail(GB300_ERR_INVALID_ARGUMENT,
                    "%s: locating needs the table, ptex offsets and a PatchCoord buffer", who);
    if (numFaces == 0) return ok();
    cudaStream_t s = as_stream(stream);

    GenArgs a;
    a.reg = regularFaceSize;
    a.numFaces = numFaces;
    a.uniformRate = uniformRate;
    a.fs = o.fs;
    a.pq = o.pq;
    a.coordStride = o.coordStride;
    a.facetStride = o.facetStride;
    a.faceSizes = faceSizes;
    a.rateOffsets = rateOffsets;
    a.rates = rates;
    a.co = coordOffsets;
    a.fo = facetOffsets;
    a.po = ptexOffsets;
    a.coords = coords;
    a.facets = facets;
    a.offsetIndices = offsetFacetIndices != 0;
    a.coordPairs = o.coordStride == 2 && ((uintptr_t)coords & 7) == 0;
    a.shared = rates == nullptr && uniformRate >= 1;
    a.patCoords = nullptr;
    a.patFacets = nullptr;
    a.locate = table != nullptr;
    a.patchCoords = (int *)patchCoords;
    if (table) a.map = view_of(*patch_map_of(table));

    Patterns scratchPat;
    if (a.shared) {
        int dev = 0;
        if ((st = check_cuda(cudaGetDevice(&dev), who)) != GB300_OK) return st;
        const PatternKey key{dev, regularFaceSize, uniformRate, o.fs, o.pq};
        const Patterns *use = nullptr;
        {
            std::lock_guard<std::mutex> lock(g_patMutex);
            for (auto &e : g_patterns)
                if (e.first == key) use = &e.second;
            if (!use) {
                Patterns p;
                pattern_sizes(regularFaceSize, uniformRate, o.fs, o.pq, p);
                if (g_patBytes + p.bytes <= kPatternCacheBytes) {
                    if ((st = check_cuda(cudaMalloc(&p.mem, p.bytes), who)) != GB300_OK) return st;
                    if ((st = build_patterns(regularFaceSize, uniformRate, o.fs, o.pq, p, s,
                                             who)) != GB300_OK) {
                        cudaFree(p.mem);
                        return st;
                    }
                    g_patterns.emplace_back(key, p);
                    g_patBytes += p.bytes;
                    use = &g_patterns.back().second;
                }
            }
            if (use) {
                for (int k = 0; k <= kNumShared; ++k) a.patC[k] = use->patC[k], a.patF[k] = use->patF[k];
                const size_t cb = sizeof(float) * 2 * (size_t)use->patC[kNumShared];
                a.patCoords = (const float *)use->mem;
                a.patFacets = (const int *)((const char *)use->mem + ((cb + 15) & ~size_t(15)));
            }
        }
        if (!use) {
            pattern_sizes(regularFaceSize, uniformRate, o.fs, o.pq, scratchPat);
            if ((st = scratch_alloc(&scratchPat.mem, scratchPat.bytes, s, who)) != GB300_OK)
                return st;
            if ((st = build_patterns(regularFaceSize, uniformRate, o.fs, o.pq, scratchPat, s,
                                     who)) != GB300_OK) {
                scratch_free(scratchPat.mem, s);
                return st;
            }
            for (int k = 0; k <= kNumShared; ++k)
                a.patC[k] = scratchPat.patC[k], a.patF[k] = scratchPat.patF[k];
            const size_t cb = sizeof(float) * 2 * (size_t)scratchPat.patC[kNumShared];
            a.patCoords = (const float *)scratchPat.mem;
            a.patFacets = (const int *)((const char *)scratchPat.mem + ((cb + 15) & ~size_t(15)));
        }
    }

    // faces without a shared pattern (per-face rates, polygons above 10 sides)
    void *dd = nullptr;
    a.dedupe = 0;
    if (!a.shared && st == GB300_OK) {
        unsigned int cap = 1024;
        while (cap < 2u * (unsigned int)numFaces && cap < (1u << 30)) cap <<= 1;
        const size_t kb = sizeof(unsigned long long) * cap, ob = sizeof(int) * cap;
        const size_t fb = sizeof(int) * (size_t)numFaces;
        st = scratch_alloc(&dd, kb + ob + fb, s, who);
        if (st == GB300_OK) {
            a.keys = (unsigned long long *)dd;
            a.owners = (int *)((char *)dd + kb);
            a.faceSlot = (int *)((char *)dd + kb + ob);
            a.slotMask = cap - 1;
            st = check_cuda(cudaMemsetAsync(a.keys, 0xff, kb, s), who);
            if (st == GB300_OK) st = check_cuda(cudaMemsetAsync(a.owners, 0x7f, ob, s), who);
        }
        if (st == GB300_OK) {
            k_tess_dedupe<<<grid_for(numFaces, 256, 8), 256, 0, s>>>(a);
            count_launch();
            st = check_launch(who);
            a.dedupe = 1;
        }
    }
    if (st == GB300_OK) {
        // with shared patterns only polygons above 10 sides are generated per face: none for
        // a triangle scheme, only quad sub-face polygons for a quad scheme
        const int grid = grid_for(numFaces, 128, 16);
        if (regularFaceSize == 3) {
            if (!a.shared) {
                k_tess_generate<tess::kTri><<<grid, 128, 0, s>>>(a);
                count_launch();
            }
        } else {
            if (!a.shared) {
                k_tess_generate<tess::kQuad><<<grid, 128, 0, s>>>(a);
                count_launch();
            }
            k_tess_generate<tess::kQsub><<<grid, 128, 0, s>>>(a);
            count_launch();
        }
        st = check_launch(who);
    }
    if (st == GB300_OK && (a.shared || a.locate || a.dedupe)) {
        const int blocks = grid_for((long long)numFaces * 32, 256, 8);
        if (o.fs == 4)
            k_tess_finish<4><<<blocks, 256, 0, s>>>(a);
        else
            k_tess_finish<3><<<blocks, 256, 0, s>>>(a);
        count_launch();
        st = check_launch(who);
    }
    if (dd) scratch_free(dd, s);
    if (scratchPat.mem) scratch_free(scratchPat.mem, s);
    return st;
}

extern "C" int GB300TessellationShare(
    int regularFaceSize, int numFaces, const int *faceSizes, const int *rateOffsets,
    const int *rates, int uniformRate, const GB300TessellationOptions *options,
    const int64_t *coordOffsets, const int64_t *facetOffsets, const int *faceVerts,
    const int *faceEdges, int64_t numCorners, int numVertices, int numEdges, int *facets,
    int meshFacetIndices,
    const void *coordPatchCoords, const float *coords, int64_t *pointOffsets,
    void *pointPatchCoords, float *pointCoords, int *pointFaces, int *vertexPoints,
    int *edgePoints, int64_t *numPoints, void *stream) {
    const char *who = "GB300TessellationShare";
    int st = check_faces(regularFaceSize, numFaces, faceSizes, who);
    if (st != GB300_OK) return st;
    Opts o;
    if ((st = read_options(options, o, who)) != GB300_OK) return st;
    if (!coordOffsets || !facetOffsets || !facets || !pointOffsets || !numPoints)
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: null offsets, facets or outputs", who);
    if (numVertices < 0 || numEdges < 0 || numCorners < 0 ||
        (numCorners > 0 && (!faceVerts || !faceEdges)))
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: bad face vertices or edges", who);
    if ((pointPatchCoords && !coordPatchCoords) || (pointCoords && !coords))
        return fail(GB300_ERR_INVALID_ARGUMENT,
                    "%s: per-point outputs need the per-coord inputs they copy", who);
    cudaStream_t s = as_stream(stream);
    ShareArgs a;
    a.reg = regularFaceSize;
    a.numFaces = numFaces;
    a.uniformRate = uniformRate;
    a.fs = o.fs;
    a.pq = o.pq;
    a.coordStride = o.coordStride;
    a.facetStride = o.facetStride;
    a.meshIndices = meshFacetIndices != 0;
    a.numVertices = numVertices;
    a.numEdges = numEdges;
    a.numCorners = numCorners;
    a.faceSizes = faceSizes;
    a.faceVerts = faceVerts;
    a.faceEdges = faceEdges;
    a.rateOffsets = rateOffsets;
    a.rates = rates;
    a.co = coordOffsets;
    a.fo = facetOffsets;
    a.po = pointOffsets;
    a.facets = facets;
    a.coordPC = (const int *)coordPatchCoords;
    a.coords = coords;
    a.pointPC = (int *)pointPatchCoords;
    a.pointCoords = pointCoords;
    a.pointFaces = pointFaces;

    // scratch: corner offsets and counts (numFaces + 1 each), corner records, vertex and edge
    // keys, inside counts of edges, the point arrays the caller did not ask for, error words
    const size_t n1 = (size_t)numFaces + 1, nv = (size_t)numVertices, ne = (size_t)numEdges;
    auto up = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t bOff = up(sizeof(int64_t) * n1), bKeyV = up(sizeof(unsigned long long) * nv),
                 bKeyE = up(sizeof(unsigned long long) * ne), bEdgeN = up(sizeof(int) * ne),
                 bVP = vertexPoints ? 0 : up(sizeof(int) * nv),
                 bEP = edgePoints ? 0 : up(sizeof(int) * ne), bErr = up(sizeof(int) * 8),
                 bCorner = up(sizeof(int4) * (size_t)numCorners);
    size_t scanBytes = 0;
    if ((st = check_cuda(cub::DeviceScan::ExclusiveSum(nullptr, scanBytes, (int64_t *)nullptr,
                                                       (int64_t *)nullptr, (int)n1, s),
                         who)) != GB300_OK)
        return st;
    char *mem = nullptr;
    const size_t total =
        2 * bOff + bCorner + bKeyV + bKeyE + bEdgeN + bVP + bEP + bErr + up(scanBytes);
    if ((st = scratch_alloc((void **)&mem, total, s, who)) != GB300_OK) return st;
    char *q = mem;
    a.cornerOff = (int64_t *)q, q += bOff;
    a.counts = (int64_t *)q, q += bOff;
    a.cornerInfo = (int4 *)q, q += bCorner;
    a.vertKey = (unsigned long long *)q, q += bKeyV;
    a.edgeKey = (unsigned long long *)q, q += bKeyE;
    a.edgeN = (int *)q, q += bEdgeN;
    a.vertPoint = vertexPoints ? vertexPoints : (int *)q, q += bVP;
    a.edgePoint = edgePoints ? edgePoints : (int *)q, q += bEP;
    a.err = (int *)q, q += bErr;
    void *scan = q;

    const int grid = grid_for((long long)n1, 256, 16);
    const size_t most = n1 > nv ? (n1 > ne ? n1 : ne) : (nv > ne ? nv : ne);
    k_share_init<<<grid_for((long long)most, 256, 16), 256, 0, s>>>(a);
    count_launch();
    st = check_launch(who);
    if (st == GB300_OK)
        st = check_cuda(cub::DeviceScan::ExclusiveSum(scan, scanBytes, a.counts, a.cornerOff,
                                                      (int)n1, s),
                        who);
    if (st == GB300_OK) {
        k_share_own<<<grid, 256, 0, s>>>(a);
        count_launch();
        k_share_count<<<grid, 256, 0, s>>>(a);
        count_launch();
        st = check_launch(who);
    }
    if (st == GB300_OK)
        st = check_cuda(cub::DeviceScan::ExclusiveSum(scan, scanBytes, a.counts, pointOffsets,
                                                      (int)n1, s),
                        who);
    if (st == GB300_OK && numFaces > 0) {
        k_share_assign<<<grid, 256, 0, s>>>(a);
        count_launch();
        k_share_corners<<<grid, 256, 0, s>>>(a);
        count_launch();
        const int blocks = grid_for((long long)numFaces * 32, 256, 8);
        if (o.fs == 4)
            k_share_emit<4><<<blocks, 256, 0, s>>>(a);
        else
            k_share_emit<3><<<blocks, 256, 0, s>>>(a);
        count_launch();
        st = check_launch(who);
    }
    int host[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (st == GB300_OK) {
        k_share_totals<<<1, 32, 0, s>>>(a);
        count_launch();
        st = check_launch(who);
    }
    if (st == GB300_OK)
        st = check_cuda(cudaMemcpyAsync(host, a.err, sizeof(host), cudaMemcpyDeviceToHost, s), who);
    scratch_free(mem, s);
    if (st == GB300_OK) st = check_cuda(cudaStreamSynchronize(s), who);
    if (st != GB300_OK) return st;
    int64_t points = 0, corners = 0;
    std::memcpy(&points, host + 4, sizeof(points));
    std::memcpy(&corners, host + 6, sizeof(corners));
    if (corners != numCorners)
        return fail(GB300_ERR_INVALID_ARGUMENT,
                    "%s: the face sizes add up to %lld corners, the face vertices and edges "
                    "have %lld", who, (long long)corners, (long long)numCorners);
    if (host[0])
        return fail(GB300_ERR_INVALID_ARGUMENT,
                    "%s: %d vertex, edge or facet indices out of range, or faces whose coords "
                    "disagree with Count (first in face %d)", who, host[0], host[1]);
    if (host[2])
        return fail(GB300_ERR_INVALID_ARGUMENT,
                    "%s: %d face edges run at another rate than the face that made the edge's "
                    "points (first in face %d): shared points need one rate per edge",
                    who, host[2], host[3]);
    *numPoints = points;
    return ok();
}

extern "C" int GB300TessellationEdgeRates(int numFaces, const int *faceSizes,
                                          const int *faceVerts, int64_t numCorners,
                                          const float *points, int numPoints, int pointStride,
                                          int pointsPerCorner, float interval, int maxRate,
                                          int *rateOffsets, int *rates, void *stream) {
    const char *who = "GB300TessellationEdgeRates";
    if (numFaces < 0 || numCorners < 0 || (numFaces > 0 && !faceSizes) || !rates ||
        !points || pointStride < 3 || !(interval > 0.0f) || maxRate < 1 ||
        (!pointsPerCorner && (!faceVerts || numPoints < 0)))
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: bad arguments", who);
    cudaStream_t s = as_stream(stream);
    const size_t n1 = (size_t)numFaces + 1;
    auto up = [](size_t b) { return (b + 255) & ~size_t(255); };
    size_t scanBytes = 0;
    int st = check_cuda(cub::DeviceScan::ExclusiveSum(nullptr, scanBytes, (int64_t *)nullptr,
                                                      (int64_t *)nullptr, (int)n1, s),
                        who);
    if (st != GB300_OK) return st;
    char *mem = nullptr;
    if ((st = scratch_alloc((void **)&mem, 2 * up(8 * n1) + up(8 * 4) + up(scanBytes), s,
                            who)) != GB300_OK)
        return st;
    ShareArgs sa{};
    sa.numFaces = numFaces;
    sa.faceSizes = faceSizes;
    sa.counts = (int64_t *)mem;
    sa.err = (int *)(mem + 2 * up(8 * n1));
    sa.numVertices = sa.numEdges = 0;
    RateArgs a{};
    a.numFaces = numFaces;
    a.perCorner = pointsPerCorner != 0;
    a.stride = pointStride;
    a.maxRate = maxRate;
    a.numPoints = pointsPerCorner ? 0 : numPoints;
    a.numCorners = numCorners;
    a.interval = interval;
    a.faceSizes = faceSizes;
    a.faceVerts = faceVerts;
    a.cornerOff = (const int64_t *)(mem + up(8 * n1));
    a.points = points;
    a.rates = rates;
    a.rateOffsets = rateOffsets;
    a.err = sa.err;
    const int grid = grid_for((long long)n1, 256, 16);
    k_share_init<<<grid, 256, 0, s>>>(sa);  // face sizes into counts, error words cleared
    count_launch();
    st = check_launch(who);
    if (st == GB300_OK)
        st = check_cuda(cub::DeviceScan::ExclusiveSum(mem + 2 * up(8 * n1) + up(32), scanBytes,
                                                      sa.counts, (int64_t *)a.cornerOff,
                                                      (int)n1, s),
                        who);
    if (st == GB300_OK) {
        k_edge_rates<<<grid, 256, 0, s>>>(a);
        count_launch();
        st = check_launch(who);
    }
    int host[2] = {0, 0};
    int64_t corners = 0;
    if (st == GB300_OK)
        st = check_cuda(cudaMemcpyAsync(host, a.err, sizeof(host), cudaMemcpyDeviceToHost, s), who);
    if (st == GB300_OK)
        st = check_cuda(cudaMemcpyAsync(&corners, a.cornerOff + numFaces, sizeof(corners),
                                        cudaMemcpyDeviceToHost, s),
                        who);
    scratch_free(mem, s);
    if (st == GB300_OK) st = check_cuda(cudaStreamSynchronize(s), who);
    if (st != GB300_OK) return st;
    if (corners != numCorners)
        return fail(GB300_ERR_INVALID_ARGUMENT,
                    "%s: the face sizes add up to %lld corners, not %lld", who,
                    (long long)corners, (long long)numCorners);
    if (host[0])
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: %d vertex indices out of range", who,
                    host[0]);
    return ok();
}
