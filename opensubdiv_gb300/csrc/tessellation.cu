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
// A staged variant (faces generated into a shared-memory arena, copied out coalesced) was
// slower: about 900 bytes of arena per face left too few warps resident to hide latency.
#include "common.cuh"
#include "patchmap.h"
#include "patchmap_walk.cuh"
#include "tess_pattern.cuh"

#include <cub/device/device_scan.cuh>

#include <atomic>
#include <climits>
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
