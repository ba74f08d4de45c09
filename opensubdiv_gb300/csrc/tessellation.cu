// Bfr::Tessellation over every face of a mesh at once (bfr/tessellation.h:142-262), with the
// points located on a device patch table for evaluation.
//
// Three launches on one stream:
//   count    one thread per face: the face's coord, facet and ptex-face counts, then device
//            exclusive scans into the caller's offset arrays (the only host sync is the read
//            of the three totals, which the caller needs to size its buffers);
//   generate one thread per face pattern: with a single uniform rate every face of the same
//            size has the same pattern, so one thread builds it per face size (3..10) into
//            library scratch; other faces (per-face rates, larger polygons) are generated by
//            one thread each straight into their slice of the output;
//   finish   one warp per face, lanes over the face's coords and facets (coalesced): copies
//            the shared pattern out, offsets facet indices to the mesh-wide coord numbering
//            (Tessellation::TransformFacetCoordIndices, tessellation.cpp:2429-2447), and turns
//            each coord into a PatchCoord: Parameterization::ConvertCoordToNormalizedSubFace
//            (bfr/parameterization.cpp:135-162) picks the ptex sub-face of an N-gon, and the
//            PatchMap walk finds the patch -- the lookup the reference's Bfr regression does
//            for every tessellation coord (regression/bfr_evaluate/farPatchEvaluator.cpp:
//            190-207).
#include "common.cuh"
#include "patchmap.h"
#include "patchmap_walk.cuh"
#include "tess_pattern.cuh"

#include <cub/device/device_scan.cuh>

#include <climits>

namespace gb300 {
namespace {

using tess::Face;
using tess::Sink;

constexpr int kFirstShared = 3;  // face sizes with a shared uniform pattern: 3 .. 10
constexpr int kNumShared = 8;

struct FaceRates {
    int one;  // storage for a single rate (uniform or one per face)
    const int *p;
    int n;
};

__device__ __forceinline__ void rates_of(const int *rateOffsets, const int *rates,
                                         int uniformRate, int f, FaceRates &r) {
    if (!rates) {
        r.one = uniformRate;
        r.p = &r.one;
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
        const bool ok = face.init(a.reg, N, r.n, r.p, a.fs, a.pq);
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
    // shared uniform patterns for face sizes kFirstShared + k (packed: stride 2 / fs)
    int shared;
    int patC[kNumShared + 1], patF[kNumShared + 1];
    float *patCoords;
    int *patFacets;
    // location on a patch table (optional)
    int locate;
    PatchMapView map;
    int *patchCoords;  // 5 x 32 bit per coord
};

__device__ __forceinline__ bool uses_shared(const GenArgs &a, int N) {
    return a.shared && N >= kFirstShared && N < kFirstShared + kNumShared;
}

__global__ void __launch_bounds__(128) k_tess_generate(const GenArgs a) {
    const int nShared = a.shared ? kNumShared : 0;
    const int total = nShared + a.numFaces;
    const int stride = gridDim.x * blockDim.x;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += stride) {
        Face face;
        if (t < nShared) {
            const int rate = a.uniformRate;
            if (!face.init(a.reg, kFirstShared + t, 1, &rate, a.fs, a.pq)) continue;
            Sink o{a.patCoords + 2 * (int64_t)a.patC[t], 2, a.patFacets + (int64_t)a.fs * a.patF[t],
                   a.fs, a.fs};
            face.coords(o);
            face.facets(o);
            continue;
        }
        const int f = t - nShared;
        const int N = a.faceSizes[f];
        if (uses_shared(a, N)) continue;
        FaceRates r;
        rates_of(a.rateOffsets, a.rates, a.uniformRate, f, r);
        if (!face.init(a.reg, N, r.n, r.p, a.fs, a.pq)) continue;
        Sink o{a.coords + a.co[f] * a.coordStride, a.coordStride,
               a.facets + a.fo[f] * a.facetStride, a.fs, a.facetStride};
        face.coords(o);
        face.facets(o);
    }
}

__global__ void __launch_bounds__(256) k_tess_finish(const GenArgs a) {
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int f = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; f < a.numFaces; f += warps) {
        const int64_t c0 = a.co[f];
        const int nc = (int)(a.co[f + 1] - c0);
        if (nc == 0) continue;
        const int64_t f0 = a.fo[f];
        const int nf = (int)(a.fo[f + 1] - f0);
        const int N = a.faceSizes[f];
        const bool sh = uses_shared(a, N);
        const int k = N - kFirstShared;
        const float *src = sh ? a.patCoords + 2 * (int64_t)a.patC[k] : a.coords + c0 * a.coordStride;
        const int srcStride = sh ? 2 : a.coordStride;

        if (sh || a.locate) {
            // Parameterization of the face (bfr/parameterization.cpp:40-66)
            const bool subfaces = N != a.reg;
            const int udim = !subfaces ? 0 : (N < 10) ? 2 + (N > 4) : 1 + (int)sqrtf((float)(N - 1));
            const int ptex0 = a.locate ? (int)a.po[f] : 0;
            for (int i = lane; i < nc; i += 32) {
                const float u = src[(int64_t)i * srcStride], v = src[(int64_t)i * srcStride + 1];
                if (sh) {
                    float *d = a.coords + (c0 + i) * a.coordStride;
                    d[0] = u;
                    d[1] = v;
                }
                if (!a.locate) continue;
                int sub = 0;
                float s = u, t = v;
                if (subfaces) {
                    int ut = (int)u, vt = (int)v;
                    float uf = __fsub_rn(u, (float)ut), vf = __fsub_rn(v, (float)vt);
                    if (uf > 0.75f) { ut++; uf = __fsub_rn(uf, 1.0f); }
                    if (vf > 0.75f) { vt++; vf = __fsub_rn(vf, 1.0f); }
                    s = __fmul_rn(uf, 2.0f);
                    t = __fmul_rn(vf, 2.0f);
                    sub = udim * vt + ut;
                }
                const int4 h = patch_map_find(a.map, ptex0 + sub, s, t);
                int *o = a.patchCoords + 5 * (c0 + i);
                o[0] = h.x;
                o[1] = h.y;
                o[2] = h.z;
                o[3] = __float_as_int(s);
                o[4] = __float_as_int(t);
            }
        }
        if (sh || a.offsetIndices) {
            const int off = a.offsetIndices ? (int)c0 : 0;
            const int *pf = sh ? a.patFacets + (int64_t)a.fs * a.patF[k] : nullptr;
            for (int j = lane; j < nf * a.fs; j += 32) {
                const int q = j / a.fs, c = j - q * a.fs;
                int *d = a.facets + (f0 + q) * a.facetStride + c;
                const int v = sh ? pf[j] : *d;
                *d = v >= 0 ? v + off : v;
            }
        }
    }
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
    a.shared = rates == nullptr;
    a.patCoords = nullptr;
    a.patFacets = nullptr;
    a.locate = table != nullptr;
    a.patchCoords = (int *)patchCoords;
    if (table) a.map = view_of(*patch_map_of(table));

    void *pat = nullptr;
    if (a.shared) {
        // sizes of the shared patterns, from the same inventory the device uses
        a.patC[0] = a.patF[0] = 0;
        for (int k = 0; k < kNumShared; ++k) {
            tess::Face face;
            const int rate = uniformRate;
            const bool v = face.init(regularFaceSize, kFirstShared + k, 1, &rate, o.fs, o.pq);
            a.patC[k + 1] = a.patC[k] + (v ? face.num_coords() : 0);
            a.patF[k + 1] = a.patF[k] + (v ? face.nFacets : 0);
        }
        const size_t cb = sizeof(float) * 2 * (size_t)a.patC[kNumShared];
        const size_t fb = sizeof(int) * (size_t)o.fs * a.patF[kNumShared];
        if ((st = scratch_alloc(&pat, cb + fb + 16, s, who)) != GB300_OK) return st;
        a.patCoords = (float *)pat;
        a.patFacets = (int *)((char *)pat + ((cb + 15) & ~size_t(15)));
    }
    k_tess_generate<<<grid_for((a.shared ? kNumShared : 0) + (long long)numFaces, 128, 16), 128,
                      0, s>>>(a);
    count_launch();
    st = check_launch(who);
    if (st == GB300_OK && (a.shared || a.locate || a.offsetIndices)) {
        k_tess_finish<<<grid_for((long long)numFaces * 32, 256, 8), 256, 0, s>>>(a);
        count_launch();
        st = check_launch(who);
    }
    if (pat) scratch_free(pat, s);
    return st;
}
