// Device-resident tables and buffers: the GB300 counterparts of CudaStencilTable
// (osd/cudaEvaluator.cpp:100-145), CudaPatchTable (osd/cudaPatchTable.cpp:59-162) and
// CudaVertexBuffer (osd/cudaVertexBuffer.cpp:35-91).  Unlike the reference, a failed
// allocation or copy frees everything allocated so far and reports a status.
#include "common.cuh"
#include "patchmap.h"
#include "sell.h"
#include "stencils_batch.h"
#include "tables.h"

#include <algorithm>
#include <new>
#include <thread>
#include <vector>

using namespace gb300;

namespace {

// Allocates `bytes` (rounded up to 16 so bulk copies of the tail stay in bounds; 16 zero bytes
// for an empty array, so a present array is never null) and copies `host` into it; returns
// false (with the status recorded) on failure.  A null `host` leaves *dptr null.
bool upload(void **dptr, const void *host, size_t bytes, cudaStream_t s, const char *what) {
    *dptr = nullptr;
    if (!host) return true;
    size_t padded = std::max<size_t>(16, (bytes + 15) & ~(size_t)15);
    if (check_cuda(cudaMalloc(dptr, padded), what) != GB300_OK) {
        *dptr = nullptr;
        return false;
    }
    if (padded != bytes &&
        check_cuda(cudaMemsetAsync((char *)*dptr + bytes, 0, padded - bytes, s), what) != GB300_OK)
        return false;
    if (bytes && check_cuda(cudaMemcpyAsync(*dptr, host, bytes, cudaMemcpyHostToDevice, s),
                            what) != GB300_OK)
        return false;
    return true;
}

void release(void *&p) {
    if (p) cudaFree(p);
    p = nullptr;
}

// Device layout of an owned stencil table: the entries of every stencil are stored in
// ascending control-vertex order (weights permuted alongside).  The stencil -- a weighted
// sum -- is unchanged; neighbouring stencils then touch the same source rows at the same
// entry position, which cuts the distinct rows per warp-wide gather.  Applied only when the
// stencils' entry ranges are disjoint and inside [0, nnz); returns false otherwise.
bool sort_entries(int numStencils, int64_t nnz, const int *sizes, const int *offsets,
                  const int *indices, const float *const *w, std::vector<int> &idxOut,
                  std::vector<std::vector<float>> &wOut) {
    int64_t prevEnd = 0;
    for (int i = 0; i < numStencils; ++i) {
        if (sizes[i] < 0 || offsets[i] < prevEnd || (int64_t)offsets[i] + sizes[i] > nnz)
            return false;
        prevEnd = (int64_t)offsets[i] + sizes[i];
    }
    idxOut.assign(indices, indices + nnz);
    wOut.assign(9, {});
    for (int k = 0; k < 6; ++k)
        if (w[k]) wOut[k].assign(w[k], w[k] + nnz);
    const int nth = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<std::thread> pool;
    for (int t = 0; t < nth; ++t) {
        pool.emplace_back([&, t]() {
            const int lo = (int)((int64_t)numStencils * t / nth);
            const int hi = (int)((int64_t)numStencils * (t + 1) / nth);
            for (int i = lo; i < hi; ++i) {
                const int o = offsets[i], n = sizes[i];
                // insertion sort of (index, weights) pairs by index: stencils are short
                for (int a = o + 1; a < o + n; ++a) {
                    const int key = idxOut[a];
                    float wk[6] = {0, 0, 0, 0, 0, 0};
                    for (int k = 0; k < 6; ++k)
                        if (!wOut[k].empty()) wk[k] = wOut[k][a];
                    int b = a - 1;
                    while (b >= o && idxOut[b] > key) {
                        idxOut[b + 1] = idxOut[b];
                        for (int k = 0; k < 6; ++k)
                            if (!wOut[k].empty()) wOut[k][b + 1] = wOut[k][b];
                        --b;
                    }
                    idxOut[b + 1] = key;
                    for (int k = 0; k < 6; ++k)
                        if (!wOut[k].empty()) wOut[k][b + 1] = wk[k];
                }
            }
        });
    }
    for (auto &th : pool) th.join();
    return true;
}

}  // namespace

struct GB300StencilTable {
    int numStencils = 0;
    int64_t nnz = 0;
    int numControl = 0;  // largest control index + 1 (rows of the source the table reads)
    void *buf[9] = {nullptr};  // sizes, offsets, indices, w, du, dv, duu, duv, dvv
    // Sliced evaluation layout (sell.h): sz, sliceSlot, idx, w x 6, outRow
    gb300::SellTable sell;
    void *sbuf[10] = {nullptr};
    ~GB300StencilTable() {
        for (auto &p : buf) release(p);
        for (auto &p : sbuf) release(p);
    }
};

// A varying or face-varying (arrays, indices[, params]) set evaluated with the vertex table's
// patch handles (osd/cpuPatchTable.cpp:75-114).
struct PatchSet {
    int numArrays = 0, numParams = 0;
    int quadFamily = 0;
    int64_t numIndices = 0;
    void *arrays = nullptr, *indices = nullptr, *params = nullptr;
    void free() {
        release(arrays);
        release(indices);
        release(params);
        numArrays = 0;
    }
};

struct GB300PatchTable {
    int numArrays = 0, numPatches = 0;
    int quadFamily = 0;  // all arrays REGULAR / GREGORY_BASIS / QUADS
    int64_t numIndices = 0;
    void *arrays = nullptr, *indices = nullptr, *params = nullptr;
    PatchMapDevice map;
    std::vector<int> hostArrays;  // 6 ints per array (validation of varying / fvar sets)
    PatchSet varying;
    std::vector<PatchSet> fvar;
    ~GB300PatchTable() {
        release(arrays);
        release(indices);
        release(params);
        release(map.nodes);
        release(map.handles);
        varying.free();
        for (PatchSet &f : fvar) f.free();
    }
};

namespace gb300 {
const PatchMapDevice *patch_map_of(const GB300PatchTable *table) {
    return table ? &table->map : nullptr;
}
}  // namespace gb300

struct GB300VertexBuffer {
    int numElements = 0, numVertices = 0;
    float *mem = nullptr;
    ~GB300VertexBuffer() {
        if (mem) cudaFree(mem);
    }
};

extern "C" {

GB300StencilTable *GB300StencilTableCreate(int numStencils, int64_t nnz, const int *sizes,
                                           const int *offsets, const int *indices,
                                           const float *weights, const float *duWeights,
                                           const float *dvWeights, const float *duuWeights,
                                           const float *duvWeights, const float *dvvWeights,
                                           void *stream) {
    if (numStencils < 0 || nnz < 0 || (numStencils > 0 && (!sizes || !offsets)) ||
        (nnz > 0 && (!indices || !weights))) {
        fail(GB300_ERR_INVALID_ARGUMENT, "GB300StencilTableCreate: bad arguments");
        return nullptr;
    }
    for (int i = 0; i < numStencils; ++i) {
        if (sizes[i] < 0 || offsets[i] < 0 || (int64_t)offsets[i] + sizes[i] > nnz) {
            fail(GB300_ERR_INVALID_ARGUMENT,
                 "GB300StencilTableCreate: stencil %d's entries [%d, %d + %d) outside [0, %lld)",
                 i, offsets[i], offsets[i], sizes[i], (long long)nnz);
            return nullptr;
        }
    }
    cudaStream_t s = as_stream(stream);
    GB300StencilTable *t = new (std::nothrow) GB300StencilTable;
    if (!t) {
        fail(GB300_ERR_OUT_OF_MEMORY, "GB300StencilTableCreate: host allocation");
        return nullptr;
    }
    t->numStencils = numStencils;
    t->nnz = nnz;
    {
        int mx = -1;
        for (int64_t e = 0; e < nnz; ++e) mx = std::max(mx, indices[e]);
        t->numControl = mx + 1;
    }
    const float *wsrc[6] = {weights, duWeights, dvWeights, duuWeights, duvWeights, dvvWeights};
    std::vector<int> sortedIdx;
    std::vector<std::vector<float>> sortedW;
    if (nnz > 0 && sort_entries(numStencils, nnz, sizes, offsets, indices, wsrc, sortedIdx,
                                sortedW)) {
        indices = sortedIdx.data();
        for (int k = 0; k < 6; ++k)
            if (wsrc[k]) wsrc[k] = sortedW[k].data();
    }
    const void *host[9] = {sizes, offsets, indices, wsrc[0], wsrc[1],
                           wsrc[2], wsrc[3], wsrc[4], wsrc[5]};
    const size_t bytes[9] = {(size_t)numStencils * 4, (size_t)numStencils * 4,
                             (size_t)nnz * 4, (size_t)nnz * 4, (size_t)nnz * 4,
                             (size_t)nnz * 4, (size_t)nnz * 4, (size_t)nnz * 4,
                             (size_t)nnz * 4};
    for (int k = 0; k < 9; ++k) {
        if (!upload(&t->buf[k], host[k], bytes[k], s, "GB300StencilTableCreate")) {
            delete t;
            return nullptr;
        }
    }
    const int r = gb300::build_sell(numStencils, (const int *)t->buf[0], (const int *)t->buf[1],
                                    (const int *)t->buf[2], (const float *const *)(t->buf + 3), s,
                                    t->sell, t->sbuf, "GB300StencilTableCreate");
    if (r != GB300_OK && r != GB300_ERR_UNSUPPORTED) {
        delete t;
        return nullptr;
    }
    if (check_cuda(cudaStreamSynchronize(s), "GB300StencilTableCreate") != GB300_OK) {
        delete t;
        return nullptr;
    }
    ok();
    return t;
}

void GB300StencilTableDestroy(GB300StencilTable *t) { delete t; }

int GB300StencilTableGetNumStencils(const GB300StencilTable *t) { return t ? t->numStencils : 0; }

int64_t GB300StencilTableGetNumIndices(const GB300StencilTable *t) { return t ? t->nnz : 0; }

void *GB300StencilTableGetBuffer(const GB300StencilTable *t, int which) {
    if (!t || which < 0 || which > 8) return nullptr;
    return t->buf[which];
}

}  // extern "C"

namespace gb300 {
namespace batch {
int stencil_table_num_control(const GB300StencilTable *t) { return t ? t->numControl : 0; }
}  // namespace batch

const SellTable *stencil_table_sell(const GB300StencilTable *t) { return t ? &t->sell : nullptr; }

GB300StencilTable *adopt_stencil_table(int numStencils, int64_t nnz, int numControl,
                                       void *const buf[9], cudaStream_t s, const char *who) {
    GB300StencilTable *t = new (std::nothrow) GB300StencilTable;
    if (!t) {
        fail(GB300_ERR_OUT_OF_MEMORY, "%s: host allocation", who);
        return nullptr;
    }
    t->numStencils = numStencils;
    t->nnz = nnz;
    t->numControl = numControl;
    const int r = build_sell(numStencils, (const int *)buf[0], (const int *)buf[1],
                             (const int *)buf[2], (const float *const *)buf + 3, s, t->sell,
                             t->sbuf, who);
    if (r != GB300_OK && r != GB300_ERR_UNSUPPORTED) {
        delete t;  // buffers not yet owned
        return nullptr;
    }
    for (int k = 0; k < 9; ++k) t->buf[k] = buf[k];
    return t;
}
}  // namespace gb300

extern "C" int GB300StencilTableCopyBuffer(const GB300StencilTable *t, int which, void *hostDst,
                                           void *stream) {
    if (!t || which < 0 || which > 8 || !hostDst)
        return fail(GB300_ERR_INVALID_ARGUMENT, "GB300StencilTableCopyBuffer: bad arguments");
    const size_t n = which < 2 ? (size_t)t->numStencils : (size_t)t->nnz;
    if (!t->buf[which] || n == 0) return ok();
    cudaStream_t s = as_stream(stream);
    if (check_cuda(cudaMemcpyAsync(hostDst, t->buf[which], n * 4, cudaMemcpyDeviceToHost, s),
                   "GB300StencilTableCopyBuffer") != GB300_OK)
        return GB300_ERR_CUDA;
    if (check_cuda(cudaStreamSynchronize(s), "GB300StencilTableCopyBuffer") != GB300_OK)
        return GB300_ERR_CUDA;
    return ok();
}

extern "C" {

namespace {

int table_eval(const GB300StencilTable *t, const float *src, float *const *d, const int *st,
               int length, int srcStride, cudaStream_t s);

}  // namespace

int GB300StencilTableEval(const GB300StencilTable *t, const float *src, float *dst, float *du,
                          float *dv, float *duu, float *duv, float *dvv, int length,
                          int srcStride, int dstStride, int duStride, int dvStride,
                          int duuStride, int duvStride, int dvvStride, void *stream) {
    if (!t) return fail(GB300_ERR_INVALID_ARGUMENT, "GB300StencilTableEval: null table");
    float *d[6] = {dst, du, dv, duu, duv, dvv};
    const int st[6] = {dstStride, duStride, dvStride, duuStride, duvStride, dvvStride};
    cudaStream_t s = as_stream(stream);
    // Unaligned source rows (no vector gathers) of a large table: gather from a padded copy
    // (rows of 4, 8, 12 or 16 floats: vector loads) made on the same stream in stream-ordered
    // memory from the library's scratch pool.
    auto al = [](const void *p, uintptr_t m) { return ((uintptr_t)p & (m - 1)) == 0; };
    const bool unaligned = src && !((al(src, 32) && srcStride % 8 == 0) ||
                                    (al(src, 16) && srcStride % 4 == 0));
    const int ps = batch::padded_stride(length);
    if (unaligned && length > 0 && ps > 0 && srcStride >= length &&
        t->nnz >= (int64_t)t->numControl * 4 && t->nnz >= (1 << 20) && t->numControl > 0) {
        float *padded = nullptr;
        if (scratch_alloc((void **)&padded, (size_t)t->numControl * ps * 4, s,
                          "GB300StencilTableEval") == GB300_OK) {
            batch::PadJob j{src, padded, srcStride, length, t->numControl, ps, 0};
            int r = batch::launch_pad_one(j, s);
            if (r == GB300_OK) r = table_eval(t, padded, d, st, length, ps, s);
            scratch_free(padded, s);
            return r != GB300_OK ? r : check_launch("GB300StencilTableEval");
        }
        cudaGetLastError();  // no stream-ordered memory: evaluate in place
    }
    return table_eval(t, src, d, st, length, srcStride, s);
}

namespace {

int table_eval(const GB300StencilTable *t, const float *src, float *const *dIn, const int *st,
               int length, int srcStride, cudaStream_t s) {
    float *d[6] = {dIn[0], dIn[1], dIn[2], dIn[3], dIn[4], dIn[5]};
    const float *w[6];
    for (int k = 0; k < 6; ++k) {
        w[k] = (const float *)t->buf[3 + k];
        if (d[k] && !w[k])
            return fail(GB300_ERR_INVALID_ARGUMENT,
                        "GB300StencilTableEval: output %d requested but the table has no such "
                        "weights",
                        k);
    }
    if (t->sell.numSlices > 0 && t->sell.idx) {
        const float *sw[6];
        for (int k = 0; k < 6; ++k) sw[k] = d[k] ? t->sell.w[k] : nullptr;
        return eval_stencils_sell(t->sell, src, d, st, sw, length, srcStride, s,
                                  "GB300StencilTableEval");
    }
    return eval_stencils(src, d, st, w, length, srcStride, (const int *)t->buf[0],
                         (const int *)t->buf[1], (const int *)t->buf[2], 0, t->numStencils, s,
                         "GB300StencilTableEval");
}

}  // namespace

namespace {

// Patch arrays reference only evaluable types and stay inside the index / param buffers.
int check_patch_arrays(const char *who, int numArrays, const int *arr, int64_t numIndices,
                       int numPatches) {
    for (int a = 0; a < numArrays; ++a) {
        for (int k = 0; k < 2; ++k) {
            const int type = arr[6 * a + k];
            if (type != GB300_PATCH_QUADS && type != GB300_PATCH_TRIANGLES &&
                type != GB300_PATCH_LOOP && type != GB300_PATCH_REGULAR &&
                type != GB300_PATCH_GREGORY_BASIS && type != GB300_PATCH_GREGORY_TRIANGLE)
                return fail(GB300_ERR_UNSUPPORTED, "%s: patch type %d in array %d", who, type, a);
        }
        const int64_t last =
            (int64_t)arr[6 * a + 3] + (int64_t)arr[6 * a + 4] * arr[6 * a + 2];
        if (last > numIndices || arr[6 * a + 5] < 0 ||
            arr[6 * a + 5] + (int64_t)arr[6 * a + 2] > numPatches)
            return fail(GB300_ERR_INVALID_ARGUMENT, "%s: array %d out of range", who, a);
    }
    return GB300_OK;
}

int quad_family(int numArrays, const int *arr) {
    int q = numArrays > 0;
    for (int a = 0; a < numArrays; ++a)
        for (int k = 0; k < 2; ++k) {
            const int type = arr[6 * a + k];
            if (type != GB300_PATCH_REGULAR && type != GB300_PATCH_GREGORY_BASIS &&
                type != GB300_PATCH_QUADS)
                q = 0;
        }
    return q;
}

// A varying / face-varying set must describe the vertex table's patches: same arrays, same
// patch counts and first patch of each array, so the vertex patch handles index it.
int make_set(GB300PatchTable *t, const char *who, int numArrays, const void *patchArrays,
             int64_t numIndices, const int *patchIndices, int numParams, const void *params,
             cudaStream_t s, PatchSet &out) {
    if (!t || numArrays != t->numArrays || numIndices < 0 ||
        (numArrays > 0 && (!patchArrays || (numIndices > 0 && !patchIndices))))
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: bad arguments", who);
    const int *arr = (const int *)patchArrays;
    for (int a = 0; a < numArrays; ++a)
        if (arr[6 * a + 2] != t->hostArrays[6 * a + 2] ||
            arr[6 * a + 5] != t->hostArrays[6 * a + 5])
            return fail(GB300_ERR_INVALID_ARGUMENT,
                        "%s: array %d does not match the vertex patch array", who, a);
    const int patches = params ? numParams : t->numPatches;
    if (params && numParams != t->numPatches)
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: %d params for %d patches", who, numParams,
                    t->numPatches);
    int st = check_patch_arrays(who, numArrays, arr, numIndices, patches);
    if (st != GB300_OK) return st;
    PatchSet set;
    set.numArrays = numArrays;
    set.numIndices = numIndices;
    set.numParams = params ? numParams : 0;
    set.quadFamily = quad_family(numArrays, arr);
    if (!upload(&set.arrays, patchArrays, (size_t)numArrays * 24, s, who) ||
        !upload(&set.indices, patchIndices, (size_t)numIndices * 4, s, who) ||
        (params && !upload(&set.params, params, (size_t)numParams * 12, s, who)) ||
        check_cuda(cudaStreamSynchronize(s), who) != GB300_OK) {
        set.free();
        return GB300_ERR_OUT_OF_MEMORY;
    }
    out = set;
    return ok();
}

int eval_set(const GB300PatchTable *t, const PatchSet &set, const void *params,
             const float *src, float *dst, float *du, float *dv, float *duu, float *duv,
             float *dvv, int length, int srcStride, int dstStride, int duStride, int dvStride,
             int duuStride, int duvStride, int dvvStride, int n, const void *coords,
             void *stream, const char *who) {
    float *d[6] = {dst, du, dv, duu, duv, dvv};
    const int st[6] = {dstStride, duStride, dvStride, duuStride, duvStride, dvvStride};
    return eval_patches(src, d, st, length, srcStride, n, coords, set.arrays,
                        (const int *)set.indices, params, as_stream(stream), who,
                        set.quadFamily);
}

}  // namespace

GB300PatchTable *GB300PatchTableCreate(int numArrays, const void *patchArrays,
                                       int64_t numIndices, const int *patchIndices,
                                       int numPatches, const void *patchParams, int triangular,
                                       void *stream) {
    if (numArrays < 0 || numIndices < 0 || numPatches < 0 ||
        (numArrays > 0 && !patchArrays) || (numIndices > 0 && !patchIndices) ||
        (numPatches > 0 && !patchParams)) {
        fail(GB300_ERR_INVALID_ARGUMENT, "GB300PatchTableCreate: bad arguments");
        return nullptr;
    }
    const int *arr = (const int *)patchArrays;
    if (check_patch_arrays("GB300PatchTableCreate", numArrays, arr, numIndices, numPatches) !=
        GB300_OK)
        return nullptr;
    PatchMapHost hm;
    if (build_patch_map(numArrays, arr, numPatches, (const int *)patchParams, triangular, hm) !=
        GB300_OK)
        return nullptr;
    cudaStream_t s = as_stream(stream);
    GB300PatchTable *t = new (std::nothrow) GB300PatchTable;
    if (!t) {
        fail(GB300_ERR_OUT_OF_MEMORY, "GB300PatchTableCreate: host allocation");
        return nullptr;
    }
    t->numArrays = numArrays;
    t->numPatches = numPatches;
    t->numIndices = numIndices;
    t->quadFamily = quad_family(numArrays, arr);
    t->hostArrays.assign(arr, arr + 6 * (size_t)numArrays);
    const char *w = "GB300PatchTableCreate";
    if (!upload(&t->arrays, patchArrays, (size_t)numArrays * 24, s, w) ||
        !upload(&t->indices, patchIndices, (size_t)numIndices * 4, s, w) ||
        !upload(&t->params, patchParams, (size_t)numPatches * 12, s, w) ||
        !upload(&t->map.nodes, hm.nodes.data(), hm.nodes.size() * 4, s, w) ||
        !upload(&t->map.handles, hm.handles.data(), hm.handles.size() * 4, s, w) ||
        check_cuda(cudaStreamSynchronize(s), w) != GB300_OK) {
        delete t;
        return nullptr;
    }
    t->map.triangular = triangular;
    t->map.minFace = hm.minFace;
    t->map.maxFace = hm.maxFace;
    t->map.maxDepth = hm.maxDepth;
    t->map.numPatches = numPatches;
    ok();
    return t;
}

void GB300PatchTableDestroy(GB300PatchTable *t) { delete t; }

void *GB300PatchTableGetBuffer(const GB300PatchTable *t, int which) {
    if (!t) return nullptr;
    return which == 0 ? t->arrays : which == 1 ? t->indices : which == 2 ? t->params : nullptr;
}

int GB300PatchTableGetNumArrays(const GB300PatchTable *t) { return t ? t->numArrays : 0; }

int GB300PatchTableGetNumPatches(const GB300PatchTable *t) { return t ? t->numPatches : 0; }

int GB300PatchTableFindPatches(const GB300PatchTable *t, int n, const int *faces, const float *u,
                               const float *v, void *coordsOut, void *stream) {
    if (!t) return fail(GB300_ERR_INVALID_ARGUMENT, "GB300PatchTableFindPatches: null table");
    return find_patches(t->map, n, faces, u, v, coordsOut, as_stream(stream));
}

int GB300PatchTableEval(const GB300PatchTable *t, const float *src, float *dst, float *du,
                        float *dv, float *duu, float *duv, float *dvv, int length,
                        int srcStride, int dstStride, int duStride, int dvStride,
                        int duuStride, int duvStride, int dvvStride, int numPatchCoords,
                        const void *patchCoords, void *stream) {
    if (!t) return fail(GB300_ERR_INVALID_ARGUMENT, "GB300PatchTableEval: null table");
    float *d[6] = {dst, du, dv, duu, duv, dvv};
    const int st[6] = {dstStride, duStride, dvStride, duuStride, duvStride, dvvStride};
    return eval_patches(src, d, st, length, srcStride, numPatchCoords, patchCoords, t->arrays,
                        (const int *)t->indices, t->params, as_stream(stream),
                        "GB300PatchTableEval", t->quadFamily);
}

int GB300TessellationEvaluate(const GB300PatchTable *t, const float *src, float *P, float *du,
                              float *dv, float *duu, float *duv, float *dvv, int length,
                              int srcStride, int pStride, int duStride, int dvStride,
                              int duuStride, int duvStride, int dvvStride, int numCoords,
                              const void *patchCoords, void *stream) {
    if (!t) return fail(GB300_ERR_INVALID_ARGUMENT, "GB300TessellationEvaluate: null table");
    float *d[6] = {P, du, dv, duu, duv, dvv};
    const int st[6] = {pStride, duStride, dvStride, duuStride, duvStride, dvvStride};
    return eval_patches(src, d, st, length, srcStride, numCoords, patchCoords, t->arrays,
                        (const int *)t->indices, t->params, as_stream(stream),
                        "GB300TessellationEvaluate", t->quadFamily, 1);
}

GB300StencilTable *GB300TessellationStencils(const GB300PatchTable *t, int numPoints,
                                             const void *patchCoords, int baseNumStencils,
                                             int64_t baseNumIndices, const int *baseSizes,
                                             const int *baseOffsets, const int *baseIndices,
                                             const float *baseWeights, int numChannels,
                                             int sortEntries, void *stream) {
    const char *who = "GB300TessellationStencils";
    if (!t || numPoints < 0 || (numPoints > 0 && !patchCoords) || baseNumStencils < 0 ||
        baseNumIndices < 0 || (baseNumStencils > 0 && (!baseSizes || !baseOffsets)) ||
        (baseNumIndices > 0 && (!baseIndices || !baseWeights)) ||
        !(numChannels == 1 || numChannels == 3 || numChannels == 6)) {
        fail(GB300_ERR_INVALID_ARGUMENT, "%s: bad arguments", who);
        return nullptr;
    }
    return tess_stencils(t->arrays, (const int *)t->indices, t->params, numPoints, patchCoords,
                         baseNumStencils, baseNumIndices, baseSizes, baseOffsets, baseIndices,
                         baseWeights, numChannels, sortEntries, as_stream(stream), who);
}

int GB300PatchTableTessFactors(const GB300PatchTable *t, const float *src, int srcStride,
                               const GB300PatchTessOptions *options, float *outer, float *inner,
                               float *outerLo, float *outerHi, void *stream) {
    if (!t) return fail(GB300_ERR_INVALID_ARGUMENT, "GB300PatchTableTessFactors: null table");
    return tess_factors(t->arrays, t->numArrays, (const int *)t->indices, t->params,
                        t->numPatches, src, srcStride, options, outer, inner, outerLo, outerHi,
                        as_stream(stream));
}

int GB300PatchTableSetVarying(GB300PatchTable *t, int numArrays, const void *patchArrays,
                              int64_t numIndices, const int *patchIndices, void *stream) {
    PatchSet set;
    const int st = make_set(t, "GB300PatchTableSetVarying", numArrays, patchArrays, numIndices,
                            patchIndices, 0, nullptr, as_stream(stream), set);
    if (st != GB300_OK) return st;
    t->varying.free();
    t->varying = set;
    return ok();
}

int GB300PatchTableAddFVarChannel(GB300PatchTable *t, int numArrays, const void *patchArrays,
                                  int64_t numIndices, const int *patchIndices, int numParams,
                                  const void *patchParams, int *channel, void *stream) {
    if (!patchParams || !channel)
        return fail(GB300_ERR_INVALID_ARGUMENT, "GB300PatchTableAddFVarChannel: null params");
    PatchSet set;
    const int st = make_set(t, "GB300PatchTableAddFVarChannel", numArrays, patchArrays,
                            numIndices, patchIndices, numParams, patchParams, as_stream(stream),
                            set);
    if (st != GB300_OK) return st;
    t->fvar.push_back(set);
    *channel = (int)t->fvar.size() - 1;
    return ok();
}

int GB300PatchTableGetNumFVarChannels(const GB300PatchTable *t) {
    return t ? (int)t->fvar.size() : 0;
}

void *GB300PatchTableGetVaryingBuffer(const GB300PatchTable *t, int which) {
    if (!t || !t->varying.arrays) return nullptr;
    return which == 0 ? t->varying.arrays : which == 1 ? t->varying.indices : nullptr;
}

void *GB300PatchTableGetFVarBuffer(const GB300PatchTable *t, int channel, int which) {
    if (!t || channel < 0 || channel >= (int)t->fvar.size()) return nullptr;
    const PatchSet &f = t->fvar[channel];
    return which == 0 ? f.arrays : which == 1 ? f.indices : which == 2 ? f.params : nullptr;
}

int GB300PatchTableEvalVarying(const GB300PatchTable *t, const float *src, float *dst,
                               float *du, float *dv, float *duu, float *duv, float *dvv,
                               int length, int srcStride, int dstStride, int duStride,
                               int dvStride, int duuStride, int duvStride, int dvvStride,
                               int numPatchCoords, const void *patchCoords, void *stream) {
    if (!t || !t->varying.arrays)
        return fail(GB300_ERR_INVALID_ARGUMENT,
                    "GB300PatchTableEvalVarying: table without varying patches");
    return eval_set(t, t->varying, t->params, src, dst, du, dv, duu, duv, dvv, length,
                    srcStride, dstStride, duStride, dvStride, duuStride, duvStride, dvvStride,
                    numPatchCoords, patchCoords, stream, "GB300PatchTableEvalVarying");
}

int GB300PatchTableEvalFaceVarying(const GB300PatchTable *t, int channel, const float *src,
                                   float *dst, float *du, float *dv, float *duu, float *duv,
                                   float *dvv, int length, int srcStride, int dstStride,
                                   int duStride, int dvStride, int duuStride, int duvStride,
                                   int dvvStride, int numPatchCoords, const void *patchCoords,
                                   void *stream) {
    if (!t || channel < 0 || channel >= (int)t->fvar.size())
        return fail(GB300_ERR_INVALID_ARGUMENT,
                    "GB300PatchTableEvalFaceVarying: no face-varying channel %d", channel);
    const PatchSet &f = t->fvar[channel];
    return eval_set(t, f, f.params, src, dst, du, dv, duu, duv, dvv, length, srcStride,
                    dstStride, duStride, dvStride, duuStride, duvStride, dvvStride,
                    numPatchCoords, patchCoords, stream, "GB300PatchTableEvalFaceVarying");
}

GB300VertexBuffer *GB300VertexBufferCreate(int numElements, int numVertices) {
    if (numElements <= 0 || numVertices < 0) {
        fail(GB300_ERR_INVALID_ARGUMENT, "GB300VertexBufferCreate: bad size");
        return nullptr;
    }
    GB300VertexBuffer *b = new (std::nothrow) GB300VertexBuffer;
    if (!b) {
        fail(GB300_ERR_OUT_OF_MEMORY, "GB300VertexBufferCreate: host allocation");
        return nullptr;
    }
    b->numElements = numElements;
    b->numVertices = numVertices;
    const size_t bytes = (size_t)numElements * (size_t)numVertices * sizeof(float);
    if (bytes > 0 && check_cuda(cudaMalloc((void **)&b->mem, bytes), "GB300VertexBufferCreate") !=
                         GB300_OK) {
        b->mem = nullptr;
        delete b;
        return nullptr;
    }
    ok();
    return b;
}

void GB300VertexBufferDestroy(GB300VertexBuffer *b) { delete b; }

int GB300VertexBufferUpdateData(GB300VertexBuffer *b, const float *src, int startVertex,
                                int numVertices, void *stream) {
    if (!b || !src || startVertex < 0 || numVertices < 0 ||
        (int64_t)startVertex + numVertices > b->numVertices)
        return fail(GB300_ERR_INVALID_ARGUMENT, "GB300VertexBufferUpdateData: bad range");
    if (numVertices == 0) return ok();
    const size_t off = (size_t)startVertex * b->numElements;
    const size_t bytes = (size_t)numVertices * b->numElements * sizeof(float);
    return check_cuda(cudaMemcpyAsync(b->mem + off, src, bytes, cudaMemcpyHostToDevice,
                                      as_stream(stream)),
                      "GB300VertexBufferUpdateData");
}

float *GB300VertexBufferBindCudaBuffer(GB300VertexBuffer *b) { return b ? b->mem : nullptr; }

int GB300VertexBufferGetNumElements(const GB300VertexBuffer *b) { return b ? b->numElements : 0; }

int GB300VertexBufferGetNumVertices(const GB300VertexBuffer *b) { return b ? b->numVertices : 0; }

}  // extern "C"
