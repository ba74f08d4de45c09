//
// gb300Evaluator.h -- Osd::GB300Evaluator, a drop-in beside Osd::CpuEvaluator and
// Osd::CudaEvaluator for NVIDIA GB300 (sm_103a), plus its device objects.
//
// Header-only C++ layer over the C ABI of libosd_gb300.so (include/osd_gb300.h).  It mirrors
// the reference interfaces member for member:
//   GB300StencilTable   <-> Osd::CudaStencilTable   (opensubdiv/osd/cudaEvaluator.h:52-92)
//   GB300PatchTable     <-> Osd::CudaPatchTable     (opensubdiv/osd/cudaPatchTable.h:51-110)
//   GB300VertexBuffer   <-> Osd::CudaVertexBuffer   (opensubdiv/osd/cudaVertexBuffer.h:42-79)
//   GB300Evaluator      <-> Osd::CudaEvaluator      (opensubdiv/osd/cudaEvaluator.h:94-1262)
// Differences: `deviceContext`, ignored by CudaEvaluator, may carry a cudaStream_t (cast to
// void*) on which the work is queued; the bool results are false on invalid requests (as
// CpuEvaluator's) and on device errors, with the reason in GB300GetLastErrorString().
//
// Build: compile with -I<repo>/include and, when OpenSubdiv's headers are on the include
// path, the real Osd::BufferDescriptor / PatchCoord / PatchArray / PatchParam types are
// used; otherwise layout-identical stand-ins are declared here.  Link libosd_gb300.so.
//
#ifndef OPENSUBDIV_GB300_OSD_GB300_EVALUATOR_H
#define OPENSUBDIV_GB300_OSD_GB300_EVALUATOR_H

#include <cstddef>
#include <vector>

#include "../../osd_gb300.h"

#if defined(__has_include)
#if __has_include(<opensubdiv/osd/types.h>) && !defined(OSD_GB300_NO_OPENSUBDIV)
#define OSD_GB300_HAVE_OPENSUBDIV 1
#include <opensubdiv/osd/bufferDescriptor.h>
#include <opensubdiv/osd/types.h>
#include <opensubdiv/osd/cpuPatchTable.h>
#endif
#endif

#ifdef OSD_GB300_HAVE_OPENSUBDIV
#define OSD_GB300_NAMESPACE_BEGIN \
    namespace OpenSubdiv {        \
    namespace OPENSUBDIV_VERSION {  \
    namespace Osd {
#define OSD_GB300_NAMESPACE_END \
    }                           \
    }                           \
    }
#else
#define OSD_GB300_NAMESPACE_BEGIN \
    namespace OpenSubdiv {        \
    namespace Osd {
#define OSD_GB300_NAMESPACE_END \
    }                           \
    }
#endif

#ifndef OSD_GB300_HAVE_OPENSUBDIV
// Layout-identical stand-ins for the Osd types the evaluator signatures use
// (osd/bufferDescriptor.h:61-103, osd/types.h:42-130).
namespace OpenSubdiv {
namespace Osd {
struct BufferDescriptor {
    BufferDescriptor() : offset(0), length(0), stride(0) {}
    BufferDescriptor(int o, int l, int s) : offset(o), length(l), stride(s) {}
    int GetLocalOffset() const { return stride > 0 ? offset % stride : 0; }
    bool IsValid() const { return length > 0 && length <= stride - GetLocalOffset(); }
    int offset, length, stride;
};
struct PatchHandle { int arrayIndex, patchIndex, vertIndex; };
struct PatchCoord {
    PatchCoord() : s(0), t(0) { handle.arrayIndex = handle.patchIndex = handle.vertIndex = 0; }
    PatchCoord(PatchHandle h, float s_, float t_) : handle(h), s(s_), t(t_) {}
    PatchHandle handle;
    float s, t;
};
struct PatchArray { int regDesc, desc, numPatches, indexBase, stride, primitiveIdBase; };
struct PatchParam { unsigned int field0, field1; float sharpness; };
}  // namespace Osd
}  // namespace OpenSubdiv
#endif

OSD_GB300_NAMESPACE_BEGIN

namespace gb300_detail {
inline void *stream_of(void *deviceContext) { return deviceContext; }
inline bool ok(int status) { return status == GB300_OK; }

// Picks LimitStencilTable weight arrays when the table type has them.
template <class T>
auto du_of(T const *t, int) -> decltype(&t->GetDuWeights()[0]) {
    return t->GetDuWeights().empty() ? nullptr : &t->GetDuWeights()[0];
}
template <class T>
const float *du_of(T const *, long) { return nullptr; }
template <class T>
auto dv_of(T const *t, int) -> decltype(&t->GetDvWeights()[0]) {
    return t->GetDvWeights().empty() ? nullptr : &t->GetDvWeights()[0];
}
template <class T>
const float *dv_of(T const *, long) { return nullptr; }
template <class T>
auto duu_of(T const *t, int) -> decltype(&t->GetDuuWeights()[0]) {
    return t->GetDuuWeights().empty() ? nullptr : &t->GetDuuWeights()[0];
}
template <class T>
const float *duu_of(T const *, long) { return nullptr; }
template <class T>
auto duv_of(T const *t, int) -> decltype(&t->GetDuvWeights()[0]) {
    return t->GetDuvWeights().empty() ? nullptr : &t->GetDuvWeights()[0];
}
template <class T>
const float *duv_of(T const *, long) { return nullptr; }
template <class T>
auto dvv_of(T const *t, int) -> decltype(&t->GetDvvWeights()[0]) {
    return t->GetDvvWeights().empty() ? nullptr : &t->GetDvvWeights()[0];
}
template <class T>
const float *dvv_of(T const *, long) { return nullptr; }
}  // namespace gb300_detail

/// Device copy of a Far::StencilTable or Far::LimitStencilTable (CudaStencilTable).
class GB300StencilTable {
public:
    /// FAR_TABLE: Far::StencilTable or Far::LimitStencilTable (or any type with the same
    /// GetSizes / GetOffsets / GetControlIndices / GetWeights [/ GetDu..DvvWeights] members).
    template <class FAR_TABLE>
    static GB300StencilTable *Create(FAR_TABLE const *table, void *deviceContext = NULL) {
        using namespace gb300_detail;
        const int n = table->GetNumStencils();
        const int64_t nnz = (int64_t)table->GetControlIndices().size();
        ::GB300StencilTable *h = GB300StencilTableCreate(
            n, nnz, n ? &table->GetSizes()[0] : nullptr, n ? &table->GetOffsets()[0] : nullptr,
            nnz ? &table->GetControlIndices()[0] : nullptr,
            nnz ? &table->GetWeights()[0] : nullptr, du_of(table, 0), dv_of(table, 0),
            duu_of(table, 0), duv_of(table, 0), dvv_of(table, 0), stream_of(deviceContext));
        return h ? new GB300StencilTable(h) : nullptr;
    }
    ~GB300StencilTable() { GB300StencilTableDestroy(_h); }

    void *GetSizesBuffer() const { return GB300StencilTableGetBuffer(_h, 0); }
    void *GetOffsetsBuffer() const { return GB300StencilTableGetBuffer(_h, 1); }
    void *GetIndicesBuffer() const { return GB300StencilTableGetBuffer(_h, 2); }
    void *GetWeightsBuffer() const { return GB300StencilTableGetBuffer(_h, 3); }
    void *GetDuWeightsBuffer() const { return GB300StencilTableGetBuffer(_h, 4); }
    void *GetDvWeightsBuffer() const { return GB300StencilTableGetBuffer(_h, 5); }
    void *GetDuuWeightsBuffer() const { return GB300StencilTableGetBuffer(_h, 6); }
    void *GetDuvWeightsBuffer() const { return GB300StencilTableGetBuffer(_h, 7); }
    void *GetDvvWeightsBuffer() const { return GB300StencilTableGetBuffer(_h, 8); }
    int GetNumStencils() const { return GB300StencilTableGetNumStencils(_h); }
    ::GB300StencilTable *GetHandle() const { return _h; }
    /// Takes ownership of a table made by the C ABI (e.g. GB300StencilTableFactoryCreate).
    static GB300StencilTable *Adopt(::GB300StencilTable *h) {
        return h ? new GB300StencilTable(h) : nullptr;
    }

private:
    explicit GB300StencilTable(::GB300StencilTable *h) : _h(h) {}
    GB300StencilTable(GB300StencilTable const &) = delete;
    GB300StencilTable &operator=(GB300StencilTable const &) = delete;
    ::GB300StencilTable *_h;
};

/// Device copy of a flattened Far::PatchTable plus its device PatchMap (CudaPatchTable).
class GB300PatchTable {
public:
#ifdef OSD_GB300_HAVE_OPENSUBDIV
    /// Flattens like CpuPatchTable (osd/cpuPatchTable.cpp:35-158) and uploads.
    static GB300PatchTable *Create(Far::PatchTable const *farTable, void *deviceContext = NULL) {
        CpuPatchTable cpu(farTable);
        const bool tri = farTable->GetVaryingPatchDescriptor().GetNumControlVertices() == 3;
        GB300PatchTable *t = Create((int)cpu.GetNumPatchArrays(), cpu.GetPatchArrayBuffer(),
                                    (int64_t)cpu.GetPatchIndexSize(), cpu.GetPatchIndexBuffer(),
                                    (int)cpu.GetPatchParamSize(), cpu.GetPatchParamBuffer(), tri,
                                    deviceContext);
        if (!t) return nullptr;
        void *s = gb300_detail::stream_of(deviceContext);
        // varying and face-varying tables (osd/cpuPatchTable.cpp:75-114)
        bool good = cpu.GetVaryingPatchIndexSize() == 0 ||
                    GB300PatchTableSetVarying(t->_h, (int)cpu.GetNumPatchArrays(),
                                              cpu.GetVaryingPatchArrayBuffer(),
                                              (int64_t)cpu.GetVaryingPatchIndexSize(),
                                              cpu.GetVaryingPatchIndexBuffer(), s) == GB300_OK;
        for (int c = 0; good && c < cpu.GetNumFVarChannels(); ++c) {
            int ch = -1;
            good = GB300PatchTableAddFVarChannel(
                       t->_h, (int)cpu.GetNumPatchArrays(), cpu.GetFVarPatchArrayBuffer(c),
                       (int64_t)cpu.GetFVarPatchIndexSize(c), cpu.GetFVarPatchIndexBuffer(c),
                       (int)cpu.GetFVarPatchParamSize(c), cpu.GetFVarPatchParamBuffer(c), &ch,
                       s) == GB300_OK;
        }
        if (!good) {
            delete t;
            return nullptr;
        }
        return t;
    }
#endif
    /// From a flattened host table (Osd::CpuPatchTable layout).
    static GB300PatchTable *Create(int numArrays, PatchArray const *arrays, int64_t numIndices,
                                   int const *indices, int numPatches, PatchParam const *params,
                                   bool triangular, void *deviceContext = NULL) {
        ::GB300PatchTable *h = GB300PatchTableCreate(numArrays, arrays, numIndices, indices,
                                                     numPatches, params, triangular ? 1 : 0,
                                                     gb300_detail::stream_of(deviceContext));
        return h ? new GB300PatchTable(h) : nullptr;
    }
    ~GB300PatchTable() { GB300PatchTableDestroy(_h); }

    /// Varying and face-varying tables for a table created from flattened arrays (Create from
    /// a Far::PatchTable fills them itself).  AddFVarChannel returns the channel or -1.
    bool SetVarying(int numArrays, PatchArray const *arrays, int64_t numIndices,
                    int const *indices, void *deviceContext = NULL) {
        return gb300_detail::ok(GB300PatchTableSetVarying(
            _h, numArrays, arrays, numIndices, indices, gb300_detail::stream_of(deviceContext)));
    }
    int AddFVarChannel(int numArrays, PatchArray const *arrays, int64_t numIndices,
                       int const *indices, int numParams, PatchParam const *params,
                       void *deviceContext = NULL) {
        int ch = -1;
        return gb300_detail::ok(GB300PatchTableAddFVarChannel(
                   _h, numArrays, arrays, numIndices, indices, numParams, params, &ch,
                   gb300_detail::stream_of(deviceContext)))
                   ? ch
                   : -1;
    }

    void *GetPatchArrayBuffer() const { return GB300PatchTableGetBuffer(_h, 0); }
    void *GetPatchIndexBuffer() const { return GB300PatchTableGetBuffer(_h, 1); }
    void *GetPatchParamBuffer() const { return GB300PatchTableGetBuffer(_h, 2); }
    int GetNumPatchArrays() const { return GB300PatchTableGetNumArrays(_h); }
    void *GetVaryingPatchArrayBuffer() const { return GB300PatchTableGetVaryingBuffer(_h, 0); }
    void *GetVaryingPatchIndexBuffer() const { return GB300PatchTableGetVaryingBuffer(_h, 1); }
    int GetNumFVarChannels() const { return GB300PatchTableGetNumFVarChannels(_h); }
    void *GetFVarPatchArrayBuffer(int fvarChannel = 0) const {
        return GB300PatchTableGetFVarBuffer(_h, fvarChannel, 0);
    }
    void *GetFVarPatchIndexBuffer(int fvarChannel = 0) const {
        return GB300PatchTableGetFVarBuffer(_h, fvarChannel, 1);
    }
    void *GetFVarPatchParamBuffer(int fvarChannel = 0) const {
        return GB300PatchTableGetFVarBuffer(_h, fvarChannel, 2);
    }

    /// Device Far::PatchMap::FindPatch for n device-resident (face, u, v) queries, writing
    /// PatchCoords (s, t = u, v) to device memory; misses get handle (-1, -1, -1).
    bool FindPatches(int n, int const *faces, float const *u, float const *v,
                     PatchCoord *coordsOut, void *deviceContext = NULL) const {
        return gb300_detail::ok(GB300PatchTableFindPatches(
            _h, n, faces, u, v, coordsOut, gb300_detail::stream_of(deviceContext)));
    }
    /// Draw-time tessellation factors of every patch (GB300PatchTableTessFactors): the
    /// tess-control math of the patch shaders (osd/glslPatchCommonTess.glsl), per patch in
    /// param order, into DEVICE arrays of 4 (outer, 16-byte aligned) and 2 (inner) floats.
    bool TessFactors(GB300PatchTessOptions const &options, float const *src, int srcStride,
                     float *outer, float *inner, float *outerLo = NULL, float *outerHi = NULL,
                     void *deviceContext = NULL) const {
        return gb300_detail::ok(GB300PatchTableTessFactors(
            _h, src, srcStride, &options, outer, inner, outerLo, outerHi,
            gb300_detail::stream_of(deviceContext)));
    }

    ::GB300PatchTable *GetHandle() const { return _h; }

private:
    explicit GB300PatchTable(::GB300PatchTable *h) : _h(h) {}
    GB300PatchTable(GB300PatchTable const &) = delete;
    GB300PatchTable &operator=(GB300PatchTable const &) = delete;
    ::GB300PatchTable *_h;
};

/// Owning device float buffer (CudaVertexBuffer), sizes computed in 64 bits.
class GB300VertexBuffer {
public:
    static GB300VertexBuffer *Create(int numElements, int numVertices,
                                     void *deviceContext = NULL) {
        (void)deviceContext;
        ::GB300VertexBuffer *h = GB300VertexBufferCreate(numElements, numVertices);
        return h ? new GB300VertexBuffer(h) : nullptr;
    }
    ~GB300VertexBuffer() { GB300VertexBufferDestroy(_h); }
    void UpdateData(const float *src, int startVertex, int numVertices,
                    void *deviceContext = NULL) {
        GB300VertexBufferUpdateData(_h, src, startVertex, numVertices,
                                    gb300_detail::stream_of(deviceContext));
    }
    int GetNumElements() const { return GB300VertexBufferGetNumElements(_h); }
    int GetNumVertices() const { return GB300VertexBufferGetNumVertices(_h); }
    float *BindCudaBuffer() { return GB300VertexBufferBindCudaBuffer(_h); }

private:
    explicit GB300VertexBuffer(::GB300VertexBuffer *h) : _h(h) {}
    GB300VertexBuffer(GB300VertexBuffer const &) = delete;
    GB300VertexBuffer &operator=(GB300VertexBuffer const &) = delete;
    ::GB300VertexBuffer *_h;
};

/// Static, stateless evaluator with CudaEvaluator's interface.
class GB300Evaluator {
public:
    // ---- EvalStencils, raw device pointers (offsets applied here, cudaEvaluator.cpp:159) ----
    static bool EvalStencils(const float *src, BufferDescriptor const &srcDesc, float *dst,
                             BufferDescriptor const &dstDesc, const int *sizes,
                             const int *offsets, const int *indices, const float *weights,
                             int start, int end, void *deviceContext = NULL) {
        if (!dst || srcDesc.length != dstDesc.length) return false;
        return gb300_detail::ok(GB300EvalStencils(
            src + srcDesc.offset, dst + dstDesc.offset, srcDesc.length, srcDesc.stride,
            dstDesc.stride, sizes, offsets, indices, weights, start, end,
            gb300_detail::stream_of(deviceContext)));
    }
    static bool EvalStencils(const float *src, BufferDescriptor const &srcDesc, float *dst,
                             BufferDescriptor const &dstDesc, float *du,
                             BufferDescriptor const &duDesc, float *dv,
                             BufferDescriptor const &dvDesc, const int *sizes,
                             const int *offsets, const int *indices, const float *weights,
                             const float *duWeights, const float *dvWeights, int start, int end,
                             void *deviceContext = NULL) {
        return EvalStencils(src, srcDesc, dst, dstDesc, du, duDesc, dv, dvDesc, nullptr,
                            BufferDescriptor(), nullptr, BufferDescriptor(), nullptr,
                            BufferDescriptor(), sizes, offsets, indices, weights, duWeights,
                            dvWeights, nullptr, nullptr, nullptr, start, end, deviceContext);
    }
    static bool EvalStencils(const float *src, BufferDescriptor const &srcDesc, float *dst,
                             BufferDescriptor const &dstDesc, float *du,
                             BufferDescriptor const &duDesc, float *dv,
                             BufferDescriptor const &dvDesc, float *duu,
                             BufferDescriptor const &duuDesc, float *duv,
                             BufferDescriptor const &duvDesc, float *dvv,
                             BufferDescriptor const &dvvDesc, const int *sizes,
                             const int *offsets, const int *indices, const float *weights,
                             const float *duWeights, const float *dvWeights,
                             const float *duuWeights, const float *duvWeights,
                             const float *dvvWeights, int start, int end,
                             void *deviceContext = NULL) {
        BufferDescriptor const *d[6] = {&dstDesc, &duDesc, &dvDesc, &duuDesc, &duvDesc, &dvvDesc};
        float *o[6] = {dst, du, dv, duu, duv, dvv};
        for (int k = 0; k < 6; ++k) {
            if (o[k]) {
                if (d[k]->length != srcDesc.length) return false;
                o[k] += d[k]->offset;
            }
        }
        return gb300_detail::ok(GB300EvalStencilsWithDerivatives(
            src + srcDesc.offset, o[0], o[1], o[2], o[3], o[4], o[5], srcDesc.length,
            srcDesc.stride, dstDesc.stride, duDesc.stride, dvDesc.stride, duuDesc.stride,
            duvDesc.stride, dvvDesc.stride, sizes, offsets, indices, weights, duWeights,
            dvWeights, duuWeights, duvWeights, dvvWeights, start, end,
            gb300_detail::stream_of(deviceContext)));
    }

    // ---- EvalStencils over a stencil table (template forms, cudaEvaluator.h:125-142,
    // 219-249, 352-375).  STENCIL_TABLE: GB300StencilTable (evaluated through its own device
    // layout) or any type with CudaStencilTable's accessors (GetSizesBuffer ... GetDvvWeights-
    // Buffer, GetNumStencils), evaluated through the raw entry points over those buffers. ----
    template <typename SRC_BUFFER, typename DST_BUFFER, typename STENCIL_TABLE>
    static bool EvalStencils(SRC_BUFFER *srcBuffer, BufferDescriptor const &srcDesc,
                             DST_BUFFER *dstBuffer, BufferDescriptor const &dstDesc,
                             STENCIL_TABLE const *stencilTable, const void *instance = NULL,
                             void *deviceContext = NULL) {
        (void)instance;
        float *o[6] = {dstBuffer->BindCudaBuffer(), 0, 0, 0, 0, 0};
        BufferDescriptor const *d[6] = {&dstDesc, &srcDesc, &srcDesc, &srcDesc, &srcDesc,
                                        &srcDesc};
        return stencils_over(stencilTable, srcBuffer->BindCudaBuffer(), srcDesc, o, d,
                             deviceContext);
    }
    template <typename SRC_BUFFER, typename DST_BUFFER, typename STENCIL_TABLE>
    static bool EvalStencils(SRC_BUFFER *srcBuffer, BufferDescriptor const &srcDesc,
                             DST_BUFFER *dstBuffer, BufferDescriptor const &dstDesc,
                             DST_BUFFER *duBuffer, BufferDescriptor const &duDesc,
                             DST_BUFFER *dvBuffer, BufferDescriptor const &dvDesc,
                             STENCIL_TABLE const *stencilTable,
                             GB300Evaluator const *instance = NULL, void *deviceContext = NULL) {
        (void)instance;
        float *o[6] = {dstBuffer->BindCudaBuffer(), duBuffer->BindCudaBuffer(),
                       dvBuffer->BindCudaBuffer(), 0, 0, 0};
        BufferDescriptor const *d[6] = {&dstDesc, &duDesc, &dvDesc, &srcDesc, &srcDesc,
                                        &srcDesc};
        return stencils_over(stencilTable, srcBuffer->BindCudaBuffer(), srcDesc, o, d,
                             deviceContext);
    }
    template <typename SRC_BUFFER, typename DST_BUFFER, typename STENCIL_TABLE>
    static bool EvalStencils(SRC_BUFFER *srcBuffer, BufferDescriptor const &srcDesc,
                             DST_BUFFER *dstBuffer, BufferDescriptor const &dstDesc,
                             DST_BUFFER *duBuffer, BufferDescriptor const &duDesc,
                             DST_BUFFER *dvBuffer, BufferDescriptor const &dvDesc,
                             DST_BUFFER *duuBuffer, BufferDescriptor const &duuDesc,
                             DST_BUFFER *duvBuffer, BufferDescriptor const &duvDesc,
                             DST_BUFFER *dvvBuffer, BufferDescriptor const &dvvDesc,
                             STENCIL_TABLE const *stencilTable,
                             GB300Evaluator const *instance = NULL, void *deviceContext = NULL) {
        (void)instance;
        float *o[6] = {dstBuffer->BindCudaBuffer(), duBuffer->BindCudaBuffer(),
                       dvBuffer->BindCudaBuffer(), duuBuffer->BindCudaBuffer(),
                       duvBuffer->BindCudaBuffer(), dvvBuffer->BindCudaBuffer()};
        BufferDescriptor const *d[6] = {&dstDesc, &duDesc, &dvDesc, &duuDesc, &duvDesc,
                                        &dvvDesc};
        return stencils_over(stencilTable, srcBuffer->BindCudaBuffer(), srcDesc, o, d,
                             deviceContext);
    }

    // ---- EvalPatches, raw device pointers (cudaEvaluator.cpp:295-372) -----------------------
    static bool EvalPatches(const float *src, BufferDescriptor const &srcDesc, float *dst,
                            BufferDescriptor const &dstDesc, int numPatchCoords,
                            const PatchCoord *patchCoords, const PatchArray *patchArrays,
                            const int *patchIndices, const PatchParam *patchParams,
                            void *deviceContext = NULL) {
        if (!dst || srcDesc.length != dstDesc.length) return false;
        return gb300_detail::ok(GB300EvalPatches(
            src + srcDesc.offset, dst + dstDesc.offset, srcDesc.length, srcDesc.stride,
            dstDesc.stride, numPatchCoords, patchCoords, patchArrays, patchIndices, patchParams,
            gb300_detail::stream_of(deviceContext)));
    }
    static bool EvalPatches(const float *src, BufferDescriptor const &srcDesc, float *dst,
                            BufferDescriptor const &dstDesc, float *du,
                            BufferDescriptor const &duDesc, float *dv,
                            BufferDescriptor const &dvDesc, int numPatchCoords,
                            const PatchCoord *patchCoords, const PatchArray *patchArrays,
                            const int *patchIndices, const PatchParam *patchParams,
                            void *deviceContext = NULL) {
        return EvalPatches(src, srcDesc, dst, dstDesc, du, duDesc, dv, dvDesc, nullptr,
                           BufferDescriptor(), nullptr, BufferDescriptor(), nullptr,
                           BufferDescriptor(), numPatchCoords, patchCoords, patchArrays,
                           patchIndices, patchParams, deviceContext);
    }
    static bool EvalPatches(const float *src, BufferDescriptor const &srcDesc, float *dst,
                            BufferDescriptor const &dstDesc, float *du,
                            BufferDescriptor const &duDesc, float *dv,
                            BufferDescriptor const &dvDesc, float *duu,
                            BufferDescriptor const &duuDesc, float *duv,
                            BufferDescriptor const &duvDesc, float *dvv,
                            BufferDescriptor const &dvvDesc, int numPatchCoords,
                            const PatchCoord *patchCoords, const PatchArray *patchArrays,
                            const int *patchIndices, const PatchParam *patchParams,
                            void *deviceContext = NULL) {
        BufferDescriptor const *d[6] = {&dstDesc, &duDesc, &dvDesc, &duuDesc, &duvDesc, &dvvDesc};
        float *o[6] = {dst, du, dv, duu, duv, dvv};
        for (int k = 0; k < 6; ++k) {
            if (o[k]) {
                if (d[k]->length != srcDesc.length) return false;
                o[k] += d[k]->offset;
            }
        }
        return gb300_detail::ok(GB300EvalPatchesWithDerivatives(
            src + srcDesc.offset, o[0], o[1], o[2], o[3], o[4], o[5], srcDesc.length,
            srcDesc.stride, dstDesc.stride, duDesc.stride, dvDesc.stride, duuDesc.stride,
            duvDesc.stride, dvvDesc.stride, numPatchCoords, patchCoords, patchArrays,
            patchIndices, patchParams, gb300_detail::stream_of(deviceContext)));
    }

    // ---- EvalPatches / EvalPatchesVarying / EvalPatchesFaceVarying over a patch table
    // (template forms, cudaEvaluator.h:502-680, 857-1255).  PATCH_TABLE: GB300PatchTable, or
    // any type with CudaPatchTable's accessors (GetPatchArrayBuffer, GetPatchIndexBuffer,
    // GetPatchParamBuffer, the varying and face-varying ones), evaluated through the raw
    // entry points over those buffers.  PATCHCOORD_BUFFER: any type whose BindCudaBuffer()
    // returns device PatchCoords. ----
#define OSD_GB300_PATCH_FORMS(NAME, KIND, CH_PARAM, CH_ARG)                                     \
    template <typename SRC_BUFFER, typename DST_BUFFER, typename PATCHCOORD_BUFFER,            \
              typename PATCH_TABLE>                                                             \
    static bool NAME(SRC_BUFFER *srcBuffer, BufferDescriptor const &srcDesc,                   \
                     DST_BUFFER *dstBuffer, BufferDescriptor const &dstDesc,                   \
                     int numPatchCoords, PATCHCOORD_BUFFER *patchCoords,                       \
                     PATCH_TABLE *patchTable CH_PARAM, const void *instance = NULL,            \
                     void *deviceContext = NULL) {                                             \
        (void)instance;                                                                         \
        float *o[6] = {dstBuffer->BindCudaBuffer(), 0, 0, 0, 0, 0};                            \
        BufferDescriptor const *d[6] = {&dstDesc, &srcDesc, &srcDesc, &srcDesc, &srcDesc,      \
                                        &srcDesc};                                              \
        return patches_over(patchTable, KIND, CH_ARG, srcBuffer->BindCudaBuffer(), srcDesc, o, \
                            d, numPatchCoords, patchCoords->BindCudaBuffer(), deviceContext);  \
    }                                                                                           \
    template <typename SRC_BUFFER, typename DST_BUFFER, typename PATCHCOORD_BUFFER,            \
              typename PATCH_TABLE>                                                             \
    static bool NAME(SRC_BUFFER *srcBuffer, BufferDescriptor const &srcDesc,                   \
                     DST_BUFFER *dstBuffer, BufferDescriptor const &dstDesc,                   \
                     DST_BUFFER *duBuffer, BufferDescriptor const &duDesc,                     \
                     DST_BUFFER *dvBuffer, BufferDescriptor const &dvDesc,                     \
                     int numPatchCoords, PATCHCOORD_BUFFER *patchCoords,                       \
                     PATCH_TABLE *patchTable CH_PARAM, GB300Evaluator const *instance = NULL,  \
                     void *deviceContext = NULL) {                                             \
        (void)instance;                                                                         \
        float *o[6] = {dstBuffer->BindCudaBuffer(), duBuffer->BindCudaBuffer(),                \
                       dvBuffer->BindCudaBuffer(), 0, 0, 0};                                    \
        BufferDescriptor const *d[6] = {&dstDesc, &duDesc, &dvDesc, &srcDesc, &srcDesc,        \
                                        &srcDesc};                                              \
        return patches_over(patchTable, KIND, CH_ARG, srcBuffer->BindCudaBuffer(), srcDesc, o, \
                            d, numPatchCoords, patchCoords->BindCudaBuffer(), deviceContext);  \
    }                                                                                           \
    template <typename SRC_BUFFER, typename DST_BUFFER, typename PATCHCOORD_BUFFER,            \
              typename PATCH_TABLE>                                                             \
    static bool NAME(SRC_BUFFER *srcBuffer, BufferDescriptor const &srcDesc,                   \
                     DST_BUFFER *dstBuffer, BufferDescriptor const &dstDesc,                   \
                     DST_BUFFER *duBuffer, BufferDescriptor const &duDesc,                     \
                     DST_BUFFER *dvBuffer, BufferDescriptor const &dvDesc,                     \
                     DST_BUFFER *duuBuffer, BufferDescriptor const &duuDesc,                   \
                     DST_BUFFER *duvBuffer, BufferDescriptor const &duvDesc,                   \
                     DST_BUFFER *dvvBuffer, BufferDescriptor const &dvvDesc,                   \
                     int numPatchCoords, PATCHCOORD_BUFFER *patchCoords,                       \
                     PATCH_TABLE *patchTable CH_PARAM, GB300Evaluator const *instance = NULL,  \
                     void *deviceContext = NULL) {                                             \
        (void)instance;                                                                         \
        float *o[6] = {dstBuffer->BindCudaBuffer(), duBuffer->BindCudaBuffer(),                \
                       dvBuffer->BindCudaBuffer(), duuBuffer->BindCudaBuffer(),                \
                       duvBuffer->BindCudaBuffer(), dvvBuffer->BindCudaBuffer()};              \
        BufferDescriptor const *d[6] = {&dstDesc, &duDesc, &dvDesc, &duuDesc, &duvDesc,        \
                                        &dvvDesc};                                              \
        return patches_over(patchTable, KIND, CH_ARG, srcBuffer->BindCudaBuffer(), srcDesc, o, \
                            d, numPatchCoords, patchCoords->BindCudaBuffer(), deviceContext);  \
    }
#define OSD_GB300_NO_CHANNEL
#define OSD_GB300_CHANNEL , int fvarChannel = 0
    OSD_GB300_PATCH_FORMS(EvalPatches, 0, OSD_GB300_NO_CHANNEL, 0)
    OSD_GB300_PATCH_FORMS(EvalPatchesVarying, 1, OSD_GB300_NO_CHANNEL, 0)
    OSD_GB300_PATCH_FORMS(EvalPatchesFaceVarying, 2, OSD_GB300_CHANNEL, fvarChannel)
#undef OSD_GB300_PATCH_FORMS
#undef OSD_GB300_NO_CHANNEL
#undef OSD_GB300_CHANNEL

    /// Waits for the work queued on deviceContext's stream (CudaEvaluator::Synchronize).
    static void Synchronize(void *deviceContext = NULL) {
        GB300Synchronize(gb300_detail::stream_of(deviceContext));
    }

private:
    // Requested outputs o[k] (null = not requested; k = P, du, dv, duu, duv, dvv) with their
    // descriptors: false when a requested output's length differs from the source's (as
    // CpuEvaluator), else the pointers with the descriptor offsets applied.
    static bool apply_offsets(BufferDescriptor const &srcDesc, float *o[6],
                              BufferDescriptor const *const d[6]) {
        for (int k = 0; k < 6; ++k) {
            if (!o[k]) continue;
            if (d[k]->length != srcDesc.length) return false;
            o[k] += d[k]->offset;
        }
        return true;
    }
    // GB300StencilTable: its own evaluation layout.
    static bool stencils_over(GB300StencilTable const *t, const float *src,
                              BufferDescriptor const &sd, float *o[6],
                              BufferDescriptor const *const d[6], void *ctx) {
        if (!apply_offsets(sd, o, d)) return false;
        return gb300_detail::ok(GB300StencilTableEval(
            t->GetHandle(), src + sd.offset, o[0], o[1], o[2], o[3], o[4], o[5], sd.length,
            sd.stride, d[0]->stride, d[1]->stride, d[2]->stride, d[3]->stride, d[4]->stride,
            d[5]->stride, gb300_detail::stream_of(ctx)));
    }
    // Any other table with CudaStencilTable's accessors: the raw entry points over its device
    // buffers (weights of outputs not requested are not read).
    template <class TABLE>
    static bool stencils_over(TABLE const *t, const float *src, BufferDescriptor const &sd,
                              float *o[6], BufferDescriptor const *const d[6], void *ctx) {
        if (!apply_offsets(sd, o, d)) return false;
        const float *w[6] = {(const float *)t->GetWeightsBuffer(),
                             o[1] ? (const float *)t->GetDuWeightsBuffer() : nullptr,
                             o[2] ? (const float *)t->GetDvWeightsBuffer() : nullptr,
                             o[3] ? (const float *)t->GetDuuWeightsBuffer() : nullptr,
                             o[4] ? (const float *)t->GetDuvWeightsBuffer() : nullptr,
                             o[5] ? (const float *)t->GetDvvWeightsBuffer() : nullptr};
        return gb300_detail::ok(GB300EvalStencilsWithDerivatives(
            src + sd.offset, o[0], o[1], o[2], o[3], o[4], o[5], sd.length, sd.stride,
            d[0]->stride, d[1]->stride, d[2]->stride, d[3]->stride, d[4]->stride, d[5]->stride,
            (const int *)t->GetSizesBuffer(), (const int *)t->GetOffsetsBuffer(),
            (const int *)t->GetIndicesBuffer(), w[0], w[1], w[2], w[3], w[4], w[5], 0,
            t->GetNumStencils(), gb300_detail::stream_of(ctx)));
    }
    // kind: 0 vertex, 1 varying, 2 face-varying channel `ch`.
    static bool patches_over(GB300PatchTable const *t, int kind, int ch, const float *src,
                             BufferDescriptor const &sd, float *o[6],
                             BufferDescriptor const *const d[6], int n, const void *coords,
                             void *ctx) {
        if (!apply_offsets(sd, o, d)) return false;
        void *s = gb300_detail::stream_of(ctx);
        if (kind == 2)
            return gb300_detail::ok(GB300PatchTableEvalFaceVarying(
                t->GetHandle(), ch, src + sd.offset, o[0], o[1], o[2], o[3], o[4], o[5],
                sd.length, sd.stride, d[0]->stride, d[1]->stride, d[2]->stride, d[3]->stride,
                d[4]->stride, d[5]->stride, n, coords, s));
        return gb300_detail::ok(
            (kind == 1 ? GB300PatchTableEvalVarying : GB300PatchTableEval)(
                t->GetHandle(), src + sd.offset, o[0], o[1], o[2], o[3], o[4], o[5], sd.length,
                sd.stride, d[0]->stride, d[1]->stride, d[2]->stride, d[3]->stride, d[4]->stride,
                d[5]->stride, n, coords, s));
    }
    template <class TABLE>
    static bool patches_over(TABLE *t, int kind, int ch, const float *src,
                             BufferDescriptor const &sd, float *o[6],
                             BufferDescriptor const *const d[6], int n, const void *coords,
                             void *ctx) {
        if (!apply_offsets(sd, o, d)) return false;
        const void *arrays = kind == 2   ? (const void *)t->GetFVarPatchArrayBuffer(ch)
                             : kind == 1 ? (const void *)t->GetVaryingPatchArrayBuffer()
                                         : (const void *)t->GetPatchArrayBuffer();
        const int *indices = kind == 2   ? (const int *)t->GetFVarPatchIndexBuffer(ch)
                             : kind == 1 ? (const int *)t->GetVaryingPatchIndexBuffer()
                                         : (const int *)t->GetPatchIndexBuffer();
        const void *params = kind == 2 ? (const void *)t->GetFVarPatchParamBuffer(ch)
                                       : (const void *)t->GetPatchParamBuffer();
        return gb300_detail::ok(GB300EvalPatchesWithDerivatives(
            src + sd.offset, o[0], o[1], o[2], o[3], o[4], o[5], sd.length, sd.stride,
            d[0]->stride, d[1]->stride, d[2]->stride, d[3]->stride, d[4]->stride, d[5]->stride,
            n, coords, arrays, indices, params, gb300_detail::stream_of(ctx)));
    }
};

OSD_GB300_NAMESPACE_END

#endif  // OPENSUBDIV_GB300_OSD_GB300_EVALUATOR_H
