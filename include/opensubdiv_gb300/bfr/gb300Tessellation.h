//
// Bfr-shaped C++ layer over the batched device tessellation of libosd_gb300.so
// (GB300TessellationCount / GB300TessellationGenerate, include/osd_gb300.h).
//
// The reference's Bfr tutorials tessellate a mesh face by face (tutorials/bfr/tutorial_1_2/
// bfr_tutorial_1_2.cpp:170-238): a Bfr::Tessellation per face, its coords evaluated by
// Bfr::Surface::Evaluate, its facets offset by the points written so far
// (Tessellation::TransformFacetCoordIndices).  GB300MeshTessellation does every face of the mesh
// in one pass on the device: the same coords (bit for bit) and facets, each coord located as a
// PatchCoord on a device patch table, which the GB300Evaluator's EvalPatches turns into P, Du,
// Dv (and second derivatives).  Options mirror Bfr::Tessellation::Options
// (bfr/tessellation.h:60-100); with the reference's headers on the include path they convert
// from it.
//
#ifndef OPENSUBDIV_GB300_BFR_GB300_TESSELLATION_H
#define OPENSUBDIV_GB300_BFR_GB300_TESSELLATION_H

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "../osd/gb300Evaluator.h"

#if defined(OSD_GB300_HAVE_OPENSUBDIV) && defined(__has_include)
#if __has_include(<opensubdiv/bfr/tessellation.h>)
#define OSD_GB300_HAVE_BFR 1
#include <opensubdiv/bfr/tessellation.h>
#include <opensubdiv/far/patchTableFactory.h>
#include <opensubdiv/far/topologyRefiner.h>
#endif
#endif

#ifdef OSD_GB300_HAVE_OPENSUBDIV
#define OSD_GB300_BFR_NAMESPACE_BEGIN \
    namespace OpenSubdiv {            \
    namespace OPENSUBDIV_VERSION {    \
    namespace Bfr {
#define OSD_GB300_BFR_NAMESPACE_END \
    }                               \
    }                               \
    }
#else
#define OSD_GB300_BFR_NAMESPACE_BEGIN \
    namespace OpenSubdiv {            \
    namespace Bfr {
#define OSD_GB300_BFR_NAMESPACE_END \
    }                               \
    }
#endif

OSD_GB300_BFR_NAMESPACE_BEGIN

/// Bfr::Tessellation of every face of a mesh, on the device.
class GB300MeshTessellation {
public:
    /// Bfr::Tessellation::Options (facet size 3 or 4, quad preservation, strides).
    class Options {
    public:
        Options() { _o.facetSize = 3, _o.preserveQuads = 0, _o.coordStride = 0, _o.facetStride = 0; }
#ifdef OSD_GB300_HAVE_BFR
        Options(Tessellation::Options const &b) {
            _o.facetSize = b.GetFacetSize();
            _o.preserveQuads = b.PreserveQuads() ? 1 : 0;
            _o.coordStride = b.GetCoordStride();
            _o.facetStride = b.GetFacetStride();
        }
#endif
        Options &PreserveQuads(bool on) { _o.preserveQuads = on ? 1 : 0; return *this; }
        bool PreserveQuads() const { return _o.preserveQuads != 0; }
        Options &SetFacetSize(int n) { _o.facetSize = (n == 4) ? 4 : 3; return *this; }
        int GetFacetSize() const { return _o.facetSize == 4 ? 4 : 3; }
        Options &SetFacetStride(int s) { _o.facetStride = s; return *this; }
        int GetFacetStride() const { return _o.facetStride; }
        Options &SetCoordStride(int s) { _o.coordStride = s; return *this; }
        int GetCoordStride() const { return _o.coordStride; }
        GB300TessellationOptions const *get() const { return &_o; }

    private:
        GB300TessellationOptions _o;
    };

    /// Per-edge rates from edge lengths, as the reference's Bfr tutorial 2.1 computes them
    /// (GB300TessellationEdgeRates): for each face corner, 1 + (int)(length / interval) capped
    /// at maxRate, the length between the points of the corner and the next corner -- mesh
    /// vertex points named by faceVerts (the hull option), or one point per corner
    /// (pointsPerCorner: the limit option).  Writes DEVICE rateOffsets (numFaces + 1) and rates
    /// (numCorners) for Create's per-face form.
    static bool ComputeEdgeRates(int numFaces, int const *faceSizes, int const *faceVerts,
                                 int64_t numCorners, float const *points, int numPoints,
                                 int pointStride, bool pointsPerCorner, float interval,
                                 int maxRate, int *rateOffsets, int *rates,
                                 void *stream = NULL) {
        return GB300TessellationEdgeRates(numFaces, faceSizes, faceVerts, numCorners, points,
                                          numPoints, pointStride, pointsPerCorner ? 1 : 0,
                                          interval, maxRate, rateOffsets, rates,
                                          stream) == GB300_OK;
    }

    /// Every face at one uniform rate (Tessellation(param, uniformRate, options)).
    /// faceSizes: DEVICE array of numFaces face sizes; regularFaceSize: the scheme's regular
    /// face size (Sdc::SchemeTypeTraits::GetRegularFaceSize).  NULL on failure
    /// (GB300GetLastErrorString says why).
    static GB300MeshTessellation *Create(int regularFaceSize, int numFaces, int const *faceSizes,
                                         int uniformRate, Options const &options = Options(),
                                         void *stream = NULL) {
        return create(regularFaceSize, numFaces, faceSizes, NULL, NULL, uniformRate, options,
                      stream);
    }

    /// Per-face rates (Tessellation(param, numRates, rates, options)): face f takes
    /// rates[rateOffsets[f] .. rateOffsets[f+1]) -- DEVICE arrays.  A face with an invalid
    /// tessellation (rate < 1, a size the scheme rejects) gets no coords, as an invalid
    /// Bfr::Tessellation has none: give faces without a limit surface a rate of 0.
    static GB300MeshTessellation *Create(int regularFaceSize, int numFaces, int const *faceSizes,
                                         int const *rateOffsets, int const *rates,
                                         Options const &options = Options(),
                                         void *stream = NULL) {
        return create(regularFaceSize, numFaces, faceSizes, rateOffsets, rates, 0, options,
                      stream);
    }

    ~GB300MeshTessellation() { cudaFree(_offsets); }

    int GetNumFaces() const { return _numFaces; }
    int GetNumCoords() const { return (int)_totals[0]; }
    int GetNumFacets() const { return (int)_totals[1]; }
    int GetNumPtexFaces() const { return (int)_totals[2]; }
    int GetFacetSize() const { return _options.GetFacetSize(); }
    int GetCoordStride() const { return _options.GetCoordStride() ? _options.GetCoordStride() : 2; }
    int GetFacetStride() const {
        return _options.GetFacetStride() ? _options.GetFacetStride() : GetFacetSize();
    }
    /// DEVICE exclusive scans (numFaces + 1 entries) of coords, facets and ptex faces.
    int64_t const *GetCoordOffsets() const { return _offsets; }
    int64_t const *GetFacetOffsets() const { return _offsets + (_numFaces + 1); }
    int64_t const *GetPtexOffsets() const { return _offsets + 2 * (size_t)(_numFaces + 1); }

    /// Writes the coords (Tessellation::GetCoords of each face) and facets (GetFacets, offset
    /// to the mesh-wide coord numbering unless meshIndices is false) into DEVICE buffers of
    /// GetNumCoords() x coord stride floats and GetNumFacets() x facet stride ints; with a
    /// patch table, also one PatchCoord per coord for GB300Evaluator::EvalPatches.
    bool Generate(float *coords, int *facets, bool meshIndices = true,
                  Osd::GB300PatchTable const *table = NULL, Osd::PatchCoord *patchCoords = NULL,
                  void *stream = NULL) const {
        return GB300TessellationGenerate(
                   _reg, _numFaces, _faceSizes, _rateOffsets, _rates, _uniformRate,
                   _options.get(), GetCoordOffsets(), GetFacetOffsets(), GetPtexOffsets(), coords,
                   facets, meshIndices ? 1 : 0, table ? table->GetHandle() : NULL, patchCoords,
                   stream) == GB300_OK;
    }

    /// Bfr::Surface::Evaluate at every coord (GB300TessellationEvaluate): P and any of Du, Dv,
    /// Duu, Duv, Dvv (NULL to skip) of `length`-wide points from the patch points `src`, at the
    /// PatchCoords Generate located on `table`; DEVICE buffers, outputs `length` floats apart.
    bool Evaluate(Osd::GB300PatchTable const *table, Osd::PatchCoord const *patchCoords,
                  float const *src, int length, int srcStride, float *P, float *Du = NULL,
                  float *Dv = NULL, float *Duu = NULL, float *Duv = NULL, float *Dvv = NULL,
                  void *stream = NULL) const {
        return table && GB300TessellationEvaluate(table->GetHandle(), src, P, Du, Dv, Duu, Duv,
                                                  Dvv, length, srcStride, length, length,
                                                  length, length, length, length,
                                                  GetNumCoords(), patchCoords,
                                                  stream) == GB300_OK;
    }

    /// Shared (watertight) points, as the reference's Bfr tutorial 2.2 shares the points of
    /// mesh vertices and edges (tutorials/bfr/tutorial_2_2/bfr_tutorial_2_2.cpp:244-430;
    /// GB300TessellationShare): after Generate, `facets` (mesh-wide coord indices, or
    /// face-local ones when meshIndices is false) become point indices in place; each point is
    /// made once, by the first face (in face order) that reaches it, and numbered as the
    /// tutorial numbers it.  faceVerts / faceEdges: DEVICE face vertices and edges per corner of
    /// the base level, numCorners each (GB300GetFaceVerticesAndEdges).  pointOffsets (DEVICE, GetNumFaces() + 1)
    /// receives each face's first point; pointPatchCoords (DEVICE, capacity GetNumCoords()) one
    /// PatchCoord per point, copied from Generate's patchCoords, for EvaluatePoints.  Every
    /// edge needs one rate in all its faces.  Returns the number of points, or -1
    /// (GB300GetLastErrorString says why).
    int64_t Share(int const *faceVerts, int const *faceEdges, int64_t numCorners,
                  int numVertices, int numEdges, int *facets,
                  Osd::PatchCoord const *patchCoords, int64_t *pointOffsets,
                  Osd::PatchCoord *pointPatchCoords, bool meshIndices = true,
                  void *stream = NULL) const {
        int64_t n = 0;
        if (GB300TessellationShare(_reg, _numFaces, _faceSizes, _rateOffsets, _rates,
                                   _uniformRate, _options.get(), GetCoordOffsets(),
                                   GetFacetOffsets(), faceVerts, faceEdges, numCorners,
                                   numVertices, numEdges, facets, meshIndices ? 1 : 0,
                                   patchCoords, NULL,
                                   pointOffsets, pointPatchCoords, NULL, NULL, NULL, NULL, &n,
                                   stream) != GB300_OK)
            return -1;
        return n;
    }

    /// Evaluate at `numPoints` PatchCoords -- the shared points of Share, each evaluated once.
    bool EvaluatePoints(Osd::GB300PatchTable const *table, Osd::PatchCoord const *pointCoords,
                        int numPoints, float const *src, int length, int srcStride, float *P,
                        float *Du = NULL, float *Dv = NULL, float *Duu = NULL,
                        float *Duv = NULL, float *Dvv = NULL, void *stream = NULL) const {
        return table && GB300TessellationEvaluate(table->GetHandle(), src, P, Du, Dv, Duu, Duv,
                                                  Dvv, length, srcStride, length, length,
                                                  length, length, length, length, numPoints,
                                                  pointCoords, stream) == GB300_OK;
    }

    /// Varying values at `numPoints` PatchCoords: the linear surfaces of
    /// Bfr::SurfaceFactory::InitVaryingSurface (bfr/surfaceFactory.h:252), as the table's
    /// varying patches (GB300PatchTableEvalVarying) over `src` holding the varying values of
    /// the control and refined vertices (Far::StencilTableFactory, INTERPOLATE_VARYING).
    bool EvaluateVarying(Osd::GB300PatchTable const *table, Osd::PatchCoord const *patchCoords,
                         int numPoints, float const *src, int length, int srcStride,
                         float *value, float *du = NULL, float *dv = NULL,
                         void *stream = NULL) const {
        return table && GB300PatchTableEvalVarying(table->GetHandle(), src, value, du, dv, NULL,
                                                   NULL, NULL, length, srcStride, length,
                                                   length, length, length, length, length,
                                                   numPoints, patchCoords, stream) == GB300_OK;
    }

    /// Bfr::Surface::EvaluateStencil at `numPoints` PatchCoords (those of Generate, or the
    /// shared points of Share; GB300TessellationStencils): a limit stencil table over the
    /// mesh's control vertices -- P and, with numChannels 3, Du and Dv (6: also the second
    /// derivatives) -- for Osd::GB300Evaluator::EvalStencils each frame, with no refinement.
    /// `pointStencils`: one stencil per point the patch indices name (control vertices first,
    /// then refined and local points: Far::StencilTableFactory with generateControlVerts plus
    /// Far::PatchTable::GetLocalPointStencilTable appended, as LimitStencilTableFactory
    /// builds it).  The caller owns the result; NULL on failure.
    static Osd::GB300StencilTable *EvaluateStencils(Osd::GB300PatchTable const *table,
                                                    Osd::PatchCoord const *patchCoords,
                                                    int numPoints,
                                                    Osd::GB300StencilTable const *pointStencils,
                                                    int numChannels = 3, void *stream = NULL) {
        if (!table || !pointStencils) return NULL;
        ::GB300StencilTable *h = GB300TessellationStencils(
            table->GetHandle(), numPoints, patchCoords, pointStencils->GetNumStencils(),
            GB300StencilTableGetNumIndices(pointStencils->GetHandle()),
            (int const *)pointStencils->GetSizesBuffer(),
            (int const *)pointStencils->GetOffsetsBuffer(),
            (int const *)pointStencils->GetIndicesBuffer(),
            (float const *)pointStencils->GetWeightsBuffer(), numChannels, 1, stream);
        return Osd::GB300StencilTable::Adopt(h);
    }

private:
    GB300MeshTessellation() {}

    static GB300MeshTessellation *create(int reg, int numFaces, int const *faceSizes,
                                         int const *rateOffsets, int const *rates,
                                         int uniformRate, Options const &options, void *stream) {
        GB300MeshTessellation *t = new GB300MeshTessellation;
        t->_reg = reg;
        t->_numFaces = numFaces;
        t->_faceSizes = faceSizes;
        t->_rateOffsets = rateOffsets;
        t->_rates = rates;
        t->_uniformRate = uniformRate;
        t->_options = options;
        if (numFaces < 0 ||
            cudaMalloc(&t->_offsets, sizeof(int64_t) * 3 * ((size_t)numFaces + 1)) !=
                cudaSuccess ||
            GB300TessellationCount(reg, numFaces, faceSizes, rateOffsets, rates, uniformRate,
                                   options.get(), t->_offsets, t->_offsets + (numFaces + 1),
                                   t->_offsets + 2 * ((size_t)numFaces + 1), t->_totals,
                                   stream) != GB300_OK) {
            delete t;
            return NULL;
        }
        return t;
    }

    int _reg = 4, _numFaces = 0, _uniformRate = 0;
    int const *_faceSizes = NULL, *_rateOffsets = NULL, *_rates = NULL;
    Options _options;
    int64_t *_offsets = NULL;
    int64_t _totals[3] = {0, 0, 0};
};

#ifdef OSD_GB300_HAVE_BFR
/// The base level's face vertices and face edges, one entry per face corner, faces in order
/// (Far::TopologyLevel::GetFaceVertices / GetFaceEdges): the topology
/// GB300MeshTessellation::Share shares points along.  Host vectors, to upload.
inline void GB300GetFaceVerticesAndEdges(Far::TopologyRefiner const &refiner,
                                         std::vector<int> &faceVerts,
                                         std::vector<int> &faceEdges) {
    Far::TopologyLevel const &base = refiner.GetLevel(0);
    faceVerts.clear();
    faceEdges.clear();
    faceVerts.reserve((size_t)base.GetNumFaceVertices());
    faceEdges.reserve((size_t)base.GetNumFaceVertices());
    for (int f = 0; f < base.GetNumFaces(); ++f) {
        Far::ConstIndexArray v = base.GetFaceVertices(f), e = base.GetFaceEdges(f);
        faceVerts.insert(faceVerts.end(), v.begin(), v.end());
        faceEdges.insert(faceEdges.end(), e.begin(), e.end());
    }
}

/// The Far patch table whose patches are the surfaces Bfr::SurfaceFactory builds with the given
/// approximation levels (its defaults: 6 for sharp and 2 for smooth features), with the options
/// the reference's Bfr regression pairs with them (regression/bfr_evaluate/
/// farPatchEvaluator.cpp:52-78): adaptive refinement of `refiner` to those levels, Gregory-basis
/// end caps, infinitely sharp patches, no shared end-cap points, no legacy corner patches, and
/// non-linear face-varying patches when the refiner has face-varying channels.  The refiner is
/// refined adaptively in place; the caller owns the returned table.
inline Far::PatchTable const *GB300CreateSurfacePatchTable(Far::TopologyRefiner &refiner,
                                                            int approxLevelSharp = 6,
                                                            int approxLevelSmooth = 2) {
    Far::PatchTableFactory::Options po(approxLevelSharp);
    po.useInfSharpPatch = true;
    po.generateLegacySharpCornerPatches = false;
    po.shareEndCapPatchPoints = false;
    po.endCapType = Far::PatchTableFactory::Options::ENDCAP_GREGORY_BASIS;
    if (refiner.GetNumFVarChannels() > 0) {
        // face-varying surfaces (SurfaceFactory::InitFaceVaryingSurface): non-linear
        // face-varying patches for every channel, isolated like the reference's Bfr regression
        po.generateFVarTables = true;
        po.generateFVarLegacyLinearPatches = false;
    }
    Far::TopologyRefiner::AdaptiveOptions ro = po.GetRefineAdaptiveOptions();
    ro.SetIsolationLevel(approxLevelSharp);
    ro.SetSecondaryLevel(approxLevelSmooth);
    refiner.RefineAdaptive(ro);
    return Far::PatchTableFactory::Create(refiner, po);
}
#endif

OSD_GB300_BFR_NAMESPACE_END

#endif  // OPENSUBDIV_GB300_BFR_GB300_TESSELLATION_H
